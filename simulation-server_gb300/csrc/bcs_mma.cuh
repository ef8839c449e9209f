// bcs_mma.cuh — device helpers shared by the network kernels: the bf16
// tensor-core product (mma.sync m16n8k16, FP32 accumulation) and silu.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace bcs {

// silu and its derivative with the fast exponential and division intrinsics
// (a few ulp, far below the bf16 rounding the network applies around them);
// for x < -88 the denominator is infinite and both give 0.
__device__ inline float silu_f(float x) { return __fdividef(x, 1.0f + __expf(-x)); }
__device__ inline float dsilu_f(float x) {
    const float s = __fdividef(1.0f, 1.0f + __expf(-x));
    return s * (1.0f + x * (1.0f - s));
}

// D (16 x 8, FP32) += A (16 x 16, bf16, row-major fragment) x B (16 x 8, bf16, column fragment).
__device__ inline void mma_bf16(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ inline uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// B fragments of two adjacent n-tiles (n0..n0+15) for one k-step (k0..k0+15)
// from a W^T tile in shared memory (row n, `stride` bf16 per row, rows 16-byte
// aligned): one ldmatrix.x4; b0/b1 feed the first n-tile, b2/b3 the second,
// in the layout mma_bf16 takes.
__device__ inline void ldsm_b_pair(const __nv_bfloat16* Wt, int stride, int n0, int k0, int lane, uint32_t& b0,
                                   uint32_t& b1, uint32_t& b2, uint32_t& b3) {
    const int mat = lane >> 3;
    const __nv_bfloat16* row = Wt + (n0 + ((mat >> 1) << 3) + (lane & 7)) * stride + k0 + ((mat & 1) << 3);
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(b0), "=r"(b1), "=r"(b2), "=r"(b3)
                 : "r"(a));
}

// Two FP32 values as a packed bf16 pair (round to nearest even), low half first.
__device__ inline uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ inline float round_bf16(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

}  // namespace bcs
