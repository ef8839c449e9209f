// bcs_mpnn.cu — kernels of the learned sub-step network (forward, backward,
// optimiser).  The hidden x hidden products use mma.sync m16n8k16 bf16 tensor
// core instructions with FP32 accumulation; messages, encoder, decoder and
// the optimiser are FP32 SIMT kernels.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "bcs_internal.cuh"
#include "bcs_mma.cuh"
#include "bcs_mpnn.cuh"

namespace bcs {

namespace {

constexpr int kTileRows = 128;            // rows (nodes) per GEMM CTA
constexpr int kPad = kHidden + 8;         // smem row stride (bf16): conflict-free fragment loads
constexpr int kGemmSmem = 2 * kTileRows * kPad * (int)sizeof(__nv_bfloat16);

// Rows [r0, r0 + 128) of an FP32 [rows][128] matrix into bf16 smem (zero past `rows`).
__device__ inline void stage_rows(const float* __restrict__ X, int r0, int rows, __nv_bfloat16* As) {
    for (int q = threadIdx.x; q < kTileRows * (kHidden / 4); q += blockDim.x) {
        const int r = q / (kHidden / 4), c = (q % (kHidden / 4)) * 4;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (r0 + r < rows) v = *reinterpret_cast<const float4*>(X + (size_t)(r0 + r) * kHidden + c);
        __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
        *reinterpret_cast<__nv_bfloat162*>(As + r * kPad + c) = lo;
        *reinterpret_cast<__nv_bfloat162*>(As + r * kPad + c + 2) = hi;
    }
}

// A bf16 [128][128] matrix (row n holds the k-contiguous operand column) into smem.
__device__ inline void stage_b(const __nv_bfloat16* __restrict__ W, __nv_bfloat16* Bs) {
    for (int q = threadIdx.x; q < kHidden * (kHidden / 8); q += blockDim.x) {
        const int n = q / (kHidden / 8), k = (q % (kHidden / 8)) * 8;
        *reinterpret_cast<uint4*>(Bs + n * kPad + k) = *reinterpret_cast<const uint4*>(W + n * kHidden + k);
    }
}

// acc (16 rows x 128 cols of this warp) += As[warp rows] x Bs^T.
__device__ inline void warp_mma_128(const __nv_bfloat16* As, const __nv_bfloat16* Bs, float (&acc)[16][4]) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* a_lo = As + (warp * 16 + g) * kPad + 2 * t;
    const __nv_bfloat16* a_hi = a_lo + 8 * kPad;
#pragma unroll
    for (int ks = 0; ks < kHidden / 16; ++ks) {
        const int k0 = ks * 16;
        const uint32_t a0 = ld32(a_lo + k0), a1 = ld32(a_hi + k0), a2 = ld32(a_lo + k0 + 8), a3 = ld32(a_hi + k0 + 8);
#pragma unroll
        for (int nt = 0; nt < 16; ++nt) {
            const __nv_bfloat16* b = Bs + (nt * 8 + g) * kPad + k0 + 2 * t;
            mma_bf16(acc[nt], a0, a1, a2, a3, ld32(b), ld32(b + 8));
        }
    }
}

// Y = epi(X1 B1 + X2 B2 + bias), B given as [n][k] bf16 (the transposed weight).
__global__ void __launch_bounds__(256) k_gemm(const float* __restrict__ X1, const __nv_bfloat16* __restrict__ B1,
                                              const float* __restrict__ X2, const __nv_bfloat16* __restrict__ B2,
                                              const float* __restrict__ bias, float* Y, float* Z, int rows, int silu,
                                              int accumulate) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    __nv_bfloat16* Bs = As + kTileRows * kPad;
    const int r0 = blockIdx.x * kTileRows;
    float acc[16][4];
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
    for (int in = 0; in < 2; ++in) {
        const float* X = in ? X2 : X1;
        const __nv_bfloat16* B = in ? B2 : B1;
        if (!X) break;
        if (in) __syncthreads();
        stage_rows(X, r0, rows, As);
        stage_b(B, Bs);
        __syncthreads();
        warp_mma_128(As, Bs, acc);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
        const int col = nt * 8 + 2 * t;
        const float b0 = bias ? bias[col] : 0.f, b1 = bias ? bias[col + 1] : 0.f;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = r0 + warp * 16 + g + 8 * h;
            if (r >= rows) continue;
            float v0 = acc[nt][2 * h] + b0, v1 = acc[nt][2 * h + 1] + b1;
            float* yp = Y + (size_t)r * kHidden + col;
            if (Z) *reinterpret_cast<float2*>(Z + (size_t)r * kHidden + col) = make_float2(v0, v1);
            if (silu) {
                v0 = silu_f(v0);
                v1 = silu_f(v1);
            }
            if (accumulate) {
                const float2 o = *reinterpret_cast<const float2*>(yp);
                v0 += o.x;
                v1 += o.y;
            }
            *reinterpret_cast<float2*>(yp) = make_float2(v0, v1);
        }
    }
}

// dW[k][n] += sum_r X[r][k] dY[r][n], operands rounded to bf16.  A CTA takes
// `chunk` rows in tiles of 64 and adds its 128 x 128 partial into dW.
constexpr int kWgRows = 64;
constexpr int kWgPad = kWgRows + 8;
__global__ void __launch_bounds__(256) k_wgrad(const float* __restrict__ X, const float* __restrict__ dY, float* dW,
                                               int rows, int chunk) {
    __shared__ __align__(16) __nv_bfloat16 Xt[kHidden * kWgPad];   // [k][r]
    __shared__ __align__(16) __nv_bfloat16 Yt[kHidden * kWgPad];   // [n][r]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float acc[16][4];
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
    const int rbeg = blockIdx.x * chunk, rend = min(rows, rbeg + chunk);
    for (int r0 = rbeg; r0 < rend; r0 += kWgRows) {
        for (int q = threadIdx.x; q < kWgRows * (kHidden / 4); q += blockDim.x) {
            const int r = q / (kHidden / 4), c = (q % (kHidden / 4)) * 4;
            float4 x = make_float4(0.f, 0.f, 0.f, 0.f), y = x;
            if (r0 + r < rend) {
                x = *reinterpret_cast<const float4*>(X + (size_t)(r0 + r) * kHidden + c);
                y = *reinterpret_cast<const float4*>(dY + (size_t)(r0 + r) * kHidden + c);
            }
            Xt[(c + 0) * kWgPad + r] = __float2bfloat16_rn(x.x);
            Xt[(c + 1) * kWgPad + r] = __float2bfloat16_rn(x.y);
            Xt[(c + 2) * kWgPad + r] = __float2bfloat16_rn(x.z);
            Xt[(c + 3) * kWgPad + r] = __float2bfloat16_rn(x.w);
            Yt[(c + 0) * kWgPad + r] = __float2bfloat16_rn(y.x);
            Yt[(c + 1) * kWgPad + r] = __float2bfloat16_rn(y.y);
            Yt[(c + 2) * kWgPad + r] = __float2bfloat16_rn(y.z);
            Yt[(c + 3) * kWgPad + r] = __float2bfloat16_rn(y.w);
        }
        __syncthreads();
        const __nv_bfloat16* a_lo = Xt + (warp * 16 + g) * kWgPad + 2 * t;
        const __nv_bfloat16* a_hi = a_lo + 8 * kWgPad;
#pragma unroll
        for (int ks = 0; ks < kWgRows / 16; ++ks) {
            const int k0 = ks * 16;
            const uint32_t a0 = ld32(a_lo + k0), a1 = ld32(a_hi + k0), a2 = ld32(a_lo + k0 + 8),
                           a3 = ld32(a_hi + k0 + 8);
#pragma unroll
            for (int nt = 0; nt < 16; ++nt) {
                const __nv_bfloat16* b = Yt + (nt * 8 + g) * kWgPad + k0 + 2 * t;
                mma_bf16(acc[nt], a0, a1, a2, a3, ld32(b), ld32(b + 8));
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
        const int col = nt * 8 + 2 * t, row = warp * 16 + g;
        atomicAdd(&dW[row * kHidden + col], acc[nt][0]);
        atomicAdd(&dW[row * kHidden + col + 1], acc[nt][1]);
        atomicAdd(&dW[(row + 8) * kHidden + col], acc[nt][2]);
        atomicAdd(&dW[(row + 8) * kHidden + col + 1], acc[nt][3]);
    }
}

// ------------------------------------------------------------ SIMT -------
__device__ inline float wv(const __nv_bfloat16* w, int i) { return __bfloat162float(w[i]); }

// h = silu(Z), Z = f W_in + b_in: one warp per node, lane -> 4 columns.
__global__ void k_encode(const float* __restrict__ f, const __nv_bfloat16* __restrict__ W, const float* __restrict__ b,
                         float* Z, float* H, int n) {
    const int node = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (node >= n) return;
    float fr[kFeatIn];
#pragma unroll
    for (int q = 0; q < kFeatIn; ++q) fr[q] = f[(size_t)node * kFeatIn + q];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int c = lane * 4 + j;
        float z = b[c];
#pragma unroll
        for (int q = 0; q < kFeatIn; ++q) z = fmaf(fr[q], wv(W, q * kHidden + c), z);
        Z[(size_t)node * kHidden + c] = z;
        H[(size_t)node * kHidden + c] = silu_f(z);
    }
}

// dZ = dH silu'(Z); dW_in += f^T dZ, db_in += sum dZ (block partials in
// shared memory, one atomic per weight per block).
__global__ void __launch_bounds__(256) k_encode_bwd(const float* __restrict__ f, const float* __restrict__ Z,
                                                    const float* __restrict__ dH, float* gW, float* gb, int n) {
    __shared__ float sW[kFeatIn * kHidden];
    __shared__ float sb[kHidden];
    for (int i = threadIdx.x; i < kFeatIn * kHidden; i += blockDim.x) sW[i] = 0.f;
    for (int i = threadIdx.x; i < kHidden; i += blockDim.x) sb[i] = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    float aw[kFeatIn][4] = {};
    float ab[4] = {};
    for (int node = blockIdx.x * wpb + (threadIdx.x >> 5); node < n; node += gridDim.x * wpb) {
        float fr[kFeatIn];
#pragma unroll
        for (int q = 0; q < kFeatIn; ++q) fr[q] = f[(size_t)node * kFeatIn + q];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const size_t o = (size_t)node * kHidden + lane * 4 + j;
            const float dz = dH[o] * dsilu_f(Z[o]);
            ab[j] += dz;
#pragma unroll
            for (int q = 0; q < kFeatIn; ++q) aw[q][j] = fmaf(fr[q], dz, aw[q][j]);
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        atomicAdd(&sb[lane * 4 + j], ab[j]);
#pragma unroll
        for (int q = 0; q < kFeatIn; ++q) atomicAdd(&sW[q * kHidden + lane * 4 + j], aw[q][j]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kFeatIn * kHidden; i += blockDim.x) atomicAdd(&gW[i], sW[i]);
    for (int i = threadIdx.x; i < kHidden; i += blockDim.x) atomicAdd(&gb[i], sb[i]);
}

// M_i = (sum over the springs of i of B_j, bf16) / deg_i + ebar_i W_e + b_e,
// with ebar_i the mean of node i's edge features: one warp per node, lane ->
// 4 columns.
__global__ void k_aggregate(const float* __restrict__ B, const float* __restrict__ E,
                            const __nv_bfloat16* __restrict__ We, const float* __restrict__ be, MpnnGraph g,
                            const int* __restrict__ edge_base, float* M, int n) {
    const int node = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (node >= n) return;
    const int cell = node / g.pic, li = node - cell * g.pic, cb = cell * g.pic;
    const int e0 = g.adj_off[li], e1 = g.adj_off[li + 1];
    const float* e = E + (size_t)(edge_base[cell] + e0) * kEdgeIn;
    const float inv = 1.0f / (float)max(1, e1 - e0);
    float eb[kEdgeIn];
#pragma unroll
    for (int q = 0; q < kEdgeIn; ++q) eb[q] = 0.f;
    for (int k = 0; k < e1 - e0; ++k)
#pragma unroll
        for (int q = 0; q < kEdgeIn; ++q) eb[q] += e[k * kEdgeIn + q];
#pragma unroll
    for (int q = 0; q < kEdgeIn; ++q) eb[q] *= inv;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int c = lane * 4 + j;
        float acc = 0.f;
        for (int k = e0; k < e1; ++k) acc += round_bf16(B[(size_t)(cb + g.adj_nbr[k]) * kHidden + c]);
        float t = be[c];
#pragma unroll
        for (int q = 0; q < kEdgeIn; ++q) t = fmaf(eb[q], wv(We, q * kHidden + c), t);
        M[(size_t)node * kHidden + c] = acc * inv + t;
    }
}

// Backward of k_aggregate for node j: dB_j = sum over the springs i of j of
// dM_i / deg_i (the spring graph is symmetric), and the W_e / b_e gradients
// of node j's own row.
__global__ void __launch_bounds__(256) k_aggregate_bwd(const float* __restrict__ E, MpnnGraph g,
                                                       const int* __restrict__ edge_base, const float* __restrict__ dM,
                                                       float* dB, float* gWe, float* gbe, int n) {
    __shared__ float sW[kEdgeIn * kHidden];
    __shared__ float sb[kHidden];
    for (int i = threadIdx.x; i < kEdgeIn * kHidden; i += blockDim.x) sW[i] = 0.f;
    for (int i = threadIdx.x; i < kHidden; i += blockDim.x) sb[i] = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    float aw[kEdgeIn][4] = {};
    float ab[4] = {};
    for (int node = blockIdx.x * wpb + (threadIdx.x >> 5); node < n; node += gridDim.x * wpb) {
        const int cell = node / g.pic, li = node - cell * g.pic, cb = cell * g.pic;
        const int e0 = g.adj_off[li], e1 = g.adj_off[li + 1];
        const float* e = E + (size_t)(edge_base[cell] + e0) * kEdgeIn;
        const float inv = 1.0f / (float)max(1, e1 - e0);
        float eb[kEdgeIn];
#pragma unroll
        for (int q = 0; q < kEdgeIn; ++q) eb[q] = 0.f;
        for (int k = 0; k < e1 - e0; ++k)
#pragma unroll
            for (int q = 0; q < kEdgeIn; ++q) eb[q] += e[k * kEdgeIn + q];
#pragma unroll
        for (int q = 0; q < kEdgeIn; ++q) eb[q] *= inv;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = lane * 4 + j;
            const float dm = dM[(size_t)node * kHidden + c];
            ab[j] += dm;
#pragma unroll
            for (int q = 0; q < kEdgeIn; ++q) aw[q][j] = fmaf(eb[q], dm, aw[q][j]);
            float db = 0.f;
            for (int k = e0; k < e1; ++k) {
                const int li2 = g.adj_nbr[k];
                const float inv_i = 1.0f / (float)max(1, g.adj_off[li2 + 1] - g.adj_off[li2]);
                db += dM[(size_t)(cb + li2) * kHidden + c] * inv_i;
            }
            dB[(size_t)node * kHidden + c] = db;
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        atomicAdd(&sb[lane * 4 + j], ab[j]);
#pragma unroll
        for (int q = 0; q < kEdgeIn; ++q) atomicAdd(&sW[q * kHidden + lane * 4 + j], aw[q][j]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kEdgeIn * kHidden; i += blockDim.x) atomicAdd(&gWe[i], sW[i]);
    for (int i = threadIdx.x; i < kHidden; i += blockDim.x) atomicAdd(&gbe[i], sb[i]);
}

// y = h W_out + b_out: one warp per node, lane -> 4 inputs, warp sums.
__global__ void k_decode(const float* __restrict__ H, const __nv_bfloat16* __restrict__ W, const float* __restrict__ b,
                         float* Y, int n) {
    const int node = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (node >= n) return;
    float acc[kOut] = {};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int c = lane * 4 + j;
        const float h = H[(size_t)node * kHidden + c];
#pragma unroll
        for (int o = 0; o < kOut; ++o) acc[o] = fmaf(h, wv(W, c * kOut + o), acc[o]);
    }
#pragma unroll
    for (int o = 0; o < kOut; ++o) {
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) acc[o] += __shfl_xor_sync(0xffffffffu, acc[o], s);
    }
    if (lane < kOut) {
        float v = acc[0];
#pragma unroll
        for (int o = 1; o < kOut; ++o)
            if (lane == o) v = acc[o];
        Y[(size_t)node * kOut + lane] = v + b[lane];
    }
}

// Loss and dY: delta = 0 mean((y - t)^2), dY = 2 (y - t) / count; delta > 0
// the pseudo-Huber mean(delta^2 (sqrt(1 + (d/delta)^2) - 1)), dY = d /
// sqrt(1 + (d/delta)^2) / count.  The loss is summed into *loss.
__global__ void k_loss(const float* __restrict__ Y, const float* __restrict__ T, float* dY, float* loss, int count,
                       float delta) {
    float acc = 0.f;
    const float sc = 2.0f / (float)count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float d = Y[i] - T[i];
        if (delta > 0.f) {
            const float q = sqrtf(1.0f + (d / delta) * (d / delta));
            dY[i] = d / q / (float)count;
            acc += delta * delta * (q - 1.0f);
        } else {
            dY[i] = sc * d;
            acc += d * d;
        }
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc / (float)count);
}

// dH = dY W_out^T (+= when accumulate); gW_out += h^T dY; gb_out += sum dY.
__global__ void __launch_bounds__(256) k_decode_bwd(const float* __restrict__ H, const __nv_bfloat16* __restrict__ W,
                                                    const float* __restrict__ dY, float* dH, float* gW, float* gb, int n) {
    __shared__ float sW[kHidden * kOut];
    __shared__ float sb[kOut];
    for (int i = threadIdx.x; i < kHidden * kOut; i += blockDim.x) sW[i] = 0.f;
    if (threadIdx.x < kOut) sb[threadIdx.x] = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    float aw[4][kOut] = {};
    float ab = 0.f;
    for (int node = blockIdx.x * wpb + (threadIdx.x >> 5); node < n; node += gridDim.x * wpb) {
        float dy[kOut];
#pragma unroll
        for (int o = 0; o < kOut; ++o) dy[o] = dY[(size_t)node * kOut + o];
        if (lane < kOut) ab += dy[lane];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = lane * 4 + j;
            const float h = H[(size_t)node * kHidden + c];
            float d = 0.f;
#pragma unroll
            for (int o = 0; o < kOut; ++o) {
                d = fmaf(dy[o], wv(W, c * kOut + o), d);
                aw[j][o] = fmaf(h, dy[o], aw[j][o]);
            }
            dH[(size_t)node * kHidden + c] = d;
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int o = 0; o < kOut; ++o) atomicAdd(&sW[(lane * 4 + j) * kOut + o], aw[j][o]);
    if (lane < kOut) atomicAdd(&sb[lane], ab);
    __syncthreads();
    for (int i = threadIdx.x; i < kHidden * kOut; i += blockDim.x) atomicAdd(&gW[i], sW[i]);
    if (threadIdx.x < kOut) atomicAdd(&gb[threadIdx.x], sb[threadIdx.x]);
}

// dZ = dH silu'(Z) (elementwise), written over dZ.
__global__ void k_dsilu(const float* __restrict__ dH, const float* __restrict__ Z, float* dZ, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
        dZ[i] = dH[i] * dsilu_f(Z[i]);
}

// sum over rows of X [rows][128] into g[128].
__global__ void __launch_bounds__(256) k_colsum(const float* __restrict__ X, float* g, int rows) {
    __shared__ float sb[kHidden];
    if (threadIdx.x < kHidden) sb[threadIdx.x] = 0.f;
    __syncthreads();
    const int c = threadIdx.x & (kHidden - 1);
    float acc = 0.f;
    for (int r = blockIdx.x * 2 + (threadIdx.x >> 7); r < rows; r += gridDim.x * 2) acc += X[(size_t)r * kHidden + c];
    atomicAdd(&sb[c], acc);
    __syncthreads();
    if (threadIdx.x < kHidden) atomicAdd(&g[threadIdx.x], sb[threadIdx.x]);
}

// Adam (Kingma & Ba 2015) on the FP32 master copy; c1, c2 are the bias
// corrections 1 / (1 - b^t).
__global__ void k_adam(float* p, const float* __restrict__ g, float* m, float* v, long long count, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// bf16 copies of the parameters; the transposed copy for the square blocks
// listed in `blocks` (offsets of hidden x hidden matrices).
__global__ void k_bf16_copies(const float* __restrict__ p, __nv_bfloat16* pb, __nv_bfloat16* pbt,
                              const long long* __restrict__ blocks, int nblocks, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
        pb[i] = __float2bfloat16_rn(p[i]);
    const long long sq = (long long)kHidden * kHidden;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nblocks * sq;
         i += (long long)gridDim.x * blockDim.x) {
        const long long b = i / sq, e = i - b * sq;
        const int r = (int)(e / kHidden), c = (int)(e % kHidden);
        pbt[blocks[b] + (long long)c * kHidden + r] = __float2bfloat16_rn(p[blocks[b] + e]);
    }
}

// ------------------------------------------------------------ tcgen05 ----
// The same product on the 5th-generation tensor cores: a CTA of 128 threads
// takes 128 rows; the bf16 operands sit in shared memory in the canonical
// K-major layout without swizzle (core matrices of 8 rows x 16 bytes; the
// next core matrix along K 128 bytes on, the next 8-row group 2048 bytes
// on); one thread issues eight tcgen05.mma (M 128, N 128, K 16) per input
// into a 128-column FP32 accumulator in tensor memory and commits them to an
// mbarrier; the warps read their 32 rows back with tcgen05.ld.  Every wait is
// bounded: on expiry the CTA flags the error word, waits once more (bounded)
// and frees its tensor memory.
constexpr int kTcTile = 128 * 128 * 2;          // bytes of one operand tile
constexpr long long kTcWaitBound = 1LL << 24;   // mbarrier polls before giving up

__device__ inline uint32_t tc_offset(int m, int k) {
    return (uint32_t)((m >> 3) * 2048 + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2);
}

__device__ inline uint64_t tc_desc(uint32_t saddr, uint32_t sbo = 2048) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)(128 >> 4) << 16;    // leading byte offset: next core matrix along K
    d |= (uint64_t)(sbo >> 4) << 32;    // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;             // descriptor version of tcgen05
    return d;                           // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: FP32 D, bf16 A and B, both K-major, N 128, M 128.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

// Testing aid (bcs_set_tensor_wait_probe): when positive, the first product
// wait of every CTA polls, that many times, an mbarrier nothing arrives at
// instead of the product's own, so it expires exactly as a lost completion
// would; the give-up path then waits for the product's own completion with
// the full bound before tensor memory is freed.
__device__ int g_tc_probe_polls = 0;

__device__ inline bool tc_wait(uint32_t mbar, uint32_t phase, long long bound = kTcWaitBound) {
    for (long long i = 0; i < bound; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

__global__ void __launch_bounds__(128) k_gemm_tc(const float* __restrict__ X1, const __nv_bfloat16* __restrict__ B1,
                                                 const float* __restrict__ X2, const __nv_bfloat16* __restrict__ B2,
                                                 const float* __restrict__ bias, float* Y, float* Z, int rows,
                                                 int silu, int accumulate, unsigned* err) {
    extern __shared__ __align__(1024) unsigned char smem_tc[];
    unsigned char* As = smem_tc;
    unsigned char* Bs = smem_tc + kTcTile;
    __shared__ __align__(8) uint64_t mbar, probe;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int r0 = blockIdx.x * 128;
    const uint32_t mbar_a = (uint32_t)__cvta_generic_to_shared(&mbar);
    const uint32_t probe_a = (uint32_t)__cvta_generic_to_shared(&probe);
    const int probe_polls = g_tc_probe_polls;
    if (warp == 0) {
        const uint32_t slot = (uint32_t)__cvta_generic_to_shared(&tmem_slot);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(slot) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_a) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(probe_a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem_slot;
    const uint32_t a_base = (uint32_t)__cvta_generic_to_shared(As), b_base = (uint32_t)__cvta_generic_to_shared(Bs);
    bool ok = true;
    uint32_t phase = 0;
    for (int in = 0; in < 2; ++in) {
        const float* X = in ? X2 : X1;
        const __nv_bfloat16* B = in ? B2 : B1;
        if (!X) break;
        // one 16-byte core-matrix row per thread; the 8 lanes of a store
        // phase fill the 8 rows of one core matrix (128 contiguous bytes)
#pragma unroll 4
        for (int q = tid; q < 128 * 16; q += 128) {
            const int r = (q >> 7) * 8 + (q & 7), k = ((q >> 3) & 15) * 8;
            float4 v0 = make_float4(0.f, 0.f, 0.f, 0.f), v1 = v0;
            if (r0 + r < rows) {
                const float4* src = reinterpret_cast<const float4*>(X + (size_t)(r0 + r) * kHidden + k);
                v0 = src[0];
                v1 = src[1];
            }
            uint4 pk;
            pk.x = pack_bf16(v0.x, v0.y);
            pk.y = pack_bf16(v0.z, v0.w);
            pk.z = pack_bf16(v1.x, v1.y);
            pk.w = pack_bf16(v1.z, v1.w);
            *reinterpret_cast<uint4*>(As + tc_offset(r, k)) = pk;
        }
        for (int q = tid; q < 128 * 16; q += 128) {
            const int n = (q >> 7) * 8 + (q & 7), k = ((q >> 3) & 15) * 8;
            *reinterpret_cast<uint4*>(Bs + tc_offset(n, k)) = *reinterpret_cast<const uint4*>(B + n * kHidden + k);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int ks = 0; ks < kHidden / 16; ++ks) {
                const uint64_t ad = tc_desc(a_base + ks * 256), bd = tc_desc(b_base + ks * 256);
                const uint32_t acc = (in > 0 || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                    ::"r"(taddr), "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_a)
                         : "memory");
        }
        // the same verdict on every thread: a CTA stops issuing (and
        // restaging the operands) as a whole
        const bool seen = in == 0 && probe_polls > 0 ? tc_wait(probe_a, 0, probe_polls) : tc_wait(mbar_a, phase);
        ok = __syncthreads_and(seen ? 1 : 0) != 0;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!ok) break;
    }
    if (!ok) {
        if (tid == 0) atomicAdd(err, 1u);
        // the products already issued complete before tensor memory is freed
        tc_wait(mbar_a, phase ^ 1u);
    } else {
        const int row = r0 + warp * 32 + lane;
#pragma unroll
        for (int chunk = 0; chunk < 4; ++chunk) {
            uint32_t v[32];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)(chunk * 32)));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < rows) {
#pragma unroll
                for (int j = 0; j < 32; j += 2) {
                    const int col = chunk * 32 + j;
                    float v0 = __uint_as_float(v[j]) + (bias ? bias[col] : 0.f);
                    float v1 = __uint_as_float(v[j + 1]) + (bias ? bias[col + 1] : 0.f);
                    float* yp = Y + (size_t)row * kHidden + col;
                    if (Z) *reinterpret_cast<float2*>(Z + (size_t)row * kHidden + col) = make_float2(v0, v1);
                    if (silu) {
                        v0 = silu_f(v0);
                        v1 = silu_f(v1);
                    }
                    if (accumulate) {
                        const float2 o = *reinterpret_cast<const float2*>(yp);
                        v0 += o.x;
                        v1 += o.y;
                    }
                    *reinterpret_cast<float2*>(yp) = make_float2(v0, v1);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(taddr) : "memory");
}

// dW[k][n] += sum_r X[r][k] dY[r][n] on the tensor cores: A = X^T and B =
// dY^T are staged transposed (K = rows, 64 per stage, canonical K-major
// layout, stride byte offset 1024), four tcgen05.mma per stage accumulate in
// a 128-column tensor-memory tile across the CTA's `chunk` rows, and the
// tile is added into dW with FP32 atomics.
constexpr int kTcWgRows = 64;
constexpr int kTcWgTile = 128 * kTcWgRows * 2;

__device__ inline uint32_t tc_offset64(int m, int k) {
    return (uint32_t)((m >> 3) * 1024 + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2);
}

__global__ void __launch_bounds__(128) k_wgrad_tc(const float* __restrict__ X, const float* __restrict__ dY, float* dW,
                                                  int rows, int chunk, unsigned* err) {
    __shared__ __align__(1024) unsigned char smem_wg[2 * kTcWgTile];
    __shared__ __align__(8) uint64_t mbar, probe;
    __shared__ uint32_t tmem_slot;
    unsigned char* As = smem_wg;
    unsigned char* Bs = smem_wg + kTcWgTile;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t mbar_a = (uint32_t)__cvta_generic_to_shared(&mbar);
    const uint32_t probe_a = (uint32_t)__cvta_generic_to_shared(&probe);
    const int probe_polls = g_tc_probe_polls;
    if (warp == 0) {
        const uint32_t slot = (uint32_t)__cvta_generic_to_shared(&tmem_slot);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(slot) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_a) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(probe_a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem_slot;
    const uint32_t a_base = (uint32_t)__cvta_generic_to_shared(As), b_base = (uint32_t)__cvta_generic_to_shared(Bs);
    const int rbeg = blockIdx.x * chunk, rend = min(rows, rbeg + chunk);
    bool ok = true, any = false;
    uint32_t phase = 0;
    for (int r0 = rbeg; r0 < rend; r0 += kTcWgRows) {
        // thread = feature (warp-coalesced column reads); 8 rows packed
        // into one 16-byte core-matrix row of X^T and of dY^T
#pragma unroll 2
        for (int j = 0; j < kTcWgRows / 8; ++j) {
            float x[8], y[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int r = r0 + j * 8 + i;
                x[i] = r < rend ? X[(size_t)r * kHidden + tid] : 0.f;
                y[i] = r < rend ? dY[(size_t)r * kHidden + tid] : 0.f;
            }
            const uint4 px = make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]),
                                        pack_bf16(x[6], x[7]));
            const uint4 py = make_uint4(pack_bf16(y[0], y[1]), pack_bf16(y[2], y[3]), pack_bf16(y[4], y[5]),
                                        pack_bf16(y[6], y[7]));
            *reinterpret_cast<uint4*>(As + tc_offset64(tid, j * 8)) = px;
            *reinterpret_cast<uint4*>(Bs + tc_offset64(tid, j * 8)) = py;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int ks = 0; ks < kTcWgRows / 16; ++ks) {
                const uint64_t ad = tc_desc(a_base + ks * 256, 1024), bd = tc_desc(b_base + ks * 256, 1024);
                const uint32_t acc = (any || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                    ::"r"(taddr), "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_a)
                         : "memory");
        }
        const bool seen = !any && probe_polls > 0 ? tc_wait(probe_a, 0, probe_polls) : tc_wait(mbar_a, phase);
        any = true;
        ok = __syncthreads_and(seen ? 1 : 0) != 0;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!ok) break;
    }
    if (!ok) {
        if (tid == 0) atomicAdd(err, 1u);
        // the products already issued complete before tensor memory is freed
        tc_wait(mbar_a, phase ^ 1u);
    } else if (any) {
        const int row = warp * 32 + lane;   // feature k of X
#pragma unroll
        for (int chunk32 = 0; chunk32 < 4; ++chunk32) {
            uint32_t v[32];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)(chunk32 * 32)));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 32; ++j) atomicAdd(&dW[row * kHidden + chunk32 * 32 + j], __uint_as_float(v[j]));
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(taddr) : "memory");
}

}  // namespace

namespace {
// 0: tcgen05, 1: mma.sync; BCS_TENSOR_PATH in the environment sets the start value
int initial_path() {
    const char* e = std::getenv("BCS_TENSOR_PATH");
    return e && e[0] == '1' ? 1 : 0;
}
int g_gemm_path = initial_path();
unsigned* g_gemm_err = nullptr;      // tcgen05 wait expiries (device word)
}  // namespace

void mpnn_set_gemm_path(int path) { g_gemm_path = path; }
bool mpnn_set_wait_probe(int polls) {
    return cudaDeviceSynchronize() == cudaSuccess &&
           cudaMemcpyToSymbol(g_tc_probe_polls, &polls, sizeof(int)) == cudaSuccess &&
           cudaDeviceSynchronize() == cudaSuccess;
}
int mpnn_gemm_path() { return g_gemm_path; }
unsigned* mpnn_gemm_error_word() {
    if (!g_gemm_err) {
        cudaMalloc(&g_gemm_err, sizeof(unsigned));
        cudaMemset(g_gemm_err, 0, sizeof(unsigned));
        cudaDeviceSynchronize();   // cleared before any stream's kernel can write it
    }
    return g_gemm_err;
}

void mpnn_gemm(const float* X1, const __nv_bfloat16* W1t, const float* X2, const __nv_bfloat16* W2t,
               const float* bias, float* Y, float* Zout, int rows, bool silu, bool accumulate, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
        cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * kTcTile);
        attr = true;
    }
    if (rows <= 0) return;
    if (g_gemm_path == 0) {
        k_gemm_tc<<<(rows + 127) / 128, 128, 2 * kTcTile, s>>>(X1, W1t, X2, W2t, bias, Y, Zout, rows, silu ? 1 : 0,
                                                              accumulate ? 1 : 0, mpnn_gemm_error_word());
        return;
    }
    k_gemm<<<(rows + kTileRows - 1) / kTileRows, 256, kGemmSmem, s>>>(X1, W1t, X2, W2t, bias, Y, Zout, rows,
                                                                     silu ? 1 : 0, accumulate ? 1 : 0);
}

void mpnn_gemm_t(const float* dY, const __nv_bfloat16* W, float* dX, int rows, bool accumulate, cudaStream_t s) {
    // dX = dY W^T: the B operand in [n][k] form is W itself (row-major [in][out]).
    mpnn_gemm(dY, W, nullptr, nullptr, nullptr, dX, nullptr, rows, false, accumulate, s);
}

void mpnn_wgrad(const float* X, const float* dY, float* dW, int rows, cudaStream_t s) {
    if (rows <= 0) return;
    const int chunk = 1024;
    if (g_gemm_path == 0) {
        // about two CTAs per SM, in whole 64-row stages
        const int tc_chunk = std::max(kTcWgRows, (rows / 304 + kTcWgRows - 1) / kTcWgRows * kTcWgRows);
        k_wgrad_tc<<<(rows + tc_chunk - 1) / tc_chunk, 128, 0, s>>>(X, dY, dW, rows, tc_chunk, mpnn_gemm_error_word());
        return;
    }
    k_wgrad<<<(rows + chunk - 1) / chunk, 256, 0, s>>>(X, dY, dW, rows, chunk);
}

// ------------------------------------------------------------ MpnnNet ----
namespace {
int grid_for(long long n, int threads, int cap = 4096) {
    return (int)std::max(1LL, std::min<long long>(cap, (n + threads - 1) / threads));
}
// SplitMix64 for the initial weights (Steele, Lea, Flood, OOPSLA 2014).
unsigned long long splitmix(unsigned long long& x) {
    unsigned long long z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
}  // namespace

MpnnNet::~MpnnNet() {
    for (void* p : allocs_) cudaFree(p);
}

float* MpnnNet::alloc(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(float)) != cudaSuccess) {
        (void)cudaGetLastError();   // reported by the caller's status
        return nullptr;
    }
    allocs_.push_back(p);
    bytes_ += n * sizeof(float);
    return static_cast<float*>(p);
}

int MpnnNet::init(int layers, int pic, const int* adj_off, const int* adj_nbr, const float* adj_len, int max_cells,
                  unsigned long long seed, cudaStream_t stream) {
    st_ = stream;
    L_ = mpnn_layout(layers);
    pic_ = pic;
    edges_ = adj_off[pic];
    max_cells_ = max_cells;
    // the aggregation's backward relies on a symmetric spring graph
    std::vector<int> base(max_cells);
    for (int i = 0; i < pic; ++i)
        for (int k = adj_off[i]; k < adj_off[i + 1]; ++k) {
            const int j = adj_nbr[k];
            bool back = false;
            for (int q = adj_off[j]; q < adj_off[j + 1]; ++q) back = back || adj_nbr[q] == i;
            if (!back) return (int)cudaErrorInvalidValue;
        }
    for (int c = 0; c < max_cells; ++c) base[c] = c * edges_;
    auto up = [&](auto** dst, const auto* src, size_t n) {
        *dst = reinterpret_cast<std::remove_pointer_t<decltype(dst)>>(alloc((n * sizeof(**dst) + 3) / 4));
        return *dst && cudaMemcpyAsync(*dst, src, n * sizeof(**dst), cudaMemcpyHostToDevice, st_) == cudaSuccess;
    };
    if (!up(&adj_off_, adj_off, pic + 1) || !up(&adj_nbr_, adj_nbr, edges_) || !up(&adj_len_, adj_len, edges_) ||
        !up(&edge_base_, base.data(), max_cells))
        return (int)cudaErrorMemoryAllocation;
    const long long P = L_.total;
    p_ = alloc(P); g_ = alloc(P); m_ = alloc(P); v_ = alloc(P);
    pb_ = reinterpret_cast<__nv_bfloat16*>(alloc((P + 1) / 2));
    pbt_ = reinterpret_cast<__nv_bfloat16*>(alloc((P + 1) / 2));
    std::vector<long long> sq;
    for (int l = 0; l < layers; ++l) {
        sq.push_back(L_.wb[l]); sq.push_back(L_.wu[l]); sq.push_back(L_.wv[l]);
    }
    nsq_ = (int)sq.size();
    sq_ = reinterpret_cast<long long*>(alloc(2 * sq.size()));
    if (!p_ || !g_ || !m_ || !v_ || !pb_ || !pbt_ || !sq_) return (int)cudaErrorMemoryAllocation;
    cudaMemcpyAsync(sq_, sq.data(), sizeof(long long) * sq.size(), cudaMemcpyHostToDevice, st_);
    // weights uniform in +-1/sqrt(fan_in), biases 0
    std::vector<float> h(P, 0.f);
    unsigned long long x = seed;
    auto fill = [&](long long off, int fan_in, long long n) {
        const double lim = 1.0 / std::sqrt((double)fan_in);
        for (long long i = 0; i < n; ++i) {
            const double u = (double)(splitmix(x) >> 11) * (1.0 / 9007199254740992.0);
            h[off + i] = (float)((2.0 * u - 1.0) * lim);
        }
    };
    fill(L_.w_in, kFeatIn, (long long)kFeatIn * kHidden);
    for (int l = 0; l < layers; ++l) {
        fill(L_.wb[l], kHidden, (long long)kHidden * kHidden);
        fill(L_.we[l], kEdgeIn, (long long)kEdgeIn * kHidden);
        fill(L_.wu[l], kHidden, (long long)kHidden * kHidden);
        fill(L_.wv[l], kHidden, (long long)kHidden * kHidden);
    }
    fill(L_.w_out, kHidden, (long long)kHidden * kOut);
    // stream-ordered uploads: the kernels below run on st_, which does not
    // wait for the legacy stream
    cudaMemcpyAsync(p_, h.data(), sizeof(float) * P, cudaMemcpyHostToDevice, st_);
    cudaMemsetAsync(m_, 0, sizeof(float) * P, st_);
    cudaMemsetAsync(v_, 0, sizeof(float) * P, st_);
    // activations
    const size_t n = (size_t)max_cells * pic, H = kHidden;
    f_ = alloc(n * kFeatIn); e_ = alloc((size_t)max_cells * edges_ * kEdgeIn); t_ = alloc(n * kOut);
    y_ = alloc(n * kOut); dy_ = alloc(n * kOut); loss_ = alloc(1);
    z0_ = alloc(n * H); dh_ = alloc(n * H); db_ = alloc(n * H); dm_ = alloc(n * H); dz_ = alloc(n * H);
    for (int l = 0; l <= layers; ++l) h_[l] = alloc(n * H);
    for (int l = 0; l < layers; ++l) {
        zb_[l] = alloc(n * H); b_[l] = alloc(n * H); mm_[l] = alloc(n * H); zu_[l] = alloc(n * H);
    }
    if (!f_ || !e_ || !t_ || !y_ || !dy_ || !loss_ || !z0_ || !dh_ || !db_ || !dm_ || !dz_ || !h_[layers] ||
        !zu_[layers - 1])
        return (int)cudaErrorMemoryAllocation;
    refresh_bf16();
    cudaStreamSynchronize(st_);
    return (int)cudaGetLastError();
}

void MpnnNet::refresh_bf16() {
    k_bf16_copies<<<grid_for(L_.total, 256), 256, 0, st_>>>(p_, pb_, pbt_, sq_, nsq_, L_.total);
}

void MpnnNet::forward(const float* f, const float* E, int cells, bool keep) {
    const int n = cells * pic_;
    const MpnnGraph g{cells, pic_, adj_off_, adj_nbr_, adj_len_};
    const int wgrid = (n * 32 + 255) / 256;
    last_f_ = f;
    last_e_ = E;
    k_encode<<<wgrid, 256, 0, st_>>>(f, pb_ + L_.w_in, p_ + L_.b_in, z0_, h_[0], n);
    for (int l = 0; l < L_.layers; ++l) {
        float* hin = keep ? h_[l] : h_[l & 1];
        float* hout = keep ? h_[l + 1] : h_[(l + 1) & 1];
        float* ZB = keep ? zb_[l] : zb_[0];
        float* B = keep ? b_[l] : b_[0];
        float* M = keep ? mm_[l] : mm_[0];
        float* ZU = keep ? zu_[l] : zu_[0];
        mpnn_gemm(hin, pbt_ + L_.wb[l], nullptr, nullptr, p_ + L_.bb[l], B, ZB, n, true, false, st_);
        k_aggregate<<<wgrid, 256, 0, st_>>>(B, E, pb_ + L_.we[l], p_ + L_.be[l], g, edge_base_, M, n);
        cudaMemcpyAsync(hout, hin, sizeof(float) * (size_t)n * kHidden, cudaMemcpyDeviceToDevice, st_);
        mpnn_gemm(hin, pbt_ + L_.wu[l], M, pbt_ + L_.wv[l], p_ + L_.bu[l], hout, ZU, n, true, true, st_);
    }
    float* hl = keep ? h_[L_.layers] : h_[L_.layers & 1];
    k_decode<<<wgrid, 256, 0, st_>>>(hl, pb_ + L_.w_out, p_ + L_.b_out, y_, n);
}

void MpnnNet::backward(const float* T, int cells) {
    const int n = cells * pic_;
    const MpnnGraph g{cells, pic_, adj_off_, adj_nbr_, adj_len_};
    const size_t nh = (size_t)n * kHidden;
    cudaMemsetAsync(g_, 0, sizeof(float) * L_.total, st_);
    cudaMemsetAsync(loss_, 0, sizeof(float), st_);
    k_loss<<<grid_for((long long)n * kOut, 256, 1024), 256, 0, st_>>>(y_, T, dy_, loss_, n * kOut, huber_);
    const int rgrid = grid_for((long long)n * 32, 256, 1216);
    k_decode_bwd<<<rgrid, 256, 0, st_>>>(h_[L_.layers], pb_ + L_.w_out, dy_, dh_, g_ + L_.w_out, g_ + L_.b_out, n);
    for (int l = L_.layers - 1; l >= 0; --l) {
        k_dsilu<<<grid_for((long long)nh, 256), 256, 0, st_>>>(dh_, zu_[l], dz_, (long long)nh);
        mpnn_wgrad(h_[l], dz_, g_ + L_.wu[l], n, st_);
        mpnn_wgrad(mm_[l], dz_, g_ + L_.wv[l], n, st_);
        k_colsum<<<grid_for(n, 2, 1216), 256, 0, st_>>>(dz_, g_ + L_.bu[l], n);
        mpnn_gemm_t(dz_, pb_ + L_.wv[l], dm_, n, false, st_);
        mpnn_gemm_t(dz_, pb_ + L_.wu[l], dh_, n, true, st_);
        k_aggregate_bwd<<<rgrid, 256, 0, st_>>>(last_e_, g, edge_base_, dm_, db_, g_ + L_.we[l], g_ + L_.be[l], n);
        k_dsilu<<<grid_for((long long)nh, 256), 256, 0, st_>>>(db_, zb_[l], dz_, (long long)nh);
        mpnn_wgrad(h_[l], dz_, g_ + L_.wb[l], n, st_);
        k_colsum<<<grid_for(n, 2, 1216), 256, 0, st_>>>(dz_, g_ + L_.bb[l], n);
        mpnn_gemm_t(dz_, pb_ + L_.wb[l], dh_, n, true, st_);
    }
    k_encode_bwd<<<rgrid, 256, 0, st_>>>(last_f_, z0_, dh_, g_ + L_.w_in, g_ + L_.b_in, n);
}

void MpnnNet::adam(float lr) {
    ++t_adam_;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f / (1.0f - std::pow(b1, (float)t_adam_)), c2 = 1.0f / (1.0f - std::pow(b2, (float)t_adam_));
    k_adam<<<grid_for(L_.total, 256), 256, 0, st_>>>(p_, g_, m_, v_, L_.total, lr, b1, b2, 1e-8f, c1, c2);
    refresh_bf16();
}

}  // namespace bcs
