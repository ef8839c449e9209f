// bcs_sort.cu — stable LSD radix sort of (int key, int value) pairs, the
// replacement of thrust::stable_sort_by_key (src/grids/uniform_grid.cu:144-147).
//
// Keys are grid cell ids in [0, cells), so only ceil(log2(cells)) bits are
// sorted, 8 per pass.  Each pass is three kernels over tiles of 4096 pairs:
//   upsweep   per-tile digit histogram (shared-memory atomics), stored
//             digit-major so one exclusive scan gives every (digit, tile) its
//             global output offset in stable order;
//   scan      one CTA per digit scans that digit's row over the tiles and
//             records the digit total; the downsweep adds the exclusive scan
//             of the 256 totals;
//   downsweep each warp ranks its 16 rounds of 32 consecutive pairs with
//             __match_any_sync (rank = peers below me + running count of the
//             digit in this warp), warps are offset by an exclusive scan of
//             their per-digit counts, so the scatter keeps input order.
#include <cuda_runtime.h>

#include <cstdint>

namespace bcs {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;   // 4096
constexpr int kRadix = 256;
constexpr int kSortWarps = kSortThreads / 32;

__global__ void __launch_bounds__(kSortThreads) k_radix_upsweep(const int* __restrict__ keys, int n, int shift,
                                                                int ntiles, unsigned* __restrict__ hist) {
    __shared__ unsigned s_hist[kRadix];
    s_hist[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        int i = base + k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&s_hist[((unsigned)keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = s_hist[threadIdx.x];
}

// Exclusive block scan of one value per thread (256 threads); returns the
// prefix and leaves the block total in *total.
__device__ inline unsigned block_scan_256(unsigned v, unsigned* s_warp, unsigned* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned w = threadIdx.x < kSortWarps ? s_warp[threadIdx.x] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (threadIdx.x >= o) w += y;
        }
        if (threadIdx.x < kSortWarps) s_warp[threadIdx.x] = w;
    }
    __syncthreads();
    unsigned excl = x - v + (warp ? s_warp[warp - 1] : 0u);
    *total = s_warp[kSortWarps - 1];
    __syncthreads();
    return excl;
}

// One CTA per digit: exclusive scan of hist[digit][0..ntiles) in place, the
// row total into totals[digit].
__global__ void __launch_bounds__(kSortThreads) k_scan_rows(unsigned* hist, int ntiles, unsigned* totals) {
    __shared__ unsigned s_warp[kSortWarps];
    unsigned* row = hist + (size_t)blockIdx.x * ntiles;
    unsigned carry = 0;
    for (int base = 0; base < ntiles; base += kSortThreads) {
        const int i = base + threadIdx.x;
        const unsigned v = i < ntiles ? row[i] : 0u;
        unsigned tot;
        const unsigned ex = block_scan_256(v, s_warp, &tot);
        if (i < ntiles) row[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kSortThreads) k_radix_downsweep(const int* __restrict__ keys_in,
                                                                  const int* __restrict__ vals_in, int* keys_out,
                                                                  int* vals_out, int n, int shift, int ntiles,
                                                                  const unsigned* __restrict__ offsets,
                                                                  const unsigned* __restrict__ totals) {
    __shared__ unsigned s_cnt[kSortWarps][kRadix];
    __shared__ unsigned s_base[kRadix];
    __shared__ unsigned s_warp[kSortWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int d = lane; d < kRadix; d += 32) s_cnt[warp][d] = 0;
    {
        unsigned tot;
        const unsigned digit_base = block_scan_256(totals[threadIdx.x], s_warp, &tot);
        s_base[threadIdx.x] = digit_base + offsets[(size_t)threadIdx.x * ntiles + blockIdx.x];
    }
    __syncwarp();
    const int wbase = blockIdx.x * kSortTile + warp * (kSortTile / kSortWarps);
    const unsigned lt = (1u << lane) - 1u;
    int key[kSortItems], val[kSortItems];
    unsigned rank[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int i = wbase + r * 32 + lane;
        const bool ok = i < n;
        key[r] = ok ? keys_in[i] : 0;
        val[r] = ok ? vals_in[i] : 0;
        const unsigned d = ok ? (((unsigned)key[r] >> shift) & 0xFFu) : 0x100u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned before = __popc(peers & lt);
        const unsigned cnt = ok ? s_cnt[warp][d] : 0u;
        rank[r] = cnt + before;
        __syncwarp();
        if (ok && before == 0) s_cnt[warp][d] = cnt + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        // Exclusive scan over warps of each digit's count.
        unsigned run = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            unsigned c = s_cnt[w][threadIdx.x];
            s_cnt[w][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int i = wbase + r * 32 + lane;
        if (i >= n) continue;
        const unsigned d = ((unsigned)key[r] >> shift) & 0xFFu;
        const unsigned pos = s_base[d] + s_cnt[warp][d] + rank[r];
        keys_out[pos] = key[r];
        vals_out[pos] = val[r];
    }
}

int radix_tiles(int n) { return (n + kSortTile - 1) / kSortTile; }
size_t radix_temp_words(int n) { return (size_t)kRadix * radix_tiles(n) + kRadix; }

// Sort n pairs on `bits` low key bits from (in_k, in_v), which is left
// untouched, ping-ponging through (a_k, a_v) and (b_k, b_v).  Returns 0 when
// the result is in (a_k, a_v), 1 when it is in (b_k, b_v).
int radix_sort_pairs(const int* in_k, const int* in_v, int* a_k, int* a_v, int* b_k, int* b_v, int n, int bits,
                     unsigned* temp, cudaStream_t s) {
    if (n <= 0) return 0;
    if (bits <= 0 || n == 1) {
        cudaMemcpyAsync(a_k, in_k, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(a_v, in_v, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
        return 0;
    }
    const int ntiles = radix_tiles(n);
    int pass = 0;
    for (int shift = 0; shift < bits; shift += 8, ++pass) {
        const int* ki = pass == 0 ? in_k : ((pass & 1) ? a_k : b_k);
        const int* vi = pass == 0 ? in_v : ((pass & 1) ? a_v : b_v);
        int* ko = (pass & 1) ? b_k : a_k;
        int* vo = (pass & 1) ? b_v : a_v;
        unsigned* totals = temp + (size_t)kRadix * ntiles;
        k_radix_upsweep<<<ntiles, kSortThreads, 0, s>>>(ki, n, shift, ntiles, temp);
        k_scan_rows<<<kRadix, kSortThreads, 0, s>>>(temp, ntiles, totals);
        k_radix_downsweep<<<ntiles, kSortThreads, 0, s>>>(ki, vi, ko, vo, n, shift, ntiles, temp, totals);
    }
    return (pass & 1) ? 0 : 1;
}

}  // namespace bcs
