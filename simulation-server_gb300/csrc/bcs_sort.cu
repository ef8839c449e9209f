// bcs_sort.cu — stable sort of (int key, int value) pairs, the replacement
// of thrust::stable_sort_by_key (src/grids/uniform_grid.cu:144-147).
//
// Full sort: LSD radix over ceil(log2(cells)) key bits, 8 per pass.  Each
// pass is three kernels over tiles of 4096 pairs:
//   upsweep   per-tile digit histogram (shared-memory atomics), stored
//             digit-major so one exclusive scan gives every (digit, tile) its
//             global output offset in stable order;
//   scan      one CTA per digit scans that digit's row over the tiles and
//             records the digit total; the downsweep adds the exclusive scan
//             of the 256 totals;
//   downsweep each warp ranks its 16 rounds of 32 consecutive pairs with
//             __match_any_sync (rank = peers below me + running count of the
//             digit in this warp); the tile is staged in shared memory in
//             output order and written out in coalesced runs.
// Every kernel can take its element count from device memory, so a sort of
// a data-dependent number of pairs runs inside a captured graph.
//
// Incremental sort (sort_grid_incremental): between frames only a few
// percent of the particles change cell.  Pairs whose key is unchanged keep
// their relative order (they were sorted by (key, id) and still are), so the
// new order is that kept subsequence merged with the "movers" sorted by
// (key, id).  Since every (key, id) pair is distinct the result equals the
// full stable sort bit for bit.
#include <cuda_runtime.h>

#include <cstdint>

namespace bcs {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;   // 4096
constexpr int kRadix = 256;
constexpr int kSortWarps = kSortThreads / 32;

__device__ inline int dyn_n(int n, const int* d_n) { return d_n ? *d_n : n; }

__global__ void __launch_bounds__(kSortThreads) k_radix_upsweep(const int* __restrict__ keys, int n_max,
                                                                const int* __restrict__ d_n, int shift, int ntiles,
                                                                unsigned* __restrict__ hist) {
    __shared__ unsigned s_hist[kRadix];
    const int n = dyn_n(n_max, d_n);
    const int live = (n + kSortTile - 1) / kSortTile;
    for (int tile = blockIdx.x; tile < live; tile += gridDim.x) {
        s_hist[threadIdx.x] = 0;
        __syncthreads();
        const int base = tile * kSortTile;
#pragma unroll
        for (int k = 0; k < kSortItems; ++k) {
            int i = base + k * kSortThreads + threadIdx.x;
            if (i < n) atomicAdd(&s_hist[((unsigned)keys[i] >> shift) & 0xFFu], 1u);
        }
        __syncthreads();
        hist[(size_t)threadIdx.x * ntiles + tile] = s_hist[threadIdx.x];
        __syncthreads();
    }
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

// One CTA per row: exclusive scan of row[0..live) in place (rows of stride
// `stride`; live = the tiles holding the d_n pairs, or all), the row total
// into totals[row].
__global__ void __launch_bounds__(kSortThreads) k_scan_rows(unsigned* rows, int stride, const int* __restrict__ d_n,
                                                            unsigned* totals) {
    __shared__ unsigned s_warp[kSortWarps];
    unsigned* row = rows + (size_t)blockIdx.x * stride;
    const int len = d_n ? (*d_n + kSortTile - 1) / kSortTile : stride;
    unsigned carry = 0;
    for (int base = 0; base < len; base += kSortThreads) {
        const int i = base + threadIdx.x;
        const unsigned v = i < len ? row[i] : 0u;
        unsigned tot;
        const unsigned ex = block_scan_256(v, s_warp, &tot);
        if (i < len) row[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kSortThreads) k_radix_downsweep(const int* __restrict__ keys_in,
                                                                  const int* __restrict__ vals_in, int* keys_out,
                                                                  int* vals_out, int n_max, const int* __restrict__ d_n,
                                                                  int shift, int ntiles,
                                                                  const unsigned* __restrict__ offsets,
                                                                  const unsigned* __restrict__ totals) {
    __shared__ unsigned s_cnt[kSortWarps][kRadix];
    __shared__ unsigned s_base[kRadix];      // global start of the tile's run of each digit
    __shared__ unsigned s_tile[kRadix];      // tile-local start of each digit
    __shared__ unsigned s_warp[kSortWarps];
    __shared__ int2 s_stage[kSortTile];
    const int n = dyn_n(n_max, d_n);
    const int live = (n + kSortTile - 1) / kSortTile;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned digit_base_total;
    {
        unsigned tot;
        digit_base_total = block_scan_256(totals[threadIdx.x], s_warp, &tot);
    }
    for (int tile = blockIdx.x; tile < live; tile += gridDim.x) {
        const int tile0 = tile * kSortTile;
        for (int d = lane; d < kRadix; d += 32) s_cnt[warp][d] = 0;
        s_base[threadIdx.x] = digit_base_total + offsets[(size_t)threadIdx.x * ntiles + tile];
        __syncwarp();
        const int wbase = tile0 + warp * (kSortTile / kSortWarps);
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
        unsigned digit_total;
        {
            // Exclusive scan over warps of each digit's count.
            unsigned run = 0;
    #pragma unroll
            for (int w = 0; w < kSortWarps; ++w) {
                unsigned c = s_cnt[w][threadIdx.x];
                s_cnt[w][threadIdx.x] = run;
                run += c;
            }
            digit_total = run;
        }
        {
            unsigned tot;
            s_tile[threadIdx.x] = block_scan_256(digit_total, s_warp, &tot);
        }
        __syncthreads();
        // Stage in output order, then write each digit's run contiguously.
    #pragma unroll
        for (int r = 0; r < kSortItems; ++r) {
            const int i = wbase + r * 32 + lane;
            if (i >= n) continue;
            const unsigned d = ((unsigned)key[r] >> shift) & 0xFFu;
            s_stage[s_tile[d] + s_cnt[warp][d] + rank[r]] = make_int2(key[r], val[r]);
        }
        __syncthreads();
        const int count = min(kSortTile, n - tile0);
        for (int j = threadIdx.x; j < count; j += kSortThreads) {
            const int2 kv = s_stage[j];
            const unsigned d = ((unsigned)kv.x >> shift) & 0xFFu;
            const unsigned pos = s_base[d] + (j - s_tile[d]);
            keys_out[pos] = kv.x;
            vals_out[pos] = kv.y;
        }
        __syncthreads();
    }
}

int radix_tiles(int n) { return (n + kSortTile - 1) / kSortTile; }
size_t radix_temp_words(int n) { return (size_t)kRadix * radix_tiles(n) + kRadix; }

// Sort pairs on `bits` low key bits from (in_k, in_v), which is read only by
// the first pass, ping-ponging through (a_k, a_v) and (b_k, b_v).  The count
// is n, or *d_n when d_n is given (n then bounds it).  Returns 0 when the
// result is in (a_k, a_v), 1 when it is in (b_k, b_v).
int radix_sort_pairs_n(const int* in_k, const int* in_v, int* a_k, int* a_v, int* b_k, int* b_v, int n,
                       const int* d_n, int bits, unsigned* temp, cudaStream_t s) {
    if (n <= 0) return 0;
    if (bits <= 0) bits = 1;
    const int ntiles = radix_tiles(n);
    unsigned* totals = temp + (size_t)kRadix * ntiles;
    // a device-side count is usually far below n: a bounded grid strides
    // over the tiles that hold data
    const int grid = d_n ? (ntiles < 4 * 152 ? ntiles : 4 * 152) : ntiles;
    int pass = 0;
    for (int shift = 0; shift < bits; shift += 8, ++pass) {
        const int* ki = pass == 0 ? in_k : ((pass & 1) ? a_k : b_k);
        const int* vi = pass == 0 ? in_v : ((pass & 1) ? a_v : b_v);
        int* ko = (pass & 1) ? b_k : a_k;
        int* vo = (pass & 1) ? b_v : a_v;
        k_radix_upsweep<<<grid, kSortThreads, 0, s>>>(ki, n, d_n, shift, ntiles, temp);
        k_scan_rows<<<kRadix, kSortThreads, 0, s>>>(temp, ntiles, d_n, totals);
        k_radix_downsweep<<<grid, kSortThreads, 0, s>>>(ki, vi, ko, vo, n, d_n, shift, ntiles, temp, totals);
    }
    return (pass & 1) ? 0 : 1;
}

int radix_sort_pairs(const int* in_k, const int* in_v, int* a_k, int* a_v, int* b_k, int* b_v, int n, int bits,
                     unsigned* temp, cudaStream_t s) {
    if (n <= 0) return 0;
    if (bits <= 0 || n == 1) {
        cudaMemcpyAsync(a_k, in_k, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(a_v, in_v, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
        return 0;
    }
    return radix_sort_pairs_n(in_k, in_v, a_k, a_v, b_k, b_v, n, nullptr, bits, temp, s);
}

// ------------------------------------------------------------ incremental --
__device__ inline unsigned long long pack_pair(int key, int id) {
    return ((unsigned long long)(unsigned)key << 32) | (unsigned)id;
}

// Count, per tile of 4096 sorted slots, the pairs whose particle kept its key.
__global__ void __launch_bounds__(kSortThreads) k_inc_count(const int* __restrict__ old_k, const int* __restrict__ old_v,
                                                            const int* __restrict__ new_key_of, int n,
                                                            unsigned* __restrict__ tile_kept) {
    __shared__ unsigned s_warp[kSortWarps];
    const int base = blockIdx.x * kSortTile;
    unsigned c = 0;
#pragma unroll 4
    for (int k = 0; k < kSortItems; ++k) {
        const int i = base + k * kSortThreads + threadIdx.x;
        if (i < n) c += __ldg(&new_key_of[old_v[i]]) == old_k[i];
    }
    unsigned tot;
    block_scan_256(c, s_warp, &tot);
    if (threadIdx.x == 0) tile_kept[blockIdx.x] = tot;
}

// Exclusive scan of the per-tile kept counts (one CTA); writes the number of
// movers to *movers.
__global__ void __launch_bounds__(kSortThreads) k_inc_scan(unsigned* tile_kept, int ntiles, int n, int* movers) {
    __shared__ unsigned s_warp[kSortWarps];
    unsigned carry = 0;
    for (int base = 0; base < ntiles; base += kSortThreads) {
        const int i = base + threadIdx.x;
        const unsigned v = i < ntiles ? tile_kept[i] : 0u;
        unsigned tot;
        const unsigned ex = block_scan_256(v, s_warp, &tot);
        if (i < ntiles) tile_kept[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) *movers = n - (int)carry;
}

// Order-preserving split of the old sorted slots into kept pairs and movers.
__global__ void __launch_bounds__(kSortThreads) k_inc_split(const int* __restrict__ old_k, const int* __restrict__ old_v,
                                                            const int* __restrict__ new_key_of, int n,
                                                            const unsigned* __restrict__ tile_kept_base,
                                                            int* kept_k, int* kept_v, int* mov_k, int* mov_v) {
    __shared__ unsigned s_warp[kSortWarps];
    const int base = blockIdx.x * kSortTile;
    unsigned kept_run = tile_kept_base[blockIdx.x];
    unsigned mov_run = (unsigned)base - kept_run;
    for (int k = 0; k < kSortItems; ++k) {
        const int chunk = base + k * kSortThreads;
        const int i = chunk + threadIdx.x;
        int key = 0, id = 0;
        unsigned keep = 0;
        if (i < n) {
            id = old_v[i];
            key = __ldg(&new_key_of[id]);
            keep = key == old_k[i];
        }
        unsigned tot;
        const unsigned ex = block_scan_256(keep, s_warp, &tot);
        if (i < n) {
            if (keep) {
                kept_k[kept_run + ex] = key;
                kept_v[kept_run + ex] = id;
            } else {
                const unsigned m = mov_run + (threadIdx.x - ex);
                mov_k[m] = key;
                mov_v[m] = id;
            }
        }
        const int valid = min(kSortThreads, max(0, n - chunk));
        kept_run += tot;
        mov_run += (unsigned)valid - tot;
    }
}

// Merge the kept pairs (n - m) and the sorted movers (m) by (key, id): each
// thread finds its 8-output diagonal on the merge path, then merges.
__global__ void __launch_bounds__(256) k_inc_merge(const int* __restrict__ a_k, const int* __restrict__ a_v,
                                                   const int* __restrict__ b_k, const int* __restrict__ b_v, int n,
                                                   const int* __restrict__ movers, int* out_k, int* out_v) {
    constexpr int kItems = 8;
    const int m = *movers;
    const int na = n - m, nb = m;
    const long long diag = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kItems;
    if (diag >= n) return;
    // largest i with A[i-1] before B[diag-i]: the number of kept pairs among
    // the first `diag` outputs
    int lo = (int)max(0LL, diag - nb), hi = (int)min((long long)na, diag);
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int j = (int)(diag - mid);
        if (pack_pair(a_k[mid - 1], a_v[mid - 1]) < pack_pair(b_k[j], b_v[j])) lo = mid;
        else hi = mid - 1;
    }
    int i = lo, j = (int)(diag - lo);
    const int end = (int)min((long long)n, diag + kItems);
    for (int o = (int)diag; o < end; ++o) {
        bool take_a;
        if (i >= na) take_a = false;
        else if (j >= nb) take_a = true;
        else take_a = pack_pair(a_k[i], a_v[i]) < pack_pair(b_k[j], b_v[j]);
        if (take_a) { out_k[o] = a_k[i]; out_v[o] = a_v[i]; ++i; }
        else { out_k[o] = b_k[j]; out_v[o] = b_v[j]; ++j; }
    }
}

struct IncrementalBuffers {
    int* kept_k; int* kept_v;      // n each
    int* mov_k; int* mov_v;        // n each (movers, unsorted)
    int* t1_k; int* t1_v;          // n each (mover sort ping-pong)
    int* t2_k; int* t2_v;          // n each
    unsigned* tile_kept;           // radix_tiles(n)
    unsigned* temp;                // radix_temp_words(n)
    int* movers;                   // 1
};

// New sorted (out_k, out_v) from the previous frame's sorted (old_k, old_v)
// and the new keys by particle id.
void sort_grid_incremental(const int* old_k, const int* old_v, const int* new_key_of, int* out_k, int* out_v, int n,
                           int key_bits, int id_bits, const IncrementalBuffers& b, cudaStream_t s) {
    if (n <= 0) return;
    const int ntiles = radix_tiles(n);
    k_inc_count<<<ntiles, kSortThreads, 0, s>>>(old_k, old_v, new_key_of, n, b.tile_kept);
    k_inc_scan<<<1, kSortThreads, 0, s>>>(b.tile_kept, ntiles, n, b.movers);
    k_inc_split<<<ntiles, kSortThreads, 0, s>>>(old_k, old_v, new_key_of, n, b.tile_kept, b.kept_k, b.kept_v, b.mov_k,
                                                b.mov_v);
    // movers by id (values: keys), then stably by key (values: ids)
    const int w1 = radix_sort_pairs_n(b.mov_v, b.mov_k, b.t1_k, b.t1_v, b.t2_k, b.t2_v, n, b.movers, id_bits, b.temp, s);
    const int* by_id_k = w1 ? b.t2_k : b.t1_k;   // ids
    const int* by_id_v = w1 ? b.t2_v : b.t1_v;   // keys
    int* free_k = w1 ? b.t1_k : b.t2_k;
    int* free_v = w1 ? b.t1_v : b.t2_v;
    const int w2 =
        radix_sort_pairs_n(by_id_v, by_id_k, b.mov_k, b.mov_v, free_k, free_v, n, b.movers, key_bits, b.temp, s);
    const int* ms_k = w2 ? free_k : b.mov_k;
    const int* ms_v = w2 ? free_v : b.mov_v;
    const int threads = (n + 7) / 8;
    k_inc_merge<<<(threads + 255) / 256, 256, 0, s>>>(b.kept_k, b.kept_v, ms_k, ms_v, n, b.movers, out_k, out_v);
}

}  // namespace bcs
