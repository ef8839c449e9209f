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

#include "bcs_internal.cuh"

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
    after_previous();
    __shared__ unsigned s_hist[kRadix];
    const int n = dyn_n(n_max, d_n);
    if (d_n && n <= kSortTile) return;   // k_radix_small sorted them
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
    after_previous();
    __shared__ unsigned s_warp[kSortWarps];
    if (d_n && *d_n <= kSortTile) return;   // k_radix_small sorted them
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
    after_previous();
    __shared__ unsigned s_cnt[kSortWarps][kRadix];
    __shared__ unsigned s_base[kRadix];      // global start of the tile's run of each digit
    __shared__ unsigned s_tile[kRadix];      // tile-local start of each digit
    __shared__ unsigned s_warp[kSortWarps];
    __shared__ int2 s_stage[kSortTile];
    const int n = dyn_n(n_max, d_n);
    if (d_n && n <= kSortTile) return;   // k_radix_small sorted them
    const int live = (n + kSortTile - 1) / kSortTile;
    if ((int)blockIdx.x >= live) return;   // no tile for this CTA (a device-side count far below n_max)
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

// Up to one tile (4 096 pairs) sorted by one CTA through every pass in
// shared memory, with the downsweep's stable ranking (pair j: warp j / 512,
// round j % 512 / 32, lane j % 32).  in and out may be the same arrays.
__device__ inline void sort_one_tile(const int* in_k, const int* in_v, int* out_k, int* out_v, int n, int bits,
                                     unsigned (*s_cnt)[kRadix], unsigned* s_tile, unsigned* s_warp, int2* s_stage) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wbase = warp * (kSortTile / kSortWarps);
    const unsigned lt = (1u << lane) - 1u;
    int key[kSortItems], val[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int i = wbase + r * 32 + lane;
        key[r] = i < n ? in_k[i] : 0;
        val[r] = i < n ? in_v[i] : 0;
    }
    for (int shift = 0; shift < bits; shift += 8) {
        for (int d = lane; d < kRadix; d += 32) s_cnt[warp][d] = 0;
        __syncwarp();
        unsigned rank[kSortItems];
#pragma unroll
        for (int r = 0; r < kSortItems; ++r) {
            const bool ok = wbase + r * 32 + lane < n;
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
        unsigned run = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            const unsigned c = s_cnt[w][threadIdx.x];
            s_cnt[w][threadIdx.x] = run;
            run += c;
        }
        {
            unsigned tot;
            s_tile[threadIdx.x] = block_scan_256(run, s_warp, &tot);
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kSortItems; ++r) {
            if (wbase + r * 32 + lane >= n) continue;
            const unsigned d = ((unsigned)key[r] >> shift) & 0xFFu;
            s_stage[s_tile[d] + s_cnt[warp][d] + rank[r]] = make_int2(key[r], val[r]);
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kSortItems; ++r) {
            const int i = wbase + r * 32 + lane;
            if (i < n) {
                const int2 kv = s_stage[i];
                key[r] = kv.x;
                val[r] = kv.y;
            }
        }
        __syncthreads();   // s_cnt and s_stage are rewritten by the next pass
    }
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int i = wbase + r * 32 + lane;
        if (i < n) {
            out_k[i] = key[r];
            out_v[i] = val[r];
        }
    }
}

// A device-side count of at most one tile, sorted by one CTA (sort_one_tile);
// larger counts are left to the pass kernels, which return at once for
// small ones.
__global__ void __launch_bounds__(kSortThreads) k_radix_small(const int* in_k, const int* in_v, int* out_k, int* out_v,
                                                              const int* __restrict__ d_n, int bits) {
    after_previous();
    __shared__ unsigned s_cnt[kSortWarps][kRadix];
    __shared__ unsigned s_tile[kRadix];
    __shared__ unsigned s_warp[kSortWarps];
    __shared__ int2 s_stage[kSortTile];
    const int n = *d_n;
    if (n > kSortTile) return;
    sort_one_tile(in_k, in_v, out_k, out_v, n, bits, s_cnt, s_tile, s_warp, s_stage);
}

// A device-side count of any size sorted by one CTA, with no pass kernels
// after it: up to one tile as k_radix_small does; a larger count through the
// passes of the full sort (in -> a -> b -> a ...) with every tile ranked in
// turn by the same stable per-warp ranking and scattered from a running
// offset per digit.  The result lands where the pass kernels would leave it:
// (a_k, a_v) after an odd number of passes, (b_k, b_v) after an even one.
// Meant for frames whose movers fit one tile; a larger count is sorted
// correctly but slowly.
__global__ void __launch_bounds__(kSortThreads) k_radix_onecta(const int* in_k, const int* in_v, int* a_k, int* a_v,
                                                               int* b_k, int* b_v, const int* __restrict__ d_n,
                                                               int bits) {
    after_previous();
    __shared__ unsigned s_cnt[kSortWarps][kRadix];
    __shared__ unsigned s_tile[kRadix];
    __shared__ unsigned s_warp[kSortWarps];
    __shared__ unsigned s_base[kRadix];
    __shared__ int2 s_stage[kSortTile];
    const int n = *d_n;
    const int passes = (bits + 7) / 8;
    if (n <= kSortTile) {
        sort_one_tile(in_k, in_v, (passes & 1) ? a_k : b_k, (passes & 1) ? a_v : b_v, n, bits, s_cnt, s_tile,
                      s_warp, s_stage);
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wbase = warp * (kSortTile / kSortWarps);
    const unsigned lt = (1u << lane) - 1u;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        const int* ik = p == 0 ? in_k : ((p & 1) ? a_k : b_k);
        const int* iv = p == 0 ? in_v : ((p & 1) ? a_v : b_v);
        int* ok_ = (p & 1) ? b_k : a_k;
        int* ov_ = (p & 1) ? b_v : a_v;
        // the digit counts of all n keys, then their exclusive scan: the
        // first output slot of every digit
        s_base[threadIdx.x] = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += kSortThreads) atomicAdd(&s_base[((unsigned)ik[i] >> shift) & 0xFFu], 1u);
        __syncthreads();
        {
            unsigned tot;
            const unsigned c = s_base[threadIdx.x];
            const unsigned ex = block_scan_256(c, s_warp, &tot);
            s_base[threadIdx.x] = ex;
        }
        __syncthreads();
        // the tiles in order: each ranked stably, scattered after the
        // digits' earlier tiles
        for (int t0 = 0; t0 < n; t0 += kSortTile) {
            int key[kSortItems], val[kSortItems];
            unsigned rank[kSortItems];
            for (int d = lane; d < kRadix; d += 32) s_cnt[warp][d] = 0;
            __syncwarp();
#pragma unroll
            for (int r = 0; r < kSortItems; ++r) {
                const int i = t0 + wbase + r * 32 + lane;
                const bool ok = i < n;
                key[r] = ok ? ik[i] : 0;
                val[r] = ok ? iv[i] : 0;
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
            unsigned run = 0;
#pragma unroll
            for (int w = 0; w < kSortWarps; ++w) {
                const unsigned c = s_cnt[w][threadIdx.x];
                s_cnt[w][threadIdx.x] = run;
                run += c;
            }
            s_tile[threadIdx.x] = run;   // this tile's count of digit threadIdx.x
            __syncthreads();
#pragma unroll
            for (int r = 0; r < kSortItems; ++r) {
                if (t0 + wbase + r * 32 + lane >= n) continue;
                const unsigned d = ((unsigned)key[r] >> shift) & 0xFFu;
                const unsigned pos = s_base[d] + s_cnt[warp][d] + rank[r];
                ok_[pos] = key[r];
                ov_[pos] = val[r];
            }
            __syncthreads();
            s_base[threadIdx.x] += s_tile[threadIdx.x];
            __syncthreads();
        }
        // this pass's output is the next one's input: the CTA's writes are
        // visible to its own threads after the barrier above
    }
}

int radix_tiles(int n) { return (n + kSortTile - 1) / kSortTile; }
size_t radix_temp_words(int n) { return (size_t)kRadix * radix_tiles(n) + kRadix; }

// Sort pairs on `bits` low key bits from (in_k, in_v), which is read only by
// the first pass, ping-ponging through (a_k, a_v) and (b_k, b_v).  The count
// is n, or *d_n when d_n is given (n then bounds it).  Returns 0 when the
// result is in (a_k, a_v), 1 when it is in (b_k, b_v).
int radix_sort_pairs_n(const int* in_k, const int* in_v, int* a_k, int* a_v, int* b_k, int* b_v, int n,
                       const int* d_n, int bits, unsigned* temp, cudaStream_t s, bool one_cta) {
    if (n <= 0) return 0;
    if (bits <= 0) bits = 1;
    if (d_n && one_cta) {
        // one kernel whatever the count (no pass kernels in the stream)
        launch_after(k_radix_onecta, 1, kSortThreads, s, in_k, in_v, a_k, a_v, b_k, b_v, d_n, bits);
        return (((bits + 7) / 8) & 1) ? 0 : 1;
    }
    const int ntiles = radix_tiles(n);
    unsigned* totals = temp + (size_t)kRadix * ntiles;
    // a device-side count is usually far below n: a bounded grid strides
    // over the tiles that hold data
    const int grid = d_n ? (ntiles < 4 * 152 ? ntiles : 4 * 152) : ntiles;
    if (d_n) {
        // where the passes would leave the result: (a) after an odd number
        const int passes = (bits + 7) / 8;
        launch_after(k_radix_small, 1, kSortThreads, s, in_k, in_v, (passes & 1) ? a_k : b_k,
                     (passes & 1) ? a_v : b_v, d_n, bits);
    }
    int pass = 0;
    for (int shift = 0; shift < bits; shift += 8, ++pass) {
        const int* ki = pass == 0 ? in_k : ((pass & 1) ? a_k : b_k);
        const int* vi = pass == 0 ? in_v : ((pass & 1) ? a_v : b_v);
        int* ko = (pass & 1) ? b_k : a_k;
        int* vo = (pass & 1) ? b_v : a_v;
        // after the small sort (device-side count) or the previous pass
        if (d_n || pass > 0) launch_after(k_radix_upsweep, grid, kSortThreads, s, ki, n, d_n, shift, ntiles, temp);
        else k_radix_upsweep<<<grid, kSortThreads, 0, s>>>(ki, n, d_n, shift, ntiles, temp);
        launch_after(k_scan_rows, kRadix, kSortThreads, s, temp, ntiles, d_n, totals);
        launch_after(k_radix_downsweep, grid, kSortThreads, s, ki, vi, ko, vo, n, d_n, shift, ntiles,
                     (const unsigned*)temp, (const unsigned*)totals);
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
    return radix_sort_pairs_n(in_k, in_v, a_k, a_v, b_k, b_v, n, nullptr, bits, temp, s, false);
}

// ------------------------------------------------------------ incremental --
__device__ inline unsigned long long pack_pair(int key, int id) {
    return ((unsigned long long)(unsigned)key << 32) | (unsigned)id;
}

// The compaction kernels run 1 024 threads per 4 096-slot tile (two CTAs
// fill an SM): slot i of a tile belongs to warp (i % 4096) / 128, round
// (i % 128) / 32, lane i % 32, so each warp compacts its own 128 consecutive
// slots.
constexpr int kIncThreads = 1024;
constexpr int kIncWarps = kIncThreads / 32;            // 32
constexpr int kWarpSlots = kSortTile / kIncWarps;      // 128
constexpr int kWarpRounds = kWarpSlots / 32;           // 4

// Per warp of every 4096-slot tile, the pairs whose particle kept its key;
// the movers' particle ids are flagged and counted per 4096-id tile.
__global__ void __launch_bounds__(kIncThreads) k_inc_count(const int* __restrict__ old_k, const int* __restrict__ old_v,
                                                            const int* __restrict__ new_key_of, int n,
                                                            unsigned* __restrict__ warp_kept,
                                                            unsigned* __restrict__ tile_kept, unsigned char* moved,
                                                            unsigned* id_movers) {
    after_previous();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wbase = blockIdx.x * kSortTile + warp * kWarpSlots;
    unsigned kept = 0;
#pragma unroll
    for (int r = 0; r < kWarpRounds; ++r) {
        const int i = wbase + r * 32 + lane;
        bool keep = true;
        int id = 0;
        if (i < n) {
            id = old_v[i];
            keep = __ldg(&new_key_of[id]) == old_k[i];
        }
        kept += __popc(__ballot_sync(0xffffffffu, i < n && keep));
        if (!keep) {
            moved[id] = 1;
            // one atomic per id tile among the warp's movers
            const unsigned mask = __activemask();
            const unsigned peers = __match_any_sync(mask, id >> 12);
            if ((peers & ((1u << lane) - 1u)) == 0) atomicAdd(&id_movers[id >> 12], (unsigned)__popc(peers));
        }
    }
    __shared__ unsigned s_kept[kIncWarps];
    if (lane == 0) {
        warp_kept[blockIdx.x * kIncWarps + warp] = kept;
        s_kept[warp] = kept;
    }
    __syncthreads();
    if (warp == 0) {
        unsigned t = s_kept[lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) tile_kept[blockIdx.x] = t;
    }
}

// One CTA: exclusive scans of the per-tile kept counts (slot tiles) and of
// the per-id-tile mover counts (which it clears for the next build), side by
// side; the number of movers into *movers.
__global__ void __launch_bounds__(kSortThreads) k_inc_scan(const unsigned* __restrict__ tile_kept, int ntiles, int n,
                                                           unsigned* tile_base, unsigned* id_movers, unsigned* id_base,
                                                           int* movers, int* host_movers) {
    after_previous();
    __shared__ unsigned s_warp[2][kSortWarps];
    unsigned carry = 0, mcarry = 0;
    for (int base = 0; base < ntiles; base += kSortThreads) {
        const int i = base + threadIdx.x;
        const unsigned v = i < ntiles ? tile_kept[i] : 0u, w = i < ntiles ? id_movers[i] : 0u;
        unsigned tot, mtot;
        const unsigned ex = block_scan_256(v, s_warp[0], &tot);
        const unsigned mex = block_scan_256(w, s_warp[1], &mtot);
        if (i < ntiles) {
            tile_base[i] = carry + ex;
            id_base[i] = mcarry + mex;
            id_movers[i] = 0u;
        }
        carry += tot;
        mcarry += mtot;
    }
    if (threadIdx.x == 0) {
        *movers = n - (int)carry;
        if (host_movers) *host_movers = n - (int)carry;   // read by the host to pick the next frames' mover sort
    }
}

// The kept pairs in their old order (each warp from its offset).
__global__ void __launch_bounds__(kIncThreads) k_inc_split(const int* __restrict__ old_k, const int* __restrict__ old_v,
                                                            const int* __restrict__ new_key_of, int n,
                                                            const unsigned* __restrict__ warp_kept,
                                                            const unsigned* __restrict__ tile_base, int* kept_k,
                                                            int* kept_v) {
    after_previous();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wbase = blockIdx.x * kSortTile + warp * kWarpSlots;
    if (wbase >= n) return;
    // this warp's offset: the tile's, plus the kept counts of the warps before it
    const unsigned lt = (1u << lane) - 1u;
    unsigned before = lane < warp ? warp_kept[blockIdx.x * kIncWarps + lane] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) before += __shfl_xor_sync(0xffffffffu, before, o);
    unsigned off = tile_base[blockIdx.x] + before;
#pragma unroll
    for (int r = 0; r < kWarpRounds; ++r) {
        const int i = wbase + r * 32 + lane;
        int key = 0, id = 0;
        bool keep = false;
        if (i < n) {
            id = old_v[i];
            key = __ldg(&new_key_of[id]);
            keep = key == old_k[i];
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            kept_k[off + __popc(bal & lt)] = key;
            kept_v[off + __popc(bal & lt)] = id;
        }
        off += __popc(bal);
    }
}

// The movers in id order (keys: their new keys), from the flags, which it
// clears: one CTA per 4096 ids, 16 per thread.
__global__ void __launch_bounds__(kSortThreads) k_inc_movers(const int* __restrict__ new_key_of, int n,
                                                             uint4* moved, const unsigned* __restrict__ id_base,
                                                             int* mov_k, int* mov_v) {
    after_previous();
    __shared__ unsigned s_warp[kSortWarps];
    const int id0 = blockIdx.x * kSortTile + threadIdx.x * 16;
    uint4 f = make_uint4(0u, 0u, 0u, 0u);
    if (id0 < n) f = moved[id0 / 16];   // the flags are padded to whole tiles
    const unsigned w[4] = {f.x, f.y, f.z, f.w};
    unsigned cnt = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q)
        cnt += __popc(w[q] & 0x01010101u);
    unsigned tot;
    unsigned off = id_base[blockIdx.x] + block_scan_256(cnt, s_warp, &tot);
    if (cnt == 0) return;
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int b = 0; b < 4; ++b)
            if ((w[q] >> (8 * b)) & 1u) {
                const int id = id0 + 4 * q + b;
                mov_k[off] = __ldg(&new_key_of[id]);
                mov_v[off] = id;
                ++off;
            }
    moved[id0 / 16] = make_uint4(0u, 0u, 0u, 0u);
}

// Merge path: how many of the first `diag` outputs of merging sorted A (na)
// and B (nb) come from A (the pairs are distinct, so the split is unique).
template <class GetA, class GetB>
__device__ inline int merge_split(int diag, int na, int nb, GetA A, GetB B) {
    int lo = max(0, diag - nb), hi = min(diag, na);
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A(mid - 1) < B(diag - mid)) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// First index in [lo, hi) whose pair is not below x.
__device__ inline int pairs_below(const int* __restrict__ k, const int* __restrict__ v, int lo, int hi,
                                  unsigned long long x) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (pack_pair(__ldg(&k[mid]), __ldg(&v[mid])) < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Merge the kept pairs A (n - m, sorted) and the sorted movers B (m) by
// (key, id), into the same result by one of two methods chosen on the device:
//  * few movers (m <= n / 16): every pair's output index is its own index
//    plus the number of pairs of the other list below it.  CTAs [0, a_ctas)
//    place A, 2048 pairs each (thread t: pairs t, t + 256, ..., its count of
//    B found once and then advanced), so the writes stay coalesced; the other
//    CTAs place B, each mover by a binary search of A;
//  * otherwise a CTA of the first a_ctas makes 2048 consecutive outputs: its
//    two merge-path splits on global memory, its runs of A and B staged in
//    shared memory, each thread's 8 outputs merged there and the tile written
//    out coalesced.
constexpr int kMergeItems = 8;
constexpr int kMergeTile = kSortThreads * kMergeItems;
__global__ void __launch_bounds__(kSortThreads) k_inc_merge(const int* __restrict__ a_k, const int* __restrict__ a_v,
                                                            const int* __restrict__ b_k, const int* __restrict__ b_v,
                                                            int n, const int* __restrict__ movers, int a_ctas,
                                                            int* out_k, int* out_v) {
    after_previous();
    __shared__ unsigned long long s_in[kMergeTile];
    __shared__ int s_split[2];
    const int m = *movers, na = n - m, nb = m;
    if (m <= n / 16) {
        if ((int)blockIdx.x < a_ctas) {
            const int base = blockIdx.x * kMergeTile + threadIdx.x;
            int c = -1;
#pragma unroll 1
            for (int k = 0; k < kMergeItems; ++k) {
                const int i = base + k * kSortThreads;
                if (i >= na) break;
                const int key = a_k[i], id = a_v[i];
                const unsigned long long x = pack_pair(key, id);
                if (c < 0) {
                    c = pairs_below(b_k, b_v, 0, nb, x);
                } else {
                    int step = 0;
                    while (c < nb && step < 4 && pack_pair(__ldg(&b_k[c]), __ldg(&b_v[c])) < x) ++c, ++step;
                    if (step == 4) c = pairs_below(b_k, b_v, c, nb, x);
                }
                out_k[i + c] = key;
                out_v[i + c] = id;
            }
        } else {
            const int stride = (gridDim.x - a_ctas) * kSortThreads;
            for (int j = (blockIdx.x - a_ctas) * kSortThreads + threadIdx.x; j < nb; j += stride) {
                const int key = b_k[j], id = b_v[j];
                const int r = pairs_below(a_k, a_v, 0, na, pack_pair(key, id));
                out_k[j + r] = key;
                out_v[j + r] = id;
            }
        }
        return;
    }
    const int o0 = blockIdx.x * kMergeTile;
    if ((int)blockIdx.x >= a_ctas || o0 >= n) return;
    const int o1 = min(n, o0 + kMergeTile);
    if (threadIdx.x < 2) {
        auto A = [&](int i) { return pack_pair(__ldg(&a_k[i]), __ldg(&a_v[i])); };
        auto B = [&](int j) { return pack_pair(__ldg(&b_k[j]), __ldg(&b_v[j])); };
        s_split[threadIdx.x] = merge_split(threadIdx.x ? o1 : o0, na, nb, A, B);
    }
    __syncthreads();
    const int i0 = s_split[0], i1 = s_split[1];
    const int j0 = o0 - i0, la = i1 - i0, lb = (o1 - i1) - j0, len = la + lb;
    for (int q = threadIdx.x; q < len; q += kSortThreads)
        s_in[q] = q < la ? pack_pair(a_k[i0 + q], a_v[i0 + q]) : pack_pair(b_k[j0 + q - la], b_v[j0 + q - la]);
    __syncthreads();
    const int d = threadIdx.x * kMergeItems;
    unsigned long long out[kMergeItems];
    if (d < len) {
        auto A = [&](int i) { return s_in[i]; };
        auto B = [&](int j) { return s_in[la + j]; };
        int i = merge_split(d, la, lb, A, B), j = d - i;
#pragma unroll
        for (int k = 0; k < kMergeItems; ++k) {
            if (d + k >= len) break;
            const bool take_a = j >= lb || (i < la && s_in[i] < s_in[la + j]);
            out[k] = take_a ? s_in[i++] : s_in[la + j++];
        }
    }
    __syncthreads();
    if (d < len) {
#pragma unroll
        for (int k = 0; k < kMergeItems; ++k)
            if (d + k < len) s_in[d + k] = out[k];
    }
    __syncthreads();
    for (int q = threadIdx.x; q < len; q += kSortThreads) {
        const unsigned long long x = s_in[q];
        out_k[o0 + q] = (int)(unsigned)(x >> 32);
        out_v[o0 + q] = (int)(unsigned)x;
    }
}


// New sorted (out_k, out_v) from the previous frame's sorted (old_k, old_v)
// and the new keys by particle id.  Movers are gathered in id order, so one
// stable sort by key puts them in (key, id) order.  With `side` (and its
// fork / join events) the movers are gathered and sorted there, beside the
// compaction of the kept pairs on `s`.
void sort_grid_incremental(const int* old_k, const int* old_v, const int* new_key_of, int* out_k, int* out_v, int n,
                           int key_bits, int id_bits, const IncrementalBuffers& b, cudaStream_t s,
                           cudaStream_t side, cudaEvent_t fork, cudaEvent_t join) {
    (void)id_bits;
    if (n <= 0) return;
    const int ntiles = radix_tiles(n);
    k_inc_count<<<ntiles, kIncThreads, 0, s>>>(old_k, old_v, new_key_of, n, b.warp_kept, b.tile_kept, b.moved,
                                               b.id_movers);
    launch_after(k_inc_scan, 1, kSortThreads, s, (const unsigned*)b.tile_kept, ntiles, n, b.tile_base, b.id_movers,
                 b.id_base, b.movers, b.host_movers);
    cudaStream_t ms = s;
    if (side) {
        cudaEventRecord(fork, s);
        cudaStreamWaitEvent(side, fork, 0);
        ms = side;
    }
    k_inc_movers<<<ntiles, kSortThreads, 0, ms>>>(new_key_of, n, reinterpret_cast<uint4*>(b.moved), b.id_base,
                                                  b.mov_k, b.mov_v);
    const int w = radix_sort_pairs_n(b.mov_k, b.mov_v, b.t1_k, b.t1_v, b.mov_k, b.mov_v, n, b.movers, key_bits,
                                     b.temp, ms, b.one_cta);
    if (side) cudaEventRecord(join, side);
    launch_after(k_inc_split, ntiles, kIncThreads, s, old_k, old_v, new_key_of, n, (const unsigned*)b.warp_kept,
                 (const unsigned*)b.tile_base, b.kept_k, b.kept_v);
    if (side) cudaStreamWaitEvent(s, join, 0);
    const int* ms_k = w ? b.mov_k : b.t1_k;
    const int* ms_v = w ? b.mov_v : b.t1_v;
    const int a_ctas = (n + kMergeTile - 1) / kMergeTile;
    const int b_ctas = ntiles < 4 * 152 ? ntiles : 4 * 152;
    k_inc_merge<<<a_ctas + b_ctas, kSortThreads, 0, s>>>(b.kept_k, b.kept_v, ms_k, ms_v, n, b.movers, a_ctas, out_k,
                                                          out_v);
}

}  // namespace bcs
