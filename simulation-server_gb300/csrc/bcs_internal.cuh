// bcs_internal.cuh — device-side data layout and math shared by the kernels.
//
// A simulation holds one or more independent scenes (a batch).  Every scene
// keeps its own coordinates, so its FP32 arithmetic is the same as when it
// runs alone; the scenes share one set of buffers and one launch per kernel.
//
// HBM layout (batch of S scenes, N particles, V vein vertices, T triangles):
//   pos[2], vel[2], frc[2]   float4 x N each, ping-pong, scene-major.  pos.w
//                            carries the particle's collision radius, so a
//                            neighbour gather returns position and radius in
//                            one 16-byte load.
//   particle grid            keys live in one batch-wide key space: a scene's
//                            cell c has key key_offset(scene) + c, so one sort
//                            and one table serve every scene.
//   ptable                   int4 x (all scenes' cells): (first, last, epoch)
//                            of every occupied cell.  Never cleared: each grid
//                            build bumps the grid's epoch and rewrites exactly
//                            the occupied cells, so an entry is trusted only
//                            when its epoch is current; stale entries of
//                            emptied cells are rejected with no clear pass and
//                            no second, dependent load.
//   vpos, vvel, vfrc         float4 x V (all scenes' veins, scene-major)
//   vnb_ids[9], vnb_len[9]   int32 / float x V, the reference's nine
//                            neighbour-slot arrays (VeinNeighbors)
//   row_start                int32 per grid row (cy x cz rows of cx cells, all
//                            scenes) + 1: the first sorted slot whose key is in
//                            the row or after it; with the sorted keys it
//                            bounds a stencil row's slots without the table
//   coll                     float4 x N: each particle's collision force from
//                            the grid-order collision kernel
//   tkeys, tids, ttable      triangle grid, same representation as particles
//   tcache                   3 float4 per sorted triangle slot: (v0, id),
//                            (v1 - v0), (v2 - v0) — the Moller-Trumbore
//                            operands, streamed contiguously per grid cell.
//   tbox                     2 float4 per triangle-grid cell: bounds of the
//                            cell's triangles widened by the rebuild margin,
//                            for ray culling
//   tocc                     uint32 per triangle-grid cell: bit 9 (dx + 1) +
//                            3 (dy + 1) + (dz + 1) set when that stencil
//                            neighbour exists and holds triangles (rebuilt
//                            with the triangle grid)
//   wall_mask                uint8 per wall-mask cell: the mask epoch where a
//                            triangle lies within vein_impact_distance (plus
//                            the rebuild margin) of the cell's centre, widened
//                            by the cell's half-diagonal
//   scenes, types, work      per-scene geometry, per (scene, cell type) ranges,
//                            per-CTA work items (device arrays)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/bcs.h"

namespace bcs {

constexpr int kMaxChunk = 768;          // largest particles-per-CTA of any step shape
constexpr int kMaxCellsPerChunk = 64;
constexpr int kMaxEndings = 8;
constexpr int kPropagateThreads = 256;

// Launch shapes of the step kernel: threads per CTA, particles per CTA
// (whole cells, at most this many) and the CTAs per SM the register budget
// is sized for.  Every shape computes the same per-particle arithmetic.
struct StepShape {
    int threads, chunk, min_blocks;
};
constexpr int kStepShapes = 6;
constexpr StepShape kShapes[kStepShapes] = {
    {256, 512, 3}, {128, 256, 6}, {384, 768, 2}, {256, 512, 4}, {256, 512, 2}, {128, 256, 8}};

struct TypeDev {          // one cell type of one scene
    int count;            // cells
    int pic;              // particles per cell
    int particle_start;   // first particle (batch-wide)
    int cell_start;       // first cell within the scene (respawn counter)
    int cell_global;      // first cell, batch-wide
    int model_start;      // first model vertex in the per-model tables
    int adj_start;        // CSR offsets start for the model
    int scene;
};

struct WorkItem {         // one CTA of the step kernel: whole cells of one type
    int type;
    int first_cell;       // within the type
    int ncells;
};

struct GridGeom {         // one scene's uniform grid (uniform_grid.cu:83-104)
    float lo[3];          // minX, minY, minZ
    float hi[3];          // maxX, maxY, maxZ
    float ext[3];         // width, height, depth
    float cell[3];        // cell width, height, depth
    int cx, cy, cz;       // cell counts (int(extent / cell))
    long long cells;
    long long key_offset; // first key of the scene in the batch key space
    long long row_offset; // first grid row (cy * cz rows of cx cells) of the scene in the batch row space
};

struct MaskGeom {         // one scene's wall-proximity mask
    float lo[3];
    float inv_cell;
    int nx, ny, nz;
    long long offset;     // first byte of the scene in the mask array
};

struct SceneDev {
    GridGeom pg, tg;
    MaskGeom wall;
    float upper, lower, right, left, front, back;   // vein-end thresholds
    float cylinder_radius, min_spawn_y;
    unsigned seed_lo, seed_hi;
    int ending_count;
    float4 endings[kMaxEndings];                    // (cx, cy, cz, r)
    int flow_start, flow_count;
    int particle_start, particle_end;
    int tri_start, tri_end;
};

struct GridDev {          // batch-wide sorted grid
    int uniform;
    long long cells;      // table entries (all scenes)
    const int* keys;      // sorted keys
    const int* ids;       // sorted object ids
    const int4* table;    // (first, last, epoch) per cell
    const int* epoch;     // current epoch of the table
    const unsigned* occ;  // occupancy bitmap, 1 bit per cell, or null
    const float4* spos;   // positions in sorted order (particle grid), or null
    const float4* svel;   // velocities in sorted order (set with spos), or null
    const int* row_start; // particle grid, grid-order collisions: first sorted slot of each grid row
                          // (batch row space, one entry past the last row), or null
    const int4* tiles;    // with row_start: 3 int4 per block of 256 sorted slots, the collision
                          // kernel's tile record (k_tile_setup)
    int count;            // objects
};

struct StepArgs {
    // particle state
    const float4* __restrict__ pos_in;
    const float4* __restrict__ vel_in;
    const float4* __restrict__ frc_in;
    float4* pos_out;
    float4* vel_out;
    float4* frc_out;
    int* keys_out;        // next-step grid keys by particle id, or null (the ids beside them
                          // stay the identity the key kernel wrote once)
    float4* fext;         // macro steps: external force of sub-step 1 (held), or null
    const unsigned char* skip_cell;   // macro steps: cells the network advanced (k_substeps skips them), or null
    int n;
    // layout
    const WorkItem* work;
    int work_count;
    int* work_counter;    // persistent launches: next item, CTAs finished
    int* crowded;         // crowded particles off the grid's regular stencils, left to k_crowded (capacity n)
    int* crowded_cells;   // one particle per crowded grid cell, left to k_crowded (capacity n)
    int* crowded_counter; // [0] crowded entries, [1] CTAs of k_crowded finished, [2] crowded_cells entries,
                          // [3] particles of the listed cells taken, [4..5] 64-bit running total
    float4* cent;         // this step's cell centroids (batch-wide cell index), for k_crowded
    float4* coll;         // grid-order collisions: each particle's collision force, written by
                          // k_collide before the step kernel reads it; null: the step kernel
                          // searches the stencil itself
    int collide_search;   // grid-order collisions: 0 = linear scan of each row window, 1 = binary
                          // search, 2 = binary search on candidates staged in shared memory
    const TypeDev* types;
    int type_count;
    const SceneDev* scenes;
    int scene_count;
    const int* adj_off;   // CSR offsets per model vertex
    const int* adj_nbr;   // neighbour index within the cell
    const float* adj_len; // rest length
    const float* r0;      // per model vertex: distance to the model centroid
    const float4* respawn;// per model vertex: (m_i - m_0), for respawns
    // grids
    GridDev pg, tg;
    // vein
    const float4* vpos;
    float4* vfrc;
    const uint32_t* tri;  // 3 * T vertex indices (batch-wide)
    const float4* tcache; // 3 per sorted triangle slot
    const float4* tbox;   // 2 per triangle-grid cell
    const unsigned* tocc; // per triangle-grid cell: which of its 27 stencil cells hold triangles, or null
    const unsigned char* wall_mask;
    const int* wall_epoch;
    int T;
    const bcs_flow_segment* flows;
    // constants shared by all scenes
    bcs_params p;
    const long long* steps;  // device step counter
    unsigned* err;        // device error word
};

// The learned sub-step path: one entry per surrogate cell (cells of every
// type that shares the surrogate's cell model), and the normalisation of the
// network's inputs and outputs.
struct SurScales {
    float fm[16], fs[16];   // node features: mean, 1 / std
    float tm[9], ts[9];     // targets: mean, std
    float er, el, eu;       // edge scales: relative position, stretch, relative velocity
};

struct SurDev {
    const int* cell_type;   // per surrogate cell: type index
    const int* cell_index;  // per surrogate cell: cell within its type
    int cells, pic, K;
    float T;                // (K - 1) dt: the span the network covers
    float tolerance;        // residual threshold (length units)
    float* raw;             // [cells][pic][16] raw node features of sub-step 1's state
    float4* start;          // [cells][pic][3] x, v, F after sub-step 1
    unsigned char* skip;    // per blood cell (batch-wide): 1 = advanced by the network this macro step
    unsigned long long* counts;   // [0] cells predicted, [1] cells that fell back
};

// ------------------------------------------------------------- float3 ----
__host__ __device__ inline float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ inline float3 xyz(float4 a) { return make_float3(a.x, a.y, a.z); }
__host__ __device__ inline float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ inline float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__host__ __device__ inline float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline float3 cross3(float3 u, float3 v) {
    return f3(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
}
__host__ __device__ inline float len3(float3 v) { return sqrtf(dot3(v, v)); }

// v / |v|, or the zero vector (and a flag) when that is NaN — the rule of
// the reference's normalize (src/utilities/math.cuh:95-104).
__device__ inline float3 normalize_or_zero(float3 v, unsigned& e) {
    float s = sqrtf(dot3(v, v));
    float3 n = f3(v.x / s, v.y / s, v.z / s);
    if (isnan(n.x) || isnan(n.y) || isnan(n.z)) {
        e |= BCS_ERRW_NAN_NORMALIZE;
        return f3(0.f, 0.f, 0.f);
    }
    return n;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}
// Odd multiples of 2^-24 in (0, 1): exact in float.
__host__ __device__ inline float uniform_open(uint32_t r) {
    return (float)((r >> 9) * 2u + 1u) * (1.0f / 16777216.0f);
}

// Grid key of a position within its scene, FP32 arithmetic identical to
// calculateIdForCell (src/grids/uniform_grid.cu:24-36): per axis int(min(
// extent, max(0, (p - min) / cell))), then clamped to the last cell (the
// reference's extent clamp can step past it).  Out-of-box positions raise
// BCS_ERRW_OUT_OF_GRID.  The batch key adds the scene's key offset.
__device__ inline int axis_clamp(float t, float ext, int count) {
    float m = 0.0f > t ? 0.0f : t;
    float c = ext > m ? m : ext;
    int i = (int)c;
    i = i > count - 1 ? count - 1 : i;
    return i < 0 ? 0 : i;
}

// The per-axis quotient (p - min) / cell, FP32 IEEE division as in the
// reference; its truncation is also the stencil's unclamped cell coordinate.
__device__ inline float axis_quotient(float p, float lo, float cell) { return __fdiv_rn(p - lo, cell); }

__device__ inline int axis_index(float p, float lo, float ext, float cell, int count) {
    return axis_clamp(axis_quotient(p, lo, cell), ext, count);
}

// Scene-local key from the three quotients (same int arithmetic as local_key).
__device__ inline int key_of_quotients(const GridGeom& g, float tx, float ty, float tz) {
    return axis_clamp(tz, g.ext[2], g.cz) * g.cx * g.cy + axis_clamp(ty, g.ext[1], g.cy) * g.cx +
           axis_clamp(tx, g.ext[0], g.cx);
}

__device__ inline int local_key(const GridGeom& g, float3 q, unsigned& e) {
    if (q.x < g.lo[0] || q.x > g.hi[0] || q.y < g.lo[1] || q.y > g.hi[1] || q.z < g.lo[2] || q.z > g.hi[2])
        e |= BCS_ERRW_OUT_OF_GRID;
    int ix = axis_index(q.x, g.lo[0], g.ext[0], g.cell[0], g.cx);
    int iy = axis_index(q.y, g.lo[1], g.ext[1], g.cell[1], g.cy);
    int iz = axis_index(q.z, g.lo[2], g.ext[2], g.cell[2], g.cz);
    return iz * g.cx * g.cy + iy * g.cx + ix;
}

__device__ inline int grid_key(const GridGeom& g, float3 q, unsigned& e) {
    return (int)(g.key_offset + local_key(g, q, e));
}

// Lookup of an occupied cell's (first, last) sorted slots, cell given
// within the scene: valid only when the entry carries the current epoch.
__device__ inline bool cell_range(const GridDev& g, const GridGeom& geo, int epoch, long long c, int& first,
                                  int& last) {
    if (c < 0 || c >= geo.cells) return false;
    int4 r = __ldg(&g.table[geo.key_offset + c]);
    if (r.z != epoch) return false;
    first = r.x;
    last = r.y;
    return true;
}

// Index of the range holding `x` among `n` ascending starts (start_of(0) <= x).
template <class T, class F>
__device__ inline int find_range(int n, T x, F start_of) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (start_of(mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Scratch of the incremental grid sort (bcs_sort.cu), owned by the grid.
struct IncrementalBuffers {
    int* kept_k; int* kept_v;      // n each
    int* mov_k; int* mov_v;        // n each (movers; sorted in place through t1)
    int* t1_k; int* t1_v;          // n each
    unsigned* warp_kept;           // 32 per tile
    unsigned* tile_kept;           // per tile
    unsigned* tile_base;           // per tile
    unsigned* id_movers;           // per id tile, zero between builds
    unsigned* id_base;             // per id tile
    unsigned char* moved;          // 4096 per id tile, zero between builds
    unsigned* temp;                // radix_temp_words(n)
    int* movers;                   // 1
    int* host_movers;              // mapped host int the scan copies the mover count into, or null
    bool one_cta;                  // sort the movers with k_radix_onecta alone (no pass kernels)
};

// Programmatic dependent launch: a kernel launched with launch_after may be
// scheduled while the kernel before it in the stream finishes; it calls
// after_previous() before it touches memory that kernel (or anything before
// it) writes.  The wait returns once that kernel has completed and its writes
// are visible; in a kernel launched without the attribute it returns at once.
__device__ __forceinline__ void after_previous() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... Params, typename... Args>
inline void launch_after(void (*kernel)(Params...), unsigned grid, unsigned block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace bcs
