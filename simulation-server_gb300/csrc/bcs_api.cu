// bcs_api.cu — host side of the engine and the C ABI of include/bcs.h.
//
// Creation folds the runtime scene the way the reference's meta_factory folds
// its compile-time one (src/meta_factory/blood_cell_factory.hpp:172-328,
// src/meta_factory/vein_factory.hpp:21-174) and the way SimulationController
// derives its per-model tables (src/simulation/simulation_controller.cu:93-153),
// uploads everything once, and builds the static triangle grid.  The step
// then runs entirely on the handle's stream; bcs_step replays a captured
// CUDA graph of one frame.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <new>
#include <vector>

#include "bcs_internal.cuh"
#include "bcs_mpnn.cuh"

namespace bcs {
// bcs_kernels.cu
void launch_step(const StepArgs& a, int items, int mode, int shape, int persistent_grid, cudaStream_t s,
                 cudaEvent_t after_collisions = nullptr);
int step_persistent_grid(int mode, int shape);
void launch_gather_rows(const float4* src, const int* idx, int n, float4* out, cudaStream_t s);
void launch_propagate(const StepArgs& a, int blocks, cudaStream_t s);
void launch_keys(const float4* pos, int n, int uniform, const SceneDev* scenes, int scene_count, int* keys, int* ids,
                 unsigned* err, cudaStream_t s);
void launch_tri_keys(const float4* vpos, const uint32_t* tri, int T, const SceneDev* scenes, int scene_count,
                     int* keys, int* ids, cudaStream_t s);
void launch_cell_ranges(const int* keys, int n, int4* table, int* epoch, unsigned* occ, const int* ids,
                        const float4* pos, float4* spos, const float4* vel, float4* svel, cudaStream_t s);
void launch_occ_update(const int* keys, int n, unsigned* occ, bool set, cudaStream_t s);
void launch_row_starts(const int* keys, int n, const SceneDev* scenes, int scene_count, long long rows, int* row_start,
                       int4* tiles, cudaStream_t s);
int tile_records(int n);
void launch_tri_occupancy(const int4* table, const int* epoch, const SceneDev* scenes, int scene_count, long long cells,
                          unsigned* occ, cudaStream_t s);
void launch_dense_ranges(const int4* table, const int* epoch, long long cells, int* starts, int* ends,
                         cudaStream_t s);
void launch_vein_end(const StepArgs& a, int cells, cudaStream_t s);
void launch_tri_boxes(const int* keys, const int* ids, int T, const uint32_t* tri, const float4* vpos, float4* box,
                      const SceneDev* scenes, int scene_count, unsigned char* mask, float reach, int* mask_epoch,
                      float margin, float* disp2, float4* vref, int V, cudaStream_t s);
void launch_vein_springs(const float4* vpos, const float4* vvel, float4* vfrc, const int* nb_ids, const float* nb_len,
                         int V, float k, float d, unsigned* err, cudaStream_t s);
void launch_vein_integrate(float4* vpos, float4* vvel, float4* vfrc, int V, float dt, cudaStream_t s);
void launch_tri_cache(const int* ids, const uint32_t* tri, const float4* vpos, int T, float4* cache, cudaStream_t s);
void launch_bump_step(long long* steps, int by, cudaStream_t s);
void launch_substeps(const StepArgs& a, int items, int K, int chunk, cudaStream_t s);
void launch_sur_features(const StepArgs& a, const SurDev& d, cudaStream_t s);
void launch_sur_targets(const StepArgs& a, const SurDev& d, float* raw_t, unsigned char* valid, cudaStream_t s);
void launch_sur_inputs(const float* raw, const float* raw_t, const int* list, int nvalid, unsigned long long seed,
                       int first, int cells, int pic, const int* adj_off, const int* adj_nbr, const float* adj_len,
                       const SurScales& sc, float* f, float* E, float* T, cudaStream_t s);
void launch_sur_apply(const StepArgs& a, const SurDev& d, const float* Y, const SurScales& sc, int first, int cells,
                      cudaStream_t s);
bool launch_sur_fused(const StepArgs& a, const SurDev& d, const SurScales& sc, const float* P,
                      const __nv_bfloat16* PB, const __nv_bfloat16* PBT, const MpnnLayout& L, const int* goff,
                      const int* gnbr, const float* glen, int first, int cells, cudaStream_t s);
void launch_sur_eval(const float* Y, const float* raw_t, const unsigned char* valid, const SurScales& sc, int first,
                     int cells, int pic, double* sums, cudaStream_t s);
void launch_export(const float4* pos, int n, const float4* vpos, int V, float* pvbo, float* poff, float* vvbo,
                   cudaStream_t s);
void launch_pack(const float* x, const float* y, const float* z, int n, float4* out, const float* wsrc,
                 cudaStream_t s);
void launch_unpack(const float4* in, int n, float* x, float* y, float* z, cudaStream_t s);
void launch_init_reference(const StepArgs& a, float4* pos, float4* vel, float4* frc, const float4* model,
                           const float* radius, unsigned long long seed, cudaStream_t s);
void launch_lattice_sites(const SceneDev* scenes, int scene, float3 lo, int nx, int ny, int nz, float spacing,
                          float clear, float ymin, float ymax, const bcs_flow_segment* flows, unsigned long long seed,
                          int* keys, int* ids, int* valid_count, cudaStream_t s);
void launch_lattice_place(const StepArgs& a, int scene, int count, float4* pos, float4* vel, float4* frc,
                          const float4* model, const float* centroid, const float* radius, const int* site_ids,
                          float3 lo, int nx, int ny, float spacing, float sigma, unsigned long long seed,
                          cudaStream_t s);
// bcs_sort.cu
int radix_sort_pairs(const int* in_k, const int* in_v, int* a_k, int* a_v, int* b_k, int* b_v, int n, int bits,
                     unsigned* temp, cudaStream_t s);
size_t radix_temp_words(int n);
int radix_tiles(int n);
void sort_grid_incremental(const int* old_k, const int* old_v, const int* new_key_of, int* out_k, int* out_v, int n,
                           int key_bits, int id_bits, const IncrementalBuffers& b, cudaStream_t s,
                           cudaStream_t side, cudaEvent_t fork, cudaEvent_t join);
}  // namespace bcs

using namespace bcs;

namespace {

struct DeviceGrid {
    GridDev g{};           // geometry + pointers to the sorted result
    int* in_k = nullptr;   // unsorted keys / ids (written by the key kernels)
    int* in_v = nullptr;
    int* s_k[2] = {nullptr, nullptr};   // sorted results, alternating per build
    int* s_v[2] = {nullptr, nullptr};
    int slot = 0;          // s_*[slot] holds the current sorted result
    bool sorted_once = false;
    bool incremental = false;           // rebuild from the previous order
    IncrementalBuffers inc{};
    bool full_now = false;     // this build sorts all pairs from scratch even when incremental
    int4* table = nullptr;
    int* epoch = nullptr;
    unsigned* occ = nullptr;   // occupancy bitmap; while occ_on it holds the
    bool occ_on = false;       // bits of the cells of s_k[slot]
    float4* spos = nullptr;    // positions in sorted order, kept while spos_on
    float4* svel = nullptr;    // velocities in sorted order, with spos
    bool spos_on = false;
    bool table_on = true;      // every build writes the range table (off under grid-order collisions,
    bool table_current = false;// which need only the row starts; the getters then build it on demand)
    int* row_start = nullptr;  // first sorted slot of every grid row (+1 entry), kept while rows_on
    int4* tiles = nullptr;     // the collision kernel's tile records, built with row_start
    long long rows = 0;        // grid rows of all scenes
    bool rows_on = false;
    const SceneDev* scenes = nullptr;   // the batch's scenes (row geometry)
    int scene_count = 0;
    unsigned* temp = nullptr;
    int bits = 0;
    int id_bits = 0;
    int count = 0;
};

}  // namespace

struct bcs_sim {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bcs_params p{};
    int N = 0, C = 0, V = 0, T = 0;
    int S = 0;                   // scenes in the batch
    std::vector<TypeDev> types;
    std::vector<WorkItem> work_host;
    std::vector<SceneDev> scenes_host;
    bcs_tuning tune{0, 0, 0, 0, 0, 0, 0};
    float4* coll = nullptr;      // grid-order collision sums (float4 x N)
    int max_pic = 0;
    int work_capacity = 0;       // work items of the smallest shape
    int persistent_grid[2] = {0, 0};   // by mode, 0 until first needed
    int* work_counter = nullptr;
    int* crowded = nullptr;      // crowded-particle lists of the step kernel (N each)
    int* crowded_cells = nullptr;
    int* crowded_counter = nullptr;
    float4* cent = nullptr;      // cell centroids of the step (C)
    int* order_idx = nullptr;    // first particle per work item (spatial order)
    float4* order_pos = nullptr;
    std::vector<int> scene_cells;       // blood cells per scene
    std::vector<int> scene_cell_start;
    std::vector<int> scene_vertex_start, scene_vertex_count;
    size_t bytes = 0;
    std::vector<void*> allocations;
    // particle state
    float4* pos[2] = {nullptr, nullptr};
    float4* vel[2] = {nullptr, nullptr};
    float4* frc[2] = {nullptr, nullptr};
    float* radius_of_particle = nullptr;
    int cur = 0;
    bool mid_frame = false;      // between calculate_next_frame and propagate_all
    bool keys_valid = false;     // pgrid.in_k holds keys of pos[cur]
    bool grid_ready = false;
    // layout tables
    WorkItem* work = nullptr;
    TypeDev* types_dev = nullptr;
    SceneDev* scenes = nullptr;
    bcs_flow_segment* flows = nullptr;
    int* adj_off = nullptr;
    int* adj_nbr = nullptr;
    float* adj_len = nullptr;
    float* r0 = nullptr;
    float4* respawn = nullptr;
    // vein
    float4* vpos = nullptr;
    float4* vvel = nullptr;
    float4* vfrc = nullptr;
    int* nb_ids = nullptr;
    float* nb_len = nullptr;
    uint32_t* tri = nullptr;
    float4* tcache = nullptr;
    float4* tbox = nullptr;         // 2 per triangle-grid cell
    unsigned* tocc = nullptr;       // per triangle-grid cell: occupied stencil neighbours
    unsigned char* wall_mask = nullptr;
    int* wall_epoch = nullptr;
    float* wall_disp2 = nullptr;     // dynamic wall: max squared vertex move since the last bounds build
    float4* wall_ref = nullptr;      // vein positions at that build
    // grids
    DeviceGrid pg, tg;
    // misc
    long long* steps = nullptr;
    long long host_steps = 0;
    unsigned* err = nullptr;
    StepArgs args{};
    std::map<long long, cudaGraphExec_t> graphs;   // by (sub-steps, sort form, cur, sorted slot)
    // the incremental sort's mover count of a recent frame, written by its
    // scan kernel into mapped host memory (-1 until one was seen), and how the
    // grid is sorted: 0 = by that count, 1 = movers by the pass kernels,
    // 2 = movers by one CTA, 3 = every pair from scratch
    int* movers_seen = nullptr;
    int mover_sort = 0;
    // the automatic choice reads a count that is as old as the host's lead:
    // run_steps keeps it within kLeadFrames launched frames (event per frame)
    cudaEvent_t lead_ev[8] = {};
    long long frames_launched = 0;
    float4* fext = nullptr;      // macro steps: held external force per particle
    bcs_surrogate* surrogate = nullptr;   // enabled learned sub-step path, or null
    std::vector<bcs_surrogate*> surrogates;   // every live surrogate of this simulation
    // host copies of the per-model tables (surrogate graphs and tolerances)
    std::vector<int> h_adj_off, h_adj_nbr;
    std::vector<float> h_adj_len, h_radius_model;
    // scene start: absolute model vertices, per-type centroid and bounding
    // radius, per-scene vein box (min xyz, max xyz)
    float4* model = nullptr;
    float* type_centroid = nullptr;
    std::vector<float> h_type_bound, h_vein_box;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t pev[BCS_PHASE_COUNT + 1] = {};
    // a second stream for independent work within a frame (the vein springs
    // beside the grid build, the vein update beside the vein-end rule, the
    // row starts and tile records beside the sorted copies), forked and
    // joined with events
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev[4] = {}, join_ev[4] = {};
    float* scratch = nullptr;      // 3 * max(N, V) floats for host transfers
    int kernels_per_step = 0;
    // asynchronous reads of the particle state (bcs_get_particles_async):
    // two slots of 9 N floats, converted on `stream`, copied on `copy_stream`
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t aready[2] = {}, adone[2] = {};
    float* ascratch[2] = {};
    bool ainflight[2] = {};
    int aslot = 0;
};

namespace {

// A dynamic wall's triangle bounds and wall mask are rebuilt only when some
// vertex has moved more than this since the last build; they carry it as
// extra width, so they always contain the current triangles.
constexpr float kWallMargin = 0.5f;
constexpr int kDefaultShape = 3;

// A failed runtime call is reported once, by its own status: the runtime's
// last-error slot is cleared so that the next call's check does not report it
// again (a sticky error keeps failing every later call anyway).
#define BCS_CUDA(call)                                          \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) {                                \
            (void)cudaGetLastError();                           \
            return e_ == cudaErrorMemoryAllocation ? BCS_ERR_OUT_OF_MEMORY : BCS_ERR_CUDA; \
        }                                                       \
    } while (0)

// Device scratch of one call, freed on every return path.
struct ScopedDevice {
    void* p = nullptr;
    ScopedDevice() = default;
    ScopedDevice(const ScopedDevice&) = delete;
    ScopedDevice& operator=(const ScopedDevice&) = delete;
    ~ScopedDevice() {
        if (p) cudaFree(p);
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

template <class T>
bcs_status dalloc(bcs_sim* s, T** ptr, size_t count) {
    *ptr = nullptr;
    if (count == 0) count = 1;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, sizeof(T) * count);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? BCS_ERR_OUT_OF_MEMORY : BCS_ERR_CUDA;
    }
    s->allocations.push_back(p);
    s->bytes += sizeof(T) * count;
    *ptr = static_cast<T*>(p);
    return BCS_OK;
}

template <class T>
bcs_status upload(bcs_sim* s, T** ptr, const std::vector<T>& host) {
    bcs_status st = dalloc(s, ptr, host.size());
    if (st != BCS_OK) return st;
    // stream-ordered: the handle's stream does not wait for the legacy one
    if (!host.empty())
        BCS_CUDA(cudaMemcpyAsync(*ptr, host.data(), sizeof(T) * host.size(), cudaMemcpyHostToDevice, s->stream));
    return BCS_OK;
}

int bits_for(long long cells) {
    int b = 0;
    while (b < 31 && (1LL << b) < cells) ++b;
    return b;
}

bcs_status alloc_grid(bcs_sim* s, DeviceGrid& dg, int count, bool incremental) {
    dg.count = count;
    dg.g.count = count;
    dg.incremental = incremental;
    bcs_status st;
    if ((st = dalloc(s, &dg.in_k, count)) || (st = dalloc(s, &dg.in_v, count)) ||
        (st = dalloc(s, &dg.s_k[0], count)) || (st = dalloc(s, &dg.s_v[0], count)) ||
        (st = dalloc(s, &dg.s_k[1], count)) || (st = dalloc(s, &dg.s_v[1], count)) ||
        (st = dalloc(s, &dg.inc.t1_k, count)) || (st = dalloc(s, &dg.inc.t1_v, count)) ||
        (st = dalloc(s, &dg.temp, radix_temp_words(count))))
        return st;
    dg.inc.temp = dg.temp;
    if (incremental) {
        const int tiles = radix_tiles(count);
        if ((st = dalloc(s, &dg.inc.kept_k, count)) || (st = dalloc(s, &dg.inc.kept_v, count)) ||
            (st = dalloc(s, &dg.inc.mov_k, count)) || (st = dalloc(s, &dg.inc.mov_v, count)) ||
            (st = dalloc(s, &dg.inc.warp_kept, 32 * (size_t)tiles)) || (st = dalloc(s, &dg.inc.tile_kept, tiles)) ||
            (st = dalloc(s, &dg.inc.tile_base, tiles)) ||
            (st = dalloc(s, &dg.inc.id_movers, tiles)) || (st = dalloc(s, &dg.inc.id_base, tiles)) ||
            (st = dalloc(s, &dg.inc.moved, 4096 * (size_t)tiles)) || (st = dalloc(s, &dg.inc.movers, 1)))
            return st;
        // mover flags and counts are zero between builds
        BCS_CUDA(cudaMemsetAsync(dg.inc.id_movers, 0, sizeof(unsigned) * tiles, s->stream));
        BCS_CUDA(cudaMemsetAsync(dg.inc.moved, 0, 4096 * (size_t)tiles, s->stream));
    }
    int idb = 0;
    while (idb < 31 && (1LL << idb) < count) ++idb;
    dg.id_bits = idb;
    if ((st = dalloc(s, &dg.epoch, 1))) return st;
    BCS_CUDA(cudaMemsetAsync(dg.epoch, 0, sizeof(int), s->stream));
    dg.g.epoch = dg.epoch;
    if (dg.g.uniform) {
        if ((st = dalloc(s, &dg.table, (size_t)dg.g.cells))) return st;
        // every field -1: no entry matches an epoch before the grid's first build
        BCS_CUDA(cudaMemsetAsync(dg.table, 0xFF, sizeof(int4) * (size_t)dg.g.cells, s->stream));
        if (incremental) {
            const size_t words = (size_t)((dg.g.cells + 31) / 32);
            if ((st = dalloc(s, &dg.occ, words)) || (st = dalloc(s, &dg.spos, count)) ||
                (st = dalloc(s, &dg.svel, count)))
                return st;
            BCS_CUDA(cudaMemsetAsync(dg.occ, 0, sizeof(unsigned) * words, s->stream));
        }
    }
    dg.bits = bits_for(dg.g.cells);
    return BCS_OK;
}

// Sort the grid's unsorted keys into the other result slot and rebuild the
// range table.  After the first build, a grid flagged incremental starts
// from the previous order (any permutation works; few movers make it cheap).
// With `side` (and its fork / join events) the row starts and the collision
// tile records are built there, beside the sorted copies on `st`, and
// (fork2 / join2) an incremental build's movers are sorted there beside the
// compaction of the kept pairs.  dg.full_now sorts an incremental grid from
// scratch for this build (late in a trajectory most particles move).
void sort_grid(DeviceGrid& dg, cudaStream_t st, const float4* pos = nullptr, const float4* vel = nullptr,
               cudaStream_t side = nullptr, cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr,
               cudaEvent_t fork2 = nullptr, cudaEvent_t join2 = nullptr) {
    const int out = dg.slot ^ 1;
    if (dg.incremental && dg.sorted_once && !dg.full_now) {
        sort_grid_incremental(dg.s_k[dg.slot], dg.s_v[dg.slot], dg.in_k, dg.s_k[out], dg.s_v[out], dg.count, dg.bits,
                              dg.id_bits, dg.inc, st, side, side ? fork2 : nullptr, side ? join2 : nullptr);
    } else {
        // the full sort's result lands in its first ping-pong buffer after an
        // odd number of passes (or none), in the second after an even number
        const int passes = (dg.bits + 7) / 8;
        const bool first = passes == 0 || dg.count <= 1 || (passes & 1);
        radix_sort_pairs(dg.in_k, dg.in_v, first ? dg.s_k[out] : dg.inc.t1_k, first ? dg.s_v[out] : dg.inc.t1_v,
                         first ? dg.inc.t1_k : dg.s_k[out], first ? dg.inc.t1_v : dg.s_v[out], dg.count, dg.bits,
                         dg.temp, st);
    }
    // the previous build's cells leave the bitmap before the new ones enter
    if (dg.occ_on && dg.sorted_once) launch_occ_update(dg.s_k[dg.slot], dg.count, dg.occ, false, st);
    dg.slot = out;
    dg.sorted_once = true;
    dg.g.keys = dg.s_k[dg.slot];
    dg.g.ids = dg.s_v[dg.slot];
    dg.g.table = dg.table;
    dg.g.occ = dg.occ_on ? dg.occ : nullptr;
    dg.g.spos = dg.spos_on && pos ? dg.spos : nullptr;
    dg.g.svel = dg.spos_on && pos && vel ? dg.svel : nullptr;
    float4* svel_out = dg.spos_on && pos && vel ? dg.svel : nullptr;
    const bool beside = dg.rows_on && side;
    if (beside) {
        cudaEventRecord(fork, st);
        cudaStreamWaitEvent(side, fork, 0);
        launch_row_starts(dg.g.keys, dg.count, dg.scenes, dg.scene_count, dg.rows, dg.row_start, dg.tiles, side);
        cudaEventRecord(join, side);
    }
    launch_cell_ranges(dg.g.keys, dg.count, dg.table_on ? dg.table : nullptr, dg.epoch,
                       dg.occ_on && dg.table_on ? dg.occ : nullptr, dg.g.ids, pos, dg.spos_on && pos ? dg.spos : nullptr,
                       vel, svel_out, st);
    dg.table_current = dg.table_on;
    if (beside) cudaStreamWaitEvent(st, join, 0);
    else if (dg.rows_on)
        launch_row_starts(dg.g.keys, dg.count, dg.scenes, dg.scene_count, dg.rows, dg.row_start, dg.tiles, st);
    dg.g.row_start = dg.rows_on ? dg.row_start : nullptr;
    dg.g.tiles = dg.rows_on ? dg.tiles : nullptr;
}

// The range table of the current sorted keys, when the last build left it
// out (grid-order collisions need only the row starts).
void ensure_table(DeviceGrid& dg, cudaStream_t st) {
    if (dg.table_current || !dg.sorted_once || !dg.table) return;
    launch_cell_ranges(dg.g.keys, dg.count, dg.table, dg.epoch, dg.occ_on ? dg.occ : nullptr, dg.g.ids, nullptr,
                       nullptr, nullptr, nullptr, st);
    dg.table_current = true;
}

void refresh_args(bcs_sim* s, int in, int out, bool write_keys) {
    StepArgs& a = s->args;
    a.pos_in = s->pos[in];
    a.vel_in = s->vel[in];
    a.frc_in = s->frc[in];
    a.pos_out = s->pos[out];
    a.vel_out = s->vel[out];
    a.frc_out = s->frc[out];
    a.keys_out = write_keys ? s->pg.in_k : nullptr;
    a.pg = s->pg.g;
    // grid-order collisions once the grid carries its row starts and sorted copies
    a.coll = s->pg.rows_on && a.pg.row_start && a.pg.spos && a.pg.svel ? s->coll : nullptr;
    a.tg = s->tg.g;
    a.tcache = s->tcache;
    a.tbox = s->tbox;
    a.tocc = s->tocc;
    a.wall_mask = s->wall_mask;
    a.wall_epoch = s->wall_epoch;
}

// Triangle grid, Moller-Trumbore cache, per-cell triangle bounds and the
// wall-proximity mask from the current vein positions.
void build_triangle_grid(bcs_sim* s, bool regrid) {
    if (s->T == 0) return;
    if (s->tg.g.uniform) {
        if (regrid) {
            launch_tri_keys(s->vpos, s->tri, s->T, s->scenes, s->S, s->tg.in_k, s->tg.in_v, s->stream);
            sort_grid(s->tg, s->stream);
            if (s->tocc)
                launch_tri_occupancy(s->tg.table, s->tg.epoch, s->scenes, s->S, s->tg.g.cells, s->tocc, s->stream);
        }
        launch_tri_cache(s->tg.g.ids, s->tri, s->vpos, s->T, s->tcache, s->stream);
        launch_tri_boxes(s->tg.g.keys, s->tg.g.ids, s->T, s->tri, s->vpos, s->tbox, s->scenes, s->S, s->wall_mask,
                         s->p.vein_impact_distance * 1.001f + 1e-3f, s->wall_epoch,
                         s->wall_disp2 ? kWallMargin : 0.0f, s->wall_disp2, s->wall_ref, s->V, s->stream);
    } else {
        launch_tri_cache(nullptr, s->tri, s->vpos, s->T, s->tcache, s->stream);
    }
}

// ≙ main.cu:175-176.
void enqueue_grids(bcs_sim* s) {
    if (!s->keys_valid) {
        launch_keys(s->pos[s->cur], s->N, s->pg.g.uniform, s->scenes, s->S, s->pg.in_k, s->pg.in_v, s->err, s->stream);
        s->keys_valid = true;
    }
    if (s->pg.g.uniform)
        sort_grid(s->pg, s->stream, s->pos[s->cur], s->vel[s->cur], s->side, s->fork_ev[0], s->join_ev[0],
                  s->fork_ev[3], s->join_ev[3]);
    if (s->p.refresh_triangle_centers) build_triangle_grid(s, true);
    s->grid_ready = true;
}

void enqueue_vein_forces(bcs_sim* s) {
    if (s->p.vein_dynamic && s->V > 0)
        launch_vein_springs(s->vpos, s->vvel, s->vfrc, s->nb_ids, s->nb_len, s->V, s->p.vein_k_sniff, s->p.vein_d_fact,
                            s->err, s->stream);
}

void enqueue_vein_propagate(bcs_sim* s, bool bump = true) {
    if (s->p.vein_dynamic && s->V > 0) {
        launch_vein_integrate(s->vpos, s->vvel, s->vfrc, s->V, s->p.dt, s->stream);
        build_triangle_grid(s, false);
    }
    if (bump) launch_bump_step(s->steps, 1, s->stream);
}

// Work enqueued while it lives goes to the side stream, after everything
// enqueued on the main stream so far (fork event k); join() makes the main
// stream wait for it (join event k).
struct OnSide {
    bcs_sim* s;
    cudaStream_t main;
    int k;
    OnSide(bcs_sim* sim, int slot) : s(sim), main(sim->stream), k(slot) {
        cudaEventRecord(s->fork_ev[k], main);
        cudaStreamWaitEvent(s->side, s->fork_ev[k], 0);
        s->stream = s->side;
    }
    ~OnSide() {
        cudaEventRecord(s->join_ev[k], s->side);
        s->stream = main;
    }
    static void join(bcs_sim* sim, int slot) { cudaStreamWaitEvent(sim->stream, sim->join_ev[slot], 0); }
};

// One fused frame on the stream (no host synchronisation).  With `ev`, an
// event is recorded before each phase and after the last one.
void enqueue_frame(bcs_sim* s, cudaEvent_t* ev = nullptr) {
    if (ev) cudaEventRecord(ev[0], s->stream);
    // The vein springs read only the vein and add into its forces: they run
    // beside the grid build and end before the step kernel adds its impacts.
    const bool vein = s->p.vein_dynamic && s->V > 0;
    if (vein) {
        OnSide side(s, 1);
        enqueue_vein_forces(s);
    }
    enqueue_grids(s);
    if (ev) cudaEventRecord(ev[1], s->stream);
    if (vein) OnSide::join(s, 1);
    else enqueue_vein_forces(s);
    if (ev) cudaEventRecord(ev[2], s->stream);
    const int in = s->cur, out = s->cur ^ 1;
    refresh_args(s, in, out, true);
    launch_step(s->args, (int)s->work_host.size(), 0, s->tune.step_shape, s->persistent_grid[0], s->stream,
                ev ? ev[3] : nullptr);
    // The vein update (integration, triangle operands for the next frame)
    // runs beside the vein-end rule, which touches only particles.
    if (vein) {
        OnSide side(s, 2);
        enqueue_vein_propagate(s, false);
    }
    if (s->p.use_blood_flow) launch_vein_end(s->args, s->C, s->stream);
    if (ev) cudaEventRecord(ev[4], s->stream);
    if (vein) OnSide::join(s, 2);
    launch_bump_step(s->steps, 1, s->stream);   // after the vein-end rule, which reads the counter
    if (ev) cudaEventRecord(ev[5], s->stream);
    s->cur = out;
    s->keys_valid = true;    // k_step wrote keys of the new positions
    ++s->host_steps;
}

// Points where the learned sub-step path joins a macro step: after sub-step 1
// (the state in the output buffers, the held force in fext) and after
// sub-steps 2..K.
struct MacroHooks {
    void (*after_first)(bcs_sim*) = nullptr;
    void (*after_substeps)(bcs_sim*) = nullptr;
};

// One multi-rate macro step of K sub-steps (K >= 2): sub-step 1 is the
// fused frame, which also records each particle's external force (collisions
// and the vein's force adjustment); sub-steps 2..K re-integrate cell springs
// and environment with that force held (k_substeps), the vein mesh takes K
// sub-steps with the particle impacts in the first, and the step counter
// advances by K.
const MacroHooks* inference_hooks(bcs_sim* s, int K);

void enqueue_macro(bcs_sim* s, int K, const MacroHooks* hooks = nullptr) {
    if (!hooks) hooks = inference_hooks(s, K);
    enqueue_grids(s);
    enqueue_vein_forces(s);
    const int in = s->cur, out = s->cur ^ 1;
    refresh_args(s, in, out, false);
    s->args.fext = s->fext;
    launch_step(s->args, (int)s->work_host.size(), 0, s->tune.step_shape, s->persistent_grid[0], s->stream);
    if (s->p.use_blood_flow) launch_vein_end(s->args, s->C, s->stream);
    refresh_args(s, in, out, true);
    if (hooks && hooks->after_first) hooks->after_first(s);
    launch_substeps(s->args, (int)s->work_host.size(), K, kShapes[s->tune.step_shape].chunk, s->stream);
    if (hooks && hooks->after_substeps) hooks->after_substeps(s);
    s->args.fext = nullptr;
    s->args.skip_cell = nullptr;
    if (s->p.vein_dynamic && s->V > 0) {
        for (int k = 1; k <= K; ++k) {
            if (k > 1)
                launch_vein_springs(s->vpos, s->vvel, s->vfrc, s->nb_ids, s->nb_len, s->V, s->p.vein_k_sniff,
                                    s->p.vein_d_fact, s->err, s->stream);
            launch_vein_integrate(s->vpos, s->vvel, s->vfrc, s->V, s->p.dt, s->stream);
        }
        build_triangle_grid(s, false);
    }
    launch_bump_step(s->steps, K, s->stream);
    s->cur = out;
    s->keys_valid = true;
    s->host_steps += K;
}

bcs_status check_last() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? BCS_ERR_OUT_OF_MEMORY : BCS_ERR_CUDA;
    return BCS_OK;
}

void drop_graphs(bcs_sim* s) {
    for (auto& kv : s->graphs)
        if (kv.second) cudaGraphExecDestroy(kv.second);
    s->graphs.clear();
}

bcs_status validate(const bcs_scene_desc* d) {
    if (!d || d->type_count <= 0 || !d->types) return BCS_ERR_INVALID_ARGUMENT;
    long long n = 0;
    for (int t = 0; t < d->type_count; ++t) {
        const bcs_cell_type& c = d->types[t];
        if (c.count < 0 || c.particles_in_cell <= 0 || !c.vertices) return BCS_ERR_INVALID_ARGUMENT;
        if (c.particles_in_cell > kMaxChunk) return BCS_ERR_UNSUPPORTED;
        if (c.spring_count < 0 || (c.spring_count > 0 && (!c.springs || !c.spring_lengths)))
            return BCS_ERR_INVALID_ARGUMENT;
        for (int k = 0; k < 2 * c.spring_count; ++k)
            if (c.springs[k] < 0 || c.springs[k] >= c.particles_in_cell) return BCS_ERR_INVALID_ARGUMENT;
        n += (long long)c.count * c.particles_in_cell;
    }
    if (n <= 0 || n > INT32_MAX / 2) return BCS_ERR_INVALID_ARGUMENT;
    const bcs_vein& v = d->vein;
    if (v.vertex_count <= 0 || !v.positions || v.triangle_count < 0 || (v.triangle_count > 0 && !v.indices))
        return BCS_ERR_INVALID_ARGUMENT;
    for (long long k = 0; k < 3LL * v.triangle_count; ++k)
        if (v.indices[k] >= (uint32_t)v.vertex_count) return BCS_ERR_INVALID_ARGUMENT;
    if (v.ending_count < 0 || v.ending_count > kMaxEndings ||
        (v.ending_count > 0 && (!v.ending_centers || !v.ending_radii)))
        return BCS_ERR_INVALID_ARGUMENT;
    if (d->flow_segment_count < 0 || (d->flow_segment_count > 0 && !d->flow_segments))
        return BCS_ERR_INVALID_ARGUMENT;
    const bcs_params& p = d->params;
    if (!(p.cell_width > 0 && p.cell_height > 0 && p.cell_depth > 0 && p.cell_width_triangles > 0 &&
          p.cell_height_triangles > 0 && p.cell_depth_triangles > 0 && p.bounding_spheres_coeff != 0))
        return BCS_ERR_INVALID_ARGUMENT;
    return BCS_OK;
}

// Scenes of one batch share every physics constant; grid cell sizes,
// margins, respawn spread and height and the seed may differ per scene.
bool same_physics(const bcs_params& a, const bcs_params& b) {
    bcs_params x = a, y = b;
    for (bcs_params* q : {&x, &y}) {
        q->cell_width = q->cell_height = q->cell_depth = 0;
        q->cell_width_triangles = q->cell_height_triangles = q->cell_depth_triangles = 0;
        q->grid_y_margin = q->grid_xz_margin = 0;
        q->cylinder_radius = q->min_spawn_y = 0;
        q->seed = 0;
    }
    return std::memcmp(&x, &y, sizeof(bcs_params)) == 0;
}

// One scene's uniform grid over its vein's bounds (vein_factory.hpp:21-86,
// uniform_grid.cu:83-104), FP32 like the reference's constexpr floats.
bcs_status scene_grid(const float* mn, const float* mx, const bcs_params& p, float cw, float ch, float cd, bool uniform,
                      GridGeom& g) {
    g.lo[0] = mn[0] - p.grid_xz_margin; g.hi[0] = mx[0] + p.grid_xz_margin;
    g.lo[1] = mn[1] - p.grid_y_margin;  g.hi[1] = mx[1] + p.grid_y_margin;
    g.lo[2] = mn[2] - p.grid_xz_margin; g.hi[2] = mx[2] + p.grid_xz_margin;
    for (int k = 0; k < 3; ++k) g.ext[k] = g.hi[k] - g.lo[k];
    g.cell[0] = cw; g.cell[1] = ch; g.cell[2] = cd;
    g.cx = (int)(g.ext[0] / cw); g.cy = (int)(g.ext[1] / ch); g.cz = (int)(g.ext[2] / cd);
    g.cells = (long long)g.cx * g.cy * g.cz;
    if (uniform && (g.cx < 1 || g.cy < 1 || g.cz < 1 || g.cells > INT32_MAX)) return BCS_ERR_INVALID_ARGUMENT;
    if (!uniform) g.cells = 0;
    return BCS_OK;
}

// Work items of the step kernel for one shape: whole cells of one type, at
// most the shape's particles per CTA and kMaxCellsPerChunk cells.
std::vector<WorkItem> work_items(const std::vector<TypeDev>& types, int chunk) {
    std::vector<WorkItem> w;
    for (int t = 0; t < (int)types.size(); ++t) {
        const TypeDev& td = types[t];
        const int per = std::max(1, std::min(kMaxCellsPerChunk, chunk / td.pic));
        for (int c0 = 0; c0 < td.count; c0 += per) w.push_back(WorkItem{t, c0, std::min(per, td.count - c0)});
    }
    return w;
}

// Brick coordinate of a position for the spatial work order (non-finite
// values sort last).
long long brick(float v) {
    if (!std::isfinite(v)) return std::numeric_limits<long long>::max();
    return (long long)std::floor((double)v / 8.0);
}

// Reorder the work items by scene, then by the brick of their first
// particle (y, x, z), from the current positions.
bcs_status order_work_spatially(bcs_sim* s) {
    const int n = (int)s->work_host.size();
    if (n == 0) return BCS_OK;
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) {
        const WorkItem& w = s->work_host[i];
        const TypeDev& t = s->types[w.type];
        idx[i] = t.particle_start + w.first_cell * t.pic;
    }
    BCS_CUDA(cudaMemcpyAsync(s->order_idx, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s->stream));
    launch_gather_rows(s->pos[s->cur], s->order_idx, n, s->order_pos, s->stream);
    std::vector<float4> q(n);
    BCS_CUDA(cudaMemcpyAsync(q.data(), s->order_pos, sizeof(float4) * n, cudaMemcpyDeviceToHost, s->stream));
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    struct Key {
        int scene;
        long long y, x, z;
        int item;
    };
    std::vector<Key> k(n);
    for (int i = 0; i < n; ++i)
        k[i] = Key{s->types[s->work_host[i].type].scene, brick(q[i].y), brick(q[i].x), brick(q[i].z), i};
    std::stable_sort(k.begin(), k.end(), [](const Key& a, const Key& b) {
        if (a.scene != b.scene) return a.scene < b.scene;
        if (a.y != b.y) return a.y < b.y;
        if (a.x != b.x) return a.x < b.x;
        return a.z < b.z;
    });
    std::vector<WorkItem> w(n);
    for (int i = 0; i < n; ++i) w[i] = s->work_host[k[i].item];
    s->work_host.swap(w);
    return BCS_OK;
}

bcs_status upload_work(bcs_sim* s) {
    BCS_CUDA(cudaStreamSynchronize(s->stream));   // earlier frames may still read the table
    BCS_CUDA(cudaMemcpyAsync(s->work, s->work_host.data(), sizeof(WorkItem) * s->work_host.size(),
                             cudaMemcpyHostToDevice, s->stream));
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    s->args.work = s->work;
    s->args.work_count = (int)s->work_host.size();
    s->args.work_counter = s->work_counter;
    return BCS_OK;
}

bool tuning_valid(const bcs_sim* s, const bcs_tuning& t) {
    return t.step_shape >= 0 && t.step_shape < kStepShapes && kShapes[t.step_shape].chunk >= s->max_pic &&
           (t.persistent == 0 || t.persistent == 1) && (t.spatial_order == 0 || t.spatial_order == 1) &&
           (t.full_sort == 0 || t.full_sort == 1) && (t.occupancy_filter == 0 || t.occupancy_filter == 1) &&
           (t.sorted_positions == 0 || t.sorted_positions == 1) && t.grid_collisions >= 0 && t.grid_collisions <= 3;
}

bcs_status apply_tuning(bcs_sim* s, const bcs_tuning& t) {
    if (!tuning_valid(s, t)) return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    s->tune = t;
    s->work_host = work_items(s->types, kShapes[t.step_shape].chunk);
    bcs_status st;
    if (t.spatial_order && (st = order_work_spatially(s))) return st;
    if ((st = upload_work(s))) return st;
    s->pg.incremental = !t.full_sort;
    const bool occ = t.occupancy_filter && s->pg.occ;
    if (occ && !s->pg.occ_on) {
        // start the bitmap from the current sorted cells
        BCS_CUDA(cudaMemsetAsync(s->pg.occ, 0, sizeof(unsigned) * (size_t)((s->pg.g.cells + 31) / 32), s->stream));
        if (s->pg.sorted_once) launch_occ_update(s->pg.s_k[s->pg.slot], s->pg.count, s->pg.occ, true, s->stream);
        BCS_CUDA(cudaStreamSynchronize(s->stream));
    }
    s->pg.occ_on = occ;
    s->pg.g.occ = occ ? s->pg.occ : nullptr;
    // grid-order collisions read the sorted copies and the row-start table
    const bool gc = t.grid_collisions && s->pg.g.uniform && s->pg.row_start && s->coll;
    const bool sp = (t.sorted_positions || gc) && s->pg.spos;
    if (sp && !s->pg.spos_on && s->pg.sorted_once) {
        launch_gather_rows(s->pos[s->cur], s->pg.s_v[s->pg.slot], s->pg.count, s->pg.spos, s->stream);
        launch_gather_rows(s->vel[s->cur], s->pg.s_v[s->pg.slot], s->pg.count, s->pg.svel, s->stream);
    }
    if (gc && !s->pg.rows_on && s->pg.sorted_once)
        launch_row_starts(s->pg.g.keys, s->pg.count, s->pg.scenes, s->pg.scene_count, s->pg.rows, s->pg.row_start,
                          s->pg.tiles, s->stream);
    s->pg.spos_on = sp;
    s->pg.g.spos = sp && s->pg.sorted_once ? s->pg.spos : nullptr;
    s->pg.g.svel = sp && s->pg.sorted_once ? s->pg.svel : nullptr;
    s->pg.rows_on = gc;
    s->pg.table_on = !gc;
    if (!gc) ensure_table(s->pg, s->stream);
    s->pg.g.row_start = gc && s->pg.sorted_once ? s->pg.row_start : nullptr;
    s->pg.g.tiles = gc && s->pg.sorted_once ? s->pg.tiles : nullptr;
    s->args.pg = s->pg.g;
    s->args.coll = gc && s->pg.g.row_start && s->pg.g.spos && s->pg.g.svel ? s->coll : nullptr;
    s->args.collide_search = t.grid_collisions >= 2 ? t.grid_collisions - 1 : 0;
    s->persistent_grid[0] = t.persistent ? step_persistent_grid(0, t.step_shape) : 0;
    s->persistent_grid[1] = t.persistent ? step_persistent_grid(1, t.step_shape) : 0;
    drop_graphs(s);
    return check_last();
}

bcs_status create_impl(const bcs_scene_desc* descs, int scene_count, void* stream, bcs_sim* s) {
    bcs_status st;
    s->p = descs[0].params;
    s->S = scene_count;
    BCS_CUDA(cudaGetDevice(&s->device));
    if (stream) {
        s->stream = static_cast<cudaStream_t>(stream);
    } else {
        BCS_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->own_stream = true;
    }
    BCS_CUDA(cudaEventCreate(&s->ev0));
    BCS_CUDA(cudaEventCreate(&s->ev1));
    for (auto& e : s->pev) BCS_CUDA(cudaEventCreate(&e));
    BCS_CUDA(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
    for (int k = 0; k < 4; ++k) {
        BCS_CUDA(cudaEventCreateWithFlags(&s->fork_ev[k], cudaEventDisableTiming));
        BCS_CUDA(cudaEventCreateWithFlags(&s->join_ev[k], cudaEventDisableTiming));
    }
    const bool puniform = s->p.particle_grid == BCS_GRID_UNIFORM;
    const bool tuniform = s->p.triangle_grid == BCS_GRID_UNIFORM;

    std::vector<int> adj_off, adj_nbr;
    std::vector<float> adj_len, r0, radius_model, centroids;
    std::vector<float4> model_abs;
    std::vector<float4> respawn, vpos;
    std::vector<uint32_t> tri;
    std::vector<int> nb_ids;
    std::vector<float> nb_len;
    std::vector<bcs_flow_segment> flows;
    std::vector<int> nb_scene_ids[9];
    std::vector<float> nb_scene_len[9];
    long long key_total = 0, tkey_total = 0, mask_total = 0, row_total = 0;
    int pstart = 0, mstart = 0, cglobal = 0;
    for (int si = 0; si < scene_count; ++si) {
        const bcs_scene_desc* d = descs + si;
        const bcs_params& sp = d->params;
        SceneDev sd{};
        sd.particle_start = pstart;
        // ---- cell types: offsets, CSR springs, radii (blood_cell_factory.hpp:172-328,
        //      simulation_controller.cu:93-153)
        int cstart = 0;
        for (int t = 0; t < d->type_count; ++t) {
            const bcs_cell_type& c = d->types[t];
            const int pic = c.particles_in_cell;
            TypeDev td{c.count, pic, pstart, cstart, cglobal, mstart, (int)adj_off.size(), si};
            // Dense graph with the reference's rules: later springs overwrite
            // earlier ones, a rest length of 0 is "no spring".
            std::vector<float> dense((size_t)pic * pic, 0.0f);
            for (int k = 0; k < c.spring_count; ++k) {
                int a = c.springs[2 * k], b = c.springs[2 * k + 1];
                dense[(size_t)a * pic + b] = c.spring_lengths[k];
                dense[(size_t)b * pic + a] = c.spring_lengths[k];
            }
            for (int i = 0; i < pic; ++i) {
                adj_off.push_back((int)adj_nbr.size());
                for (int j = 0; j < pic; ++j) {
                    float L = dense[(size_t)j * pic + i];
                    if (L == 0.0f || j == i) continue;   // a self spring contributes exactly 0
                    adj_nbr.push_back(j);
                    adj_len.push_back(L);
                }
            }
            adj_off.push_back((int)adj_nbr.size());
            const float* m = c.vertices;
            float cx = 0, cy = 0, cz = 0;
            for (int j = 0; j < pic; ++j) {
                float best = std::numeric_limits<float>::max();
                for (int k = 0; k < pic; ++k) {
                    if (j == k) continue;
                    double len = std::sqrt(std::pow((double)(m[3 * j] - m[3 * k]), 2) +
                                           std::pow((double)(m[3 * j + 1] - m[3 * k + 1]), 2) +
                                           std::pow((double)(m[3 * j + 2] - m[3 * k + 2]), 2)) /
                                 (2 * (double)sp.bounding_spheres_coeff);
                    if (len < best) best = (float)len;
                }
                radius_model.push_back(c.collision_radius ? c.collision_radius[j] : best);
                cx += m[3 * j]; cy += m[3 * j + 1]; cz += m[3 * j + 2];
            }
            cx /= pic; cy /= pic; cz /= pic;
            float bound = 0.f;
            for (int j = 0; j < pic; ++j) {
                float dx = m[3 * j] - cx, dy = m[3 * j + 1] - cy, dz = m[3 * j + 2] - cz;
                r0.push_back(sqrtf(dx * dx + dy * dy + dz * dz));
                bound = std::max(bound, r0.back());
                respawn.push_back(make_float4(m[3 * j] - m[0], m[3 * j + 1] - m[1], m[3 * j + 2] - m[2], 0.f));
                model_abs.push_back(make_float4(m[3 * j], m[3 * j + 1], m[3 * j + 2], 0.f));
            }
            centroids.push_back(cx); centroids.push_back(cy); centroids.push_back(cz);
            s->h_type_bound.push_back(bound);
            s->types.push_back(td);
            s->max_pic = std::max(s->max_pic, pic);
            pstart += c.count * pic;
            cstart += c.count;
            cglobal += c.count;
            mstart += pic;
        }
        sd.particle_end = pstart;
        s->scene_cells.push_back(cstart);
        s->scene_cell_start.push_back(cglobal - cstart);

        // ---- vein: bounds (vein_factory.hpp:21-86), neighbours (:130-174)
        const bcs_vein& vn = d->vein;
        const int v0 = (int)vpos.size();
        s->scene_vertex_start.push_back(v0);
        s->scene_vertex_count.push_back(vn.vertex_count);
        sd.tri_start = (int)(tri.size() / 3);
        for (int i = 0; i < vn.vertex_count; ++i)
            vpos.push_back(make_float4(vn.positions[3 * i], vn.positions[3 * i + 1], vn.positions[3 * i + 2], 0.f));
        for (long long k = 0; k < 3LL * vn.triangle_count; ++k) tri.push_back(vn.indices[k] + (uint32_t)v0);
        sd.tri_end = (int)(tri.size() / 3);
        float mn[3] = {vn.positions[0], vn.positions[1], vn.positions[2]}, mx[3] = {mn[0], mn[1], mn[2]};
        for (int i = 1; i < vn.vertex_count; ++i)
            for (int k = 0; k < 3; ++k) {
                mn[k] = std::min(mn[k], vn.positions[3 * i + k]);
                mx[k] = std::max(mx[k], vn.positions[3 * i + k]);
            }
        for (int k = 0; k < 3; ++k) s->h_vein_box.push_back(mn[k]);
        for (int k = 0; k < 3; ++k) s->h_vein_box.push_back(mx[k]);
        if ((st = scene_grid(mn, mx, sp, sp.cell_width, sp.cell_height, sp.cell_depth, puniform, sd.pg)) ||
            (st = scene_grid(mn, mx, sp, sp.cell_width_triangles, sp.cell_height_triangles, sp.cell_depth_triangles,
                             tuniform, sd.tg)))
            return st;
        sd.pg.key_offset = key_total;
        sd.tg.key_offset = tkey_total;
        sd.pg.row_offset = row_total;
        row_total += (long long)sd.pg.cy * sd.pg.cz;
        key_total += sd.pg.cells;
        tkey_total += sd.tg.cells;
        // Wall-proximity mask, cells of half the impact distance (1..8).
        const float mc = std::min(8.0f, std::max(1.0f, sp.vein_impact_distance * 0.5f));
        sd.wall.lo[0] = sd.pg.lo[0]; sd.wall.lo[1] = sd.pg.lo[1]; sd.wall.lo[2] = sd.pg.lo[2];
        sd.wall.inv_cell = 1.0f / mc;
        sd.wall.nx = (int)std::ceil(sd.pg.ext[0] / mc) + 1;
        sd.wall.ny = (int)std::ceil(sd.pg.ext[1] / mc) + 1;
        sd.wall.nz = (int)std::ceil(sd.pg.ext[2] / mc) + 1;
        sd.wall.offset = mask_total;
        mask_total += (long long)sd.wall.nx * sd.wall.ny * sd.wall.nz;
        // vein_end.cu:12-17, FP32 like the constexpr thresholds.
        sd.upper = sd.pg.hi[1] - 3 * sp.grid_y_margin / 4;
        sd.lower = sd.pg.lo[1] + sp.grid_y_margin / 2;
        sd.right = sd.pg.hi[0] - sp.grid_xz_margin / 2;
        sd.left = sd.pg.lo[0] + sp.grid_xz_margin / 2;
        sd.front = sd.pg.hi[2] - sp.grid_xz_margin / 2;
        sd.back = sd.pg.lo[2] + sp.grid_xz_margin / 2;
        sd.cylinder_radius = sp.cylinder_radius;
        sd.min_spawn_y = sp.min_spawn_y;
        sd.seed_lo = (unsigned)sp.seed;
        sd.seed_hi = (unsigned)(sp.seed >> 32);
        sd.ending_count = vn.ending_count;
        for (int k = 0; k < vn.ending_count; ++k)
            sd.endings[k] = make_float4(vn.ending_centers[3 * k], vn.ending_centers[3 * k + 1],
                                        vn.ending_centers[3 * k + 2], vn.ending_radii[k]);
        sd.flow_start = (int)flows.size();
        sd.flow_count = d->flow_segment_count;
        for (int k = 0; k < d->flow_segment_count; ++k) flows.push_back(d->flow_segments[k]);
        // Vein neighbours: both other vertices of every triangle, sorted
        // ascending, the first nine kept, FP32 rest lengths.
        std::vector<std::vector<uint32_t>> nb(vn.vertex_count);
        for (int t = 0; t < vn.triangle_count; ++t) {
            uint32_t i0 = vn.indices[3 * t], i1 = vn.indices[3 * t + 1], i2 = vn.indices[3 * t + 2];
            nb[i0].push_back(i1); nb[i0].push_back(i2);
            nb[i1].push_back(i0); nb[i1].push_back(i2);
            nb[i2].push_back(i0); nb[i2].push_back(i1);
        }
        for (int k = 0; k < 9; ++k) {
            nb_scene_ids[k].resize(v0 + vn.vertex_count, -1);
            nb_scene_len[k].resize(v0 + vn.vertex_count, -1.0f);
        }
        for (int i = 0; i < vn.vertex_count; ++i) {
            std::sort(nb[i].begin(), nb[i].end());
            for (size_t k = 0; k < std::min<size_t>(nb[i].size(), 9); ++k) {
                uint32_t j = nb[i][k];
                float dx = vn.positions[3 * i] - vn.positions[3 * j];
                float dy = vn.positions[3 * i + 1] - vn.positions[3 * j + 1];
                float dz = vn.positions[3 * i + 2] - vn.positions[3 * j + 2];
                float l = sqrtf(dx * dx + dy * dy + dz * dz);
                nb_scene_ids[k][v0 + i] = (int)j + v0;
                nb_scene_len[k][v0 + i] = l < 0 ? -l : l;
            }
        }
        s->scenes_host.push_back(sd);
    }
    s->N = pstart;
    s->C = cglobal;
    s->V = (int)vpos.size();
    s->T = (int)(tri.size() / 3);
    if (key_total > INT32_MAX || tkey_total > INT32_MAX) return BCS_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < 9; ++k) {
        nb_ids.insert(nb_ids.end(), nb_scene_ids[k].begin(), nb_scene_ids[k].end());
        nb_len.insert(nb_len.end(), nb_scene_len[k].begin(), nb_scene_len[k].end());
    }
    s->h_adj_off = adj_off;
    s->h_adj_nbr = adj_nbr;
    s->h_adj_len = adj_len;
    s->h_radius_model = radius_model;
    std::vector<float> radius_particle(s->N);
    for (const TypeDev& td : s->types)
        for (int i = 0; i < td.count * td.pic; ++i)
            radius_particle[td.particle_start + i] = radius_model[td.model_start + i % td.pic];
    s->pg.g.uniform = puniform;
    s->pg.g.cells = key_total;
    s->tg.g.uniform = tuniform;
    s->tg.g.cells = tkey_total;

    // ---- device buffers
    for (int b = 0; b < 2; ++b)
        if ((st = dalloc(s, &s->pos[b], s->N)) || (st = dalloc(s, &s->vel[b], s->N)) ||
            (st = dalloc(s, &s->frc[b], s->N)))
            return st;
    if ((st = dalloc(s, &s->fext, s->N))) return st;
    BCS_CUDA(cudaMemsetAsync(s->fext, 0, sizeof(float4) * s->N, s->stream));
    for (int b = 0; b < 2; ++b) {
        BCS_CUDA(cudaMemsetAsync(s->pos[b], 0, sizeof(float4) * s->N, s->stream));
        BCS_CUDA(cudaMemsetAsync(s->vel[b], 0, sizeof(float4) * s->N, s->stream));
        BCS_CUDA(cudaMemsetAsync(s->frc[b], 0, sizeof(float4) * s->N, s->stream));
    }
    for (int k = 0; k < kStepShapes; ++k)
        s->work_capacity = std::max(s->work_capacity, (int)work_items(s->types, kShapes[k].chunk).size());
    if ((st = dalloc(s, &s->work, s->work_capacity)) || (st = dalloc(s, &s->order_idx, s->work_capacity)) ||
        (st = dalloc(s, &s->order_pos, s->work_capacity)) || (st = dalloc(s, &s->work_counter, 2)) ||
        (st = dalloc(s, &s->crowded, s->N)) || (st = dalloc(s, &s->crowded_cells, s->N)) ||
        (st = dalloc(s, &s->crowded_counter, 6)) || (st = dalloc(s, &s->cent, s->C)))
        return st;
    BCS_CUDA(cudaMemsetAsync(s->work_counter, 0, 2 * sizeof(int), s->stream));
    BCS_CUDA(cudaMemsetAsync(s->crowded_counter, 0, 6 * sizeof(int), s->stream));
    s->args.crowded = s->crowded;
    s->args.crowded_cells = s->crowded_cells;
    s->args.crowded_counter = s->crowded_counter;
    s->args.cent = s->cent;
    if ((st = upload(s, &s->radius_of_particle, radius_particle)) ||
        (st = upload(s, &s->types_dev, s->types)) || (st = upload(s, &s->scenes, s->scenes_host)) ||
        (st = upload(s, &s->adj_off, adj_off)) || (st = upload(s, &s->adj_nbr, adj_nbr)) ||
        (st = upload(s, &s->adj_len, adj_len)) || (st = upload(s, &s->r0, r0)) ||
        (st = upload(s, &s->respawn, respawn)) || (st = upload(s, &s->flows, flows)) ||
        (st = upload(s, &s->model, model_abs)) || (st = upload(s, &s->type_centroid, centroids)))
        return st;
    if ((st = upload(s, &s->vpos, vpos)) || (st = dalloc(s, &s->vvel, s->V)) || (st = dalloc(s, &s->vfrc, s->V)) ||
        (st = upload(s, &s->nb_ids, nb_ids)) || (st = upload(s, &s->nb_len, nb_len)) || (st = upload(s, &s->tri, tri)) ||
        (st = dalloc(s, &s->tcache, 3 * (size_t)s->T)))
        return st;
    BCS_CUDA(cudaMemsetAsync(s->vvel, 0, sizeof(float4) * s->V, s->stream));
    BCS_CUDA(cudaMemsetAsync(s->vfrc, 0, sizeof(float4) * s->V, s->stream));
    if ((st = alloc_grid(s, s->pg, s->N, true)) || (st = alloc_grid(s, s->tg, std::max(1, s->T), false))) return st;
    {
        int* dev = nullptr;
        if (cudaHostAlloc((void**)&s->movers_seen, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer((void**)&dev, s->movers_seen, 0) != cudaSuccess) {
            (void)cudaGetLastError();
            return BCS_ERR_CUDA;
        }
        *s->movers_seen = -1;
        s->pg.inc.host_movers = dev;
    }
    if (s->pg.g.uniform) {
        // grid-order collisions: the row-start table and the collision sums
        s->pg.rows = row_total;
        s->pg.scenes = s->scenes;
        s->pg.scene_count = s->S;
        if ((st = dalloc(s, &s->pg.row_start, (size_t)row_total + 1)) || (st = dalloc(s, &s->coll, s->N)) ||
            (st = dalloc(s, &s->pg.tiles, 3 * (size_t)tile_records(s->N))))
            return st;
    }
    s->tg.count = s->T;
    s->tg.g.count = s->T;
    if (tuniform) {
        if ((st = dalloc(s, &s->tbox, 2 * (size_t)std::max(1LL, tkey_total))) ||
            (st = dalloc(s, &s->tocc, (size_t)std::max(1LL, tkey_total))))
            return st;
        if (s->p.vein_dynamic && s->T > 0) {
            if ((st = dalloc(s, &s->wall_disp2, 1)) || (st = dalloc(s, &s->wall_ref, s->V))) return st;
            const float huge = 3.0e38f;
            BCS_CUDA(cudaMemcpyAsync(s->wall_disp2, &huge, sizeof(float), cudaMemcpyHostToDevice, s->stream));
        }
        if (s->T > 0 && mask_total <= (1LL << 31)) {
            if ((st = dalloc(s, &s->wall_mask, (size_t)mask_total)) || (st = dalloc(s, &s->wall_epoch, 1))) return st;
            BCS_CUDA(cudaMemsetAsync(s->wall_mask, 0, (size_t)mask_total, s->stream));
            BCS_CUDA(cudaMemsetAsync(s->wall_epoch, 0, sizeof(int), s->stream));
        }
    }
    if ((st = dalloc(s, &s->steps, 1)) || (st = dalloc(s, &s->err, 1))) return st;
    BCS_CUDA(cudaMemsetAsync(s->steps, 0, sizeof(long long), s->stream));
    BCS_CUDA(cudaMemsetAsync(s->err, 0, sizeof(unsigned), s->stream));

    // ---- kernel arguments that never change
    StepArgs& a = s->args;
    a.n = s->N;
    a.types = s->types_dev;
    a.type_count = (int)s->types.size();
    a.scenes = s->scenes;
    a.scene_count = s->S;
    a.adj_off = s->adj_off;
    a.adj_nbr = s->adj_nbr;
    a.adj_len = s->adj_len;
    a.r0 = s->r0;
    a.respawn = s->respawn;
    a.vpos = s->vpos;
    a.vfrc = s->vfrc;
    a.tri = s->tri;
    a.T = s->T;
    a.flows = s->flows;
    a.p = s->p;
    a.steps = s->steps;
    a.err = s->err;

    // ---- static triangle grid from the initial mesh
    build_triangle_grid(s, true);
    if ((st = check_last())) return st;
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    // ---- default launch: 256 threads / 512 particles / 4 CTAs per SM (the
    // fastest shape at the 4.2M-particle bifurcation), else the first shape
    // that holds the largest cell
    bcs_tuning t{kDefaultShape, 0, 0, 0, 0, 0, 3};
    if (kShapes[t.step_shape].chunk < s->max_pic) {
        t.step_shape = 0;
        while (kShapes[t.step_shape].chunk < s->max_pic) ++t.step_shape;
    }
    return apply_tuning(s, t);
}

void detach_surrogates(bcs_sim* s);

void destroy_impl(bcs_sim* s) {
    detach_surrogates(s);
    drop_graphs(s);
    if (s->stream) cudaStreamSynchronize(s->stream);
    // reads still in flight copy out of device scratch: finish them first
    if (s->copy_stream) {
        cudaStreamSynchronize(s->copy_stream);
        cudaStreamDestroy(s->copy_stream);
    }
    for (void* p : s->allocations) cudaFree(p);
    if (s->movers_seen) cudaFreeHost(s->movers_seen);
    for (auto& e : s->lead_ev)
        if (e) cudaEventDestroy(e);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    for (auto& e : s->pev)
        if (e) cudaEventDestroy(e);
    if (s->side) {
        cudaStreamSynchronize(s->side);
        cudaStreamDestroy(s->side);
    }
    for (int k = 0; k < 4; ++k) {
        if (s->fork_ev[k]) cudaEventDestroy(s->fork_ev[k]);
        if (s->join_ev[k]) cudaEventDestroy(s->join_ev[k]);
    }
    for (int k = 0; k < 2; ++k) {
        if (s->aready[k]) cudaEventDestroy(s->aready[k]);
        if (s->adone[k]) cudaEventDestroy(s->adone[k]);
    }
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
}

bool bad_vec(const bcs_vec3& v) { return !v.x || !v.y || !v.z; }

bcs_status ensure_scratch(bcs_sim* s) {
    if (s->scratch) return BCS_OK;
    return dalloc(s, &s->scratch, 3 * (size_t)std::max(s->N, s->V));
}

// Copy three SoA arrays (host or device) into a float4 buffer.  Host arrays
// are copied by DMA into a device scratch (fast when they are pinned) and
// packed on the device.
bcs_status set_vec(bcs_sim* s, const bcs_vec3& v, int n, float4* dst, const float* wsrc, bcs_memory where) {
    if (where == BCS_MEM_DEVICE) {
        launch_pack(v.x, v.y, v.z, n, dst, wsrc, s->stream);
        return check_last();
    }
    bcs_status st = ensure_scratch(s);
    if (st != BCS_OK) return st;
    const size_t b = sizeof(float) * (size_t)n;
    BCS_CUDA(cudaMemcpyAsync(s->scratch, v.x, b, cudaMemcpyHostToDevice, s->stream));
    BCS_CUDA(cudaMemcpyAsync(s->scratch + n, v.y, b, cudaMemcpyHostToDevice, s->stream));
    BCS_CUDA(cudaMemcpyAsync(s->scratch + 2 * (size_t)n, v.z, b, cudaMemcpyHostToDevice, s->stream));
    launch_pack(s->scratch, s->scratch + n, s->scratch + 2 * (size_t)n, n, dst, wsrc, s->stream);
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    return check_last();
}

bcs_status get_vec(bcs_sim* s, const float4* src, int n, const bcs_vec3& v, bcs_memory where) {
    if (!v.x && !v.y && !v.z) return BCS_OK;
    if (where == BCS_MEM_DEVICE) {
        launch_unpack(src, n, v.x, v.y, v.z, s->stream);
        return check_last();
    }
    bcs_status st = ensure_scratch(s);
    if (st != BCS_OK) return st;
    float* d[3] = {s->scratch, s->scratch + n, s->scratch + 2 * (size_t)n};
    launch_unpack(src, n, v.x ? d[0] : nullptr, v.y ? d[1] : nullptr, v.z ? d[2] : nullptr, s->stream);
    const size_t b = sizeof(float) * (size_t)n;
    if (v.x) BCS_CUDA(cudaMemcpyAsync(v.x, d[0], b, cudaMemcpyDeviceToHost, s->stream));
    if (v.y) BCS_CUDA(cudaMemcpyAsync(v.y, d[1], b, cudaMemcpyDeviceToHost, s->stream));
    if (v.z) BCS_CUDA(cudaMemcpyAsync(v.z, d[2], b, cudaMemcpyDeviceToHost, s->stream));
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    return check_last();
}

}  // namespace

// ================================================================ C ABI ====
// ------------------------------------------------- learned sub-steps ----
struct bcs_surrogate {
    bcs_sim* sim = nullptr;
    int K = 8;
    float tolerance = 0.f;
    int cells = 0, pic = 0, model_type = 0;
    std::vector<int> cell_type, cell_index;
    int *d_cell_type = nullptr, *d_cell_index = nullptr;
    MpnnNet net;
    float* raw = nullptr;              // features of the current macro step
    float4* start = nullptr;
    unsigned char* skip = nullptr;     // per blood cell of the simulation
    unsigned long long* counts = nullptr;
    // training set
    int capacity = 0, stored = 0, nvalid = 0;
    float *ds_raw = nullptr, *ds_t = nullptr;
    unsigned char* ds_valid = nullptr;
    int* valid_list = nullptr;
    bool collecting = false, enabled = false, scales_set = false;
    int mode = 1;                      // 1: fused inference kernel, 2: layer-by-layer kernels
    SurScales scales{};
    unsigned long long seed = 0, draws = 0;
    long long iterations = 0;
    float last_loss = 0.f;
    int infer_cells = 0;               // cells per inference chunk
    std::vector<void*> allocs;
    size_t bytes = 0;
    ~bcs_surrogate() {
        for (void* p : allocs) cudaFree(p);
    }
    template <class T>
    bool alloc(T** p, size_t n) {
        void* q = nullptr;
        if (cudaMalloc(&q, sizeof(T) * std::max<size_t>(1, n)) != cudaSuccess) {
            (void)cudaGetLastError();
            return false;
        }
        allocs.push_back(q);
        bytes += sizeof(T) * n;
        *p = static_cast<T*>(q);
        return true;
    }
    SurDev dev(float* raw_to) const {
        SurDev d{};
        d.cell_type = d_cell_type;
        d.cell_index = d_cell_index;
        d.cells = cells;
        d.pic = pic;
        d.K = K;
        d.T = (float)(K - 1) * sim->p.dt;
        d.tolerance = tolerance;
        d.raw = raw_to;
        d.start = start;
        d.skip = skip;
        d.counts = counts;
        return d;
    }
};

namespace {
// A surrogate outlives its simulation only as a handle to destroy: every
// other call on it is refused.
void detach_surrogates(bcs_sim* s) {
    for (bcs_surrogate* z : s->surrogates) z->sim = nullptr;
    s->surrogates.clear();
    s->surrogate = nullptr;
}

bool live(const bcs_surrogate* z) { return z && z->sim; }

void collect_after_first(bcs_sim* s) {
    bcs_surrogate* z = s->surrogate;
    launch_sur_features(s->args, z->dev(z->ds_raw + (size_t)z->stored * z->pic * 16), s->stream);
}
void collect_after_substeps(bcs_sim* s) {
    bcs_surrogate* z = s->surrogate;
    launch_sur_targets(s->args, z->dev(nullptr), z->ds_t + (size_t)z->stored * z->pic * 9,
                       z->ds_valid + z->stored, s->stream);
}
void infer_after_first(bcs_sim* s) {
    bcs_surrogate* z = s->surrogate;
    launch_sur_features(s->args, z->dev(z->raw), s->stream);
    if (z->mode == 1 && launch_sur_fused(s->args, z->dev(z->raw), z->scales, z->net.params(), z->net.weights_bf16(),
                                         z->net.weights_bf16_t(), z->net.layout(), z->net.dev_adj_off(),
                                         z->net.dev_adj_nbr(), z->net.dev_adj_len(), 0, z->cells, s->stream)) {
        s->args.skip_cell = z->skip;
        return;
    }
    for (int first = 0; first < z->cells; first += z->infer_cells) {
        const int n = std::min(z->infer_cells, z->cells - first);
        launch_sur_inputs(z->raw, nullptr, nullptr, 0, 0, first, n, z->pic, z->net.dev_adj_off(), z->net.dev_adj_nbr(),
                          z->net.dev_adj_len(), z->scales, z->net.input_buf(), z->net.edge_buf(), nullptr, s->stream);
        z->net.forward(z->net.input_buf(), z->net.edge_buf(), n, false);
        launch_sur_apply(s->args, z->dev(z->raw), z->net.output(), z->scales, first, n, s->stream);
    }
    s->args.skip_cell = z->skip;
}
const MacroHooks kCollectHooks{collect_after_first, collect_after_substeps};
const MacroHooks kInferHooks{infer_after_first, nullptr};

// Means and spreads of the network's inputs and targets over (a sample of)
// the training set.
bcs_status compute_scales(bcs_surrogate* z) {
    // a strided sample of up to 4096 samples over the whole training set
    const int n = std::min(z->stored, 4096);
    if (n <= 0) return BCS_ERR_INVALID_ARGUMENT;
    const long long stride = std::max(1, z->stored / n);
    const size_t fs_cell = (size_t)z->pic * 16, ts_cell = (size_t)z->pic * 9;
    std::vector<float> f((size_t)n * fs_cell), t((size_t)n * ts_cell);
    std::vector<unsigned char> ok(n);
    for (int c = 0; c < n; ++c) {
        const long long src = (long long)c * stride;
        BCS_CUDA(cudaMemcpy(&f[c * fs_cell], z->ds_raw + src * fs_cell, sizeof(float) * fs_cell, cudaMemcpyDeviceToHost));
        BCS_CUDA(cudaMemcpy(&t[c * ts_cell], z->ds_t + src * ts_cell, sizeof(float) * ts_cell, cudaMemcpyDeviceToHost));
        BCS_CUDA(cudaMemcpy(&ok[c], z->ds_valid + src, 1, cudaMemcpyDeviceToHost));
    }
    double fs[16] = {}, fq[16] = {}, ts[9] = {}, tq[9] = {}, rq = 0, uq = 0, lq = 0;
    long long nodes = 0, edges = 0;
    const std::vector<int>& off = z->sim->h_adj_off;
    const std::vector<int>& nbr = z->sim->h_adj_nbr;
    const std::vector<float>& len = z->sim->h_adj_len;
    const int a0 = z->sim->types[z->model_type].adj_start;
    auto len_k = [&](int k) { return (double)len[k]; };
    for (int c = 0; c < n; ++c) {
        if (!ok[c]) continue;
        for (int i = 0; i < z->pic; ++i) {
            const float* fi = &f[((size_t)c * z->pic + i) * 16];
            const float* ti = &t[((size_t)c * z->pic + i) * 9];
            for (int q = 0; q < 16; ++q) { fs[q] += fi[q]; fq[q] += (double)fi[q] * fi[q]; }
            for (int q = 0; q < 9; ++q) { ts[q] += ti[q]; tq[q] += (double)ti[q] * ti[q]; }
            ++nodes;
            for (int k = off[a0 + i]; k < off[a0 + i + 1]; ++k) {
                const float* fj = &f[((size_t)c * z->pic + nbr[k]) * 16];
                double d[3] = {fj[0] - fi[0], fj[1] - fi[1], fj[2] - fi[2]};
                double du[3] = {fj[3] - fi[3], fj[4] - fi[4], fj[5] - fi[5]};
                const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                const double st = len - len_k(k);
                const double vn = len > 0 ? (du[0] * d[0] + du[1] * d[1] + du[2] * d[2]) / len : 0.0;
                rq += (fi[0] * fi[0] + fi[1] * fi[1] + fi[2] * fi[2]) / 3;
                lq += st * st;
                uq += vn * vn;
                ++edges;
            }
        }
    }
    if (nodes == 0) return BCS_ERR_INVALID_ARGUMENT;
    auto spread = [](double q, double m, long long k) {
        const double v = q / k - m * m;
        return v > 1e-20 ? std::sqrt(v) : 1.0;
    };
    for (int q = 0; q < 16; ++q) {
        const double m = fs[q] / nodes;
        z->scales.fm[q] = (float)m;
        z->scales.fs[q] = (float)(1.0 / spread(fq[q], m, nodes));
    }
    // targets: median and 1.4826 x median absolute deviation (heavy tails:
    // contact events), falling back to the mean / spread when degenerate
    for (int q = 0; q < 9; ++q) {
        std::vector<float> col;
        col.reserve((size_t)nodes);
        for (int c = 0; c < n; ++c)
            if (ok[c])
                for (int i = 0; i < z->pic; ++i) col.push_back(t[((size_t)c * z->pic + i) * 9 + q]);
        std::nth_element(col.begin(), col.begin() + col.size() / 2, col.end());
        const float med = col[col.size() / 2];
        for (float& v : col) v = std::fabs(v - med);
        std::nth_element(col.begin(), col.begin() + col.size() / 2, col.end());
        const double mad = 1.4826 * col[col.size() / 2];
        const double m = ts[q] / nodes;
        z->scales.tm[q] = mad > 1e-20 ? med : (float)m;
        z->scales.ts[q] = mad > 1e-20 ? (float)mad : (float)spread(tq[q], m, nodes);
    }
    auto rms = [](double q, long long k) { return q > 1e-30 && k ? (float)std::sqrt(q / k) : 1.0f; };
    z->scales.er = rms(rq, edges);
    z->scales.eu = rms(uq, edges);
    z->scales.el = rms(lq, edges);
    z->scales_set = true;
    return BCS_OK;
}

const MacroHooks* inference_hooks(bcs_sim* s, int K) {
    bcs_surrogate* z = s->surrogate;
    if (!z) return nullptr;
    if (z->collecting) return &kCollectHooks;
    return z->enabled && z->K == K ? &kInferHooks : nullptr;
}
}  // namespace

extern "C" {

void bcs_default_params(bcs_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    // src/config/simulation.hpp:3-21
    p->dt = 0.008f;
    p->use_blood_flow = 1;
    p->enable_reaction_force = 1;
    p->enable_big_cells_brake = 1;
    p->cell_width = p->cell_height = p->cell_depth = 2.0f;
    p->cell_width_triangles = p->cell_height_triangles = p->cell_depth_triangles = 25.0f;
    p->bounding_spheres_coeff = 3.0f;
    p->grid_y_margin = 40.0f;
    p->grid_xz_margin = 40.0f;
    p->min_spawn_y = -20.0f;
    // src/config/physics.hpp:4-34
    p->velocity_collision_damping = 0.96f;
    p->particle_k_sniff = 25.0f;
    p->vein_k_sniff = 0.1f;
    p->particle_d_fact = 10.0f;
    p->vein_d_fact = 0.7f;
    p->vein_collision_force_intensity = 0.005f;
    p->viscous_damping = 0.39f;
    p->collision_spring_coeff = 6.0f;
    p->collision_damping_coeff = 6.0f;
    p->collision_shear_coeff = 4.0f;
    p->max_cell_size_factor_before_brake = 1.5f;
    p->big_particle_braking_intensity = 0.8f;
    p->init_velocity[0] = 0.0f; p->init_velocity[1] = -80.0f; p->init_velocity[2] = 0.0f;
    p->vein_impact_distance = 6.0f;
    p->vein_impact_minimal_force_distance = 0.001f;
    p->gravity[0] = 0.0f; p->gravity[1] = -25.0f; p->gravity[2] = 0.0f;
    // src/meta_factory/vein_factory.hpp:88
    p->cylinder_radius = 50.0f;
    p->particle_grid = BCS_GRID_UNIFORM;
    p->triangle_grid = BCS_GRID_UNIFORM;   // UNIFORM_TRIANGLES_GRID, main.cu:44
    p->vein_dynamic = 1;
    p->refresh_triangle_centers = 0;
    p->seed = 0;
}

const char* bcs_status_string(bcs_status s) {
    switch (s) {
        case BCS_OK: return "ok";
        case BCS_ERR_INVALID_ARGUMENT: return "invalid argument";
        case BCS_ERR_CUDA: return "CUDA runtime error";
        case BCS_ERR_OUT_OF_MEMORY: return "out of device memory";
        case BCS_ERR_NO_DEVICE: return "no CUDA device";
        case BCS_ERR_UNSUPPORTED: return "unsupported";
        case BCS_ERR_TIMEOUT: return "a bounded device wait expired";
    }
    return "unknown status";
}

int bcs_abi_version(void) { return BCS_ABI_VERSION; }

bcs_status bcs_set_device(int device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return BCS_ERR_NO_DEVICE;
    if (device < 0 || device >= n) return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaSetDevice(device));
    return BCS_OK;
}

bcs_status bcs_create_batch(const bcs_scene_desc* descs, int scene_count, void* stream, bcs_sim** out) {
    if (!out) return BCS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!descs || scene_count <= 0) return BCS_ERR_INVALID_ARGUMENT;
    bcs_status st;
    long long particles = 0;   // batch-wide particle ids are int32
    for (int k = 0; k < scene_count; ++k) {
        if ((st = validate(descs + k)) != BCS_OK) return st;
        if (!same_physics(descs[0].params, descs[k].params)) return BCS_ERR_INVALID_ARGUMENT;
        for (int t = 0; t < descs[k].type_count; ++t)
            particles += (long long)descs[k].types[t].count * descs[k].types[t].particles_in_cell;
    }
    if (particles > INT32_MAX / 2) return BCS_ERR_INVALID_ARGUMENT;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return BCS_ERR_NO_DEVICE;
    bcs_sim* s = new (std::nothrow) bcs_sim();
    if (!s) return BCS_ERR_OUT_OF_MEMORY;
    st = create_impl(descs, scene_count, stream, s);
    if (st != BCS_OK) {
        destroy_impl(s);
        delete s;
        return st;
    }
    *out = s;
    return BCS_OK;
}

bcs_status bcs_create(const bcs_scene_desc* desc, void* stream, bcs_sim** out) {
    if (!desc) {
        if (out) *out = nullptr;
        return BCS_ERR_INVALID_ARGUMENT;
    }
    return bcs_create_batch(desc, 1, stream, out);
}

bcs_status bcs_destroy(bcs_sim* s) {
    if (!s) return BCS_ERR_INVALID_ARGUMENT;
    destroy_impl(s);
    delete s;
    return BCS_OK;
}

bcs_status bcs_get_info(bcs_sim* s, bcs_info* o) {
    if (!s || !o) return BCS_ERR_INVALID_ARGUMENT;
    std::memset(o, 0, sizeof(*o));
    o->particle_count = s->N;
    o->blood_cell_count = s->C;
    o->type_count = (int)s->types.size();
    o->vertex_count = s->V;
    o->triangle_count = s->T;
    const SceneDev& z = s->scenes_host[0];
    o->min_x = z.pg.lo[0]; o->max_x = z.pg.hi[0];
    o->min_y = z.pg.lo[1]; o->max_y = z.pg.hi[1];
    o->min_z = z.pg.lo[2]; o->max_z = z.pg.hi[2];
    o->cell_count_x = z.pg.cx; o->cell_count_y = z.pg.cy; o->cell_count_z = z.pg.cz;
    o->cell_count = s->pg.g.cells;
    o->tri_cell_count_x = z.tg.cx; o->tri_cell_count_y = z.tg.cy; o->tri_cell_count_z = z.tg.cz;
    o->tri_cell_count = s->tg.g.cells;
    o->steps_done = s->host_steps;
    o->device_bytes = s->bytes;
    o->kernels_per_step = s->kernels_per_step;
    o->scene_count = s->S;
    return BCS_OK;
}

bcs_status bcs_get_scene_info(bcs_sim* s, int k, bcs_scene_info* o) {
    if (!s || !o || k < 0 || k >= s->S) return BCS_ERR_INVALID_ARGUMENT;
    std::memset(o, 0, sizeof(*o));
    const SceneDev& z = s->scenes_host[k];
    o->particle_start = z.particle_start;
    o->particle_count = z.particle_end - z.particle_start;
    o->blood_cell_start = s->scene_cell_start[k];
    o->blood_cell_count = s->scene_cells[k];
    o->vertex_start = s->scene_vertex_start[k];
    o->vertex_count = s->scene_vertex_count[k];
    o->triangle_start = z.tri_start;
    o->triangle_count = z.tri_end - z.tri_start;
    o->min_x = z.pg.lo[0]; o->max_x = z.pg.hi[0];
    o->min_y = z.pg.lo[1]; o->max_y = z.pg.hi[1];
    o->min_z = z.pg.lo[2]; o->max_z = z.pg.hi[2];
    o->cell_count_x = z.pg.cx; o->cell_count_y = z.pg.cy; o->cell_count_z = z.pg.cz;
    o->cell_count = z.pg.cells;
    o->cell_key_offset = z.pg.key_offset;
    o->tri_cell_count_x = z.tg.cx; o->tri_cell_count_y = z.tg.cy; o->tri_cell_count_z = z.tg.cz;
    o->tri_cell_count = z.tg.cells;
    o->tri_cell_key_offset = z.tg.key_offset;
    return BCS_OK;
}

bcs_status bcs_set_particles(bcs_sim* s, bcs_vec3 positions, bcs_vec3 velocities, bcs_vec3 forces, bcs_memory where) {
    if (!s || bad_vec(positions) || bad_vec(velocities)) return BCS_ERR_INVALID_ARGUMENT;
    bcs_status st;
    if ((st = set_vec(s, positions, s->N, s->pos[s->cur], s->radius_of_particle, where))) return st;
    if ((st = set_vec(s, velocities, s->N, s->vel[s->cur], nullptr, where))) return st;
    if (forces.x && forces.y && forces.z) {
        if ((st = set_vec(s, forces, s->N, s->frc[s->cur], nullptr, where))) return st;
    } else {
        BCS_CUDA(cudaMemsetAsync(s->frc[s->cur], 0, sizeof(float4) * s->N, s->stream));
    }
    s->keys_valid = false;
    s->mid_frame = false;
    // a grid built before this call still serves the next calculate_next_frame
    if (s->pg.spos_on && s->pg.sorted_once) {
        launch_gather_rows(s->pos[s->cur], s->pg.s_v[s->pg.slot], s->pg.count, s->pg.spos, s->stream);
        launch_gather_rows(s->vel[s->cur], s->pg.s_v[s->pg.slot], s->pg.count, s->pg.svel, s->stream);
    }
    if (s->tune.spatial_order && ((st = order_work_spatially(s)) || (st = upload_work(s)))) return st;
    return check_last();
}

bcs_status bcs_get_particles(bcs_sim* s, bcs_vec3 positions, bcs_vec3 velocities, bcs_vec3 forces, bcs_memory where) {
    if (!s) return BCS_ERR_INVALID_ARGUMENT;
    const int b = s->mid_frame ? (s->cur ^ 1) : s->cur;
    bcs_status st;
    if ((st = get_vec(s, s->pos[b], s->N, positions, where))) return st;
    if ((st = get_vec(s, s->vel[b], s->N, velocities, where))) return st;
    return get_vec(s, s->frc[b], s->N, forces, where);
}

bcs_status bcs_get_particles_async(bcs_sim* s, bcs_vec3 positions, bcs_vec3 velocities, bcs_vec3 forces) {
    if (!s) return BCS_ERR_INVALID_ARGUMENT;
    const bcs_vec3 req[3] = {positions, velocities, forces};
    if (!s->copy_stream) {
        BCS_CUDA(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            BCS_CUDA(cudaEventCreateWithFlags(&s->aready[k], cudaEventDisableTiming));
            BCS_CUDA(cudaEventCreateWithFlags(&s->adone[k], cudaEventDisableTiming));
        }
    }
    const int k = s->aslot;
    if (!s->ascratch[k]) {
        bcs_status st = dalloc(s, &s->ascratch[k], 9 * (size_t)s->N);
        if (st != BCS_OK) return st;
    }
    // the slot's previous copy must be done before its scratch is rewritten
    if (s->ainflight[k]) BCS_CUDA(cudaStreamWaitEvent(s->stream, s->adone[k], 0));
    const int b = s->mid_frame ? (s->cur ^ 1) : s->cur;
    const float4* src[3] = {s->pos[b], s->vel[b], s->frc[b]};
    const size_t n = (size_t)s->N, bytes = sizeof(float) * n;
    for (int q = 0; q < 3; ++q) {
        const bcs_vec3& v = req[q];
        if (!v.x && !v.y && !v.z) continue;
        float* d = s->ascratch[k] + 3 * n * q;
        launch_unpack(src[q], s->N, v.x ? d : nullptr, v.y ? d + n : nullptr, v.z ? d + 2 * n : nullptr, s->stream);
    }
    BCS_CUDA(cudaEventRecord(s->aready[k], s->stream));
    BCS_CUDA(cudaStreamWaitEvent(s->copy_stream, s->aready[k], 0));
    for (int q = 0; q < 3; ++q) {
        const bcs_vec3& v = req[q];
        float* d = s->ascratch[k] + 3 * n * q;
        if (v.x) BCS_CUDA(cudaMemcpyAsync(v.x, d, bytes, cudaMemcpyDeviceToHost, s->copy_stream));
        if (v.y) BCS_CUDA(cudaMemcpyAsync(v.y, d + n, bytes, cudaMemcpyDeviceToHost, s->copy_stream));
        if (v.z) BCS_CUDA(cudaMemcpyAsync(v.z, d + 2 * n, bytes, cudaMemcpyDeviceToHost, s->copy_stream));
    }
    BCS_CUDA(cudaEventRecord(s->adone[k], s->copy_stream));
    s->ainflight[k] = true;
    s->aslot ^= 1;
    return check_last();
}

bcs_status bcs_get_crowded(bcs_sim* s, long long* particles) {
    if (!s || !particles) return BCS_ERR_INVALID_ARGUMENT;
    unsigned long long v = 0;
    BCS_CUDA(cudaMemcpyAsync(&v, s->crowded_counter + 4, sizeof(v), cudaMemcpyDeviceToHost, s->stream));
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    *particles = (long long)v;
    return check_last();
}

bcs_status bcs_wait_particles(bcs_sim* s) {
    if (!s) return BCS_ERR_INVALID_ARGUMENT;
    if (s->copy_stream) BCS_CUDA(cudaStreamSynchronize(s->copy_stream));
    s->ainflight[0] = s->ainflight[1] = false;
    return check_last();
}

bcs_status bcs_set_vein(bcs_sim* s, bcs_vec3 positions, bcs_vec3 velocities, bcs_memory where) {
    if (!s) return BCS_ERR_INVALID_ARGUMENT;
    bcs_status st;
    if (!bad_vec(positions)) {
        if ((st = set_vec(s, positions, s->V, s->vpos, nullptr, where))) return st;
        if (s->wall_disp2) {
            const float huge = 3.0e38f;   // force a bounds / mask rebuild
            BCS_CUDA(cudaMemcpyAsync(s->wall_disp2, &huge, sizeof(float), cudaMemcpyHostToDevice, s->stream));
        }
        build_triangle_grid(s, s->p.refresh_triangle_centers != 0);
    }
    if (!bad_vec(velocities) && (st = set_vec(s, velocities, s->V, s->vvel, nullptr, where))) return st;
    return check_last();
}

bcs_status bcs_get_vein(bcs_sim* s, bcs_vec3 positions, bcs_vec3 velocities, bcs_vec3 forces, bcs_memory where) {
    if (!s) return BCS_ERR_INVALID_ARGUMENT;
    bcs_status st;
    if ((st = get_vec(s, s->vpos, s->V, positions, where))) return st;
    if ((st = get_vec(s, s->vvel, s->V, velocities, where))) return st;
    return get_vec(s, s->vfrc, s->V, forces, where);
}

// Movers of at most one tile in a recent frame: the next frames sort theirs
// with one CTA and no pass kernels (a larger count is still sorted correctly
// by it, only slower).  The count is that of a frame a few frames back (the
// host runs ahead of the device); on the 4.2M-particle bifurcation one CTA
// stays faster than the passes up to about 7 000 movers, while the count
// grows by a few percent per frame.
constexpr int kOneCtaMovers = 4096;

// Frames the host may launch ahead of the device under the automatic mover
// sort (several frames of queued work, a mover count at most this stale).
constexpr int kLeadFrames = 4;

// How a frame's grid sort runs: 0 = incremental, movers by the radix passes;
// 1 = incremental, movers by one CTA; 2 = every pair from scratch.  When
// more than half the particles moved in a recent frame the sort from scratch
// is the faster (late in the 4.2M trajectory: grid phase 0.36 against
// 0.57 ms); every kProbeFrames-th frame stays incremental so that the count
// keeps being measured.
constexpr int kProbeFrames = 16;

int mover_form(const bcs_sim* s) {
    if (s->mover_sort != 0) return s->mover_sort - 1;
    if (!s->movers_seen) return 0;
    const int seen = *(volatile const int*)s->movers_seen;
    if (seen < 0) return 0;
    if (seen <= kOneCtaMovers) return 1;
    if (seen > s->N / 2 && s->frames_launched % kProbeFrames != 0) return 2;
    return 0;
}

void set_mover_form(bcs_sim* s, int form) {
    s->pg.inc.one_cta = form == 1;
    s->pg.full_now = form == 2;
}

bcs_status bcs_calculate_grids(bcs_sim* s) {
    if (!s) return BCS_ERR_INVALID_ARGUMENT;
    if (s->mid_frame) return BCS_ERR_INVALID_ARGUMENT;
    s->keys_valid = false;
    set_mover_form(s, s->mover_sort > 1 ? s->mover_sort - 1 : 0);   // unpaced calls: the passes unless fixed
    enqueue_grids(s);
    return check_last();
}

bcs_status bcs_calculate_next_frame(bcs_sim* s) {
    if (!s || s->mid_frame) return BCS_ERR_INVALID_ARGUMENT;
    set_mover_form(s, s->mover_sort > 1 ? s->mover_sort - 1 : 0);
    if (!s->grid_ready) enqueue_grids(s);
    enqueue_vein_forces(s);
    refresh_args(s, s->cur, s->cur ^ 1, false);
    launch_step(s->args, (int)s->work_host.size(), 1, s->tune.step_shape, s->persistent_grid[1], s->stream);
    s->mid_frame = true;
    return check_last();
}

bcs_status bcs_propagate_all(bcs_sim* s) {
    if (!s || !s->mid_frame) return BCS_ERR_INVALID_ARGUMENT;
    refresh_args(s, s->cur, s->cur ^ 1, false);
    launch_propagate(s->args, (int)s->work_host.size(), s->stream);
    enqueue_vein_propagate(s);
    s->cur ^= 1;
    s->mid_frame = false;
    s->keys_valid = false;
    s->grid_ready = false;
    ++s->host_steps;
    return check_last();
}

// n fused frames (substeps = 1) or multi-rate macro steps, each replayed
// from a CUDA graph captured per (sub-steps, sort form, buffer parity,
// sorted slot).
static bcs_status run_steps(bcs_sim* s, int n, int substeps = 1) {
    auto enqueue = [&]() {
        if (substeps > 1) enqueue_macro(s, substeps);
        else enqueue_frame(s);
    };
    // an event after every launched frame (the automatic mover sort waits
    // for the one kLeadFrames launches back)
    auto mark = [&]() -> bcs_status {
        cudaEvent_t& ev = s->lead_ev[s->frames_launched % 8];
        if (!ev) BCS_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        BCS_CUDA(cudaEventRecord(ev, s->stream));
        ++s->frames_launched;
        return BCS_OK;
    };
    for (int i = 0; i < n; ++i) {
        if (s->mover_sort == 0 && s->frames_launched >= kLeadFrames) {
            cudaEvent_t& back = s->lead_ev[(s->frames_launched - kLeadFrames) % 8];
            if (back) BCS_CUDA(cudaEventSynchronize(back));
        }
        const int form = mover_form(s);
        set_mover_form(s, form);
        // the first frame of a grid, or with triangle centres refreshed, runs
        // eagerly (its sort is a full one)
        if (s->p.refresh_triangle_centers || (!s->keys_valid && !s->pg.sorted_once)) {
            enqueue();
            if (bcs_status st = mark()) return st;
            continue;
        }
        if (!s->keys_valid) {
            // keys of positions set from outside, then the frame's usual graph
            launch_keys(s->pos[s->cur], s->N, s->pg.g.uniform, s->scenes, s->S, s->pg.in_k, s->pg.in_v, s->err,
                        s->stream);
            s->keys_valid = true;
        }
        cudaGraphExec_t& g = s->graphs[((long long)substeps * 3 + form) * 4 + s->cur * 2 + s->pg.slot];
        if (!g) {
            const int cur0 = s->cur;
            const int slot0 = s->pg.slot;
            const long long hs = s->host_steps;
            cudaGraph_t graph = nullptr;
            BCS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            enqueue();
            cudaError_t ce = cudaStreamEndCapture(s->stream, &graph);
            s->cur = cur0;
            s->pg.slot = slot0;
            s->host_steps = hs;
            if (ce != cudaSuccess) return BCS_ERR_CUDA;
            {
                size_t nn = 0;
                cudaGraphGetNodes(graph, nullptr, &nn);
                std::vector<cudaGraphNode_t> nodes(nn);
                cudaGraphGetNodes(graph, nodes.data(), &nn);
                int kernels = 0;
                for (auto nd : nodes) {
                    cudaGraphNodeType t;
                    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
                }
                if (substeps == 1) s->kernels_per_step = kernels;
            }
            ce = cudaGraphInstantiate(&g, graph, 0);
            cudaGraphDestroy(graph);
            if (ce != cudaSuccess) { g = nullptr; return BCS_ERR_CUDA; }
        }
        BCS_CUDA(cudaGraphLaunch(g, s->stream));
        if (bcs_status st = mark()) return st;
        // A replay is one whole enqueue_frame: mirror its host-side state.
        s->cur ^= 1;
        s->pg.slot ^= 1;
        s->pg.g.keys = s->pg.s_k[s->pg.slot];
        s->pg.g.ids = s->pg.s_v[s->pg.slot];
        s->keys_valid = true;
        s->grid_ready = true;
        s->host_steps += substeps;
    }
    return BCS_OK;
}

bcs_status bcs_macro_step(bcs_sim* s, int substeps, int n) {
    if (!s || n < 0 || substeps < 1 || substeps > BCS_MAX_SUBSTEPS || s->mid_frame) return BCS_ERR_INVALID_ARGUMENT;
    bcs_status st = run_steps(s, n, substeps);
    if (st != BCS_OK) return st;
    return check_last();
}

bcs_status bcs_step(bcs_sim* s, int nsteps) {
    if (!s || nsteps < 0) return BCS_ERR_INVALID_ARGUMENT;
    if (s->mid_frame) return BCS_ERR_INVALID_ARGUMENT;
    bcs_status st = run_steps(s, nsteps);
    if (st != BCS_OK) return st;
    return check_last();
}

bcs_status bcs_init_particles(bcs_sim* s, const bcs_init_desc* d) {
    if (!s || !d || s->mid_frame || (d->kind != BCS_INIT_REFERENCE && d->kind != BCS_INIT_LATTICE) ||
        d->velocity_sigma < 0.f || d->gap < 0.f)
        return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    float4 *P = s->pos[s->cur], *Vv = s->vel[s->cur], *F = s->frc[s->cur];
    bcs_status st = BCS_OK;
    if (d->kind == BCS_INIT_REFERENCE) {
        launch_init_reference(s->args, P, Vv, F, s->model, s->radius_of_particle, d->seed, s->stream);
    } else {
        for (int k = 0; k < s->S && st == BCS_OK; ++k) {
            const SceneDev& z = s->scenes_host[k];
            float spacing = 0.f;
            int cells = 0;
            for (size_t t = 0; t < s->types.size(); ++t) {
                if (s->types[t].scene != k) continue;
                float rmax = 0.f;
                for (int i = 0; i < s->types[t].pic; ++i)
                    rmax = std::max(rmax, s->h_radius_model[s->types[t].model_start + i]);
                spacing = std::max(spacing, 2.f * (s->h_type_bound[t] + rmax) + d->gap);
                cells += s->types[t].count;
            }
            if (cells == 0) continue;
            const float* box = &s->h_vein_box[6 * k];
            const float3 lo = make_float3(box[0], box[1], box[2]);
            const long long nx = std::max(1LL, (long long)((box[3] - box[0]) / spacing));
            const long long ny = std::max(1LL, (long long)((box[4] - box[1]) / spacing));
            const long long nz = std::max(1LL, (long long)((box[5] - box[2]) / spacing));
            const long long total = nx * ny * nz;
            if (total > (1LL << 30)) { st = BCS_ERR_UNSUPPORTED; break; }
            int *keys = nullptr, *ids = nullptr, *k2 = nullptr, *i2 = nullptr, *cnt = nullptr;
            unsigned* temp = nullptr;
            const int n = (int)total;
            if (cudaMalloc(&keys, sizeof(int) * n) || cudaMalloc(&ids, sizeof(int) * n) ||
                cudaMalloc(&k2, sizeof(int) * n) || cudaMalloc(&i2, sizeof(int) * n) || cudaMalloc(&cnt, sizeof(int)) ||
                cudaMalloc(&temp, sizeof(unsigned) * radix_temp_words(n))) {
                (void)cudaGetLastError();
                st = BCS_ERR_OUT_OF_MEMORY;
            } else {
                cudaMemsetAsync(cnt, 0, sizeof(int), s->stream);
                launch_lattice_sites(s->scenes, k, lo, (int)nx, (int)ny, (int)nz, spacing, 0.5f * spacing, box[1],
                                     box[4], s->flows, d->seed, keys, ids, cnt, s->stream);
                // keys: 30-bit priorities of valid sites, 2^30 for the rest
                const int where = radix_sort_pairs(keys, ids, k2, i2, keys, ids, n, 31, temp, s->stream);
                int valid = 0;
                cudaMemcpyAsync(&valid, cnt, sizeof(int), cudaMemcpyDeviceToHost, s->stream);
                if (cudaStreamSynchronize(s->stream) != cudaSuccess) st = BCS_ERR_CUDA;
                else if (valid < cells) st = BCS_ERR_INVALID_ARGUMENT;   // the vessel holds too few sites
                else
                    launch_lattice_place(s->args, k, z.particle_end - z.particle_start, P, Vv, F, s->model,
                                         s->type_centroid, s->radius_of_particle, where ? ids : i2, lo, (int)nx,
                                         (int)ny, spacing, d->velocity_sigma, d->seed, s->stream);
                if (st == BCS_OK && cudaStreamSynchronize(s->stream) != cudaSuccess) st = BCS_ERR_CUDA;
            }
            cudaFree(keys); cudaFree(ids); cudaFree(k2); cudaFree(i2); cudaFree(cnt); cudaFree(temp);
        }
    }
    if (st != BCS_OK) return st;
    s->keys_valid = false;
    s->grid_ready = false;
    s->mid_frame = false;
    if (s->tune.spatial_order && ((st = order_work_spatially(s)) || (st = upload_work(s)))) return st;
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    return check_last();
}

bcs_status bcs_set_mover_sort(bcs_sim* s, int mode) {
    if (!s || mode < 0 || mode > 3) return BCS_ERR_INVALID_ARGUMENT;
    s->mover_sort = mode;
    return BCS_OK;
}

bcs_status bcs_get_tuning(bcs_sim* s, bcs_tuning* out) {
    if (!s || !out) return BCS_ERR_INVALID_ARGUMENT;
    *out = s->tune;
    return BCS_OK;
}

bcs_status bcs_set_tuning(bcs_sim* s, const bcs_tuning* t) {
    if (!s || !t || s->mid_frame) return BCS_ERR_INVALID_ARGUMENT;
    return apply_tuning(s, *t);
}

namespace {
// Device copy of everything a frame reads and writes that carries physics:
// particle and vein state, the step counter (respawn draws) and the error
// word.  The grids, caches and culling structures are rebuilt from it.
struct Snapshot {
    float4* particles = nullptr;   // pos, vel, frc
    float4* vein = nullptr;        // vpos, vvel, vfrc
    long long* steps = nullptr;
    unsigned* err = nullptr;
    long long host_steps = 0;
    void release() {
        cudaFree(particles);
        cudaFree(vein);
        cudaFree(steps);
        cudaFree(err);
    }
};

bcs_status take_snapshot(bcs_sim* s, Snapshot& z) {
    const size_t n = (size_t)s->N, v = (size_t)std::max(1, s->V);
    BCS_CUDA(cudaMalloc(&z.particles, 3 * n * sizeof(float4)));
    BCS_CUDA(cudaMalloc(&z.vein, 3 * v * sizeof(float4)));
    BCS_CUDA(cudaMalloc(&z.steps, sizeof(long long)));
    BCS_CUDA(cudaMalloc(&z.err, sizeof(unsigned)));
    const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
    BCS_CUDA(cudaMemcpyAsync(z.particles, s->pos[s->cur], n * sizeof(float4), k, s->stream));
    BCS_CUDA(cudaMemcpyAsync(z.particles + n, s->vel[s->cur], n * sizeof(float4), k, s->stream));
    BCS_CUDA(cudaMemcpyAsync(z.particles + 2 * n, s->frc[s->cur], n * sizeof(float4), k, s->stream));
    if (s->V > 0) {
        BCS_CUDA(cudaMemcpyAsync(z.vein, s->vpos, v * sizeof(float4), k, s->stream));
        BCS_CUDA(cudaMemcpyAsync(z.vein + v, s->vvel, v * sizeof(float4), k, s->stream));
        BCS_CUDA(cudaMemcpyAsync(z.vein + 2 * v, s->vfrc, v * sizeof(float4), k, s->stream));
    }
    BCS_CUDA(cudaMemcpyAsync(z.steps, s->steps, sizeof(long long), k, s->stream));
    BCS_CUDA(cudaMemcpyAsync(z.err, s->err, sizeof(unsigned), k, s->stream));
    z.host_steps = s->host_steps;
    return BCS_OK;
}

bcs_status restore_snapshot(bcs_sim* s, const Snapshot& z) {
    const size_t n = (size_t)s->N, v = (size_t)std::max(1, s->V);
    const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
    BCS_CUDA(cudaMemcpyAsync(s->pos[s->cur], z.particles, n * sizeof(float4), k, s->stream));
    BCS_CUDA(cudaMemcpyAsync(s->vel[s->cur], z.particles + n, n * sizeof(float4), k, s->stream));
    BCS_CUDA(cudaMemcpyAsync(s->frc[s->cur], z.particles + 2 * n, n * sizeof(float4), k, s->stream));
    if (s->V > 0) {
        BCS_CUDA(cudaMemcpyAsync(s->vpos, z.vein, v * sizeof(float4), k, s->stream));
        BCS_CUDA(cudaMemcpyAsync(s->vvel, z.vein + v, v * sizeof(float4), k, s->stream));
        BCS_CUDA(cudaMemcpyAsync(s->vfrc, z.vein + 2 * v, v * sizeof(float4), k, s->stream));
    }
    BCS_CUDA(cudaMemcpyAsync(s->steps, z.steps, sizeof(long long), k, s->stream));
    BCS_CUDA(cudaMemcpyAsync(s->err, z.err, sizeof(unsigned), k, s->stream));
    s->host_steps = z.host_steps;
    s->keys_valid = false;
    s->grid_ready = false;
    s->mid_frame = false;
    if (s->p.vein_dynamic && s->T > 0) {
        if (s->wall_disp2) {
            const float huge = 3.0e38f;   // force a bounds / mask rebuild
            BCS_CUDA(cudaMemcpyAsync(s->wall_disp2, &huge, sizeof(float), cudaMemcpyHostToDevice, s->stream));
        }
        build_triangle_grid(s, s->p.refresh_triangle_centers != 0);
    }
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    return check_last();
}
}  // namespace

bcs_status bcs_autotune(bcs_sim* s, int frames, bcs_tuning* chosen, float* ms_per_frame) {
    if (!s || frames <= 0 || s->mid_frame) return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    Snapshot z;
    bcs_status st = take_snapshot(s, z);
    // Coordinate descent from the current tuning: each field in turn takes
    // every value with the others held; two sweeps.
    bcs_tuning best = s->tune;
    float best_ms = std::numeric_limits<float>::max();
    auto trial = [&](const bcs_tuning& t, float& ms) -> bcs_status {
        bcs_status r;
        if ((r = restore_snapshot(s, z)) || (r = apply_tuning(s, t)) || (r = run_steps(s, 2))) return r;
        if (cudaEventRecord(s->ev0, s->stream) != cudaSuccess) return BCS_ERR_CUDA;
        if ((r = run_steps(s, frames))) return r;
        if (cudaEventRecord(s->ev1, s->stream) != cudaSuccess || cudaEventSynchronize(s->ev1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, s->ev0, s->ev1) != cudaSuccess)
            return BCS_ERR_CUDA;
        ms /= (float)frames;
        return BCS_OK;
    };
    if (st == BCS_OK) st = trial(best, best_ms);
    int bcs_tuning::*fields[] = {&bcs_tuning::step_shape, &bcs_tuning::persistent, &bcs_tuning::spatial_order,
                                 &bcs_tuning::full_sort, &bcs_tuning::occupancy_filter,
                                 &bcs_tuning::sorted_positions, &bcs_tuning::grid_collisions};
    const int limits[] = {kStepShapes, 2, 2, 2, 2, 2, 4};
    constexpr int kFields = sizeof(limits) / sizeof(limits[0]);
    for (int sweep = 0; sweep < 2 && st == BCS_OK; ++sweep) {
        bool improved = false;
        for (int f = 0; f < kFields && st == BCS_OK; ++f)
            for (int v = 0; v < limits[f] && st == BCS_OK; ++v) {
                bcs_tuning t = best;
                if (t.*fields[f] == v) continue;
                t.*fields[f] = v;
                if (!tuning_valid(s, t)) continue;
                float ms = 0.f;
                if ((st = trial(t, ms))) break;
                if (ms < best_ms) {
                    best_ms = ms;
                    best = t;
                    improved = true;
                }
            }
        if (!improved) break;
    }
    if (st == BCS_OK) st = restore_snapshot(s, z);
    if (st == BCS_OK) st = apply_tuning(s, best);
    z.release();
    if (st != BCS_OK) return st;
    if (chosen) *chosen = best;
    if (ms_per_frame) *ms_per_frame = best_ms;
    return BCS_OK;
}

bcs_status bcs_get_grid(bcs_sim* s, int which, int* cell_ids, int* object_ids, int* cell_starts, int* cell_ends,
                        bcs_memory where) {
    if (!s || (which != 0 && which != 1)) return BCS_ERR_INVALID_ARGUMENT;
    DeviceGrid& dg = which ? s->tg : s->pg;
    if (!dg.g.uniform || !dg.g.keys) return BCS_ERR_INVALID_ARGUMENT;
    const int n = dg.count;
    const cudaMemcpyKind kind = where == BCS_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (cell_ids) BCS_CUDA(cudaMemcpyAsync(cell_ids, dg.g.keys, sizeof(int) * n, kind, s->stream));
    if (object_ids) BCS_CUDA(cudaMemcpyAsync(object_ids, dg.g.ids, sizeof(int) * n, kind, s->stream));
    if (cell_starts || cell_ends) {
        int* ds = nullptr;
        int* de = nullptr;
        ScopedDevice hs, he;   // host destinations go through device scratch
        if (where == BCS_MEM_DEVICE) {
            ds = cell_starts;
            de = cell_ends;
        } else {
            if (cell_starts) BCS_CUDA(cudaMalloc(&hs.p, sizeof(int) * (size_t)dg.g.cells));
            if (cell_ends) BCS_CUDA(cudaMalloc(&he.p, sizeof(int) * (size_t)dg.g.cells));
            ds = hs.as<int>();
            de = he.as<int>();
        }
        ensure_table(dg, s->stream);
        launch_dense_ranges(dg.table, dg.epoch, dg.g.cells, ds, de, s->stream);
        if (where == BCS_MEM_HOST) {
            if (ds) BCS_CUDA(cudaMemcpyAsync(cell_starts, ds, sizeof(int) * (size_t)dg.g.cells, kind, s->stream));
            if (de) BCS_CUDA(cudaMemcpyAsync(cell_ends, de, sizeof(int) * (size_t)dg.g.cells, kind, s->stream));
            BCS_CUDA(cudaStreamSynchronize(s->stream));
        }
    }
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    return check_last();
}

bcs_status bcs_export_render(bcs_sim* s, float* particle_vbo, float* particle_offsets, float* vein_vbo,
                             bcs_memory where) {
    if (!s) return BCS_ERR_INVALID_ARGUMENT;
    const int b = s->mid_frame ? (s->cur ^ 1) : s->cur;
    if (where == BCS_MEM_DEVICE) {
        launch_export(s->pos[b], s->N, s->vpos, s->V, particle_vbo, particle_offsets, vein_vbo, s->stream);
        return check_last();
    }
    ScopedDevice sp, soff, sv;
    if (particle_vbo) BCS_CUDA(cudaMalloc(&sp.p, sizeof(float) * 6 * (size_t)s->N));
    if (particle_offsets) BCS_CUDA(cudaMalloc(&soff.p, sizeof(float) * 3 * (size_t)s->N));
    if (vein_vbo) BCS_CUDA(cudaMalloc(&sv.p, sizeof(float) * 6 * (size_t)s->V));
    float *dp = sp.as<float>(), *doff = soff.as<float>(), *dv = sv.as<float>();
    launch_export(s->pos[b], s->N, s->vpos, s->V, dp, doff, dv, s->stream);
    if (dp) BCS_CUDA(cudaMemcpyAsync(particle_vbo, dp, sizeof(float) * 6 * (size_t)s->N, cudaMemcpyDeviceToHost, s->stream));
    if (doff) BCS_CUDA(cudaMemcpyAsync(particle_offsets, doff, sizeof(float) * 3 * (size_t)s->N, cudaMemcpyDeviceToHost, s->stream));
    if (dv) BCS_CUDA(cudaMemcpyAsync(vein_vbo, dv, sizeof(float) * 6 * (size_t)s->V, cudaMemcpyDeviceToHost, s->stream));
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    return check_last();
}

bcs_status bcs_get_error_word(bcs_sim* s, uint32_t* out, int clear) {
    if (!s || !out) return BCS_ERR_INVALID_ARGUMENT;
    unsigned h = 0;
    BCS_CUDA(cudaMemcpyAsync(&h, s->err, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    if (clear) BCS_CUDA(cudaMemsetAsync(s->err, 0, sizeof(unsigned), s->stream));
    *out = h;
    return BCS_OK;
}

bcs_status bcs_synchronize(bcs_sim* s) {
    if (!s) return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    return check_last();
}

bcs_status bcs_time_steps(bcs_sim* s, int nsteps, float* ms_out) {
    if (!s || !ms_out || nsteps < 0 || s->mid_frame) return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaEventRecord(s->ev0, s->stream));
    bcs_status st = run_steps(s, nsteps);
    if (st != BCS_OK) return st;
    BCS_CUDA(cudaEventRecord(s->ev1, s->stream));
    BCS_CUDA(cudaEventSynchronize(s->ev1));
    BCS_CUDA(cudaEventElapsedTime(ms_out, s->ev0, s->ev1));
    return check_last();
}

bcs_status bcs_time_macro_steps(bcs_sim* s, int substeps, int n, float* ms_out) {
    if (!s || !ms_out || n < 0 || substeps < 1 || substeps > BCS_MAX_SUBSTEPS || s->mid_frame)
        return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaEventRecord(s->ev0, s->stream));
    bcs_status st = run_steps(s, n, substeps);
    if (st != BCS_OK) return st;
    BCS_CUDA(cudaEventRecord(s->ev1, s->stream));
    BCS_CUDA(cudaEventSynchronize(s->ev1));
    BCS_CUDA(cudaEventElapsedTime(ms_out, s->ev0, s->ev1));
    return check_last();
}

bcs_status bcs_run(bcs_sim* s, bcs_control* control, int max_frames, int* frames_run) {
    if (!s || max_frames < 0) return BCS_ERR_INVALID_ARGUMENT;
    int count = 0, frames = 0;
    bcs_status st = BCS_OK;
    for (bool running = true; running;) {
        if ((st = bcs_step(s, 1)) != BCS_OK) break;
        ++frames;
        if (control) {
            bcs_control_state cs{};
            if ((st = bcs_control_handle(control, &cs)) != BCS_OK) break;
            if (cs.stop_requested) running = false;
        }
        if (++count > max_frames) running = false;
    }
    if (frames_run) *frames_run = frames;
    if (st != BCS_OK) return st;
    if (control) {
        bcs_event done{BCS_EVENT_STREAM_SUCCESSFULLY_ENDED, BCS_EVENT_NOT_RELEVANT};
        if ((st = bcs_control_send(control, done)) != BCS_OK) return st;
    }
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    return check_last();
}

bcs_status bcs_profile_steps(bcs_sim* s, int nsteps, float* phase_ms) {
    if (!s || !phase_ms || nsteps < 0 || s->mid_frame) return BCS_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < nsteps; ++i) {
        set_mover_form(s, mover_form(s));   // the previous frame's count: this loop waits for each frame
        enqueue_frame(s, s->pev);
        ++s->frames_launched;   // paces the probe frames (its events are not needed: each frame is waited for)
        BCS_CUDA(cudaEventSynchronize(s->pev[BCS_PHASE_COUNT]));
        for (int k = 0; k < BCS_PHASE_COUNT; ++k) {
            float ms = 0.f;
            BCS_CUDA(cudaEventElapsedTime(&ms, s->pev[k], s->pev[k + 1]));
            phase_ms[k] += ms;
        }
    }
    return check_last();
}

bcs_status bcs_surrogate_create(bcs_sim* s, const bcs_surrogate_desc* d, bcs_surrogate** out) {
    if (!s || !d || !out) return BCS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (d->cell_type < 0 || d->cell_type >= (int)s->types.size() || d->substeps < 2 ||
        d->substeps > BCS_MAX_SUBSTEPS || d->layers < 1 || d->layers > kMaxLayers || d->max_samples < 1 ||
        d->tolerance < 0.f || d->huber_delta < 0.f)
        return BCS_ERR_INVALID_ARGUMENT;
    const TypeDev& t0 = s->types[d->cell_type];
    if (t0.pic > 6 * 32) return BCS_ERR_UNSUPPORTED;
    std::unique_ptr<bcs_surrogate> z(new (std::nothrow) bcs_surrogate());
    if (!z) return BCS_ERR_OUT_OF_MEMORY;
    z->sim = s;
    z->K = d->substeps;
    z->model_type = d->cell_type;
    z->pic = t0.pic;
    z->seed = d->seed;
    // every type with the same cell model (batches repeat a model per scene)
    auto same_model = [&](const TypeDev& t) {
        if (t.pic != t0.pic) return false;
        for (int i = 0; i <= t.pic; ++i)
            if (s->h_adj_off[t.adj_start + i] - s->h_adj_off[t.adj_start] !=
                s->h_adj_off[t0.adj_start + i] - s->h_adj_off[t0.adj_start])
                return false;
        const int e = s->h_adj_off[t0.adj_start + t0.pic] - s->h_adj_off[t0.adj_start];
        const int b = s->h_adj_off[t.adj_start], b0 = s->h_adj_off[t0.adj_start];
        for (int k = 0; k < e; ++k)
            if (s->h_adj_nbr[b + k] != s->h_adj_nbr[b0 + k] || s->h_adj_len[b + k] != s->h_adj_len[b0 + k])
                return false;
        return true;
    };
    float rmin = std::numeric_limits<float>::max();
    for (int i = 0; i < t0.pic; ++i) rmin = std::min(rmin, s->h_radius_model[t0.model_start + i]);
    z->tolerance = d->tolerance > 0.f ? d->tolerance : 1e-3f * rmin;
    for (int ti = 0; ti < (int)s->types.size(); ++ti)
        if (same_model(s->types[ti]))
            for (int c = 0; c < s->types[ti].count; ++c) {
                z->cell_type.push_back(ti);
                z->cell_index.push_back(c);
            }
    z->cells = (int)z->cell_type.size();
    if (z->cells == 0) return BCS_ERR_INVALID_ARGUMENT;
    // graph of one cell, neighbour indices within the cell
    const int a0 = s->h_adj_off[t0.adj_start];
    std::vector<int> off(t0.pic + 1), nbr;
    std::vector<float> len;
    for (int i = 0; i <= t0.pic; ++i) off[i] = s->h_adj_off[t0.adj_start + i] - a0;
    nbr.assign(s->h_adj_nbr.begin() + a0, s->h_adj_nbr.begin() + a0 + off[t0.pic]);
    len.assign(s->h_adj_len.begin() + a0, s->h_adj_len.begin() + a0 + off[t0.pic]);
    const int train_cells = std::max(1, std::min(d->max_samples, 1024));
    z->infer_cells = std::max(train_cells, std::min(z->cells, 2048));
    if (z->net.init(d->layers, t0.pic, off.data(), nbr.data(), len.data(), z->infer_cells, d->seed, s->stream) !=
        (int)cudaSuccess)
        return BCS_ERR_OUT_OF_MEMORY;
    z->net.set_huber(d->huber_delta);
    z->capacity = d->max_samples;
    if (!z->alloc(&z->d_cell_type, z->cells) || !z->alloc(&z->d_cell_index, z->cells) ||
        !z->alloc(&z->raw, (size_t)z->cells * z->pic * 16) || !z->alloc(&z->start, (size_t)z->cells * z->pic * 3) ||
        !z->alloc(&z->skip, s->C) || !z->alloc(&z->counts, 2) ||
        !z->alloc(&z->ds_raw, (size_t)z->capacity * z->pic * 16) || !z->alloc(&z->ds_t, (size_t)z->capacity * z->pic * 9) ||
        !z->alloc(&z->ds_valid, z->capacity) || !z->alloc(&z->valid_list, z->capacity))
        return BCS_ERR_OUT_OF_MEMORY;
    BCS_CUDA(cudaMemcpyAsync(z->d_cell_type, z->cell_type.data(), sizeof(int) * z->cells, cudaMemcpyHostToDevice,
                             s->stream));
    BCS_CUDA(cudaMemcpyAsync(z->d_cell_index, z->cell_index.data(), sizeof(int) * z->cells, cudaMemcpyHostToDevice,
                             s->stream));
    BCS_CUDA(cudaMemsetAsync(z->skip, 0, s->C, s->stream));
    BCS_CUDA(cudaMemsetAsync(z->counts, 0, 2 * sizeof(unsigned long long), s->stream));
    BCS_CUDA(cudaMemsetAsync(z->ds_valid, 0, z->capacity, s->stream));
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    s->surrogates.push_back(z.get());
    *out = z.release();
    return BCS_OK;
}

bcs_status bcs_surrogate_destroy(bcs_surrogate* z) {
    if (!z) return BCS_ERR_INVALID_ARGUMENT;
    if (bcs_sim* s = z->sim) {
        if (s->surrogate == z) {
            s->surrogate = nullptr;
            drop_graphs(s);
        }
        s->surrogates.erase(std::remove(s->surrogates.begin(), s->surrogates.end(), z), s->surrogates.end());
        cudaStreamSynchronize(s->stream);
    }
    delete z;
    return BCS_OK;
}

bcs_status bcs_surrogate_collect(bcs_surrogate* z, int macro_steps) {
    if (!live(z) || macro_steps < 0) return BCS_ERR_INVALID_ARGUMENT;
    bcs_sim* s = z->sim;
    if (s->mid_frame || (s->surrogate && s->surrogate != z)) return BCS_ERR_INVALID_ARGUMENT;
    bcs_surrogate* prev = s->surrogate;
    s->surrogate = z;
    z->collecting = true;
    bcs_status st = BCS_OK;
    for (int i = 0; i < macro_steps && z->stored + z->cells <= z->capacity; ++i) {
        set_mover_form(s, s->mover_sort > 1 ? s->mover_sort - 1 : 0);
        enqueue_macro(s, z->K, &kCollectHooks);
        if ((st = check_last())) break;
        z->stored += z->cells;
    }
    z->collecting = false;
    s->surrogate = prev;
    if (st != BCS_OK) return st;
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    // list of valid samples
    std::vector<unsigned char> ok(z->stored);
    if (z->stored) BCS_CUDA(cudaMemcpy(ok.data(), z->ds_valid, z->stored, cudaMemcpyDeviceToHost));
    std::vector<int> list;
    for (int i = 0; i < z->stored; ++i)
        if (ok[i]) list.push_back(i);
    z->nvalid = (int)list.size();
    if (z->nvalid)
        BCS_CUDA(cudaMemcpyAsync(z->valid_list, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice,
                                 s->stream));
    return check_last();
}

bcs_status bcs_surrogate_train(bcs_surrogate* z, int iterations, int batch_cells, float lr, float* loss) {
    if (!live(z) || iterations < 0 || batch_cells < 1 || batch_cells > z->net.max_cells() || !(lr > 0.f))
        return BCS_ERR_INVALID_ARGUMENT;
    if (z->nvalid == 0) return BCS_ERR_INVALID_ARGUMENT;
    bcs_status st;
    if (!z->scales_set && (st = compute_scales(z))) return st;
    cudaStream_t stream = z->sim->stream;
    for (int it = 0; it < iterations; ++it) {
        launch_sur_inputs(z->ds_raw, z->ds_t, z->valid_list, z->nvalid, z->seed * 0x9E3779B97F4A7C15ull + (++z->draws),
                          0, batch_cells, z->pic, z->net.dev_adj_off(), z->net.dev_adj_nbr(), z->net.dev_adj_len(),
                          z->scales, z->net.input_buf(), z->net.edge_buf(), z->net.target_buf(), stream);
        z->net.forward(z->net.input_buf(), z->net.edge_buf(), batch_cells, true);
        z->net.backward(z->net.target_buf(), batch_cells);
        z->net.adam(lr);
        ++z->iterations;
    }
    if (iterations > 0) {
        BCS_CUDA(cudaMemcpyAsync(&z->last_loss, z->net.loss_dev(), sizeof(float), cudaMemcpyDeviceToHost, stream));
        BCS_CUDA(cudaStreamSynchronize(stream));
    }
    if (loss) *loss = z->last_loss;
    return check_last();
}

bcs_status bcs_surrogate_enable(bcs_surrogate* z, int on) {
    if (!live(z)) return BCS_ERR_INVALID_ARGUMENT;
    bcs_sim* s = z->sim;
    if (s->mid_frame || (s->surrogate && s->surrogate != z)) return BCS_ERR_INVALID_ARGUMENT;
    if (on && !z->scales_set) return BCS_ERR_INVALID_ARGUMENT;   // train (or set the scales) first
    if (on < 0 || on > 2) return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaStreamSynchronize(s->stream));
    z->enabled = on != 0;
    if (on) z->mode = on;
    s->surrogate = z->enabled ? z : nullptr;
    BCS_CUDA(cudaMemsetAsync(z->skip, 0, s->C, s->stream));
    drop_graphs(s);
    return BCS_OK;
}

bcs_status bcs_surrogate_get_stats(bcs_surrogate* z, bcs_surrogate_stats* o) {
    if (!live(z) || !o) return BCS_ERR_INVALID_ARGUMENT;
    unsigned long long c[2] = {0, 0};
    BCS_CUDA(cudaStreamSynchronize(z->sim->stream));
    BCS_CUDA(cudaMemcpy(c, z->counts, sizeof(c), cudaMemcpyDeviceToHost));
    std::memset(o, 0, sizeof(*o));
    o->cells = z->cells;
    o->samples = z->stored;
    o->valid_samples = z->nvalid;
    o->predicted_cells = (int64_t)c[0];
    o->fallback_cells = (int64_t)c[1];
    o->iterations = z->iterations;
    o->last_loss = z->last_loss;
    o->parameters = z->net.param_count();
    o->tolerance = z->tolerance;
    // multiply-adds x 2 of one forward pass over one cell
    const double n = z->pic, e = z->net.edges(), H = kHidden;
    o->flops_per_cell = 2.0 * (n * kFeatIn * H + z->net.layers() * (3.0 * n * H * H + n * kEdgeIn * H) + n * H * kOut) +
                        z->net.layers() * e * H;
    o->device_bytes = z->bytes + z->net.bytes();
    return BCS_OK;
}

bcs_status bcs_surrogate_reset_stats(bcs_surrogate* z) {
    if (!live(z)) return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaMemsetAsync(z->counts, 0, 2 * sizeof(unsigned long long), z->sim->stream));
    return BCS_OK;
}

int64_t bcs_surrogate_param_count(bcs_surrogate* z) { return z ? z->net.param_count() : 0; }

bcs_status bcs_surrogate_get_params(bcs_surrogate* z, float* out, int64_t count) {
    if (!live(z) || !out || count != z->net.param_count()) return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaStreamSynchronize(z->sim->stream));
    BCS_CUDA(cudaMemcpy(out, z->net.params(), sizeof(float) * count, cudaMemcpyDeviceToHost));
    return BCS_OK;
}

bcs_status bcs_surrogate_set_params(bcs_surrogate* z, const float* in, int64_t count) {
    if (!live(z) || !in || count != z->net.param_count()) return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaMemcpyAsync(z->net.params(), in, sizeof(float) * count, cudaMemcpyHostToDevice, z->sim->stream));
    z->net.refresh_bf16();
    BCS_CUDA(cudaStreamSynchronize(z->sim->stream));
    return check_last();
}

bcs_status bcs_surrogate_loss_grad(bcs_surrogate* z, int cells, const float* features, const float* edge_features,
                                   const float* targets, float* loss, float* grads) {
    if (!live(z) || cells < 1 || cells > z->net.max_cells() || !features || !edge_features || !targets)
        return BCS_ERR_INVALID_ARGUMENT;
    cudaStream_t st = z->sim->stream;
    const size_t n = (size_t)cells * z->pic;
    BCS_CUDA(cudaMemcpyAsync(z->net.input_buf(), features, sizeof(float) * n * kFeatIn, cudaMemcpyHostToDevice, st));
    BCS_CUDA(cudaMemcpyAsync(z->net.edge_buf(), edge_features, sizeof(float) * (size_t)cells * z->net.edges() * kEdgeIn,
                             cudaMemcpyHostToDevice, st));
    BCS_CUDA(cudaMemcpyAsync(z->net.target_buf(), targets, sizeof(float) * n * kOut, cudaMemcpyHostToDevice, st));
    const unsigned expired = bcs_tensor_wait_expiries();
    z->net.forward(z->net.input_buf(), z->net.edge_buf(), cells, true);
    z->net.backward(z->net.target_buf(), cells);
    if (loss) BCS_CUDA(cudaMemcpyAsync(loss, z->net.loss_dev(), sizeof(float), cudaMemcpyDeviceToHost, st));
    if (grads)
        BCS_CUDA(cudaMemcpyAsync(grads, z->net.grad(), sizeof(float) * z->net.param_count(), cudaMemcpyDeviceToHost, st));
    BCS_CUDA(cudaStreamSynchronize(st));
    bcs_status r = check_last();
    if (r == BCS_OK && bcs_tensor_wait_expiries() != expired) r = BCS_ERR_TIMEOUT;
    return r;
}

bcs_status bcs_surrogate_forward(bcs_surrogate* z, int cells, const float* features, const float* edge_features,
                                 float* outputs) {
    if (!live(z) || cells < 1 || cells > z->net.max_cells() || !features || !edge_features || !outputs)
        return BCS_ERR_INVALID_ARGUMENT;
    cudaStream_t st = z->sim->stream;
    const size_t n = (size_t)cells * z->pic;
    BCS_CUDA(cudaMemcpyAsync(z->net.input_buf(), features, sizeof(float) * n * kFeatIn, cudaMemcpyHostToDevice, st));
    BCS_CUDA(cudaMemcpyAsync(z->net.edge_buf(), edge_features, sizeof(float) * (size_t)cells * z->net.edges() * kEdgeIn,
                             cudaMemcpyHostToDevice, st));
    const unsigned expired = bcs_tensor_wait_expiries();
    z->net.forward(z->net.input_buf(), z->net.edge_buf(), cells, false);
    BCS_CUDA(cudaMemcpyAsync(outputs, z->net.output(), sizeof(float) * n * kOut, cudaMemcpyDeviceToHost, st));
    BCS_CUDA(cudaStreamSynchronize(st));
    bcs_status r = check_last();
    if (r == BCS_OK && bcs_tensor_wait_expiries() != expired) r = BCS_ERR_TIMEOUT;
    return r;
}

bcs_status bcs_surrogate_evaluate(bcs_surrogate* z, int first, int count, double* net_error, double* base_error) {
    if (!live(z) || first < 0 || count < 1 || first + count > z->stored || !z->scales_set) return BCS_ERR_INVALID_ARGUMENT;
    cudaStream_t st = z->sim->stream;
    ScopedDevice scratch;
    BCS_CUDA(cudaMalloc(&scratch.p, 3 * sizeof(double)));
    double* sums = scratch.as<double>();
    BCS_CUDA(cudaMemsetAsync(sums, 0, 3 * sizeof(double), st));
    for (int b = first; b < first + count; b += z->net.max_cells()) {
        const int n = std::min(z->net.max_cells(), first + count - b);
        launch_sur_inputs(z->ds_raw, nullptr, nullptr, 0, 0, b, n, z->pic, z->net.dev_adj_off(), z->net.dev_adj_nbr(),
                          z->net.dev_adj_len(), z->scales, z->net.input_buf(), z->net.edge_buf(), nullptr, st);
        z->net.forward(z->net.input_buf(), z->net.edge_buf(), n, false);
        launch_sur_eval(z->net.output(), z->ds_t, z->ds_valid, z->scales, b, n, z->pic, sums, st);
    }
    double h[3] = {0, 0, 0};
    cudaError_t e = cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return BCS_ERR_CUDA;
    if (h[2] <= 0) return BCS_ERR_INVALID_ARGUMENT;
    if (net_error) *net_error = h[0] / h[2];
    if (base_error) *base_error = h[1] / h[2];
    return check_last();
}

int bcs_set_tensor_path(int path) {
    if (path != 0 && path != 1) return -1;
    const int prev = mpnn_gemm_path();
    mpnn_set_gemm_path(path);
    return prev;
}

bcs_status bcs_set_tensor_wait_probe(int polls) {
    if (polls < 0) return BCS_ERR_INVALID_ARGUMENT;
    return mpnn_set_wait_probe(polls) ? BCS_OK : BCS_ERR_CUDA;
}

unsigned bcs_tensor_wait_expiries(void) {
    unsigned h = 0;
    // the word is written by kernels on the simulations' own streams
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(&h, mpnn_gemm_error_word(), sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
        return 0xFFFFFFFFu;
    return h;
}

bcs_status bcs_surrogate_set_scales(bcs_surrogate* z, const float* in) {
    if (!live(z) || !in) return BCS_ERR_INVALID_ARGUMENT;
    BCS_CUDA(cudaStreamSynchronize(z->sim->stream));
    std::memcpy(&z->scales, in, sizeof(SurScales));
    z->scales_set = true;
    drop_graphs(z->sim);   // captured macro steps hold the old scales
    return BCS_OK;
}

bcs_status bcs_surrogate_get_scales(bcs_surrogate* z, float* out) {
    if (!live(z) || !out) return BCS_ERR_INVALID_ARGUMENT;
    std::memcpy(out, &z->scales, sizeof(SurScales));
    return z->scales_set ? BCS_OK : BCS_ERR_INVALID_ARGUMENT;
}

}  // extern "C"
