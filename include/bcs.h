/*
 * bcs.h — C ABI of the GB300-native blood-cell physics step.
 *
 * This is the drop-in boundary for the per-frame physics of
 * GPU-Blood-Cell-Simulation/Simulation-Server.  The reference has no runtime
 * API: its scene is compile-time (the headers of src/config folded by
 * the headers of src/meta_factory) and its step is a sequence of member calls in
 * src/main.cu.  Each entry point below states which reference construct it
 * replaces (paths are relative to the reference project root).
 *
 * Conventions
 *  - Every call returns bcs_status; nothing exits the process or prints.
 *  - The library owns its device buffers.  A handle is used by one host
 *    thread at a time; different handles are independent.
 *  - All device work is enqueued on the handle's stream.  Inside a frame the
 *    library forks independent work onto an internal stream of the handle
 *    and joins it back before the frame's last operation, so the handle's
 *    stream orders every call as if it ran all the work.  Getters that write
 *    host memory synchronise that stream.
 *  - Vectors cross the boundary as three SoA float arrays, the layout of the
 *    reference's cudaVec3 (src/utilities/cuda_vec3.cuh:11-72).
 *  - Plain pointers and sizes only; no C++ or framework types.
 */
#ifndef BCS_H
#define BCS_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BCS_ABI_VERSION 3

typedef struct bcs_sim bcs_sim;

typedef enum bcs_status {
    BCS_OK = 0,
    BCS_ERR_INVALID_ARGUMENT = 1, /* malformed scene, bad pointer or size   */
    BCS_ERR_CUDA = 2,             /* a CUDA runtime call failed             */
    BCS_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed               */
    BCS_ERR_NO_DEVICE = 4,        /* no CUDA device / extension unusable    */
    BCS_ERR_UNSUPPORTED = 5,      /* valid request the library cannot serve */
    BCS_ERR_TIMEOUT = 6           /* a bounded device wait gave up; the work
                                     it guarded was skipped                 */
} bcs_status;

/* Grid choice, replaces `using Grid = std::variant<UniformGrid*, NoGrid*>`
 * (src/grids/grid_definition.hpp:6) and the UNIFORM_TRIANGLES_GRID switch
 * (src/main.cu:44,130-135). */
typedef enum bcs_grid_kind {
    BCS_GRID_UNIFORM = 0,
    BCS_GRID_NONE = 1
} bcs_grid_kind;

typedef enum bcs_memory {
    BCS_MEM_HOST = 0,
    BCS_MEM_DEVICE = 1
} bcs_memory;

/* Bits of the device error word (bcs_get_error_word). */
enum {
    BCS_ERRW_OUT_OF_GRID = 1u << 0,  /* a position fell outside the grid box; its
                                        key was clamped (the reference only prints,
                                        src/grids/uniform_grid.cu:26-29)            */
    BCS_ERRW_NAN_NORMALIZE = 1u << 1,/* normalize() of a zero vector returned 0
                                        (src/utilities/math.cuh:95-104)             */
    BCS_ERRW_NONFINITE = 1u << 2     /* a non-finite position or velocity appeared */
};

/* Three SoA arrays, the layout of the reference's cudaVec3. */
typedef struct bcs_vec3 {
    float* x;
    float* y;
    float* z;
} bcs_vec3;

/* One blood-cell type, replaces BloodCellDef<Count, ParticlesInCell,
 * IndicesInCell, Color, Springs, Vertices, Indices, Normals>
 * (src/meta_factory/blood_cells_def_type.hpp:21-31).  Types are laid out in
 * the order given (the reference's folded, sorted BloodCellList,
 * src/meta_factory/blood_cell_factory.hpp:117-162); particles are cell-major
 * inside a type. */
typedef struct bcs_cell_type {
    int count;                    /* cells of this type                        */
    int particles_in_cell;        /* model vertices per cell                   */
    const float* vertices;        /* [particles_in_cell][3] model positions    */
    int spring_count;
    const int* springs;           /* [spring_count][2] (start, end), Spring<> */
    const float* spring_lengths;  /* [spring_count] rest lengths; a length of
                                     0 means "no spring" as in the dense graph
                                     (src/objects/blood_cells.cu:14)          */
    const float* collision_radius;/* optional [particles_in_cell] collision
                                     radii; NULL derives them like
                                     generateBoundingSpheres
                                     (src/simulation/simulation_controller.cu:93-153) */
} bcs_cell_type;

/* The vein mesh, replaces veinPositions / veinIndices / VeinEndingCenters /
 * VeinEndingRadii (src/config/vein_definition.hpp:12,15965,31768-31776). */
typedef struct bcs_vein {
    int vertex_count;
    const float* positions;       /* [vertex_count][3]                         */
    int triangle_count;
    const uint32_t* indices;      /* [triangle_count][3]                       */
    int ending_count;
    const float* ending_centers;  /* [ending_count][3]                         */
    const float* ending_radii;    /* [ending_count]                            */
} bcs_vein;

/* Axial flow force of one vessel segment (no reference counterpart: the
 * reference applies the constant G of src/config/physics.hpp:32-34).  A
 * particle takes the segment whose axis is nearest; the force along the
 * segment axis is peak_force * max(0, 1 - r^2 / radius^2). */
typedef struct bcs_flow_segment {
    float origin[3];
    float direction[3];           /* unit axis, downstream                     */
    float length;
    float radius;
    float peak_force;
} bcs_flow_segment;

/* Scalar scene constants.  Names follow src/config/simulation.hpp:3-21 and
 * src/config/physics.hpp:4-34; bcs_default_params fills the reference's
 * shipped values. */
typedef struct bcs_params {
    float dt;
    int   use_blood_flow;
    int   enable_reaction_force;
    int   enable_big_cells_brake;
    float cell_width, cell_height, cell_depth;                   /* particle grid */
    float cell_width_triangles, cell_height_triangles, cell_depth_triangles;
    float bounding_spheres_coeff;
    float grid_y_margin;
    float grid_xz_margin;
    float min_spawn_y;
    float velocity_collision_damping;
    float particle_k_sniff;
    float vein_k_sniff;
    float particle_d_fact;
    float vein_d_fact;
    float vein_collision_force_intensity;
    float viscous_damping;
    float collision_spring_coeff;
    float collision_damping_coeff;
    float collision_shear_coeff;
    float max_cell_size_factor_before_brake;
    float big_particle_braking_intensity;
    float init_velocity[3];
    float vein_impact_distance;
    float vein_impact_minimal_force_distance;
    float gravity[3];                  /* Gx, Gy, Gz                              */
    float cylinder_radius;             /* respawn spread, vein_factory.hpp:88    */
    int   particle_grid;               /* bcs_grid_kind                           */
    int   triangle_grid;               /* bcs_grid_kind                           */
    int   vein_dynamic;                /* 1: vein springs + integration (the
                                          reference); 0: fixed wall              */
    int   refresh_triangle_centers;    /* 1: rebuild the triangle grid from the
                                          moved mesh every step (the reference's
                                          MULTI_GPU behaviour, main.cu:168-171);
                                          0: centres from the initial mesh, as
                                          its single-GPU loop does              */
    uint64_t seed;                     /* respawn RNG (Philox4x32-10)             */
} bcs_params;

typedef struct bcs_scene_desc {
    int type_count;
    const bcs_cell_type* types;
    bcs_vein vein;
    int flow_segment_count;
    const bcs_flow_segment* flow_segments;
    bcs_params params;
} bcs_scene_desc;

/* Sizes and grid geometry derived at creation (the meta_factory constants
 * particleCount, bloodCellCount, minX..maxZ, cellCountX.. of
 * blood_cell_factory.hpp:172-192, vein_factory.hpp:46-86,
 * uniform_grid.cu:83-104). */
typedef struct bcs_info {
    int particle_count;
    int blood_cell_count;
    int type_count;
    int vertex_count;
    int triangle_count;
    float min_x, max_x, min_y, max_y, min_z, max_z;
    int cell_count_x, cell_count_y, cell_count_z;              /* particle grid */
    int64_t cell_count;
    int tri_cell_count_x, tri_cell_count_y, tri_cell_count_z;  /* triangle grid */
    int64_t tri_cell_count;
    int64_t steps_done;
    size_t device_bytes;
    int kernels_per_step;          /* kernel nodes in one captured frame (0
                                      until the first bcs_step replay)      */
    int scene_count;               /* scenes in the simulation (1 unless
                                      built by bcs_create_batch); the bounds
                                      and per-axis cell counts above are
                                      scene 0's, the cell counts are totals */
} bcs_info;

/* One scene of a batch.  Particles, blood cells, vertices and triangles of
 * the scenes lie back to back in the batch-wide arrays (scene-major), in
 * the order of the descriptors given to bcs_create_batch.  The grid keys of
 * scene k are its own calculateIdForCell keys plus cell_key_offset. */
typedef struct bcs_scene_info {
    int particle_start, particle_count;
    int blood_cell_start, blood_cell_count;
    int vertex_start, vertex_count;
    int triangle_start, triangle_count;
    float min_x, max_x, min_y, max_y, min_z, max_z;
    int cell_count_x, cell_count_y, cell_count_z;
    int64_t cell_count, cell_key_offset;
    int tri_cell_count_x, tri_cell_count_y, tri_cell_count_z;
    int64_t tri_cell_count, tri_cell_key_offset;
} bcs_scene_info;

/* Fill *p with the reference's shipped constants (src/config/physics.hpp, simulation.hpp). */
void bcs_default_params(bcs_params* p);

const char* bcs_status_string(bcs_status s);
int bcs_abi_version(void);

/* Make `device` current for the calling thread in the library's CUDA
 * runtime (the library links its own runtime, so a caller's cudaSetDevice
 * through another runtime copy does not reach it).  Replaces the
 * cudaSetDevice(0) of src/main.cu:58. */
bcs_status bcs_set_device(int device);

/* Build the scene on the current CUDA device.  Replaces the constructors in
 * src/main.cu:122-138 (BloodCells, VeinTriangles, UniformGrid x2,
 * SimulationController) minus the curand seeding: initial particle state
 * comes from bcs_set_particles.  `stream` is a cudaStream_t or NULL (the
 * library then creates its own non-blocking stream). */
bcs_status bcs_create(const bcs_scene_desc* desc, void* stream, bcs_sim** out);

/* Build `scene_count` independent scenes as one simulation: every kernel of
 * a frame runs once over all scenes (one sort, one step launch), and each
 * scene computes exactly what it computes alone under bcs_create.  The
 * scenes must share every physics constant of bcs_params except the grid
 * cell sizes and margins, cylinder_radius, min_spawn_y and seed, and share
 * the grid kinds.  The whole batch holds fewer than 2^30 particles, and its
 * particle and triangle grids at most 2^31 - 1 cells each (keys are int32).
 * The reference runs one compile-time scene per process; this is the
 * batched form of src/main.cu:122-138. */
bcs_status bcs_create_batch(const bcs_scene_desc* descs, int scene_count, void* stream,
                            bcs_sim** out);
/* Waits for the handle's stream and for reads still in flight
 * (bcs_get_particles_async), then frees everything it allocated. */
bcs_status bcs_destroy(bcs_sim* sim);
bcs_status bcs_get_info(bcs_sim* sim, bcs_info* out);
bcs_status bcs_get_scene_info(bcs_sim* sim, int scene, bcs_scene_info* out);

/* How the frame is launched.  Every setting computes the same particle
 * state bit for bit (the per-particle arithmetic and its order do not depend
 * on it); only the speed changes.
 *   step_shape     launch shape of the fused step kernel, 0..BCS_STEP_SHAPES-1:
 *                  (threads per CTA, particles per CTA, CTAs per SM) =
 *                  0 (256, 512, 3), 1 (128, 256, 6), 2 (384, 768, 2),
 *                  3 (256, 512, 4), 4 (256, 512, 2), 5 (128, 256, 8).
 *                  The default is 3 (or the first shape that holds the
 *                  largest cell type).  A CTA holds whole
 *                  blood cells, so a shape needs particles_in_cell <= its
 *                  particles per CTA.
 *   persistent     0: one CTA per work item; 1: (SMs x resident CTAs) CTAs
 *                  that pull work items from a device counter.
 *   spatial_order  0: work items in cell-type order; 1: ordered by scene and
 *                  by the position of their first particle (y, then x, then
 *                  z, in 8-unit bricks), refreshed by bcs_set_particles, so
 *                  CTAs running together touch neighbouring cells.
 *   full_sort      0: each frame's grid sort starts from the previous
 *                  frame's order; 1: full radix sort every frame.
 *   occupancy_filter  1: keep a bitmap of the occupied particle-grid cells
 *                  (1 bit per cell) and let the collision stencil load only
 *                  the first and last occupied cell entries of each row.
 *   sorted_positions  1: the grid build also writes the positions in sorted
 *                  order, and the collision stencil reads its candidates
 *                  from there (contiguous) instead of through their ids. */
typedef struct bcs_tuning {
    int step_shape;
    int persistent;
    int spatial_order;
    int full_sort;
    int occupancy_filter;
    int sorted_positions;
    int grid_collisions;   /* particle collisions in grid order (a kernel of their own over
                              the sorted slots, before the step kernel), which implies the
                              sorted copies of positions and velocities: 0 = off (the step
                              kernel searches each stencil), 1 = each row's window found by
                              a linear scan from the row's first slot, 2 = by a binary
                              search of the row's keys, 3 = the same on the candidates
                              staged in shared memory per block of sorted slots */
} bcs_tuning;
#define BCS_STEP_SHAPES 6

bcs_status bcs_get_tuning(bcs_sim* sim, bcs_tuning* out);
bcs_status bcs_set_tuning(bcs_sim* sim, const bcs_tuning* tuning);

/* How a frame's grid sort runs (the reference's thrust::stable_sort_by_key,
 * src/grids/uniform_grid.cu:144-147, has no such choice; every mode gives
 * the same order, bit for bit).  0 (default) = by the number of particles
 * that changed cell in a recent frame: the incremental sort with its movers
 * sorted by one CTA while they fit one tile (4 096), by the multi-CTA radix
 * passes above that, and every pair sorted from scratch while more than half
 * the particles move; 1 = always incremental with the passes; 2 = always
 * incremental with one CTA (correct for any count, slow for many); 3 =
 * always from scratch.  Returns BCS_ERR_INVALID_ARGUMENT for another value. */
bcs_status bcs_set_mover_sort(bcs_sim* sim, int mode);

/* Autotuner: coordinate descent over the tuning fields (each field takes
 * every valid value with the others held, two sweeps), each trial timed on
 * `frames` fused frames after two warm-up frames, all starting from the
 * current state.  It keeps the fastest and restores the state, so the
 * simulation continues exactly as if the call had not happened.  Writes the choice to *chosen and its mean frame time to
 * *ms_per_frame (either may be NULL).  Allocates a state snapshot
 * (48 bytes per particle and per vein vertex) for the duration of the call. */
bcs_status bcs_autotune(bcs_sim* sim, int frames, bcs_tuning* chosen, float* ms_per_frame);

/* Particle state (positions, velocities, forces) as written by
 * setBloodCellsPositionsFromRandom (simulation_controller.cu:224-243) and
 * read by the renderer from bloodCells.particles.positions[0]
 * (main.cu:183-184).  A NULL forces.x zeroes the forces. */
bcs_status bcs_set_particles(bcs_sim* sim, bcs_vec3 positions, bcs_vec3 velocities,
                             bcs_vec3 forces, bcs_memory where);
bcs_status bcs_get_particles(bcs_sim* sim, bcs_vec3 positions, bcs_vec3 velocities,
                             bcs_vec3 forces, bcs_memory where);
/* The same read into host memory without waiting, for a renderer that
 * takes frame f while frame f + 1 is computed (the per-frame read of
 * main.cu:183-184, overlapped).  The state as bcs_get_particles would read
 * it now is converted on the simulation's stream and copied to the host
 * buffers (pinned memory for speed) on a copy stream; the call returns at
 * once and later frames run meanwhile.  The buffers must stay valid and
 * must not be read before bcs_wait_particles returns.  Two reads may be in
 * flight; a third makes the simulation's stream (not the host) wait for the
 * oldest.  A NULL component is skipped.  Allocates 36 bytes per particle
 * for each of two slots on first use. */
bcs_status bcs_get_particles_async(bcs_sim* sim, bcs_vec3 positions, bcs_vec3 velocities,
                                   bcs_vec3 forces);
/* Waits until every bcs_get_particles_async read has reached the host. */
bcs_status bcs_wait_particles(bcs_sim* sim);
/* Particles the step kernel set aside as crowded (more than 128 sorted slots
 * in their 27-cell collision stencil; a second kernel finishes them), summed
 * over every step since the simulation was created.  A diagnostic of piled-up
 * cells (no reference counterpart). */
bcs_status bcs_get_crowded(bcs_sim* sim, long long* particles);
/* Initial particle state on the device (no reference counterpart as an
 * API; the reference places its cells in SimulationController's
 * constructor).
 *   BCS_INIT_REFERENCE  the reference's rule (generateRandomPositonsAndVelocitiesKernel,
 *                       setBloodCellsPositionsFromRandom, simulation_controller.cu:176-220):
 *                       cell origin x, z uniform in +-0.6 cylinder_radius, y = min_spawn_y -
 *                       180 u min(N / 1000, 1); particles at origin + model vertex; velocity
 *                       init_velocity; overlaps allowed, as there.
 *   BCS_INIT_LATTICE    non-overlapping: cells at randomly chosen sites of a cubic lattice
 *                       (spacing 2 (bounding radius + collision radius) + gap) whose sphere
 *                       lies inside the lumen (the flow segments, or the cylinder of
 *                       cylinder_radius about the y axis); velocities init_velocity +
 *                       Gaussian(0, velocity_sigma) per component.
 * Random draws are Philox4x32-10 keyed by `seed` and the cell (particle) within its
 * scene, so a scene starts the same in a batch as alone.  Forces are zeroed. */
typedef enum bcs_init_kind { BCS_INIT_REFERENCE = 0, BCS_INIT_LATTICE = 1 } bcs_init_kind;
typedef struct bcs_init_desc {
    int kind;
    uint64_t seed;
    float velocity_sigma;   /* lattice only */
    float gap;              /* lattice only: extra spacing between cells */
} bcs_init_desc;
bcs_status bcs_init_particles(bcs_sim* sim, const bcs_init_desc* desc);

/* Vein vertex state (VeinTriangles positions/velocities/forces,
 * src/objects/vein_triangles.cuh:53-55).  NULL members are skipped. */
bcs_status bcs_set_vein(bcs_sim* sim, bcs_vec3 positions, bcs_vec3 velocities,
                        bcs_memory where);
bcs_status bcs_get_vein(bcs_sim* sim, bcs_vec3 positions, bcs_vec3 velocities,
                        bcs_vec3 forces, bcs_memory where);

/* ≙ particleGrid.calculateGrid(positions, particleCount) and
 *   triangleCentersGrid.calculateGrid(centers, triangleCount)
 *   (src/main.cu:175-176 → src/grids/uniform_grid.cu:129-155). */
bcs_status bcs_calculate_grids(bcs_sim* sim);
/* ≙ SimulationController::calculateNextFrame
 *   (src/simulation/simulation_controller.cu:246-313). */
bcs_status bcs_calculate_next_frame(bcs_sim* sim);
/* ≙ SimulationController::propagateAll (simulation_controller.cu:315-331). */
bcs_status bcs_propagate_all(bcs_sim* sim);
/* `nsteps` whole frames of grids → next frame → propagate (the loop body of
 * src/main.cu:158-247 minus rendering), fused and replayed from a CUDA graph.
 * Same results as the three calls above in sequence. */
bcs_status bcs_step(bcs_sim* sim, int nsteps);

/* Multi-rate macro steps (no reference counterpart): each of the `n` macro
 * steps advances `substeps` time steps of dt.  Sub-step 1 is the full frame
 * of bcs_step; the external part of its force (particle collisions and the
 * vein's force adjustment) is held for sub-steps 2..substeps, which
 * re-evaluate centroids, cell springs and environment, integrate, and apply
 * the vein-end rule (a respawned cell drops its held force).  Particle
 * impacts reach the vein mesh in sub-step 1; the mesh takes every sub-step.
 * With substeps = 1 this is bcs_step.  1 <= substeps <= BCS_MAX_SUBSTEPS. */
#define BCS_MAX_SUBSTEPS 64
bcs_status bcs_macro_step(bcs_sim* sim, int substeps, int n);

/* ---- Learned sub-steps (no reference counterpart) ------------------------
 * A message-passing network over one cell model's spring graph (3 layers,
 * hidden width 128, bfloat16 weights, FP32 accumulation; node messages
 * silu(h W_b + b_b) averaged over each node's springs, with the springs'
 * stretch and relative velocity along the spring as edge inputs) predicts a cell's
 * state after sub-steps 2..K of a macro step from the state after sub-step
 * 1: positions and velocities relative to the cell's centroid and mean
 * velocity, the current, held external and environment forces, and a
 * wall-proximity flag.  It is trained on the GPU, by the library's own
 * forward and backward kernels (Adam), on macro steps the plain sub-steps
 * computed.  While it is enabled, each macro step of K sub-steps predicts
 * every cell of the model and checks the prediction's residual: the
 * trapezoid rule over the span, |x_K - x_1 - (K-1) dt / 2 (v_1 + v_K)|,
 * per particle.  A cell whose residual exceeds the tolerance, or whose
 * prediction is not finite, falls back to the plain sub-steps.  The
 * vein-end rule runs once, on the predicted state. */
typedef struct bcs_surrogate bcs_surrogate;

typedef struct bcs_surrogate_desc {
    int cell_type;       /* type index (all types with the same cell model join) */
    int substeps;        /* K of the macro steps it serves, 2..BCS_MAX_SUBSTEPS */
    int layers;          /* message-passing layers, 1..4 (3) */
    int max_samples;     /* capacity of the training set, in cell-steps */
    uint64_t seed;       /* weights and training draws */
    float tolerance;     /* residual threshold in length units; 0 = 1e-3 x the
                            model's smallest collision radius */
    float huber_delta;   /* training loss: 0 = mean squared error, > 0 = pseudo-
                            Huber delta^2 (sqrt(1 + (d/delta)^2) - 1) on the
                            normalised outputs */
} bcs_surrogate_desc;

typedef struct bcs_surrogate_stats {
    int64_t cells;            /* cells of the model in the simulation */
    int64_t samples;          /* cell-steps collected */
    int64_t valid_samples;    /* of those, without a respawn */
    int64_t predicted_cells;  /* cell macro steps taken from the network */
    int64_t fallback_cells;   /* cell macro steps that fell back */
    int64_t iterations;       /* training iterations so far */
    int64_t parameters;
    float last_loss;          /* mean squared error of the last batch (normalised) */
    float tolerance;
    double flops_per_cell;    /* one forward pass over one cell */
    size_t device_bytes;
} bcs_surrogate_stats;

bcs_status bcs_surrogate_create(bcs_sim* sim, const bcs_surrogate_desc* desc, bcs_surrogate** out);
/* Either order of destruction is safe: bcs_destroy detaches the simulation's
 * surrogates, after which every call on them but this one returns
 * BCS_ERR_INVALID_ARGUMENT. */
bcs_status bcs_surrogate_destroy(bcs_surrogate* sur);
/* Run `macro_steps` plain macro steps of the surrogate's K and record every
 * cell of the model as a training sample (stops at the capacity). */
bcs_status bcs_surrogate_collect(bcs_surrogate* sur, int macro_steps);
/* `iterations` Adam steps on batches of `batch_cells` cells drawn from the
 * training set; *loss (optional) = the last batch's loss. */
bcs_status bcs_surrogate_train(bcs_surrogate* sur, int iterations, int batch_cells, float learning_rate,
                               float* loss);
/* Use the network in this simulation's macro steps of K sub-steps: on = 1
 * runs it as one fused kernel per macro step (a CTA per cell, the network
 * on chip), on = 2 as the layer-by-layer kernels the training uses, on = 0
 * stops using it. */
bcs_status bcs_surrogate_enable(bcs_surrogate* sur, int on);
bcs_status bcs_surrogate_get_stats(bcs_surrogate* sur, bcs_surrogate_stats* out);
bcs_status bcs_surrogate_reset_stats(bcs_surrogate* sur);
int64_t bcs_surrogate_param_count(bcs_surrogate* sur);
/* FP32 parameters, in the order W_in, b_in, then per layer W_b, b_b, W_e,
 * b_e, W_u, W_v, b_u, then W_out, b_out; matrices row-major [in][out]. */
bcs_status bcs_surrogate_get_params(bcs_surrogate* sur, float* params, int64_t count);
bcs_status bcs_surrogate_set_params(bcs_surrogate* sur, const float* params, int64_t count);
/* Loss (the training loss of the descriptor) and parameter gradients of the
 * network on given normalised host inputs: features [cells * pic][16], edge features [cells * edges][8] in
 * the order of the cell's spring lists, targets [cells * pic][9]. */
bcs_status bcs_surrogate_loss_grad(bcs_surrogate* sur, int cells, const float* features,
                                   const float* edge_features, const float* targets, float* loss,
                                   float* grads);
/* The network's outputs [cells * pic][9] on given normalised host inputs. */
bcs_status bcs_surrogate_forward(bcs_surrogate* sur, int cells, const float* features,
                                 const float* edge_features, float* outputs);
/* Mean position error (length units, per particle) after the network's
 * span on the stored samples [first, first + count): of its prediction
 * (*net_error) and of the constant-force extrapolation x_1 + T v_1 +
 * T^2/2 F_1 that it corrects (*base_error), against the plain sub-steps. */
bcs_status bcs_surrogate_evaluate(bcs_surrogate* sur, int first, int count, double* net_error,
                                  double* base_error);
/* Tensor-core instructions of the network's 128 x 128 products (training
 * and layer-by-layer inference): 0 = tcgen05 with tensor-memory
 * accumulators (the default; BCS_TENSOR_PATH=1 in the environment starts
 * with mma.sync), 1 = mma.sync.  Returns the previous setting,
 * or -1 for an invalid value.  bcs_tensor_wait_expiries counts the CTAs
 * whose tcgen05 completion was not seen within the kernel's bounded wait
 * (the product is then skipped, not stalled; the CTA still waits, bounded,
 * for the products it issued before it frees its tensor memory); it
 * synchronises the device first, or returns 0xFFFFFFFF when that fails.
 * bcs_surrogate_forward and bcs_surrogate_loss_grad return BCS_ERR_TIMEOUT
 * when the count grew during the call. */
int bcs_set_tensor_path(int path);
unsigned bcs_tensor_wait_expiries(void);
/* Testing aid with no counterpart in the reference: with polls > 0 the first
 * product wait of every CTA of the tcgen05 kernels polls, that many times,
 * an mbarrier that nothing arrives at, so it gives up as a lost completion
 * would and the give-up path runs; 0 restores the normal waits.
 * Synchronises the device. */
bcs_status bcs_set_tensor_wait_probe(int polls);
/* The normalisation derived from the training set: 53 floats (feature means
 * [16], feature 1/std [16], target medians [9], target robust spreads [9]
 * (1.4826 x the median absolute deviation), edge scales of position,
 * stretch and velocity along the spring). */
bcs_status bcs_surrogate_get_scales(bcs_surrogate* sur, float* out53);
/* Install a normalisation (as bcs_surrogate_get_scales writes it), e.g.
 * with parameters trained by another surrogate of the same model. */
bcs_status bcs_surrogate_set_scales(bcs_surrogate* sur, const float* in53);

/* Grid arrays for parity checks, the UniformGrid members gridCellIds,
 * particleIds, gridCellStarts, gridCellEnds (src/grids/uniform_grid.cuh:32-35)
 * after the last bcs_calculate_grids / bcs_step.  which = 0: particle grid,
 * 1: triangle grid.  cell_ids/object_ids hold `object count` entries (sorted
 * keys and the object ids they carry); cell_starts/cell_ends hold the grid's
 * cell count entries (inclusive ranges; empty cells read start 0, end -1).
 * Any pointer may be NULL. */
bcs_status bcs_get_grid(bcs_sim* sim, int which, int* cell_ids, int* object_ids,
                        int* cell_starts, int* cell_ends, bcs_memory where);

/* Headless replacement of the CUDA-GL interop kernels
 * calculatePositionsKernel / calculateTriangleVerticesKernel
 * (src/graphics/glcontroller.cu:22-49): particle vertices into a stride-6
 * buffer (xyz + 3 zeros), one instance offset (stride 3) per particle, and
 * vein vertices at stride 6.  NULL outputs are skipped. */
bcs_status bcs_export_render(bcs_sim* sim, float* particle_vbo, float* particle_offsets,
                             float* vein_vbo, bcs_memory where);

/* Sticky device error word (BCS_ERRW_* bits) accumulated since the last
 * clear; synchronises the stream. */
bcs_status bcs_get_error_word(bcs_sim* sim, uint32_t* out, int clear);
bcs_status bcs_synchronize(bcs_sim* sim);

/* Time `nsteps` of bcs_step on the device with CUDA events recorded on the
 * handle's stream; writes milliseconds.  For benchmarking. */
bcs_status bcs_time_steps(bcs_sim* sim, int nsteps, float* ms_out);
/* bcs_macro_step(sim, substeps, n) timed the same way. */
bcs_status bcs_time_macro_steps(bcs_sim* sim, int substeps, int n, float* ms_out);

/* Largest object count bcs_grid_sort_static accepts. */
#define BCS_GRID_SORT_STATIC_MAX 262144

/* Grid keys and their stable sort without allocating device memory.  This
 * entry point has no counterpart in the reference.  It is for callers that
 * cannot allocate: a host application that owns the whole device-memory
 * budget, or a frame loop that must not stall on cudaMalloc / cudaFree
 * (either can synchronise the device).  It needs no bcs_sim handle.
 *
 * x, y, z: device arrays of n positions (cudaVec3 layout).  bounds6: host
 * array (min_x, max_x, min_y, max_y, min_z, max_z), cell3: host array (cell
 * width, height, depth) — the values bcs_get_info / bcs_params carry.
 * cell_ids, object_ids: device outputs of n ints, the sorted keys and the
 * object ids they carry, equal to what bcs_get_grid returns for the same
 * positions.  The work is enqueued on `stream` (a cudaStream_t or NULL).
 *
 * Scratch lives in a fixed array inside the library (about 2.1 MiB, held by
 * every device that loads the library until exit); n above
 * BCS_GRID_SORT_STATIC_MAX returns BCS_ERR_INVALID_ARGUMENT.  The first call
 * on a device looks up that array's device address (cudaGetSymbolAddress)
 * with the device current; make that first call before any stream capture.
 * All calls share the array, so calls that overlap on the GPU race.
 * A position outside the grid box gets the key of the nearest edge cell,
 * exactly as on the allocating path; the call records that in the array's
 * error word (BCS_ERRW_OUT_OF_GRID), which bcs_grid_sort_static_error_word
 * reads back. */
bcs_status bcs_grid_sort_static(const float* x, const float* y, const float* z, int n, const float* bounds6,
                                const float* cell3, int* cell_ids, int* object_ids, void* stream);

/* Error word of the most recent bcs_grid_sort_static call on the current
 * device (0, or BCS_ERRW_OUT_OF_GRID when some position lay outside the grid
 * box), into *out.  Enqueued on `stream` after that call and synchronises
 * the stream; allocates nothing.  This entry point has no counterpart in
 * the reference (which only printf()s such positions, uniform_grid.cu:31-34). */
bcs_status bcs_grid_sort_static_error_word(void* stream, uint32_t* out);

/* ---- Control messages of the streaming server, without the network and
 * the renderer.  The reference's client sends one byte per message over
 * ENet (src/communication/server_endpoint.hpp:19-63, server_endpoint.cpp:
 * 6-8,140-185): the low seven bits name the event, the high bit is set for
 * "start" (a key pressed) and clear for "stop" (released).  Its
 * MsgController (msg_controller.cpp:27-148) handles at most one message per
 * frame.  Here a transport of the application's choosing posts the bytes it
 * receives and takes the bytes to send; a renderer reads the held events and
 * the render toggles. */
typedef enum bcs_event_type {
    BCS_EVENT_NO_MESSAGE = 0,
    BCS_EVENT_CAMERA_LEFT, BCS_EVENT_CAMERA_RIGHT, BCS_EVENT_CAMERA_FORWARD, BCS_EVENT_CAMERA_BACK,
    BCS_EVENT_CAMERA_ASCEND, BCS_EVENT_CAMERA_DESCEND,
    BCS_EVENT_CAMERA_ROTATE_LEFT, BCS_EVENT_CAMERA_ROTATE_RIGHT, BCS_EVENT_CAMERA_ROTATE_UP,
    BCS_EVENT_CAMERA_ROTATE_DOWN,
    BCS_EVENT_TOGGLE_POLYGON_MODE, BCS_EVENT_TOGGLE_SPRINGS_RENDERING, BCS_EVENT_TOGGLE_SPHERES_RENDERING,
    BCS_EVENT_STREAM_SUCCESSFULLY_ENDED, BCS_EVENT_STOP_RENDERING,
    BCS_EVENT_NEW_CONNECTION, BCS_EVENT_PEER_DISCONNECTED,
    BCS_EVENT_INVALID_MESSAGE
} bcs_event_type;   /* EventType, same values */
typedef enum bcs_event_state {
    BCS_EVENT_START = 0, BCS_EVENT_STOP = 1, BCS_EVENT_NOT_RELEVANT = 2
} bcs_event_state;  /* EventState */
typedef struct bcs_event {
    int32_t type;   /* bcs_event_type */
    int32_t state;  /* bcs_event_state */
} bcs_event;

/* parseEvent (server_endpoint.cpp:168-185): one message's bytes; a length
 * other than 1 or an unknown event gives BCS_EVENT_INVALID_MESSAGE. */
bcs_event bcs_event_decode(const uint8_t* data, size_t length);
/* SendEvent's byte (server_endpoint.cpp:140-163) into *byte; returns the
 * channel + 1 (2 for the important events streamSuccessfullyEnded and
 * stopRendering, 1 otherwise), or 0 for an invalid event. */
int bcs_event_encode(bcs_event event, uint8_t* byte);

/* The controller's state after a message. */
typedef struct bcs_control_state {
    uint32_t held;               /* bit t set while event t is held (started, not stopped) */
    int32_t polygon_mode_line;   /* togglePolygonMode: vein drawn as lines (starts as fill) */
    int32_t springs_rendering;   /* toggleSpringsRendering (starts on) */
    int32_t spheres_rendering;   /* toggleSpheresRendering (starts on) */
    int32_t stop_requested;      /* a stopRendering message was handled */
    int32_t connected;           /* newConnection seen, no peerDisconnected since */
    int64_t handled;             /* messages handled */
} bcs_control_state;

typedef struct bcs_control bcs_control;
bcs_status bcs_control_create(bcs_control** out);
void bcs_control_destroy(bcs_control* control);
/* Queue one received message (the bytes of one packet); thread-safe. */
bcs_status bcs_control_post(bcs_control* control, const uint8_t* data, size_t length);
/* Queue a transport event (BCS_EVENT_NEW_CONNECTION / PEER_DISCONNECTED with
 * BCS_EVENT_NOT_RELEVANT, as pollEvents reports them); thread-safe. */
bcs_status bcs_control_post_event(bcs_control* control, bcs_event event);
/* handleMsgs: handle the oldest queued message, if any, and write the
 * state.  A start adds the event to the held set; a stop removes it and then,
 * as in the reference (msg_controller.cpp:40-45), also takes the
 * single-message path: render toggles flip, stopRendering requests the end
 * of the run, peerDisconnected clears the held set. */
bcs_status bcs_control_handle(bcs_control* control, bcs_control_state* state_out);
/* Queue a message for the transport (SendEvent); bcs_control_take_outgoing
 * hands the queued bytes out in order, returning 0 when none is left. */
bcs_status bcs_control_send(bcs_control* control, bcs_event event);
int bcs_control_take_outgoing(bcs_control* control, uint8_t* byte);

/* The server loop of main.cu:158-245 without rendering and streaming: every
 * frame is bcs_step(sim, 1) (the grids, calculateNextFrame, propagateAll),
 * then one control message is handled (control may be NULL).  The loop ends
 * once a handled message requested the stop, or after the frame that takes
 * its frame count past max_frames (the count starts at 0, so max_frames + 1
 * frames, as in the reference); then streamSuccessfullyEnded is queued for
 * the transport (msg_controller.cpp:55-59).  Writes the frames run. */
bcs_status bcs_run(bcs_sim* sim, bcs_control* control, int max_frames, int* frames_run);

/* Phases of one frame timed by bcs_profile_steps. */
enum {
    BCS_PHASE_GRID = 0,         /* key sort + cell ranges                   */
    BCS_PHASE_VEIN_FORCES = 1,  /* vein spring gather                       */
    BCS_PHASE_COLLISIONS = 2,   /* grid-order particle collisions (empty when
                                   the step kernel searches the stencils)   */
    BCS_PHASE_PARTICLES = 3,    /* the particle step kernel (springs, vein
                                   ray, integration) and the vein-end rule  */
    BCS_PHASE_VEIN_UPDATE = 4,  /* vein integration + triangle cache         */
    BCS_PHASE_COUNT = 5
};

/* Run `nsteps` frames eagerly (no graph) with CUDA events between phases on
 * the handle's stream; adds each phase's milliseconds into
 * phase_ms[BCS_PHASE_COUNT].  Same results as bcs_step. */
bcs_status bcs_profile_steps(bcs_sim* sim, int nsteps, float* phase_ms);

#ifdef __cplusplus
}
#endif

#endif /* BCS_H */
