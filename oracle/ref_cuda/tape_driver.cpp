// tape_driver.cpp — records the reference's own construction and frame
// launches as a tape (test infrastructure, see tape_shim.h).  Compiled with
// g++ together with the reference's hot-path translation units
// (grids/uniform_grid.cu, objects/blood_cells.cu, objects/vein_triangles.cu,
// objects/vein_neighbors.cu, utilities/cuda_vec3.cu,
// simulation/vein_collisions.cu), whose launches and key sort the recipe
// routes to the recorder, and against a generated src/config set.
//
// What the driver restates, as the CPU pin's driver does: the construction
// of src/main.cu:122-138 and SimulationController's constructor
// (simulation_controller.cu:27-54: one stream per cell type, the bounding
// spheres of generateBoundingSpheres, :93-153, in a zero-padded table) without
// the curand start (the replay injects a seeded state into the buffers marked
// here), and the frame
// of src/main.cu:175-208: calculateGrid for both grids, calculateNextFrame
// (simulation_controller.cu:246-294) and propagateAll (:315-323), with the
// reference's device synchronisations, without HandleVeinEnd (the recorded
// scenes set useBloodFlow = 0).
//
// Usage: tape_driver <out.tape> <reference|pinned> <frames>
//   reference: the reference's calls exactly (timing);
//   pinned: also the Q5 clears before each grid build and the last occupied
//           cell's range after it, as the CPU pin does (parity).
//        tape_driver --replay-cpu <tape> <state.bin|-> <frames> <out.bin>
//   runs a tape this executable recorded on the CPU (tape_runtime.cpp).
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "grids/uniform_grid.cuh"
#include "meta_factory/blood_cell_factory.hpp"
#include "meta_factory/vein_factory.hpp"
#include "objects/blood_cells.cuh"
#include "objects/vein_triangles.cuh"
#include "simulation/particle_collisions.cuh"
#include "simulation/vein_collisions.cuh"
#include "utilities/cuda_threads.hpp"

static bool g_pinned = false;

// main.cu:175-176 (UniformGrid::calculateGrid, uniform_grid.cu:129-155)
static void calculate_grid(UniformGrid& g, const cudaVec3& pos, int n) {
    if (g_pinned) {
        cudaMemset(g.gridCellStarts[0], 0, sizeof(int) * (size_t)g.cellCount);
        cudaMemset(g.gridCellEnds[0], 0xFF, sizeof(int) * (size_t)g.cellCount);
    }
    g.calculateGrid(pos, n);
    if (g_pinned) bcs_tape_fix_last_cell(g.gridCellIds[0], n, g.gridCellStarts[0], g.gridCellEnds[0]);
}

static void mark_vec3(const char* name, const cudaVec3& v, int n) {
    const std::string s(name);
    bcs_tape_mark_buffer((s + ".x").c_str(), v.x, sizeof(float) * (size_t)n);
    bcs_tape_mark_buffer((s + ".y").c_str(), v.y, sizeof(float) * (size_t)n);
    bcs_tape_mark_buffer((s + ".z").c_str(), v.z, sizeof(float) * (size_t)n);
}

int bcs_tape_replay_cpu(const char* tape, const char* state, int frames, const char* out);

int main(int argc, char** argv) {
    if (argc == 6 && std::strcmp(argv[1], "--replay-cpu") == 0)
        return bcs_tape_replay_cpu(argv[2], argv[3], std::atoi(argv[4]), argv[5]);
    if (argc < 4) {
        std::fprintf(stderr, "usage: tape_driver <out.tape> <reference|pinned> <frames>\n");
        return 1;
    }
    g_pinned = std::strcmp(argv[2], "pinned") == 0;
    const int frames = std::atoi(argv[3]);

    // ---- objects (src/main.cu:122-132)
    BloodCells bloodCells;
    VeinTriangles triangles;
    UniformGrid particleGrid(0, particleCount, cellWidth, cellHeight, cellDepth);
    UniformGrid triangleGrid(0, triangleCount, cellWidthTriangles, cellHeightTriangles, cellDepthTriangles);

    // ---- SimulationController's constructor without the curand start
    std::array<cudaStream_t, bloodCellTypeCount> streams{};
    for (auto& s : streams) cudaStreamCreate(&s);
    // The bounding-sphere table, with particleDistinctCellsCount zeros in
    // front: the collision kernel indexes it with the launching type's model
    // start and size for the particle of any sorted slot in the type's range
    // (particle_collisions.cuh:124), which for a particle of an earlier type
    // is a negative remainder, up to one model size before the table (Q15).
    // The padding keeps those reads inside the allocation.
    float* spheres_mem = nullptr;
    cudaMalloc(reinterpret_cast<void**>(&spheres_mem), sizeof(float) * 2 * particleDistinctCellsCount);
    float* spheres_dev = spheres_mem + particleDistinctCellsCount;
    {
        // generateBoundingSpheres (simulation_controller.cu:93-153), restated
        // on the compile-time models
        std::vector<float> hm[3];
        for (auto& h : hm) h.reserve(particleDistinctCellsCount);
        mp_for_each<mp_iota_c<bloodCellTypeCount>>([&](auto i) {
            using Def = mp_at_c<BloodCellList, i>;
            mp_for_each<mp_iota_c<Def::particlesInCell>>([&](auto j) {
                using V = mp_at_c<typename Def::Vertices, j>;
                hm[0].push_back(V::x);
                hm[1].push_back(V::y);
                hm[2].push_back(V::z);
            });
        });
        std::vector<float> spheres(particleDistinctCellsCount, std::numeric_limits<float>::max());
        std::vector<float> radii(particleDistinctCellsCount);
        for (int i = 0; i < bloodCellTypeCount; ++i) {
            const int start = bloodCellModelStarts[i];
            const int size = i + 1 == bloodCellTypeCount ? particleDistinctCellsCount - bloodCellModelStarts[i]
                                                         : bloodCellModelStarts[i + 1] - bloodCellModelStarts[i];
            float3 center{0, 0, 0};
            for (int j = 0; j < size; ++j) {
                for (int k = 0; k < size; ++k) {
                    if (j == k) continue;
                    float l = sqrt(pow((hm[0][start + j] - hm[0][start + k]), 2) +
                                   pow((hm[1][start + j] - hm[1][start + k]), 2) +
                                   pow((hm[2][start + j] - hm[2][start + k]), 2)) /
                              (2 * boundingSpheresCoeff);
                    if (l < spheres[start + j]) spheres[start + j] = l;
                }
                center = center + make_float3(hm[0][start + j], hm[1][start + j], hm[2][start + j]);
            }
            center = center / size;
            for (int j = 0; j < size; ++j)
                radii[start + j] = length(make_float3(hm[0][start + j], hm[1][start + j], hm[2][start + j]) - center);
        }
        cudaMemcpy(spheres_dev, spheres.data(), sizeof(float) * spheres.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(bloodCells.initialRadiuses[0], radii.data(), sizeof(float) * radii.size(), cudaMemcpyHostToDevice);
    }
    cudaDeviceSynchronize();

    // buffers the replay fills with the seeded state or reads back
    mark_vec3("positions", bloodCells.particles.positions[0], particleCount);
    mark_vec3("velocities", bloodCells.particles.velocities[0], particleCount);
    mark_vec3("forces", bloodCells.particles.forces[0], particleCount);
    mark_vec3("vein_positions", triangles.positions[0], VeinTriangles::vertexCount);
    mark_vec3("vein_velocities", triangles.velocities[0], VeinTriangles::vertexCount);
    bcs_tape_mark_buffer("particle_keys", particleGrid.gridCellIds[0], sizeof(int) * (size_t)particleCount);
    bcs_tape_mark_buffer("particle_ids", particleGrid.particleIds[0], sizeof(int) * (size_t)particleCount);
    // the folded type order (blood_cell_factory.hpp:117-162 merges and sorts
    // the user's types), which the injected state must follow:
    // "layout:pic,count,first particle;..."
    {
        std::string layout = "layout:";
        mp_for_each<mp_iota_c<bloodCellTypeCount>>([&](auto i) {
            using Def = mp_at_c<BloodCellList, i>;
            layout += std::to_string(Def::particlesInCell) + "," + std::to_string(Def::count) + "," +
                      std::to_string(particleStarts[i]) + ";";
        });
        bcs_tape_mark(layout.c_str());
    }
    bcs_tape_mark("setup_end");

    CudaThreads veinTrianglesThreads(triangleCount);
    CudaThreads bloodCellsThreads(particleCount);
    CudaThreads veinVerticesThreads(VeinTriangles::vertexCount);
    for (int f = 0; f < frames; ++f) {
        bcs_tape_mark("frame");
        calculate_grid(particleGrid, bloodCells.particles.positions[0], particleCount);
        calculate_grid(triangleGrid, triangles.centers, triangleCount);
        // calculateNextFrame, single-GPU branch (simulation_controller.cu:254-294)
        triangles.gatherForcesFromNeighbors(0, verticesGpuStarts[0], verticesGpuEnds[0], veinTrianglesThreads.blocks,
                                            veinTrianglesThreads.threadsPerBlock);
        cudaDeviceSynchronize();
        bloodCells.gatherForcesFromNeighbors(0, bloodCellGpuStarts[0], bloodCellGpuEnds[0], particleGpuStarts[0],
                                             particleGpuEnds[0], streams);
        cudaDeviceSynchronize();
        mp_for_each<mp_iota_c<bloodCellTypeCount>>([&](auto i) {
            using Def = mp_at_c<BloodCellList, i>;
            constexpr int particlesStart = particleStarts[i];
            constexpr int modelStart = bloodCellModelStarts[i];
            CudaThreads threads(Def::count * Def::particlesInCell);
            bcs_tape_launch(bcs_cfg(threads.blocks, threads.threadsPerBlock, 0, streams[i]),
                            sim::calculateParticleCollisions<UniformGrid>, 0, particleGpuStarts[0],
                            particleGpuEnds[0], bloodCells, particleGrid, spheres_dev, Def::count,
                            Def::particlesInCell, modelStart, particlesStart);
        });
        cudaDeviceSynchronize();
        mp_for_each<mp_iota_c<bloodCellTypeCount>>([&](auto i) {
            using Def = mp_at_c<BloodCellList, i>;
            constexpr int particlesStart = particleStarts[i];
            constexpr int modelStart = bloodCellModelStarts[i];
            CudaThreads threads(Def::count * Def::particlesInCell);
            bcs_tape_launch(bcs_cfg(threads.blocks, threads.threadsPerBlock, 0, streams[i]),
                            sim::detectVeinCollisions<UniformGrid>, 0, particleGpuStarts[0], particleGpuEnds[0],
                            bloodCells, triangles, triangleGrid, spheres_dev, Def::count, Def::particlesInCell,
                            modelStart, particlesStart);
        });
        cudaDeviceSynchronize();
        // propagateAll (simulation_controller.cu:315-323)
        bloodCells.propagateForcesIntoPositions(bloodCellsThreads.blocks, bloodCellsThreads.threadsPerBlock);
        cudaDeviceSynchronize();
        triangles.propagateForcesIntoPositions(veinVerticesThreads.blocks, veinVerticesThreads.threadsPerBlock);
        cudaDeviceSynchronize();
        bcs_tape_mark("frame_end");
    }
    if (bcs_tape_write(argv[1])) {
        std::perror(argv[1]);
        return 2;
    }
    return 0;
}
