// ref_driver.cpp — headless host driver of the reference's own step (pin
// recipe, test infrastructure).  It is compiled together with the
// reference's hot-path translation units (grids/uniform_grid.cu,
// objects/blood_cells.cu, objects/vein_triangles.cu, objects/vein_neighbors.cu,
// utilities/cuda_vec3.cu, simulation/vein_collisions.cu), rewritten only so
// that their <<<>>> launches go through the serial CPU launch shim, and
// against a generated src/config set.  The reference's kernels, physics and
// grid code therefore run unmodified on the CPU.
//
// What the driver itself restates (it lives in simulation_controller.cu,
// which pulls curand and does not compile for the host):
//   * generateBoundingSpheres (simulation_controller.cu:93-153);
//   * the call order of calculateNextFrame / propagateAll
//     (simulation_controller.cu:246-331), single-GPU branch, without
//     HandleVeinEnd (the pinned scene sets useBloodFlow = 0);
//   * Q5: cellStarts = 0 / cellEnds = -1 before every calculateGrid, and the
//     last occupied cell's range (which calculateStartAndEndOfCellKernel
//     never writes correctly, uniform_grid.cu:78) recomputed afterwards.
//
// Usage: ref_driver <out_dir> [<state.bin> <steps>]
//   without a state file: dump the compile-time layout only;
//   with one: inject positions / velocities ([N][3] float32 each, then vein
//   [V][3] positions are taken from the config), run `steps` frames and dump
//   grids after the first grid build and the state after frame 1 and `steps`.
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

static std::string g_dir;

template <class T>
static void dump(const char* name, const T* p, size_t n) {
    std::string f = g_dir + "/" + name + ".bin";
    FILE* fp = std::fopen(f.c_str(), "wb");
    if (!fp) { std::perror(f.c_str()); std::exit(2); }
    std::fwrite(p, sizeof(T), n, fp);
    std::fclose(fp);
}

static void dump_vec3(const char* name, const cudaVec3& v, int n) {
    std::vector<float> a(3 * (size_t)n);
    for (int i = 0; i < n; ++i) { a[3 * i] = v.x[i]; a[3 * i + 1] = v.y[i]; a[3 * i + 2] = v.z[i]; }
    dump(name, a.data(), a.size());
}

static void calculate_grid(UniformGrid& g, const cudaVec3& pos, int n) {
    std::memset(g.gridCellStarts[0], 0, sizeof(int) * (size_t)g.cellCount);
    std::memset(g.gridCellEnds[0], 0xFF, sizeof(int) * (size_t)g.cellCount);
    g.calculateGrid(pos, n);
    const int* k = g.gridCellIds[0];
    int last = k[n - 1], first = n - 1;
    while (first > 0 && k[first - 1] == last) --first;
    g.gridCellStarts[0][last] = first;
    g.gridCellEnds[0][last] = n - 1;
}

static void dump_grid(const char* tag, const UniformGrid& g, int n) {
    std::string t(tag);
    dump((t + "_keys").c_str(), g.gridCellIds[0], n);
    dump((t + "_ids").c_str(), g.particleIds[0], n);
    dump((t + "_starts").c_str(), g.gridCellStarts[0], (size_t)g.cellCount);
    dump((t + "_ends").c_str(), g.gridCellEnds[0], (size_t)g.cellCount);
}

int main(int argc, char** argv) {
    if (argc < 2) { std::fprintf(stderr, "usage: ref_driver <out_dir> [state.bin steps]\n"); return 1; }
    g_dir = argv[1];

    // ---- compile-time layout (blood_cell_factory.hpp:172-328, vein_factory.hpp:12-86)
    int scalars_i[] = {particleCount, bloodCellCount, bloodCellTypeCount, particleDistinctCellsCount, totalGraphSize,
                       veinPositionCount, triangleCount};
    dump("layout_ints", scalars_i, sizeof(scalars_i) / sizeof(int));
    dump("particle_starts", particleStarts.data(), particleStarts.size());
    dump("cell_type_starts", bloodCellTypesStarts.data(), bloodCellTypesStarts.size());
    dump("model_starts", bloodCellModelStarts.data(), bloodCellModelStarts.size());
    dump("graph_starts", accumulatedGraphSizes.data(), accumulatedGraphSizes.size());
    dump("spring_graph", springGraph.data(), springGraph.size());
    float bounds[] = {minX, maxX, minY, maxY, minZ, maxZ, width, height, depth};
    dump("bounds", bounds, 9);
    std::vector<int> pics;
    std::vector<float> models;
    mp_for_each<mp_iota_c<bloodCellTypeCount>>([&](auto i) {
        using Def = mp_at_c<BloodCellList, i>;
        pics.push_back(Def::particlesInCell);
        pics.push_back(Def::count);
        mp_for_each<mp_iota_c<Def::particlesInCell>>([&](auto j) {
            using V = mp_at_c<typename Def::Vertices, j>;
            models.push_back(V::x);
            models.push_back(V::y);
            models.push_back(V::z);
        });
    });
    dump("type_pic_count", pics.data(), pics.size());
    dump("models", models.data(), models.size());

    // Vein neighbour tables from the reference's own builder (vein_factory.hpp:130-174).
    {
        auto t = calculateSpringLengths();
        const auto& ids = std::get<0>(t);
        const auto& len = std::get<1>(t);
        std::vector<int> a;
        std::vector<float> b;
        for (int k = 0; k < veinVertexMaxNeighbors; ++k) {
            a.insert(a.end(), ids[k].begin(), ids[k].end());
            b.insert(b.end(), len[k].begin(), len[k].end());
        }
        dump("vein_nb_ids", a.data(), a.size());
        dump("vein_nb_len", b.data(), b.size());
    }

    // ---- bounding spheres and initial radii (generateBoundingSpheres restated)
    std::vector<float> hm[3];
    for (auto& h : hm) h.resize(particleDistinctCellsCount);
    {
        size_t k = 0;
        for (int m = 0; m < particleDistinctCellsCount; ++m) {
            hm[0][m] = models[k++]; hm[1][m] = models[k++]; hm[2][m] = models[k++];
        }
    }
    std::vector<float> spheres(particleDistinctCellsCount, std::numeric_limits<float>::max());
    std::vector<float> radii(particleDistinctCellsCount);
    for (int i = 0; i < bloodCellTypeCount; ++i) {
        int start = bloodCellModelStarts[i];
        int size = i + 1 == bloodCellTypeCount ? particleDistinctCellsCount - bloodCellModelStarts[i]
                                               : bloodCellModelStarts[i + 1] - bloodCellModelStarts[i];
        float3 center{0, 0, 0};
        for (int j = 0; j < size; ++j) {
            for (int k = 0; k < size; ++k) {
                if (j == k) continue;
                float l = sqrt(pow((hm[0][start + j] - hm[0][start + k]), 2) + pow((hm[1][start + j] - hm[1][start + k]), 2) +
                               pow((hm[2][start + j] - hm[2][start + k]), 2)) / (2 * boundingSpheresCoeff);
                if (l < spheres[start + j]) spheres[start + j] = l;
            }
            center = center + make_float3(hm[0][start + j], hm[1][start + j], hm[2][start + j]);
        }
        center = center / size;
        for (int j = 0; j < size; ++j)
            radii[start + j] = length(make_float3(hm[0][start + j], hm[1][start + j], hm[2][start + j]) - center);
    }
    dump("bounding_spheres", spheres.data(), spheres.size());
    dump("initial_radii", radii.data(), radii.size());
    if (argc < 4) return 0;

    // ---- objects (src/main.cu:122-132)
    BloodCells bloodCells;
    VeinTriangles triangles;
    UniformGrid particleGrid(0, particleCount, cellWidth, cellHeight, cellDepth);
    UniformGrid triangleGrid(0, triangleCount, cellWidthTriangles, cellHeightTriangles, cellDepthTriangles);
    std::memcpy(bloodCells.initialRadiuses[0], radii.data(), sizeof(float) * radii.size());
    float* boundingSpheresModel = spheres.data();
    int dims[] = {particleGrid.cellCountX, particleGrid.cellCountY, particleGrid.cellCountZ,
                  triangleGrid.cellCountX, triangleGrid.cellCountY, triangleGrid.cellCountZ};
    dump("grid_dims", dims, 6);

    // ---- injected state
    std::vector<float> st(6 * (size_t)particleCount);
    FILE* fp = std::fopen(argv[2], "rb");
    if (!fp || std::fread(st.data(), sizeof(float), st.size(), fp) != st.size()) {
        std::fprintf(stderr, "bad state file\n");
        return 2;
    }
    std::fclose(fp);
    cudaVec3& P = bloodCells.particles.positions[0];
    cudaVec3& Vv = bloodCells.particles.velocities[0];
    cudaVec3& F = bloodCells.particles.forces[0];
    for (int i = 0; i < particleCount; ++i) {
        P.x[i] = st[3 * i]; P.y[i] = st[3 * i + 1]; P.z[i] = st[3 * i + 2];
        const float* v = &st[3 * (size_t)particleCount + 3 * i];
        Vv.x[i] = v[0]; Vv.y[i] = v[1]; Vv.z[i] = v[2];
        F.x[i] = F.y[i] = F.z[i] = 0.0f;
    }
    const int steps = std::atoi(argv[3]);
    std::array<cudaStream_t, bloodCellTypeCount> streams{};
    CudaThreads veinTrianglesThreads(triangleCount);
    CudaThreads bloodCellsThreads(particleCount);
    CudaThreads veinVerticesThreads(VeinTriangles::vertexCount);

    for (int s = 0; s < steps; ++s) {
        // main.cu:175-176
        calculate_grid(particleGrid, bloodCells.particles.positions[0], particleCount);
        calculate_grid(triangleGrid, triangles.centers, triangleCount);
        if (s == 0) {
            dump_grid("pgrid", particleGrid, particleCount);
            dump_grid("tgrid", triangleGrid, triangleCount);
        }
        // calculateNextFrame (simulation_controller.cu:254-294)
        triangles.gatherForcesFromNeighbors(0, verticesGpuStarts[0], verticesGpuEnds[0], veinTrianglesThreads.blocks,
                                            veinTrianglesThreads.threadsPerBlock);
        bloodCells.gatherForcesFromNeighbors(0, bloodCellGpuStarts[0], bloodCellGpuEnds[0], particleGpuStarts[0],
                                             particleGpuEnds[0], streams);
        mp_for_each<mp_iota_c<bloodCellTypeCount>>([&](auto i) {
            using Def = mp_at_c<BloodCellList, i>;
            constexpr int particlesStart = particleStarts[i];
            constexpr int modelStart = bloodCellModelStarts[i];
            CudaThreads threads(Def::count * Def::particlesInCell);
            bcs_launch(bcs_cfg(threads.blocks, threads.threadsPerBlock), [&]() {
                sim::calculateParticleCollisions<UniformGrid>(0, particleGpuStarts[0], particleGpuEnds[0], bloodCells,
                                                              particleGrid, boundingSpheresModel, Def::count,
                                                              Def::particlesInCell, modelStart, particlesStart);
            });
        });
        mp_for_each<mp_iota_c<bloodCellTypeCount>>([&](auto i) {
            using Def = mp_at_c<BloodCellList, i>;
            constexpr int particlesStart = particleStarts[i];
            constexpr int modelStart = bloodCellModelStarts[i];
            CudaThreads threads(Def::count * Def::particlesInCell);
            bcs_launch(bcs_cfg(threads.blocks, threads.threadsPerBlock), [&]() {
                sim::detectVeinCollisions<UniformGrid>(0, particleGpuStarts[0], particleGpuEnds[0], bloodCells,
                                                       triangles, triangleGrid, boundingSpheresModel, Def::count,
                                                       Def::particlesInCell, modelStart, particlesStart);
            });
        });
        if (s == 0) {
            dump_vec3("frame1_forces_next", F, particleCount);
            dump_vec3("frame1_velocities_next", Vv, particleCount);
        }
        // propagateAll (simulation_controller.cu:315-323)
        bloodCells.propagateForcesIntoPositions(bloodCellsThreads.blocks, bloodCellsThreads.threadsPerBlock);
        triangles.propagateForcesIntoPositions(veinVerticesThreads.blocks, veinVerticesThreads.threadsPerBlock);
        if (s == 0 || s == steps - 1) {
            std::string t = s == 0 ? "frame1_" : "frameN_";
            dump_vec3((t + "positions").c_str(), P, particleCount);
            dump_vec3((t + "velocities").c_str(), Vv, particleCount);
            dump_vec3((t + "forces").c_str(), F, particleCount);
            dump_vec3((t + "vein_positions").c_str(), triangles.positions[0], VeinTriangles::vertexCount);
            dump_vec3((t + "vein_velocities").c_str(), triangles.velocities[0], VeinTriangles::vertexCount);
        }
    }
    return 0;
}
