// bcs_oracle.cpp — FP64 host oracle of the reference's per-frame blood-cell
// physics.  TEST INFRASTRUCTURE ONLY: tests, the smoke check and the CPU
// baseline leg of the benchmark call it as a checker; the product library
// never links or calls it.
//
// It restates, in double precision and in the reference's order of
// operations, the update rules of GPU-Blood-Cell-Simulation/Simulation-Server
// (paths relative to that project's root):
//   layout       src/meta_factory/blood_cell_factory.hpp:172-328
//   bounds       src/meta_factory/vein_factory.hpp:21-86
//   vein springs src/meta_factory/vein_factory.hpp:130-174,
//                src/objects/vein_triangles.cu:125-154
//   grid         src/grids/uniform_grid.cu:24-80,129-155 (keys in FP32 exactly)
//   centroids    src/objects/blood_cells.cu:44-61
//   cell springs src/objects/blood_cells.cu:66-120, src/simulation/physics.cuh:24-120
//   collisions   src/simulation/particle_collisions.cuh:26-269, physics.cuh:133-145
//   vein hits    src/simulation/vein_collisions.cu:11-61,198-277,
//                src/simulation/vein_collisions.cuh:60-93
//   integrate    src/objects/blood_cells.cu:155-179, vein_triangles.cu:88-117
//   vein ends    src/simulation/vein_end.cu:12-108
//   radii        src/simulation/simulation_controller.cu:93-153
//   frame order  src/simulation/simulation_controller.cu:246-331, src/main.cu:175-208
//
// Pinned semantics where the reference is racy or undefined:
//   Q1 collision radius of a particle's own type; Q3 Jacobi read of the
//   previous forces; Q4 exact sum of the vein-force scatter; Q5 empty grid
//   cells are empty ranges and every occupied cell (the last one included)
//   has its true [start, end]; Q6 out-of-box keys are clamped per axis and
//   flagged; Q8 triangle centres from the initial mesh unless
//   refresh_triangle_centers; Q10 normalize(0) = 0; Q11 respawn offsets from
//   Philox4x32-10 keyed by (seed, cell, step), one draw per cell; Q12 the
//   block-sync vein-end rule (ending spheres + thresholds) for every type;
//   Q13 grid "none" is a brute-force scan with the same rules as "uniform";
//   Q15 (reference order only) a radius index before the table reads 0.
#include "../include/bcs.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef double real;

struct V3 {
    real x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(real s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, real s) { return {a.x / s, a.y / s, a.z / s}; }
inline real dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 u, V3 v) {
    return {u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x};
}
inline real length(V3 v) { return std::sqrt(dot(v, v)); }
// src/utilities/math.cuh:95-104: v / |v|, or 0 when that is NaN.
inline V3 normalize(V3 v, unsigned* err) {
    V3 n = v / std::sqrt(dot(v, v));
    if (std::isnan(n.x) || std::isnan(n.y) || std::isnan(n.z)) {
        if (err) *err |= BCS_ERRW_NAN_NORMALIZE;
        return {0, 0, 0};
    }
    return n;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11), counter (c0..c3), key (k0, k1).
void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
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
// Odd multiples of 2^-24: exactly representable in float and double, in (0,1).
inline real uniform_open(uint32_t r) { return (real)((r >> 9) * 2u + 1u) * (1.0 / 16777216.0); }

struct TypeLayout {
    int count, pic, particle_start, cell_start, model_start;
    std::vector<float> model;      // pic*3
    std::vector<float> graph;      // pic*pic dense rest lengths, 0 = none
    std::vector<float> radius;     // collision radius per model vertex
    std::vector<real> r0;          // distance to the model centroid
};

struct Grid {
    bool uniform = true;
    float cw = 1, ch = 1, cd = 1;
    int cx = 0, cy = 0, cz = 0;
    int64_t cells = 0;
    std::vector<int> keys, ids;            // sorted
};

// [first, last] sorted slots of a cell (empty: first > last).  A binary
// search on the sorted keys gives the ranges calculateStartAndEndOfCellKernel
// writes (uniform_grid.cu:51-80) without a dense per-cell array.
inline bool cell_slots(const Grid& g, long long c, int& first, int& last) {
    auto r = std::equal_range(g.keys.begin(), g.keys.end(), (int)c);
    first = (int)(r.first - g.keys.begin());
    last = (int)(r.second - g.keys.begin()) - 1;
    return first <= last;
}

void dense_ranges(const Grid& g, int* starts, int* ends) {
    if (starts) std::fill(starts, starts + g.cells, 0);
    if (ends) std::fill(ends, ends + g.cells, -1);
    const int n = (int)g.keys.size();
    for (int i = 0; i < n; ++i) {
        int k = g.keys[i];
        if (starts && (i == 0 || k != g.keys[i - 1])) starts[k] = i;
        if (ends && (i == n - 1 || k != g.keys[i + 1])) ends[k] = i;
    }
}

struct Sim {
    bcs_params p{};
    std::vector<TypeLayout> types;
    int N = 0, C = 0, V = 0, T = 0;
    std::vector<int> type_of_particle;     // particle -> type index
    // particle state
    std::vector<V3> x, v, f;
    // vein
    std::vector<V3> vx, vv, vf;
    std::vector<uint32_t> tri;             // 3*T
    std::vector<int> nb_ids[9];
    std::vector<float> nb_len[9];
    std::vector<float> ecent;               // ending centres
    std::vector<float> erad;
    std::vector<bcs_flow_segment> flow;
    float minX, maxX, minY, maxY, minZ, maxZ, width, height, depth;
    Grid pgrid, tgrid;
    std::vector<float> tcenters;            // 3*T float, from the initial mesh
    int64_t steps = 0;
    unsigned err = 0;
    int threads = 1;
    // Reference-order mode, used only to pin the oracle against the
    // reference's kernels executed serially on the CPU: neighbour forces
    // already rewritten earlier in the same pass are read (the serial
    // outcome of the Q3 race) and collision radii use the launch type's
    // model index (Q1, particle_collisions.cuh:76,124).
    bool reference_order = false;
    std::vector<float> model_radius;        // all types' radius tables, concatenated
};

// ---------------------------------------------------------------- grid ----
// src/grids/uniform_grid.cu:24-36, evaluated in FP32 like the reference:
// each axis index = int(min(extent, max(0, (p - min) / cell))).  The clamp by
// the extent (Q6) can yield an index past the last cell; the oracle clamps it
// to the last cell and flags positions outside the box.
inline int axis_index(float p, float lo, float extent, float cell, int count) {
    float t = (p - lo) / cell;
    float m = 0.0f > t ? 0.0f : t;
    float c = extent > m ? m : extent;
    int i = (int)c;
    if (i > count - 1) i = count - 1;
    if (i < 0) i = 0;
    return i;
}

int cell_key(const Sim& s, const Grid& g, float px, float py, float pz, unsigned* err) {
    if (px < s.minX || px > s.maxX || py < s.minY || py > s.maxY || pz < s.minZ || pz > s.maxZ)
        if (err) *err |= BCS_ERRW_OUT_OF_GRID;
    int ix = axis_index(px, s.minX, s.width, g.cw, g.cx);
    int iy = axis_index(py, s.minY, s.height, g.ch, g.cy);
    int iz = axis_index(pz, s.minZ, s.depth, g.cd, g.cz);
    return iz * (int)(s.width / g.cw) * (int)(s.height / g.ch) + iy * (int)(s.width / g.cw) + ix;
}

// calculateCellIdKernel + thrust::stable_sort_by_key +
// calculateStartAndEndOfCellKernel (uniform_grid.cu:38-80,129-155).
void build_grid(const Sim& s, Grid& g, const std::vector<float>& px, const std::vector<float>& py,
                const std::vector<float>& pz, unsigned* err) {
    const int n = (int)px.size();
    g.keys.resize(n);
    g.ids.resize(n);
    for (int i = 0; i < n; ++i) {
        g.keys[i] = cell_key(s, g, px[i], py[i], pz[i], err);
        g.ids[i] = i;
    }
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return g.keys[a] < g.keys[b]; });
    std::vector<int> sk(n);
    for (int i = 0; i < n; ++i) sk[i] = g.keys[order[i]];
    g.keys.swap(sk);
    g.ids.swap(order);
}

void particle_positions_f32(const Sim& s, std::vector<float>& px, std::vector<float>& py,
                            std::vector<float>& pz) {
    px.resize(s.N); py.resize(s.N); pz.resize(s.N);
    for (int i = 0; i < s.N; ++i) {
        px[i] = (float)s.x[i].x; py[i] = (float)s.x[i].y; pz[i] = (float)s.x[i].z;
    }
}

void triangle_centers_f32(const Sim& s, std::vector<float>& cx, std::vector<float>& cy,
                          std::vector<float>& cz, bool current) {
    // calculateCentersKernel (vein_triangles.cu:14-27), FP32 sum / 3.
    cx.resize(s.T); cy.resize(s.T); cz.resize(s.T);
    for (int t = 0; t < s.T; ++t) {
        if (!current) {
            cx[t] = s.tcenters[3 * t]; cy[t] = s.tcenters[3 * t + 1]; cz[t] = s.tcenters[3 * t + 2];
            continue;
        }
        float a[3][3];
        for (int k = 0; k < 3; ++k) {
            const V3& q = s.vx[s.tri[3 * t + k]];
            a[k][0] = (float)q.x; a[k][1] = (float)q.y; a[k][2] = (float)q.z;
        }
        cx[t] = (a[0][0] + a[1][0] + a[2][0]) / 3;
        cy[t] = (a[0][1] + a[1][1] + a[2][1]) / 3;
        cz[t] = (a[0][2] + a[1][2] + a[2][2]) / 3;
    }
}

// ------------------------------------------------------------- physics ----
// physics.cuh:24-27 and :53-77 (Heun branch): spring with damping that sees
// dt * (F_i - F_j) of the previous forces.
inline V3 cell_spring(const Sim& s, V3 dP, V3 dv, V3 f1, V3 f2, real L, unsigned* err) {
    const bcs_params& p = s.p;
    V3 nshift = normalize((real)-1 * dP, err);
    V3 dvv = dv + (real)p.dt * (f1 - f2);
    real mag = (length(dP) - L) * p.particle_k_sniff + dot(normalize(dP, err), dvv) * p.particle_d_fact;
    return mag * nshift;
}

// physics.cuh:102-120, with G replaced by the segment flow when one is given.
inline V3 environment(const Sim& s, V3 pos, V3 vel, real ratio) {
    const bcs_params& p = s.p;
    V3 g{p.gravity[0], p.gravity[1], p.gravity[2]};
    if (!s.flow.empty()) {
        real best = std::numeric_limits<real>::max();
        V3 force{0, 0, 0};
        for (const auto& seg : s.flow) {
            V3 o{seg.origin[0], seg.origin[1], seg.origin[2]};
            V3 d{seg.direction[0], seg.direction[1], seg.direction[2]};
            real t = dot(pos - o, d);
            real tc = std::min<real>(std::max<real>(t, 0), seg.length);
            V3 c = o + tc * d;
            real dist2 = dot(pos - c, pos - c);
            if (dist2 < best) {
                best = dist2;
                V3 radial = (pos - o) - t * d;
                real r2 = dot(radial, radial);
                real prof = 1 - r2 / ((real)seg.radius * seg.radius);
                if (prof < 0) prof = 0;
                force = (real)seg.peak_force * prof * d;
            }
        }
        g = force;
    }
    if (p.enable_big_cells_brake && ratio > p.max_cell_size_factor_before_brake)
        return g - (real)p.viscous_damping * ratio * p.big_particle_braking_intensity * vel;
    return g - (real)p.viscous_damping * vel;
}

// physics.cuh:133-145 with the 0.5 intensity of particle_collisions.cuh:36.
inline V3 resilient(const Sim& s, V3 rp, V3 rv, real d2, real radius, unsigned* err) {
    const bcs_params& p = s.p;
    V3 dir = normalize(rp, err);
    V3 tang = rv - dot(rv, dir) * dir;
    V3 spring = (-(real)p.collision_spring_coeff * (radius * 2 - std::sqrt(d2))) * dir;
    V3 damp = (real)p.collision_damping_coeff * rv;
    V3 shear = (real)p.collision_shear_coeff * tang;
    return (real)0.5 * (spring + damp + shear);
}

struct Ray {
    V3 o, d, n;
    real t = 1e10;
    int obj = 0;
};

// Moller-Trumbore, vein_collisions.cu:11-45.
bool ray_triangle(V3 v0, V3 v1, V3 v2, Ray& r, V3& refl, unsigned* err) {
    const real EPS = 0.000001;
    V3 e1 = v1 - v0, e2 = v2 - v0;
    V3 h = cross(r.d, e2);
    real a = dot(e1, h);
    if (a > -EPS && a < EPS) return false;
    real f = 1 / a;
    V3 s = r.o - v0;
    real u = f * dot(s, h);
    if (u < 0 || u > 1) return false;
    V3 q = cross(s, e1);
    real v = f * dot(r.d, q);
    if (v < 0 || u + v > 1) return false;
    real t = f * dot(e2, q);
    if (t > EPS) {
        r.t = t;
        r.n = normalize(cross(e2, e1), err);
        refl = r.d - (2 * dot(r.d, r.n)) * r.n;
        return true;
    }
    return false;
}

// vein_collisions.cu:47-61 (note e1 = v2 - v1).
V3 barycentric(V3 pt, V3 v0, V3 v1, V3 v2) {
    V3 e0 = v1 - v0, e1 = v2 - v1, e2 = pt - v0;
    real d00 = dot(e0, e0), d01 = dot(e0, e1), d11 = dot(e1, e1), d20 = dot(e2, e0), d21 = dot(e2, e1);
    real den = d00 * d11 - d01 * d01;
    V3 b;
    b.x = (d11 * d20 - d01 * d21) / den;
    b.y = (d00 * d21 - d01 * d20) / den;
    b.z = 1 - b.x - b.y;
    return b;
}

// Stencil clip of particle_collisions.cuh:125-268 / vein_collisions.cu:221-367.
inline void stencil_range(long long id, long long count, int& lo, int& hi) {
    lo = -1; hi = 1;
    if (id < 1) lo = 0;
    else if (id > count - 2) hi = 0;
}

// --------------------------------------------------------------- step -----
void vein_springs(Sim& s) {
    // vein_triangles.cu:125-154; forces accumulate onto the zeroed buffer.
    if (!s.p.vein_dynamic) return;
    const bcs_params& p = s.p;
#pragma omp parallel for schedule(static) num_threads(s.threads)
    for (int i = 0; i < s.V; ++i) {
        unsigned e = 0;
        V3 fsum{0, 0, 0};
        for (int k = 0; k < 9; ++k) {
            int j = s.nb_ids[k][i];
            if (j == -1) continue;
            real L = s.nb_len[k][i];
            V3 pi = s.vx[i], pj = s.vx[j];
            real mag = (length(pi - pj) - L) * p.vein_k_sniff +
                       dot(normalize(pi - pj, &e), s.vv[i] - s.vv[j]) * p.vein_d_fact;
            fsum = fsum + mag * normalize(pj - pi, &e);
        }
        s.vf[i] = s.vf[i] + fsum;
        if (e) {
#pragma omp atomic
            s.err |= e;
        }
    }
}

void cell_springs(Sim& s) {
    // calculateBloodCellsCenters + gatherForcesKernel (blood_cells.cu:44-120),
    // every read of f is the previous step's value (Q3).
    std::vector<V3> fnew(s.N);
    for (const auto& ty : s.types) {
#pragma omp parallel for schedule(static) num_threads(s.threads)
        for (int c = 0; c < ty.count; ++c) {
            unsigned e = 0;
            const int first = ty.particle_start + c * ty.pic;
            V3 center{0, 0, 0};
            for (int k = 0; k < ty.pic; ++k) center = center + s.x[first + k];
            center = center / (real)ty.pic;
            for (int i = 0; i < ty.pic; ++i) {
                const int pi = first + i;
                V3 acc{0, 0, 0};
                for (int j = 0; j < ty.pic; ++j) {
                    float L = ty.graph[(size_t)j * ty.pic + i];
                    if (L == 0.0f) continue;
                    const int pj = first + j;
                    const V3 fj = (s.reference_order && j < i) ? fnew[pj] : s.f[pj];
                    acc = acc + cell_spring(s, s.x[pi] - s.x[pj], s.v[pi] - s.v[pj], s.f[pi], fj, L, &e);
                }
                real ratio = length(s.x[pi] - center) / ty.r0[i];
                acc = acc + environment(s, s.x[pi], s.v[pi], ratio);
                fnew[pi] = (s.f[pi] + acc) / (real)2;
            }
            if (e) {
#pragma omp atomic
                s.err |= e;
            }
        }
    }
    s.f.swap(fnew);
}

real particle_radius(const Sim& s, int particle) {
    const TypeLayout& ty = s.types[s.type_of_particle[particle]];
    return ty.radius[(particle - ty.particle_start) % ty.pic];
}

void particle_collisions(Sim& s) {
    // calculateParticleCollisions<UniformGrid> (particle_collisions.cuh:104-269).
    const Grid& g = s.pgrid;
    std::vector<V3> add(s.N, V3{0, 0, 0});
#pragma omp parallel for schedule(dynamic, 256) num_threads(s.threads)
    for (int slot = 0; slot < s.N; ++slot) {
        unsigned e = 0;
        const int pid = g.uniform ? g.ids[slot] : slot;
        const V3 p1 = s.x[pid], v1 = s.v[pid];
        // Q1: in reference order the radius index comes from the type whose
        // sorted-slot range holds `slot`, applied to any particle id.
        const TypeLayout& launch = s.types[s.type_of_particle[slot]];
        auto radius_of = [&](int particle) -> real {
            if (!s.reference_order) return particle_radius(s, particle);
            // Q15: a particle of an earlier type gives a negative remainder,
            // an index before the radius table (read as 0 here, as in the
            // zero-padded table the reference's replay gets)
            int m = launch.model_start + (particle - launch.particle_start) % launch.pic;
            return m < 0 ? 0.0 : s.model_radius[m];
        };
        const real r1 = radius_of(pid);
        V3 acc{0, 0, 0};
        auto test = [&](int q) {
            if (q == pid) return;
            V3 rp = p1 - s.x[q];
            real d2 = dot(rp, rp);
            real md = r1 + radius_of(q);
            if (d2 <= md * md && d2 >= 0.0001)
                acc = acc + resilient(s, rp, v1 - s.v[q], d2, r1, &e);
        };
        if (!g.uniform) {
            for (int q = 0; q < s.N; ++q) test(q);
        } else {
            const int cellId = g.keys[slot];
            const float fx = (float)p1.x, fy = (float)p1.y, fz = (float)p1.z;
            const int xId = (int)((fx - s.minX) / g.cw);
            const int yId = (int)((fy - s.minY) / g.ch);
            const int zId = (int)((fz - s.minZ) / g.cd);
            int x0, x1, y0, y1, z0, z1;
            stencil_range(xId, g.cx, x0, x1);
            stencil_range(yId, g.cy, y0, y1);
            stencil_range(zId, g.cz, z0, z1);
            for (int dx = x0; dx <= x1; ++dx)
                for (int dy = y0; dy <= y1; ++dy)
                    for (int dz = z0; dz <= z1; ++dz) {
                        long long nc = (long long)cellId + (long long)dz * g.cx * g.cy + (long long)dy * g.cx + dx;
                        int f, l;
                        if (nc < 0 || nc >= g.cells || !cell_slots(g, nc, f, l)) continue;
                        for (int i = f; i <= l; ++i) test(g.ids[i]);
                    }
        }
        add[pid] = acc;
        if (e) {
#pragma omp atomic
            s.err |= e;
        }
    }
    for (int i = 0; i < s.N; ++i) s.f[i] = s.f[i] + add[i];
}

void vein_collisions(Sim& s) {
    // detectVeinCollisions<UniformGrid> (vein_collisions.cu:198-277).
    const bcs_params& p = s.p;
    const Grid& g = s.tgrid;
    std::vector<V3> vadd(s.V, V3{0, 0, 0});
    const int nthr = s.threads;
    std::vector<std::vector<std::pair<int, V3>>> scatter(nthr);
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthr)
    for (int pid = 0; pid < s.N; ++pid) {
        unsigned e = 0;
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        const V3 vel = s.v[pid], pos = s.x[pid];
        Ray r;
        r.o = pos;
        r.d = normalize(vel, &e);
        V3 refl{0, 0, 0};
        bool hit = false;
        auto tri_vertex = [&](int t, int k) { return s.vx[s.tri[3 * t + k]]; };
        auto test = [&](int t) {
            if (!ray_triangle(tri_vertex(t, 0), tri_vertex(t, 1), tri_vertex(t, 2), r, refl, &e)) return false;
            r.obj = t;
            return true;
        };
        if (!g.uniform) {
            for (int t = 0; t < s.T && !hit; ++t) hit = test(t);
        } else {
            const float fx = (float)pos.x, fy = (float)pos.y, fz = (float)pos.z;
            const unsigned cellId = (unsigned)cell_key(s, g, fx, fy, fz, nullptr);
            auto uidx = [](float t) -> unsigned { return t <= 0.0f ? 0u : (unsigned)t; };
            const unsigned xId = uidx((fx - s.minX) / g.cw);
            const unsigned yId = uidx((fy - s.minY) / g.ch);
            const unsigned zId = uidx((fz - s.minZ) / g.cd);
            auto urange = [](unsigned id, int count, int& lo, int& hi) {
                lo = -1; hi = 1;
                if (id < 1u) lo = 0;
                else if (id > (unsigned)(count - 2)) hi = 0;
            };
            int x0, x1, y0, y1, z0, z1;
            urange(xId, g.cx, x0, x1);
            urange(yId, g.cy, y0, y1);
            urange(zId, g.cz, z0, z1);
            for (int dx = x0; dx <= x1 && !hit; ++dx)
                for (int dy = y0; dy <= y1 && !hit; ++dy)
                    for (int dz = z0; dz <= z1 && !hit; ++dz) {
                        long long nc = (long long)cellId + (long long)dz * g.cx * g.cy + (long long)dy * g.cx + dx;
                        int f, l;
                        if (nc < 0 || nc >= g.cells || !cell_slots(g, nc, f, l)) continue;
                        for (int i = f; i <= l; ++i)
                            if (test(g.ids[i])) { hit = true; break; }
                    }
        }
        V3 rel = pos - (pos + r.t * r.d);
        real d2 = dot(rel, rel);
        if (hit && d2 <= (real)p.vein_impact_distance * p.vein_impact_distance) {
            if (d2 > (real)p.vein_impact_minimal_force_distance * p.vein_impact_minimal_force_distance) {
                if (p.enable_reaction_force) {
                    V3 F = s.f[pid];
                    V3 resp = ((real)-1 * dot(F, r.n)) * r.n / dot(r.n, r.n);
                    s.f[pid] = F + resp;
                } else {
                    // vein_collisions.cu:258-262
                    s.f[pid] = s.f[pid] + resilient(s, rel, vel, d2, particle_radius(s, pid), &e);
                }
            }
            real speed = length(vel);
            V3 dv = ((real)p.velocity_collision_damping * speed) * refl - vel;
            s.v[pid] = s.v[pid] + dv;
            if (p.vein_dynamic) {
                V3 ds = (real)p.vein_collision_force_intensity * vel;
                int i0 = s.tri[3 * r.obj], i1 = s.tri[3 * r.obj + 1], i2 = s.tri[3 * r.obj + 2];
                V3 b = barycentric(pos + r.t * r.d, s.vx[i0], s.vx[i1], s.vx[i2]);
                scatter[tid].push_back({i0, b.x * ds});
                scatter[tid].push_back({i1, b.y * ds});
                scatter[tid].push_back({i2, b.z * ds});
            }
        }
        if (e) {
#pragma omp atomic
            s.err |= e;
        }
    }
    for (auto& sc : scatter)
        for (auto& kv : sc) s.vf[kv.first] = s.vf[kv.first] + kv.second;
}

void integrate(Sim& s) {
    // propagateParticleForcesKernel (blood_cells.cu:155-179), Heun branch.
    const real dt = s.p.dt;
#pragma omp parallel for schedule(static) num_threads(s.threads)
    for (int i = 0; i < s.N; ++i) {
        V3 v0 = s.v[i];
        V3 v1 = v0 + dt * s.f[i];
        s.v[i] = v1;
        s.x[i] = s.x[i] + ((real)0.5 * dt) * (v1 + v0);
    }
    // propagateForcesIntoPositionsKernel + memsets (vein_triangles.cu:88-117).
    if (s.p.vein_dynamic) {
        for (int i = 0; i < s.V; ++i) {
            s.vv[i] = s.vv[i] + dt * s.vf[i];
            s.vx[i] = s.vx[i] + dt * s.vv[i];
            s.vf[i] = V3{0, 0, 0};
        }
    }
}

void vein_end(Sim& s) {
    // handleVeinEndsBlockSync (vein_end.cu:12-18,57-108).
    if (!s.p.use_blood_flow) return;
    const bcs_params& p = s.p;
    const real upper = (real)s.maxY - 3 * (real)p.grid_y_margin / 4;
    const real lower = (real)s.minY + (real)p.grid_y_margin / 2;
    const real right = (real)s.maxX - (real)p.grid_xz_margin / 2;
    const real left = (real)s.minX + (real)p.grid_xz_margin / 2;
    const real front = (real)s.maxZ - (real)p.grid_xz_margin / 2;
    const real back = (real)s.minZ + (real)p.grid_xz_margin / 2;
    for (const auto& ty : s.types) {
#pragma omp parallel for schedule(static) num_threads(s.threads)
        for (int c = 0; c < ty.count; ++c) {
            const int first = ty.particle_start + c * ty.pic;
            bool tp = false;
            for (int i = 0; i < ty.pic && !tp; ++i) {
                V3 q = s.x[first + i];
                for (size_t k = 0; k < s.erad.size(); ++k) {
                    V3 d{q.x - s.ecent[3 * k], q.y - s.ecent[3 * k + 1], q.z - s.ecent[3 * k + 2]};
                    if (dot(d, d) <= (real)s.erad[k] * s.erad[k]) tp = true;
                }
                if (q.y <= lower || q.y >= upper || q.x <= left || q.x >= right || q.z <= back || q.z >= front)
                    tp = true;
            }
            if (!tp) continue;
            uint32_t ctr[4] = {(uint32_t)(ty.cell_start + c), (uint32_t)s.steps, (uint32_t)(s.steps >> 32), 0u};
            philox4x32_10(ctr, (uint32_t)s.p.seed, (uint32_t)(s.p.seed >> 32));
            real ux = uniform_open(ctr[0]), uz = uniform_open(ctr[1]);
            for (int i = 0; i < ty.pic; ++i) {
                const float* m = &ty.model[3 * i];
                const float* m0 = &ty.model[0];
                s.x[first + i].x = (ux - 0.5) * 1.2 * p.cylinder_radius + ((real)m[0] - m0[0]);
                s.x[first + i].y = (real)p.min_spawn_y + ((real)m[1] - m0[1]);
                s.x[first + i].z = (uz - 0.5) * 1.2 * p.cylinder_radius + ((real)m[2] - m0[2]);
                s.v[first + i] = V3{p.init_velocity[0], p.init_velocity[1], p.init_velocity[2]};
            }
        }
    }
}

void calculate_grids(Sim& s) {
    if (s.pgrid.uniform) {
        std::vector<float> px, py, pz;
        particle_positions_f32(s, px, py, pz);
        build_grid(s, s.pgrid, px, py, pz, &s.err);
    }
    if (s.tgrid.uniform && s.p.refresh_triangle_centers) {
        std::vector<float> cx, cy, cz;
        triangle_centers_f32(s, cx, cy, cz, true);
        build_grid(s, s.tgrid, cx, cy, cz, nullptr);
    }
}

void full_step(Sim& s) {
    calculate_grids(s);           // main.cu:175-176
    vein_springs(s);              // simulation_controller.cu:254-256
    cell_springs(s);              // :259-261
    particle_collisions(s);       // :265-277
    vein_collisions(s);           // :281-293
    integrate(s);                 // :315-323
    vein_end(s);                  // :325-329
    ++s.steps;
}

// Multi-rate macro step of K sub-steps (no reference counterpart; the
// surrogate's plain form).  Sub-step 1 is full_step: grid, vein springs, cell
// springs, collisions, the vein ray, integration and the vein-end rule.  The
// external part of its force (collisions + the vein's force adjustment) is
// held for sub-steps 2..K, which re-evaluate only cell springs and
// environment (and the vein mesh's springs); particle impacts on the vein
// enter in sub-step 1 only.  The vein-end rule runs after every sub-step as
// in full_step; a respawned cell's held force is dropped.  With K = 1 this
// is full_step.
void macro_step(Sim& s, int K) {
    calculate_grids(s);
    vein_springs(s);
    cell_springs(s);
    const std::vector<V3> favg = s.f;
    particle_collisions(s);
    vein_collisions(s);
    std::vector<V3> fext(s.N);
    for (int i = 0; i < s.N; ++i) fext[i] = s.f[i] - favg[i];
    auto end_of_substep = [&]() {
        const std::vector<V3> before = s.x;
        vein_end(s);
        ++s.steps;
        for (const auto& ty : s.types)
            for (int c = 0; c < ty.count; ++c) {
                const int first = ty.particle_start + c * ty.pic;
                bool moved = false;
                for (int i = 0; i < ty.pic && !moved; ++i) {
                    const V3 a = before[first + i], b = s.x[first + i];
                    moved = a.x != b.x || a.y != b.y || a.z != b.z;
                }
                if (moved)
                    for (int i = 0; i < ty.pic; ++i) fext[first + i] = V3{0, 0, 0};
            }
    };
    integrate(s);
    end_of_substep();
    for (int k = 2; k <= K; ++k) {
        vein_springs(s);
        cell_springs(s);
        for (int i = 0; i < s.N; ++i) s.f[i] = s.f[i] + fext[i];
        integrate(s);
        end_of_substep();
    }
}

bool finite3(const float* a) { return std::isfinite(a[0]) && std::isfinite(a[1]) && std::isfinite(a[2]); }

}  // namespace

// ================================================================ C ABI ====
extern "C" {

typedef struct bcso_sim bcso_sim;

int bcso_create(const bcs_scene_desc* d, bcso_sim** out) {
    if (!d || !out || d->type_count <= 0 || !d->types) return BCS_ERR_INVALID_ARGUMENT;
    Sim* s = new Sim();
    s->p = d->params;
    // Layout (blood_cell_factory.hpp:172-282).
    int pstart = 0, cstart = 0, mstart = 0;
    for (int t = 0; t < d->type_count; ++t) {
        const bcs_cell_type& ct = d->types[t];
        if (ct.count < 0 || ct.particles_in_cell <= 0 || !ct.vertices) { delete s; return BCS_ERR_INVALID_ARGUMENT; }
        TypeLayout L;
        L.count = ct.count; L.pic = ct.particles_in_cell;
        L.particle_start = pstart; L.cell_start = cstart; L.model_start = mstart;
        L.model.assign(ct.vertices, ct.vertices + 3 * L.pic);
        // Dense graph, last definition wins, 0 = no spring (:292-328).
        L.graph.assign((size_t)L.pic * L.pic, 0.0f);
        for (int k = 0; k < ct.spring_count; ++k) {
            int a = ct.springs[2 * k], b = ct.springs[2 * k + 1];
            if (a < 0 || b < 0 || a >= L.pic || b >= L.pic) { delete s; return BCS_ERR_INVALID_ARGUMENT; }
            L.graph[(size_t)a * L.pic + b] = ct.spring_lengths[k];
            L.graph[(size_t)b * L.pic + a] = ct.spring_lengths[k];
        }
        // generateBoundingSpheres (simulation_controller.cu:119-145).
        L.radius.assign(L.pic, std::numeric_limits<float>::max());
        float cxs = 0, cys = 0, czs = 0;
        for (int j = 0; j < L.pic; ++j) {
            for (int k = 0; k < L.pic; ++k) {
                if (j == k) continue;
                double len = std::sqrt(std::pow((double)(L.model[3 * j] - L.model[3 * k]), 2) +
                                       std::pow((double)(L.model[3 * j + 1] - L.model[3 * k + 1]), 2) +
                                       std::pow((double)(L.model[3 * j + 2] - L.model[3 * k + 2]), 2)) /
                             (2 * (double)s->p.bounding_spheres_coeff);
                if (len < L.radius[j]) L.radius[j] = (float)len;
            }
            cxs += L.model[3 * j]; cys += L.model[3 * j + 1]; czs += L.model[3 * j + 2];
        }
        if (ct.collision_radius)
            for (int j = 0; j < L.pic; ++j) L.radius[j] = ct.collision_radius[j];
        L.r0.resize(L.pic);
        {
            // The reference sums in float and divides by the model size.
            float ccx = cxs / L.pic, ccy = cys / L.pic, ccz = czs / L.pic;
            for (int j = 0; j < L.pic; ++j) {
                V3 m{L.model[3 * j], L.model[3 * j + 1], L.model[3 * j + 2]};
                L.r0[j] = length(m - V3{ccx, ccy, ccz});
            }
        }
        pstart += L.count * L.pic;
        cstart += L.count;
        mstart += L.pic;
        s->types.push_back(std::move(L));
    }
    s->N = pstart; s->C = cstart;
    for (const auto& L : s->types) s->model_radius.insert(s->model_radius.end(), L.radius.begin(), L.radius.end());
    s->type_of_particle.resize(s->N);
    for (size_t t = 0; t < s->types.size(); ++t)
        for (int i = 0; i < s->types[t].count * s->types[t].pic; ++i)
            s->type_of_particle[s->types[t].particle_start + i] = (int)t;
    s->x.assign(s->N, V3{0, 0, 0}); s->v = s->x; s->f = s->x;
    // Vein.
    const bcs_vein& vn = d->vein;
    if (vn.vertex_count <= 0 || !vn.positions || vn.triangle_count < 0) { delete s; return BCS_ERR_INVALID_ARGUMENT; }
    s->V = vn.vertex_count; s->T = vn.triangle_count;
    s->vx.resize(s->V); s->vv.assign(s->V, V3{0, 0, 0}); s->vf.assign(s->V, V3{0, 0, 0});
    for (int i = 0; i < s->V; ++i) s->vx[i] = V3{vn.positions[3 * i], vn.positions[3 * i + 1], vn.positions[3 * i + 2]};
    s->tri.assign(vn.indices, vn.indices + 3 * (size_t)s->T);
    for (uint32_t id : s->tri) if (id >= (uint32_t)s->V) { delete s; return BCS_ERR_INVALID_ARGUMENT; }
    s->ecent.assign(vn.ending_centers, vn.ending_centers + 3 * vn.ending_count);
    s->erad.assign(vn.ending_radii, vn.ending_radii + vn.ending_count);
    if (d->flow_segment_count > 0) s->flow.assign(d->flow_segments, d->flow_segments + d->flow_segment_count);
    // Bounds (vein_factory.hpp:21-86), FP32 like the constexpr floats.
    float mn[3] = {vn.positions[0], vn.positions[1], vn.positions[2]}, mx[3] = {mn[0], mn[1], mn[2]};
    for (int i = 1; i < s->V; ++i)
        for (int k = 0; k < 3; ++k) {
            mn[k] = std::min(mn[k], vn.positions[3 * i + k]);
            mx[k] = std::max(mx[k], vn.positions[3 * i + k]);
        }
    s->minX = mn[0] - s->p.grid_xz_margin; s->maxX = mx[0] + s->p.grid_xz_margin;
    s->minY = mn[1] - s->p.grid_y_margin; s->maxY = mx[1] + s->p.grid_y_margin;
    s->minZ = mn[2] - s->p.grid_xz_margin; s->maxZ = mx[2] + s->p.grid_xz_margin;
    s->width = s->maxX - s->minX; s->height = s->maxY - s->minY; s->depth = s->maxZ - s->minZ;
    auto setup_grid = [&](Grid& g, int kind, float cw, float ch, float cd) {
        g.uniform = kind == BCS_GRID_UNIFORM;
        g.cw = cw; g.ch = ch; g.cd = cd;
        g.cx = (int)(s->width / cw); g.cy = (int)(s->height / ch); g.cz = (int)(s->depth / cd);
        g.cells = (int64_t)g.cx * g.cy * g.cz;
    };
    setup_grid(s->pgrid, s->p.particle_grid, s->p.cell_width, s->p.cell_height, s->p.cell_depth);
    setup_grid(s->tgrid, s->p.triangle_grid, s->p.cell_width_triangles, s->p.cell_height_triangles,
               s->p.cell_depth_triangles);
    if ((s->pgrid.uniform && (s->pgrid.cells <= 0 || s->pgrid.cells > INT32_MAX)) ||
        (s->tgrid.uniform && (s->tgrid.cells <= 0 || s->tgrid.cells > INT32_MAX))) {
        delete s; return BCS_ERR_INVALID_ARGUMENT;
    }
    // Vein neighbours (vein_factory.hpp:130-174): both other vertices of
    // every triangle, sorted ascending, first 9 kept, FP32 rest lengths.
    {
        std::vector<std::vector<uint32_t>> nb(s->V);
        for (int t = 0; t < s->T; ++t) {
            uint32_t i0 = s->tri[3 * t], i1 = s->tri[3 * t + 1], i2 = s->tri[3 * t + 2];
            nb[i0].push_back(i1); nb[i0].push_back(i2);
            nb[i1].push_back(i0); nb[i1].push_back(i2);
            nb[i2].push_back(i0); nb[i2].push_back(i1);
        }
        for (int k = 0; k < 9; ++k) { s->nb_ids[k].assign(s->V, -1); s->nb_len[k].assign(s->V, -1.0f); }
        for (int i = 0; i < s->V; ++i) {
            std::sort(nb[i].begin(), nb[i].end());
            for (size_t k = 0; k < std::min<size_t>(nb[i].size(), 9); ++k) {
                uint32_t j = nb[i][k];
                float dx = vn.positions[3 * i] - vn.positions[3 * j];
                float dy = vn.positions[3 * i + 1] - vn.positions[3 * j + 1];
                float dz = vn.positions[3 * i + 2] - vn.positions[3 * j + 2];
                float l = sqrtf(dx * dx + dy * dy + dz * dz);
                s->nb_ids[k][i] = (int)j;
                s->nb_len[k][i] = l < 0 ? -l : l;
            }
        }
    }
    // Triangle centres from the initial mesh and the triangle grid.
    s->tcenters.resize(3 * (size_t)s->T);
    {
        std::vector<float> cx, cy, cz;
        triangle_centers_f32(*s, cx, cy, cz, true);
        for (int t = 0; t < s->T; ++t) { s->tcenters[3 * t] = cx[t]; s->tcenters[3 * t + 1] = cy[t]; s->tcenters[3 * t + 2] = cz[t]; }
        if (s->tgrid.uniform) build_grid(*s, s->tgrid, cx, cy, cz, nullptr);
    }
#ifdef _OPENMP
    s->threads = omp_get_max_threads();
#endif
    *out = reinterpret_cast<bcso_sim*>(s);
    return BCS_OK;
}

void bcso_destroy(bcso_sim* h) { delete reinterpret_cast<Sim*>(h); }

void bcso_set_threads(bcso_sim* h, int n) { reinterpret_cast<Sim*>(h)->threads = n < 1 ? 1 : n; }

void bcso_set_reference_order(bcso_sim* h, int on) { reinterpret_cast<Sim*>(h)->reference_order = on != 0; }

int bcso_counts(bcso_sim* h, int* out6) {
    Sim* s = reinterpret_cast<Sim*>(h);
    out6[0] = s->N; out6[1] = s->C; out6[2] = s->V; out6[3] = s->T;
    out6[4] = (int)s->pgrid.cells; out6[5] = (int)s->tgrid.cells;
    return 0;
}

void bcso_bounds(bcso_sim* h, float* b6, int* dims6) {
    Sim* s = reinterpret_cast<Sim*>(h);
    b6[0] = s->minX; b6[1] = s->maxX; b6[2] = s->minY; b6[3] = s->maxY; b6[4] = s->minZ; b6[5] = s->maxZ;
    dims6[0] = s->pgrid.cx; dims6[1] = s->pgrid.cy; dims6[2] = s->pgrid.cz;
    dims6[3] = s->tgrid.cx; dims6[4] = s->tgrid.cy; dims6[5] = s->tgrid.cz;
}

// Particle state as double [N][3] arrays (set from float inputs).
int bcso_set_particles(bcso_sim* h, const float* pos3, const float* vel3, const float* f3) {
    Sim* s = reinterpret_cast<Sim*>(h);
    for (int i = 0; i < s->N; ++i) {
        s->x[i] = V3{pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]};
        s->v[i] = V3{vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2]};
        s->f[i] = f3 ? V3{f3[3 * i], f3[3 * i + 1], f3[3 * i + 2]} : V3{0, 0, 0};
        if (!finite3(pos3 + 3 * i) || !finite3(vel3 + 3 * i)) return BCS_ERR_INVALID_ARGUMENT;
    }
    return BCS_OK;
}

void bcso_get_particles(bcso_sim* h, double* pos3, double* vel3, double* f3) {
    Sim* s = reinterpret_cast<Sim*>(h);
    for (int i = 0; i < s->N; ++i) {
        if (pos3) { pos3[3 * i] = s->x[i].x; pos3[3 * i + 1] = s->x[i].y; pos3[3 * i + 2] = s->x[i].z; }
        if (vel3) { vel3[3 * i] = s->v[i].x; vel3[3 * i + 1] = s->v[i].y; vel3[3 * i + 2] = s->v[i].z; }
        if (f3) { f3[3 * i] = s->f[i].x; f3[3 * i + 1] = s->f[i].y; f3[3 * i + 2] = s->f[i].z; }
    }
}

int bcso_set_vein(bcso_sim* h, const float* pos3, const float* vel3) {
    Sim* s = reinterpret_cast<Sim*>(h);
    for (int i = 0; i < s->V; ++i) {
        if (pos3) s->vx[i] = V3{pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]};
        if (vel3) s->vv[i] = V3{vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2]};
    }
    return BCS_OK;
}

void bcso_get_vein(bcso_sim* h, double* pos3, double* vel3, double* f3) {
    Sim* s = reinterpret_cast<Sim*>(h);
    for (int i = 0; i < s->V; ++i) {
        if (pos3) { pos3[3 * i] = s->vx[i].x; pos3[3 * i + 1] = s->vx[i].y; pos3[3 * i + 2] = s->vx[i].z; }
        if (vel3) { vel3[3 * i] = s->vv[i].x; vel3[3 * i + 1] = s->vv[i].y; vel3[3 * i + 2] = s->vv[i].z; }
        if (f3) { f3[3 * i] = s->vf[i].x; f3[3 * i + 1] = s->vf[i].y; f3[3 * i + 2] = s->vf[i].z; }
    }
}

// Whole frames: grids, next frame, propagate (main.cu:175-208).
void bcso_step(bcso_sim* h, int n) {
    Sim* s = reinterpret_cast<Sim*>(h);
    for (int i = 0; i < n; ++i) full_step(*s);
}

// The three phases separately, for phase-level comparisons.
void bcso_macro_step(bcso_sim* h, int substeps, int n) {
    Sim& s = *reinterpret_cast<Sim*>(h);
    for (int i = 0; i < n; ++i) macro_step(s, substeps < 1 ? 1 : substeps);
}

void bcso_calculate_grids(bcso_sim* h) { calculate_grids(*reinterpret_cast<Sim*>(h)); }
void bcso_calculate_next_frame(bcso_sim* h) {
    Sim* s = reinterpret_cast<Sim*>(h);
    vein_springs(*s); cell_springs(*s); particle_collisions(*s); vein_collisions(*s);
}
void bcso_propagate_all(bcso_sim* h) {
    Sim* s = reinterpret_cast<Sim*>(h);
    integrate(*s); vein_end(*s); ++s->steps;
}

// Grid arrays after the last grid build (which: 0 particles, 1 triangles).
void bcso_get_grid(bcso_sim* h, int which, int* keys, int* ids, int* starts, int* ends) {
    Sim* s = reinterpret_cast<Sim*>(h);
    Grid& g = which ? s->tgrid : s->pgrid;
    if (keys) std::copy(g.keys.begin(), g.keys.end(), keys);
    if (ids) std::copy(g.ids.begin(), g.ids.end(), ids);
    dense_ranges(g, starts, ends);
}

// Grid of arbitrary FP32 points with the scene's bounds and particle-grid
// cells: keys (sorted), ids, dense starts/ends.
void bcso_grid_of_points(bcso_sim* h, int n, const float* pts3, int* keys, int* ids, int* starts, int* ends,
                         unsigned* err) {
    Sim* s = reinterpret_cast<Sim*>(h);
    std::vector<float> px(n), py(n), pz(n);
    for (int i = 0; i < n; ++i) { px[i] = pts3[3 * i]; py[i] = pts3[3 * i + 1]; pz[i] = pts3[3 * i + 2]; }
    Grid g = s->pgrid;
    unsigned e = 0;
    build_grid(*s, g, px, py, pz, &e);
    std::copy(g.keys.begin(), g.keys.end(), keys);
    std::copy(g.ids.begin(), g.ids.end(), ids);
    dense_ranges(g, starts, ends);
    if (err) *err = e;
}

// Layout tables for tests: per type (particle_start, cell_start, model_start)
// and the collision radius / r0 of every model vertex (concatenated).
void bcso_layout(bcso_sim* h, int* starts3, float* radius, double* r0) {
    Sim* s = reinterpret_cast<Sim*>(h);
    int k = 0;
    for (size_t t = 0; t < s->types.size(); ++t) {
        const TypeLayout& L = s->types[t];
        starts3[3 * t] = L.particle_start; starts3[3 * t + 1] = L.cell_start; starts3[3 * t + 2] = L.model_start;
        for (int j = 0; j < L.pic; ++j, ++k) { radius[k] = L.radius[j]; r0[k] = L.r0[j]; }
    }
}

void bcso_vein_neighbors(bcso_sim* h, int* ids9, float* len9) {
    Sim* s = reinterpret_cast<Sim*>(h);
    for (int k = 0; k < 9; ++k) {
        std::copy(s->nb_ids[k].begin(), s->nb_ids[k].end(), ids9 + (size_t)k * s->V);
        std::copy(s->nb_len[k].begin(), s->nb_len[k].end(), len9 + (size_t)k * s->V);
    }
}

unsigned bcso_error_word(bcso_sim* h, int clear) {
    Sim* s = reinterpret_cast<Sim*>(h);
    unsigned e = s->err;
    if (clear) s->err = 0;
    return e;
}

long long bcso_steps_done(bcso_sim* h) { return reinterpret_cast<Sim*>(h)->steps; }

// ---- function-level entry points for known-answer tests -----------------
void bcso_philox4x32_10(const uint32_t* ctr4, const uint32_t* key2, uint32_t* out4) {
    uint32_t c[4] = {ctr4[0], ctr4[1], ctr4[2], ctr4[3]};
    philox4x32_10(c, key2[0], key2[1]);
    for (int i = 0; i < 4; ++i) out4[i] = c[i];
}

// springMassForceWithDampingForParticle (physics.cuh:24-27) for tests:
// returns the scalar magnitude.
double bcso_spring_scalar(const double* dP, const double* dv, double L, double k, double d) {
    V3 p{dP[0], dP[1], dP[2]}, vv{dv[0], dv[1], dv[2]};
    return (length(p) - L) * k + dot(normalize(p, nullptr), vv) * d;
}

int bcso_ray_triangle(const double* v0, const double* v1, const double* v2, const double* o, const double* d,
                      double* t_n_refl7) {
    Ray r;
    r.o = V3{o[0], o[1], o[2]};
    r.d = V3{d[0], d[1], d[2]};
    V3 refl{0, 0, 0};
    bool hit = ray_triangle(V3{v0[0], v0[1], v0[2]}, V3{v1[0], v1[1], v1[2]}, V3{v2[0], v2[1], v2[2]}, r, refl, nullptr);
    t_n_refl7[0] = r.t;
    t_n_refl7[1] = r.n.x; t_n_refl7[2] = r.n.y; t_n_refl7[3] = r.n.z;
    t_n_refl7[4] = refl.x; t_n_refl7[5] = refl.y; t_n_refl7[6] = refl.z;
    return hit ? 1 : 0;
}

void bcso_barycentric(const double* pt, const double* v0, const double* v1, const double* v2, double* out3) {
    V3 b = barycentric(V3{pt[0], pt[1], pt[2]}, V3{v0[0], v0[1], v0[2]}, V3{v1[0], v1[1], v1[2]}, V3{v2[0], v2[1], v2[2]});
    out3[0] = b.x; out3[1] = b.y; out3[2] = b.z;
}

void bcso_resilient(const bcs_params* p, const double* rp, const double* rv, double d2, double radius, double* out3) {
    Sim s;
    s.p = *p;
    V3 r = resilient(s, V3{rp[0], rp[1], rp[2]}, V3{rv[0], rv[1], rv[2]}, d2, radius, nullptr);
    out3[0] = r.x; out3[1] = r.y; out3[2] = r.z;
}

void bcso_environment(const bcs_params* p, const double* vel, double ratio, double* out3) {
    Sim s;
    s.p = *p;
    V3 r = environment(s, V3{0, 0, 0}, V3{vel[0], vel[1], vel[2]}, ratio);
    out3[0] = r.x; out3[1] = r.y; out3[2] = r.z;
}

}  // extern "C"
