// bcs_kernels.cu — the per-step kernels for sm_103a.
//
// One frame of the reference (src/main.cu:175-208) becomes, per step:
//   radix sort of the grid keys (bcs_sort.cu) → k_next_epoch → k_cell_ranges →
//   k_vein_springs → k_step<kFull> → k_vein_end → k_vein_integrate →
//   k_tri_cache → k_tri_boxes (cell bounds + wall mask) → k_bump_step
// k_step is cell-major: a CTA owns whole blood cells of one type, stages
// their positions / velocities / previous forces in shared memory, and does
// for each particle the work of calculateBloodCellsCenters, gatherForcesKernel,
// calculateParticleCollisions, detectVeinCollisions and
// propagateParticleForcesKernel, then writes the next step's grid keys.  Each
// particle's x, v, F cross HBM once per step in each direction.  k_vein_end
// (handleVeinEndsBlockSync) is a warp-per-cell pass over the new positions.
#include "bcs_internal.cuh"
#include "bcs_mma.cuh"
#include "bcs_mpnn.cuh"
#include <algorithm>

namespace bcs {

// ------------------------------------------------------------ physics ----
// springMassForceWithDampingForParticle + calculateParticlesSpringForceComponent
// (src/simulation/physics.cuh:24-27,53-77, Heun branch).  |dP| and dP/|dP|
// share one square root; normalize(-dP) is -normalize(dP).
__device__ inline float3 cell_spring(const bcs_params& p, float3 dP, float3 dv, float3 f1, float3 f2, float L,
                                     unsigned& e) {
    const float len = sqrtf(dot3(dP, dP));
    float3 n = __frcp_rn(len) * dP;
    if (isnan(n.x) || isnan(n.y) || isnan(n.z)) {
        e |= BCS_ERRW_NAN_NORMALIZE;
        n = f3(0.f, 0.f, 0.f);
    }
    const float3 dvv = dv + p.dt * (f1 - f2);
    const float mag = (len - L) * p.particle_k_sniff + dot3(n, dvv) * p.particle_d_fact;
    return (-mag) * n;
}

// accumulateEnvironmentForcesForParticles (physics.cuh:102-120); the
// constant G is replaced by the nearest segment's Poiseuille profile when
// flow segments are given.
__device__ inline float3 environment(const StepArgs& a, const SceneDev& sc, float3 x, float3 v, float ratio) {
    const bcs_params& p = a.p;
    float3 g = f3(p.gravity[0], p.gravity[1], p.gravity[2]);
    if (sc.flow_count > 0) {
        float best = 3.0e38f;
        for (int k = 0; k < sc.flow_count; ++k) {
            const bcs_flow_segment& s = a.flows[sc.flow_start + k];
            float3 o = f3(s.origin[0], s.origin[1], s.origin[2]);
            float3 d = f3(s.direction[0], s.direction[1], s.direction[2]);
            float t = dot3(x - o, d);
            float tc = fminf(fmaxf(t, 0.f), s.length);
            float3 c = o + tc * d;
            float dist2 = dot3(x - c, x - c);
            if (dist2 < best) {
                best = dist2;
                float3 radial = (x - o) - t * d;
                float prof = 1.f - dot3(radial, radial) / (s.radius * s.radius);
                g = (s.peak_force * fmaxf(prof, 0.f)) * d;
            }
        }
    }
    if (p.enable_big_cells_brake && ratio > p.max_cell_size_factor_before_brake)
        return g - p.viscous_damping * ratio * p.big_particle_braking_intensity * v;
    return g - p.viscous_damping * v;
}

// addResilientForceOnCollision (physics.cuh:133-145) times `intensity`;
// the direction and the spring term share one reciprocal square root of d2
// (every call site has d2 == dot(rp, rp) >= 1e-4 or a vein hit's distance).
__device__ inline float3 resilient(const bcs_params& p, float3 rp, float3 rv, float d2, float radius, float intensity,
                                   unsigned& e) {
    const float rs = rsqrtf(d2);
    const float d = d2 * rs;
    float3 dir = rs * rp;
    if (isnan(dir.x) || isnan(dir.y) || isnan(dir.z)) {
        e |= BCS_ERRW_NAN_NORMALIZE;
        dir = f3(0.f, 0.f, 0.f);
    }
    float3 tang = rv - dot3(rv, dir) * dir;
    float3 spring = (-p.collision_spring_coeff * (radius * 2 - d)) * dir;
    float3 damp = p.collision_damping_coeff * rv;
    float3 shear = p.collision_shear_coeff * tang;
    return intensity * (spring + damp + shear);
}

// Moller-Trumbore of realCollisionDetection (src/simulation/vein_collisions.cu:11-45)
// on precomputed edges e1 = v1 - v0, e2 = v2 - v0 (same FP32 values).
__device__ inline bool ray_triangle(float3 o, float3 d, float3 v0, float3 e1, float3 e2, float& t, float3& n,
                                    float3& refl, unsigned& e) {
    const float EPS = 0.000001f;
    float3 h = cross3(d, e2);
    float aa = dot3(e1, h);
    if (aa > -EPS && aa < EPS) return false;
    float f = 1.0f / aa;
    float3 s = o - v0;
    float u = f * dot3(s, h);
    if (u < 0.f || u > 1.f) return false;
    float3 q = cross3(s, e1);
    float v = f * dot3(d, q);
    if (v < 0.f || u + v > 1.f) return false;
    float tt = f * dot3(e2, q);
    if (tt > EPS) {
        t = tt;
        n = normalize_or_zero(cross3(e2, e1), e);
        refl = d - (2.0f * dot3(d, n)) * n;
        return true;
    }
    return false;
}

// calculateBaricentric (vein_collisions.cu:47-61), e1 = v2 - v1 as there.
__device__ inline float3 barycentric(float3 pt, float3 v0, float3 v1, float3 v2) {
    float3 e0 = v1 - v0, e1 = v2 - v1, e2 = pt - v0;
    float d00 = dot3(e0, e0), d01 = dot3(e0, e1), d11 = dot3(e1, e1), d20 = dot3(e2, e0), d21 = dot3(e2, e1);
    float den = d00 * d11 - d01 * d01;
    float bx = (d11 * d20 - d01 * d21) / den;
    float by = (d00 * d21 - d01 * d20) / den;
    return f3(bx, by, 1.0f - bx - by);
}

__device__ inline void stencil_range(int id, int count, int& lo, int& hi) {
    lo = -1; hi = 1;
    if (id < 1) lo = 0;
    else if (id > count - 2) hi = 0;
}

__device__ inline void stencil_range_u(unsigned id, int count, int& lo, int& hi) {
    lo = -1; hi = 1;
    if (id < 1u) lo = 0;
    else if (id > (unsigned)(count - 2)) hi = 0;
}

// Saturating float -> unsigned, the value cvt.rzi.u32.f32 gives for the
// reference's static_cast<unsigned int> of the cell coordinate.
__device__ inline unsigned to_u32_sat(float t) { return t <= 0.f ? 0u : (t >= 4294967040.f ? 0xFFFFFFFFu : (unsigned)t); }

// Collision stencil of a particle in the uniform grid (particle_collisions.cuh:
// 104-124): the centre cell comes from the clamped key, the stencil's edges
// from the unclamped quotients (Q7).
struct Stencil {
    int cell;                  // scene-local key of the centre cell
    int ix, iy, iz;            // its cell coordinates
    int x0, x1, y0, y1, z0, z1;
    bool regular;              // the unclamped cell indices are the key's: every
                               // such particle of the cell has this stencil
};

__device__ inline Stencil particle_stencil(const GridGeom& geo, float3 x) {
    const float tx = axis_quotient(x.x, geo.lo[0], geo.cell[0]);
    const float ty = axis_quotient(x.y, geo.lo[1], geo.cell[1]);
    const float tz = axis_quotient(x.z, geo.lo[2], geo.cell[2]);
    Stencil st;
    const int ix = axis_clamp(tx, geo.ext[0], geo.cx), iy = axis_clamp(ty, geo.ext[1], geo.cy),
              iz = axis_clamp(tz, geo.ext[2], geo.cz);
    st.cell = iz * geo.cx * geo.cy + iy * geo.cx + ix;   // key_of_quotients
    st.ix = ix;
    st.iy = iy;
    st.iz = iz;
    st.regular = (int)tx == ix && (int)ty == iy && (int)tz == iz;
    stencil_range((int)tx, geo.cx, st.x0, st.x1);
    stencil_range((int)ty, geo.cy, st.y0, st.y1);
    stencil_range((int)tz, geo.cz, st.z0, st.z1);
    return st;
}

// Sorted-slot range [first, last] of stencil row (dz, dy): the row's (up to)
// three cells are consecutive keys, so their occupied slots are one
// contiguous range.  Empty: last < first.
__device__ inline int2 row_range(const GridDev& g, const GridGeom& geo, int ep, const Stencil& st, int dz, int dy) {
    const int4* __restrict__ table = g.table + geo.key_offset;
    const long long row = (long long)st.cell + dz * ((long long)geo.cx * geo.cy) + (long long)dy * geo.cx;
    int first = 0x7fffffff, last = -1;
    if (g.occ) {
        // Occupied cells of the window from the bitmap: only the first and
        // the last occupied entries are loaded.
        const long long ca = max(row + st.x0, 0LL), cb = min(row + st.x1, geo.cells - 1);
        if (ca > cb) return make_int2(first, last);
        const long long ga = geo.key_offset + ca, gb = geo.key_offset + cb;
        const int sh = (int)(ga & 31);
        unsigned long long m = __ldg(&g.occ[ga >> 5]) >> sh;
        if ((gb >> 5) != (ga >> 5)) m |= (unsigned long long)__ldg(&g.occ[gb >> 5]) << (32 - sh);
        m &= (1ull << (int)(cb - ca + 1)) - 1ull;
        if (!m) return make_int2(first, last);
        const int lo = __ffsll((long long)m) - 1, hi = 63 - __clzll((long long)m);
        const int4 r = __ldg(&table[ca + lo]);
        first = r.x;
        last = hi != lo ? __ldg(&table[ca + hi]).y : r.y;
    } else {
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
            const long long c = row + dx;
            if (dx >= st.x0 && dx <= st.x1 && c >= 0 && c < geo.cells) {
                const int4 r = __ldg(&table[c]);
                if (r.z == ep) {
                    first = min(first, r.x);
                    last = max(last, r.y);
                }
            }
        }
    }
    return make_int2(first, last);
}

// A particle whose stencil holds more sorted slots (itself included) than
// this is crowded: a whole warp takes its collision search
// (heavy_collisions).  The split depends only on the state, so every launch
// shape sums each particle's collisions in the same order.
constexpr int kCrowdedSlots = 128;

// One candidate of particle (x, v, R): detectCollision's test, then the
// resilient force with the neighbour's velocity (fetched only on a hit).
template <class VelocityOf>
__device__ inline void collide(const StepArgs& a, float3 x, float3 v, float R, float4 pq, VelocityOf velocity_of,
                               float3& acc, unsigned& e) {
    const float3 rp = x - xyz(pq);
    const float d2 = dot3(rp, rp);
    const float md = R + pq.w;
    if (d2 <= md * md && d2 >= 0.0001f) acc = acc + resilient(a.p, rp, v - xyz(velocity_of()), d2, R, 0.5f, e);
}

// calculateParticleCollisions<UniformGrid> (particle_collisions.cuh:26-38,
// 53-83,104-269) for one particle, rows in stencil order, into `acc`.
// Returns false, with `acc` incomplete, as soon as the rows seen so far hold
// more than kCrowdedSlots slots (a crowded particle).
__device__ inline bool particle_collisions(const StepArgs& a, const SceneDev& sc, int pid, float3 x, float3 v,
                                           float R, float3& acc, unsigned& e) {
    acc = f3(0.f, 0.f, 0.f);
    const GridDev& g = a.pg;
    const GridGeom& geo = sc.pg;
    auto test = [&](int q) { collide(a, x, v, R, __ldg(&a.pos_in[q]), [&a, q] { return __ldg(&a.vel_in[q]); }, acc, e); };
    if (!g.uniform) {
        for (int q = sc.particle_start; q < sc.particle_end; ++q)
            if (q != pid) test(q);
        return true;
    }
    const int ep = __ldg(g.epoch);
    const Stencil st = particle_stencil(geo, x);
    int slots = 0;
    for (int dz = st.z0; dz <= st.z1; ++dz)
        for (int dy = st.y0; dy <= st.y1; ++dy) {
            const int2 r = row_range(g, geo, ep, st, dz, dy);
            slots += max(0, r.y - r.x + 1);
            if (slots > kCrowdedSlots) return false;
            if (g.spos) {
                // Sorted positions (and velocities): contiguous loads; the
                // particle itself (d2 = 0) fails the d2 >= 1e-4 test, so no
                // id is needed.
                auto vel_of = [&a, &g](int j) {
                    return g.svel ? __ldg(&g.svel[j]) : __ldg(&a.vel_in[__ldg(&g.ids[j])]);
                };
                // two slots per step, their position reads issued together
                int j = r.x;
                for (; j < r.y; j += 2) {
                    const float4 p0 = __ldg(&g.spos[j]), p1 = __ldg(&g.spos[j + 1]);
                    collide(a, x, v, R, p0, [&vel_of, j] { return vel_of(j); }, acc, e);
                    collide(a, x, v, R, p1, [&vel_of, j] { return vel_of(j + 1); }, acc, e);
                }
                if (j == r.y) collide(a, x, v, R, __ldg(&g.spos[j]), [&vel_of, j] { return vel_of(j); }, acc, e);
            } else {
                for (int j = r.x; j <= r.y; ++j) {
                    const int q = __ldg(&g.ids[j]);
                    if (q != pid) test(q);
                }
            }
        }
    return true;
}

// The nine rows of a stencil for a whole warp: lanes 0..8 look up one row
// each; every lane receives each row's first slot (rf) and its start in the
// stencil's slot numbering (rs, rows in stencil order); returns the number
// of slots.  Slot number c lies in the last row with rs[r] <= c (an empty
// row starts where the next one does).
__device__ inline int stencil_rows(const GridDev& g, const GridGeom& geo, const Stencil& st, int lane, int (&rs)[9],
                                   int (&rf)[9]) {
    const int ep = __ldg(g.epoch);
    int first = 0, len = 0;
    if (lane < 9) {
        const int dz = lane / 3 - 1, dy = lane % 3 - 1;
        if (dz >= st.z0 && dz <= st.z1 && dy >= st.y0 && dy <= st.y1) {
            const int2 r = row_range(g, geo, ep, st, dz, dy);
            if (r.y >= r.x) {
                first = r.x;
                len = r.y - r.x + 1;
            }
        }
    }
    int incl = len;
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 8);
    const int start = incl - len;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        rs[r] = __shfl_sync(0xffffffffu, start, r);
        rf[r] = __shfl_sync(0xffffffffu, first, r);
    }
    return total;
}

__device__ inline int stencil_slot(int c, const int (&rs)[9], const int (&rf)[9]) {
    int j = rf[0];
#pragma unroll
    for (int r = 0; r < 9; ++r)
        if (c >= rs[r]) j = rf[r] + (c - rs[r]);
    return j;
}

// The same sum for one crowded particle, taken by a whole warp: the slots of
// the nine rows are numbered in stencil order and lane l takes slots l,
// l + 32, ...; a fixed butterfly combines the lanes' partial sums (every
// lane returns the total).
__device__ inline float3 heavy_collisions(const StepArgs& a, const SceneDev& sc, int pid, float3 x, float3 v,
                                         float R, int lane, unsigned& e) {
    const GridDev& g = a.pg;
    const Stencil st = particle_stencil(sc.pg, x);
    int rs[9], rf[9];
    const int total = stencil_rows(g, sc.pg, st, lane, rs, rf);
    float3 acc = f3(0.f, 0.f, 0.f);
    // Four slots per lane and pass (c, c + 32, c + 64, c + 96), their loads
    // issued together: ids, then positions (sorted copy, or by id) and
    // velocities whether or not the pair touches; the lane still adds its
    // slots in increasing order.
    constexpr int U = 4;
    for (int c0 = lane; c0 < total; c0 += 32 * U) {
        int q[U];
        float4 pq[U], vq[U];
        bool live[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int c = c0 + 32 * u;
            live[u] = c < total;
            const int j = stencil_slot(c, rs, rf);
            if (g.spos && g.svel) {
                // sorted copies: no id (the particle itself fails d2 >= 1e-4)
                q[u] = live[u] ? -1 : pid;
                pq[u] = live[u] ? __ldg(&g.spos[j]) : make_float4(x.x, x.y, x.z, 0.f);
                vq[u] = live[u] ? __ldg(&g.svel[j]) : make_float4(0.f, 0.f, 0.f, 0.f);
            } else {
                q[u] = live[u] ? __ldg(&g.ids[j]) : pid;
                if (g.spos) pq[u] = live[u] ? __ldg(&g.spos[j]) : make_float4(x.x, x.y, x.z, 0.f);
            }
        }
        if (!(g.spos && g.svel)) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (!g.spos) pq[u] = __ldg(&a.pos_in[q[u]]);
                vq[u] = __ldg(&a.vel_in[q[u]]);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (!live[u] || q[u] == pid) continue;
            const float3 rp = x - xyz(pq[u]);
            const float d2 = dot3(rp, rp);
            const float md = R + pq[u].w;
            if (d2 <= md * md && d2 >= 0.0001f) acc = acc + resilient(a.p, rp, v - xyz(vq[u]), d2, R, 0.5f, e);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
    }
    return acc;
}

// Parametric entry of the ray o + t d (t >= 0) into an axis-aligned box, or
// 3e38 when the ray misses it.  inv holds 1/d (components with |d| < 1e-30
// are treated as parallel to that slab).
__device__ inline float ray_box_entry(float3 o, float3 d, float3 inv, float4 lo, float4 hi) {
    float t0 = 0.f, t1 = 3.0e38f;
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z}, ii[3] = {inv.x, inv.y, inv.z};
    const float ll[3] = {lo.x, lo.y, lo.z}, hh[3] = {hi.x, hi.y, hi.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (fabsf(dd[k]) < 1e-30f) {
            if (oo[k] < ll[k] || oo[k] > hh[k]) return 3.0e38f;
        } else {
            const float ta = (ll[k] - oo[k]) * ii[k], tb = (hh[k] - oo[k]) * ii[k];
            t0 = fmaxf(t0, fminf(ta, tb));
            t1 = fminf(t1, fmaxf(ta, tb));
        }
    }
    return t0 <= t1 ? t0 : 3.0e38f;
}

// detectVeinCollisions<UniformGrid> (vein_collisions.cu:198-277,
// vein_collisions.cuh:60-93) for one particle: the first triangle hit in
// stencil order (x, then y, then z; sorted order inside a cell) decides, and
// only a hit within vein_impact_distance acts.  Two exact shortcuts leave that
// outcome unchanged:
//  * a particle whose wall-mask cell has no triangle within the impact
//    distance (+ margin) cannot be hit that close: no collision;
//  * a stencil cell whose triangle bounds the ray does not enter holds no hit,
//    and once every remaining cell is entered only beyond the impact distance,
//    the first hit, if any, is too far: no collision.
__device__ inline void vein_collision(const StepArgs& a, const SceneDev& sc, float3 x, float3& v, float3& F,
                                      float R, unsigned& e) {
    if (a.T == 0) return;   // no wall to hit (and no triangle grid was built)
    const bcs_params& p = a.p;
    const GridDev& g = a.tg;
    const GridGeom& geo = sc.tg;
    const float reach = p.vein_impact_distance * 1.001f + 1e-3f;
    if (g.uniform && a.wall_mask) {
        const MaskGeom& m = sc.wall;
        int ix = (int)((x.x - m.lo[0]) * m.inv_cell), iy = (int)((x.y - m.lo[1]) * m.inv_cell),
            iz = (int)((x.z - m.lo[2]) * m.inv_cell);
        if (ix >= 0 && iy >= 0 && iz >= 0 && ix < m.nx && iy < m.ny && iz < m.nz) {
            const unsigned char mark = (unsigned char)__ldg(a.wall_epoch);
            if (__ldg(&a.wall_mask[m.offset + ((long long)iz * m.ny + iy) * m.nx + ix]) != mark) return;
        }
    }
    const float3 vel = v;
    const float3 dir = normalize_or_zero(vel, e);
    float t = 1e10f;
    float3 n = f3(0.f, 0.f, 0.f), refl = f3(0.f, 0.f, 0.f);
    int obj = -1;
    auto test_slot = [&](int s) -> bool {
        float4 c0 = __ldg(&a.tcache[3 * s]);
        float4 c1 = __ldg(&a.tcache[3 * s + 1]);
        float4 c2 = __ldg(&a.tcache[3 * s + 2]);
        if (ray_triangle(x, dir, xyz(c0), xyz(c1), xyz(c2), t, n, refl, e)) {
            obj = __float_as_int(c0.w);
            return true;
        }
        return false;
    };
    if (!g.uniform) {
        for (int s = sc.tri_start; s < sc.tri_end; ++s)
            if (test_slot(s)) break;
    } else {
        const int ep = __ldg(g.epoch);
        const float tx = axis_quotient(x.x, geo.lo[0], geo.cell[0]);
        const float ty = axis_quotient(x.y, geo.lo[1], geo.cell[1]);
        const float tz = axis_quotient(x.z, geo.lo[2], geo.cell[2]);
        const unsigned cellId = (unsigned)key_of_quotients(geo, tx, ty, tz);
        const unsigned xId = to_u32_sat(tx), yId = to_u32_sat(ty), zId = to_u32_sat(tz);
        int x0, x1, y0, y1, z0, z1;
        stencil_range_u(xId, geo.cx, x0, x1);
        stencil_range_u(yId, geo.cy, y0, y1);
        stencil_range_u(zId, geo.cz, z0, z1);
        const long long cxy = (long long)geo.cx * geo.cy;
        // Stencil cell k = 9 (dx + 1) + 3 (dy + 1) + (dz + 1): stencil order
        // (x, then y, then z).  Pass 0: which cells are in the stencil and
        // hold triangles: the cell's precomputed neighbour word masked by
        // the particle's stencil edges, or the 27 table reads (independent,
        // in flight together).
        unsigned occ = 0u;
        if (a.tocc) {
            // neighbour-word bits of the dx, dy and dz values
            constexpr unsigned kDx[3] = {0x000001FFu, 0x0003FE00u, 0x07FC0000u};
            constexpr unsigned kDy[3] = {0x001C0E07u, 0x00E07038u, 0x070381C0u};
            constexpr unsigned kDz[3] = {0x01249249u, 0x02492492u, 0x04924924u};
            const unsigned mx = (x0 < 0 ? kDx[0] : 0u) | kDx[1] | (x1 > 0 ? kDx[2] : 0u);
            const unsigned my = (y0 < 0 ? kDy[0] : 0u) | kDy[1] | (y1 > 0 ? kDy[2] : 0u);
            const unsigned mz = (z0 < 0 ? kDz[0] : 0u) | kDz[1] | (z1 > 0 ? kDz[2] : 0u);
            occ = __ldg(&a.tocc[geo.key_offset + cellId]) & mx & my & mz;
        } else {
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx)
#pragma unroll
                for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                    for (int dz = -1; dz <= 1; ++dz) {
                        if (dx < x0 || dx > x1 || dy < y0 || dy > y1 || dz < z0 || dz > z1) continue;
                        const long long c = (long long)cellId + dz * cxy + (long long)dy * geo.cx + dx;
                        if (c < 0 || c >= geo.cells) continue;
                        if (__ldg(&g.table[geo.key_offset + c]).z == ep)
                            occ |= 1u << (9 * (dx + 1) + 3 * (dy + 1) + dz + 1);
                    }
        }
        // Pass 1: which of them the ray enters, and the last one it enters
        // within reach.
        const float3 inv = f3(__frcp_rn(dir.x), __frcp_rn(dir.y), __frcp_rn(dir.z));
        unsigned live = 0u;
        int last_near = -1;
        for (unsigned m = occ; m; m &= m - 1u) {
            const int k = __ffs(m) - 1;
            const int dz = k % 3 - 1, dy = (k / 3) % 3 - 1, dx = k / 9 - 1;
            const long long cg = geo.key_offset + (long long)cellId + dz * cxy + (long long)dy * geo.cx + dx;
            const float te = ray_box_entry(x, dir, inv, __ldg(&a.tbox[2 * cg]), __ldg(&a.tbox[2 * cg + 1]));
            if (te > 2.9e38f) continue;
            live |= 1u << k;
            if (te <= reach) last_near = k;
        }
        // Pass 2: triangles of the entered cells up to the last one in reach,
        // in stencil order.
        if (last_near >= 0) live &= (2u << last_near) - 1u;
        else live = 0u;
        while (live) {
            const int kk = __ffs(live) - 1;
            live &= live - 1u;
            const int dz = kk % 3 - 1, dy = (kk / 3) % 3 - 1, dx = kk / 9 - 1;
            const long long c = (long long)cellId + dz * cxy + (long long)dy * geo.cx + dx;
            int f, l;
            if (!cell_range(g, geo, ep, c, f, l)) continue;
            bool found = false;
            for (int s2 = f; s2 <= l; ++s2)
                if (test_slot(s2)) { found = true; break; }
            if (found) break;
        }
    }
    if (obj < 0) return;
    float3 rel = x - (x + t * dir);
    float d2 = dot3(rel, rel);
    if (d2 > p.vein_impact_distance * p.vein_impact_distance) return;
    if (d2 > p.vein_impact_minimal_force_distance * p.vein_impact_minimal_force_distance) {
        if (p.enable_reaction_force) {
            float3 resp = (-1.0f * dot3(F, n)) * n / dot3(n, n);
            F = F + resp;
        } else {
            F = F + resilient(p, rel, vel, d2, R, 0.5f, e);
        }
    }
    float speed = len3(vel);
    float3 dv = (p.velocity_collision_damping * speed) * refl - vel;
    v = v + dv;
    if (p.vein_dynamic) {
        float3 ds = p.vein_collision_force_intensity * vel;
        uint32_t i0 = a.tri[3 * obj], i1 = a.tri[3 * obj + 1], i2 = a.tri[3 * obj + 2];
        float3 b = barycentric(x + t * dir, xyz(a.vpos[i0]), xyz(a.vpos[i1]), xyz(a.vpos[i2]));
        float d[9];
        const float3 d0 = b.x * ds, d1 = b.y * ds, d2v = b.z * ds;
        d[0] = d0.x; d[1] = d0.y; d[2] = d0.z;
        d[3] = d1.x; d[4] = d1.y; d[5] = d1.z;
        d[6] = d2v.x; d[7] = d2v.y; d[8] = d2v.z;
        // The reference's scatter (vein_collisions.cu:272-274) as
        // warp-aggregated atomics: the lanes here that hit the same triangle
        // add their shares in lane order and the lowest of them issues the
        // nine atomics, once per distinct triangle per warp.
        const unsigned act = __activemask();
        const unsigned peers = __match_any_sync(act, obj);
        const int lane = threadIdx.x & 31;
        float sum[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) sum[k] = 0.f;
        for (unsigned m = act; m; m &= m - 1u) {
            const int l = __ffs(m) - 1;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const float v = __shfl_sync(act, d[k], l);
                if ((peers >> l) & 1u) sum[k] += v;
            }
        }
        if (lane == __ffs(peers) - 1) {
            atomicAdd(&a.vfrc[i0].x, sum[0]); atomicAdd(&a.vfrc[i0].y, sum[1]); atomicAdd(&a.vfrc[i0].z, sum[2]);
            atomicAdd(&a.vfrc[i1].x, sum[3]); atomicAdd(&a.vfrc[i1].y, sum[4]); atomicAdd(&a.vfrc[i1].z, sum[5]);
            atomicAdd(&a.vfrc[i2].x, sum[6]); atomicAdd(&a.vfrc[i2].y, sum[7]); atomicAdd(&a.vfrc[i2].z, sum[8]);
        }
    }
}

// Vein-end rule of handleVeinEndsBlockSync (src/simulation/vein_end.cu:12-18,73-87).
__device__ inline bool leaves_vein(const SceneDev& sc, float3 q) {
    bool tp = false;
    for (int k = 0; k < sc.ending_count; ++k) {
        float4 c = sc.endings[k];
        float3 d = f3(q.x - c.x, q.y - c.y, q.z - c.z);
        tp = tp || dot3(d, d) <= c.w * c.w;
    }
    return tp || q.y <= sc.lower || q.y >= sc.upper || q.x <= sc.left || q.x >= sc.right || q.z <= sc.back ||
           q.z >= sc.front;
}

// Respawn of a whole cell at the inflow (vein_end.cu:101-107): one Philox
// draw per (scene seed, cell within the scene, step) gives the cell's x and
// z offsets.
__device__ inline void respawn(const StepArgs& a, const SceneDev& sc, int cell_in_scene, long long step,
                               int model_vertex, float3& x, float3& v) {
    uint32_t c[4] = {(uint32_t)cell_in_scene, (uint32_t)step, (uint32_t)((unsigned long long)step >> 32), 0u};
    philox4x32_10(c, sc.seed_lo, sc.seed_hi);
    float ux = uniform_open(c[0]), uz = uniform_open(c[1]);
    float4 off = __ldg(&a.respawn[model_vertex]);
    x = f3((ux - 0.5f) * 1.2f * sc.cylinder_radius + off.x, sc.min_spawn_y + off.y,
           (uz - 0.5f) * 1.2f * sc.cylinder_radius + off.z);
    v = f3(a.p.init_velocity[0], a.p.init_velocity[1], a.p.init_velocity[2]);
}

// Asynchronous global -> shared copies (cp.async): a thread issues all of
// its copies, then waits once (cp_async_wait_all) for every copy it issued;
// a barrier after that publishes them to the CTA.  Staging through them
// keeps every copy of a CTA in flight at once, where a load-then-store loop
// waits for each of its loads in turn, and the threads can compute while
// the copies land.
__device__ inline void cp_async4(void* smem, const void* gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ inline void cp_async16(void* smem, const void* gmem) {   // both 16-byte aligned
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ inline void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// The scene of a CTA, staged in shared memory (copies left in flight).
__device__ inline void stage_scene(const SceneDev* src, SceneDev* dst) {
    const int* s = reinterpret_cast<const int*>(src);
    int* d = reinterpret_cast<int*>(dst);
    for (int i = threadIdx.x; i < (int)(sizeof(SceneDev) / sizeof(int)); i += blockDim.x) cp_async4(d + i, s + i);
}

// ------------------------------------------------------------- k_step ----
constexpr int kFull = 0;    // whole frame: forces, integration, vein end, next keys
constexpr int kForces = 1;  // calculateNextFrame only: forces and collision velocities

// Everything of one particle after the staging and its collision sum
// `coll`: springs, environment and the force average, the vein ray,
// integration (MODE kFull) and the outputs.
// cpos / cvel / cfrc hold the particle's blood cell (vertex li of it), in
// shared memory (k_step) or global memory (k_crowded); cent is its centroid.
template <int MODE>
__device__ inline void advance_particle(const StepArgs& a, const SceneDev& sc, const TypeDev& ty, int pid, int li,
                                        const float4* cpos, const float4* cvel, const float4* cfrc, float3 cent,
                                        float3 coll, unsigned& e) {
    const float4 px = cpos[li];
    const float3 x = xyz(px), v = xyz(cvel[li]), fprev = xyz(cfrc[li]);
    // Intra-cell springs, gatherForcesKernel (blood_cells.cu:66-120) over
    // the CSR form of the dense spring graph (same ascending order).
    float3 F = f3(0.f, 0.f, 0.f);
    const int e0 = __ldg(&a.adj_off[ty.adj_start + li]), e1 = __ldg(&a.adj_off[ty.adj_start + li + 1]);
    for (int k = e0; k < e1; ++k) {
        const int j = __ldg(&a.adj_nbr[k]);
        F = F + cell_spring(a.p, x - xyz(cpos[j]), v - xyz(cvel[j]), fprev, xyz(cfrc[j]), __ldg(&a.adj_len[k]), e);
    }
    const float ratio = len3(x - cent) / __ldg(&a.r0[ty.model_start + li]);
    F = F + environment(a, sc, x, v, ratio);
    F = (fprev + F) / 2.0f;
    const float3 favg = F;
    // Particle-particle collisions.
    F = F + coll;
    // Particle-vein collision.
    float3 vv = v;
    vein_collision(a, sc, x, vv, F, px.w, e);
    float3 nx = x, nv = vv;
    if (MODE == kFull) {
        // propagateParticleForcesKernel (blood_cells.cu:155-179), Heun.
        const float3 v1 = vv + a.p.dt * F;
        nx = x + (0.5f * a.p.dt) * (v1 + vv);
        nv = v1;
    }
    if (!(isfinite(nx.x) && isfinite(nx.y) && isfinite(nx.z) && isfinite(nv.x) && isfinite(nv.y) && isfinite(nv.z)))
        e |= BCS_ERRW_NONFINITE;
    a.pos_out[pid] = make_float4(nx.x, nx.y, nx.z, px.w);
    a.vel_out[pid] = make_float4(nv.x, nv.y, nv.z, 0.f);
    a.frc_out[pid] = make_float4(F.x, F.y, F.z, 0.f);
    if (MODE == kFull && a.keys_out) a.keys_out[pid] = a.pg.uniform ? grid_key(sc.pg, nx, e) : 0;
    if (MODE == kFull && a.fext) {
        // macro step: the external part of this force, held by sub-steps 2..K
        const float3 fx = F - favg;
        a.fext[pid] = make_float4(fx.x, fx.y, fx.z, 0.f);
    }
}

// One work item: stage the cells and their centroids, then every particle:
// its collision sum, then advance_particle.  A crowded particle (more than
// kCrowdedSlots sorted slots in its stencil) is set aside as soon as its
// search sees that many, and k_crowded finishes it.
template <int MODE, int THREADS>
__device__ inline void step_item(const StepArgs& a, int item, float4* s_pos, float4* s_vel, float4* s_frc,
                                 float3* s_cent, SceneDev& sc) {
    const WorkItem w = a.work[item];
    const TypeDev ty = a.types[w.type];
    const int pic = ty.pic;
    const int p0 = ty.particle_start + w.first_cell * pic;
    const int np = w.ncells * pic;
    stage_scene(a.scenes + ty.scene, &sc);
    for (int i = threadIdx.x; i < np; i += THREADS) {
        cp_async16(s_pos + i, a.pos_in + p0 + i);
        cp_async16(s_vel + i, a.vel_in + p0 + i);
        cp_async16(s_frc + i, a.frc_in + p0 + i);
    }
    cp_async_wait_all();
    __syncthreads();

    // Cell centroids (blood_cells.cu:44-61), one warp per cell, fixed-order
    // butterfly reduction (deterministic).
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < w.ncells; c += THREADS / 32) {
        float3 acc = f3(0.f, 0.f, 0.f);
        for (int k = lane; k < pic; k += 32) acc = acc + xyz(s_pos[c * pic + k]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
            acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
        }
        if (lane == 0) {
            const float3 m = acc / (float)pic;
            s_cent[c] = m;
            a.cent[ty.cell_global + w.first_cell + c] = make_float4(m.x, m.y, m.z, 0.f);
        }
    }
    __syncthreads();

    unsigned e = 0;
    for (int i = threadIdx.x; i < np; i += THREADS) {
        const float4 px = s_pos[i];
        float3 coll;
        if (a.coll) {
            coll = xyz(__ldg(&a.coll[p0 + i]));   // k_collide's sum
        } else if (!particle_collisions(a, sc, p0 + i, xyz(px), xyz(s_vel[i]), px.w, coll, e)) {
            // crowded: every particle of the cell that shares this stencil is
            // crowded too, and the first to claim the cell (the table entry's
            // spare word, zero after each build) lists it once for k_crowded
            const Stencil st = particle_stencil(sc.pg, xyz(px));
            if (st.regular) {
                int4* entry = const_cast<int4*>(a.pg.table) + sc.pg.key_offset + st.cell;
                if (atomicExch(&entry->w, 1) == 0) a.crowded_cells[atomicAdd(&a.crowded_counter[2], 1)] = p0 + i;
            } else {
                a.crowded[atomicAdd(&a.crowded_counter[0], 1)] = p0 + i;
            }
            continue;
        }
        const int c = i / pic;
        advance_particle<MODE>(a, sc, ty, p0 + i, i - c * pic, s_pos + c * pic, s_vel + c * pic, s_frc + c * pic,
                               s_cent[c], coll, e);
    }
    if (e) atomicOr(a.err, e);
}

// The step kernel for one launch shape.  PERSIST: a grid of (SMs x resident
// CTAs) pulls work items from a counter; the last CTA to finish resets the
// counter for the next launch, so the launch replays from a CUDA graph.
template <int MODE, int THREADS, int CHUNK, int MINB, bool PERSIST>
__global__ void __launch_bounds__(THREADS, MINB) k_step(const StepArgs a) {
    __shared__ float4 s_pos[CHUNK];
    __shared__ float4 s_vel[CHUNK];
    __shared__ float4 s_frc[CHUNK];
    __shared__ float3 s_cent[kMaxCellsPerChunk];
    __shared__ SceneDev sc;
    if (!PERSIST) {
        step_item<MODE, THREADS>(a, blockIdx.x, s_pos, s_vel, s_frc, s_cent, sc);
        return;
    }
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(&a.work_counter[0], 1);
        __syncthreads();
        const int item = s_item;
        if (item >= a.work_count) break;
        step_item<MODE, THREADS>(a, item, s_pos, s_vel, s_frc, s_cent, sc);
        __syncthreads();   // shared buffers and s_item are reused
    }
    if (threadIdx.x == 0 && atomicAdd(&a.work_counter[1], 1) == (int)gridDim.x - 1) {
        // every CTA has taken its last item: reset for the next launch
        a.work_counter[0] = 0;
        a.work_counter[1] = 0;
    }
}

__device__ inline int type_of_particle(const StepArgs& a, int p) {
    return find_range(a.type_count, p, [&](int i) { return a.types[i].particle_start; });
}

// The crowded particles k_step set aside.
//  * Crowded grid cells (a.crowded_cells, one particle of each): a warp
//    takes a cell, up to 32 of its particles at a time, and stages the slots
//    of their common stencil in shared memory, 64 at a time and in stencil
//    order.  With G particles in a pass each has L = 32 / G lanes (rounded
//    down to a power of two); lane `sub` of a particle sums slots sub,
//    sub + L, ... in order and a fixed butterfly adds the L partial sums.
//    Only particles of the cell with the cell's regular stencil are taken;
//    the others are the light path's or in a.crowded.
//  * Crowded particles off the regular stencils (a.crowded: outside the grid
//    box, rare): a warp takes a batch of up to 32, sums the collisions of
//    each with the whole warp (heavy_collisions), then every lane finishes
//    its own particle.
// Each particle is then finished by advance_particle from the step's input
// state in global memory.  The last CTA to finish empties both lists.
constexpr int kCrowdedThreads = 256;
constexpr int kCrowdedStage = 64;    // stencil slots staged per warp and pass

template <int MODE>
__global__ void __launch_bounds__(kCrowdedThreads, 3) k_crowded(const StepArgs a) {
    __shared__ float4 s_cpos[kCrowdedThreads / 32][kCrowdedStage];
    __shared__ float4 s_cvel[kCrowdedThreads / 32][kCrowdedStage];
    const int count = a.crowded_counter[0], ncells = a.crowded_counter[2];
    if (count == 0 && ncells == 0) return;   // every CTA sees the same counts: nothing to reset
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gwarp = (blockIdx.x * kCrowdedThreads + threadIdx.x) >> 5;
    const int nwarps = gridDim.x * (kCrowdedThreads / 32);
    const GridDev& g = a.pg;
    unsigned e = 0;
    for (int k = gwarp; k < ncells; k += nwarps) {
        const int leader = a.crowded_cells[k];
        const TypeDev& lt = a.types[type_of_particle(a, leader)];
        const SceneDev& sc = a.scenes[lt.scene];
        const Stencil st = particle_stencil(sc.pg, xyz(a.pos_in[leader]));
        int rs[9], rf[9];
        const int total = stencil_rows(g, sc.pg, st, lane, rs, rf);
        const int4 own = __ldg(&g.table[sc.pg.key_offset + st.cell]);
        int taken = 0;   // particles of the cell this warp finished
        for (int s0 = own.x; s0 <= own.y; s0 += 32) {
            // G particles of the cell in this pass, L lanes each (the
            // largest power of two with G * L <= 32): lane = particle * L +
            // sub, and sub takes the staged slots sub, sub + L, ...
            const int G = min(32, own.y - s0 + 1);
            const int L = G > 16 ? 1 : G > 8 ? 2 : G > 4 ? 4 : G > 2 ? 8 : G > 1 ? 16 : 32;
            const int gp = lane / L, sub = lane - gp * L;
            const int my_slot = s0 + gp;
            int pid = -1;
            float3 x = f3(0.f, 0.f, 0.f), v = x;
            float R = 0.f;
            if (gp < G) {
                pid = __ldg(&g.ids[my_slot]);
                const float4 px = a.pos_in[pid];
                const Stencil ps = particle_stencil(sc.pg, xyz(px));
                if (ps.regular) {
                    x = xyz(px);
                    R = px.w;
                    v = xyz(a.vel_in[pid]);
                } else {
                    pid = -1;
                }
            }
            float3 acc = f3(0.f, 0.f, 0.f);
            for (int c0 = 0; c0 < total; c0 += kCrowdedStage) {
                const int n = min(kCrowdedStage, total - c0);
                for (int t = lane; t < n; t += 32) {
                    const int j = stencil_slot(c0 + t, rs, rf);
                    float4 vq;
                    if (g.spos && g.svel) {
                        s_cpos[wib][t] = __ldg(&g.spos[j]);
                        vq = __ldg(&g.svel[j]);
                    } else {
                        const int q = __ldg(&g.ids[j]);
                        s_cpos[wib][t] = g.spos ? __ldg(&g.spos[j]) : __ldg(&a.pos_in[q]);
                        vq = __ldg(&a.vel_in[q]);
                    }
                    s_cvel[wib][t] = make_float4(vq.x, vq.y, vq.z, __int_as_float(j));   // w: the slot
                }
                __syncwarp();
                if (pid >= 0) {
                    auto pair = [&](float4 pq, float4 vq) {
                        if (__float_as_int(vq.w) == my_slot) return;
                        const float3 rp = x - xyz(pq);
                        const float d2 = dot3(rp, rp);
                        const float md = R + pq.w;
                        if (d2 <= md * md && d2 >= 0.0001f) acc = acc + resilient(a.p, rp, v - xyz(vq), d2, R, 0.5f, e);
                    };
                    // two slots per step, their shared-memory reads issued
                    // together; the sum keeps the slots' order
                    int t = sub;
                    for (; t + L < n; t += 2 * L) {
                        const float4 p0 = s_cpos[wib][t], v0 = s_cvel[wib][t];
                        const float4 p1 = s_cpos[wib][t + L], v1 = s_cvel[wib][t + L];
                        pair(p0, v0);
                        pair(p1, v1);
                    }
                    if (t < n) pair(s_cpos[wib][t], s_cvel[wib][t]);
                }
                __syncwarp();
            }
            // the particle's L partial sums, fixed butterfly within its lanes
            for (int o = L >> 1; o > 0; o >>= 1) {
                acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
                acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
                acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
            }
            taken += __popc(__ballot_sync(0xffffffffu, pid >= 0 && sub == 0));
            if (pid >= 0 && sub == 0) {
                const TypeDev& ty = a.types[type_of_particle(a, pid)];
                const int rel = pid - ty.particle_start, cell = rel / ty.pic, li = rel - cell * ty.pic;
                const int first = pid - li;
                advance_particle<MODE>(a, sc, ty, pid, li, a.pos_in + first, a.vel_in + first, a.frc_in + first,
                                       xyz(a.cent[ty.cell_global + cell]), acc, e);
            }
        }
        // release the claim: the table is clean for a step on the same grid
        if (lane == 0) {
            const_cast<int4*>(g.table)[sc.pg.key_offset + st.cell].w = 0;
            atomicAdd(&a.crowded_counter[3], taken);
        }
    }
    // batches of up to 32 particles, as small as the list allows: a warp's
    // collision sums run one after another
    const int per = min(32, (count + nwarps - 1) / nwarps);
    for (int b0 = gwarp * per; b0 < count; b0 += nwarps * per) {
        const int nb = min(per, count - b0);
        const int mine = lane < nb ? a.crowded[b0 + lane] : -1;
        float3 my_coll = f3(0.f, 0.f, 0.f);
        for (int k = 0; k < nb; ++k) {
            const int pid = __shfl_sync(0xffffffffu, mine, k);
            const TypeDev& ty = a.types[type_of_particle(a, pid)];
            const float4 px = a.pos_in[pid];
            const float3 c = heavy_collisions(a, a.scenes[ty.scene], pid, xyz(px), xyz(a.vel_in[pid]), px.w, lane, e);
            if (lane == k) my_coll = c;
        }
        if (lane < nb) {
            const TypeDev& ty = a.types[type_of_particle(a, mine)];
            const int rel = mine - ty.particle_start, cell = rel / ty.pic, li = rel - cell * ty.pic;
            const int first = mine - li;
            advance_particle<MODE>(a, a.scenes[ty.scene], ty, mine, li, a.pos_in + first, a.vel_in + first,
                                   a.frc_in + first, xyz(a.cent[ty.cell_global + cell]), my_coll, e);
        }
    }
    if (e) atomicOr(a.err, e);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&a.crowded_counter[1], 1) == (int)gridDim.x - 1) {
            __threadfence();
            // running total of crowded particles (64 bits at [4]); atomic
            // reads, since this CTA's cache may hold the counters' line
            const unsigned listed = (unsigned)atomicExch(&a.crowded_counter[0], 0);
            const unsigned taken = (unsigned)atomicExch(&a.crowded_counter[3], 0);
            atomicAdd(reinterpret_cast<unsigned long long*>(a.crowded_counter + 4),
                      (unsigned long long)listed + taken);
            atomicExch(&a.crowded_counter[2], 0);
            atomicExch(&a.crowded_counter[1], 0);
        }
    }
}

// ------------------------------------------------ grid-order collisions ----
// First sorted slot of every grid row (the cx cells sharing y and z), batch
// row space: the lower bound of the row's first key in the sorted keys of
// its scene (a scene's keys fill exactly its particle range of slots).  One
// entry past the last row holds n.
__global__ void k_row_starts(const int* __restrict__ keys, int n, const SceneDev* __restrict__ scenes,
                             int scene_count, long long rows, int* row_start) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r > rows) return;
    if (r == rows) {
        row_start[r] = n;
        return;
    }
    const int s = find_range(scene_count, r, [&](int k) { return scenes[k].pg.row_offset; });
    const GridGeom& g = scenes[s].pg;
    const long long target = g.key_offset + (r - g.row_offset) * (long long)g.cx;
    int lo = scenes[s].particle_start, hi = scenes[s].particle_end;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((long long)__ldg(&keys[mid]) < target) lo = mid + 1;
        else hi = mid;
    }
    row_start[r] = lo;
}

// calculateParticleCollisions<UniformGrid> (particle_collisions.cuh:26-38,
// 53-83,104-269) in grid order: one thread per sorted slot, so a warp holds
// particles of neighbouring cells that share most of their stencil (in a
// crowded cell, all of it: every candidate load is a broadcast and the
// loops are warp-uniform).  A stencil row (dz, dy) is the key window
// [centre + dz cx cy + dy cx + x0, ... + x1] clipped to the scene's cells;
// its slots are found from the row-start table and the sorted keys, and its
// candidates are read from the sorted copies of positions and velocities.
// Rows in stencil order and slots ascending within each: the same
// candidates in the same order as particle_collisions, hence the same sum.
// The particle's sum lands in a.coll at its id, for the step kernel.
constexpr int kCollideThreads = 256;

// Halvings that take a binary search over `len` slots to an empty range,
// the same for every active lane of the warp (the largest of theirs): the
// nine searches then run a warp-uniform loop, with no per-step test of
// whether any search is still open.
__device__ inline int search_steps(int len) { return __reduce_max_sync(__activemask(), 32 - __clz(len)); }

template <int SEARCH>
__device__ inline void collide_slot(const StepArgs& a, int j) {
    const GridDev& g = a.pg;
    const int s = find_range(a.scene_count, j, [&](int k) { return a.scenes[k].particle_start; });
    const SceneDev& sc = a.scenes[s];
    const GridGeom& geo = sc.pg;
    const float4 px = __ldg(&g.spos[j]);
    const float3 x = xyz(px), v = xyz(__ldg(&g.svel[j]));
    const float R = px.w;
    const Stencil st = particle_stencil(geo, x);
    const long long cxy = (long long)geo.cx * geo.cy;
    const int send = sc.particle_end;
    const int* __restrict__ keys = g.keys;
    float3 acc = f3(0.f, 0.f, 0.f);
    unsigned e = 0;
    // When the whole stencil lies inside the grid (every particle inside the
    // grid box, and nearly all outside it), each window lies inside its row,
    // takes its row from the cell coordinates and spans x1 - x0 + 1 keys;
    // otherwise the windows are clipped to the grid row by row.
    const bool inside = st.ix + st.x0 >= 0 && st.ix + st.x1 <= geo.cx - 1 && st.iy + st.y0 >= 0 &&
                        st.iy + st.y1 <= geo.cy - 1 && st.iz + st.z0 >= 0 && st.iz + st.z1 <= geo.cz - 1;
    if (SEARCH != 0 && inside) {
        // The nine rows' key windows, then one binary search per row for the
        // window's first slot, the nine searches advancing together (their
        // loads are independent), then each window's slots in stencil order.
        int lo[9], hi[9], end[9], wlo[9];
        const int kbase = (int)geo.key_offset, rbase = (int)geo.row_offset;
#pragma unroll
        for (int r = 0; r < 9; ++r) {
            const int dz = r / 3 - 1, dy = r % 3 - 1;
            lo[r] = hi[r] = end[r] = 0;
            wlo[r] = 0;
            if (dz < st.z0 || dz > st.z1 || dy < st.y0 || dy > st.y1) continue;
            const int rr = (st.iz + dz) * geo.cy + st.iy + dy;   // the window's row
            wlo[r] = kbase + rr * geo.cx + st.ix + st.x0;
            lo[r] = __ldg(&g.row_start[rbase + rr]);
            hi[r] = end[r] = __ldg(&g.row_start[rbase + rr + 1]);
        }
        int len = 0;
#pragma unroll
        for (int r = 0; r < 9; ++r) len = max(len, hi[r] - lo[r]);
        const int steps = search_steps(len);
        for (int it = 0; it < steps; ++it) {
#pragma unroll
            for (int r = 0; r < 9; ++r) {
                if (lo[r] < hi[r]) {
                    const int m = (lo[r] + hi[r]) >> 1;
                    if (__ldg(&keys[m]) < wlo[r]) lo[r] = m + 1;
                    else hi[r] = m;
                }
            }
        }
        const int wx = st.x1 - st.x0;
        // four candidates per step, their keys, positions and velocities
        // loaded together (a crowded window holds hundreds); the sum keeps
        // the slots' order
#pragma unroll 1
        for (int r = 0; r < 9; ++r) {
            int t = lo[r];
            for (bool more = t < end[r]; more;) {
                int k[4];
                float4 pq[4], vq[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const bool in = t + u < end[r];
                    k[u] = in ? __ldg(&keys[t + u]) : 0x7fffffff;
                    pq[u] = in ? __ldg(&g.spos[t + u]) : make_float4(0.f, 0.f, 0.f, 0.f);
                    vq[u] = in ? __ldg(&g.svel[t + u]) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (k[u] - wlo[r] > wx) {
                        more = false;
                        break;
                    }
                    collide(a, x, v, R, pq[u], [&vq, u] { return vq[u]; }, acc, e);
                }
                t += 4;
                more = more && t < end[r];
            }
        }
    } else {
        // each row's window from a linear scan of the row's first slots
        for (int dz = st.z0; dz <= st.z1; ++dz)
            for (int dy = st.y0; dy <= st.y1; ++dy) {
                const long long row = (long long)st.cell + dz * cxy + (long long)dy * geo.cx;
                const long long klo = max(row + st.x0, 0LL), khi = min(row + st.x1, geo.cells - 1);
                if (klo > khi) continue;
                const int glo = (int)(geo.key_offset + klo), ghi = (int)(geo.key_offset + khi);
                int t = __ldg(&g.row_start[geo.row_offset + klo / geo.cx]);
                while (t < send && __ldg(&keys[t]) < glo) ++t;
                for (; t < send && __ldg(&keys[t]) <= ghi; ++t)
                    collide(a, x, v, R, __ldg(&g.spos[t]), [&g, t] { return __ldg(&g.svel[t]); }, acc, e);
            }
    }
    a.coll[__ldg(&g.ids[j])] = make_float4(acc.x, acc.y, acc.z, 0.f);
    if (e) atomicOr(a.err, e);
}

template <int SEARCH>
__global__ void __launch_bounds__(kCollideThreads) k_collide(const StepArgs a) {
    const int j = blockIdx.x * kCollideThreads + threadIdx.x;
    if (j < a.n) collide_slot<SEARCH>(a, j);
}

// The same sum with the candidates staged in shared memory.  A CTA takes
// kTileSlots consecutive sorted slots of one plane of one scene (grid rows
// yf..yl of plane z).  Every stencil row of its particles lies in planes
// z - 1 .. z + 1, rows yf - 1 .. yl + 1, and those rows of a plane are one
// contiguous slot range: the CTA stages the three ranges' keys, positions
// and velocities and the rows' first slots, then every thread runs the
// nine binary searches and its windows' candidates on shared memory.  Same
// candidates, same order, same sum as collide_slot.  The tile's plane, rows
// and ranges come from its record (k_tile_setup), the staging is one round
// of asynchronous copies during which each thread computes its particle's
// stencil, and the nine searches run a warp-uniform number of halvings.  A
// tile that spans two planes or scenes, or whose ranges exceed kTileStage
// slots (crowded rows), takes the global-memory search instead; so does a
// particle whose stencil does not follow its sorted key.
constexpr int kTileSlots = 256;
constexpr int kTileStage = 1408;     // staged slots: 1408 x 36 B
constexpr int kTileRows = 40;        // grid rows staged per plane
constexpr size_t kTileSmem = (size_t)kTileStage * (2 * sizeof(float4) + sizeof(int)) + 3 * (kTileRows + 1) * sizeof(int);

// The tile record of every block of kTileSlots sorted slots, built with the
// row starts: the tile's plane and staged rows and the three planes' slot
// ranges, so that the collision kernel reads them in one round trip instead
// of looking up the tile's keys and then its rows.  One thread per tile:
//   [0] (staged?, scene, plane zf, first staged row ylo)
//   [1] (staged rows, staged slots, A0, A1)
//   [2] (A2, c0, c0 + c1, 0)
// where Ap is the first sorted slot of the staged rows of plane zf + p - 1
// and cp their number of slots (Ap = cp = 0 for a plane outside the grid),
// so that plane p starts at staged offset c0 + ... + c(p-1).
// A tile is staged when it lies in one scene and one plane, its rows with
// their neighbours number at most kTileRows and the three ranges hold at most
// kTileStage slots.
__global__ void k_tile_setup(const int* __restrict__ keys, int n, const SceneDev* __restrict__ scenes,
                             int scene_count, const int* __restrict__ row_start, int4* tiles) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= (n + kTileSlots - 1) / kTileSlots) return;
    const int s0 = b * kTileSlots, last = min(s0 + kTileSlots, n) - 1;
    const int sc_i = find_range(scene_count, s0, [&](int k) { return scenes[k].particle_start; });
    const SceneDev& sc = scenes[sc_i];
    const GridGeom& geo = sc.pg;
    const int cxy = geo.cx * geo.cy;
    const int kf = keys[s0] - (int)geo.key_offset, kl = keys[last] - (int)geo.key_offset;
    const int zf = kf / cxy, zl = kl / cxy;
    const int yf = (kf - zf * cxy) / geo.cx, yl = (kl - zl * cxy) / geo.cx;
    const int ylo = max(yf - 1, 0), yhi = min(yl + 1, geo.cy - 1);
    const bool ok = last < sc.particle_end && zf == zl && yhi - ylo + 1 <= kTileRows;
    int A[3] = {0, 0, 0}, c[3] = {0, 0, 0};
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const int z = zf + p - 1;
        if (ok && z >= 0 && z < geo.cz) {
            const int r0 = (int)geo.row_offset + z * geo.cy;
            A[p] = row_start[r0 + ylo];
            c[p] = row_start[r0 + yhi + 1] - A[p];
        }
    }
    const int total = c[0] + c[1] + c[2];
    tiles[3 * b] = make_int4(ok && total <= kTileStage ? 1 : 0, sc_i, zf, ylo);
    tiles[3 * b + 1] = make_int4(yhi - ylo + 1, total, A[0], A[1]);
    tiles[3 * b + 2] = make_int4(A[2], c[0], c[0] + c[1], 0);
}

__global__ void __launch_bounds__(kTileSlots, 4) k_collide_tile(const StepArgs a) {
    extern __shared__ __align__(16) unsigned char tile_smem[];
    float4* s_pos = reinterpret_cast<float4*>(tile_smem);
    float4* s_vel = s_pos + kTileStage;
    int* s_key = reinterpret_cast<int*>(s_vel + kTileStage);
    int* s_row = s_key + kTileStage;   // [3][kTileRows + 1]: sorted slot of each row's first particle
    const GridDev& g = a.pg;
    const int s0 = blockIdx.x * kTileSlots, j = s0 + threadIdx.x;
    const int last = min(s0 + kTileSlots, a.n) - 1;
    // the tile's record and the particle's own state and id, all in flight together
    const int4 t0 = __ldg(&g.tiles[3 * blockIdx.x]), t1 = __ldg(&g.tiles[3 * blockIdx.x + 1]),
               t2 = __ldg(&g.tiles[3 * blockIdx.x + 2]);
    const int jj = min(j, last);
    const float4 px = __ldg(&g.spos[jj]);
    const float4 pv = __ldg(&g.svel[jj]);
    const int pid = __ldg(&g.ids[jj]);
    if (!t0.x) {
        if (j <= last) collide_slot<1>(a, j);
        return;
    }
    const SceneDev& sc = a.scenes[t0.y];
    const GridGeom& geo = sc.pg;
    const int zc = t0.z, ylo = t0.w, nrows = t1.x, total = t1.y;
    const int A0 = t1.z, A1 = t1.w, A2 = t2.x, B1 = t2.y, B2 = t2.z;
    // the rows' first slots and the three ranges as asynchronous copies (a
    // plane outside the grid has no slots: its rows start at its range's
    // start, A = 0)
    for (int q = threadIdx.x; q < 3 * (nrows + 1); q += kTileSlots) {
        const int p = q / (nrows + 1), i = q - p * (nrows + 1);
        const int z = zc + p - 1;
        int* dst = &s_row[p * (kTileRows + 1) + i];
        if (z >= 0 && z < geo.cz) cp_async4(dst, &g.row_start[(int)geo.row_offset + z * geo.cy + ylo + i]);
        else *dst = p == 0 ? A0 : (p == 1 ? A1 : A2);
    }
    for (int q = threadIdx.x; q < total; q += kTileSlots) {
        const int slot = q < B1 ? A0 + q : (q < B2 ? A1 + (q - B1) : A2 + (q - B2));
        cp_async4(&s_key[q], &g.keys[slot]);
        cp_async16(&s_pos[q], &g.spos[slot]);
        cp_async16(&s_vel[q], &g.svel[slot]);
    }
    // the particle's stencil while the copies land
    const float3 x = xyz(px), v = xyz(pv);
    const float R = px.w;
    const Stencil st = particle_stencil(geo, x);
    const bool inside = st.ix + st.x0 >= 0 && st.ix + st.x1 <= geo.cx - 1 && st.iy + st.y0 >= 0 &&
                        st.iy + st.y1 <= geo.cy - 1 && st.iz + st.z0 >= 0 && st.iz + st.z1 <= geo.cz - 1;
    // the stencil's rows among the staged ones (a particle whose stencil
    // does not follow its sorted key, after bcs_set_particles, searches globally)
    const bool staged = inside && st.iz == zc && st.iy + st.y0 >= ylo && st.iy + st.y1 <= ylo + nrows - 1;
    cp_async_wait_all();
    __syncthreads();
    if (j > last) return;
    if (!staged) {
        collide_slot<1>(a, j);
        return;
    }
    int lo[9], hi[9], end[9], wlo[9];
    const int kbase = (int)geo.key_offset;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        const int dz = r / 3 - 1, dy = r % 3 - 1;
        lo[r] = hi[r] = end[r] = 0;
        wlo[r] = 0;
        if (dz < st.z0 || dz > st.z1 || dy < st.y0 || dy > st.y1) continue;
        const int i = st.iy + dy - ylo;   // the window's row among the staged ones
        // sorted slot -> staged offset
        const int shift = dz < 0 ? -A0 : (dz == 0 ? B1 - A1 : B2 - A2);
        wlo[r] = kbase + ((st.iz + dz) * geo.cy + st.iy + dy) * geo.cx + st.ix + st.x0;
        lo[r] = s_row[(dz + 1) * (kTileRows + 1) + i] + shift;
        hi[r] = end[r] = s_row[(dz + 1) * (kTileRows + 1) + i + 1] + shift;
    }
    int len = 0;
#pragma unroll
    for (int r = 0; r < 9; ++r) len = max(len, hi[r] - lo[r]);
    const int steps = search_steps(len);
    for (int it = 0; it < steps; ++it) {
#pragma unroll
        for (int r = 0; r < 9; ++r) {
            if (lo[r] < hi[r]) {
                const int m = (lo[r] + hi[r]) >> 1;
                if (s_key[m] < wlo[r]) lo[r] = m + 1;
                else hi[r] = m;
            }
        }
    }
    float3 acc = f3(0.f, 0.f, 0.f);
    unsigned e = 0;
    const int wx = st.x1 - st.x0;
#pragma unroll
    for (int r = 0; r < 9; ++r)
        for (int t = lo[r]; t < end[r] && s_key[t] - wlo[r] <= wx; ++t)
            collide(a, x, v, R, s_pos[t], [s_vel, t] { return s_vel[t]; }, acc, e);
    a.coll[pid] = make_float4(acc.x, acc.y, acc.z, 0.f);
    if (e) atomicOr(a.err, e);
}

// handleVeinEndsBlockSync (src/simulation/vein_end.cu:57-108) after the
// integration of a whole frame: one warp per blood cell ORs the vein-end
// rule over its particles and respawns the cell; the respawned particles'
// grid keys are rewritten for the next frame.
__global__ void __launch_bounds__(256) k_vein_end(const StepArgs a, int cells) {
    const int cell_g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (cell_g >= cells) return;
    const int t = find_range(a.type_count, cell_g, [&](int i) { return a.types[i].cell_global; });
    const TypeDev ty = a.types[t];
    const SceneDev& sc = a.scenes[ty.scene];
    const int cell = cell_g - ty.cell_global;
    const int p0 = ty.particle_start + cell * ty.pic;
    // every lane's positions in flight together (no early exit per lane)
    bool leave = false;
    for (int k = lane; k < ty.pic; k += 32) leave |= leaves_vein(sc, xyz(__ldg(&a.pos_out[p0 + k])));
    if (!__any_sync(0xffffffffu, leave)) return;
    const long long step = *a.steps;
    unsigned e = 0;
    for (int k = lane; k < ty.pic; k += 32) {
        float3 x, v;
        respawn(a, sc, ty.cell_start + cell, step, ty.model_start + k, x, v);
        const float w = a.pos_out[p0 + k].w;
        a.pos_out[p0 + k] = make_float4(x.x, x.y, x.z, w);
        a.vel_out[p0 + k] = make_float4(v.x, v.y, v.z, 0.f);
        if (a.keys_out) a.keys_out[p0 + k] = a.pg.uniform ? grid_key(sc.pg, x, e) : 0;
        if (a.fext) a.fext[p0 + k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (e) atomicOr(a.err, e);
}

// propagateAll for the split-phase API: integrate (blood_cells.cu:155-179)
// and the vein-end rule, in place on the buffers k_step<kForces> wrote.
__global__ void __launch_bounds__(kPropagateThreads) k_propagate(const StepArgs a) {
    __shared__ int s_tp[kMaxCellsPerChunk];
    const WorkItem w = a.work[blockIdx.x];
    const TypeDev ty = a.types[w.type];
    const int pic = ty.pic;
    const int p0 = ty.particle_start + w.first_cell * pic;
    const int np = w.ncells * pic;
    const SceneDev& sc = a.scenes[ty.scene];
    if (threadIdx.x < w.ncells) s_tp[threadIdx.x] = 0;
    __syncthreads();
    const long long step = *a.steps;
    unsigned e = 0;
    auto heun = [&](int i, float3& nx, float3& nv) {
        const float3 x = xyz(a.pos_out[p0 + i]), v0 = xyz(a.vel_out[p0 + i]), F = xyz(a.frc_out[p0 + i]);
        const float3 v1 = v0 + a.p.dt * F;
        nx = x + (0.5f * a.p.dt) * (v1 + v0);
        nv = v1;
    };
    for (int i = threadIdx.x; i < np; i += kPropagateThreads) {
        float3 nx, nv;
        heun(i, nx, nv);
        if (a.p.use_blood_flow && leaves_vein(sc, nx)) atomicOr(&s_tp[i / pic], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < np; i += kPropagateThreads) {
        float3 nx, nv;
        heun(i, nx, nv);
        const int c = i / pic;
        if (a.p.use_blood_flow && s_tp[c])
            respawn(a, sc, ty.cell_start + w.first_cell + c, step, ty.model_start + (i - c * pic), nx, nv);
        if (!(isfinite(nx.x) && isfinite(nx.y) && isfinite(nx.z))) e |= BCS_ERRW_NONFINITE;
        const float wv = a.pos_out[p0 + i].w;
        a.pos_out[p0 + i] = make_float4(nx.x, nx.y, nx.z, wv);
        a.vel_out[p0 + i] = make_float4(nv.x, nv.y, nv.z, 0.f);
    }
    if (e) atomicOr(a.err, e);
}

// calculateCellIdKernel (src/grids/uniform_grid.cu:38-49).
__global__ void k_keys(const float4* __restrict__ pos, int n, int uniform, const SceneDev* __restrict__ scenes,
                       int scene_count, int* keys, int* ids, unsigned* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned e = 0;
    const int s = find_range(scene_count, i, [&](int k) { return scenes[k].particle_start; });
    keys[i] = uniform ? grid_key(scenes[s].pg, xyz(pos[i]), e) : 0;
    ids[i] = i;
    if (e) atomicOr(err, e);
}

// calculateCentersKernel (src/objects/vein_triangles.cu:14-27) fused with
// the triangle grid's key kernel.
__global__ void k_tri_keys(const float4* __restrict__ vpos, const uint32_t* __restrict__ tri, int T,
                           const SceneDev* __restrict__ scenes, int scene_count, int* keys, int* ids) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const int sidx = find_range(scene_count, t, [&](int k) { return scenes[k].tri_start; });
    float3 a = xyz(vpos[tri[3 * t]]), b = xyz(vpos[tri[3 * t + 1]]), c = xyz(vpos[tri[3 * t + 2]]);
    float3 ctr = f3(__fdiv_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), 3.0f),
                    __fdiv_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), 3.0f),
                    __fdiv_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), 3.0f));
    unsigned e = 0;
    keys[t] = grid_key(scenes[sidx].tg, ctr, e);
    ids[t] = t;
}

__global__ void k_next_epoch(int* epoch) { *epoch += 1; }

// calculateStartAndEndOfCellKernel (uniform_grid.cu:51-80), written into
// the epoch-stamped table: the first slot of each occupied cell scans to its
// last slot and stores (first, last, epoch) at once.
// Sub-steps 2..K of a macro step, in place on the state sub-step 1 wrote:
// the cells of one work item stay in shared memory, and every sub-step
// re-evaluates centroids, cell springs and environment with the external
// force of sub-step 1 held, integrates (Heun) and applies the vein-end rule
// (a respawned cell drops its held force).  Ends with the grid keys of the
// final positions.  The cell state is double-buffered in shared memory:
// sub-step k reads one buffer and writes the other, so a thread writes its
// particles' new state as soon as it has it (no copy of every result held
// in registers until all threads have read their neighbours), and a
// sub-step takes one barrier fewer.  PER particles per thread (the launch
// shape's particles per CTA / 256); the buffers are dynamic shared memory.
constexpr int kSubstepThreads = 256;

template <int PER>
__global__ void __launch_bounds__(kSubstepThreads) k_substeps(const StepArgs a, int K) {
    extern __shared__ __align__(16) unsigned char sub_smem[];
    constexpr int CAP = PER * kSubstepThreads;
    float4* b_pos[2] = {reinterpret_cast<float4*>(sub_smem), reinterpret_cast<float4*>(sub_smem) + 3 * CAP};
    __shared__ float3 s_cent[kMaxCellsPerChunk];
    __shared__ int s_leave[kMaxCellsPerChunk];
    __shared__ SceneDev sc;
    const WorkItem w = a.work[blockIdx.x];
    const TypeDev ty = a.types[w.type];
    const int pic = ty.pic;
    const int p0 = ty.particle_start + w.first_cell * pic;
    const int np = w.ncells * pic;
    stage_scene(a.scenes + ty.scene, &sc);
    float3 fe[PER];
    bool skip[PER];
#pragma unroll
    for (int r = 0; r < PER; ++r) {
        const int i = threadIdx.x + r * kSubstepThreads;
        skip[r] = true;
        if (i < np) {
            cp_async16(b_pos[0] + i, a.pos_out + p0 + i);
            cp_async16(b_pos[0] + CAP + i, a.vel_out + p0 + i);
            cp_async16(b_pos[0] + 2 * CAP + i, a.frc_out + p0 + i);
            fe[r] = xyz(a.fext[p0 + i]);
            skip[r] = a.skip_cell && a.skip_cell[ty.cell_global + w.first_cell + i / pic];
        }
    }
    cp_async_wait_all();
    __syncthreads();
    const long long step0 = *a.steps;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned e = 0;
    int cur = 0;
    for (int k = 2; k <= K; ++k) {
        const float4* c_pos = b_pos[cur];
        const float4* c_vel = c_pos + CAP;
        const float4* c_frc = c_pos + 2 * CAP;
        float4* n_pos = b_pos[cur ^ 1];
        float4* n_vel = n_pos + CAP;
        float4* n_frc = n_pos + 2 * CAP;
        for (int c = warp; c < w.ncells; c += kSubstepThreads / 32) {
            float3 acc = f3(0.f, 0.f, 0.f);
            for (int q = lane; q < pic; q += 32) acc = acc + xyz(c_pos[c * pic + q]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
                acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
                acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
            }
            if (lane == 0) {
                s_cent[c] = acc / (float)pic;
                s_leave[c] = 0;
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < PER; ++r) {
            const int i = threadIdx.x + r * kSubstepThreads;
            if (i >= np) continue;
            if (skip[r]) {   // a cell the network advanced keeps its state
                n_pos[i] = c_pos[i];
                n_vel[i] = c_vel[i];
                n_frc[i] = c_frc[i];
                continue;
            }
            const int c = i / pic, li = i - c * pic, cb = c * pic;
            const float4 xw = c_pos[i];
            const float3 x = xyz(xw), v = xyz(c_vel[i]), fprev = xyz(c_frc[i]);
            float3 F = f3(0.f, 0.f, 0.f);
            const int e0 = __ldg(&a.adj_off[ty.adj_start + li]), e1 = __ldg(&a.adj_off[ty.adj_start + li + 1]);
            for (int q = e0; q < e1; ++q) {
                const int j = cb + __ldg(&a.adj_nbr[q]);
                F = F + cell_spring(a.p, x - xyz(c_pos[j]), v - xyz(c_vel[j]), fprev, xyz(c_frc[j]),
                                    __ldg(&a.adj_len[q]), e);
            }
            const float ratio = len3(x - s_cent[c]) / __ldg(&a.r0[ty.model_start + li]);
            F = F + environment(a, sc, x, v, ratio);
            F = (fprev + F) / 2.0f + fe[r];
            const float3 v1 = v + a.p.dt * F;
            const float3 nx = x + (0.5f * a.p.dt) * (v1 + v);
            n_pos[i] = make_float4(nx.x, nx.y, nx.z, xw.w);
            n_vel[i] = make_float4(v1.x, v1.y, v1.z, 0.f);
            n_frc[i] = make_float4(F.x, F.y, F.z, 0.f);
            if (a.p.use_blood_flow && leaves_vein(sc, nx)) atomicOr(&s_leave[c], 1);
        }
        __syncthreads();
        if (a.p.use_blood_flow) {
#pragma unroll
            for (int r = 0; r < PER; ++r) {
                const int i = threadIdx.x + r * kSubstepThreads;
                if (i >= np) continue;
                const int c = i / pic;
                if (!s_leave[c]) continue;
                float3 x, v;
                respawn(a, sc, ty.cell_start + w.first_cell + c, step0 + (k - 1), ty.model_start + (i - c * pic),
                        x, v);
                n_pos[i] = make_float4(x.x, x.y, x.z, n_pos[i].w);
                n_vel[i] = make_float4(v.x, v.y, v.z, 0.f);
                fe[r] = f3(0.f, 0.f, 0.f);
            }
            __syncthreads();
        }
        cur ^= 1;
    }
    const float4* c_pos = b_pos[cur];
#pragma unroll
    for (int r = 0; r < PER; ++r) {
        const int i = threadIdx.x + r * kSubstepThreads;
        if (i >= np || skip[r]) continue;
        const int pid = p0 + i;
        const float4 x = c_pos[i], v = c_pos[CAP + i];
        if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z)))
            e |= BCS_ERRW_NONFINITE;
        a.pos_out[pid] = x;
        a.vel_out[pid] = v;
        a.frc_out[pid] = c_pos[2 * CAP + i];
        if (a.keys_out) a.keys_out[pid] = a.pg.uniform ? grid_key(sc.pg, xyz(x), e) : 0;
    }
    if (e) atomicOr(a.err, e);
}

// ------------------------------------------------- learned sub-steps ----
// Raw node features of every surrogate cell from the state after sub-step 1
// (one warp per cell): position and velocity relative to the cell's centroid
// and mean velocity, the current force, the held external force, the
// environment force, and a wall-proximity flag (1 when the particle's
// wall-mask cell holds a triangle within the impact distance).  The state
// itself is kept in `start` for the targets and the prediction.
__global__ void k_sur_features(const StepArgs a, const SurDev d) {
    const int sc_i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (sc_i >= d.cells) return;
    const TypeDev ty = a.types[d.cell_type[sc_i]];
    const SceneDev& sc = a.scenes[ty.scene];
    const int pic = ty.pic, p0 = ty.particle_start + d.cell_index[sc_i] * pic;
    float3 cx = f3(0.f, 0.f, 0.f), cv = cx;
    for (int k = lane; k < pic; k += 32) {
        cx = cx + xyz(a.pos_out[p0 + k]);
        cv = cv + xyz(a.vel_out[p0 + k]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cx.x += __shfl_xor_sync(0xffffffffu, cx.x, o);
        cx.y += __shfl_xor_sync(0xffffffffu, cx.y, o);
        cx.z += __shfl_xor_sync(0xffffffffu, cx.z, o);
        cv.x += __shfl_xor_sync(0xffffffffu, cv.x, o);
        cv.y += __shfl_xor_sync(0xffffffffu, cv.y, o);
        cv.z += __shfl_xor_sync(0xffffffffu, cv.z, o);
    }
    cx = cx / (float)pic;
    cv = cv / (float)pic;
    for (int k = lane; k < pic; k += 32) {
        const int p = p0 + k;
        const float4 x4 = a.pos_out[p], v4 = a.vel_out[p], f4 = a.frc_out[p], e4 = a.fext[p];
        const float3 x = xyz(x4), v = xyz(v4);
        const float3 r = x - cx, u = v - cv;
        const float ratio = len3(r) / __ldg(&a.r0[ty.model_start + k]);
        const float3 env = environment(a, sc, x, v, ratio);
        float wall = 0.f;
        if (a.wall_mask) {
            const MaskGeom& m = sc.wall;
            const int ix = (int)((x.x - m.lo[0]) * m.inv_cell), iy = (int)((x.y - m.lo[1]) * m.inv_cell),
                      iz = (int)((x.z - m.lo[2]) * m.inv_cell);
            if (ix >= 0 && iy >= 0 && iz >= 0 && ix < m.nx && iy < m.ny && iz < m.nz)
                wall = a.wall_mask[m.offset + ((long long)iz * m.ny + iy) * m.nx + ix] ==
                               (unsigned char)*a.wall_epoch ? 1.f : 0.f;
        }
        float* o = d.raw + ((size_t)sc_i * d.pic + k) * 16;
        o[0] = r.x; o[1] = r.y; o[2] = r.z;
        o[3] = u.x; o[4] = u.y; o[5] = u.z;
        o[6] = f4.x; o[7] = f4.y; o[8] = f4.z;
        o[9] = e4.x; o[10] = e4.y; o[11] = e4.z;
        o[12] = env.x; o[13] = env.y; o[14] = env.z;
        o[15] = wall;
        float4* st = d.start + ((size_t)sc_i * d.pic + k) * 3;
        st[0] = x4;
        st[1] = v4;
        st[2] = f4;
    }
}

// Training targets after sub-steps 2..K: the departure of the final state
// from the constant-force extrapolation of the state after sub-step 1,
//   x_base = x1 + T v1 + T^2/2 F1,  v_base = v1 + T F1,
// and the change of the force.  A cell that was respawned (a jump of more
// than one length unit) is marked invalid.
__global__ void k_sur_targets(const StepArgs a, const SurDev d, float* raw_t, unsigned char* valid) {
    const int sc_i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (sc_i >= d.cells) return;
    const TypeDev ty = a.types[d.cell_type[sc_i]];
    const int pic = ty.pic, p0 = ty.particle_start + d.cell_index[sc_i] * pic;
    const float T = d.T;
    bool jump = false;
    for (int k = lane; k < pic; k += 32) {
        const float4* st = d.start + ((size_t)sc_i * d.pic + k) * 3;
        const float3 x1 = xyz(st[0]), v1 = xyz(st[1]), F1 = xyz(st[2]);
        const float3 xK = xyz(a.pos_out[p0 + k]), vK = xyz(a.vel_out[p0 + k]), FK = xyz(a.frc_out[p0 + k]);
        const float3 dx = xK - (x1 + T * v1 + (0.5f * T * T) * F1);
        const float3 dv = vK - (v1 + T * F1);
        const float3 dF = FK - F1;
        jump = jump || !(fabsf(dx.x) < 1.f && fabsf(dx.y) < 1.f && fabsf(dx.z) < 1.f) ||
               !(isfinite(dv.x) && isfinite(dv.y) && isfinite(dv.z) && isfinite(dF.x) && isfinite(dF.y) &&
                 isfinite(dF.z));
        float* o = raw_t + ((size_t)sc_i * d.pic + k) * 9;
        o[0] = dx.x; o[1] = dx.y; o[2] = dx.z;
        o[3] = dv.x; o[4] = dv.y; o[5] = dv.z;
        o[6] = dF.x; o[7] = dF.y; o[8] = dF.z;
    }
    jump = __any_sync(0xffffffffu, jump);
    if (lane == 0) valid[sc_i] = jump ? 0 : 1;
}

// Edge features of the spring i <- j from the raw relative positions and
// velocities of its ends and its rest length L: with d = r_j - r_i, n =
// d / |d| and the stretch s = |d| - L, (s n, ((u_j - u_i) . n) n, s, L),
// scaled; the mean over a node's springs carries the leading terms of its
// spring force and of that force's rate of change.
__device__ inline void spring_features(const float* ri, const float* rj, float L, const SurScales& sc, float* e) {
    const float3 d = f3(rj[0] - ri[0], rj[1] - ri[1], rj[2] - ri[2]);
    const float3 du = f3(rj[3] - ri[3], rj[4] - ri[4], rj[5] - ri[5]);
    const float len = len3(d);
    const float3 n = len > 0.f ? d / len : f3(0.f, 0.f, 0.f);
    const float st = len - L, vn = dot3(du, n);
    e[0] = st * n.x / sc.el; e[1] = st * n.y / sc.el; e[2] = st * n.z / sc.el;
    e[3] = vn * n.x / sc.eu; e[4] = vn * n.y / sc.eu; e[5] = vn * n.z / sc.eu;
    e[6] = st / sc.el;
    e[7] = L / sc.er;
}

// Normalised network inputs for `cells` cells: node features, edge features
// (spring_features) and, when raw_t is given, targets.  Cell b reads sample
// idx[b] of the raw arrays (b itself when idx is null), or, with `nvalid`,
// a sample drawn by Philox from list[0 .. nvalid) keyed by (seed, b).
__global__ void k_sur_inputs(const float* __restrict__ raw, const float* __restrict__ raw_t, const int* __restrict__ list,
                             int nvalid, unsigned long long seed, int first, int cells, int pic,
                             const int* __restrict__ adj_off, const int* __restrict__ adj_nbr,
                             const float* __restrict__ adj_len, const SurScales sc, float* f, float* E, float* T) {
    const int b = blockIdx.x, edges = adj_off[pic];
    if (b >= cells) return;
    int src = first + b;
    if (list) {
        uint32_t c[4] = {(uint32_t)b, (uint32_t)(seed >> 32), 0u, 0u};
        philox4x32_10(c, (uint32_t)seed, 0x5EEDu);
        src = list[c[0] % (uint32_t)nvalid];
    }
    const float* rw = raw + (size_t)src * pic * 16;
    for (int i = threadIdx.x; i < pic * 16; i += blockDim.x) {
        const int q = i & 15;
        f[(size_t)b * pic * 16 + i] = (rw[i] - sc.fm[q]) * sc.fs[q];
    }
    if (T && raw_t) {
        const float* rt = raw_t + (size_t)src * pic * 9;
        for (int i = threadIdx.x; i < pic * 9; i += blockDim.x) {
            const int q = i % 9;
            T[(size_t)b * pic * 9 + i] = (rt[i] - sc.tm[q]) / sc.ts[q];
        }
    }
    for (int i = threadIdx.x; i < pic; i += blockDim.x)
        for (int k = adj_off[i]; k < adj_off[i + 1]; ++k)
            spring_features(rw + i * 16, rw + adj_nbr[k] * 16, adj_len[k], sc, E + ((size_t)b * edges + k) * 8);
}

// The prediction of cells [first, first + cells): decode the network's
// outputs into x_K, v_K, F_K and check the residual of the trapezoid rule
// over the span T, |x_K - x1 - T/2 (v1 + v_K)|, against the tolerance.  A
// cell that passes takes the prediction (and then the vein-end rule and its
// grid keys), and is skipped by k_substeps; a cell that fails falls back to
// the plain sub-steps.
__global__ void k_sur_apply(const StepArgs a, const SurDev d, const float* __restrict__ Y, const SurScales sc,
                            int first, int cells) {
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (b >= cells) return;
    const int sc_i = first + b;
    const TypeDev ty = a.types[d.cell_type[sc_i]];
    const SceneDev& scn = a.scenes[ty.scene];
    const int pic = ty.pic, cell = d.cell_index[sc_i], p0 = ty.particle_start + cell * pic;
    const float T = d.T;
    float worst = 0.f;
    bool finite = true;
    float3 px[6], pv[6], pF[6];   // pic <= 192 particles per cell here (6 per lane)
    int nk = 0;
    for (int k = lane; k < pic && nk < 6; k += 32, ++nk) {
        const float* y = Y + ((size_t)b * d.pic + k) * 9;
        float t[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) t[q] = y[q] * sc.ts[q] + sc.tm[q];
        const float4* st = d.start + ((size_t)sc_i * d.pic + k) * 3;
        const float3 x1 = xyz(st[0]), v1 = xyz(st[1]), F1 = xyz(st[2]);
        const float3 vK = v1 + T * F1 + f3(t[3], t[4], t[5]);
        const float3 xK = x1 + T * v1 + (0.5f * T * T) * F1 + f3(t[0], t[1], t[2]);
        const float3 FK = F1 + f3(t[6], t[7], t[8]);
        const float3 res = xK - x1 - (0.5f * T) * (v1 + vK);
        worst = fmaxf(worst, len3(res));
        finite = finite && isfinite(xK.x) && isfinite(xK.y) && isfinite(xK.z) && isfinite(vK.x) &&
                 isfinite(vK.y) && isfinite(vK.z) && isfinite(FK.x) && isfinite(FK.y) && isfinite(FK.z);
        px[nk] = xK;
        pv[nk] = vK;
        pF[nk] = FK;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) worst = fmaxf(worst, __shfl_xor_sync(0xffffffffu, worst, o));
    const bool ok = __all_sync(0xffffffffu, finite) && worst <= d.tolerance && pic <= 6 * 32;
    if (lane == 0) {
        d.skip[ty.cell_global + cell] = ok ? 1 : 0;
        atomicAdd(&d.counts[ok ? 0 : 1], 1ull);
    }
    if (!ok) return;
    // vein-end rule on the predicted state, keyed by the last sub-step
    bool leave = false;
    nk = 0;
    for (int k = lane; k < pic; k += 32, ++nk) leave = leave || leaves_vein(scn, px[nk]);
    leave = a.p.use_blood_flow && __any_sync(0xffffffffu, leave);
    const long long step = *a.steps + (d.K - 1);
    unsigned e = 0;
    nk = 0;
    for (int k = lane; k < pic; k += 32, ++nk) {
        float3 x = px[nk], v = pv[nk];
        if (leave) respawn(a, scn, ty.cell_start + cell, step, ty.model_start + k, x, v);
        const int p = p0 + k;
        const float w = a.pos_out[p].w;
        a.pos_out[p] = make_float4(x.x, x.y, x.z, w);
        a.vel_out[p] = make_float4(v.x, v.y, v.z, 0.f);
        a.frc_out[p] = make_float4(pF[nk].x, pF[nk].y, pF[nk].z, 0.f);
        if (a.keys_out) a.keys_out[p] = a.pg.uniform ? grid_key(scn.pg, x, e) : 0;
    }
    if (e) atomicOr(a.err, e);
}

// Position error after the span of the network's prediction and of the
// constant-force extrapolation it corrects (whose residual is the raw
// target), summed over the valid samples' particles: sums[0] += |dx_pred -
// dx|, sums[1] += |dx|, sums[2] += particles.
__global__ void k_sur_eval(const float* __restrict__ Y, const float* __restrict__ raw_t,
                           const unsigned char* __restrict__ valid, const SurScales sc, int first, int cells, int pic,
                           double* sums) {
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (b >= cells || !valid[first + b]) return;
    double en = 0.0, eb = 0.0;
    for (int k = lane; k < pic; k += 32) {
        const float* y = Y + ((size_t)b * pic + k) * 9;
        const float* t = raw_t + ((size_t)(first + b) * pic + k) * 9;
        float d2 = 0.f, b2 = 0.f;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float pred = y[q] * sc.ts[q] + sc.tm[q];
            d2 += (pred - t[q]) * (pred - t[q]);
            b2 += t[q] * t[q];
        }
        en += sqrtf(d2);
        eb += sqrtf(b2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        en += __shfl_xor_sync(0xffffffffu, en, o);
        eb += __shfl_xor_sync(0xffffffffu, eb, o);
    }
    if (lane == 0) {
        atomicAdd(&sums[0], en);
        atomicAdd(&sums[1], eb);
        atomicAdd(&sums[2], (double)pic);
    }
}

// ------------------------------------------------------ scene start ----
// The reference's initial placement (generateRandomPositonsAndVelocitiesKernel
// and setBloodCellsPositionsFromRandom, simulation_controller.cu:176-220):
// each cell's origin at x, z uniform in +-0.6 cylinderRadius and y =
// minSpawnY - 180 u min(N / 1000, 1), its particles at origin + model
// vertex, velocity initVelocity, force 0.  Philox4x32-10 keyed by (seed,
// cell within the scene) replaces the per-thread curand states.
__global__ void k_init_reference(const StepArgs a, float4* pos, float4* vel, float4* frc, const float4* __restrict__ model,
                                 const float* __restrict__ radius, unsigned long long seed) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const TypeDev ty = a.types[type_of_particle(a, p)];
    const SceneDev& sc = a.scenes[ty.scene];
    const int cell = (p - ty.particle_start) / ty.pic, k = (p - ty.particle_start) - cell * ty.pic;
    uint32_t c[4] = {(uint32_t)(ty.cell_start + cell), 0xFFFFFFFFu, 0xFFFFFFFFu, 1u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const float n = (float)(sc.particle_end - sc.particle_start);
    const float ox = (uniform_open(c[0]) - 0.5f) * 1.2f * sc.cylinder_radius;
    const float oy = sc.min_spawn_y - 180.0f * uniform_open(c[1]) * fminf(n / 1000.0f, 1.0f);
    const float oz = (uniform_open(c[2]) - 0.5f) * 1.2f * sc.cylinder_radius;
    const float4 m = model[ty.model_start + k];
    pos[p] = make_float4(ox + m.x, oy + m.y, oz + m.z, radius[p]);
    vel[p] = make_float4(a.p.init_velocity[0], a.p.init_velocity[1], a.p.init_velocity[2], 0.f);
    frc[p] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Non-overlapping start: candidate sites of a cubic lattice of the given
// spacing over the scene's vein box; a site is valid when a sphere of
// `clear` around it lies inside the lumen (inside a flow segment, or without
// segments inside the cylinder of cylinderRadius about the y axis over the
// vein's height).  Valid sites get a Philox priority, invalid ones sort last.
__global__ void k_lattice_sites(const SceneDev* __restrict__ scenes, int scene, float3 lo, int nx, int ny, int nz,
                                float spacing, float clear, float ymin, float ymax,
                                const bcs_flow_segment* __restrict__ flows, unsigned long long seed, int* keys,
                                int* ids, int* valid_count) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)nx * ny * nz;
    if (i >= total) return;
    const SceneDev& sc = scenes[scene];
    const int ix = (int)(i % nx), iy = (int)((i / nx) % ny), iz = (int)(i / ((long long)nx * ny));
    const float3 q = f3(lo.x + (ix + 0.5f) * spacing, lo.y + (iy + 0.5f) * spacing, lo.z + (iz + 0.5f) * spacing);
    bool ok = false;
    if (sc.flow_count > 0) {
        for (int k = 0; k < sc.flow_count && !ok; ++k) {
            const bcs_flow_segment& f = flows[sc.flow_start + k];
            const float3 o = f3(f.origin[0], f.origin[1], f.origin[2]), d = f3(f.direction[0], f.direction[1], f.direction[2]);
            const float t = dot3(q - o, d);
            const float3 radial = (q - o) - t * d;
            ok = t > clear && t < f.length - clear && len3(radial) < f.radius - clear;
        }
    } else {
        ok = sqrtf(q.x * q.x + q.z * q.z) < sc.cylinder_radius - clear && q.y > ymin + clear && q.y < ymax - clear;
    }
    uint32_t c[4] = {(uint32_t)i, (uint32_t)(i >> 32), 0x51734u, 2u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    keys[i] = ok ? (int)(c[0] >> 2) : 0x40000000;
    ids[i] = (int)i;
    if (ok) atomicAdd(valid_count, 1);
}

// Cells of the scene at the first sites of the sorted order (cell order
// within the scene), particles at site + (model vertex - model centroid),
// velocities initVelocity + sigma N(0, 1) per component (Box-Muller on a
// Philox draw per particle), force 0.
__global__ void k_lattice_place(const StepArgs a, int scene, float4* pos, float4* vel, float4* frc,
                                const float4* __restrict__ model, const float* __restrict__ centroid,
                                const float* __restrict__ radius, const int* __restrict__ site_ids, float3 lo,
                                int nx, int ny, float spacing, float sigma, unsigned long long seed) {
    const SceneDev& sc = a.scenes[scene];
    const int p = sc.particle_start + blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= sc.particle_end) return;
    const int t = type_of_particle(a, p);
    const TypeDev ty = a.types[t];
    const int cell = (p - ty.particle_start) / ty.pic, k = (p - ty.particle_start) - cell * ty.pic;
    const long long site = site_ids[ty.cell_start + cell];
    const int ix = (int)(site % nx), iy = (int)((site / nx) % ny), iz = (int)(site / ((long long)nx * ny));
    const float4 m = model[ty.model_start + k];
    const float* cen = centroid + 3 * t;
    pos[p] = make_float4(lo.x + (ix + 0.5f) * spacing + (m.x - cen[0]), lo.y + (iy + 0.5f) * spacing + (m.y - cen[1]),
                         lo.z + (iz + 0.5f) * spacing + (m.z - cen[2]), radius[p]);
    uint32_t c[4] = {(uint32_t)(p - sc.particle_start), 0x7E10u, 0u, 3u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const float r1 = sqrtf(-2.0f * logf(uniform_open(c[0]))), r2 = sqrtf(-2.0f * logf(uniform_open(c[2])));
    const float a1 = 6.2831853f * uniform_open(c[1]), a2 = 6.2831853f * uniform_open(c[3]);
    vel[p] = make_float4(a.p.init_velocity[0] + sigma * r1 * cosf(a1), a.p.init_velocity[1] + sigma * r1 * sinf(a1),
                         a.p.init_velocity[2] + sigma * r2 * cosf(a2), 0.f);
    frc[p] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ------------------------------------------- fused network inference ----
// One CTA per cell of the surrogate's model runs the whole network on chip:
// the residual stream h in FP32 shared memory, B and then M in bf16 shared
// memory, each 128 x 128 weight staged once per product, the products on
// bf16 tensor cores (mma.sync m16n8k16, FP32 accumulation) with warp w
// owning rows 16w .. 16w + 15; the messages, encoder and decoder in FP32.
// The same rounding points as the layer-by-layer kernels.  The epilogue is
// k_sur_apply's: decode, residual check, state and grid keys of a passing
// cell, skip flag and counts.
constexpr int kFusedHP = kHidden + 8;   // FP32 row stride of h (8 banks apart: 64-bit fragment reads conflict-free)
constexpr int kFusedBP = kHidden + 8;   // bf16 row stride
constexpr int kFusedW = 2176;           // floats of the small-weight area
constexpr int kFusedMaxEdges = 1536;    // directed springs of one cell held in shared memory

// Small-weight area of the double-buffered layout: W_e, b_e, b_u, b_b of a
// layer, or W_out and b_out (the encoder's weights go to the second tile).
constexpr int kFusedWDb = kEdgeIn * kHidden + 3 * kHidden;

template <int MT>
__host__ __device__ constexpr int fused_smem_single() {
    return MT * 16 * kFusedHP * 4 + MT * 16 * kFusedBP * 2 + kHidden * kFusedBP * 2 + MT * 16 * kEdgeIn * 4 +
           kFusedW * 4 + MT * 16 * kOut * 4 + 16 + (MT * 16 + 1) * 4 + kFusedMaxEdges * 4;
}
// Two weight tiles (the next product's weights stream in with cp.async while
// the current one runs); the decoder's output shares the message buffer.
template <int MT>
__host__ __device__ constexpr int fused_smem_double() {
    return MT * 16 * kFusedHP * 4 + MT * 16 * kFusedBP * 2 + 2 * kHidden * kFusedBP * 2 + MT * 16 * kEdgeIn * 4 +
           kFusedWDb * 4 + 16 + (MT * 16 + 1) * 4 + kFusedMaxEdges * 4;
}
template <int MT>
__host__ __device__ constexpr bool fused_double() { return fused_smem_double<MT>() <= 227 * 1024; }
template <int MT>
__host__ __device__ constexpr int fused_smem_bytes() {
    return fused_double<MT>() ? fused_smem_double<MT>() : fused_smem_single<MT>();
}

__device__ inline void stage_weight(const __nv_bfloat16* __restrict__ Wt, __nv_bfloat16* Ws, int nthreads) {
    for (int q = threadIdx.x; q < kHidden * (kHidden / 8); q += nthreads) {
        const int n = q >> 4, k = (q & 15) * 8;
        *reinterpret_cast<uint4*>(Ws + n * kFusedBP + k) = *reinterpret_cast<const uint4*>(Wt + n * kHidden + k);
    }
}

// The same copy with cp.async (16 bytes per thread and step), left in flight:
// stage_weight_wait() completes it for this thread; a barrier after that
// publishes it to the CTA.
__device__ inline void stage_weight_async(const __nv_bfloat16* __restrict__ Wt, __nv_bfloat16* Ws, int nthreads) {
    for (int q = threadIdx.x; q < kHidden * (kHidden / 8); q += nthreads) {
        const int n = q >> 4, k = (q & 15) * 8;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(Ws + n * kFusedBP + k);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(Wt + n * kHidden + k) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ inline void stage_weight_wait() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Two warps share each 16-row group: warp half `hn` owns output columns
// 64 hn .. 64 hn + 63 (n-tiles 8 hn .. 8 hn + 7).
constexpr int kFusedNT = 8;   // n-tiles per warp

// acc (this warp's 16 rows x 64 columns) += H (FP32 smem, rounded to bf16) x Ws^T.
__device__ inline void fused_gemm_h(const float* Hs, const __nv_bfloat16* Ws, float (&acc)[kFusedNT][4], int r_lo,
                                    int hn, int t) {
    const float* lo = Hs + r_lo * kFusedHP + 2 * t;
    const float* hi = lo + 8 * kFusedHP;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int ks = 0; ks < kHidden / 16; ++ks) {
        const int k0 = ks * 16;
        const uint32_t a0 = pack_bf16(lo[k0], lo[k0 + 1]), a1 = pack_bf16(hi[k0], hi[k0 + 1]);
        const uint32_t a2 = pack_bf16(lo[k0 + 8], lo[k0 + 9]), a3 = pack_bf16(hi[k0 + 8], hi[k0 + 9]);
#pragma unroll
        for (int nt = 0; nt < kFusedNT; nt += 2) {
            uint32_t b0, b1, b2, b3;
            ldsm_b_pair(Ws, kFusedBP, (hn * kFusedNT + nt) * 8, k0, lane, b0, b1, b2, b3);
            mma_bf16(acc[nt], a0, a1, a2, a3, b0, b1);
            mma_bf16(acc[nt + 1], a0, a1, a2, a3, b2, b3);
        }
    }
}

// acc += M (bf16 smem) x Ws^T, the same 64 columns.
__device__ inline void fused_gemm_b(const __nv_bfloat16* Bs, const __nv_bfloat16* Ws, float (&acc)[kFusedNT][4],
                                    int r_lo, int hn, int t) {
    const __nv_bfloat16* lo = Bs + r_lo * kFusedBP + 2 * t;
    const __nv_bfloat16* hi = lo + 8 * kFusedBP;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int ks = 0; ks < kHidden / 16; ++ks) {
        const int k0 = ks * 16;
        const uint32_t a0 = ld32(lo + k0), a1 = ld32(hi + k0), a2 = ld32(lo + k0 + 8), a3 = ld32(hi + k0 + 8);
#pragma unroll
        for (int nt = 0; nt < kFusedNT; nt += 2) {
            uint32_t b0, b1, b2, b3;
            ldsm_b_pair(Ws, kFusedBP, (hn * kFusedNT + nt) * 8, k0, lane, b0, b1, b2, b3);
            mma_bf16(acc[nt], a0, a1, a2, a3, b0, b1);
            mma_bf16(acc[nt + 1], a0, a1, a2, a3, b2, b3);
        }
    }
}

template <int MT>
__global__ void __launch_bounds__(MT * 64, 1)
    k_sur_fused(const StepArgs a, const SurDev d, const SurScales sc, const float* __restrict__ P,
                const __nv_bfloat16* __restrict__ PB, const __nv_bfloat16* __restrict__ PBT, const MpnnLayout L,
                const int* __restrict__ goff, const int* __restrict__ gnbr, const float* __restrict__ glen, int first,
                int cells) {
    constexpr int R = MT * 16, NT = MT * 64;   // 2 MT warps: two per 16-row group
    constexpr bool DB = fused_double<MT>();
    extern __shared__ __align__(16) unsigned char smem[];
    float* Hs = reinterpret_cast<float*>(smem);
    __nv_bfloat16* Bs = reinterpret_cast<__nv_bfloat16*>(Hs + R * kFusedHP);
    __nv_bfloat16* Ws = Bs + R * kFusedBP;                     // weight tile (DB: the first of two)
    __nv_bfloat16* Ws2 = DB ? Ws + kHidden * kFusedBP : Ws;   // the second tile
    float* Node = reinterpret_cast<float*>(Ws2 + kHidden * kFusedBP);   // R x 8 ebar
    float* Wsm = Node + R * 8;
    float* Ysm = DB ? reinterpret_cast<float*>(Bs) : Wsm + kFusedW;   // DB: after the layers, B is free
    int* red = reinterpret_cast<int*>(DB ? Wsm + kFusedWDb : Ysm + R * kOut);
    float* Wenc = DB ? reinterpret_cast<float*>(Ws2) : Wsm;   // encoder weights (DB: in the idle second tile)
    int* Goff = red + 4;            // R + 1 spring-list offsets (rows past the cell: empty)
    int* Gnbr = Goff + R + 1;       // the cell's directed springs
    const int b = blockIdx.x;
    if (b >= cells) return;
    const int sc_i = first + b, pic = d.pic;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const int wr = warp % MT, hn = warp / MT;   // row group, column half
    const int r_lo = wr * 16 + g;
    for (int i = tid; i <= R; i += NT) Goff[i] = goff[min(i, pic)];
    for (int i = tid; i < goff[pic]; i += NT) Gnbr[i] = gnbr[i];

    // ---- encoder, and the mean edge features of every node
    float* F0 = reinterpret_cast<float*>(Bs);   // R x 16 normalised features, then R x 6 raw r, u
    const float* raw = d.raw + (size_t)sc_i * pic * 16;
    for (int i = tid; i < R * 16; i += NT) {
        const int r = i >> 4, q = i & 15;
        F0[i] = r < pic ? (raw[r * 16 + q] - sc.fm[q]) * sc.fs[q] : 0.f;
    }
    if (DB) stage_weight_async(PBT + L.wb[0], Ws, NT);   // streams in during the encoder
    for (int i = tid; i < kFeatIn * kHidden; i += NT) Wenc[i] = __bfloat162float(PB[L.w_in + i]);
    for (int i = tid; i < kHidden; i += NT) Wenc[kFeatIn * kHidden + i] = P[L.b_in + i];
    if (tid == 0) {
        red[0] = 0;   // worst residual (float bits)
        red[1] = 1;   // all finite
        red[2] = 0;   // leaves the vein
    }
    __syncthreads();
    // a warp per row, lane l on columns 4l..4l+3: every weight row is one
    // conflict-free 512-byte read and the row of h one 512-byte write
    for (int i = tid; i < R * (kHidden / 4); i += NT) {
        const int r = i >> 5, c0 = (i & 31) * 4;
        float fr[kFeatIn];
#pragma unroll
        for (int q = 0; q < kFeatIn; ++q) fr[q] = F0[r * 16 + q];
        const float4 b4 = *reinterpret_cast<const float4*>(Wenc + kFeatIn * kHidden + c0);
        float z[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
        for (int q = 0; q < kFeatIn; ++q) {
            const float4 w = *reinterpret_cast<const float4*>(Wenc + q * kHidden + c0);
            z[0] = fmaf(fr[q], w.x, z[0]);
            z[1] = fmaf(fr[q], w.y, z[1]);
            z[2] = fmaf(fr[q], w.z, z[2]);
            z[3] = fmaf(fr[q], w.w, z[3]);
        }
        const bool live = r < pic;
        *reinterpret_cast<float4*>(Hs + r * kFusedHP + c0) =
            make_float4(live ? silu_f(z[0]) : 0.f, live ? silu_f(z[1]) : 0.f, live ? silu_f(z[2]) : 0.f,
                        live ? silu_f(z[3]) : 0.f);
    }
    __syncthreads();
    float* RU = F0;   // raw r, u of every node (stride 6) while Bs is free
    for (int i = tid; i < R * 6; i += NT) {
        const int r = i / 6, q = i - r * 6;
        RU[i] = r < pic ? raw[r * 16 + q] : 0.f;
    }
    __syncthreads();
    for (int r = tid; r < R; r += NT) {
        float eb[kEdgeIn] = {};
        if (r < pic) {
            const int e0 = Goff[r], e1 = Goff[r + 1];
            for (int k = e0; k < e1; ++k) {
                float e[kEdgeIn];
                spring_features(RU + r * 6, RU + Gnbr[k] * 6, glen[k], sc, e);
#pragma unroll
                for (int q = 0; q < kEdgeIn; ++q) eb[q] += e[q];
            }
            const float inv = 1.0f / (float)max(1, e1 - e0);
#pragma unroll
            for (int q = 0; q < kEdgeIn; ++q) eb[q] *= inv;
        }
#pragma unroll
        for (int q = 0; q < kEdgeIn; ++q) Node[r * kEdgeIn + q] = eb[q];
    }
    __syncthreads();

    // ---- message-passing layers.  DB: the weight tiles alternate; each
    // product's successor streams into the other tile while it runs (W_b of
    // layer l is in `cur`, then W_u in `oth`, W_v in `cur`, W_b of l + 1 in
    // `oth`, which becomes the next layer's `cur`).
    __nv_bfloat16* cur = Ws;
    __nv_bfloat16* oth = Ws2;
    for (int l = 0; l < L.layers; ++l) {
        if (!DB) stage_weight(PBT + L.wb[l], Ws, NT);
        for (int i = tid; i < kEdgeIn * kHidden; i += NT) Wsm[i] = __bfloat162float(PB[L.we[l] + i]);
        for (int i = tid; i < kHidden; i += NT) {
            Wsm[kEdgeIn * kHidden + i] = P[L.be[l] + i];
            Wsm[kEdgeIn * kHidden + kHidden + i] = P[L.bu[l] + i];
            Wsm[kEdgeIn * kHidden + 2 * kHidden + i] = P[L.bb[l] + i];
        }
        if (DB) stage_weight_wait();
        __syncthreads();
        if (DB) stage_weight_async(PBT + L.wu[l], oth, NT);
        {
            // B = silu(h W_b + b_b), kept in bf16
            float acc[kFusedNT][4];
#pragma unroll
            for (int nt = 0; nt < kFusedNT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
            fused_gemm_h(Hs, cur, acc, r_lo, hn, t);
            const float* bb = Wsm + kEdgeIn * kHidden + 2 * kHidden;
#pragma unroll
            for (int nt = 0; nt < kFusedNT; ++nt) {
                const int c = (hn * kFusedNT + nt) * 8 + 2 * t;
                *reinterpret_cast<uint32_t*>(Bs + r_lo * kFusedBP + c) =
                    pack_bf16(silu_f(acc[nt][0] + bb[c]), silu_f(acc[nt][1] + bb[c + 1]));
                *reinterpret_cast<uint32_t*>(Bs + (r_lo + 8) * kFusedBP + c) =
                    pack_bf16(silu_f(acc[nt][2] + bb[c]), silu_f(acc[nt][3] + bb[c + 1]));
            }
        }
        __syncthreads();
        // single tile: W_u streams into it (free now) during the aggregation
        if (!DB) stage_weight_async(PBT + L.wu[l], Ws, NT);
        // M = mean over the springs of B_j + ebar W_e + b_e for 8 rows per
        // warp (half of its row group), one row at a time: lane l holds
        // columns 4l..4l+3, so a neighbour's row is one conflict-free
        // 256-byte read and the spring loop is the same for the whole warp
        float m[8][4];
        const float* We = Wsm;
        const float* be = Wsm + kEdgeIn * kHidden;
        const int c4 = 4 * lane;
        const int m0 = wr * 16 + hn * 8;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int r = m0 + i;
            const int e0 = Goff[r], e1 = Goff[r + 1];
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
            for (int k = e0; k < e1; ++k) {
                const uint2 v = *reinterpret_cast<const uint2*>(Bs + Gnbr[k] * kFusedBP + c4);
                const __nv_bfloat162 lo = *reinterpret_cast<const __nv_bfloat162*>(&v.x);
                const __nv_bfloat162 hi = *reinterpret_cast<const __nv_bfloat162*>(&v.y);
                s0 += __low2float(lo);
                s1 += __high2float(lo);
                s2 += __low2float(hi);
                s3 += __high2float(hi);
            }
            const float inv = 1.0f / (float)max(1, e1 - e0);
            const float4 eb0 = *reinterpret_cast<const float4*>(Node + r * kEdgeIn);
            const float4 eb1 = *reinterpret_cast<const float4*>(Node + r * kEdgeIn + 4);
            const float eb[kEdgeIn] = {eb0.x, eb0.y, eb0.z, eb0.w, eb1.x, eb1.y, eb1.z, eb1.w};
            const float4 b4 = *reinterpret_cast<const float4*>(be + c4);
            float tt[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
            for (int q = 0; q < kEdgeIn; ++q) {
                const float4 w = *reinterpret_cast<const float4*>(We + q * kHidden + c4);
                tt[0] = fmaf(eb[q], w.x, tt[0]);
                tt[1] = fmaf(eb[q], w.y, tt[1]);
                tt[2] = fmaf(eb[q], w.z, tt[2]);
                tt[3] = fmaf(eb[q], w.w, tt[3]);
            }
            const float sum[4] = {s0, s1, s2, s3};
#pragma unroll
            for (int u = 0; u < 4; ++u) m[i][u] = r < pic ? sum[u] * inv + tt[u] : 0.f;
        }
        __syncthreads();   // every read of B is done
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            uint2 w;
            w.x = pack_bf16(m[i][0], m[i][1]);
            w.y = pack_bf16(m[i][2], m[i][3]);
            *reinterpret_cast<uint2*>(Bs + (m0 + i) * kFusedBP + c4) = w;
        }
        stage_weight_wait();
        __syncthreads();
        if (DB) stage_weight_async(PBT + L.wv[l], cur, NT);   // cur's W_b is done
        float accU[kFusedNT][4];
#pragma unroll
        for (int nt = 0; nt < kFusedNT; ++nt) accU[nt][0] = accU[nt][1] = accU[nt][2] = accU[nt][3] = 0.f;
        fused_gemm_h(Hs, DB ? oth : Ws, accU, r_lo, hn, t);
        if (DB) {
            stage_weight_wait();
            __syncthreads();   // W_v landed, and every warp is done with oth's W_u
            if (l + 1 < L.layers) stage_weight_async(PBT + L.wb[l + 1], oth, NT);
        } else {
            __syncthreads();
            stage_weight(PBT + L.wv[l], Ws, NT);
            __syncthreads();
        }
        fused_gemm_b(Bs, cur, accU, r_lo, hn, t);
        const float* bu = Wsm + kEdgeIn * kHidden + kHidden;
#pragma unroll
        for (int nt = 0; nt < kFusedNT; ++nt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = r_lo + 8 * h;
                if (r >= pic) continue;
                const int c = (hn * kFusedNT + nt) * 8 + 2 * t;
                float2* hp = reinterpret_cast<float2*>(Hs + r * kFusedHP + c);
                float2 hv = *hp;
                hv.x += silu_f(accU[nt][2 * h] + bu[c]);
                hv.y += silu_f(accU[nt][2 * h + 1] + bu[c + 1]);
                *hp = hv;
            }
        __syncthreads();
        if (DB) {
            __nv_bfloat16* tmp = cur;
            cur = oth;
            oth = tmp;
        }
    }

    // ---- decoder on the tensor cores: W_out^T (9 outputs padded to 16) as a
    // bf16 tile in the free weight tile; h split into bf16 high and low
    // parts (h = hi + lo to 2^-16 relative), so y = hi W + lo W keeps the
    // FP32 decoder's accuracy.  Warp half hn takes outputs 8 hn .. 8 hn + 7.
    __nv_bfloat16* Wo = Ws;   // 16 rows (outputs) x 128 (hidden), stride kFusedBP
    for (int i = tid; i < 16 * kHidden; i += NT) {
        const int o = i / kHidden, c = i - o * kHidden;
        Wo[o * kFusedBP + c] = o < kOut ? PB[L.w_out + c * kOut + o] : __float2bfloat16_rn(0.f);
    }
    __syncthreads();
    {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        const float* lo = Hs + r_lo * kFusedHP + 2 * t;
        const float* hi = lo + 8 * kFusedHP;
#pragma unroll
        for (int ks = 0; ks < kHidden / 16; ++ks) {
            const int k0 = ks * 16;
            const float h[8] = {lo[k0], lo[k0 + 1], hi[k0], hi[k0 + 1], lo[k0 + 8], lo[k0 + 9], hi[k0 + 8], hi[k0 + 9]};
            float rem[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) rem[j] = h[j] - round_bf16(h[j]);
            uint32_t b0, b1, b2, b3;
            ldsm_b_pair(Wo, kFusedBP, 0, k0, lane, b0, b1, b2, b3);
            const uint32_t bx = hn ? b2 : b0, by = hn ? b3 : b1;
            mma_bf16(acc, pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]), pack_bf16(h[6], h[7]),
                     bx, by);
            mma_bf16(acc, pack_bf16(rem[0], rem[1]), pack_bf16(rem[2], rem[3]), pack_bf16(rem[4], rem[5]),
                     pack_bf16(rem[6], rem[7]), bx, by);
        }
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
            const int r = r_lo + 8 * h2;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int o = hn * 8 + 2 * t + u;
                if (r < pic && o < kOut) Ysm[r * kOut + o] = acc[2 * h2 + u] + P[L.b_out + o];
            }
        }
    }
    __syncthreads();

    // ---- decode, residual check, state of a passing cell
    const TypeDev ty = a.types[d.cell_type[sc_i]];
    const SceneDev& scn = a.scenes[ty.scene];
    const int cell = d.cell_index[sc_i], p0 = ty.particle_start + cell * pic;
    const float T = d.T;
    for (int k = tid; k < pic; k += NT) {
        float tt[kOut];
#pragma unroll
        for (int q = 0; q < kOut; ++q) tt[q] = Ysm[k * kOut + q] * sc.ts[q] + sc.tm[q];
        const float4* st = d.start + ((size_t)sc_i * pic + k) * 3;
        const float3 x1 = xyz(st[0]), v1 = xyz(st[1]), F1 = xyz(st[2]);
        const float3 vK = v1 + T * F1 + f3(tt[3], tt[4], tt[5]);
        const float3 xK = x1 + T * v1 + (0.5f * T * T) * F1 + f3(tt[0], tt[1], tt[2]);
        const float3 FK = F1 + f3(tt[6], tt[7], tt[8]);
        const float res = len3(xK - x1 - (0.5f * T) * (v1 + vK));
        const bool fin = isfinite(xK.x) && isfinite(xK.y) && isfinite(xK.z) && isfinite(vK.x) && isfinite(vK.y) &&
                         isfinite(vK.z) && isfinite(FK.x) && isfinite(FK.y) && isfinite(FK.z);
        if (!fin) atomicAnd(&red[1], 0);
        else atomicMax(&red[0], __float_as_int(res));
        Ysm[k * kOut + 0] = xK.x; Ysm[k * kOut + 1] = xK.y; Ysm[k * kOut + 2] = xK.z;
        Ysm[k * kOut + 3] = vK.x; Ysm[k * kOut + 4] = vK.y; Ysm[k * kOut + 5] = vK.z;
        Ysm[k * kOut + 6] = FK.x; Ysm[k * kOut + 7] = FK.y; Ysm[k * kOut + 8] = FK.z;
        if (a.p.use_blood_flow && leaves_vein(scn, xK)) atomicOr(&red[2], 1);
    }
    __syncthreads();
    const bool ok = red[1] && __int_as_float(red[0]) <= d.tolerance;
    if (tid == 0) {
        d.skip[ty.cell_global + cell] = ok ? 1 : 0;
        atomicAdd(&d.counts[ok ? 0 : 1], 1ull);
    }
    if (!ok) return;
    const bool leave = red[2] != 0;
    const long long step = *a.steps + (d.K - 1);
    unsigned e = 0;
    for (int k = tid; k < pic; k += NT) {
        float3 x = f3(Ysm[k * kOut + 0], Ysm[k * kOut + 1], Ysm[k * kOut + 2]);
        float3 v = f3(Ysm[k * kOut + 3], Ysm[k * kOut + 4], Ysm[k * kOut + 5]);
        if (leave) respawn(a, scn, ty.cell_start + cell, step, ty.model_start + k, x, v);
        const int p = p0 + k;
        const float w = a.pos_out[p].w;
        a.pos_out[p] = make_float4(x.x, x.y, x.z, w);
        a.vel_out[p] = make_float4(v.x, v.y, v.z, 0.f);
        a.frc_out[p] = make_float4(Ysm[k * kOut + 6], Ysm[k * kOut + 7], Ysm[k * kOut + 8], 0.f);
        if (a.keys_out) a.keys_out[p] = a.pg.uniform ? grid_key(scn.pg, x, e) : 0;
    }
    if (e) atomicOr(a.err, e);
}

__global__ void k_cell_ranges(const int* __restrict__ keys, int n, int4* table, const int* __restrict__ epoch,
                              unsigned* occ, const int* __restrict__ ids, const float4* __restrict__ pos,
                              float4* spos, const float4* __restrict__ vel, float4* svel) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (spos) {
        const int id = ids[i];
        spos[i] = pos[id];
        if (svel) svel[i] = vel[id];
    }
    if (!table) return;   // grid-order collisions: the range table is built on demand only
    const int k = keys[i];
    if (i > 0 && keys[i - 1] == k) return;
    int j = i;
    while (j + 1 < n && keys[j + 1] == k) ++j;
    table[k] = make_int4(i, j, *epoch, 0);
    if (occ) atomicOr(&occ[k >> 5], 1u << (k & 31));
}

// Set or clear the occupancy bits of the cells a sorted key array occupies.
__global__ void k_occ_update(const int* __restrict__ keys, int n, unsigned* occ, int set) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = keys[i];
    if (i > 0 && keys[i - 1] == k) return;
    if (set) atomicOr(&occ[k >> 5], 1u << (k & 31));
    else atomicAnd(&occ[k >> 5], ~(1u << (k & 31)));
}

// Dense starts/ends (empty = 0, -1) from the epoch-stamped table, for getters.
__global__ void k_dense_ranges(const int4* __restrict__ table, const int* __restrict__ epoch, long long cells,
                               int* starts, int* ends) {
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    int4 r = table[c];
    bool occ = r.z == *epoch;
    if (starts) starts[c] = occ ? r.x : 0;
    if (ends) ends[c] = occ ? r.y : -1;
}

// Vein springs, gatherForcesKernel (vein_triangles.cu:125-154), nine
// neighbour slots per vertex (VeinNeighbors).
__global__ void k_vein_springs(const float4* __restrict__ vpos, const float4* __restrict__ vvel, float4* vfrc,
                               const int* __restrict__ nb_ids, const float* __restrict__ nb_len, int V, float k_sniff,
                               float d_fact, unsigned* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    unsigned e = 0;
    const float3 pi = xyz(vpos[i]), vi = xyz(vvel[i]);
    float3 acc = f3(0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        int j = nb_ids[(size_t)k * V + i];
        if (j == -1) continue;
        float L = nb_len[(size_t)k * V + i];
        float3 pj = xyz(vpos[j]);
        float mag = (len3(pi - pj) - L) * k_sniff + dot3(normalize_or_zero(pi - pj, e), vi - xyz(vvel[j])) * d_fact;
        acc = acc + mag * normalize_or_zero(pj - pi, e);
    }
    float4 f = vfrc[i];
    vfrc[i] = make_float4(f.x + acc.x, f.y + acc.y, f.z + acc.z, 0.f);
    if (e) atomicOr(err, e);
}

// propagateForcesIntoPositionsKernel + the three force memsets
// (vein_triangles.cu:88-117): semi-implicit Euler, then F = 0.
__global__ void k_vein_integrate(float4* vpos, float4* vvel, float4* vfrc, int V, float dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    float3 f = xyz(vfrc[i]);
    float3 v = xyz(vvel[i]) + dt * f;
    float3 x = xyz(vpos[i]) + dt * v;
    vvel[i] = make_float4(v.x, v.y, v.z, 0.f);
    vpos[i] = make_float4(x.x, x.y, x.z, 0.f);
    vfrc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Moller-Trumbore operands per sorted triangle slot (ids == null: identity).
__global__ void k_tri_cache(const int* __restrict__ ids, const uint32_t* __restrict__ tri,
                            const float4* __restrict__ vpos, int T, float4* cache) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= T) return;
    int t = ids ? ids[s] : s;
    float3 v0 = xyz(vpos[tri[3 * t]]), v1 = xyz(vpos[tri[3 * t + 1]]), v2 = xyz(vpos[tri[3 * t + 2]]);
    float3 e1 = v1 - v0, e2 = v2 - v0;
    cache[3 * s] = make_float4(v0.x, v0.y, v0.z, __int_as_float(t));
    cache[3 * s + 1] = make_float4(e1.x, e1.y, e1.z, 0.f);
    cache[3 * s + 2] = make_float4(e2.x, e2.y, e2.z, 0.f);
}

// Bounds of each occupied triangle-grid cell's triangles (from the exact
// vertex positions), widened by a margin that covers FP32 rounding in the
// ray-box test.  With a wall mask, every mask cell that meets those bounds
// widened by `reach` gets the current mark: a particle in an unmarked mask
// cell is farther than `reach` from every triangle.
__global__ void k_tri_boxes(const int* __restrict__ keys, const int* __restrict__ ids, int T,
                            const uint32_t* __restrict__ tri, const float4* __restrict__ vpos, float4* box,
                            const SceneDev* __restrict__ scenes, int scene_count, unsigned char* mask,
                            const int* __restrict__ mask_epoch, float reach, float margin,
                            const float* __restrict__ disp2) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= T) return;
    if (disp2 && *disp2 <= margin * margin) return;   // the last build still covers the wall
    const int k = keys[s];
    if (s > 0 && keys[s - 1] == k) return;
    float3 lo = f3(3.0e38f, 3.0e38f, 3.0e38f), hi = f3(-3.0e38f, -3.0e38f, -3.0e38f);
    for (int j = s; j < T && keys[j] == k; ++j) {
        const int t = ids[j];
        for (int c = 0; c < 3; ++c) {
            float3 q = xyz(vpos[tri[3 * t + c]]);
            lo = f3(fminf(lo.x, q.x), fminf(lo.y, q.y), fminf(lo.z, q.z));
            hi = f3(fmaxf(hi.x, q.x), fmaxf(hi.y, q.y), fmaxf(hi.z, q.z));
        }
    }
    const float mg = margin + 1e-3f + 1e-5f * fmaxf(fmaxf(fmaxf(fabsf(lo.x), fabsf(hi.x)), fmaxf(fabsf(lo.y), fabsf(hi.y))),
                                                    fmaxf(fabsf(lo.z), fabsf(hi.z)));
    lo = f3(lo.x - mg, lo.y - mg, lo.z - mg);
    hi = f3(hi.x + mg, hi.y + mg, hi.z + mg);
    box[2 * (size_t)k] = make_float4(lo.x, lo.y, lo.z, 0.f);
    box[2 * (size_t)k + 1] = make_float4(hi.x, hi.y, hi.z, 0.f);
    if (!mask) return;
    const int sidx = find_range(scene_count, (long long)k, [&](int q) { return scenes[q].tg.key_offset; });
    const MaskGeom& m = scenes[sidx].wall;
    const int x0 = max(0, (int)floorf((lo.x - reach - m.lo[0]) * m.inv_cell));
    const int x1 = min(m.nx - 1, (int)floorf((hi.x + reach - m.lo[0]) * m.inv_cell));
    const int y0 = max(0, (int)floorf((lo.y - reach - m.lo[1]) * m.inv_cell));
    const int y1 = min(m.ny - 1, (int)floorf((hi.y + reach - m.lo[1]) * m.inv_cell));
    const int z0 = max(0, (int)floorf((lo.z - reach - m.lo[2]) * m.inv_cell));
    const int z1 = min(m.nz - 1, (int)floorf((hi.z + reach - m.lo[2]) * m.inv_cell));
    const unsigned char mark = (unsigned char)*mask_epoch;
    for (int z = z0; z <= z1; ++z)
        for (int y = y0; y <= y1; ++y)
            for (int xx = x0; xx <= x1; ++xx) mask[m.offset + ((long long)z * m.ny + y) * m.nx + xx] = mark;
}

// Per triangle-grid cell, the 27-bit word of its stencil neighbours that
// exist (key inside the scene's grid, the reference's key arithmetic) and
// hold triangles in the current build: bit 9 (dx + 1) + 3 (dy + 1) + dz + 1.
__global__ void k_tri_occupancy(const int4* __restrict__ table, const int* __restrict__ epoch,
                                const SceneDev* __restrict__ scenes, int scene_count, long long cells, unsigned* occ) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cells) return;
    const int sidx = find_range(scene_count, k, [&](int q) { return scenes[q].tg.key_offset; });
    const GridGeom& geo = scenes[sidx].tg;
    const long long c = k - geo.key_offset, cxy = (long long)geo.cx * geo.cy;
    const int ep = *epoch;
    unsigned w = 0u;
#pragma unroll
    for (int dx = -1; dx <= 1; ++dx)
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
            for (int dz = -1; dz <= 1; ++dz) {
                const long long n = c + dz * cxy + (long long)dy * geo.cx + dx;
                if (n >= 0 && n < geo.cells && table[geo.key_offset + n].z == ep)
                    w |= 1u << (9 * (dx + 1) + 3 * (dy + 1) + dz + 1);
            }
    occ[k] = w;
}

// Squared distance from p to the triangle (a, b, c): the closest point by
// its Voronoi region (vertex, edge or face), the method of Ericson, Real-Time
// Collision Detection (2005), section 5.1.5.
__device__ inline float point_triangle_d2(float3 p, float3 a, float3 b, float3 c) {
    const float3 ab = b - a, ac = c - a, ap = p - a;
    const float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    float3 q;
    if (d1 <= 0.f && d2 <= 0.f) {
        q = a;
    } else {
        const float3 bp = p - b;
        const float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
        const float3 cp = p - c;
        const float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
        const float vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
        if (d3 >= 0.f && d4 <= d3) q = b;
        else if (d6 >= 0.f && d5 <= d6) q = c;
        else if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) q = a + (d1 / (d1 - d3)) * ab;
        else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) q = a + (d2 / (d2 - d6)) * ac;
        else if (va <= 0.f && d4 - d3 >= 0.f && d5 - d6 >= 0.f) q = b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b);
        else {
            const float den = 1.f / (va + vb + vc);
            q = a + (vb * den) * ab + (vc * den) * ac;
        }
    }
    const float3 d = p - q;
    return dot3(d, d);
}

// Wall mask from the triangles themselves: a mask cell is marked when its
// centre lies within reach (the impact distance, with the rebuild margin)
// plus the cell's half-diagonal of some triangle, so every point of an
// unmarked cell is farther than reach from every triangle: a particle there
// cannot be hit within the impact distance.  One thread per triangle over
// the cells of its widened bounds; a distance that does not come out finite
// (a degenerate triangle) marks the cell.
__global__ void k_wall_mask_tris(const uint32_t* __restrict__ tri, const float4* __restrict__ vpos, int T,
                                 const SceneDev* __restrict__ scenes, int scene_count, unsigned char* mask,
                                 const int* __restrict__ mask_epoch, float reach, float margin,
                                 const float* __restrict__ disp2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    if (disp2 && *disp2 <= margin * margin) return;   // the last build still covers the wall
    const int sidx = find_range(scene_count, t, [&](int q) { return scenes[q].tri_start; });
    const MaskGeom& m = scenes[sidx].wall;
    const float3 a = xyz(vpos[tri[3 * t]]), b = xyz(vpos[tri[3 * t + 1]]), c = xyz(vpos[tri[3 * t + 2]]);
    const float cell = 1.0f / m.inv_cell;
    const float big = fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fmaxf(fabsf(a.z), fabsf(b.x))),
                            fmaxf(fmaxf(fabsf(b.y), fabsf(b.z)), fmaxf(fmaxf(fabsf(c.x), fabsf(c.y)), fabsf(c.z))));
    const float r = reach + 0.8661f * cell + 1e-3f + 1e-5f * big;
    const float r2 = r * r;
    const float3 lo = f3(fminf(a.x, fminf(b.x, c.x)) - r, fminf(a.y, fminf(b.y, c.y)) - r, fminf(a.z, fminf(b.z, c.z)) - r);
    const float3 hi = f3(fmaxf(a.x, fmaxf(b.x, c.x)) + r, fmaxf(a.y, fmaxf(b.y, c.y)) + r, fmaxf(a.z, fmaxf(b.z, c.z)) + r);
    const int x0 = max(0, (int)floorf((lo.x - m.lo[0]) * m.inv_cell)), x1 = min(m.nx - 1, (int)floorf((hi.x - m.lo[0]) * m.inv_cell));
    const int y0 = max(0, (int)floorf((lo.y - m.lo[1]) * m.inv_cell)), y1 = min(m.ny - 1, (int)floorf((hi.y - m.lo[1]) * m.inv_cell));
    const int z0 = max(0, (int)floorf((lo.z - m.lo[2]) * m.inv_cell)), z1 = min(m.nz - 1, (int)floorf((hi.z - m.lo[2]) * m.inv_cell));
    const unsigned char mark = (unsigned char)*mask_epoch;
    // a (nearly) degenerate triangle marks its whole widened bounds
    const float3 n = cross3(b - a, c - a);
    const bool flat = !(dot3(n, n) > 1e-10f * dot3(b - a, b - a) * dot3(c - a, c - a));
    for (int z = z0; z <= z1; ++z)
        for (int y = y0; y <= y1; ++y)
            for (int xx = x0; xx <= x1; ++xx) {
                const float3 p = f3(m.lo[0] + (xx + 0.5f) * cell, m.lo[1] + (y + 0.5f) * cell, m.lo[2] + (z + 0.5f) * cell);
                if (flat || !(point_triangle_d2(p, a, b, c) > r2))
                    mask[m.offset + ((long long)z * m.ny + y) * m.nx + xx] = mark;
            }
}

// Largest squared displacement of any vein vertex since the last bounds
// build (as the int bits of a non-negative float, so atomicMax orders it).
__global__ void k_vein_disp(const float4* __restrict__ vpos, const float4* __restrict__ ref, int V, float* disp2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float d = 0.f;
    if (i < V) {
        const float3 a = xyz(vpos[i]), b = xyz(ref[i]);
        d = dot3(a - b, a - b);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, o));
    if ((threadIdx.x & 31) == 0 && d > 0.f) atomicMax(reinterpret_cast<int*>(disp2), __float_as_int(d));
}

// After a rebuild: the current vein positions become the reference.
__global__ void k_vein_snapshot(const float4* __restrict__ vpos, float4* ref, int V, const float* disp2, float margin) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < V && *disp2 > margin * margin) ref[i] = vpos[i];
}

__global__ void k_disp_reset(float* disp2, float margin) {
    if (*disp2 > margin * margin) *disp2 = 0.f;
}

__global__ void k_next_epoch_if(int* epoch, const float* disp2, float margin) {
    if (!disp2 || *disp2 > margin * margin) *epoch += 1;
}

__global__ void k_bump_step(long long* steps, int by) { *steps += by; }

__global__ void k_gather_rows(const float4* __restrict__ src, const int* __restrict__ idx, int n, float4* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = src[idx[i]];
}

// Headless stand-in for calculatePositionsKernel / calculateTriangleVerticesKernel
// (src/graphics/glcontroller.cu:22-49).
__global__ void k_export(const float4* __restrict__ pos, int n, const float4* __restrict__ vpos, int V, float* pvbo,
                         float* poff, float* vvbo) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float4 q = pos[i];
        if (pvbo) {
            pvbo[6 * i] = q.x; pvbo[6 * i + 1] = q.y; pvbo[6 * i + 2] = q.z;
            pvbo[6 * i + 3] = 0.f; pvbo[6 * i + 4] = 0.f; pvbo[6 * i + 5] = 0.f;
        }
        if (poff) { poff[3 * i] = q.x; poff[3 * i + 1] = q.y; poff[3 * i + 2] = q.z; }
    }
    if (i < V && vvbo) {
        float4 q = vpos[i];
        vvbo[6 * i] = q.x; vvbo[6 * i + 1] = q.y; vvbo[6 * i + 2] = q.z;
        vvbo[6 * i + 3] = 0.f; vvbo[6 * i + 4] = 0.f; vvbo[6 * i + 5] = 0.f;
    }
}

// SoA (cudaVec3) <-> float4 packing for the state getters and setters.
__global__ void k_pack(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ z, int n,
                       float4* out, const float* __restrict__ wsrc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = make_float4(x ? x[i] : 0.f, y ? y[i] : 0.f, z ? z[i] : 0.f, wsrc ? wsrc[i] : 0.f);
}

__global__ void k_unpack(const float4* __restrict__ in, int n, float* x, float* y, float* z) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 q = in[i];
    if (x) x[i] = q.x;
    if (y) y[i] = q.y;
    if (z) z[i] = q.z;
}


// ------------------------------------------------------------ launches ---
#define BCS_GRID1(n, b) dim3((unsigned)(((n) + (b) - 1) / (b))), dim3(b)

using StepKernel = void (*)(const StepArgs);

template <int MODE, int S, bool P>
constexpr StepKernel step_kernel() {
    return k_step<MODE, kShapes[S].threads, kShapes[S].chunk, kShapes[S].min_blocks, P>;
}

template <int MODE, bool P>
StepKernel step_kernel_of(int shape) {
    switch (shape) {
        case 0: return step_kernel<MODE, 0, P>();
        case 1: return step_kernel<MODE, 1, P>();
        case 2: return step_kernel<MODE, 2, P>();
        case 3: return step_kernel<MODE, 3, P>();
        case 4: return step_kernel<MODE, 4, P>();
        default: return step_kernel<MODE, 5, P>();
    }
}

StepKernel step_kernel_for(int mode, int shape, bool persistent) {
    if (mode == kFull) return persistent ? step_kernel_of<kFull, true>(shape) : step_kernel_of<kFull, false>(shape);
    return persistent ? step_kernel_of<kForces, true>(shape) : step_kernel_of<kForces, false>(shape);
}

// CTAs of a persistent step launch: resident CTAs per SM x SMs.
int step_persistent_grid(int mode, int shape) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, step_kernel_for(mode, shape, true), kShapes[shape].threads, 0);
    return std::max(1, per) * std::max(1, sms);
}

void launch_step(const StepArgs& a, int items, int mode, int shape, int persistent_grid, cudaStream_t s,
                 cudaEvent_t after_collisions) {
    if (items <= 0) return;
    const bool persistent = persistent_grid > 0;
    const int blocks = persistent ? std::min(items, persistent_grid) : items;
    if (a.coll && a.pg.uniform && a.pg.row_start && a.pg.spos && a.pg.svel && a.n > 0) {
        const int blocks = (a.n + kCollideThreads - 1) / kCollideThreads;
        if (a.collide_search == 2) {
            static bool attr = false;
            if (!attr) {
                cudaFuncSetAttribute(k_collide_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmem);
                attr = true;
            }
            k_collide_tile<<<(a.n + kTileSlots - 1) / kTileSlots, kTileSlots, kTileSmem, s>>>(a);
        } else if (a.collide_search) {
            k_collide<1><<<blocks, kCollideThreads, 0, s>>>(a);
        } else {
            k_collide<0><<<blocks, kCollideThreads, 0, s>>>(a);
        }
    }
    if (after_collisions) cudaEventRecord(after_collisions, s);
    step_kernel_for(mode, shape, persistent)<<<blocks, kShapes[shape].threads, 0, s>>>(a);
    if (!a.pg.uniform || a.coll) return;   // no stencil, or no crowded particles set aside
    static int grid = 0;
    if (!grid) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = 4 * std::max(1, sms);
    }
    if (mode == 0) k_crowded<0><<<grid, kCrowdedThreads, 0, s>>>(a);
    else k_crowded<1><<<grid, kCrowdedThreads, 0, s>>>(a);
}
void launch_gather_rows(const float4* src, const int* idx, int n, float4* out, cudaStream_t s) {
    if (n > 0) k_gather_rows<<<BCS_GRID1(n, 256), 0, s>>>(src, idx, n, out);
}
void launch_propagate(const StepArgs& a, int blocks, cudaStream_t s) {
    if (blocks > 0) k_propagate<<<blocks, kPropagateThreads, 0, s>>>(a);
}
void launch_keys(const float4* pos, int n, int uniform, const SceneDev* scenes, int scene_count, int* keys, int* ids,
                 unsigned* err, cudaStream_t s) {
    if (n > 0) k_keys<<<BCS_GRID1(n, 256), 0, s>>>(pos, n, uniform, scenes, scene_count, keys, ids, err);
}
void launch_tri_keys(const float4* vpos, const uint32_t* tri, int T, const SceneDev* scenes, int scene_count,
                     int* keys, int* ids, cudaStream_t s) {
    if (T > 0) k_tri_keys<<<BCS_GRID1(T, 256), 0, s>>>(vpos, tri, T, scenes, scene_count, keys, ids);
}
void launch_cell_ranges(const int* keys, int n, int4* table, int* epoch, unsigned* occ, const int* ids,
                        const float4* pos, float4* spos, const float4* vel, float4* svel, cudaStream_t s) {
    k_next_epoch<<<1, 1, 0, s>>>(epoch);
    if (n > 0) k_cell_ranges<<<BCS_GRID1(n, 256), 0, s>>>(keys, n, table, epoch, occ, ids, pos, spos, vel, svel);
}
void launch_row_starts(const int* keys, int n, const SceneDev* scenes, int scene_count, long long rows, int* row_start,
                       int4* tiles, cudaStream_t s) {
    k_row_starts<<<(unsigned)((rows + 1 + 255) / 256), 256, 0, s>>>(keys, n, scenes, scene_count, rows, row_start);
    const int nt = (n + kTileSlots - 1) / kTileSlots;
    if (tiles && nt > 0) k_tile_setup<<<(nt + 127) / 128, 128, 0, s>>>(keys, n, scenes, scene_count, row_start, tiles);
}
int tile_records(int n) { return (n + kTileSlots - 1) / kTileSlots; }
void launch_occ_update(const int* keys, int n, unsigned* occ, bool set, cudaStream_t s) {
    if (n > 0) k_occ_update<<<BCS_GRID1(n, 256), 0, s>>>(keys, n, occ, set ? 1 : 0);
}
void launch_dense_ranges(const int4* table, const int* epoch, long long cells, int* starts, int* ends,
                         cudaStream_t s) {
    if (cells > 0) k_dense_ranges<<<BCS_GRID1(cells, 256), 0, s>>>(table, epoch, cells, starts, ends);
}
void launch_vein_end(const StepArgs& a, int cells, cudaStream_t s) {
    if (cells > 0) k_vein_end<<<BCS_GRID1((long long)cells * 32, 256), 0, s>>>(a, cells);
}
// Triangle bounds + wall mask.  With disp2 (dynamic wall) the build runs
// only when a vertex moved more than `margin` since the last one, and the
// bounds carry that margin.
void launch_tri_boxes(const int* keys, const int* ids, int T, const uint32_t* tri, const float4* vpos, float4* box,
                      const SceneDev* scenes, int scene_count, unsigned char* mask, float reach, int* mask_epoch,
                      float margin, float* disp2, float4* vref, int V, cudaStream_t s) {
    if (disp2) k_vein_disp<<<BCS_GRID1(V, 256), 0, s>>>(vpos, vref, V, disp2);
    if (mask) k_next_epoch_if<<<1, 1, 0, s>>>(mask_epoch, disp2, margin);
    if (T > 0) {
        // boxes per cell; the mask from the triangles themselves
        k_tri_boxes<<<BCS_GRID1(T, 256), 0, s>>>(keys, ids, T, tri, vpos, box, scenes, scene_count, nullptr, mask_epoch,
                                                 reach + margin, margin, disp2);
        if (mask)
            k_wall_mask_tris<<<BCS_GRID1(T, 128), 0, s>>>(tri, vpos, T, scenes, scene_count, mask, mask_epoch,
                                                           reach + margin, margin, disp2);
    }
    if (disp2) {
        k_vein_snapshot<<<BCS_GRID1(V, 256), 0, s>>>(vpos, vref, V, disp2, margin);
        k_disp_reset<<<1, 1, 0, s>>>(disp2, margin);
    }
}
void launch_tri_occupancy(const int4* table, const int* epoch, const SceneDev* scenes, int scene_count, long long cells,
                          unsigned* occ, cudaStream_t s) {
    if (cells > 0) k_tri_occupancy<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(table, epoch, scenes, scene_count, cells, occ);
}
void launch_vein_springs(const float4* vpos, const float4* vvel, float4* vfrc, const int* nb_ids, const float* nb_len,
                         int V, float k, float d, unsigned* err, cudaStream_t s) {
    if (V > 0) k_vein_springs<<<BCS_GRID1(V, 256), 0, s>>>(vpos, vvel, vfrc, nb_ids, nb_len, V, k, d, err);
}
void launch_vein_integrate(float4* vpos, float4* vvel, float4* vfrc, int V, float dt, cudaStream_t s) {
    if (V > 0) k_vein_integrate<<<BCS_GRID1(V, 256), 0, s>>>(vpos, vvel, vfrc, V, dt);
}
void launch_tri_cache(const int* ids, const uint32_t* tri, const float4* vpos, int T, float4* cache, cudaStream_t s) {
    if (T > 0) k_tri_cache<<<BCS_GRID1(T, 256), 0, s>>>(ids, tri, vpos, T, cache);
}
void launch_bump_step(long long* steps, int by, cudaStream_t s) { k_bump_step<<<1, 1, 0, s>>>(steps, by); }
void launch_sur_features(const StepArgs& a, const SurDev& d, cudaStream_t s) {
    if (d.cells > 0) k_sur_features<<<(d.cells * 32 + 255) / 256, 256, 0, s>>>(a, d);
}
void launch_sur_targets(const StepArgs& a, const SurDev& d, float* raw_t, unsigned char* valid, cudaStream_t s) {
    if (d.cells > 0) k_sur_targets<<<(d.cells * 32 + 255) / 256, 256, 0, s>>>(a, d, raw_t, valid);
}
void launch_sur_inputs(const float* raw, const float* raw_t, const int* list, int nvalid, unsigned long long seed,
                       int first, int cells, int pic, const int* adj_off, const int* adj_nbr, const float* adj_len,
                       const SurScales& sc, float* f, float* E, float* T, cudaStream_t s) {
    if (cells > 0)
        k_sur_inputs<<<cells, 128, 0, s>>>(raw, raw_t, list, nvalid, seed, first, cells, pic, adj_off, adj_nbr,
                                           adj_len, sc, f, E, T);
}
void launch_sur_apply(const StepArgs& a, const SurDev& d, const float* Y, const SurScales& sc, int first, int cells,
                      cudaStream_t s) {
    if (cells > 0) k_sur_apply<<<(cells * 32 + 255) / 256, 256, 0, s>>>(a, d, Y, sc, first, cells);
}
void launch_sur_eval(const float* Y, const float* raw_t, const unsigned char* valid, const SurScales& sc, int first,
                     int cells, int pic, double* sums, cudaStream_t s) {
    if (cells > 0) k_sur_eval<<<(cells * 32 + 255) / 256, 256, 0, s>>>(Y, raw_t, valid, sc, first, cells, pic, sums);
}
void launch_init_reference(const StepArgs& a, float4* pos, float4* vel, float4* frc, const float4* model,
                           const float* radius, unsigned long long seed, cudaStream_t s) {
    if (a.n > 0) k_init_reference<<<BCS_GRID1(a.n, 256), 0, s>>>(a, pos, vel, frc, model, radius, seed);
}
void launch_lattice_sites(const SceneDev* scenes, int scene, float3 lo, int nx, int ny, int nz, float spacing,
                          float clear, float ymin, float ymax, const bcs_flow_segment* flows, unsigned long long seed,
                          int* keys, int* ids, int* valid_count, cudaStream_t s) {
    const long long total = (long long)nx * ny * nz;
    if (total > 0)
        k_lattice_sites<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(scenes, scene, lo, nx, ny, nz, spacing, clear,
                                                                        ymin, ymax, flows, seed, keys, ids,
                                                                        valid_count);
}
void launch_lattice_place(const StepArgs& a, int scene, int count, float4* pos, float4* vel, float4* frc,
                          const float4* model, const float* centroid, const float* radius, const int* site_ids,
                          float3 lo, int nx, int ny, float spacing, float sigma, unsigned long long seed,
                          cudaStream_t s) {
    if (count > 0)
        k_lattice_place<<<BCS_GRID1(count, 256), 0, s>>>(a, scene, pos, vel, frc, model, centroid, radius, site_ids,
                                                          lo, nx, ny, spacing, sigma, seed);
}
// The fused inference kernel for a cell of `pic` particles: false when no
// instance holds it.
template <int MT>
bool launch_fused_mt(const StepArgs& a, const SurDev& d, const SurScales& sc, const float* P, const __nv_bfloat16* PB,
                     const __nv_bfloat16* PBT, const MpnnLayout& L, const int* goff, const int* gnbr,
                     const float* glen, int first, int cells, cudaStream_t s) {
    constexpr int bytes = fused_smem_bytes<MT>();
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_sur_fused<MT>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        attr = true;
    }
    k_sur_fused<MT><<<cells, MT * 64, bytes, s>>>(a, d, sc, P, PB, PBT, L, goff, gnbr, glen, first, cells);
    return true;
}
bool launch_sur_fused(const StepArgs& a, const SurDev& d, const SurScales& sc, const float* P,
                      const __nv_bfloat16* PB, const __nv_bfloat16* PBT, const MpnnLayout& L, const int* goff,
                      const int* gnbr, const float* glen, int first, int cells, cudaStream_t s) {
    if (cells <= 0) return true;
    const int mt = (d.pic + 15) / 16;
    if (mt <= 3) return launch_fused_mt<3>(a, d, sc, P, PB, PBT, L, goff, gnbr, glen, first, cells, s);
    if (mt <= 6) return launch_fused_mt<6>(a, d, sc, P, PB, PBT, L, goff, gnbr, glen, first, cells, s);
    if (mt <= 11) return launch_fused_mt<11>(a, d, sc, P, PB, PBT, L, goff, gnbr, glen, first, cells, s);
    if (mt <= 12) return launch_fused_mt<12>(a, d, sc, P, PB, PBT, L, goff, gnbr, glen, first, cells, s);
    return false;
}
void launch_substeps(const StepArgs& a, int items, int K, int chunk, cudaStream_t s) {
    if (items <= 0 || K <= 1) return;
    {
        static bool attr = false;
        const size_t b1 = 6 * (size_t)kSubstepThreads * sizeof(float4);
        if (!attr) {
            cudaFuncSetAttribute(k_substeps<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b1);
            cudaFuncSetAttribute(k_substeps<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(2 * b1));
            cudaFuncSetAttribute(k_substeps<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(3 * b1));
            attr = true;
        }
        const int per = (chunk + kSubstepThreads - 1) / kSubstepThreads;
        if (per <= 1) k_substeps<1><<<items, kSubstepThreads, b1, s>>>(a, K);
        else if (per == 2) k_substeps<2><<<items, kSubstepThreads, 2 * b1, s>>>(a, K);
        else k_substeps<3><<<items, kSubstepThreads, 3 * b1, s>>>(a, K);
    }
}
void launch_export(const float4* pos, int n, const float4* vpos, int V, float* pvbo, float* poff, float* vvbo,
                   cudaStream_t s) {
    int m = n > V ? n : V;
    if (m > 0) k_export<<<BCS_GRID1(m, 256), 0, s>>>(pos, n, vpos, V, pvbo, poff, vvbo);
}
void launch_pack(const float* x, const float* y, const float* z, int n, float4* out, const float* wsrc,
                 cudaStream_t s) {
    if (n > 0) k_pack<<<BCS_GRID1(n, 256), 0, s>>>(x, y, z, n, out, wsrc);
}
void launch_unpack(const float4* in, int n, float* x, float* y, float* z, cudaStream_t s) {
    if (n > 0) k_unpack<<<BCS_GRID1(n, 256), 0, s>>>(in, n, x, y, z);
}

}  // namespace bcs
