"""Seeded synthetic scenes: cell models, vein meshes, placements.

The reference ships one compile-time scene (src/config/blood_cell_presets.hpp,
src/config/vein_definition.hpp).  These generators build the runtime
equivalents the benchmarks and tests use:
  * icosphere shells (42 or 162 vertices, edge springs with their initial
    lengths as rest lengths) and a 162-vertex biconcave disc (Evans-Fung
    profile) with the same edge graph;
  * a straight cylinder and a Y bifurcation wall mesh whose triangle winding
    follows the reference's mesh (normals from cross(e2, e1) point into the
    lumen, src/simulation/vein_collisions.cu:28-30), flow along -Y as the
    reference's G and initVelocity (src/config/physics.hpp:24-34);
  * non-overlapping placement: lattice sites inside the lumen (hexagonal in
    x-z, layers along y), a seeded random subset per cell type.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from bcs import GRID_UNIFORM, Params, default_params


# ---------------------------------------------------------------- cells ----
def icosphere(subdiv: int):
    """Unit icosphere: (vertices [V,3] float64, faces [F,3])."""
    t = (1.0 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, float) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(subdiv):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]
        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, dtype=np.int64)


def edges_of(faces: np.ndarray) -> np.ndarray:
    e = set()
    for a, b, c in faces:
        for u, w in ((a, b), (b, c), (c, a)):
            e.add((min(u, w), max(u, w)))
    return np.array(sorted(e), dtype=np.int32)


@dataclasses.dataclass
class CellModel:
    name: str
    vertices: np.ndarray           # [pic, 3] float32
    springs: np.ndarray            # [S, 2] int32
    spring_lengths: np.ndarray     # [S] float32
    radius: float                  # bounding radius of the model


def _model(name, verts, faces):
    verts = verts.astype(np.float32)
    sp = edges_of(faces)
    d = verts[sp[:, 0]] - verts[sp[:, 1]]
    lengths = np.sqrt((d.astype(np.float32) ** 2).sum(1)).astype(np.float32)
    return CellModel(name, verts, sp, lengths, float(np.linalg.norm(verts, axis=1).max()))


def sphere_cell(radius: float = 3.0, subdiv: int = 1) -> CellModel:
    """Icosphere shell: subdiv 1 = 42 vertices / 120 springs, 2 = 162 / 480."""
    v, f = icosphere(subdiv)
    return _model(f"icosphere{len(v)}", v * radius, f)


def biconcave_cell(radius: float = 4.0, subdiv: int = 2) -> CellModel:
    """Red-cell disc: icosphere mapped onto the Evans-Fung biconcave profile
    h(r) = 0.5 R sqrt(1 - r^2) (0.207 + 2.003 r^2 - 1.123 r^4), axis along y."""
    v, f = icosphere(subdiv)
    rr = np.sqrt(v[:, 0] ** 2 + v[:, 2] ** 2).clip(0, 1)
    h = 0.5 * radius * np.sqrt(np.clip(1 - rr ** 2, 0, 1)) * (0.207 + 2.003 * rr ** 2 - 1.123 * rr ** 4)
    out = np.stack([v[:, 0] * radius, np.sign(v[:, 1]) * h, v[:, 2] * radius], 1)
    # keep the equator ring distinct where sign(y) == 0
    return _model(f"biconcave{len(v)}", out, f)


# ----------------------------------------------------------------- vein ----
def tube(origin, axis, radius, length, around, rings, angle_z=0.0):
    """Open cylinder wall.  Ring r, vertex j at origin + r*dl*axis +
    R(cos th u + sin th w); the trunk frame (u, axis, w) = (+x, -y, +z) is
    rotated by angle_z about z.  Triangles per quad follow the reference mesh
    order (a=(r+1)A+j, b=rA+j, c=rA+j+1), (a, c, d=(r+1)A+j+1)."""
    ca, sa = math.cos(angle_z), math.sin(angle_z)
    u = np.array([ca, sa, 0.0])
    ax = np.array([sa, -ca, 0.0]) if axis is None else np.asarray(axis, float)
    w = np.array([0.0, 0.0, 1.0])
    th = 2 * np.pi * np.arange(around) / around
    dl = length / (rings - 1)
    r = np.arange(rings)[:, None]
    pts = (np.asarray(origin, float)[None, None, :] + (r * dl)[:, :, None] * ax[None, None, :]
           + radius * (np.cos(th)[None, :, None] * u + np.sin(th)[None, :, None] * w))
    pts = pts.reshape(-1, 3)
    j = np.arange(around)
    j1 = (j + 1) % around
    tris = []
    for rr in range(rings - 1):
        a = (rr + 1) * around + j
        b = rr * around + j
        c = rr * around + j1
        d = (rr + 1) * around + j1
        # the two triangles of each quad in turn, like the reference mesh
        tris.append(np.stack([np.stack([a, b, c], 1), np.stack([a, c, d], 1)], 1).reshape(-1, 3))
    tris = np.concatenate(tris) if tris else np.zeros((0, 3), np.int64)
    return pts, tris, ax


@dataclasses.dataclass
class VeinMesh:
    positions: np.ndarray          # [V, 3] float32
    indices: np.ndarray            # [T, 3] uint32
    ending_centers: np.ndarray     # [E, 3]
    ending_radii: np.ndarray       # [E]
    segments: list                 # lumen segments: dict(origin, direction, length, radius)


def straight_vein(radius=30.0, length=300.0, around=64, rings=100) -> VeinMesh:
    pts, tris, ax = tube((0, 0, 0), (0, -1, 0), radius, length, around, rings)
    seg = dict(origin=(0.0, 0.0, 0.0), direction=(0.0, -1.0, 0.0), length=length, radius=radius)
    return VeinMesh(pts.astype(np.float32), tris.astype(np.uint32), np.array([[0.0, -length, 0.0]], np.float32),
                    np.array([0.7 * radius], np.float32), [seg])


def bifurcation_vein(trunk_radius=40.0, branch_radius=28.0, trunk_length=1500.0, branch_length=1500.0,
                     half_angle_deg=15.0, trunk_around=60, branch_around=44, ring_spacing=3.1) -> VeinMesh:
    """Y bifurcation: a trunk along -Y from the origin, two branches from the
    trunk's end at +-half_angle in the x-y plane.  Triangles of one tube that
    lie inside another tube are removed, which opens the junction."""
    tr = max(2, int(round(trunk_length / ring_spacing)) + 1)
    br = max(2, int(round(branch_length / ring_spacing)) + 1)
    parts = []
    segs = []
    p, t, ax = tube((0, 0, 0), (0, -1, 0), trunk_radius, trunk_length, trunk_around, tr)
    parts.append((p, t))
    segs.append(dict(origin=(0.0, 0.0, 0.0), direction=(0.0, -1.0, 0.0), length=trunk_length, radius=trunk_radius))
    J = np.array([0.0, -trunk_length, 0.0])
    ends, radii = [], []
    for sgn in (-1.0, 1.0):
        a = math.radians(half_angle_deg) * sgn
        p, t, ax = tube(J, None, branch_radius, branch_length, branch_around, br, angle_z=a)
        parts.append((p, t))
        segs.append(dict(origin=tuple(J), direction=tuple(float(x) for x in ax), length=branch_length,
                         radius=branch_radius))
        ends.append(J + branch_length * ax)
        radii.append(0.7 * branch_radius)

    def inside(seg, q, margin=0.0):
        o = np.asarray(seg["origin"]); d = np.asarray(seg["direction"])
        tt = (q - o) @ d
        rad = np.linalg.norm((q - o) - tt[:, None] * d[None, :], axis=1)
        return (tt > 0) & (tt < seg["length"]) & (rad < seg["radius"] - margin)

    pos_all, tri_all = [], []
    off = 0
    for k, (p, t) in enumerate(parts):
        cen = p[t].mean(1)
        keep = np.ones(len(t), bool)
        for m, seg in enumerate(segs):
            if m != k:
                keep &= ~inside(seg, cen, margin=0.5)
        pos_all.append(p)
        tri_all.append(t[keep] + off)
        off += len(p)
    return VeinMesh(np.concatenate(pos_all).astype(np.float32), np.concatenate(tri_all).astype(np.uint32),
                    np.array(ends, np.float32), np.array(radii, np.float32), segs)


# ------------------------------------------------------------ placement ----
def _inside_lumen(segs, c, clearance):
    ok = np.zeros(len(c), bool)
    for seg in segs:
        o = np.asarray(seg["origin"]); d = np.asarray(seg["direction"])
        tt = (c - o) @ d
        rad = np.linalg.norm((c - o) - tt[:, None] * d[None, :], axis=1)
        ok |= (tt > clearance) & (tt < seg["length"] - clearance) & (rad < seg["radius"] - clearance)
    return ok


def lattice_sites(segs, models, pattern, gap=0.2, particle_radius=0.5, y_top=-1.0):
    """Candidate centres per model: layers along -y in `pattern` order, each a
    hexagonal x-z lattice sized to the model's extent; a site is kept when the
    whole cell (bounding radius + particle radius + gap) is inside a lumen
    segment."""
    lo = np.min([np.asarray(s["origin"]) + np.minimum(0, np.asarray(s["direction"]) * s["length"]) - s["radius"]
                 for s in segs], 0)
    hi = np.max([np.asarray(s["origin"]) + np.maximum(0, np.asarray(s["direction"]) * s["length"]) + s["radius"]
                 for s in segs], 0)
    ext = [m.vertices.max(0) - m.vertices.min(0) + 2 * particle_radius + gap for m in models]
    sites = [[] for _ in models]
    y = y_top
    k = 0
    while True:
        mi = pattern[k % len(pattern)]
        m = models[mi]
        ex, ey, ez = ext[mi]
        yc = y - ey / 2
        if yc < lo[1]:
            break
        xs = np.arange(lo[0], hi[0] + ex, ex)
        zs = np.arange(lo[2], hi[2] + ez, ez * math.sqrt(3) / 2)
        X, Z = np.meshgrid(xs, zs, indexing="ij")
        X = X + (np.arange(len(zs))[None, :] % 2) * ex / 2
        c = np.stack([X.ravel(), np.full(X.size, yc), Z.ravel()], 1)
        clear = m.radius + particle_radius + gap
        sites[mi].append(c[_inside_lumen(segs, c, clear)])
        y -= ey
        k += 1
    return [np.concatenate(s) if s else np.zeros((0, 3)) for s in sites]


# ---------------------------------------------------------------- scene ----
@dataclasses.dataclass
class CellTypeSpec:
    count: int
    vertices: np.ndarray
    springs: np.ndarray
    spring_lengths: np.ndarray
    collision_radius: np.ndarray | None = None
    name: str = ""


@dataclasses.dataclass
class Scene:
    name: str
    types: list
    vein_positions: np.ndarray
    vein_indices: np.ndarray
    ending_centers: np.ndarray
    ending_radii: np.ndarray
    flow_segments: list
    params: Params
    positions: np.ndarray          # [N, 3] float32 initial particle positions
    velocities: np.ndarray         # [N, 3]

    @property
    def particle_count(self) -> int:
        return int(sum(t.count * len(t.vertices) for t in self.types))


def _instantiate(models, counts, centers_per_type, vel_sigma, rng):
    pos, vel = [], []
    for m, n, cen in zip(models, counts, centers_per_type):
        p = (cen[:, None, :] + m.vertices[None, :, :]).reshape(-1, 3)
        pos.append(p)
        vel.append(rng.normal(0.0, vel_sigma, size=p.shape) if vel_sigma > 0 else np.zeros_like(p))
    return np.concatenate(pos).astype(np.float32), np.concatenate(vel).astype(np.float32)


def _choose(sites, n, rng, what):
    if len(sites) < n:
        raise ValueError(f"vessel holds {len(sites)} {what} sites, {n} requested")
    idx = np.sort(rng.choice(len(sites), size=n, replace=False))
    ch = sites[idx]
    # cells numbered along the flow (descending y): neighbours in space stay
    # near each other in memory
    return ch[np.lexsort((ch[:, 2], ch[:, 0], -ch[:, 1]))]


def straight_scene(cells=256, radius=30.0, length=300.0, around=64, rings=100, seed=0, cell_size=1.0,
                   tri_cell=6.0, dt=1e-3, k=50.0, d=0.5, particle_radius=0.5, vein_dynamic=False,
                   use_blood_flow=True, model: CellModel | None = None, vel_sigma=0.0) -> Scene:
    """Plain method, small: straight cylinder R=30, L=300, 64 x 100 mesh,
    256 icosphere-42 cells (R=3, 120 springs, k=50, d=0.5), particle radius
    0.5, v=0, constant axial force G, grid cell 1.0, dt=1e-3."""
    rng = np.random.default_rng(seed)
    vein = straight_vein(radius, length, around, rings)
    m = model or sphere_cell(3.0, 1)
    sites = lattice_sites(vein.segments, [m], [0], particle_radius=particle_radius)[0]
    cen = _choose(sites, cells, rng, m.name)
    pos, vel = _instantiate([m], [cells], [cen], vel_sigma, rng)
    p = default_params()
    p.dt = dt
    p.particle_k_sniff = k
    p.particle_d_fact = d
    p.cell_width = p.cell_height = p.cell_depth = cell_size
    p.cell_width_triangles = p.cell_height_triangles = p.cell_depth_triangles = tri_cell
    p.cylinder_radius = radius
    p.vein_dynamic = int(vein_dynamic)
    p.use_blood_flow = int(use_blood_flow)
    p.seed = seed
    t = CellTypeSpec(cells, m.vertices, m.springs, m.spring_lengths,
                     np.full(len(m.vertices), particle_radius, np.float32), m.name)
    return Scene("straight", [t], vein.positions, vein.indices, vein.ending_centers, vein.ending_radii, [], p, pos,
                 vel)


def bifurcation_scene(cells_per_type=20588, seed=0, cell_size=1.0, tri_cell=6.0, dt=5e-4, k=50.0, d=0.5,
                      particle_radius=0.5, vel_sigma=0.01, peak_force=25.0, half_angle_deg=15.0,
                      trunk_length=None, branch_length=None, fill=0.85, trunk_radius=40.0, branch_radius=28.0,
                      trunk_around=60, branch_around=44) -> Scene:
    """Plain method, large: half 42-vertex spheres (R=3), half 162-vertex
    biconcave discs (R=4, 480 springs) in a Y bifurcation (trunk R=40,
    branches R=28), deformable spring wall, Gaussian velocities (sigma 0.01),
    Poiseuille axial force per segment, dt=5e-4.  The vessel length is grown
    until the lattice holds the cells at ~`fill` occupancy."""
    rng = np.random.default_rng(seed)
    models = [sphere_cell(3.0, 1), biconcave_cell(4.0, 2)]
    pattern = [0, 1, 1]
    need = [cells_per_type, cells_per_type]
    L = trunk_length or 200.0
    while True:
        Lb = branch_length or L
        vein = bifurcation_vein(trunk_radius, branch_radius, L, Lb, half_angle_deg, trunk_around, branch_around)
        sites = lattice_sites(vein.segments, models, pattern, particle_radius=particle_radius)
        if all(len(s) * fill >= n for s, n in zip(sites, need)) or trunk_length:
            break
        short = max(n / max(1, len(s) * fill) for s, n in zip(sites, need))
        L = L * min(4.0, max(1.05, short * 1.02))
    cen = [_choose(s, n, rng, m.name) for s, n, m in zip(sites, need, models)]
    pos, vel = _instantiate(models, need, cen, vel_sigma, rng)
    p = default_params()
    p.dt = dt
    p.particle_k_sniff = k
    p.particle_d_fact = d
    p.cell_width = p.cell_height = p.cell_depth = cell_size
    p.cell_width_triangles = p.cell_height_triangles = p.cell_depth_triangles = tri_cell
    p.cylinder_radius = trunk_radius
    p.vein_dynamic = 1
    p.seed = seed
    flows = [dict(origin=s["origin"], direction=s["direction"], length=s["length"], radius=s["radius"],
                  peak_force=peak_force) for s in vein.segments]
    types = [CellTypeSpec(n, m.vertices, m.springs, m.spring_lengths,
                          np.full(len(m.vertices), particle_radius, np.float32), m.name)
             for m, n in zip(models, need)]
    return Scene("bifurcation", types, vein.positions, vein.indices, vein.ending_centers, vein.ending_radii, flows, p,
                 pos, vel)


def tiny_scene(cells=4, seed=1, **kw) -> Scene:
    """A few cells in a short straight vein, sized for the oracle's loops."""
    kw.setdefault("radius", 12.0)
    kw.setdefault("length", 40.0)
    kw.setdefault("around", 24)
    kw.setdefault("rings", 14)
    return straight_scene(cells=cells, seed=seed, **kw)


def mixed_straight_scene(spheres, discs, length, seed=0, base_radius=30.0, cell_size=1.0, tri_cell=6.0, dt=1e-3,
                         k=50.0, d=0.5, particle_radius=0.5, fill=0.85, ring_spacing=3.0) -> Scene:
    """A straight vessel of the given length holding `spheres` 42-vertex and
    `discs` 162-vertex cells.  The radius starts at `base_radius` and grows
    until the lattice holds both populations at `fill` occupancy (a 50k-cell
    population does not fit a radius-30 vessel of length <= 600); the mesh
    keeps ~`ring_spacing` between rings and around the circumference."""
    rng = np.random.default_rng(seed)
    models = [sphere_cell(3.0, 1), biconcave_cell(4.0, 2)]
    need = [spheres, discs]
    R = base_radius
    while True:
        seg = dict(origin=(0.0, 0.0, 0.0), direction=(0.0, -1.0, 0.0), length=length, radius=R)
        sites = lattice_sites([seg], models, [0, 1], particle_radius=particle_radius)
        short = max((n / max(1.0, len(s) * fill) for s, n in zip(sites, need) if n), default=0.0)
        if short <= 1.0:
            break
        R *= min(2.0, max(1.03, math.sqrt(short) * 1.02))
    around = max(24, int(round(2 * math.pi * R / ring_spacing)))
    rings = max(2, int(round(length / ring_spacing)) + 1)
    vein = straight_vein(R, length, around, rings)
    cen = [_choose(s, n, rng, m.name) for s, n, m in zip(sites, need, models)]
    keep = [i for i in range(2) if need[i] > 0]
    pos, vel = _instantiate([models[i] for i in keep], [need[i] for i in keep], [cen[i] for i in keep], 0.0, rng)
    p = default_params()
    p.dt = dt
    p.particle_k_sniff = k
    p.particle_d_fact = d
    p.cell_width = p.cell_height = p.cell_depth = cell_size
    p.cell_width_triangles = p.cell_height_triangles = p.cell_depth_triangles = tri_cell
    p.cylinder_radius = R
    p.vein_dynamic = 0
    p.seed = seed
    types = [CellTypeSpec(need[i], models[i].vertices, models[i].springs, models[i].spring_lengths,
                          np.full(len(models[i].vertices), particle_radius, np.float32), models[i].name)
             for i in keep]
    return Scene("straight-mixed", types, vein.positions, vein.indices, vein.ending_centers, vein.ending_radii, [],
                 p, pos, vel)


def batched_scenes(count=64, seed=0, min_cells=500, max_cells=50000, min_length=150.0, max_length=600.0,
                   **kw) -> list:
    """Batched plain method: `count` independent straight vessels, cell counts
    log-uniform in [min_cells, max_cells], lengths uniform in
    [min_length, max_length], each cell a sphere or a biconcave disc with
    probability 1/2; dt=1e-3 and the constants of the small straight scene."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        n = int(round(math.exp(rng.uniform(math.log(min_cells), math.log(max_cells)))))
        L = float(rng.uniform(min_length, max_length))
        spheres = int(rng.binomial(n, 0.5))
        out.append(mixed_straight_scene(spheres, n - spheres, L, seed=seed * 1000 + s, **kw))
    return out


def scale_scene(cells=1_000_000, seed=0, cell_size=1.0, widen=6.0, **kw) -> Scene:
    """Surrogate at scale: `cells` cells, half 42-vertex spheres and half
    162-vertex biconcave discs (1M cells = 102M particles), in the Y
    bifurcation of `bifurcation_scene` with radii (40, 28) and the mesh
    resolution around them widened by `widen`.  At 1M cells and widen 6 the
    segments settle at ~1270 long and the grid box at cell 1.0 holds 1.56e9
    cells, inside the 31-bit key space; the large workload's proportions
    (widen 1, ~25x the length) would need ~5e11."""
    return bifurcation_scene(cells_per_type=cells // 2, seed=seed, cell_size=cell_size,
                             trunk_radius=40.0 * widen, branch_radius=28.0 * widen,
                             trunk_around=int(round(60 * widen)), branch_around=int(round(44 * widen)), **kw)


def subset_scene(scene: Scene, cells: int, seed=0, positions=None, velocities=None) -> Scene:
    """A seeded subset of `cells` cells of `scene` (drawn across types in
    proportion to their counts) in the same vessel with the same constants;
    `positions`/`velocities` (the full scene's state, default its initial
    one) give the subset's particles."""
    rng = np.random.default_rng(seed)
    pos = scene.positions if positions is None else positions
    vel = scene.velocities if velocities is None else velocities
    total = sum(t.count for t in scene.types)
    cells = min(cells, total)
    pick = np.sort(rng.choice(total, size=cells, replace=False))
    types, P, V = [], [], []
    cell0, part0 = 0, 0
    for t in scene.types:
        pic = len(t.vertices)
        mine = pick[(pick >= cell0) & (pick < cell0 + t.count)] - cell0
        rows = (part0 + mine[:, None] * pic + np.arange(pic)[None, :]).ravel()
        P.append(pos[rows])
        V.append(vel[rows])
        types.append(dataclasses.replace(t, count=int(len(mine))))
        cell0 += t.count
        part0 += t.count * pic
    return dataclasses.replace(scene, name=scene.name + f"-subset{cells}", types=types,
                               positions=np.concatenate(P).astype(np.float32),
                               velocities=np.concatenate(V).astype(np.float32))
