"""Crowded particles.  Two collision paths take them:

  * grid order (tuning grid_collisions = 1, 2, 3): every sorted slot gets a
    thread; the particles of a crowded cell sit in neighbouring lanes and
    share their whole stencil, so each lane sums its candidates in stencil
    order with warp-uniform loops (3 stages a block's candidates in shared
    memory and falls back to the global search when a crowded block's rows
    exceed its capacity);
  * cell order (grid_collisions = 0): a particle whose collision stencil
    holds more than 128 sorted slots is left by the step kernel to
    k_crowded: inside the grid box a warp takes its whole grid cell (the
    stencil's slots staged in shared memory, the lanes of each particle
    splitting them), outside it a warp takes the particle alone (lanes split
    the slots); fixed butterflies add the partial sums.

Scenes with cells piled onto a few points put many particles on both paths:
the result must match the FP64 oracle like any other step on either path,
and stay bit-identical across every launch shape and grid option of a path.

Tolerances as the plain parity tests: one step 1e-5 relative (FP32 against
FP64, elementwise against |oracle| + rms(oracle)); after a few steps 1e-3 of
the particle radius.
"""
import numpy as np
import pytest

import bcs
import bcs_scenes as S
import oracle as O

pytestmark = pytest.mark.gpu

CROWDED = 128


def rel_err(g, o):
    o = np.asarray(o, np.float64)
    scale = np.abs(o) + np.sqrt(np.mean(o * o)) + 1e-30
    return float(np.max(np.abs(np.asarray(g, np.float64) - o) / scale))


def crowded_scene(seed=4, spread=0.7, vel=2.0, anchors=None, cells=60, length=90.0, **kw):
    """Icosphere cells of a straight vessel piled onto the given points (by
    default all 60 onto one), each cell a little off its point."""
    sc = S.straight_scene(cells=cells, seed=seed, radius=14.0, length=length, around=32, rings=int(length / 2.25),
                          **kw)
    rng = np.random.default_rng(seed)
    pic = len(sc.types[0].vertices)
    if anchors is None:
        anchors = [[0.0, -45.0, 0.0]]
    anchors = np.array(anchors, np.float32)
    P = sc.positions.reshape(-1, pic, 3)
    off = anchors[np.arange(len(P)) % len(anchors)][:, None, :] + rng.normal(0, spread, (len(P), 1, 3)).astype(np.float32)
    sc.positions[:] = (P - P.mean(1, keepdims=True) + off).reshape(-1, 3)
    sc.velocities[:] = rng.normal(0, vel, sc.velocities.shape).astype(np.float32)
    return sc


def stencil_slots(sc, pos):
    """Host count of the slots in each particle's 27-cell stencil (grid cell
    1.0 over the vein's box and margins)."""
    p = sc.params
    m = np.array([p.grid_xz_margin, p.grid_y_margin, p.grid_xz_margin])
    lo = sc.vein_positions.min(0) - m
    q = np.floor((pos - lo) / 1.0).astype(np.int64)
    dims = q.max(0) + 3
    key = (q[:, 2] * dims[1] + q[:, 1]) * dims[0] + q[:, 0]
    uk, cnt = np.unique(key, return_counts=True)
    n = np.zeros(len(pos), np.int64)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                k2 = key + (dz * dims[1] + dy) * dims[0] + dx
                ix = np.minimum(np.searchsorted(uk, k2), len(uk) - 1)
                n += np.where(uk[ix] == k2, cnt[ix], 0)
    return n


def make(sc, **tuning):
    sim = bcs.Simulation(sc)
    sim.set_particles(sc.positions, sc.velocities)
    if tuning:
        sim.set_tuning(**tuning)
    return sim


def test_scene_is_crowded():
    sc = crowded_scene()
    n = stencil_slots(sc, sc.positions)
    assert (n > CROWDED).sum() > 1000 and (n <= CROWDED).sum() > 100


def test_crowded_count(lib):
    """bcs_get_crowded counts the particles the cell-order path sets aside,
    once per step; the grid-order path sets none aside."""
    sc = crowded_scene()
    g = make(sc)
    g.step(2)
    assert g.crowded_particles() == 0
    sim = make(sc, grid_collisions=0)
    assert sim.crowded_particles() == 0
    sim.step(1)
    host = int((stencil_slots(sc, sc.positions) > CROWDED).sum())
    got = sim.crowded_particles()
    assert abs(got - host) <= 0.01 * host, (got, host)
    sim.step(2)
    assert sim.crowded_particles() > 2 * got


@pytest.mark.parametrize("gc", [3, 2, 1, 0])
def test_one_step_matches_oracle(lib, gc):
    sc = crowded_scene()
    sim = make(sc, grid_collisions=gc)
    sim.step(1)
    o = O.OracleSim(sc)
    o.step(1)
    for name, a, b in zip(("position", "velocity", "force"), sim.get_particles(), o.get_particles()):
        e = rel_err(a, b)
        assert e <= 1e-5, f"{name}: relative error {e:.3e}"


@pytest.mark.parametrize("gc", [3, 2, 1, 0])
def test_few_steps_within_1e3_radius(lib, gc):
    sc = crowded_scene(vel=0.5)
    sim = make(sc, grid_collisions=gc)
    sim.step(4)
    o = O.OracleSim(sc)
    o.step(4)
    gp, op = sim.get_particles()[0], o.get_particles()[0]
    assert np.abs(gp - op).max() < 1e-3 * 0.5
    assert (stencil_slots(sc, gp) > CROWDED).sum() > 1000


FLAGS = ("persistent", "spatial_order", "full_sort", "occupancy_filter", "sorted_positions")


@pytest.mark.parametrize("gc", [3, 2, 1, 0])
@pytest.mark.parametrize("shape", range(len(bcs.STEP_SHAPES)))
@pytest.mark.parametrize("flags", [0, 1])
def test_every_shape_same_state(lib, shape, flags, gc):
    sc = crowded_scene()
    want = make(sc, grid_collisions=gc)
    want.step(5)
    want = want.get_particles()
    sim = make(sc, step_shape=shape, grid_collisions=gc, **{f: flags for f in FLAGS})
    sim.step(5)
    for a, b in zip(sim.get_particles(), want):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("gc", [3, 2, 1, 0])
def test_split_phases_match_fused(lib, gc):
    sc = crowded_scene()
    a, b = make(sc, grid_collisions=gc), make(sc, occupancy_filter=1, sorted_positions=1, grid_collisions=gc)
    for _ in range(3):
        a.calculate_grids()
        a.calculate_next_frame()
        a.propagate_all()
    b.step(3)
    for x, y in zip(a.get_particles(), b.get_particles()):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("gc", [3, 2, 1, 0])
def test_macro_steps_match_oracle(lib, gc):
    sc = crowded_scene(vel=0.5)
    sim = make(sc, grid_collisions=gc)
    o = O.OracleSim(sc)
    sim.macro_step(4, 1)
    o.macro_step(4, 1)
    g, r = sim.get_particles(), o.get_particles()
    assert rel_err(g[0], r[0]) <= 4e-5
    assert rel_err(g[1], r[1]) <= 4e-4


@pytest.mark.parametrize("gc", [3, 2, 1, 0])
def test_crowded_outside_the_grid_box(lib, gc):
    """A pile beyond the grid box's top face: clamped keys, so those
    particles' stencils are not their cell's regular one (on the cell-order
    path the per-particle warp path); the other two piles are inside."""
    sc = crowded_scene(anchors=[[0.0, 47.0, 0.0], [3.0, -45.0, -2.0]], cells=120, length=150.0, use_blood_flow=False)
    inside = sc.positions[:, 1] < 0
    assert (stencil_slots(sc, sc.positions)[inside] > CROWDED).sum() > 1000
    top = sc.positions[:, 1].max()
    assert top > sc.vein_positions[:, 1].max() + sc.params.grid_y_margin
    sim = make(sc, grid_collisions=gc)
    sim.step(1)
    o = O.OracleSim(sc)
    o.step(1)
    for name, a, b in zip(("position", "velocity", "force"), sim.get_particles(), o.get_particles()):
        e = rel_err(a, b)
        assert e <= 1e-5, f"{name}: relative error {e:.3e}"
    want = sim.get_particles()
    for shape in range(len(bcs.STEP_SHAPES)):
        other = make(sc, step_shape=shape, grid_collisions=gc, **{f: shape % 2 for f in FLAGS})
        other.step(1)
        for a, b in zip(other.get_particles(), want):
            np.testing.assert_array_equal(a, b)



@pytest.mark.parametrize("gc", [3, 2, 1, 0])
def test_batched_crowded_scenes_match_standalone(lib, gc):
    """Crowded cells of several scenes in one batch (batch-wide keys and
    rows): every scene's state equals its standalone run bit for bit."""
    scenes = [crowded_scene(seed=s, anchors=[[0.0, -40.0 - 5.0 * (s - 7), 0.0]]) for s in (7, 8)]
    sim = bcs.Simulation(scenes)
    sim.set_tuning(step_shape=3, grid_collisions=gc)
    sim.set_particles(np.concatenate([s.positions for s in scenes]), np.concatenate([s.velocities for s in scenes]))
    sim.step(3)
    got = sim.get_particles()
    assert (sim.crowded_particles() > 0) == (gc == 0)
    for k, sc in enumerate(scenes):
        z = sim.scene_info(k)
        rows = slice(z.particle_start, z.particle_start + z.particle_count)
        alone = make(sc, grid_collisions=gc)
        alone.step(3)
        for a, b in zip(got, alone.get_particles()):
            np.testing.assert_array_equal(a[rows], b)
