"""GPU parity: libbcs.so (through the C ABI) against the FP64 oracle.

Tolerances (the parity contract of this path):
  * grid keys, sorted particle order, cell ranges: bit-exact;
  * one step: |gpu - oracle| <= 1e-5 * (|oracle| + rms(oracle)) elementwise
    for positions, velocities and forces (FP32 against FP64);
  * 100 steps: max position error below 1e-3 of the particle radius.
"""
import numpy as np
import pytest

import bcs
import bcs_scenes as S
import oracle as O

pytestmark = pytest.mark.gpu

RTOL_1STEP = 1e-5


def rel_err(g, o):
    o = np.asarray(o, np.float64)
    scale = np.abs(o) + np.sqrt(np.mean(o * o)) + 1e-30
    return float(np.max(np.abs(np.asarray(g, np.float64) - o) / scale))


def make(scene):
    sim = bcs.Simulation(scene)
    sim.set_particles(scene.positions, scene.velocities)
    return sim


@pytest.fixture(scope="module")
def small():
    return S.straight_scene(cells=256, seed=7)


@pytest.fixture(scope="module")
def tiny():
    return S.tiny_scene(cells=6, seed=3)


# ------------------------------------------------------------------ grids --
def test_particle_grid_bit_exact(lib, small):
    sim = make(small)
    sim.calculate_grids()
    k, i, st, en = sim.get_grid(0)
    o = O.OracleSim(small)
    o.calculate_grids()
    ok, oi, ost, oen = o.get_grid(0)
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(st, ost)
    np.testing.assert_array_equal(en, oen)


def test_particle_grid_bit_exact_random_points(lib, small):
    rng = np.random.default_rng(11)
    sim = make(small)
    info = sim.info
    lo = np.array([info.min_x, info.min_y, info.min_z], np.float32)
    hi = np.array([info.max_x, info.max_y, info.max_z], np.float32)
    n = sim.n
    pts = (lo + (hi - lo) * rng.random((n, 3))).astype(np.float32)
    # cell faces, exact bounds, a few points outside the box, many duplicates
    pts[:64] = np.floor(pts[:64])
    pts[64] = lo
    pts[65] = hi
    pts[66:70] = hi + 3.0
    pts[70:74] = lo - 3.0
    pts[100:2000] = pts[2000:3900]
    sim.set_particles(pts, np.zeros_like(pts))
    sim.calculate_grids()
    k, i, st, en = sim.get_grid(0)
    o = O.OracleSim(small)
    ok, oi, ost, oen, err = o.grid_of_points(pts, dense=True)
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(st, ost)
    np.testing.assert_array_equal(en, oen)
    assert sim.error_word() & bcs.ERRW_OUT_OF_GRID
    assert err & bcs.ERRW_OUT_OF_GRID


def test_triangle_grid_bit_exact(lib, small):
    sim = make(small)
    k, i, st, en = sim.get_grid(1)
    o = O.OracleSim(small)
    ok, oi, ost, oen = o.get_grid(1)
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(st, ost)
    np.testing.assert_array_equal(en, oen)


def test_grid_after_steps_matches_oracle_keys_of_gpu_positions(lib, small):
    # After stepping, the grid the GPU built must equal the oracle's grid of
    # the GPU's own FP32 positions (the grid is a pure function of them).
    sim = make(small)
    sim.step(5)
    pos, _, _ = sim.get_particles()
    sim.calculate_grids()
    k, i, _, _ = sim.get_grid(0, dense=False)
    o = O.OracleSim(small)
    ok, oi, _, _, _ = o.grid_of_points(pos)
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(i, oi)


# ------------------------------------------------------------------- step --
@pytest.mark.parametrize("which", ["tiny", "small"])
def test_one_step_relative_1e5(lib, which, tiny, small):
    sc = tiny if which == "tiny" else small
    sim = make(sc)
    sim.step(1)
    g = sim.get_particles()
    o = O.OracleSim(sc)
    o.step(1)
    r = o.get_particles()
    for name, a, b in zip(("position", "velocity", "force"), g, r):
        e = rel_err(a, b)
        assert e <= RTOL_1STEP, f"{name}: relative error {e:.3e}"


def test_one_step_moving_cells_with_vein_hits(lib):
    # Reference initial speed (initVelocity, physics.hpp:24-26) so that rays
    # hit the wall within veinImpactDistance and reflections fire.
    sc = S.straight_scene(cells=64, seed=5, radius=14.0, length=120.0, around=40, rings=50)
    sc.velocities[:] = np.random.default_rng(2).normal(0, 20.0, sc.velocities.shape).astype(np.float32)
    sim = make(sc)
    sim.step(1)
    g = sim.get_particles()
    o = O.OracleSim(sc)
    o.step(1)
    r = o.get_particles()
    for name, a, b in zip(("position", "velocity", "force"), g, r):
        e = rel_err(a, b)
        assert e <= RTOL_1STEP, f"{name}: relative error {e:.3e}"


def test_split_phases_match_fused(lib, small):
    a, b = make(small), make(small)
    for _ in range(3):
        a.calculate_grids()
        a.calculate_next_frame()
        a.propagate_all()
    b.step(3)
    for x, y in zip(a.get_particles(), b.get_particles()):
        np.testing.assert_allclose(x, y, rtol=1e-6, atol=1e-6)


def test_next_frame_phase_matches_oracle(lib, small):
    sim = make(small)
    sim.calculate_grids()
    sim.calculate_next_frame()
    g = sim.get_particles()
    o = O.OracleSim(small)
    o.calculate_grids()
    o.calculate_next_frame()
    r = o.get_particles()
    for name, a, b in zip(("position", "velocity", "force"), g, r):
        assert rel_err(a, b) <= RTOL_1STEP, name


def test_hundred_steps_within_1e3_radius(lib, small):
    sim = make(small)
    sim.step(100)
    pos, _, _ = sim.get_particles()
    o = O.OracleSim(small)
    o.step(100)
    opos, _, _ = o.get_particles()
    err = np.abs(pos - opos).max()
    assert err < 1e-3 * 0.5, f"max position error {err:.3e}"


def test_deformable_vein_parity(lib):
    sc = S.straight_scene(cells=24, seed=9, radius=12.0, length=60.0, around=24, rings=20, vein_dynamic=True)
    sc.velocities[:] = np.random.default_rng(4).normal(0, 15.0, sc.velocities.shape).astype(np.float32)
    sim = make(sc)
    o = O.OracleSim(sc)
    sim.step(1)
    o.step(1)
    gv = sim.get_vein()
    ov = o.get_vein()
    assert rel_err(gv[0], ov[0]) <= RTOL_1STEP
    assert rel_err(gv[1], ov[1]) <= 1e-4 * max(1.0, np.abs(ov[1]).max())
    sim.step(9)
    o.step(9)
    gp, _, _ = sim.get_particles()
    op, _, _ = o.get_particles()
    assert np.abs(gp - op).max() < 1e-3 * 0.5
    assert np.abs(sim.get_vein()[0] - o.get_vein()[0]).max() < 1e-4


def test_respawn_parity(lib):
    # Cells start just above the outlet sphere, so the vein-end rule fires.
    sc = S.straight_scene(cells=8, seed=2, radius=12.0, length=60.0, around=24, rings=20)
    sc.positions[:, 1] -= sc.positions[:, 1].max() + 44.0   # top of the stack at y = -44
    sc.velocities[:] = np.array([0, -80.0, 0], np.float32)
    sim = make(sc)
    o = O.OracleSim(sc)
    for _ in range(4):
        sim.step(1)
        o.step(1)
        gp, gv, _ = sim.get_particles()
        op, ov, _ = o.get_particles()
        assert np.abs(gp - op).max() < 1e-3
        assert np.abs(gv - ov).max() < 1e-3
    # at least one cell was recycled to the inflow
    assert (gp[:, 1] > -30).any()


@pytest.mark.parametrize("grid", ["particles_none", "both_none"])
def test_none_grids(lib, tiny, grid):
    sc = S.tiny_scene(cells=6, seed=3)
    sc.params.particle_grid = bcs.GRID_NONE
    if grid == "both_none":
        sc.params.triangle_grid = bcs.GRID_NONE
    sim = make(sc)
    sim.step(1)
    g = sim.get_particles()
    o = O.OracleSim(sc)
    o.step(1)
    r = o.get_particles()
    for a, b in zip(g, r):
        assert rel_err(a, b) <= RTOL_1STEP
    # and the same physics as the uniform grid
    u = make(tiny)
    u.step(1)
    for a, b in zip(g, u.get_particles()):
        np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-5)


def test_deterministic(lib, small):
    a, b = make(small), make(small)
    a.step(20)
    b.step(20)
    for x, y in zip(a.get_particles(), b.get_particles()):
        np.testing.assert_array_equal(x, y)


def test_error_word_and_render_export(lib, tiny):
    sim = make(tiny)
    sim.step(1)
    assert sim.error_word(clear=True) & bcs.ERRW_NAN_NORMALIZE   # v = 0 at start
    assert sim.error_word() == 0
    pv, po, vv = sim.export_render()
    pos, _, _ = sim.get_particles()
    np.testing.assert_array_equal(pv[:, :3], pos)
    np.testing.assert_array_equal(pv[:, 3:], 0)
    np.testing.assert_array_equal(po, pos)
    np.testing.assert_array_equal(vv[:, :3], sim.get_vein()[0])


def test_incremental_grid_every_frame(lib):
    # Fused frames rebuild the grid from the previous frame's order; each
    # frame's grid must equal the oracle's grid of that frame's start positions
    # (respawns included: cells start near the outlet and move fast).
    sc = S.straight_scene(cells=48, seed=13, radius=14.0, length=90.0, around=32, rings=40)
    sc.velocities[:] = np.random.default_rng(8).normal(0, 30.0, sc.velocities.shape).astype(np.float32)
    sc.velocities[:, 1] -= 60.0
    sim = make(sc)
    o = O.OracleSim(sc)
    for _ in range(12):
        pos, _, _ = sim.get_particles()
        sim.step(1)
        k, i, _, _ = sim.get_grid(0, dense=False)
        ok, oi, _, _, _ = o.grid_of_points(pos)
        np.testing.assert_array_equal(k, ok)
        np.testing.assert_array_equal(i, oi)


def test_incremental_grid_after_reshuffle(lib, small):
    # Every particle changes cell: the incremental path sorts all of them.
    sim = make(small)
    sim.step(3)
    rng = np.random.default_rng(3)
    pos = small.positions[rng.permutation(len(small.positions))]
    sim.set_particles(pos, np.zeros_like(pos))
    sim.calculate_grids()
    k, i, st, en = sim.get_grid(0)
    ok, oi, ost, oen, _ = O.OracleSim(small).grid_of_points(pos, dense=True)
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(st, ost)
    np.testing.assert_array_equal(en, oen)


@pytest.mark.parametrize("moved", [4000, 4096, 4200])
def test_incremental_grid_mover_counts(lib, small, moved):
    # Around one sort tile of movers (4 096): up to it the movers are sorted
    # by one CTA, above it by the tiled passes; both must give the oracle's
    # grid.
    sim = make(small)
    sim.step(2)
    pos0, _, _ = sim.get_particles()
    rng = np.random.default_rng(moved)
    pick = rng.choice(len(pos0), size=moved, replace=False)
    pos = pos0.copy()
    pos[pick] = pos0[np.roll(pick, 1)]   # a cycle: each picked particle takes another's place
    sim.set_particles(pos, np.zeros_like(pos))
    sim.calculate_grids()
    k, i, _, _ = sim.get_grid(0, dense=False)
    ok, oi, _, _, _ = O.OracleSim(small).grid_of_points(pos)
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(i, oi)


@pytest.mark.parametrize("moved", [3000, 6000])
def test_captured_frame_mover_counts(lib, small, moved):
    # The same inside a replayed frame graph, on both sides of one tile of
    # movers (the one-CTA sort, the tiled passes).
    sim = make(small)
    sim.step(4)   # both buffer parities captured
    pos0, _, _ = sim.get_particles()
    rng = np.random.default_rng(moved + 1)
    pick = rng.choice(len(pos0), size=moved, replace=False)
    pos = pos0.copy()
    pos[pick] = pos0[np.roll(pick, 1)]
    sim.set_particles(pos, np.zeros_like(pos))
    sim.step(1)   # keys of the uploaded state, then the captured frame
    k, i, _, _ = sim.get_grid(0, dense=False)
    ok, oi, _, _, _ = O.OracleSim(small).grid_of_points(pos)
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(i, oi)


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("moved", [3000, 9000])
def test_mover_sort_modes(lib, small, mode, moved):
    # The movers of a replayed frame sorted by the tiled radix passes (mode
    # 1) or by one CTA alone (mode 2, which also takes more than one tile of
    # movers), or every pair sorted from scratch (mode 3): the oracle's grid
    # each way.
    sim = make(small)
    sim.set_mover_sort(mode)
    sim.step(4)
    pos0, _, _ = sim.get_particles()
    rng = np.random.default_rng(moved + 7)
    pick = rng.choice(len(pos0), size=moved, replace=False)
    pos = pos0.copy()
    pos[pick] = pos0[np.roll(pick, 1)]
    sim.set_particles(pos, np.zeros_like(pos))
    sim.step(1)
    k, i, _, _ = sim.get_grid(0, dense=False)
    ok, oi, _, _, _ = O.OracleSim(small).grid_of_points(pos)
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(i, oi)


def test_mover_sort_modes_agree_over_frames(lib):
    # A fast flow, most particles moving every frame: the frames and grids
    # are the same bit for bit whichever way the grid is sorted.  The
    # automatic mode (0) switches to the sort from scratch after the first
    # frames and keeps every 16th frame incremental, so 40 frames cover
    # both.
    sc = S.straight_scene(cells=256, seed=11)
    sc.velocities[:] = np.random.default_rng(5).normal(0, 400.0, sc.velocities.shape).astype(np.float32)
    out = []
    for mode in (0, 1, 2, 3):
        sim = make(sc)
        sim.set_mover_sort(mode)
        sim.step(40)
        out.append(tuple(sim.get_particles()) + tuple(sim.get_grid(0, dense=False)[:2]))
        sim.close()
    for other in out[1:]:
        for a, b in zip(out[0], other):
            np.testing.assert_array_equal(a, b)
    sim = make(sc)
    with pytest.raises(bcs.BcsError):
        sim.set_mover_sort(4)


def test_moving_wall_rebuilds_bounds(lib):
    # Vein vertices start with a velocity that carries them past the 0.5
    # rebuild margin of the triangle bounds / wall mask within the run; the
    # frames must keep matching the oracle across rebuilds.
    sc = S.straight_scene(cells=20, seed=17, radius=12.0, length=60.0, around=24, rings=20, vein_dynamic=True)
    sc.velocities[:] = np.random.default_rng(6).normal(0, 15.0, sc.velocities.shape).astype(np.float32)
    vvel = np.random.default_rng(7).normal(0, 40.0, sc.vein_positions.shape).astype(np.float32)
    sim = make(sc)
    sim.set_vein(vel=vvel)
    o = O.OracleSim(sc)
    o.set_vein(vel=vvel)
    for _ in range(3):
        sim.step(8)
        o.step(8)
        gp, _, _ = sim.get_particles()
        op, _, _ = o.get_particles()
        assert np.abs(gp - op).max() < 1e-3 * 0.5
        assert np.abs(sim.get_vein()[0] - o.get_vein()[0]).max() < 1e-4
    # the wall has moved well past the margin by now
    assert np.abs(sim.get_vein()[0] - sc.vein_positions).max() > 0.5
