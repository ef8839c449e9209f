"""Multi-rate macro steps (bcs_macro_step) against the oracle's restatement
of the same scheme, and their exact relation to the plain frame.

Tolerances: one macro step of K sub-steps is K FP32 integrations against
FP64, so the one-step bound of the plain parity tests (1e-5 relative) is
loosened by K; positions after several macro steps are held to the plain
100-step bound (1e-3 of the particle radius).
"""
import numpy as np
import pytest

import bcs
import bcs_scenes as S
import oracle as O

pytestmark = pytest.mark.gpu


def rel_err(g, o):
    o = np.asarray(o, np.float64)
    scale = np.abs(o) + np.sqrt(np.mean(o * o)) + 1e-30
    return float(np.max(np.abs(np.asarray(g, np.float64) - o) / scale))


def make(scene):
    sim = bcs.Simulation(scene)
    sim.set_particles(scene.positions, scene.velocities)
    return sim


def moving_scene(vein_dynamic=False, seed=21):
    sc = S.straight_scene(cells=24, seed=seed, radius=12.0, length=60.0, around=24, rings=20,
                          vein_dynamic=vein_dynamic)
    sc.velocities[:] = np.random.default_rng(seed).normal(0, 15.0, sc.velocities.shape).astype(np.float32)
    return sc


def test_one_substep_is_the_frame(lib):
    sc = moving_scene(vein_dynamic=True)
    a, b = make(sc), make(sc)
    a.step(5)
    b.macro_step(1, 5)
    for x, y in zip(a.get_particles(), b.get_particles()):
        np.testing.assert_array_equal(x, y)
    assert b.refresh_info().steps_done == 5


@pytest.mark.parametrize("K", [2, 8])
@pytest.mark.parametrize("dynamic", [False, True])
def test_macro_step_matches_oracle(lib, K, dynamic):
    sc = moving_scene(vein_dynamic=dynamic)
    sim = make(sc)
    o = O.OracleSim(sc)
    sim.macro_step(K, 1)
    o.macro_step(K, 1)
    g, r = sim.get_particles(), o.get_particles()
    assert rel_err(g[0], r[0]) <= 1e-5 * K
    assert rel_err(g[1], r[1]) <= 1e-4 * K
    sim.macro_step(K, 3)
    o.macro_step(K, 3)
    gp, op = sim.get_particles()[0], o.get_particles()[0]
    assert np.abs(gp - op).max() < 1e-3 * 0.5
    assert sim.refresh_info().steps_done == 4 * K == o.steps_done()
    if dynamic:
        assert np.abs(sim.get_vein()[0] - o.get_vein()[0]).max() < 1e-4


def test_macro_step_respawns_like_the_oracle(lib):
    sc = S.straight_scene(cells=8, seed=2, radius=12.0, length=60.0, around=24, rings=20)
    sc.positions[:, 1] -= sc.positions[:, 1].max() + 44.0
    sc.velocities[:] = np.array([0, -80.0, 0], np.float32)
    sim = make(sc)
    o = O.OracleSim(sc)
    for _ in range(3):
        sim.macro_step(4, 1)
        o.macro_step(4, 1)
        gp, gv, _ = sim.get_particles()
        op, ov, _ = o.get_particles()
        assert np.abs(gp - op).max() < 1e-3
        assert np.abs(gv - ov).max() < 1e-3
    assert (gp[:, 1] > -30).any()


def test_macro_step_every_tuning_same_state(lib):
    sc = moving_scene()
    want = make(sc)
    want.macro_step(8, 3)
    want = want.get_particles()
    for t in (dict(step_shape=0), dict(step_shape=2, persistent=1, spatial_order=1),
              dict(step_shape=5, occupancy_filter=1, sorted_positions=1, full_sort=1)):
        sim = make(sc)
        sim.set_tuning(**t)
        sim.macro_step(8, 3)
        for a, b in zip(sim.get_particles(), want):
            np.testing.assert_array_equal(a, b)


def test_batched_macro_steps_match_standalone(lib):
    scenes = [moving_scene(seed=s) for s in (31, 32, 33)]
    sim = bcs.Simulation(scenes)
    sim.set_particles(np.concatenate([s.positions for s in scenes]), np.concatenate([s.velocities for s in scenes]))
    sim.macro_step(8, 2)
    got = sim.get_particles()
    for k, sc in enumerate(scenes):
        z = sim.scene_info(k)
        rows = slice(z.particle_start, z.particle_start + z.particle_count)
        alone = make(sc)
        alone.macro_step(8, 2)
        for a, b in zip(got, alone.get_particles()):
            np.testing.assert_array_equal(a[rows], b)


def test_macro_step_arguments(lib):
    sim = make(moving_scene())
    for bad in (0, bcs.MAX_SUBSTEPS + 1):
        with pytest.raises(bcs.BcsError):
            sim.macro_step(bad, 1)
