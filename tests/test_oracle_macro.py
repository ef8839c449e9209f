"""The oracle's multi-rate macro step (CPU): one sub-step is the frame, and
eight sub-steps stay close to eight frames on a calm scene."""
import numpy as np

import bcs_scenes as S
import oracle as O


def test_one_substep_is_the_frame():
    sc = S.tiny_scene(cells=5, seed=3)
    sc.velocities[:] = np.random.default_rng(1).normal(0, 10.0, sc.velocities.shape).astype(np.float32)
    a, b = O.OracleSim(sc), O.OracleSim(sc)
    a.step(4)
    b.macro_step(1, 4)
    for x, y in zip(a.get_particles(), b.get_particles()):
        np.testing.assert_array_equal(x, y)
    assert a.steps_done() == b.steps_done() == 4


def test_eight_substeps_close_to_eight_frames():
    sc = S.tiny_scene(cells=5, seed=4)
    sc.velocities[:] = np.random.default_rng(2).normal(0, 2.0, sc.velocities.shape).astype(np.float32)
    a, b = O.OracleSim(sc), O.OracleSim(sc)
    a.step(8)
    b.macro_step(8, 1)
    d = np.linalg.norm(a.get_particles()[0] - b.get_particles()[0], axis=1)
    assert np.median(d) < 1e-4 and d.max() < 5e-2
    assert b.steps_done() == 8
