"""Edge cases of the scene against the oracle: an empty cell type, a vein
with no triangles, one-particle cells without springs, and a cell model
that only the largest launch shape holds."""
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


def check(sc, frames=3, tol=1e-5):
    sim = bcs.Simulation(sc)
    sim.set_particles(sc.positions, sc.velocities)
    o = O.OracleSim(sc)
    sim.step(1)
    o.step(1)
    for g, r in zip(sim.get_particles(), o.get_particles()):
        assert rel_err(g, r) <= tol
    sim.step(frames - 1)
    o.step(frames - 1)
    assert np.abs(sim.get_particles()[0] - o.get_particles()[0]).max() < 1e-3 * 0.5
    return sim


def moving(sc, sigma=8.0, seed=0):
    sc.velocities[:] = np.random.default_rng(seed).normal(0, sigma, sc.velocities.shape).astype(np.float32)
    return sc


def test_empty_cell_type(lib):
    sc = moving(S.mixed_straight_scene(12, 0, 60.0, seed=3, base_radius=14.0))
    empty = S.CellTypeSpec(0, sc.types[0].vertices, sc.types[0].springs, sc.types[0].spring_lengths,
                           sc.types[0].collision_radius, "empty")
    sc.types = [empty] + sc.types
    sim = check(sc)
    assert sim.info.type_count == 2 and sim.info.blood_cell_count == 12


def test_vein_without_triangles(lib):
    sc = moving(S.tiny_scene(cells=6, seed=2))
    sc.vein_indices = np.zeros((0, 3), np.uint32)
    sim = check(sc)
    assert sim.info.triangle_count == 0


def test_single_particle_cells(lib):
    base = S.tiny_scene(cells=2, seed=4)
    rng = np.random.default_rng(5)
    n = 300
    pts = rng.uniform([-8, -35, -8], [8, -5, 8], (n, 3)).astype(np.float32)
    one = S.CellTypeSpec(n, np.zeros((1, 3), np.float32), np.zeros((0, 2), np.int32), np.zeros(0, np.float32),
                         np.full(1, 0.5, np.float32), "point")
    base.types = [one]
    base.positions = pts
    base.velocities = rng.normal(0, 5.0, pts.shape).astype(np.float32)
    check(base)


def test_largest_cell_model(lib):
    m = S.sphere_cell(6.0, 3)            # 642 vertices: only the 768-particle shape holds it
    assert len(m.vertices) == 642
    sc = S.tiny_scene(cells=1, seed=6, radius=16.0, length=50.0)
    t = S.CellTypeSpec(2, m.vertices, m.springs, m.spring_lengths, np.full(len(m.vertices), 0.5, np.float32), "big")
    sc.types = [t]
    c = np.array([[0.0, -14.0, 0.0], [0.0, -30.0, 0.0]], np.float32)
    sc.positions = (c[:, None, :] + m.vertices[None]).reshape(-1, 3).astype(np.float32)
    sc.velocities = np.random.default_rng(7).normal(0, 3.0, sc.positions.shape).astype(np.float32)
    sim = check(sc)
    assert bcs.STEP_SHAPES[sim.get_tuning().step_shape][1] >= 642


def test_wrong_shapes_rejected_on_the_host(lib):
    """Arrays of the wrong row count never reach the library (it reads
    exactly n rows); the state stays what it was."""
    sc = S.straight_scene(cells=4, seed=2)
    sim = bcs.Simulation(sc)
    sim.set_particles(sc.positions, sc.velocities)
    before = sim.get_particles()
    for bad in (sc.positions[:-1], sc.positions.T, np.concatenate([sc.positions, sc.positions[:1]])):
        with pytest.raises(ValueError):
            sim.set_particles(bad, sc.velocities)
    with pytest.raises(ValueError):
        sim.set_vein(pos=sc.vein_positions[:-2])
    for a, b in zip(sim.get_particles(), before):
        np.testing.assert_array_equal(a, b)
