"""Initial particle state on the device (bcs_init_particles): the reference's
placement rule restated with Philox draws, and the non-overlapping lattice
start."""
import numpy as np
import pytest

import bcs
import bcs_scenes as S
import oracle as O

pytestmark = pytest.mark.gpu


def uniform_open(r):
    return ((np.asarray(r, np.uint64) >> np.uint64(9)) * np.uint64(2) + np.uint64(1)).astype(np.float32) * np.float32(
        1.0 / 16777216.0)


def test_reference_rule(lib):
    sc = S.straight_scene(cells=12, seed=4, radius=14.0, length=90.0, around=32, rings=40)
    sim = bcs.Simulation(sc)
    seed = 0x1234_5678_9ABC
    sim.init_particles(bcs.INIT_REFERENCE, seed=seed)
    pos, vel, frc = sim.get_particles()
    p = sc.params
    m = np.asarray(sc.types[0].vertices, np.float32)
    pic = len(m)
    n = np.float32(len(sc.positions))
    for c in range(12):
        r = O.philox([c, 0xFFFFFFFF, 0xFFFFFFFF, 1], [seed & 0xFFFFFFFF, seed >> 32])
        u = uniform_open(r)
        ox = (u[0] - np.float32(0.5)) * np.float32(1.2) * np.float32(p.cylinder_radius)
        oy = np.float32(p.min_spawn_y) - np.float32(180.0) * u[1] * np.float32(min(n / np.float32(1000.0), 1.0))
        oz = (u[2] - np.float32(0.5)) * np.float32(1.2) * np.float32(p.cylinder_radius)
        want = np.stack([ox + m[:, 0], oy + m[:, 1], oz + m[:, 2]], 1)
        np.testing.assert_allclose(pos[c * pic:(c + 1) * pic], want, rtol=0, atol=2e-5)
    np.testing.assert_array_equal(vel, np.tile(np.asarray(p.init_velocity, np.float32), (len(vel), 1)))
    np.testing.assert_array_equal(frc, 0)
    sim.step(2)
    assert np.isfinite(sim.get_particles()[0]).all()


@pytest.mark.parametrize("which", ["straight", "bifurcation"])
def test_lattice_start(lib, which):
    if which == "straight":
        sc = S.mixed_straight_scene(30, 20, 120.0, seed=2, base_radius=20.0)
    else:
        sc = S.bifurcation_scene(cells_per_type=40, seed=3, trunk_length=120, branch_length=100)
    sim = bcs.Simulation(sc)
    sim.init_particles(bcs.INIT_LATTICE, seed=99, velocity_sigma=0.5, gap=0.2)
    pos, vel, frc = sim.get_particles()
    assert np.isfinite(pos).all()
    # cells do not overlap: centroids at least 2 * (bounding radius + particle radius) apart
    cents, bounds = [], []
    start = 0
    for t in sc.types:
        pic = len(t.vertices)
        c = pos[start:start + t.count * pic].reshape(t.count, pic, 3).mean(1)
        m = np.asarray(t.vertices)
        cents.append(c)
        bounds += [np.linalg.norm(m - m.mean(0), axis=1).max() + 0.5] * t.count
        start += t.count * pic
    cents = np.concatenate(cents)
    bounds = np.asarray(bounds)
    d = np.linalg.norm(cents[:, None] - cents[None], axis=2) + np.eye(len(cents)) * 1e9
    assert (d >= bounds[:, None] + bounds[None] - 1e-3).all()
    # every particle inside the lumen
    segs = ([dict(origin=f["origin"], direction=f["direction"], length=f["length"], radius=f["radius"])
             for f in sc.flow_segments] if sc.flow_segments else
            [dict(origin=(0, 0, 0), direction=(0, -1, 0), length=float(-sc.vein_positions[:, 1].min()),
                  radius=float(sc.params.cylinder_radius))])
    inside = np.zeros(len(pos), bool)
    for sg in segs:
        o, dd = np.asarray(sg["origin"]), np.asarray(sg["direction"])
        tt = (pos - o) @ dd
        rad = np.linalg.norm((pos - o) - tt[:, None] * dd, axis=1)
        inside |= (tt > 0) & (tt < sg["length"]) & (rad < sg["radius"])
    assert inside.all()
    # velocities: init velocity + N(0, 0.5)
    dv = vel - np.asarray(sc.params.init_velocity, np.float32)
    assert abs(dv.mean()) < 0.05 and abs(dv.std() - 0.5) < 0.05
    # deterministic per seed
    sim2 = bcs.Simulation(sc)
    sim2.init_particles(bcs.INIT_LATTICE, seed=99, velocity_sigma=0.5, gap=0.2)
    np.testing.assert_array_equal(sim2.get_particles()[0], pos)
    sim2.init_particles(bcs.INIT_LATTICE, seed=100, velocity_sigma=0.5, gap=0.2)
    assert not np.array_equal(sim2.get_particles()[0], pos)
    sim.step(3)
    assert np.isfinite(sim.get_particles()[0]).all()


def test_batched_start_matches_standalone(lib):
    scenes = [S.mixed_straight_scene(12, 8, 100.0, seed=s, base_radius=18.0) for s in (5, 6)]
    sim = bcs.Simulation(scenes)
    sim.init_particles(bcs.INIT_LATTICE, seed=7, velocity_sigma=0.3)
    got = sim.get_particles()
    for k, sc in enumerate(scenes):
        z = sim.scene_info(k)
        rows = slice(z.particle_start, z.particle_start + z.particle_count)
        alone = bcs.Simulation(sc)
        alone.init_particles(bcs.INIT_LATTICE, seed=7, velocity_sigma=0.3)
        for a, b in zip(got, alone.get_particles()):
            np.testing.assert_array_equal(a[rows], b)


def test_init_arguments(lib):
    sim = bcs.Simulation(S.tiny_scene(cells=2))
    with pytest.raises(bcs.BcsError):
        sim.init_particles(kind=7)
    with pytest.raises(bcs.BcsError):
        sim.init_particles(bcs.INIT_LATTICE, velocity_sigma=-1.0)
    # a vessel far too small for its cells
    small = S.tiny_scene(cells=2)
    small.types[0].count = 400
    small.positions = np.zeros((400 * 42, 3), np.float32)
    small.velocities = np.zeros_like(small.positions)
    with pytest.raises(bcs.BcsError):
        bcs.Simulation(small).init_particles(bcs.INIT_LATTICE)
