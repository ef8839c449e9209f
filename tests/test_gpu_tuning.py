"""Launch tuning and the autotuner: every tuning computes the same particle
state bit for bit, and bcs_autotune leaves the simulation where it was.

Fixed walls keep the comparisons bit-exact (a deformable wall gathers
particle impacts with float atomics, whose order is not fixed).
"""
import itertools

import numpy as np
import pytest

import bcs
import bcs_scenes as S

pytestmark = pytest.mark.gpu


def scene():
    # two cell types (42 and 162 vertices), velocities that reach the wall,
    # and a start near the outlet so cells are respawned during the run
    sc = S.mixed_straight_scene(14, 9, 70.0, seed=5, base_radius=14.0)
    sc.velocities[:] = np.random.default_rng(2).normal(0, 15.0, sc.velocities.shape).astype(np.float32)
    sc.velocities[:, 1] -= 60.0
    return sc


def run(sc, frames, tuning=None, phases=False, autotune_first=0):
    sim = bcs.Simulation(sc)
    sim.set_particles(sc.positions, sc.velocities)
    if tuning is not None:
        sim.set_tuning(**tuning)
    if autotune_first:
        sim.autotune(autotune_first)
    for _ in range(frames):
        if phases:
            sim.calculate_grids()
            sim.calculate_next_frame()
            sim.propagate_all()
        else:
            sim.step(1)
    return sim


FLAGS = ("persistent", "spatial_order", "full_sort", "occupancy_filter", "sorted_positions", "grid_collisions")
# every shape with every flag off and every flag on, and every flag
# combination on the default shape
ALL = ([dict(step_shape=a, **{f: b for f in FLAGS}) for a in range(len(bcs.STEP_SHAPES)) for b in (0, 1)] +
       [dict(step_shape=0, **dict(zip(FLAGS, bits))) for bits in itertools.product((0, 1), repeat=len(FLAGS))
        if 0 < sum(bits) < len(FLAGS)] +
       [dict(step_shape=a, persistent=a % 2, spatial_order=1 - a % 2, full_sort=0, occupancy_filter=0,
             sorted_positions=a % 2, grid_collisions=g) for a in range(len(bcs.STEP_SHAPES)) for g in (2, 3)])


def test_default_tuning(lib):
    t = bcs.Simulation(scene()).get_tuning().as_dict()
    assert t == dict(step_shape=3, persistent=0, spatial_order=0, full_sort=0, occupancy_filter=0,
                     sorted_positions=0, grid_collisions=3)


@pytest.mark.parametrize("tuning", ALL, ids=lambda t: "s{step_shape}p{persistent}o{spatial_order}f{full_sort}b{occupancy_filter}"
                         "x{sorted_positions}g{grid_collisions}".format(**t))
def test_every_tuning_same_state(lib, tuning):
    """No particle of this scene is crowded, so the grid-order collision
    kernel and the step kernel's own stencil search sum the same candidates
    in the same order."""
    sc = scene()
    frames = 12
    want = run(sc, frames).get_particles()
    sim = run(sc, frames, tuning)
    assert sim.get_tuning().as_dict() == tuning
    for a, b in zip(sim.get_particles(), want):
        np.testing.assert_array_equal(a, b)
    assert (np.abs(want[0][:, 1] - sc.positions[:, 1]) > 10).any()   # some cells were respawned


@pytest.mark.parametrize("shape", range(len(bcs.STEP_SHAPES)))
def test_split_phases_every_shape(lib, shape):
    sc = scene()
    want = run(sc, 6, phases=True).get_particles()
    got = run(sc, 6, dict(step_shape=shape, persistent=shape % 2, spatial_order=1, occupancy_filter=1 - shape % 2,
                          sorted_positions=shape % 2), phases=True).get_particles()
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)


def test_autotune_leaves_state_unchanged(lib):
    sc = scene()
    want = run(sc, 10).get_particles()
    sim = bcs.Simulation(sc)
    sim.set_particles(sc.positions, sc.velocities)
    sim.step(3)
    t, ms = sim.autotune(2)
    assert ms > 0 and sim.get_tuning().as_dict() == t.as_dict()
    assert sim.refresh_info().steps_done == 3
    sim.step(7)
    for a, b in zip(sim.get_particles(), want):
        np.testing.assert_array_equal(a, b)


def test_autotune_batch_and_deformable_wall(lib):
    scenes = []
    for i, (n, L) in enumerate([(8, 60.0), (12, 70.0)]):
        scenes.append(S.bifurcation_scene(cells_per_type=n, seed=70 + i, trunk_length=L, branch_length=L - 10.0,
                                          vel_sigma=5.0))
    def start():
        sim = bcs.Simulation(scenes)
        sim.set_particles(np.concatenate([s.positions for s in scenes]),
                          np.concatenate([s.velocities for s in scenes]))
        return sim
    a = start()
    a.step(6)
    b = start()
    b.step(2)
    b.autotune(1)
    b.step(4)
    pa, pb = a.get_particles()[0], b.get_particles()[0]
    assert np.abs(pa - pb).max() < 1e-4
    assert np.abs(a.get_vein()[0] - b.get_vein()[0]).max() < 1e-5


def test_invalid_tuning_rejected(lib):
    sim = bcs.Simulation(scene())
    for bad in (dict(step_shape=len(bcs.STEP_SHAPES)), dict(step_shape=-1), dict(persistent=2),
                dict(spatial_order=-1), dict(full_sort=3), dict(occupancy_filter=2),
                dict(sorted_positions=-1), dict(grid_collisions=4)):
        with pytest.raises(bcs.BcsError):
            sim.set_tuning(**bad)
    assert sim.get_tuning().as_dict() == dict(step_shape=3, persistent=0, spatial_order=0, full_sort=0,
                                              occupancy_filter=0, sorted_positions=0, grid_collisions=3)


def test_tuning_survives_set_particles_between_phases(lib):
    # A grid built before set_particles still serves calculate_next_frame
    # (the reference's order of calls allows it): the sorted-position copy
    # must follow the new positions.
    sc = scene()
    rng = np.random.default_rng(9)
    pos2 = sc.positions + rng.normal(0, 0.05, sc.positions.shape).astype(np.float32)
    out = []
    for t in (dict(), dict(sorted_positions=1, occupancy_filter=1, grid_collisions=0),
              dict(grid_collisions=0), dict(grid_collisions=2), dict(grid_collisions=3)):
        sim = bcs.Simulation(sc)
        sim.set_particles(sc.positions, sc.velocities)
        sim.set_tuning(**t)
        sim.calculate_grids()
        sim.set_particles(pos2, sc.velocities)
        sim.calculate_next_frame()
        sim.propagate_all()
        out.append(sim.get_particles())
    for other in out[1:]:
        for a, b in zip(other, out[0]):
            np.testing.assert_array_equal(a, b)
