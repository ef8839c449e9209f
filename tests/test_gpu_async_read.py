"""Asynchronous reads of the particle state (bcs_get_particles_async): each
read returns the state of the frame it was issued after, bit for bit, while
later frames run; more reads than the two slots in flight wait on the GPU,
not on the host."""
import numpy as np
import pytest

import bcs
import bcs_scenes as S

pytestmark = pytest.mark.gpu


def make(sc):
    sim = bcs.Simulation(sc)
    sim.set_particles(sc.positions, sc.velocities)
    return sim


def test_async_reads_match_synchronous_ones(lib):
    sc = S.straight_scene(cells=64, seed=5, radius=14.0, length=120.0, around=40, rings=50)
    sc.velocities[:] = np.random.default_rng(2).normal(0, 20.0, sc.velocities.shape).astype(np.float32)
    sim, ref = make(sc), make(sc)
    frames = 5
    bufs = [[np.empty((3, sim.n), np.float32) for _ in range(3)] for _ in range(frames)]
    for f in range(frames):
        sim.step(1)
        sim.get_particles_async(*bufs[f])
    sim.wait_particles()
    for f in range(frames):
        ref.step(1)
        for got, want in zip(bufs[f], ref.get_particles()):
            np.testing.assert_array_equal(got.T, want)


def test_async_read_of_positions_only_and_midframe(lib):
    sc = S.straight_scene(cells=16, seed=3)
    sim, ref = make(sc), make(sc)
    pos = np.empty((3, sim.n), np.float32)
    sim.calculate_grids()
    sim.calculate_next_frame()          # mid frame: the read sees the new velocities and forces
    ref.calculate_grids()
    ref.calculate_next_frame()
    sim.get_particles_async(pos)
    sim.wait_particles()
    np.testing.assert_array_equal(pos.T, ref.get_particles()[0])
    with pytest.raises(ValueError):
        sim.get_particles_async(np.empty((sim.n, 3), np.float32))


def test_close_with_reads_in_flight(lib):
    """Destroying the handle waits for the reads it started."""
    sc = S.straight_scene(cells=32, seed=6)
    sim, ref = make(sc), make(sc)
    bufs = [np.empty((3, sim.n), np.float32) for _ in range(3)]
    sim.step(2)
    sim.get_particles_async(*bufs)
    sim.close()
    ref.step(2)
    for got, want in zip(bufs, ref.get_particles()):
        np.testing.assert_array_equal(got.T, want)
