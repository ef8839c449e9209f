"""Batched scenes (bcs_create_batch): every scene of a batch must compute
exactly what it computes alone.

With fixed walls the particle state of a scene depends only on its own
particles, in its own sorted order, so the batch must reproduce a standalone
run bit for bit (grids, respawns and the fused CUDA-graph frame included).
A deformable wall gathers particle impacts with float atomics, whose order
is not fixed even between two standalone runs; there the bound is the one of
the oracle parity tests.
"""
import numpy as np
import pytest

import bcs
import bcs_scenes as S
import oracle as O

pytestmark = pytest.mark.gpu


def fixed_wall_scenes():
    """Four straight vessels of different radius, length, mesh, population
    and seed; the last one starts at the outlet so the vein-end respawn
    fires within a few frames."""
    out = []
    for i, (cells, radius, length, around, rings) in enumerate(
            [(40, 14.0, 90.0, 32, 40), (7, 12.0, 60.0, 24, 20), (64, 16.0, 120.0, 36, 50), (9, 12.0, 60.0, 24, 20)]):
        sc = S.straight_scene(cells=cells, seed=100 + i, radius=radius, length=length, around=around, rings=rings)
        sc.velocities[:] = np.random.default_rng(i).normal(0, 15.0, sc.velocities.shape).astype(np.float32)
        out.append(sc)
    last = out[-1]
    last.positions[:, 1] -= last.positions[:, 1].max() + 44.0
    last.velocities[:] = np.array([0, -80.0, 0], np.float32)
    return out


def standalone(sc, frames, phases=False):
    sim = bcs.Simulation(sc)
    sim.set_particles(sc.positions, sc.velocities)
    for _ in range(frames):
        if phases:
            sim.calculate_grids()
            sim.calculate_next_frame()
            sim.propagate_all()
        else:
            sim.step(1)
    return sim


def batch(scenes):
    sim = bcs.Simulation(scenes)
    sim.set_particles(np.concatenate([s.positions for s in scenes]),
                      np.concatenate([s.velocities for s in scenes]))
    return sim


def rows(sim, k):
    z = sim.scene_info(k)
    return slice(z.particle_start, z.particle_start + z.particle_count)


def test_scene_info_layout(lib):
    scenes = fixed_wall_scenes()
    sim = batch(scenes)
    assert sim.info.scene_count == len(scenes)
    assert sim.info.particle_count == sum(len(s.positions) for s in scenes)
    p = c = v = t = key = tkey = 0
    for k, sc in enumerate(scenes):
        z = sim.scene_info(k)
        alone = bcs.Simulation(sc).info
        assert (z.particle_start, z.blood_cell_start, z.vertex_start, z.triangle_start) == (p, c, v, t)
        assert (z.cell_key_offset, z.tri_cell_key_offset) == (key, tkey)
        assert z.particle_count == alone.particle_count and z.vertex_count == alone.vertex_count
        assert (z.cell_count_x, z.cell_count_y, z.cell_count_z) == (alone.cell_count_x, alone.cell_count_y,
                                                                     alone.cell_count_z)
        assert (z.min_x, z.max_y, z.min_z) == (alone.min_x, alone.max_y, alone.min_z)
        p += z.particle_count
        c += z.blood_cell_count
        v += z.vertex_count
        t += z.triangle_count
        key += z.cell_count
        tkey += z.tri_cell_count
    assert sim.info.cell_count == key and sim.info.tri_cell_count == tkey
    with pytest.raises(bcs.BcsError):
        sim.scene_info(len(scenes))


def test_batch_grid_is_offset_standalone_grids(lib):
    scenes = fixed_wall_scenes()
    sim = batch(scenes)
    sim.step(3)
    sim.calculate_grids()
    keys, ids, _, _ = sim.get_grid(0, dense=False)
    for k, sc in enumerate(scenes):
        z = sim.scene_info(k)
        alone = standalone(sc, 3)
        alone.calculate_grids()
        ak, ai, _, _ = alone.get_grid(0, dense=False)
        r = rows(sim, k)
        np.testing.assert_array_equal(keys[r], ak + z.cell_key_offset)
        np.testing.assert_array_equal(ids[r], ai + z.particle_start)
    # the triangle grid of the batch holds each scene's triangle grid
    tk, ti, _, _ = sim.get_grid(1, dense=False)
    for k, sc in enumerate(scenes):
        z = sim.scene_info(k)
        ak, ai, _, _ = bcs.Simulation(sc).get_grid(1, dense=False)
        r = slice(z.triangle_start, z.triangle_start + z.triangle_count)
        np.testing.assert_array_equal(tk[r], ak + z.tri_cell_key_offset)
        np.testing.assert_array_equal(ti[r], ai + z.triangle_start)


@pytest.mark.parametrize("phases", [False, True])
def test_batch_fixed_walls_bit_exact(lib, phases):
    scenes = fixed_wall_scenes()
    frames = 15
    sim = batch(scenes)
    for _ in range(frames):
        if phases:
            sim.calculate_grids()
            sim.calculate_next_frame()
            sim.propagate_all()
        else:
            sim.step(1)
    got = sim.get_particles()
    for k, sc in enumerate(scenes):
        want = standalone(sc, frames, phases).get_particles()
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a[rows(sim, k)], b)
    # the outlet scene recycled cells to the inflow
    assert (got[0][rows(sim, 3), 1] > -30).any()


def test_batch_two_cell_types_and_flow_segments(lib):
    # Bifurcations carry two cell types (spheres and biconcave discs) and
    # three Poiseuille flow segments each; the wall is held fixed
    # (vein_dynamic off) so the comparison stays bit-exact.
    scenes = []
    for i, (n, L) in enumerate([(12, 60.0), (20, 80.0), (6, 50.0)]):
        sc = S.bifurcation_scene(cells_per_type=n, seed=30 + i, trunk_length=L, branch_length=L - 10.0,
                                 vel_sigma=5.0)
        sc.params.vein_dynamic = 0
        scenes.append(sc)
    sim = batch(scenes)
    sim.step(10)
    got = sim.get_particles()
    for k, sc in enumerate(scenes):
        want = standalone(sc, 10).get_particles()
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a[rows(sim, k)], b)


def test_batch_deformable_walls_match_oracle(lib):
    scenes = []
    for i, (n, L) in enumerate([(10, 60.0), (16, 70.0)]):
        sc = S.bifurcation_scene(cells_per_type=n, seed=50 + i, trunk_length=L, branch_length=L - 10.0,
                                 vel_sigma=5.0)
        scenes.append(sc)
    sim = batch(scenes)
    sim.step(5)
    gp, gv, _ = sim.get_particles()
    vp = sim.get_vein()[0]
    for k, sc in enumerate(scenes):
        z = sim.scene_info(k)
        o = O.OracleSim(sc)
        o.step(5)
        op, ov, _ = o.get_particles()
        assert np.abs(gp[rows(sim, k)] - op).max() < 1e-3 * 0.5
        assert np.abs(vp[z.vertex_start:z.vertex_start + z.vertex_count] - o.get_vein()[0]).max() < 1e-4


def test_batch_without_particle_grid(lib):
    scenes = fixed_wall_scenes()[:2]
    for sc in scenes:
        sc.params.particle_grid = bcs.GRID_NONE
    sim = batch(scenes)
    sim.step(4)
    got = sim.get_particles()
    for k, sc in enumerate(scenes):
        want = standalone(sc, 4).get_particles()
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a[rows(sim, k)], b)
