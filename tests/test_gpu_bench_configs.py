"""The benchmark configurations themselves against the FP64 oracle.

The parity contract of tests/test_gpu_parity.py applied to the scenes the
benchmark times, built by the same generators and seeds:

  * the 4.2M-particle workload (Y bifurcation, two cell types, Poiseuille flow
    segments, deformable spring wall) at 1/8 scale (2 574 cells per type,
    525 096 particles, same seed): particle and triangle grids bit-exact, then
    one frame within 1e-5 relative elementwise for the particles' x, v, F and
    the wall's x, v;
  * the same scene family at 1 000 cells per type (204 000 particles): 100
    frames;
  * the first 8 vessels of the batched workload's draw (the same seed; the
    draw of a longer batch starts with the same 8): batched on the GPU, each
    vessel against its own oracle run, one frame within 1e-5, then three
    frames.

Over many frames the reference's dynamics is chaotic for a few particles: its
collision force pulls overlapping particles together and amplifies their
relative velocity (physics.cuh:133-145), and some disc particles reach
speeds of several hundred.  The FP64 oracle itself, restarted with its
positions moved by 1e-6, departs from its own run by 4.6e-2 after 100 frames
at the 1 000-cell scene (p99 3e-6, 0.01 % of particles above 1e-3 of the
radius), and by 2e-4 after 3 frames at the first batched vessel.  FP32
rounding is a perturbation of that size in every step; the control run here
moves every initial coordinate by one FP32 ulp.  So the long runs
hold the bulk of the particles to 1e-3 of the radius (99.9 % of them, and at
most 0.1 % above it) and bound the largest error by that of the oracle's own
control run: at most ten times the control's departure (or 1e-3 of the
radius).

The full-size 4.2M frame is checked by bench.py itself (its `parity` key).
"""
import numpy as np
import pytest

import bcs
import bcs_scenes as S
import oracle as O

pytestmark = pytest.mark.gpu

RTOL_1STEP = 1e-5
RADIUS = 0.5
BENCH_SEED = 2024


def rel_err(g, o):
    o = np.asarray(o, np.float64)
    scale = np.abs(o) + np.sqrt(np.mean(o * o)) + 1e-30
    return float(np.max(np.abs(np.asarray(g, np.float64) - o) / scale))


def make(scene):
    sim = bcs.Simulation(scene)
    sim.set_particles(scene.positions, scene.velocities)
    return sim


@pytest.fixture(scope="module")
def eighth():
    sc = S.bifurcation_scene(cells_per_type=2574, seed=BENCH_SEED)
    assert sc.params.vein_dynamic and len(sc.flow_segments) == 3 and len(sc.types) == 2
    return sc


def test_bifurcation_eighth_grids_bit_exact(lib, eighth):
    sim = make(eighth)
    sim.calculate_grids()
    o = O.OracleSim(eighth)
    o.calculate_grids()
    for which in (0, 1):
        k, i, st, en = sim.get_grid(which)
        ok, oi, ost, oen = o.get_grid(which)
        np.testing.assert_array_equal(k, ok, err_msg=f"grid {which} keys")
        np.testing.assert_array_equal(i, oi, err_msg=f"grid {which} ids")
        np.testing.assert_array_equal(st, ost, err_msg=f"grid {which} starts")
        np.testing.assert_array_equal(en, oen, err_msg=f"grid {which} ends")
    sim.close()
    o.close()


def test_bifurcation_eighth_one_frame(lib, eighth):
    sim = make(eighth)
    sim.step(1)
    g = sim.get_particles()
    gv = sim.get_vein()
    o = O.OracleSim(eighth)
    o.step(1)
    for name, a, b in zip(("position", "velocity", "force"), g, o.get_particles()):
        e = rel_err(a, b)
        assert e <= RTOL_1STEP, f"{name}: relative error {e:.3e}"
    ov = o.get_vein()
    e = rel_err(gv[0], ov[0])
    assert e <= RTOL_1STEP, f"wall position: relative error {e:.3e}"
    # After one frame a wall velocity is dt x (spring forces at rest length +
    # particle impacts); at rest length a spring force is FP32 rounding of
    # |p - q| - L, at most k_vein L 2^-23 for each of a vertex's nine
    # springs.  So the elementwise rule gets that floor: 9 dt k_vein L_max 2^-23.
    tri = eighth.vein_indices.reshape(-1, 3)
    vp = eighth.vein_positions
    edge = max(np.linalg.norm(vp[tri[:, a]] - vp[tri[:, b]], axis=1).max() for a, b in ((0, 1), (1, 2), (2, 0)))
    p = eighth.params
    floor = 9 * p.dt * p.vein_k_sniff * edge * 2.0 ** -23
    o1 = np.asarray(ov[1], np.float64)
    over = np.abs(np.asarray(gv[1], np.float64) - o1) - (1e-5 * (np.abs(o1) + np.sqrt(np.mean(o1 * o1))) + floor)
    assert over.max() <= 0, f"wall velocity: {over.max():.3e} beyond the bound (floor {floor:.3e})"
    sim.close()
    o.close()


def control_departure(scene, frames):
    """Largest position departure of the FP64 oracle from its own run when
    every initial coordinate moves by one FP32 ulp (the size of one FP32
    rounding)."""
    a = O.OracleSim(scene)
    a.step(frames)
    b = O.OracleSim(scene)
    b.set_particles(np.nextafter(scene.positions, np.float32(np.inf)), scene.velocities)
    b.step(frames)
    d = float(np.abs(a.get_particles()[0] - b.get_particles()[0]).max())
    want = a.get_particles()[0]
    a.close()
    b.close()
    return d, want


def check_long_run(got, want, control, what):
    d = np.abs(got - want).max(1)
    tol = 1e-3 * RADIUS
    assert np.quantile(d, 0.999) < tol, f"{what}: p99.9 position error {np.quantile(d, 0.999):.3e}"
    assert (d > tol).mean() <= 1e-3, f"{what}: {(d > tol).mean():.2%} of particles above 1e-3 of the radius"
    assert d.max() <= max(tol, 10.0 * control), f"{what}: max error {d.max():.3e}, oracle control {control:.3e}"


def test_bifurcation_hundred_frames(lib):
    sc = S.bifurcation_scene(cells_per_type=1000, seed=BENCH_SEED + 1)
    sim = make(sc)
    sim.step(100)
    pos = sim.get_particles()[0]
    wall = sim.get_vein()[0]
    sim.close()
    control, want = control_departure(sc, 100)
    check_long_run(pos, want, control, "100 frames")
    o = O.OracleSim(sc)
    o.step(100)
    werr = np.abs(wall - o.get_vein()[0]).max()
    assert werr < 1e-3 * RADIUS, f"max wall position error {werr:.3e}"
    o.close()


def test_batched_slice_against_oracle(lib):
    scenes = S.batched_scenes(count=8, seed=BENCH_SEED)
    sim = bcs.Simulation(scenes)
    sim.set_particles(np.concatenate([s.positions for s in scenes]),
                      np.concatenate([s.velocities for s in scenes]))
    rows = []
    for k in range(len(scenes)):
        z = sim.scene_info(k)
        rows.append(slice(z.particle_start, z.particle_start + z.particle_count))
    sim.step(1)
    g1 = sim.get_particles()
    sim.step(2)
    g3 = sim.get_particles()[0]
    sim.close()
    for k, sc in enumerate(scenes):
        o = O.OracleSim(sc)
        o.step(1)
        for name, a, b in zip(("position", "velocity", "force"), g1, o.get_particles()):
            e = rel_err(a[rows[k]], b)
            assert e <= RTOL_1STEP, f"vessel {k} {name}: relative error {e:.3e}"
        o.close()
        control, want = control_departure(sc, 3)
        check_long_run(g3[rows[k]], want, control, f"vessel {k}, 3 frames")
