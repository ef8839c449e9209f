"""Pin of the FP64 oracle against the reference itself (CPU only).

tests/golden/ref_pin_*.npz were written by oracle/ref_pin/make_golden.py: the
reference's own hot-path translation units (uniform_grid.cu, blood_cells.cu,
vein_triangles.cu, vein_neighbors.cu, cuda_vec3.cu, vein_collisions.cu)
compiled for the host and run serially on seeded states.  The oracle must
reproduce their compile-time layout, grids and neighbour tables exactly, and
their frames within FP32-vs-FP64 tolerances.  In "reference order" mode the
oracle reads forces in the order the serial run did (the reference's Q3 race
resolved sequentially) and takes collision radii by launch type (Q1).
"""
import glob
import json
import os

import numpy as np
import pytest

import bcs
import bcs_refconfig as RC
import oracle as O

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ref_pin_*.npz")))


def load(path):
    g = dict(np.load(path))
    p = bcs.Params()
    for k, v in json.loads(str(g["params_json"])).items():
        if isinstance(v, list):
            getattr(p, k)[:] = v
        else:
            setattr(p, k, v)
    lay = {k: g[k] for k in ("particle_starts", "model_starts", "graph_starts", "spring_graph", "pic", "count",
                             "models")}
    lay["type_count"] = int(g["type_count"])
    lay["particle_count"] = int(g["particle_count"])
    scene = RC.scene_from_layout(lay, g["vein_positions"], g["vein_indices"], g["ending_centers"], g["ending_radii"],
                                 p, g["init_positions"], g["init_velocities"])
    return g, scene


def rel_err(a, b):
    b = np.asarray(b, np.float64)
    scale = np.abs(b) + np.sqrt(np.mean(b * b)) + 1e-30
    return float(np.max(np.abs(np.asarray(a, np.float64) - b) / scale))


@pytest.fixture(params=GOLDEN, ids=[os.path.basename(p)[8:-4] for p in GOLDEN])
def pinned(request):
    return load(request.param)


def test_goldens_present():
    assert len(GOLDEN) >= 2


def test_layout_matches_reference_meta_factory(pinned):
    g, scene = pinned
    o = O.OracleSim(scene)
    starts, radius, r0 = o.layout(int(g["model_vertex_count"]), int(g["type_count"]))
    np.testing.assert_array_equal(starts[:, 0], g["particle_starts"])
    np.testing.assert_array_equal(starts[:, 1], g["cell_type_starts"])
    np.testing.assert_array_equal(starts[:, 2], g["model_starts"])
    assert o.n == int(g["particle_count"]) and o.cells == int(g["blood_cell_count"])
    np.testing.assert_array_equal(radius, g["bounding_spheres"])
    np.testing.assert_allclose(r0, g["initial_radii"], rtol=1e-6)
    b, dims = o.bounds()
    np.testing.assert_array_equal(b, g["bounds"][:6])
    np.testing.assert_array_equal(dims, g["grid_dims"])


def test_vein_neighbors_match_reference(pinned):
    g, scene = pinned
    o = O.OracleSim(scene)
    ids, ln = o.vein_neighbors()
    np.testing.assert_array_equal(ids, g["vein_nb_ids"])
    np.testing.assert_array_equal(ln, g["vein_nb_len"])


def test_grids_bit_exact_against_reference(pinned):
    g, scene = pinned
    o = O.OracleSim(scene)
    keys, ids, st, en, _ = o.grid_of_points(scene.positions, dense=True)
    np.testing.assert_array_equal(keys, g["pgrid_keys"])
    np.testing.assert_array_equal(ids, g["pgrid_ids"])
    np.testing.assert_array_equal(st, g["pgrid_starts"])
    np.testing.assert_array_equal(en, g["pgrid_ends"])
    tk, ti, ts, te = o.get_grid(1)
    np.testing.assert_array_equal(tk, g["tgrid_keys"])
    np.testing.assert_array_equal(ti, g["tgrid_ids"])
    np.testing.assert_array_equal(ts, g["tgrid_starts"])
    np.testing.assert_array_equal(te, g["tgrid_ends"])


def test_next_frame_matches_reference(pinned):
    g, scene = pinned
    o = O.OracleSim(scene, threads=1)
    o.set_reference_order()
    o.calculate_grids()
    o.calculate_next_frame()
    _, v, f = o.get_particles()
    assert rel_err(f, g["frame1_forces_next"]) <= 1e-5
    assert rel_err(v, g["frame1_velocities_next"]) <= 1e-5


def test_frames_match_reference(pinned):
    g, scene = pinned
    o = O.OracleSim(scene, threads=1)
    o.set_reference_order()
    o.step(1)
    p, v, f = o.get_particles()
    vp, vv, _ = o.get_vein()
    for name, a in (("positions", p), ("velocities", v), ("forces", f)):
        assert rel_err(a, g["frame1_" + name]) <= 1e-5, name
    assert np.abs(vp - g["frame1_vein_positions"]).max() <= 1e-5
    assert np.abs(vv - g["frame1_vein_velocities"]).max() <= 1e-5
    o.step(int(g["steps"]) - 1)
    p, v, f = o.get_particles()
    vp, vv, _ = o.get_vein()
    for name, a in (("positions", p), ("velocities", v), ("forces", f)):
        assert rel_err(a, g["frameN_" + name]) <= 1e-4, name
    assert np.abs(vp - g["frameN_vein_positions"]).max() <= 1e-4


def test_jacobi_oracle_against_reference(pinned):
    # The oracle's own semantics read the previous step's forces for every
    # neighbour (Jacobi).  The reference's gatherForcesKernel reads them while
    # other threads overwrite them (blood_cells.cu:99,118), so its result
    # depends on thread order.  With the small-config constants (d = 0.5,
    # dt = 1e-3) that race moves positions by < 1e-6 relative; with the
    # shipped constants (d = 10, dt = 8e-3) it changes forces by O(1), and
    # only the serial order above can be pinned.
    g, scene = pinned
    o = O.OracleSim(scene, threads=1)
    o.step(1)
    p, v, f = o.get_particles()
    gap = (rel_err(p, g["frame1_positions"]), rel_err(v, g["frame1_velocities"]), rel_err(f, g["frame1_forces"]))
    if scene.params.particle_d_fact * scene.params.dt < 1e-2:
        assert gap[0] <= 1e-6 and gap[1] <= 1e-5 and gap[2] <= 1e-2, gap
    else:
        assert gap[2] > 1e-2, gap   # the race is visible at the shipped constants
