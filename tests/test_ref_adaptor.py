"""include/bcs_reference.hpp against the Python import of the same config (CPU).

A scene with both of the benchmark's cell models (42-vertex icospheres and
162-vertex biconcave discs), a Y-bifurcation vein and its flow constants is
written as a reference-format src/config (bcs_refconfig.emit_config) into a
scratch copy of the reference's sources.  Then:

  * tests/ref_adaptor_dump.cpp, compiled against that tree, builds the
    bcs_scene_desc the adaptor fills from the reference's compile-time scene
    (meta_factory folding, dense spring graph, vein and endings, constants)
    and dumps it;
  * the reference's own translation units, compiled for the host by the pin
    recipe (oracle/ref_pin) against the same tree, dump the folded layout
    that bcs_refconfig imports (layout_from_dump).

The two must agree: type order, counts and particles per cell, model
vertices, springs and rest lengths bit for bit; the vein mesh bit for bit;
the vein endings as the config's fixed-point format stores them; and every
constant the config carries equal to the scene's.  The reference's sources
come from BCS_REFERENCE (default: a directory "reference" beside this
repository); the test skips without them.
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np
import pytest

import bcs
import bcs_refconfig as RC
import bcs_scenes as S

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "oracle", "ref_pin"))
import make_golden as MG  # noqa: E402

REF = MG.REF

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")),
                                reason="the reference's sources are not present")

# bcs_params fields the reference's config carries (simulation.hpp, physics.hpp)
CONFIG_FIELDS = ("dt", "use_blood_flow", "enable_reaction_force", "enable_big_cells_brake", "cell_width",
                 "cell_height", "cell_depth", "cell_width_triangles", "cell_height_triangles", "cell_depth_triangles",
                 "bounding_spheres_coeff", "grid_y_margin", "grid_xz_margin", "min_spawn_y",
                 "velocity_collision_damping", "particle_k_sniff", "vein_k_sniff", "particle_d_fact", "vein_d_fact",
                 "vein_collision_force_intensity", "viscous_damping", "collision_spring_coeff",
                 "collision_damping_coeff", "collision_shear_coeff", "max_cell_size_factor_before_brake",
                 "big_particle_braking_intensity", "init_velocity", "vein_impact_distance",
                 "vein_impact_minimal_force_distance", "gravity")


def scene():
    sc = S.bifurcation_scene(cells_per_type=3, seed=4, trunk_length=60.0, branch_length=50.0)
    p = sc.params
    p.use_blood_flow = 0
    p.enable_reaction_force = 1
    p.gravity[:] = (0.0, -12.5, 0.25)
    p.init_velocity[:] = (0.0, -40.0, 0.0)
    p.min_spawn_y = -7.0
    return sc


def read_dump(path):
    b = open(path, "rb").read()
    o = 0

    def take(dtype, n):
        nonlocal o
        a = np.frombuffer(b, dtype=dtype, count=n, offset=o)
        o += a.nbytes
        return a
    out = {"types": []}
    for _ in range(int(take(np.int32, 1)[0])):
        count, pic, ns = (int(v) for v in take(np.int32, 3))
        out["types"].append(dict(count=count, pic=pic, vertices=take(np.float32, 3 * pic).reshape(pic, 3),
                                 springs=take(np.int32, 2 * ns).reshape(ns, 2), lengths=take(np.float32, ns)))
    nv, nt, ne = (int(v) for v in take(np.int32, 3))
    out["vein_positions"] = take(np.float32, 3 * nv).reshape(nv, 3)
    out["vein_indices"] = take(np.uint32, 3 * nt).reshape(nt, 3)
    out["ending_centers"] = take(np.float32, 3 * ne).reshape(ne, 3)
    out["ending_radii"] = take(np.float32, ne)
    size = int(take(np.int32, 1)[0])
    assert size == C_SIZEOF_PARAMS, (size, C_SIZEOF_PARAMS)
    out["params"] = bcs.Params.from_buffer_copy(b[o:o + size])
    assert o + size == len(b)
    return out


C_SIZEOF_PARAMS = __import__("ctypes").sizeof(bcs.Params)


@pytest.fixture(scope="module")
def built(tmp_path_factory):
    sc = scene()
    work = tmp_path_factory.mktemp("adaptor")
    src = tempfile.mkdtemp(prefix="bcs_adaptor_")
    try:
        tree = os.path.join(src, "src")
        shutil.copytree(os.path.join(REF, "src"), tree)
        RC.emit_config(sc, os.path.join(tree, "config"))
        exe = str(work / "ref_adaptor_dump")
        lib = os.path.join(REPO, "simulation-server_gb300")
        r = subprocess.run(["g++", "-std=c++17", "-O0", "-w", "-I" + tree,
                            "-I" + os.path.join(REF, "Libraries", "include"), "-I" + os.path.join(REPO, "include"),
                            "-fconstexpr-ops-limit=4000000000", "-fconstexpr-loop-limit=100000000",
                            os.path.join(REPO, "tests", "ref_adaptor_dump.cpp"), "-o", exe, "-L" + lib, "-lbcs",
                            "-Wl,-rpath," + lib], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
    finally:
        shutil.rmtree(src, ignore_errors=True)
    r = subprocess.run([exe, str(work / "desc.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = read_dump(str(work / "desc.bin"))
    # the Python import of the same config, through the reference's own
    # translation units (the pin recipe's layout-only run)
    vein = S.VeinMesh(sc.vein_positions, sc.vein_indices, sc.ending_centers, sc.ending_radii, [])
    driver = MG.scene_driver("adaptor_check", vein, sc.params, [t.count for t in sc.types], "emitted", sc.types)
    lay_dir = work / "layout"
    lay_dir.mkdir()
    r = subprocess.run([driver, str(lay_dir)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    lay = RC.layout_from_dump(str(lay_dir))
    imported = RC.scene_from_layout(lay, sc.vein_positions, sc.vein_indices, sc.ending_centers, sc.ending_radii,
                                    sc.params)
    return sc, got, lay, imported


def test_cell_types_match_the_import(built):
    sc, got, lay, imported = built
    assert len(got["types"]) == lay["type_count"] == len(imported.types) == 2
    # the reference folds its types: the 162-vertex discs first
    assert [t["pic"] for t in got["types"]] == [int(v) for v in lay["pic"]] == [162, 42]
    for t, it in zip(got["types"], imported.types):
        assert t["count"] == it.count
        np.testing.assert_array_equal(t["vertices"], np.asarray(it.vertices, np.float32))
        np.testing.assert_array_equal(t["springs"], np.asarray(it.springs, np.int32))
        np.testing.assert_array_equal(t["lengths"], np.asarray(it.spring_lengths, np.float32))
    # and both carry the scene's own models, through the config's fixed-point
    # cell format (six decimals: 0.5e-6 plus the float rounding)
    by_pic = {len(t.vertices): t for t in sc.types}
    for t in got["types"]:
        src = by_pic[t["pic"]]
        np.testing.assert_allclose(t["vertices"], np.asarray(src.vertices, np.float32), atol=1e-6, rtol=0)
        springs = {tuple(sorted(ab)): L for ab, L in zip(np.asarray(src.springs).reshape(-1, 2).tolist(),
                                                        src.spring_lengths)}
        assert len(t["lengths"]) == len(springs)
        for (a, b), L in zip(t["springs"].tolist(), t["lengths"]):
            assert abs(L - springs[(a, b)]) <= 1e-6, (a, b)


def test_vein_matches_the_config(built):
    sc, got, lay, imported = built
    assert len(got["vein_positions"]) == lay["vein_vertex_count"]
    assert len(got["vein_indices"]) == lay["triangle_count"]
    np.testing.assert_array_equal(got["vein_positions"], np.asarray(imported.vein_positions, np.float32))
    np.testing.assert_array_equal(got["vein_indices"].ravel(), np.asarray(imported.vein_indices).ravel())
    # vein endings travel through the config's fixed-point format (4 decimals)
    np.testing.assert_allclose(got["ending_centers"], np.asarray(sc.ending_centers, np.float32).reshape(-1, 3),
                               atol=1e-4, rtol=0)
    np.testing.assert_allclose(got["ending_radii"], np.asarray(sc.ending_radii, np.float32), atol=1e-4, rtol=0)


def test_constants_match_the_scene(built):
    sc, got, _, _ = built
    p = got["params"]
    for name in CONFIG_FIELDS:
        a, b = getattr(p, name), getattr(sc.params, name)
        if hasattr(a, "__len__"):
            assert list(a) == [float(np.float32(v)) for v in b], name
        else:
            assert np.float32(a) == np.float32(b), (name, a, b)
