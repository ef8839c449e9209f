"""The C-ABI library loads and exports every entry point include/bcs.h declares
(no device work: these run without a GPU)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np

import bcs

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(REPO, "include", "bcs.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bcs_[a-z_0-9]+)\s*\(", text)))


def test_header_and_python_agree():
    assert declared_functions() == sorted(bcs.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", bcs.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (bcs_\w+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    for f in declared_functions():
        assert getattr(lib, f) is not None


def test_status_strings_and_version(lib):
    assert lib.bcs_abi_version() == 3
    assert lib.bcs_status_string(0) == b"ok"
    assert lib.bcs_status_string(3) == b"out of device memory"


def test_invalid_arguments_rejected_before_device_work(lib):
    h = C.c_void_p()
    assert lib.bcs_create(None, None, C.byref(h)) == 1
    d = bcs.SceneDesc()
    d.type_count = 0
    assert lib.bcs_create(C.byref(d), None, C.byref(h)) == 1
    assert not h.value
    assert lib.bcs_step(None, 1) == 1


def test_batch_arguments_rejected_before_device_work(lib, tmp_path):
    import bcs_scenes
    h = C.c_void_p()
    assert lib.bcs_create_batch(None, 1, None, C.byref(h)) == 1
    a = bcs.SceneBuffers(bcs_scenes.tiny_scene(cells=2, seed=1))
    b = bcs.SceneBuffers(bcs_scenes.tiny_scene(cells=3, seed=2))
    descs = (bcs.SceneDesc * 2)(a.desc, b.desc)
    assert lib.bcs_create_batch(descs, 0, None, C.byref(h)) == 1
    descs[1].params.particle_k_sniff = descs[0].params.particle_k_sniff * 2   # physics must match across a batch
    assert lib.bcs_create_batch(descs, 2, None, C.byref(h)) == 1
    assert not h.value
    assert lib.bcs_get_scene_info(None, 0, None) == 1


def test_batch_particle_total_bounded(lib):
    """Each scene under the limit, the batch over it (particle ids are int32):
    rejected before any device work."""
    import bcs_scenes
    bufs = [bcs.SceneBuffers(bcs_scenes.tiny_scene(cells=2, seed=s)) for s in (1, 2)]
    descs = (bcs.SceneDesc * 2)(*[b.desc for b in bufs])
    for d in descs:
        t = d.types[0]
        t.count = (1 << 29) // t.particles_in_cell + 1
    h = C.c_void_p()
    assert lib.bcs_create_batch(descs, 2, None, C.byref(h)) == 1
    assert not h.value


def test_python_harness_checks_shapes():
    rows = bcs._rows(np.zeros((4, 3)), 4, "pos")
    assert rows.dtype == np.float32
    for bad in (np.zeros((5, 3)), np.zeros((3, 4)), np.zeros(12)):
        try:
            bcs._rows(bad, 4, "pos")
        except ValueError:
            continue
        raise AssertionError(f"shape {bad.shape} accepted")
    assert bcs._dev(None, 4, "x") is None
    try:
        bcs._dev(np.zeros(4, np.float32), 4, "x")
    except ValueError:
        pass
    else:
        raise AssertionError("a host array accepted as a device pointer")


STRUCTS = {
    "bcs_vec3": bcs.Vec3, "bcs_cell_type": bcs.CellType, "bcs_vein": bcs.Vein,
    "bcs_flow_segment": bcs.FlowSegment, "bcs_params": bcs.Params, "bcs_scene_desc": bcs.SceneDesc,
    "bcs_info": bcs.Info, "bcs_scene_info": bcs.SceneInfo, "bcs_tuning": bcs.Tuning,
    "bcs_surrogate_desc": bcs.SurrogateDesc, "bcs_surrogate_stats": bcs.SurrogateStats,
    "bcs_init_desc": bcs.InitDesc,
}


def test_ctypes_mirror_matches_c_layout(tmp_path):
    """sizeof/offsetof of every struct in bcs.h, compiled by gcc, against the ctypes mirror."""
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "bcs.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    for cname, py in STRUCTS.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, f"{cname}.{fname}"


def test_step_shapes_match_header():
    text = open(os.path.join(REPO, "include", "bcs.h")).read()
    assert f"#define BCS_STEP_SHAPES {len(bcs.STEP_SHAPES)}" in text
    listed = re.findall(r"(\d) \((\d+), (\d+), (\d+)\)", text)
    assert [tuple(int(v) for v in m[1:]) for m in listed] == list(bcs.STEP_SHAPES)
    cuh = open(os.path.join(REPO, "simulation-server_gb300", "csrc", "bcs_internal.cuh")).read()
    table = re.search(r"kShapes\[kStepShapes\] = \{(.*?)\};", cuh, re.S).group(1)
    assert [tuple(int(v) for v in m) for m in re.findall(r"\{(\d+), (\d+), (\d+)\}", table)] == list(bcs.STEP_SHAPES)


def test_tuning_arguments_rejected(lib):
    assert lib.bcs_get_tuning(None, None) == 1
    assert lib.bcs_set_tuning(None, None) == 1
    assert lib.bcs_autotune(None, 1, None, None) == 1


def test_constants_match_header():
    text = open(os.path.join(REPO, "include", "bcs.h")).read()
    assert f"#define BCS_MAX_SUBSTEPS {bcs.MAX_SUBSTEPS}" in text
    assert f"#define BCS_GRID_SORT_STATIC_MAX {bcs.GRID_SORT_STATIC_MAX}" in text


def test_cell_model_too_large_rejected(lib):
    import bcs_scenes
    sc = bcs_scenes.tiny_scene(cells=1)
    m = bcs_scenes.sphere_cell(8.0, 4)         # 2562 vertices: no launch shape holds the cell
    sc.types[0].vertices = m.vertices
    sc.types[0].springs = m.springs
    sc.types[0].spring_lengths = m.spring_lengths
    sc.types[0].collision_radius = np.full(len(m.vertices), 0.5, np.float32)
    buf = bcs.SceneBuffers(sc)
    h = C.c_void_p()
    assert lib.bcs_create(C.byref(buf.desc), None, C.byref(h)) == 5   # BCS_ERR_UNSUPPORTED
    assert not h.value


def _mutations():
    """(name, mutate(bufs)) pairs, each making one field of a valid scene
    malformed."""
    def types(b):
        return b.desc.types

    def first_array(b, dtype, ndim):
        return next(a for a in b.keep if isinstance(a, np.ndarray) and a.dtype == dtype and a.ndim == ndim)

    def no_particles(b):
        for t in range(b.desc.type_count):
            types(b)[t].count = 0

    def spring_out_of_range(b):
        s = next(a for a in b.keep if isinstance(a, np.ndarray) and a.dtype == np.int32 and a.ndim == 2 and a.size)
        s[0, 0] = types(b)[0].particles_in_cell

    def triangle_out_of_range(b):
        first_array(b, np.uint32, 2)[0, 0] = b.desc.vein.vertex_count

    return [
        ("no particles", no_particles),
        ("negative count", lambda b: setattr(types(b)[0], "count", -1)),
        ("empty cell model", lambda b: setattr(types(b)[0], "particles_in_cell", 0)),
        ("no vertices", lambda b: setattr(types(b)[0], "vertices", None)),
        ("negative spring count", lambda b: setattr(types(b)[0], "spring_count", -1)),
        ("springs without arrays", lambda b: setattr(types(b)[0], "springs", None)),
        ("spring index out of range", spring_out_of_range),
        ("no vein vertices", lambda b: setattr(b.desc.vein, "vertex_count", 0)),
        ("no vein positions", lambda b: setattr(b.desc.vein, "positions", None)),
        ("negative triangle count", lambda b: setattr(b.desc.vein, "triangle_count", -1)),
        ("triangle index out of range", triangle_out_of_range),
        ("too many endings", lambda b: setattr(b.desc.vein, "ending_count", 9)),
        ("negative endings", lambda b: setattr(b.desc.vein, "ending_count", -1)),
        ("flows without an array", lambda b: (setattr(b.desc, "flow_segment_count", 1),
                                              setattr(b.desc, "flow_segments", None))),
        ("zero grid cell", lambda b: setattr(b.desc.params, "cell_width", 0.0)),
        ("NaN grid cell", lambda b: setattr(b.desc.params, "cell_height", float("nan"))),
        ("negative triangle cell", lambda b: setattr(b.desc.params, "cell_depth_triangles", -1.0)),
        ("zero bounding-sphere coefficient", lambda b: setattr(b.desc.params, "bounding_spheres_coeff", 0.0)),
    ]


def test_every_malformed_field_rejected_before_device_work(lib):
    """Each field validate() checks, made malformed on its own, returns
    BCS_ERR_INVALID_ARGUMENT before any device work (on a machine without a
    GPU the unmodified scene gets as far as BCS_ERR_NO_DEVICE)."""
    import bcs_scenes
    sc = bcs_scenes.straight_scene(cells=4, seed=3)
    h = C.c_void_p()
    base = bcs.SceneBuffers(sc)
    st = lib.bcs_create(C.byref(base.desc), None, C.byref(h))
    assert st in (0, 4), st
    if st == 0:
        lib.bcs_destroy(h)
    import copy
    for name, mutate in _mutations():
        b = bcs.SceneBuffers(copy.deepcopy(sc))   # in-place edits must not reach the next case
        mutate(b)
        h = C.c_void_p()
        assert lib.bcs_create(C.byref(b.desc), None, C.byref(h)) == 1, name
        assert not h.value, name


def test_surrogate_inputs_checked_on_the_host():
    """The sizes the library reads for `cells` cells: node features, edge
    features and targets of the wrong shape never reach it."""
    import bcs_scenes
    sc = bcs_scenes.straight_scene(cells=4, seed=3)
    assert bcs._edges_per_cell(sc.types[0]) == 240        # 42-vertex icosphere: 120 springs, both ways
    sur = object.__new__(bcs.Surrogate)                     # no device: only the host-side checks
    sur.pic, sur.edges = 42, 240
    f, e, t = np.zeros((84, 16)), np.zeros((480, 8)), np.zeros((84, 9))
    assert [a.shape for a in sur._inputs(2, f, e, t)] == [(84, 16), (480, 8), (84, 9)]
    for bad in ((f[:-1], e, t), (f, e[:-8], t), (f, e, t[:, :8]), (f.T, e, t)):
        try:
            sur._inputs(2, *bad)
        except ValueError:
            continue
        raise AssertionError("a wrongly shaped input accepted")
