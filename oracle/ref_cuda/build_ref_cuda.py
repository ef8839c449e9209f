"""Recipe: the reference's own CUDA kernels for sm_103a plus the launch tape of
its host code, so that the reference's kernels can run on a machine that
cannot build the reference itself (without its sources, or of another
architecture than the one that recorded the tape).  Test infrastructure: it reads the
reference's sources from the checkout named by BCS_REFERENCE (default: a
directory "reference" beside this repository), works on scratch copies under /tmp and writes only into
oracle/_ref/refcuda_<scene>/:

  kernels.cubin   the reference's simulation translation units, unmodified,
                  compiled with nvcc (-rdc) and device-linked into one cubin
  entries.txt     the cubin's kernel entry names, as ptxas reports them
  reference.tape  the host code's launches for construction and two frames,
                  exactly the reference's calls (timing)
  pinned.tape     the same plus the Q5 clears and last-cell ranges the CPU pin
                  applies (parity against the pin)
  kernels.txt     recorder address -> cubin entry, one line per kernel on a tape
  layout.json     counts of the scene and the folded type order (the
                  reference merges and sorts the user's types, so a state
                  handed to the replay follows reference_order())
  limits.txt      the reference's grid box and dt (the replay's guard)
  tape_recorder   the recorder (host code of the build host); it also replays
                  its tapes on the CPU (--replay-cpu), which the tests compare
                  with the CPU pin

The tape is recorded by the reference's own host code (constructors,
calculateGrid, gatherForcesFromNeighbors, propagateForcesIntoPositions),
compiled with g++ against tape_shim.h: every <<<>>> launch and the one
thrust::stable_sort_by_key become records instead of work.

  python oracle/ref_cuda/build_ref_cuda.py [scene ...]
  python oracle/ref_cuda/build_ref_cuda.py --replay    # the GPU replay, where it runs
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REPO = os.path.dirname(ORACLE)
PIN = os.path.join(ORACLE, "ref_pin")
for p in (PIN, os.path.join(REPO, "simulation-server_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import bcs  # noqa: E402
import bcs_refconfig as RC  # noqa: E402
import bcs_scenes as S  # noqa: E402
from launch_rewrite import rewrite  # noqa: E402

REF = os.environ.get("BCS_REFERENCE", os.path.join(os.path.dirname(REPO), "reference"))
OUT = os.path.join(ORACLE, "_ref")
DEVICE_TUS = ["grids/uniform_grid.cu", "objects/blood_cells.cu", "objects/vein_neighbors.cu",
              "objects/vein_triangles.cu", "simulation/simulation_controller.cu", "simulation/vein_collisions.cu",
              "simulation/vein_end.cu", "utilities/cuda_vec3.cu"]
HOST_TUS = ["grids/uniform_grid.cu", "objects/blood_cells.cu", "objects/vein_triangles.cu",
            "objects/vein_neighbors.cu", "utilities/cuda_vec3.cu", "simulation/vein_collisions.cu"]
RECIPE = [os.path.join(HERE, f) for f in ("build_ref_cuda.py", "tape_shim.h", "tape_format.h", "tape_runtime.cpp",
                                          "tape_driver.cpp")] + \
         [os.path.join(PIN, "launch_rewrite.py")]
_SORT = re.compile(r"thrust::stable_sort_by_key\(\s*(\w+)\s*,\s*\1\s*\+\s*(\w+)\s*,\s*(\w+)\s*\)\s*;")
_ENTRY = re.compile(r"Compiling entry function '([^']+)'")


def available() -> bool:
    return os.path.isdir(os.path.join(REF, "src"))


def scenes():
    """(tag, scene) pairs: the pinned small scene, a small scene with both
    of the benchmark's cell models, and the 4.2M-particle bifurcation of the
    benchmark with the reference's physics (the axial flow segments are this
    project's own and are dropped; useBloodFlow = 0)."""
    q = bcs.default_params()
    q.use_blood_flow = 0
    q.dt = 1e-3
    q.particle_k_sniff = 50.0
    q.particle_d_fact = 0.5
    q.cell_width = q.cell_height = q.cell_depth = 1.0
    q.cell_width_triangles = q.cell_height_triangles = q.cell_depth_triangles = 6.0
    vein = S.straight_vein(14.0, 80.0, 40, 30)
    ico = S.sphere_cell(3.0, 1)
    small = S.Scene("icosphere_cfg1", [S.CellTypeSpec(16, ico.vertices, ico.springs, ico.spring_lengths)],
                    vein.positions, vein.indices, vein.ending_centers, vein.ending_radii, [], q,
                    np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32))
    yield "icosphere_cfg1", small

    def two_types():
        # both cell models of the benchmark, a few cells each, with the
        # bounding-sphere radii the reference computes (its config has no
        # per-particle collision radius)
        sc = S.bifurcation_scene(cells_per_type=12, seed=7)
        sc.params.use_blood_flow = 0
        sc.flow_segments = []
        for t in sc.types:
            t.collision_radius = None
        return sc
    yield "two_types", two_types

    def bifurcation():
        sc = S.bifurcation_scene(cells_per_type=20588, seed=2024)
        sc.params.use_blood_flow = 0
        return sc
    yield "bifurcation_4.2M", bifurcation


def tape_layout(tape_path: str) -> list:
    """(particles in cell, count, first particle) of every type in the
    reference's folded order, as the recorder marked it."""
    import tape as T
    for op in T.read(tape_path):
        if op["op"] == "mark" and op["label"].startswith("layout:"):
            return [tuple(int(v) for v in t.split(",")) for t in op["label"][7:].split(";") if t]
    raise ValueError(f"{tape_path} marks no layout")


def reference_order(scene, layout) -> np.ndarray:
    """Scene particle index of each particle in the reference's order: its
    folded types take the scene's types of the same model size and count,
    first unused first."""
    starts = np.cumsum([0] + [t.count * len(t.vertices) for t in scene.types])
    used, parts = set(), []
    for pic, count, _ in layout:
        k = next((i for i, t in enumerate(scene.types)
                  if i not in used and len(t.vertices) == pic and t.count == count), None)
        if k is None:
            raise ValueError(f"no scene type of {count} cells x {pic} particles")
        used.add(k)
        parts.append(np.arange(starts[k], starts[k + 1]))
    return np.concatenate(parts)


def _scratch(scene, tape: bool) -> str:
    d = tempfile.mkdtemp(prefix="bcs_refcuda_")
    src = os.path.join(d, "src")
    shutil.copytree(os.path.join(REF, "src"), src)
    RC.emit_config(scene, os.path.join(src, "config"))
    if tape:
        for tu in HOST_TUS:
            p = os.path.join(src, tu)
            text, _ = rewrite(open(p).read(), form="tape")
            text, n = _SORT.subn(r"bcs_tape_sort(thrust::raw_pointer_cast(\1), \2, thrust::raw_pointer_cast(\3));",
                                 text)
            if tu == "grids/uniform_grid.cu" and n != 1:
                raise RuntimeError("the key sort of calculateGrid was not found")
            with open(p, "w") as f:
                f.write(text)
    return src


def _run(cmd, what):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"{what} failed\n{' '.join(cmd)}\n{r.stderr[-4000:]}")
    return r


def build_cubin(src: str, out: str) -> list:
    """Device code of every simulation TU, unmodified, linked into one cubin;
    returns the entry names ptxas reported."""
    obj = os.path.join(out, "obj")
    os.makedirs(obj, exist_ok=True)

    def one(tu):
        o = os.path.join(obj, os.path.basename(tu) + ".o")
        # the reference's own device flags (CMakeLists.txt:32,145): -O3,
        # --expt-relaxed-constexpr, --maxrregcount=40; its 1024-thread
        # launches need the register cap
        r = _run(["nvcc", "-std=c++17", "--expt-relaxed-constexpr", "--maxrregcount=40", "-rdc=true", "-gencode",
                  "arch=compute_103a,code=sm_103a", "-O3", "-I" + src,
                  "-I" + os.path.join(REF, "Libraries", "include"), "-Xptxas", "-v", "-c",
                  os.path.join(src, tu), "-o", o], "nvcc " + tu)
        return o, _ENTRY.findall(r.stderr)
    with ThreadPoolExecutor(max_workers=len(DEVICE_TUS)) as ex:
        res = list(ex.map(one, DEVICE_TUS))
    _run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-dlink", "-cubin", "-o",
          os.path.join(out, "kernels.cubin")] + [o for o, _ in res], "device link")
    entries = sorted({e for _, es in res for e in es})
    with open(os.path.join(out, "entries.txt"), "w") as f:
        f.write("\n".join(entries) + "\n")
    shutil.rmtree(obj, ignore_errors=True)
    return entries


def build_recorder(src: str, out: str) -> str:
    obj = os.path.join(out, "rec_obj")
    os.makedirs(obj, exist_ok=True)
    flags = ["-std=c++17", "-O1", "-w", "-ffp-contract=off", "-fno-pie", "-x", "c++", "-include",
             os.path.join(HERE, "tape_shim.h"), "-D__STORAGE__=extern",
             "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP", "-I" + src,
             "-I" + os.path.join(REF, "Libraries", "include"), "-I/usr/local/cuda/include/cccl",
             "-I/usr/local/cuda/include", "-fconstexpr-ops-limit=4000000000", "-fconstexpr-loop-limit=100000000"]
    jobs = [(os.path.join(src, tu), os.path.join(obj, os.path.basename(tu) + ".o"), flags) for tu in HOST_TUS]
    jobs.append((os.path.join(HERE, "tape_driver.cpp"), os.path.join(obj, "tape_driver.o"), flags))
    jobs.append((os.path.join(HERE, "tape_runtime.cpp"), os.path.join(obj, "tape_runtime.o"),
                 ["-std=c++17", "-O1", "-fno-pie", "-I" + HERE, "-I/usr/local/cuda/include"]))

    def one(job):
        s, o, fl = job
        _run(["g++"] + fl + ["-c", s, "-o", o], "g++ " + os.path.basename(s))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(one, jobs))
    exe = os.path.join(out, "tape_recorder")
    _run(["g++", "-no-pie", "-o", exe] + [j[1] for j in jobs], "link")
    shutil.rmtree(obj, ignore_errors=True)
    return exe


def recorder_symbols(exe: str) -> dict:
    """Address -> mangled name of every function in the recorder (its own
    symbol table; the recorder is linked at fixed addresses)."""
    r = _run(["nm", exe], "nm")
    out = {}
    for line in r.stdout.splitlines():
        f = line.split()
        if len(f) == 3 and f[1] in "tTwW":
            out[int(f[0], 16)] = f[2]
    return out


def cubin_entry(name: str, entries: list) -> str | None:
    """The cubin entry of a host-side kernel symbol: the same Itanium name,
    or, for a kernel nvcc gives internal linkage, that name behind the
    __nv_static_<tag>_ prefix of its translation unit (g++ may write the
    host symbol as _ZL...)."""
    if name in entries:
        return name
    base = "_Z" + name[3:] if name.startswith("_ZL") else name
    hits = [e for e in entries if e.startswith("__nv_static_") and e.endswith("_" + base)]
    return hits[0] if len(hits) == 1 else None


def _stamp(scene_key: str) -> str:
    h = hashlib.sha256(scene_key.encode())
    for f in RECIPE:
        h.update(open(f, "rb").read())
    return h.hexdigest()


def build(tag: str, scene, frames: int = 2, force: bool = False) -> str:
    """Build one scene's cubin and tapes into oracle/_ref/refcuda_<tag>;
    cached on the scene's config and the recipe."""
    import tape as T
    out = os.path.join(OUT, "refcuda_" + tag)
    if callable(scene):
        scene = scene()
    cfg_dir = tempfile.mkdtemp(prefix="bcs_refcuda_cfg_")
    try:
        RC.emit_config(scene, cfg_dir)
        key = "".join(open(os.path.join(cfg_dir, f)).read() for f in sorted(os.listdir(cfg_dir)))
    finally:
        shutil.rmtree(cfg_dir, ignore_errors=True)
    stamp = _stamp(key)
    stamp_path = os.path.join(out, "stamp")
    if not force and os.path.exists(stamp_path) and open(stamp_path).read() == stamp:
        return out
    os.makedirs(out, exist_ok=True)
    dev_src = _scratch(scene, tape=False)
    host_src = _scratch(scene, tape=True)
    try:
        with ThreadPoolExecutor(max_workers=2) as ex:
            fc = ex.submit(build_cubin, dev_src, out)
            fr = ex.submit(build_recorder, host_src, out)
            entries, exe = fc.result(), fr.result()
    finally:
        shutil.rmtree(os.path.dirname(dev_src), ignore_errors=True)
        shutil.rmtree(os.path.dirname(host_src), ignore_errors=True)
    for mode in ("reference", "pinned"):
        _run([exe, os.path.join(out, mode + ".tape"), mode, str(frames)], "recording " + mode)
    syms = recorder_symbols(exe)
    lines = []
    for addr in sorted({op["kernel"] for op in T.read(os.path.join(out, "reference.tape")) if op["op"] == "launch"} |
                       {op["kernel"] for op in T.read(os.path.join(out, "pinned.tape")) if op["op"] == "launch"}):
        name = syms.get(addr)
        entry = cubin_entry(name, entries) if name else None
        if entry is None:
            raise RuntimeError(f"kernel at {addr:#x} ({name}) has no cubin entry")
        lines.append(f"{addr:x} {entry}")
    with open(os.path.join(out, "kernels.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(os.path.join(out, "layout.json"), "w") as f:
        json.dump({"scene": tag, "particles": int(sum(t.count * len(t.vertices) for t in scene.types)),
                   "cells": int(sum(t.count for t in scene.types)), "vein_vertices": int(len(scene.vein_positions)),
                   "triangles": int(len(scene.vein_indices)), "frames_recorded": frames,
                   "types": tape_layout(os.path.join(out, "reference.tape"))}, f)
    # the reference's grid box (vein_factory.hpp:21-86) and dt, for the
    # replay's guard against particles leaving it
    p = scene.params
    lo = np.asarray(scene.vein_positions, np.float32).min(0)
    hi = np.asarray(scene.vein_positions, np.float32).max(0)
    box = [lo[0] - p.grid_xz_margin, hi[0] + p.grid_xz_margin, lo[1] - p.grid_y_margin, hi[1] + p.grid_y_margin,
           lo[2] - p.grid_xz_margin, hi[2] + p.grid_xz_margin]
    with open(os.path.join(out, "limits.txt"), "w") as f:
        f.write(" ".join(f"{float(v):.9g}" for v in box) + f" {float(p.dt):.9g}\n")
    with open(stamp_path, "w") as f:
        f.write(stamp)
    return out


def build_replay(out: str | None = None) -> str:
    """The GPU replay (replay.cu, our own source) with the local nvcc; built
    on the machine that runs it, since host code does not travel between
    architectures."""
    exe = out or os.path.join(OUT, "ref_cuda_replay")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    stubs = "/usr/local/cuda/lib64/stubs"
    _run(["nvcc", "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
          os.path.join(HERE, "replay.cu")] + (["-L" + stubs] if os.path.isdir(stubs) else []) + ["-lcuda"],
         "nvcc replay.cu")
    return exe


def build_all(tags=None) -> list:
    """Every scene (or the named ones); nothing when the reference sources
    are absent."""
    if not available():
        return []
    if HERE not in sys.path:
        sys.path.insert(0, HERE)
    return [build(tag, sc) for tag, sc in scenes() if tags is None or tag in tags]


if __name__ == "__main__":
    if sys.argv[1:] == ["--replay"]:
        print("built", build_replay())
    else:
        for d in build_all(sys.argv[1:] or None):
            print("built", d)
