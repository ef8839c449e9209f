"""Pin recipe: run the reference's own step on the CPU and record golden vectors.

Test infrastructure.  Reads the reference's sources from the checkout named by
BCS_REFERENCE (default: a directory "reference" beside this repository), works on a scratch copy under /tmp (launches
rewritten for the serial CPU shim, src/config replaced by a generated set),
compiles the hot-path translation units with g++ into oracle/_ref/, runs the
headless driver on a seeded state and writes tests/golden/ref_pin_<scene>.npz.

  python oracle/ref_pin/make_golden.py            # both pinned scenes
  python oracle/ref_pin/make_golden.py --build    # only (re)build oracle/_ref

Scenes:
  reference_presets  the reference's two shipped cell presets (20 particles,
                     White_blood_cell_One with springs, Blood_dust_One
                     without), 6 cells each, its shipped physics constants
                     (dt 0.008, grid cells 2 / 25), useBloodFlow off, a
                     straight R=20 L=70 vein mesh (32 x 24);
  icosphere_cfg1     42-vertex icospheres emitted as a preset, k=50, d=0.5,
                     dt=1e-3, grid cells 1 / 6, the small-config constants.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REPO = os.path.dirname(ORACLE)
sys.path.insert(0, os.path.join(REPO, "simulation-server_gb300"))
sys.path.insert(0, HERE)

import bcs  # noqa: E402
import bcs_refconfig as RC  # noqa: E402
import bcs_scenes as S  # noqa: E402
from launch_rewrite import rewrite  # noqa: E402

REF = os.environ.get("BCS_REFERENCE", os.path.join(os.path.dirname(REPO), "reference"))
OUT = os.path.join(ORACLE, "_ref")
GOLDEN = os.path.join(REPO, "tests", "golden")
TUS = ["grids/uniform_grid.cu", "objects/blood_cells.cu", "objects/vein_triangles.cu", "objects/vein_neighbors.cu",
       "utilities/cuda_vec3.cu", "simulation/vein_collisions.cu"]


def cxx_flags(src):
    return ["-std=c++17", "-O1", "-w", "-ffp-contract=off", "-x", "c++", "-include",
            os.path.join(HERE, "refcpu_shim.h"), "-D__STORAGE__=extern",
            "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP", "-I" + src,
            "-I" + os.path.join(REF, "Libraries", "include"), "-I/usr/local/cuda/include/cccl",
            "-I/usr/local/cuda/include", "-fconstexpr-ops-limit=4000000000", "-fconstexpr-loop-limit=100000000"]


def scratch_tree(write_config) -> str:
    d = tempfile.mkdtemp(prefix="bcs_refpin_")
    src = os.path.join(d, "src")
    shutil.copytree(os.path.join(REF, "src"), src)
    for tu in TUS:
        p = os.path.join(src, tu)
        text, _ = rewrite(open(p).read())
        with open(p, "w") as f:
            f.write(text)
    write_config(os.path.join(src, "config"))
    return src


def build_driver(src: str, tag: str) -> str:
    obj = os.path.join(OUT, "obj_" + tag)
    os.makedirs(obj, exist_ok=True)
    jobs = [(os.path.join(src, tu), os.path.join(obj, os.path.basename(tu) + ".o"), True) for tu in TUS]
    jobs.append((os.path.join(HERE, "ref_driver.cpp"), os.path.join(obj, "ref_driver.o"), True))
    jobs.append((os.path.join(HERE, "refcpu_runtime.cpp"), os.path.join(obj, "refcpu_runtime.o"), False))

    def run(job):
        s, o, ref = job
        cmd = ["g++"] + (cxx_flags(src) if ref else ["-std=c++17", "-O1", "-I/usr/local/cuda/include"]) + \
              ["-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"compile failed: {s}\n{r.stderr[-4000:]}")
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    exe = os.path.join(OUT, "ref_driver_" + tag)
    r = subprocess.run(["g++", "-o", exe] + [j[1] for j in jobs], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("link failed\n" + r.stderr[-4000:])
    return exe


def params_dict(p: bcs.Params) -> dict:
    d = {}
    for k, _ in bcs.Params._fields_:
        v = getattr(p, k)
        d[k] = list(v) if hasattr(v, "__len__") else v
    return d


def scene_driver(tag: str, vein: S.VeinMesh, params: bcs.Params, counts, preset_mode: str, models=None) -> str:
    """Compile the reference's hot-path TUs with a generated src/config for
    one scene into oracle/_ref; returns the driver executable."""
    scene_stub = S.Scene(tag, [], vein.positions, vein.indices, vein.ending_centers, vein.ending_radii, [], params,
                         np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32))

    def write_config(cfg):
        if preset_mode == "reference":
            # the reference's own presets, chosen counts
            scene_stub.types = [S.CellTypeSpec(counts[0], np.zeros((20, 3)), np.zeros((0, 2)), np.zeros(0)),
                                S.CellTypeSpec(counts[1], np.zeros((20, 3)), np.zeros((0, 2)), np.zeros(0))]
            RC.emit_config(scene_stub, cfg, preset_names=["White_blood_cell_One", "Blood_dust_One"],
                           keep_presets=True)
        else:
            scene_stub.types = [S.CellTypeSpec(c, m.vertices, m.springs, m.spring_lengths) for c, m in
                                zip(counts, models)]
            RC.emit_config(scene_stub, cfg)

    src = scratch_tree(write_config)
    try:
        return build_driver(src, tag)
    finally:
        shutil.rmtree(os.path.dirname(src), ignore_errors=True)


def build_pins() -> list:
    """Compile every pinned scene's reference driver into oracle/_ref (no
    run); nothing when the reference sources are absent."""
    if not os.path.isdir(os.path.join(REF, "src")):
        return []
    os.makedirs(OUT, exist_ok=True)
    return [scene_driver(tag, vein, params, counts, mode, models)
            for tag, vein, params, counts, _steps, _seed, mode, models in scenes()]


def run_scene(tag: str, vein: S.VeinMesh, params: bcs.Params, counts, steps: int, seed: int, preset_mode: str,
              models=None):
    """Build the driver for one scene, run it, return the golden dict."""
    exe = scene_driver(tag, vein, params, counts, preset_mode, models)
    work = tempfile.mkdtemp(prefix="bcs_refpin_run_")
    try:
        subprocess.run([exe, work], check=True)
        lay = RC.layout_from_dump(work)
        # seeded placement of the folded cell models inside the lumen
        rng = np.random.default_rng(seed)
        pos, vel = [], []
        for t in range(lay["type_count"]):
            pic = int(lay["pic"][t])
            m0 = int(lay["model_starts"][t])
            model = lay["models"][m0:m0 + pic]
            cm = S.CellModel("m", model, np.zeros((0, 2), np.int32), np.zeros(0, np.float32),
                             float(np.linalg.norm(model - model.mean(0), axis=1).max() + np.abs(model.mean(0)).max()))
            sites = S.lattice_sites(vein.segments, [cm], [0], particle_radius=0.5)[0]
            ch = sites[rng.choice(len(sites), size=int(lay["count"][t]), replace=False)]
            pos.append((ch[:, None, :] + model[None]).reshape(-1, 3))
            v = rng.normal(0.0, 15.0, size=(len(ch), 3)) + np.array([0.0, -20.0, 0.0])
            vel.append(np.repeat(v, pic, axis=0) + rng.normal(0.0, 0.5, size=(len(ch) * pic, 3)))
        pos = np.concatenate(pos).astype(np.float32)
        vel = np.concatenate(vel).astype(np.float32)
        state = os.path.join(work, "state.bin")
        np.concatenate([pos.ravel(), vel.ravel()]).astype(np.float32).tofile(state)
        subprocess.run([exe, work, state, str(steps)], check=True)
        n, nv = lay["particle_count"], lay["vein_vertex_count"]
        rd = lambda name, dt, shape=None: RC.read_dump(work, name, dt, shape)  # noqa: E731
        out = {k: v for k, v in lay.items() if isinstance(v, np.ndarray)}
        out.update({k: np.int64(v) for k, v in lay.items() if not isinstance(v, np.ndarray)})
        out["grid_dims"] = rd("grid_dims", np.int32)
        for g in ("pgrid", "tgrid"):
            for part in ("keys", "ids", "starts", "ends"):
                out[f"{g}_{part}"] = rd(f"{g}_{part}", np.int32)
        for fr in ("frame1", "frameN"):
            for q in ("positions", "velocities", "forces"):
                out[f"{fr}_{q}"] = rd(f"{fr}_{q}", np.float32, (n, 3))
            for q in ("vein_positions", "vein_velocities"):
                out[f"{fr}_{q}"] = rd(f"{fr}_{q}", np.float32, (nv, 3))
        out["frame1_forces_next"] = rd("frame1_forces_next", np.float32, (n, 3))
        out["frame1_velocities_next"] = rd("frame1_velocities_next", np.float32, (n, 3))
        out["init_positions"] = pos
        out["init_velocities"] = vel
        out["vein_positions"] = vein.positions
        out["vein_indices"] = vein.indices
        out["ending_centers"] = vein.ending_centers
        out["ending_radii"] = vein.ending_radii
        out["steps"] = np.int64(steps)
        out["params_json"] = np.array(json.dumps(params_dict(params)))
        return out
    finally:
        shutil.rmtree(work, ignore_errors=True)


def scenes():
    p = bcs.default_params()
    p.use_blood_flow = 0
    yield ("reference_presets", S.straight_vein(20.0, 70.0, 32, 24), p, (6, 6), 5, 11, "reference", None)
    q = bcs.default_params()
    q.use_blood_flow = 0
    q.dt = 1e-3
    q.particle_k_sniff = 50.0
    q.particle_d_fact = 0.5
    q.cell_width = q.cell_height = q.cell_depth = 1.0
    q.cell_width_triangles = q.cell_height_triangles = q.cell_depth_triangles = 6.0
    ico = S.sphere_cell(3.0, 1)
    yield ("icosphere_cfg1", S.straight_vein(14.0, 80.0, 40, 30), q, (16,), 5, 12, "emitted", [ico])


def main():
    if not os.path.isdir(os.path.join(REF, "src")):
        print(f"reference sources not found at {REF}; nothing to do")
        return 0
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(GOLDEN, exist_ok=True)
    if "--build" in sys.argv:
        for exe in build_pins():
            print("built", exe)
        return 0
    for tag, vein, params, counts, steps, seed, mode, models in scenes():
        g = run_scene(tag, vein, params, counts, steps, seed, mode, models)
        path = os.path.join(GOLDEN, f"ref_pin_{tag}.npz")
        np.savez_compressed(path, **g)
        print("wrote", path, os.path.getsize(path), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
