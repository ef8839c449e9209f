"""The reference's own kernels replayed on the GPU from their cubin and launch
tape (oracle/ref_cuda/replay.cu), against the CPU pin of the same sources.

The replay is built where it runs, from oracle/ref_cuda/replay.cu into
oracle/_ref/ref_cuda_replay; these tests skip while it or the recorded
artifacts are absent.

Tolerances.  nvcc contracts multiply-adds that the pin (g++
-ffp-contract=off) does not: positions agree to 1e-5 relative after one
frame and 1e-4 after five.  Velocities and forces also carry the race of the
reference's spring kernel (gatherForcesKernel reads its neighbours' previous
forces while other threads overwrite them, blood_cells.cu:79,99,118): which
value a thread reads depends on the GPU's scheduling, and the CPU pin and
the oracle's reference order take one serial outcome.  A neighbour read
either way changes one spring term by at most d dt |F_j' - F_j| <= 2 d dt
max|F|, and the average with the previous force halves it; with at most six
springs per particle a force moves by at most 6 d dt max|F| per frame and a
velocity by dt times that.  That bound is added to the elementwise rule,
once per frame replayed.
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPLAY = os.path.join(REPO, "oracle", "_ref", "ref_cuda_replay")
SMALL = os.path.join(REPO, "oracle", "_ref", "refcuda_icosphere_cfg1")


@pytest.fixture(scope="module")
def replay():
    if not (os.path.exists(REPLAY) and os.path.exists(os.path.join(SMALL, "kernels.cubin"))):
        pytest.skip("the reference's replay is not built here")
    return REPLAY


def rel_err(g, o):
    o = np.asarray(o, np.float64)
    scale = np.abs(o) + np.sqrt(np.mean(o * o)) + 1e-30
    return float(np.max(np.abs(np.asarray(g, np.float64) - o) / scale))


def within(g, o, rel, bound):
    """max over elements of |g - o| - (rel (|o| + rms(o)) + bound): <= 0 passes."""
    o = np.asarray(o, np.float64)
    scale = np.abs(o) + np.sqrt(np.mean(o * o))
    return float(np.max(np.abs(np.asarray(g, np.float64) - o) - (rel * scale + bound)))


def race_bounds(forces, dt, d, frames):
    """(force, velocity) bounds of the spring kernel's read race over
    `frames` frames, from the largest force."""
    f = 6.0 * d * dt * float(np.abs(np.asarray(forces, np.float64)).max()) * frames
    return f, dt * f


def run(replay, tmp_path, mode, frames, g):
    state = tmp_path / "state.bin"
    np.concatenate([g["init_positions"].ravel(), g["init_velocities"].ravel()]).astype(np.float32).tofile(state)
    out = tmp_path / f"{mode}{frames}.bin"
    r = subprocess.run([replay, SMALL, mode, str(state), str(frames), str(out)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.fromfile(out, np.float32).reshape(3, -1, 3), r.stdout


def test_pinned_replay_matches_the_pin(replay, tmp_path):
    g = np.load(os.path.join(REPO, "tests", "golden", "ref_pin_icosphere_cfg1.npz"))
    dt, d = 1e-3, 0.5   # the small scene's constants (oracle/ref_cuda/build_ref_cuda.py)
    for frames, tag, tol in ((1, "frame1", 1e-5), (int(g["steps"]), "frameN", 1e-4)):
        o, _ = run(replay, tmp_path, "pinned", frames, g)
        fb, vb = race_bounds(g[f"{tag}_forces"], dt, d, frames)
        e = rel_err(o[0], g[f"{tag}_positions"])
        assert e <= tol, f"{tag} positions: relative error {e:.3e}"
        for q, name, b in ((1, "velocities", vb), (2, "forces", fb)):
            over = within(o[q], g[f"{tag}_{name}"], tol, b)
            assert over <= 0, f"{tag} {name}: {over:.3e} beyond the bound (race bound {b:.3e})"


def test_reference_replay_runs_every_frame(replay, tmp_path):
    import json
    g = np.load(os.path.join(REPO, "tests", "golden", "ref_pin_icosphere_cfg1.npz"))
    o, out = run(replay, tmp_path, "reference", 20, g)
    line = json.loads(out.strip().splitlines()[-1])
    assert line["frames"] == 20 and line["ms_per_frame"] > 0 and line["launches_per_frame"] == 11
    assert np.isfinite(o).all()


def test_two_models_against_the_oracle(replay, tmp_path):
    """Both of the benchmark's cell models on the GPU, the state in the
    reference's folded type order, against the FP64 oracle in reference order
    after one frame: positions 1e-5 relative, velocities and forces 1e-5 plus
    the spring kernel's race bound."""
    import sys
    sys.path.insert(0, os.path.join(REPO, "oracle", "ref_cuda"))
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import build_ref_cuda as B
    import oracle as O
    d = os.path.join(REPO, "oracle", "_ref", "refcuda_two_types")
    if not os.path.exists(os.path.join(d, "kernels.cubin")):
        pytest.skip("the two-model tape is not built here")
    scene = next(s for t, s in B.scenes() if t == "two_types")()
    with open(os.path.join(d, "layout.json")) as f:
        import json
        order = B.reference_order(scene, [tuple(t) for t in json.load(f)["types"]])
    state = tmp_path / "state.bin"
    np.concatenate([scene.positions[order].ravel(), scene.velocities[order].ravel()]).astype(np.float32).tofile(state)
    out = tmp_path / "out.bin"
    r = subprocess.run([replay, d, "pinned", str(state), "1", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    got = np.fromfile(out, np.float32).reshape(3, -1, 3)
    back = np.empty_like(got)
    back[:, order] = got
    o = O.OracleSim(scene)
    o.set_reference_order()
    o.step(1)
    want = o.get_particles()
    p = scene.params
    fb, vb = race_bounds(want[2], p.dt, p.particle_d_fact, 1)
    e = rel_err(back[0], want[0])
    assert e <= 1e-5, f"positions: relative error {e:.3e}"
    for q, name, b in ((1, "velocities", vb), (2, "forces", fb)):
        over = within(back[q], want[q], 1e-5, b)
        assert over <= 0, f"{name}: {over:.3e} beyond the bound (race bound {b:.3e})"
