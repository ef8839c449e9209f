"""The reference's own CUDA build as a replayable cubin and launch tape
(oracle/ref_cuda), checked on the CPU: the recipe compiles the reference's
simulation translation units unmodified for sm_103a, records its host code's
launches, and every recorded launch is complete and safe to replay.

Runs where the reference's sources are present (the recipe reads them).
"""
import os
import struct
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "oracle", "ref_cuda"))

import build_ref_cuda as B  # noqa: E402
import tape as T  # noqa: E402

pytestmark = pytest.mark.skipif(not B.available(), reason="reference sources not present")

SCENE = "icosphere_cfg1"


@pytest.fixture(scope="module")
def built():
    B.build_all([SCENE])
    return os.path.join(B.OUT, "refcuda_" + SCENE)


def kernel_names(d):
    out = {}
    for line in open(os.path.join(d, "kernels.txt")):
        addr, entry = line.split()
        out[int(addr, 16)] = entry
    return out


def _shape(op):
    """An op without the bytes of class arguments: their padding holds
    whatever the recorder's copies left there, which differs between runs
    and no kernel reads.  Scalar arguments (4 and 8 bytes) stay."""
    o = dict(op)
    if "params" in o:
        o["params"] = [(len(p["bytes"]), p["bytes"] if len(p["bytes"]) <= 8 else b"",
                        tuple((r["offset"], r["id"], r["off"]) for r in p["relocs"])) for p in o["params"]]
    return repr(sorted(o.items()))


def test_artifacts(built):
    for f in ("kernels.cubin", "entries.txt", "kernels.txt", "reference.tape", "pinned.tape", "limits.txt"):
        assert os.path.getsize(os.path.join(built, f)) > 0, f
    with open(os.path.join(built, "kernels.cubin"), "rb") as f:
        assert f.read(4) == b"\x7fELF"


@pytest.mark.parametrize("mode", ["reference", "pinned"])
def test_frames_repeat_exactly(built, mode):
    """The frame is a fixed launch sequence: both recorded frames are equal
    op for op (kernels, shapes, streams, scalar arguments, every pointer),
    so replaying one frame K times is the reference's K frames."""
    seg = T.segments(T.read(os.path.join(built, mode + ".tape")))
    assert len(seg["frames"]) == 2
    assert [_shape(o) for o in seg["frames"][0]] == [_shape(o) for o in seg["frames"][1]]


def test_frame_follows_the_reference_call_order(built):
    """main.cu:175-208: two grid builds (cell ids, stable sort, ranges), the
    vein springs, centroids and springs per type, particle collisions per
    type, vein collisions per type, the two integrations."""
    names = kernel_names(built)
    seg = T.segments(T.read(os.path.join(built, "reference.tape")))
    seq = []
    for op in seg["frames"][0]:
        if op["op"] == "launch":
            n = names[op["kernel"]]
            for tag in ("calculateCellIdKernel", "calculateStartAndEndOfCellKernel", "calculateBloodCellsCenters",
                        "gatherForcesKernelILi", "gatherForcesKerneliii13VeinTriangles",
                        "calculateParticleCollisions", "detectVeinCollisions", "propagateParticleForcesKernel",
                        "propagateForcesIntoPositionsKernel"):
                if tag in n:
                    seq.append(tag)
                    break
            else:
                seq.append(n)
        elif op["op"] == "sort":
            seq.append("sort")
    assert seq == ["calculateCellIdKernel", "sort", "calculateStartAndEndOfCellKernel",
                   "calculateCellIdKernel", "sort", "calculateStartAndEndOfCellKernel",
                   "gatherForcesKerneliii13VeinTriangles", "calculateBloodCellsCenters", "gatherForcesKernelILi",
                   "calculateParticleCollisions", "detectVeinCollisions", "propagateParticleForcesKernel",
                   "propagateForcesIntoPositionsKernel"]


def test_pinned_tape_adds_only_the_q5_ops(built):
    ref = [o for o in T.read(os.path.join(built, "reference.tape")) if o["op"] not in ("memset", "fix_last_cell")]
    pin = [o for o in T.read(os.path.join(built, "pinned.tape")) if o["op"] not in ("memset", "fix_last_cell")]
    assert [_shape(o) for o in ref] == [_shape(o) for o in pin]
    seg = T.segments(T.read(os.path.join(built, "pinned.tape")))
    assert sum(o["op"] == "fix_last_cell" for o in seg["frames"][0]) == 2


def test_every_launch_is_safe_to_replay(built):
    """Each kernel has one cubin entry; every device pointer inside an
    argument lies in an allocation made before the launch; no argument word
    looks like a host address; launch shapes are legal."""
    names = kernel_names(built)
    entries = set(open(os.path.join(built, "entries.txt")).read().split())
    for mode in ("reference", "pinned"):
        allocs = {}
        for op in T.read(os.path.join(built, mode + ".tape")):
            if op["op"] == "alloc":
                allocs[op["id"]] = op["bytes"]
            if op["op"] != "launch":
                continue
            assert names[op["kernel"]] in entries
            threads = op["block"][0] * op["block"][1] * op["block"][2]
            assert 0 < threads <= 1024 and min(op["grid"]) > 0 and op["shmem"] == 0
            for p in op["params"]:
                rel = {r["offset"] for r in p["relocs"]}
                for r in p["relocs"]:
                    assert r["id"] in allocs and r["off"] <= allocs[r["id"]]
                    assert r["offset"] % 8 == 0 and r["offset"] + 8 <= len(p["bytes"])
                for off in range(0, len(p["bytes"]) - 7, 8):
                    if off in rel:
                        continue
                    w = struct.unpack_from("<Q", p["bytes"], off)[0]
                    assert not (0x550000000000 <= w < 0x800000000000), "host address in a kernel argument"


def test_cell_id_arguments(built):
    """calculateCellIdKernel(x, y, z, cellIds, particleIds, count, cellWidth,
    cellHeight, cellDepth) of the particle grid: five device pointers, then
    the particle count and the integer cell sizes (uniform_grid.cu:38-39)."""
    names = kernel_names(built)
    seg = T.segments(T.read(os.path.join(built, "reference.tape")))
    op = next(o for o in seg["frames"][0] if o["op"] == "launch")
    assert "calculateCellIdKernel" in names[op["kernel"]]
    assert [len(p["relocs"]) for p in op["params"]] == [1, 1, 1, 1, 1, 0, 0, 0, 0]
    ints = [struct.unpack("<i", p["bytes"])[0] for p in op["params"][5:]]
    assert ints == [16 * 42, 1, 1, 1]


def test_state_buffers_are_marked(built):
    ops = T.read(os.path.join(built, "reference.tape"))
    bufs = {o["name"]: o["bytes"] for o in ops if o["op"] == "buffer"}
    for q in ("positions", "velocities", "forces"):
        for c in "xyz":
            assert bufs[f"{q}.{c}"] == 4 * 16 * 42


def test_replay_builds_for_sm_103a(tmp_path):
    exe = B.build_replay(str(tmp_path / "ref_cuda_replay"))
    assert os.path.getsize(exe) > 0


def test_cpu_replay_of_the_pinned_tape_is_the_pin(built, tmp_path):
    """The recorder runs its own tape on the CPU (every launch through its
    recorded argument bytes and relocations, the sort op, the Q5 ops, the
    injected state): one frame and five frames equal the CPU pin of the same
    scene bit for bit (tests/golden/ref_pin_icosphere_cfg1.npz).  The GPU
    replay issues the same bytes with cuLaunchKernel."""
    import numpy as np
    g = np.load(os.path.join(REPO, "tests", "golden", "ref_pin_icosphere_cfg1.npz"))
    state = tmp_path / "state.bin"
    np.concatenate([g["init_positions"].ravel(), g["init_velocities"].ravel()]).astype(np.float32).tofile(state)
    for frames, tag in ((1, "frame1"), (int(g["steps"]), "frameN")):
        out = tmp_path / f"out{frames}.bin"
        r = subprocess.run([os.path.join(built, "tape_recorder"), "--replay-cpu", os.path.join(built, "pinned.tape"),
                            str(state), str(frames), str(out)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        o = np.fromfile(out, np.float32).reshape(3, -1, 3)
        for q, name in enumerate(("positions", "velocities", "forces")):
            np.testing.assert_array_equal(o[q], g[f"{tag}_{name}"], err_msg=f"{tag} {name}")


def test_cpu_replay_of_the_reference_tape_runs(built, tmp_path):
    """The timing tape (the reference's calls without the pin's Q5 ops) runs
    to the end with finite state."""
    import numpy as np
    g = np.load(os.path.join(REPO, "tests", "golden", "ref_pin_icosphere_cfg1.npz"))
    state = tmp_path / "state.bin"
    np.concatenate([g["init_positions"].ravel(), g["init_velocities"].ravel()]).astype(np.float32).tofile(state)
    out = tmp_path / "out.bin"
    r = subprocess.run([os.path.join(built, "tape_recorder"), "--replay-cpu", os.path.join(built, "reference.tape"),
                        str(state), "3", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    o = np.fromfile(out, np.float32)
    assert o.size == 9 * 16 * 42 and np.isfinite(o).all()


def _replay_cpu(d, mode, scene, frames, tmp_path):
    """CPU replay of a scene's tape from its own state, returned in the
    scene's particle order."""
    import numpy as np
    order = B.reference_order(scene, B.tape_layout(os.path.join(d, mode + ".tape")))
    state = tmp_path / "state.bin"
    np.concatenate([scene.positions[order].ravel(), scene.velocities[order].ravel()]).astype(np.float32).tofile(state)
    out = tmp_path / "out.bin"
    r = subprocess.run([os.path.join(d, "tape_recorder"), "--replay-cpu", os.path.join(d, mode + ".tape"), str(state),
                        str(frames), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    got = np.fromfile(out, np.float32).reshape(3, -1, 3)
    back = np.empty_like(got)
    back[:, order] = got
    return back


def test_two_models_against_the_oracle(tmp_path):
    """Both cell models of the benchmark (42 and 162 particles).  The
    reference folds them into its own type order (162 first), so the state
    goes in through reference_order().  Its kernels, replayed on the CPU from
    the pinned tape, agree with the FP64 oracle in reference order (the Q1
    radius of the launching type, the Q3 serial force reads): 1e-5 relative
    after one frame; after five, positions to 1e-6 and velocities and forces
    to 5e-4 (FP32 against FP64 through the contact force, which amplifies
    relative velocity, Q14; measured 1.2e-4)."""
    import numpy as np
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    tag, make = next((t, s) for t, s in B.scenes() if t == "two_types")
    d = B.build(tag, make)
    scene = make()
    layout = B.tape_layout(os.path.join(d, "pinned.tape"))
    assert [(p, c) for p, c, _ in layout] == [(162, 12), (42, 12)]

    def rel(a, b):
        b = np.asarray(b, np.float64)
        return float(np.max(np.abs(np.asarray(a, np.float64) - b) / (np.abs(b) + np.sqrt(np.mean(b * b)) + 1e-30)))
    for frames, tols in ((1, (1e-5, 1e-5, 1e-5)), (5, (1e-6, 5e-4, 5e-4))):
        got = _replay_cpu(d, "pinned", scene, frames, tmp_path)
        o = O.OracleSim(scene)
        o.set_reference_order()
        o.step(frames)
        for q, (name, want, tol) in enumerate(zip(("positions", "velocities", "forces"), o.get_particles(), tols)):
            e = rel(got[q], want)
            assert e <= tol, f"{frames} frames, {name}: relative error {e:.3e}"
