#!/usr/bin/env python
"""Benchmark of the plain blood-cell step on one GB300.

Workload (the metric's 4.2M-particle case): a Y bifurcation (trunk R=40,
branches R=28), 20 588 icosphere-42 cells (R=3) + 20 588 biconcave-162 cells
(R=4) = 4 199 952 particles, deformable spring wall, Poiseuille axial force,
Gaussian initial velocities (sigma 0.01), dt=5e-4, grid cell 1.0, triangle
cell 6.0.  A step is one whole frame (grid sort, vein springs, the fused
particle kernel, vein integration) replayed from a CUDA graph.

  value     particle-steps/s over K steps, state resident in HBM, CUDA events
            on the library's stream (the state, 403 MB of float4 buffers, is
            larger than the 129 MB L2, so no flush is needed between steps)
  e2e       the same metric through the C ABI with host buffers: each step is
            bcs_step(1) + a read of the positions into pinned host memory
            (the renderer's per-frame read, src/main.cu:183-184), issued with
            bcs_get_particles_async into two alternating buffers so that it
            overlaps the next frame; the upload of the state from pinned
            memory opens the timed region and the last read's arrival on the
            host closes it
  roofline  the particle phase (the grid-order collision kernel, the step
            kernel, the vein-end kernel): algorithmic bytes (80 B/particle:
            x, v, F read + written as 3 x 12 B, + 8 B key/id) / its mean
            CUDA-event duration, against the measured HBM copy bandwidth;
            per_kernel gives each kernel's own figure
Each of the three passes (timed run, per-phase events, e2e) starts a fresh
simulation from the same state after the warm-up frames, with the tuning the
autotuner picked in the first, so all three follow the same trajectory.
  cpu_baseline  the FP64 oracle (a C++ restatement of the reference step) on
            the host cores, on a bounded sample of the same workload
  parity    before any timing: the workload's first frame from its initial
            state against the FP64 oracle (grid bit-exact, largest relative
            error of x, v, F and of the wall's x, v)
  reference_cuda  the reference's own CUDA kernels (its sources compiled
            unmodified, its host code replayed from a launch tape) on the same
            GPU, the workload's geometry and population, per-frame CUDA events
  batched_workload  the 64-vessel batched workload (71.8M particles) at full
            size, 20 graph-replayed frames after the warm-up
  scale_workload    the 1M-cell (102M-particle) surrogate workload, shortened
            to two macro steps of each path, with its oracle subset

--impl reference times that CPU implementation alone (the reference has no
CPU path of its own; its CUDA kernels are timed beside the product through
the replay of oracle/ref_cuda, reported as reference_cuda).
Under torchrun each rank advances its own replica (the scene does not shard
without a halo exchange): value = all ranks' particle-steps / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "simulation-server_gb300"))

METRIC = "particle-steps/s @4.2M particles: plain vs learned-substep at fixed error"
UNIT = "particle-steps/s"
CELLS_PER_TYPE = 20588
ALGO_BYTES_STEP_KERNEL = 80      # per particle, see docstring
# grid-order collisions: sorted position and velocity read (24 B), key and
# id (8 B), the sum written (12 B); the step kernel reads that sum (12 B)
COLLIDE_BYTES = 44
STEP_COLL_BYTES = 12
COLLIDE_KERNELS = {1: "bcs::k_collide<0>", 2: "bcs::k_collide<1>", 3: "bcs::k_collide_tile"}
FALLBACK_HBM_GBS = 6800.0


def measured_peak():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float) -> float:
    """The largest of every rank's x (the slowest rank's time); x itself on
    one rank.  Works with the process group's backend (NCCL on GPUs, gloo
    on CPUs)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(particles_per_rank: int, steps: int, ms_per_rank: float, world: int) -> float:
    """particle-steps/s of the whole job: every rank's particle-steps over
    the slowest rank's time (weak scaling, one replica per rank)."""
    ms = max_over_ranks(ms_per_rank)
    return world * particles_per_rank * steps / (ms / 1e3)


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu_id: str):
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", gpu_id], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, mx, reasons = [], [], set()
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(self.NAMES, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def build_scene(cells_per_type, seed, widen=1.0):
    """The Y bifurcation (radii 40 and 28) with `cells_per_type` cells of each
    type; widen > 1 scales the radii and the wall's resolution around them
    (a shorter vessel for the same cells, so that the grid at cell 1.0 stays
    inside the 31-bit key space: 100k cells need widen 1.5)."""
    import bcs_scenes as S
    if widen != 1.0:
        return S.scale_scene(2 * cells_per_type, seed=seed, widen=widen)
    return S.bifurcation_scene(cells_per_type=cells_per_type, seed=seed)


def build_batch(args):
    import bcs_scenes as S
    return S.batched_scenes(args.batch_scenes, seed=args.seed)


def batch_config(scenes, n_gpus):
    cells = [int(sum(t.count for t in sc.types)) for sc in scenes]
    return {
        "workload": f"batched plain step, {len(scenes)} straight vessels in one simulation, "
                    f"{sum(len(sc.positions) for sc in scenes)} particles",
        "scenes": len(scenes),
        "particles": int(sum(len(sc.positions) for sc in scenes)),
        "cells": int(sum(cells)), "cells_per_scene_min": min(cells), "cells_per_scene_max": max(cells),
        "lengths": "U[150, 600]", "cell_mix": "Bernoulli(0.5) icosphere-42 / biconcave-162",
        "triangles": int(sum(len(sc.vein_indices) for sc in scenes)),
        "dt": round(float(scenes[0].params.dt), 8), "grid_cell": float(scenes[0].params.cell_width),
        "l2": "state exceeds the 129 MB L2; no flush", "parallelism": f"replicas x{n_gpus}",
    }


def workload_config(scene, n_gpus):
    if isinstance(scene, list):
        return batch_config(scene, n_gpus)
    p = scene.params
    return {
        "workload": f"plain step, Y bifurcation, {scene.particle_count} particles "
                    f"({scene.types[0].count} icosphere-42 + {scene.types[1].count} biconcave-162 cells)",
        "particles": scene.particle_count,
        "cells": int(sum(t.count for t in scene.types)),
        "vein_vertices": int(len(scene.vein_positions)),
        "triangles": int(len(scene.vein_indices)),
        "dt": round(float(p.dt), 8),
        "grid_cell": float(p.cell_width),
        "triangle_cell": float(p.cell_width_triangles),
        "trunk_radius": float(p.cylinder_radius),
        "l2": f"state (6 x float4 x N = {96 * scene.particle_count / 1e6:.0f} MB) exceeds the 129 MB L2; no flush",
        "parallelism": f"replicas x{n_gpus}",
    }


def sample_scene(scene, fraction):
    """The first `fraction` of each type's cells: cells are numbered along
    the flow, so this is the inflow end of the vessel at full density."""
    import copy
    sub = copy.copy(scene)
    types, pos, vel = [], [], []
    start = 0
    for t in scene.types:
        pic = len(t.vertices)
        keep = max(1, int(round(t.count * fraction)))
        types.append(copy.copy(t))
        types[-1].count = keep
        pos.append(scene.positions[start:start + keep * pic])
        vel.append(scene.velocities[start:start + keep * pic])
        start += t.count * pic
    sub.types = types
    sub.positions = np.concatenate(pos)
    sub.velocities = np.concatenate(vel)
    return sub


def time_oracle(scene, steps_budget_s, warmup=1, max_steps=None, threads=None):
    """FP64 oracle on a bounded sample: returns (particle-steps/s, info)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    threads = threads or os.cpu_count() or 1
    # calibrate on 1/32 of the scene, then size the sample to the budget
    cal = sample_scene(scene, 1 / 32)
    oc = O.OracleSim(cal, threads=threads)
    oc.step(1)
    t0 = time.perf_counter()
    oc.step(1)
    per_particle = (time.perf_counter() - t0) / cal.particle_count
    oc.close()
    steps = max_steps or 3
    frac = min(1.0, steps_budget_s / max(1e-9, per_particle * scene.particle_count * (steps + warmup)))
    sample = scene if frac >= 1.0 else sample_scene(scene, frac)
    o = O.OracleSim(sample, threads=threads)
    o.step(warmup)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    n = sample.particle_count
    info = {"steps": steps, "particles": n, "seconds": round(dt, 3)}
    return n * steps / dt, info, threads


def rel_err(g, o):
    """max |g - o| / (|o| + rms(o)) elementwise: the parity tests' rule."""
    o = np.asarray(o, np.float64)
    scale = np.abs(o) + np.sqrt(np.mean(o * o)) + 1e-30
    return float(np.max(np.abs(np.asarray(g, np.float64) - o) / scale))


def oracle_parity(bcs, scene, threads=None):
    """The timed workload's first frame on the GPU against the FP64 oracle
    from the same initial state: particle grid (keys and sorted ids)
    bit-exact, then the largest elementwise relative error of the particles'
    x, v, F and the wall's x, v after one frame (the parity tests' bound is
    1e-5).  The oracle is the checker here, outside every timed region."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    t0 = time.perf_counter()
    threads = threads or os.cpu_count() or 1
    o = O.OracleSim(scene, threads=threads)
    o.calculate_grids()
    ok, oi, _, _ = o.get_grid(0, dense=False)
    sim = bcs.Simulation(scene)
    sim.set_particles(scene.positions, scene.velocities)
    sim.calculate_grids()
    k, i, _, _ = sim.get_grid(0, dense=False)
    sim.close()
    grid_exact = bool(np.array_equal(k, ok) and np.array_equal(i, oi))
    del k, i, ok, oi
    o.close()
    o = O.OracleSim(scene, threads=threads)
    o.step(1)
    sim = bcs.Simulation(scene)
    sim.set_particles(scene.positions, scene.velocities)
    sim.step(1)
    errs = {name: rel_err(a, b) for name, a, b in zip(("position", "velocity", "force"), sim.get_particles(),
                                                       o.get_particles())}
    gv, ov = sim.get_vein(), o.get_vein()
    errs["wall_position"] = rel_err(gv[0], ov[0])
    # A wall velocity after one frame is dt x (spring forces at rest length +
    # particle impacts); at rest length a spring force is FP32 rounding of
    # |p - q| - L, at most k_vein L 2^-23 for each of a vertex's nine springs:
    # the elementwise rule plus that floor, 9 dt k_vein L_max 2^-23 (the
    # benchmark-configuration parity tests' rule).
    tri = np.asarray(scene.vein_indices).reshape(-1, 3)
    vp = np.asarray(scene.vein_positions)
    edge = max(np.linalg.norm(vp[tri[:, i]] - vp[tri[:, k]], axis=1).max() for i, k in ((0, 1), (1, 2), (2, 0)))
    p = scene.params
    floor = float(9 * p.dt * p.vein_k_sniff * edge * 2.0 ** -23)
    o1 = np.asarray(ov[1], np.float64)
    excess = float((np.abs(np.asarray(gv[1], np.float64) - o1) -
                    (1e-5 * (np.abs(o1) + np.sqrt(np.mean(o1 * o1))) + floor)).max())
    sim.close()
    o.close()
    return {"frames": 1, "from": "the workload's initial state", "grid_bit_exact": grid_exact,
            "max_rel_err": errs, "tolerance": 1e-5,
            "wall_velocity": {"excess_over_bound": excess, "floor": floor,
                              "rule": "|dv| <= 1e-5 (|v| + rms v) + 9 dt k_vein L_max 2^-23"},
            "within_tolerance": grid_exact and max(errs.values()) <= 1e-5 and excess <= 0,
            "oracle_threads": threads, "seconds": round(time.perf_counter() - t0, 2)}


def reference_cuda(scene, steps, warmup):
    """The reference's own CUDA kernels on this GPU: its simulation sources
    compiled unmodified into a cubin and its host code recorded as a launch
    tape (oracle/ref_cuda), replayed for warm-up + steps frames from the
    workload's initial state.  The recorded scene has the workload's
    geometry and population with the reference's own physics (its config
    has neither per-particle collision radii nor axial flow segments: the
    bounding-sphere radii and the constant force apply, no vein-end rule).
    Every frame is timed with its own CUDA events; the replay's box check
    runs between frames, untimed.  Returns ms per frame over the frames after
    the warm-up."""
    d = os.path.join(REPO, "oracle", "_ref", "refcuda_bifurcation_4.2M")
    exe = os.path.join(REPO, "oracle", "_ref", "ref_cuda_replay")
    for need in (exe, os.path.join(d, "kernels.cubin"), os.path.join(d, "reference.tape")):
        if not os.path.exists(need):
            return {"unavailable": f"{os.path.relpath(need, REPO)} is not built"}
    sys.path.insert(0, os.path.join(REPO, "oracle", "ref_cuda"))
    import build_ref_cuda as B
    order = B.reference_order(scene, B.tape_layout(os.path.join(d, "reference.tape")))
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        state = os.path.join(tmp, "state.bin")
        np.concatenate([scene.positions[order].ravel(), scene.velocities[order].ravel()]).astype(
            np.float32).tofile(state)
        r = subprocess.run([exe, d, "reference", state, str(warmup + steps)], capture_output=True, text=True,
                           timeout=900)
    if r.returncode != 0:
        return {"unavailable": "replay failed: " + r.stderr.strip()[-300:]}
    line = json.loads(r.stdout.strip().splitlines()[-1])
    timed = line["ms_frames"][warmup:]
    if not timed:
        return {"unavailable": f"the replay stopped after {line['frames']} frames (a particle left the guarded box)"}
    ms = float(np.mean(timed))
    return {"kind": "reference cubin + launch tape", "ms_per_step": ms,
            "value": scene.particle_count * 1e3 / ms, "unit": UNIT, "frames": len(timed), "warmup": warmup,
            "frames_run": line["frames"], "frames_requested": line["frames_requested"],
            "launches_per_frame": line["launches_per_frame"],
            "physics": "the workload's geometry and population with the reference's own constants "
                       "(bounding-sphere radii, constant G, no vein-end rule)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    scene = build_scene(args.cells_per_type, args.seed)
    budget = float(os.environ.get("BCS_REFERENCE_BUDGET_S", "150"))
    # the whole K-step run is sized to the budget: every step is one oracle
    # step of a sample of the workload
    value, info, threads = time_oracle(scene, budget, warmup=max(0, args.warmup), max_steps=args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * info["seconds"] / max(1, info["steps"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(scene, ws),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{info['particles']} particles (inflow end of the same vessel) x "
                                   f"{info['steps']} steps, FP64 oracle, {threads} OpenMP threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def grid_diagnostics(sim):
    """Occupancy of the particle grid, where its most crowded cell lies,
    particles outside the grid box, speeds, and the error word after a run."""
    keys, ids, _, _ = sim.get_grid(0, dense=False)
    if len(keys) == 0:
        return {}
    change = np.flatnonzero(np.diff(keys)) + 1
    starts = np.concatenate([[0], change])
    runs = np.diff(np.concatenate([starts, [len(keys)]]))
    pos, vel, _ = sim.get_particles()
    info = sim.info
    lo = np.array([info.min_x, info.min_y, info.min_z], np.float32)
    hi = np.array([info.max_x, info.max_y, info.max_z], np.float32)
    outside = ~np.all((pos >= lo) & (pos <= hi), axis=1)
    k = int(np.argmax(runs))
    crowded = pos[ids[starts[k]:starts[k] + runs[k]]]
    speed = np.linalg.norm(vel, axis=1)
    return {"occupied_cells": int(len(runs)), "max_particles_per_cell": int(runs.max()),
            "mean_particles_per_occupied_cell": round(float(runs.mean()), 3),
            "cells_with_over_8_particles": int((runs > 8).sum()),
            "most_crowded_cell_centre": [round(float(v), 2) for v in crowded.mean(0)],
            "particles_outside_grid_box": int(outside.sum()),
            "speed_median": round(float(np.median(speed)), 3), "speed_max": round(float(speed.max()), 3),
            "error_word": sim.error_word()}


def learned_substep(args, scene, tuning, bcs, fresh, warm):
    """The learned sub-step path at the same workload.  The network (for the
    162-vertex cells) is trained on plain macro steps of a scene built from
    a fresh seed; then plain frames, plain macro steps (K sub-steps, the
    collisions held) and macro steps with the network are timed from the
    same state, and their positions compared with the plain frames' (the
    reference for the errors).  Simulated-time throughput = particles x
    sub-steps / time."""
    K, M = args.learned_substeps, args.learned_macro_steps
    params, scales, training = train_network(args, args.cells_per_type, tuning, bcs, warm)

    # local error: one macro step against K plain frames from the same state
    sim = fresh(tuning)
    n = sim.n
    sim.step(K)
    pa1 = sim.get_particles()[0].astype(np.float64)
    sim.close()
    sim = fresh(tuning)
    sim.macro_step(K, 1)
    pb1 = sim.get_particles()[0]
    sim.close()
    sim = fresh(tuning)
    s1 = bcs.Surrogate(sim, cell_type=1, substeps=K, max_samples=1, seed=11)
    s1.set_params(params)
    s1.set_scales(scales)
    s1.enable(True)
    sim.macro_step(K, 1)
    pc1 = sim.get_particles()[0]
    s1.close()
    sim.close()

    sim = fresh(tuning)
    ms_plain = sim.time_steps(K * M)
    pa = sim.get_particles()[0]
    sim.close()
    def timed(sim):
        """M macro steps, each timed alone (CUDA events, graph replay)."""
        per = [sim.time_macro_steps(K, 1) for _ in range(M)]
        return float(sum(per)), {f"p{q}": float(np.percentile(per, q)) for q in (50, 95, 99)}

    sim = fresh(tuning)
    ms_macro, lat_macro = timed(sim)
    pb = sim.get_particles()[0]
    sim.close()
    sim = fresh(tuning)
    s2 = bcs.Surrogate(sim, cell_type=1, substeps=K, max_samples=1, seed=11)
    s2.set_params(params)
    s2.set_scales(scales)
    s2.enable(True)
    ms_sur, lat_sur = timed(sim)
    pc = sim.get_particles()[0]
    st = s2.stats()
    s2.close()
    sim.close()

    def err(p, ref=None):
        d = np.linalg.norm(p.astype(np.float64) - (pa if ref is None else ref), axis=1)
        return {"median": float(np.median(d)), "p99": float(np.percentile(d, 99)), "max": float(d.max()),
                "frac_above_1e-3_radius": float(np.mean(d > 1e-3 * 0.5))}

    # a seeded subset of the same state against the FP64 oracle
    subset = None
    if args.learned_oracle_cells > 0:
        subset = oracle_subset(args, scene, tuning, bcs, params, scales, warm, args.learned_oracle_macro_steps,
                               args.learned_oracle_cells, args.seed + 1)

    rate = lambda ms: n * K * M / (ms / 1e3)
    return {
        "_params": params, "_scales": scales,
        "substeps": K, "macro_steps": M, "simulated_time": K * M * float(scene.params.dt),
        "plain": {"ms": ms_plain, "particle_steps_per_s": rate(ms_plain)},
        "macro_plain": {"ms": ms_macro, "particle_steps_per_s": rate(ms_macro), "position_error": err(pb),
                        "one_macro_step_error": err(pb1, pa1), "macro_step_latency_ms": lat_macro},
        "surrogate": {"ms": ms_sur, "particle_steps_per_s": rate(ms_sur), "position_error": err(pc),
                      "macro_step_latency_ms": lat_sur,
                      "one_macro_step_error": err(pc1, pa1),
                      "cells_predicted": st["predicted_cells"], "cells_fallen_back": st["fallback_cells"],
                      "tolerance": st["tolerance"]},
        "speedup_vs_plain": {"macro_plain": ms_plain / ms_macro, "surrogate": ms_plain / ms_sur},
        "network": dict(training, parameters=st["parameters"], flops_per_cell=st["flops_per_cell"]),
        "error_reference": "positions after the same simulated time, against plain frames from the same state",
        "oracle_subset": subset,
    }


def train_network(args, cells_per_type, tuning, bcs, warm):
    """Trains the network for the 162-vertex cells on plain macro steps of a
    bifurcation scene of `cells_per_type` cells per type built from a fresh
    seed; returns (parameters, scales, description)."""
    K = args.learned_substeps
    t0 = time.perf_counter()
    train_scene = build_scene(cells_per_type, args.seed + 7919)
    ts = bcs.Simulation(train_scene)
    ts.set_particles(train_scene.positions, train_scene.velocities)
    ts.set_tuning(**tuning)
    ts.step(warm)
    cells = train_scene.types[1].count
    sur = bcs.Surrogate(ts, cell_type=1, substeps=K, max_samples=cells * (args.learned_collect + 1), seed=11,
                        huber_delta=1.0)
    sur.collect(args.learned_collect)
    n_train = sur.stats()["samples"]
    loss0 = sur.train(1, batch_cells=args.learned_batch, lr=1e-3)
    # learning rate 1e-3 decayed by 10 x over four phases
    loss = loss0
    for phase in range(4):
        loss = sur.train(args.learned_iters // 4, batch_cells=args.learned_batch, lr=1e-3 * 10 ** (-phase / 3))
    sur.collect(1)
    net_err, base_err = sur.evaluate(n_train, sur.stats()["samples"] - n_train)
    params, scales, st_train = sur.get_params(), sur.scales(), sur.stats()
    sur.close()
    ts.close()
    desc = {"cell_type": "biconcave-162", "layers": 3, "hidden": 128,
            "training": {"scene": f"Y bifurcation, {cells_per_type} cells per type", "scene_seed": args.seed + 7919,
                         "cell_steps": n_train, "iterations": st_train["iterations"],
                         "batch_cells": args.learned_batch, "loss": "pseudo-Huber, delta 1 (normalised)",
                         "loss_first": loss0, "loss_last": loss, "seconds": round(time.perf_counter() - t0, 2)},
            "held_out_position_error": {"network": net_err, "constant_force_extrapolation": base_err}}
    return params, scales, desc


def position_error(p, ref, radius=0.5):
    d = np.linalg.norm(np.asarray(p, np.float64) - np.asarray(ref, np.float64), axis=1)
    return {"median": float(np.median(d)), "p99": float(np.percentile(d, 99)), "max": float(d.max()),
            "frac_above_1e-3_radius": float(np.mean(d > 1e-3 * radius))}


def oracle_subset(args, scene, tuning, bcs, params, scales, warm, macro_steps, cells, seed):
    """A seeded subset of `cells` cells of `scene` (same vessel, constants and
    state) advanced by `warm` frames and `macro_steps` x K sub-steps on the
    FP64 oracle (the host cores) and on the GPU as plain frames, plain macro
    steps and macro steps with the network; each GPU path's positions against
    the oracle's."""
    import bcs_scenes as S
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    K = args.learned_substeps
    sub = S.subset_scene(scene, cells, seed=seed)
    t1 = time.perf_counter()
    o = O.OracleSim(sub, threads=os.cpu_count())
    o.step(warm + K * macro_steps)
    po = o.get_particles()[0]
    o.close()
    oracle_s = time.perf_counter() - t1

    def fresh_sub():
        sim = bcs.Simulation(sub)
        sim.set_particles(sub.positions, sub.velocities)
        sim.set_tuning(**tuning)
        sim.step(warm)
        return sim
    s1 = fresh_sub()
    s1.step(K * macro_steps)
    g_plain = s1.get_particles()[0]
    s1.close()
    s1 = fresh_sub()
    s1.macro_step(K, macro_steps)
    g_macro = s1.get_particles()[0]
    s1.close()
    s1 = fresh_sub()
    z = bcs.Surrogate(s1, cell_type=1, substeps=K, max_samples=1, seed=11)
    z.set_params(params)
    z.set_scales(scales)
    z.enable(True)
    s1.macro_step(K, macro_steps)
    g_sur = s1.get_particles()[0]
    zst = z.stats()
    z.close()
    s1.close()
    return {"cells": int(sum(t.count for t in sub.types)), "particles": sub.particle_count, "seed": seed,
            "frames": warm + K * macro_steps, "oracle_seconds": round(oracle_s, 2),
            "oracle_threads": os.cpu_count(),
            "plain_vs_oracle": position_error(g_plain, po),
            "macro_plain_vs_oracle": position_error(g_macro, po),
            "surrogate_vs_oracle": position_error(g_sur, po),
            "surrogate_cells_predicted": zst["predicted_cells"],
            "surrogate_cells_fallen_back": zst["fallback_cells"]}


def percentiles(per):
    return {f"p{q}": float(np.percentile(per, q)) for q in (50, 95, 99)}


def batched_summary(args, tuning, bcs, frames, warm):
    """The batched workload at its full size inside the default run: the 64
    seeded straight vessels (71.8M particles) in one simulation, `warm`
    frames, then `frames` graph-replayed frames timed with CUDA events.  The
    tuning is the one the autotuner picked for the bifurcation workload (the
    batched workload's own autotuning picks the same launch shape and
    collision kernel); `--workload batched` runs the full measurement."""
    t0 = time.perf_counter()
    scenes = build_batch(args)
    build_s = time.perf_counter() - t0
    sim = bcs.Simulation(scenes)
    sim.set_particles(np.concatenate([sc.positions for sc in scenes]),
                      np.concatenate([sc.velocities for sc in scenes]))
    sim.set_tuning(**tuning)
    sim.step(warm)
    ms = sim.time_steps(frames)
    n = sim.n
    errw = sim.error_word()
    sim.close()
    names = [nm for bit, nm in ((1, "a position outside the grid box"),
                                (2, "a zero vector normalised (a particle at rest meets the vein ray, "
                                    "as in the reference, whose normalize gives NaN there)"),
                                (4, "a non-finite position or velocity")) if errw & bit]
    return {"frames": frames, "warmup": warm, "ms_per_step": ms / frames,
            "particle_steps_per_s": n * frames / (ms / 1e3), "unit": UNIT, "error_word": errw,
            "error_word_bits": names,
            "tuning": tuning, "tuning_source": "the bifurcation workload's autotuned setting",
            "scene_build_seconds": round(build_s, 1), "config": batch_config(scenes, 1)}


def scale_summary(args, tuning, bcs, params, scales, macro_steps, warm):
    """The surrogate-at-scale workload inside the default run, shortened: 1M
    cells (102M particles) in the 6x widened bifurcation; plain frames, plain
    macro steps and macro steps with the network (the one trained for the
    bifurcation workload) advance `macro_steps` x K sub-steps from the same
    state, each frame or macro step timed alone; the seeded 1k-cell subset
    is checked against the FP64 oracle.  `--workload scale` runs the full
    measurement (125 macro steps)."""
    import bcs_scenes as S
    K = args.learned_substeps
    t0 = time.perf_counter()
    scene = S.scale_scene(args.scale_cells, seed=args.seed)
    build_s = time.perf_counter() - t0

    def fresh():
        sim = bcs.Simulation(scene)
        sim.set_particles(scene.positions, scene.velocities)
        sim.set_tuning(**tuning)
        sim.step(warm)
        return sim

    sim = fresh()
    n = sim.n
    per_frame = [sim.time_steps(1) for _ in range(K * macro_steps)]
    pa = sim.get_particles()[0]
    sim.close()
    sim = fresh()
    per_macro = [sim.time_macro_steps(K, 1) for _ in range(macro_steps)]
    pb = sim.get_particles()[0]
    sim.close()
    sim = fresh()
    sur = bcs.Surrogate(sim, cell_type=1, substeps=K, max_samples=1, seed=11)
    sur.set_params(params)
    sur.set_scales(scales)
    sur.enable(True)
    per_sur = [sim.time_macro_steps(K, 1) for _ in range(macro_steps)]
    pc = sim.get_particles()[0]
    st = sur.stats()
    sur.close()
    sim.close()
    ms_plain, ms_macro, ms_sur = float(sum(per_frame)), float(sum(per_macro)), float(sum(per_sur))
    rate = lambda ms: n * K * macro_steps / (ms / 1e3)
    subset = oracle_subset(args, scene, tuning, bcs, params, scales, warm, args.scale_subset_macro_steps,
                           args.scale_subset_cells, args.seed + 1)
    return {
        "substeps": K, "macro_steps": macro_steps, "plain_equivalent_steps": K * macro_steps, "warmup": warm,
        "plain": {"ms": ms_plain, "particle_steps_per_s": rate(ms_plain),
                  "frame_latency_ms": percentiles(per_frame)},
        "macro_plain": {"ms": ms_macro, "particle_steps_per_s": rate(ms_macro),
                        "macro_step_latency_ms": percentiles(per_macro),
                        "position_error_vs_plain_frames": position_error(pb, pa)},
        "surrogate": {"ms": ms_sur, "particle_steps_per_s": rate(ms_sur),
                      "macro_step_latency_ms": percentiles(per_sur),
                      "position_error_vs_plain_frames": position_error(pc, pa),
                      "cells_predicted": st["predicted_cells"], "cells_fallen_back": st["fallback_cells"]},
        "speedup_vs_plain": {"macro_plain": ms_plain / ms_macro, "surrogate": ms_plain / ms_sur},
        "oracle_subset": subset,
        "tuning_source": "the bifurcation workload's autotuned setting",
        "config": dict(workload_config(scene, 1), scene_build_seconds=round(build_s, 1),
                       workload=f"surrogate at scale, widened Y bifurcation, {scene.particle_count} particles "
                                f"({scene.types[0].count} icosphere-42 + {scene.types[1].count} "
                                f"biconcave-162 cells)"),
    }


def run_scale(args):
    """Surrogate plus batching at scale: 1M cells (half 42-, half 162-vertex,
    102M particles) in a widened Y bifurcation.  Plain frames, plain macro
    steps and macro steps with the network (trained on the 4.2M-particle
    workload's scene from a fresh seed) advance the same simulated time from
    the same state; every frame and macro step is timed alone for the latency
    percentiles.  Positions are compared with the plain frames on the whole
    scene, and on a seeded 1k-cell subset (in the same vessel) every path is
    compared with the FP64 oracle."""
    import torch
    import bcs_build
    import bcs
    import bcs_scenes as S

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    bcs_build.build()
    bcs.set_device(local)
    K, M = args.learned_substeps, args.scale_macro_steps
    t0 = time.perf_counter()
    scene = S.scale_scene(args.scale_cells, seed=args.seed + rank)
    build_s = time.perf_counter() - t0

    def fresh(sc, tuning=None, warm=args.warmup):
        sim = bcs.Simulation(sc)
        sim.set_particles(sc.positions, sc.velocities)
        if tuning is not None:
            sim.set_tuning(**tuning)
        sim.step(warm)
        return sim

    sim = fresh(scene)
    n = sim.n
    _, tune_ms = sim.autotune(args.autotune_frames)
    tuning = sim.get_tuning().as_dict()
    sim.close()
    params, scales, training = train_network(args, CELLS_PER_TYPE, tuning, bcs, args.warmup)

    def with_network(sim, max_samples=1):
        sur = bcs.Surrogate(sim, cell_type=1, substeps=K, max_samples=max_samples, seed=11)
        sur.set_params(params)
        sur.set_scales(scales)
        sur.enable(True)
        return sur

    props = torch.cuda.get_device_properties(local)
    gpu_id = str(getattr(props, "uuid", "") or local)
    if gpu_id and not gpu_id.startswith("GPU-") and len(gpu_id) > 8:
        gpu_id = "GPU-" + gpu_id
    sampler = ClockSampler(gpu_id)
    sim = fresh(scene, tuning)
    per_frame = [sim.time_steps(1) for _ in range(K * M)]
    pa = sim.get_particles()[0]
    sim.close()
    sim = fresh(scene, tuning)
    per_macro = [sim.time_macro_steps(K, 1) for _ in range(M)]
    pb = sim.get_particles()[0]
    sim.close()
    sim = fresh(scene, tuning)
    sur = with_network(sim)
    per_sur = [sim.time_macro_steps(K, 1) for _ in range(M)]
    pc = sim.get_particles()[0]
    st = sur.stats()
    sur.close()
    sim.close()
    clocks = sampler.stop()
    ms_plain, ms_macro, ms_sur = float(sum(per_frame)), float(sum(per_macro)), float(sum(per_sur))
    rate = lambda ms: n * K * M / (ms / 1e3)

    # the seeded 1k-cell subset against the FP64 oracle
    subset = oracle_subset(args, scene, tuning, bcs, params, scales, args.warmup, args.scale_subset_macro_steps,
                           args.scale_subset_cells, args.seed + 1)

    if rank == 0:
        out = {
            "metric": METRIC, "unit": UNIT, "workload": "scale",
            "scale_surrogate": {
                "substeps": K, "macro_steps": M, "plain_equivalent_steps": K * M,
                "simulated_time": K * M * float(scene.params.dt),
                "plain": {"ms": ms_plain, "particle_steps_per_s": rate(ms_plain),
                          "frame_latency_ms": percentiles(per_frame)},
                "macro_plain": {"ms": ms_macro, "particle_steps_per_s": rate(ms_macro),
                                "macro_step_latency_ms": percentiles(per_macro),
                                "position_error_vs_plain_frames": position_error(pb, pa)},
                "surrogate": {"ms": ms_sur, "particle_steps_per_s": rate(ms_sur),
                              "macro_step_latency_ms": percentiles(per_sur),
                              "position_error_vs_plain_frames": position_error(pc, pa),
                              "cells_predicted": st["predicted_cells"], "cells_fallen_back": st["fallback_cells"],
                              "tolerance": st["tolerance"]},
                "speedup_vs_plain": {"macro_plain": ms_plain / ms_macro, "surrogate": ms_plain / ms_sur},
                "oracle_subset": subset,
                "network": dict(training, parameters=st["parameters"], flops_per_cell=st["flops_per_cell"]),
                "tuning": tuning, "autotune_ms": tune_ms,
            },
            "clocks": clocks,
            "config": dict(workload_config(scene, ws), scene_build_seconds=round(build_s, 1),
                           workload=f"surrogate at scale, widened Y bifurcation, {scene.particle_count} particles "
                                    f"({scene.types[0].count} icosphere-42 + {scene.types[1].count} "
                                    f"biconcave-162 cells)",
                           trunk_radius=float(scene.params.cylinder_radius),
                           l2="state exceeds the 129 MB L2; no flush"),
        }
        print(json.dumps(out), flush=True)
    return 0


def run_ours(args):
    import torch
    import bcs_build
    import bcs

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    bcs_build.build()
    bcs.set_device(local)
    batched = args.workload == "batched"
    scene = build_batch(args) if batched else build_scene(args.cells_per_type, args.seed + rank, args.widen)
    all_pos = np.concatenate([sc.positions for sc in scene]) if batched else scene.positions
    all_vel = np.concatenate([sc.velocities for sc in scene]) if batched else scene.velocities

    def barrier(sim):
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        sim.synchronize()

    def fresh(tuning=None):
        """A new simulation at the state after the warm-up frames: every pass
        below starts from the same state and follows the same trajectory."""
        sim = bcs.Simulation(scene)
        sim.set_particles(all_pos, all_vel)
        if tuning is not None:
            sim.set_tuning(**tuning)
        sim.step(args.warmup)
        return sim

    if args.learned_only:
        # the learned sub-step pass alone (profiling); the plain tuning is the default
        sim = fresh()
        tuning = sim.get_tuning().as_dict()
        sim.close()
        learned = learned_substep(args, scene, tuning, bcs, fresh, args.warmup)
        learned.pop("_params")
        learned.pop("_scales")
        if rank == 0:
            print(json.dumps({"metric": METRIC, "unit": UNIT, "learned_substep": learned,
                              "config": workload_config(scene, ws)}), flush=True)
        return 0

    # ---- parity of the timed workload's first frame against the FP64 oracle
    parity = None
    if rank == 0 and not batched and not args.no_parity:
        parity = oracle_parity(bcs, scene)

    # ---- pass 1: the timed run (graph replay, state resident in HBM)
    sim = fresh()
    n = sim.n
    tuning, tune_ms = None, None
    if args.tuning:
        sim.set_tuning(*[int(v) for v in args.tuning.split(",")])
    elif not args.no_autotune:
        _, tune_ms = sim.autotune(args.autotune_frames)
    tuning = sim.get_tuning().as_dict()
    barrier(sim)
    props = torch.cuda.get_device_properties(local)
    gpu_id = str(getattr(props, "uuid", "") or local)
    if gpu_id and not gpu_id.startswith("GPU-") and len(gpu_id) > 8:
        gpu_id = "GPU-" + gpu_id
    sampler = ClockSampler(gpu_id)
    time.sleep(0.3)
    crowded0 = sim.crowded_particles()
    ms = sim.time_steps(args.steps)
    clocks = sampler.stop()
    barrier(sim)
    crowded_per_frame = (sim.crowded_particles() - crowded0) / args.steps
    ms_max = max_over_ranks(ms)
    value = whole_job_rate(n, args.steps, ms, ws)
    info = sim.refresh_info()
    launches = info.kernels_per_step * args.steps
    diag = grid_diagnostics(sim)
    diag["crowded_particles_per_frame"] = crowded_per_frame
    sim.close()

    # ---- pass 2: the same frames eagerly, CUDA events between the phases;
    # the particle phase is the grid-order collision kernel, the step
    # kernel (with its crowded-particle kernel when the step kernel searches
    # the stencils itself) and the vein-end kernel
    prof_steps = args.profile_steps if args.profile_steps > 0 else args.steps
    sim = fresh(tuning)
    phases = sim.profile_steps(prof_steps)
    sim.close()
    coll_ms = phases["collisions"] / prof_steps
    step_ms = phases["particles"] / prof_steps
    k_ms = coll_ms + step_ms
    peak, peak_kind = measured_peak()
    achieved = ALGO_BYTES_STEP_KERNEL * n / (k_ms / 1e3) / 1e9
    traffic, traffic_note = None, None
    tf = os.path.join(REPO, "profiles", "particle_phase_traffic.json")
    if os.path.exists(tf):
        with open(tf) as f:
            tr = json.load(f)
        traffic = sum(tr["dram_bytes_per_launch"].values()) * n / tr["particles"]
        traffic_note = tr["note"]
    per_kernel = {}
    if coll_ms > 0:
        per_kernel["collisions"] = {"ms": coll_ms, "algorithmic_bytes_per_particle": COLLIDE_BYTES,
                                    "achieved_gbs": COLLIDE_BYTES * n / (coll_ms / 1e3) / 1e9}
        per_kernel["collisions"]["frac"] = per_kernel["collisions"]["achieved_gbs"] / peak
    step_bytes = ALGO_BYTES_STEP_KERNEL + (STEP_COLL_BYTES if coll_ms > 0 else 0)
    per_kernel["step"] = {"ms": step_ms, "algorithmic_bytes_per_particle": step_bytes,
                          "achieved_gbs": step_bytes * n / (step_ms / 1e3) / 1e9}
    per_kernel["step"]["frac"] = per_kernel["step"]["achieved_gbs"] / peak
    # the whole frame against its compulsory traffic: 96 B per particle (x, v,
    # F read and written, key and id written, one sort pass over the pairs),
    # 8 B per occupied grid cell, 72 B per vertex and 24 B per triangle of a
    # deformable wall, over the graph-replayed frame time
    walls = scene if batched else [scene]
    dyn = [sc for sc in walls if int(sc.params.vein_dynamic)]
    wall_bytes = sum(72 * len(sc.vein_positions) + 24 * len(sc.vein_indices) for sc in dyn)
    occupied = diag.get("occupied_cells", 0)
    step_total = 96 * n + 8 * occupied + wall_bytes
    frame_ms = ms_max / args.steps
    whole_step = {"algorithmic_bytes_per_step": int(step_total), "ms": frame_ms,
                  "achieved_gbs": step_total / (frame_ms / 1e3) / 1e9,
                  "terms": {"particles_96B": 96 * n, "occupied_cells_8B": 8 * occupied,
                            "wall_72B_per_vertex_24B_per_triangle": wall_bytes}}
    whole_step["frac"] = whole_step["achieved_gbs"] / peak

    # ---- pass 3: end to end through the C ABI with pinned host buffers:
    # the state after the warm-up is uploaded, then every frame is
    # bcs_step(1) + a read of its positions into host memory, overlapped
    # with the next frame (bcs_get_particles_async into two alternating
    # pinned buffers, as a renderer double-buffers); the timed region ends
    # when the last read has reached the host
    e2e_steps = args.steps if args.e2e_steps <= 0 else max(1, min(args.e2e_steps, args.steps))
    sim = fresh(tuning)
    p0, v0, f0 = sim.get_particles()
    hp = [torch.empty(n, dtype=torch.float32, pin_memory=True) for _ in range(12)]
    for k in range(3):
        hp[k].copy_(torch.from_numpy(np.ascontiguousarray(p0[:, k])))
        hp[3 + k].copy_(torch.from_numpy(np.ascontiguousarray(v0[:, k])))
        hp[6 + k].copy_(torch.from_numpy(np.ascontiguousarray(f0[:, k])))
    lib = bcs.load_library()
    P, Vv, Ff = (bcs.Vec3(*(x.data_ptr() for x in hp[3 * j:3 * j + 3])) for j in range(3))
    outs = [bcs.Vec3(*(x.data_ptr() for x in hp[:3])), bcs.Vec3(*(x.data_ptr() for x in hp[9:12]))]
    barrier(sim)
    t0 = time.perf_counter()
    assert lib.bcs_set_particles(sim.h, P, Vv, Ff, bcs.MEM_HOST) == 0
    for k in range(e2e_steps):
        assert lib.bcs_step(sim.h, 1) == 0
        assert lib.bcs_get_particles_async(sim.h, outs[k & 1], bcs.Vec3(), bcs.Vec3()) == 0
    assert lib.bcs_wait_particles(sim.h) == 0
    e2e_s = time.perf_counter() - t0
    sim.close()
    e2e_value = whole_job_rate(n, e2e_steps, 1e3 * e2e_s, ws)

    learned, params, scales = None, None, None
    if rank == 0 and not args.no_learned and not batched:
        try:
            learned = learned_substep(args, scene, tuning, bcs, fresh, args.warmup)
            params, scales = learned.pop("_params"), learned.pop("_scales")
        except Exception as exc:   # the plain line is still printed
            learned = {"error": f"{type(exc).__name__}: {exc}"}

    # ---- the batched and the at-scale workloads, shortened, on the same GPU
    # (each simulation of the passes above is closed by now)
    batched_line = None
    if rank == 0 and ws == 1 and not batched and not args.no_batched:
        try:
            batched_line = batched_summary(args, tuning, bcs, args.batched_frames, args.warmup)
        except Exception as exc:
            batched_line = {"error": f"{type(exc).__name__}: {exc}"}
    scale_line = None
    if rank == 0 and ws == 1 and not batched and not args.no_scale and params is not None:
        try:
            scale_line = scale_summary(args, tuning, bcs, params, scales, args.scale_summary_macro_steps,
                                       args.warmup)
        except Exception as exc:
            scale_line = {"error": f"{type(exc).__name__}: {exc}"}

    ref_cuda = None
    if rank == 0 and not batched and not args.no_reference_cuda:
        try:
            ref_cuda = reference_cuda(scene, args.steps, args.warmup)
        except Exception as exc:
            ref_cuda = {"unavailable": f"{type(exc).__name__}: {exc}"}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline and not batched:
        v, cinfo, threads = time_oracle(scene, args.cpu_budget, warmup=1, max_steps=3)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{cinfo['particles']} particles (inflow end of the same vessel) x {cinfo['steps']} "
                         f"steps in {cinfo['seconds']} s, FP64 oracle, {threads} OpenMP threads"}
        if threads > 1:
            # the same oracle on one core, a smaller sample of the same scene
            v1, c1, _ = time_oracle(scene, args.cpu_budget / 4, warmup=1, max_steps=2, threads=1)
            cpu["one_core"] = {"value": v1, "unit": UNIT, "cores": 1,
                               "sample": f"{c1['particles']} particles x {c1['steps']} steps in {c1['seconds']} s"}

    if rank == 0:
        shape = bcs.STEP_SHAPES[tuning["step_shape"]]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(workload_config(scene, ws), tuning=tuning,
                           tuning_source="bcs_autotune" if tune_ms is not None else
                           ("--tuning" if args.tuning else "default"),
                           step_shape=dict(zip(("threads", "particles_per_cta", "ctas_per_sm"), shape))),
            "e2e": {"value": e2e_value, "unit": UNIT, "steps": e2e_steps,
                    "h2d_bytes_per_step": int(36 * n / e2e_steps), "d2h_bytes_per_step": int(12 * n)},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm",
                         "kernel": ("{} + ".format(COLLIDE_KERNELS[tuning["grid_collisions"]])
                                    if tuning["grid_collisions"] else "") +
                                   "bcs::k_step<0, {}, {}, {}, {}>".format(
                                       *shape, "true" if tuning["persistent"] else "false") +
                                   (" + k_crowded<0>" if not tuning["grid_collisions"] else "") + " + k_vein_end",
                         "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_note,
                         "algorithmic_bytes_per_launch": ALGO_BYTES_STEP_KERNEL * n, "kernel_ms": k_ms,
                         "kernel_ms_over": f"{prof_steps} eager frames of the same trajectory",
                         "per_kernel": per_kernel, "whole_step": whole_step},
            "phase_ms": {k: v / prof_steps for k, v in phases.items()},
            "diagnostics_after_timed_run": diag,
            "learned_substep": learned,
            "batched_workload": batched_line,
            "scale_workload": scale_line,
            "clocks": clocks,
            "cpu_baseline": cpu,
            "reference_cuda": ref_cuda,
            "parity": parity,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells-per-type", type=int, default=CELLS_PER_TYPE)
    ap.add_argument("--widen", type=float, default=1.0,
                    help="scale the vessel's radii (1.5 keeps 50k cells per type inside the key space)")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--profile-steps", type=int, default=0, help="0 = as many as --steps")
    ap.add_argument("--e2e-steps", type=int, default=0, help="0 = as many as --steps")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the one-frame oracle check of the workload")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="skip the replay of the reference's own kernels")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--autotune-frames", type=int, default=3)
    ap.add_argument("--tuning", default="", help="comma-separated bcs_tuning fields instead of the autotuner")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned sub-step measurements")
    ap.add_argument("--learned-only", action="store_true", help="only the learned sub-step pass (profiling)")
    ap.add_argument("--workload", default="bifurcation", choices=["bifurcation", "batched", "scale"],
                    help="bifurcation: the 4.2M-particle metric workload; batched: 64 straight vessels; "
                         "scale: plain vs learned sub-steps at 1M cells (102M particles)")
    ap.add_argument("--scale-cells", type=int, default=1_000_000)
    ap.add_argument("--scale-macro-steps", type=int, default=125)
    ap.add_argument("--scale-subset-cells", type=int, default=1000)
    ap.add_argument("--scale-subset-macro-steps", type=int, default=4)
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the shortened batched-workload run of the default line")
    ap.add_argument("--batched-frames", type=int, default=20)
    ap.add_argument("--no-scale", action="store_true",
                    help="skip the shortened at-scale surrogate run of the default line")
    ap.add_argument("--scale-summary-macro-steps", type=int, default=2)
    ap.add_argument("--learned-substeps", type=int, default=8)
    ap.add_argument("--learned-macro-steps", type=int, default=40)
    ap.add_argument("--learned-collect", type=int, default=97,
                    help="training macro steps collected (97 x 20 588 disc cells = 2.0M cell-steps)")
    ap.add_argument("--learned-iters", type=int, default=4000)
    ap.add_argument("--learned-oracle-cells", type=int, default=1000,
                    help="cells of the seeded subset checked against the FP64 oracle (0: none)")
    ap.add_argument("--learned-oracle-macro-steps", type=int, default=4)
    ap.add_argument("--learned-batch", type=int, default=256)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "scale":
        return run_scale(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
