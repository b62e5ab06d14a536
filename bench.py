#!/usr/bin/env python3
"""Benchmark: frames/s of the descent time step at relative residual <= 1e-4.

Workload (the 1M-tet roofline configuration): a 50 x 50 x 80 cube box of edge
0.005 m, 5-tet split (1,000,000 tets, 210,681 nodes), interior nodes jittered
+-0.1 cell from the seed, neo-Hookean with E = 10^U(4, 6) Pa drawn from the
seed and Poisson 0.4; the top face (z = max) pinned, the bottom face driven to
1.5x the rest length linearly over 30 steps; gravity; h = 1/30 s; every frame
iterates until |g| <= 1e-4 |g_0| (FP64 norms).  Synthetic data: the mesh is
generated, nothing is downloaded.

A "step" of this benchmark is one frame: the prescribed-boundary upload and
one pbs_step() solve through the C ABI.  Frames 0 .. W-1 are warm-up, frames
W .. W+K-1 are timed (the defaults cover the 30-frame pull).  Two arms run the
same frames on fresh handles: the plain descent, and the descent warm-started
by the learned per-node MLP (phybs_gb300/warmstart_model.npz; the plain guess
is kept whenever the prediction's energy is higher, and every frame still
iterates to the same residual).  ``value`` is the warm-started arm's frames/s
with the state resident in HBM, timed with CUDA events on the library's
stream (the 31 KB boundary upload per frame included); ``plain`` holds the
plain arm's figures and ``speedup_vs_plain`` their ratio.  ``e2e`` reruns the
headline arm through the same calls plus each frame's read-back of all
positions to pinned host memory (pbs_read_positions), on the host clock.

``--impl reference`` times the CPU restatement of the reference's descent
step (DescentOptimize with the benchmark's control, FP64, its per-tet loops
on all host threads) on the same workload: frames 0 .. W-1 untimed, frames
W .. W+K-1 timed whole on the host clock, every frame iterated to the same
residual bar.  The GPU arm's ``cpu_baseline`` times frames W .. W+2 the same
way from the plain GPU arm's state, and ``cpu_force_eval`` the port of the
reference's OpenMP force path (computeInnerForcesfromFhats2).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s at residual<=1e-4, 1M tets: warm-started vs plain descent, 1 GB300"
UNIT = "frames/s"
# Algorithmic bytes of one tet-iteration (per-tet indices 16 B + Dm^-1 36 B +
# volume 4 B, plus per node x, x~, x_last, H_d (4 x 12 B), mass 4 B read and
# x_next 12 B written, amortised over tets): 56 + 64 N / T.
STATIC_BYTES_PER_TET = 56.0
BYTES_PER_NODE = 64.0
BATCH_ITERS = 96  # doDescentOpt(h, iterations) as fvm.cpp:187 calls it


def box_workload(seed: int, scale: float = 1.0):
    from phybs_gb300 import meshes as M
    nx, ny, nz = (max(2, int(round(50 * scale))), max(2, int(round(50 * scale))), max(2, int(round(80 * scale))))
    rng = np.random.default_rng(seed)
    young = float(10.0 ** rng.uniform(4.0, 6.0))
    m = M.box_mesh(nx, ny, nz, edge=0.005 / scale if scale != 1.0 else 0.005, jitter=0.1, seed=seed,
                   young=young, poisson=0.4, pin="both")
    z = m.rest[:, 2]
    bottom = np.nonzero(z <= z.min() + 1e-9)[0].astype(np.int32)
    length = float(z.max() - z.min())
    return m, bottom, length, young


def bottom_positions(m, bottom, length, frame):
    x = m.rest[bottom].astype(np.float32).copy()
    x[:, 2] -= np.float32(0.5 * length * min((frame + 1) / 30.0, 1.0))
    return x


# Residual-target solver settings for the box workload.  The reference's
# alpha0 = 0.1 needs ~15,000 iterations per frame at 1M tets.  With the
# Chebyshev stages below, alpha0 = 0.45 is 5-21% faster than 0.4 in both arms
# on each of the five mesh seeds (E from 15 kPa to 770 kPa) and converges
# every frame of a body at the range's softest 10 kPa (15 line-search
# rejections over 27 frames); at 0.5 the softest seed's line search rejects in
# a cascade (1,740 rejections).  The GPU energy clamp max(e, 0) is used: the
# CPU reference's e > 1e-6 J clamp zeroes the energy of these small tets.
ALPHA0 = 0.45
# Chebyshev schedule: (first iteration, rho) stages, each restarting the
# recurrence, in the reference's multi-stage form (DescentOptimize.cpp:
# 156-175).  The frame's fast modes go first with a small rho, the slowest
# ones last with rho = 0.9999; against one stage of 0.9999 from iteration 10
# it is faster in total over the five mesh seeds (the plain arm's time over
# frames 3..29, 4.80 -> 4.41 s; seed 0 plain +20%, warm-started +38%), with no
# line-search rejection in the plain arm; of the schedules tried, the least
# plain time in total.
RHO = 0.9999
PROFILE = ((5, 0.99), (25, 0.999), (100, RHO))
# The step size recovers by 1.2x per accepted energy check (up to alpha0):
# with the reference's shrink-only rule one early rejection slows a whole
# frame, most of all from a good (learned) start, whose Chebyshev ramp raises
# the small remaining energy gap at the first check.  Frames 3..11 of this
# workload: plain 16,544 -> 10,724 iterations, warm-started 19,668 -> 9,400.
ALPHA_GROW = 1.2


# Stress evaluation of the passes: incremental (P(F) - P(F0) against a
# double-float force at the step's initial guess).  The full FP32 stress is ~13% faster per
# pass, but with alpha_grow its residual floor stalls the last, most stretched
# frames of this pull just above 1e-4 |g0| (frame 29 ran into the iteration
# cap in both arms); the incremental form has no floor there.
INCREMENTAL_STRESS = 1


def solver_params(h=1 / 30, tol=1e-4, max_iters=20000, alpha0=ALPHA0, profile=PROFILE, incremental=None):
    from phybs_gb300 import _lib as L
    from phybs_gb300.solver import make_params
    inc = INCREMENTAL_STRESS if incremental is None else incremental
    return make_params("gpu_reference", h=h, tol=tol, max_iters=max_iters, control=L.PBS_CONTROL_RESTART,
                       energy_slack=16.0, alpha0=alpha0, profile=profile, incremental_stress=inc,
                       alpha_grow=ALPHA_GROW)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int = 0):
        import tempfile
        self.idx = device_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"phybs_clocks_{os.getpid()}_{id(self)}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in rows for j in range(4) if r[5 + j].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(tune, stress):
    """DRAM bytes of one plain pass (k_tchunk + k_node) that ncu measured on
    this workload with the same chunk shape and stress mode; None when no
    capture of that shape is committed (the tuned shape varies run to run).
    The node kernel reads and writes the same words with one or two nodes a
    thread, so the chunk shape (threads, tets, nodes, staging) decides."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p) or tune is None:
        return None
    with open(p) as f:
        entries = json.load(f).get("entries", [])
    shape = [tune["chunk_threads"], tune["chunk_tets"], tune["chunk_nodes"], tune["chunk_staged"]]
    full = shape + [tune.get("node_npt")]
    same = [e for e in entries if e.get("shape", [])[:4] == shape and e.get("stress") == stress]
    for e in same:  # the capture of this very shape first, then one of the same chunk shape
        if e.get("shape") == full:
            return e
    return same[0] if same else None


class CpuFrames:
    """The CPU restatement of the reference's descent step (oracle/phybs_oracle.cpp,
    DescentOptimize.cpp:91-188 with the benchmark's control: RESTART, alpha0,
    alpha growth, the Chebyshev stages of PROFILE, iterate to |g| <= 1e-4 |g0|) on the
    box workload, whole frames.  Its per-tet loops (forces, energies, Hessian
    diagonal) run on `threads` host threads (0 = all cores; the reference's
    DescentOptimize itself is serial, its material classes use OpenMP); the
    results do not depend on the thread count."""

    def __init__(self, m, bottom, length, threads=0, prec=32, x=None, v=None, v_old=None):
        from oracle import restated as O
        from phybs_gb300.solver import lame_arrays
        self.O = O
        self.m, self.bottom, self.length, self.prec = m, bottom, length, prec
        self.threads = O.set_threads(threads)
        self.mu, self.lam = lame_arrays(m.young, m.poisson)
        self.pm = m.pin_mask()
        self.r = O.rest(m.rest, m.tets, self.pm, prec=prec)
        self.st = O.StepState(m.rest if x is None else x, v, v_old)
        self.p = O.make_params(h=1 / 30, max_iters=20000, tol=1e-4, control=1, body_force_scale=1.0,
                               energy_clamp=1, alpha0=ALPHA0, profile=PROFILE, alpha_grow=ALPHA_GROW,
                               hessian_closed=1)

    def frame(self, f):
        """Frame f whole: (seconds, iterations, converged)."""
        self.st.x0[self.bottom] = bottom_positions(self.m, self.bottom, self.length, f)
        t0 = time.perf_counter()
        o = self.O.step(self.st, self.p, self.m.tets, self.r, self.mu, self.lam, self.pm, prec=self.prec)
        return time.perf_counter() - t0, int(o.passes), int(o.converged)


def cpu_force_comparator(m, x, calls=3, threads=0):
    """The reference's OpenMP force evaluation computeInnerForcesfromFhats2
    (IsotropicMaterial.cpp:411-453, ported: FP32, the modified SVD of every
    tet, one global lock around the node scatter) at positions x on all host
    cores: seconds per call (best of `calls`) and the thread count."""
    from oracle import restated as O
    from phybs_gb300.solver import lame_arrays
    mu, lam = lame_arrays(m.young, m.poisson)
    r = O.rest(m.rest, m.tets, m.pin_mask(), prec=32)
    best, n = float("inf"), 0
    for _ in range(calls):
        t0 = time.perf_counter()
        O.forces_fhats2_omp(x, m.tets, r.dinv, r.an, mu, lam, threads=threads)
        best = min(best, time.perf_counter() - t0)
    if threads <= 0:
        threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    return best, threads


def run_reference(args):
    """The CPU reference arm: frames 0 .. W-1 run whole and untimed, frames
    W .. W+K-1 run whole and timed (host wall clock, all host threads)."""
    m, bottom, length, young = box_workload(args.seed, args.scale)
    cpu = CpuFrames(m, bottom, length, threads=0, prec=args.cpu_prec)
    times, iters, conv = [], [], []
    for f in range(args.warmup + args.steps):
        dt, it, c = cpu.frame(f)
        if f >= args.warmup:
            times.append(dt)
            iters.append(it)
            conv.append(c)
    total = float(np.sum(times))
    value = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": f"f{args.cpu_prec}",
        "data": "synthetic",
        "config": {"workload": f"box 50x50x80 cubes, 5-tet split: {m.n_tets} tets / {m.n_nodes} nodes; bottom face "
                               f"pulled to 1.5x over 30 frames; plain descent; every frame to |g|<=1e-4|g0|; frames "
                               f"{args.warmup}..{args.warmup + args.steps - 1} timed",
                   "seed": args.seed, "young": young, "h": 1 / 30, "tol": 1e-4, "alpha0": ALPHA0, "rho_profile": PROFILE},
        "iterations": iters, "iterations_per_frame": float(np.mean(iters)), "converged": conv,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu.threads, "kind": "port",
                         "sample": f"frames {args.warmup}..{args.warmup + args.steps - 1} whole (after frames "
                                   f"0..{args.warmup - 1} untimed), FP{args.cpu_prec} restatement of "
                                   f"DescentOptimize with the benchmark's control, per-tet loops on "
                                   f"{cpu.threads} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def launches_per_frame(graph_launches: int, warm: bool) -> int:
    """Kernels of one frame: the boundary scatter; init_ctl, prologue, the
    RESTART control's guess check and fallback, the base force (per-tet
    double-float + gather with incremental stress, the gather alone
    otherwise), epilogue; with the warm start the plain guess's corner
    forces (full stress only), reference gradient, tet F, inference, judge and
    select; 2 x 16 passes plus the closing decision (k_settle) per body of
    the step graph's loop (the counts of a launch list of one plain and one
    warm-started frame)."""
    ref = 2 if INCREMENTAL_STRESS else 1
    warm_extra = (0 if INCREMENTAL_STRESS else 1) + 5 if warm else 0
    return 1 + 3 + 2 + ref + warm_extra + (2 * 16 + 1) * graph_launches


def tune_shape(args, m):
    """The pass kernels' chunk shape for this mesh (pbs_autotune on a fresh
    handle at the workload's first frame), applied to every arm."""
    from phybs_gb300.solver import DescentSolver
    s = DescentSolver(m, params=solver_params(max_iters=args.max_iters))
    try:
        return s.autotune(16)
    except Exception:  # keep the default shape
        return None
    finally:
        s.close()


def sync_ranks(world: int) -> None:
    """Barrier over the ranks, then wait for this rank's device: both sides
    of every timed region."""
    import torch
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()


def max_over_ranks(t: float, world: int) -> float:
    """The slowest rank's time, on every rank: the job's time for `value`
    (replicas: each rank steps its own copy of the workload)."""
    if world > 1:
        import torch
        tt = torch.tensor([t], dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t = float(tt.item())
    return t


def run_arm(args, m, bottom, length, model, world, e2e: bool, tune=None):
    """One arm over frames 0 .. W+K-1 on a fresh handle.  Returns the timed
    K frames' results: device time (CUDA events on the library's stream) or,
    with e2e, host wall time including each frame's position read-back."""
    import torch

    from phybs_gb300.solver import DescentSolver

    s = DescentSolver(m, params=solver_params(max_iters=args.max_iters))
    if tune is not None:
        s.set_chunk_shape(tune["chunk_threads"], tune["chunk_tets"], tune["chunk_nodes"], tune["chunk_staged"],
                          tune["node_npt"])
    if model is not None:
        s.set_warm_start(model)
    stream = torch.cuda.ExternalStream(s.stream())
    n_frames = args.warmup + args.steps
    pin_xyz = torch.empty((n_frames, bottom.size, 3), dtype=torch.float32, pin_memory=True).numpy()
    for f in range(n_frames):
        pin_xyz[f] = bottom_positions(m, bottom, length, f)
    out = torch.empty((m.n_nodes, 3), dtype=torch.float32, pin_memory=True).numpy()
    for f in range(args.warmup):
        s.set_node_positions(bottom, pin_xyz[f])
        s.step(raise_on_error=False)

    res = {"iters": [], "passes": 0, "launches": 0, "status": [], "ws_used": 0, "rejections": [], "converged": []}
    # the state the first timed frame starts from (the CPU baseline's start)
    res["state"] = (s.positions(), *s.velocities())
    sync_ranks(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        t0 = time.perf_counter()
        e0.record(stream)
        for f in range(args.warmup, n_frames):
            s.set_node_positions(bottom, pin_xyz[f])
            it = s.step(raise_on_error=False)
            if e2e:
                s.positions(out)
            st = s.stats()
            res["iters"].append(it)
            res["passes"] += st["passes"]
            res["launches"] += launches_per_frame(st["graph_launches"], model is not None)
            res["status"].append(st["status"])
            res["ws_used"] += st["warm_start_used"]
            res["rejections"].append(st["rejections"])
            # 0: the frame stopped at the iteration limit short of the residual bar
            res["converged"].append(st["converged"])
        e1.record(stream)
        sync_ranks(world)
        t_host = time.perf_counter() - t0
    t = max_over_ranks(t_host if e2e else e0.elapsed_time(e1) / 1e3, world)
    res["seconds"] = t
    res["frames_per_s"] = world * args.steps / t
    res["clocks"] = clk.summary()
    s.close()
    return res


def profile_pass(args, m, tune=None):
    """Per-kernel times of one descent pass (CUDA events on the library's
    stream, mean of 20 passes from the workload's first frame)."""
    from phybs_gb300.solver import DescentSolver
    s = DescentSolver(m, params=solver_params(max_iters=args.max_iters))
    if tune is not None:
        s.set_chunk_shape(tune["chunk_threads"], tune["chunk_tets"], tune["chunk_nodes"], tune["chunk_staged"],
                          tune["node_npt"])
    try:
        return s.profile_kernels(20), None
    except Exception as exc:  # an instance stopped early: no valid per-kernel time
        return None, f"{exc}; {s.stats()}"
    finally:
        s.close()


def stretch_pass_ms(args, m, x, tune=None):
    """The GPU's counterpart of the CPU force evaluation: mean time of the
    per-tet pass kernel (stretch-based forces of every tet, summed per node and
    chunk) at positions x, CUDA events on the library's stream; None when it
    cannot be timed."""
    from phybs_gb300 import _lib as L
    from phybs_gb300.solver import DescentSolver
    s = DescentSolver(m, positions=x, material=L.PBS_MATERIAL_STRETCH,
                      params=solver_params(max_iters=args.max_iters, incremental=0))
    try:
        if tune is not None:
            s.set_chunk_shape(tune["chunk_threads"], tune["chunk_tets"], tune["chunk_nodes"], 0, tune["node_npt"])
        tet_ms, _ = s.profile_kernels(20)
        return tet_ms
    except Exception:
        return None
    finally:
        s.close()


def run_ours(args, rank, world):
    import torch

    from phybs_gb300.warmstart import DEFAULT_MODEL, WarmStartModel

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    m, bottom, length, young = box_workload(args.seed, args.scale)
    model = WarmStartModel.load(DEFAULT_MODEL) if os.path.exists(DEFAULT_MODEL) and not args.plain_only else None
    if args.shape:
        v = [int(x) for x in args.shape.split(",")]
        tune = {"chunk_threads": v[0], "chunk_tets": v[1], "chunk_nodes": v[2], "chunk_staged": v[3], "node_npt": v[4]}
    else:
        tune = tune_shape(args, m)
    plain = run_arm(args, m, bottom, length, None, world, e2e=False, tune=tune)
    warm = run_arm(args, m, bottom, length, model, world, e2e=False, tune=tune) if model is not None else None
    head = warm if warm is not None else plain
    head_e2e = run_arm(args, m, bottom, length, model, world, e2e=True, tune=tune)
    prof, prof_err = profile_pass(args, m, tune)
    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    T, N = m.n_tets, m.n_nodes
    alg_bytes = STATIC_BYTES_PER_TET * T + BYTES_PER_NODE * N
    roof = None
    if prof is not None:
        tet_ms, node_ms = prof
        pass_ms = tet_ms + node_ms
        achieved = alg_bytes / (pass_ms * 1e-3) / 1e9
        traffic = ncu_traffic(tune, "incremental" if INCREMENTAL_STRESS else "full")
        roof = {"bound": "hbm", "kernel": "descent pass = k_tchunk + k_node", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": (traffic or {}).get("bytes_per_pass"),
                "traffic_source": (traffic or {}).get("source", "no ncu capture of this chunk shape committed"),
                "algorithmic_bytes_per_pass": alg_bytes,
                "tet_ms": tet_ms, "node_ms": node_ms}
    else:
        roof = {"error": prof_err}

    def summary(r):
        return {"frames_per_s": r["frames_per_s"], "ms_per_frame": r["seconds"] / args.steps * 1e3,
                "iterations_per_frame": float(np.mean(r["iters"])), "iterations": r["iters"],
                "iterations_per_s": r["passes"] / r["seconds"], "status": r["status"],
                "line_search_rejections": r["rejections"], "converged": r["converged"],
                "unconverged_frames": int(len(r["converged"]) - sum(r["converged"]))}

    mode = "warm-started (learned per-node MLP, plain descent as fallback and judge)" if warm else \
        "plain descent (no trained warm-start model present)"
    line = {
        "metric": METRIC, "value": head["frames_per_s"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["seconds"] / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"box 50x50x80 cubes, 5-tet split: {T} tets / {N} nodes; bottom face pulled to "
                               f"1.5x over 30 frames; {mode}; every frame to |g|<=1e-4|g0|; frames "
                               f"{args.warmup}..{args.warmup + args.steps - 1} timed",
                   "seed": args.seed, "young": young, "h": 1 / 30, "tol": 1e-4, "alpha0": ALPHA0, "rho_profile": PROFILE,
                   "l2": "working set larger than L2 (no flush)", "parallelism": f"replicas x{world}",
                   "stress": "incremental" if INCREMENTAL_STRESS else "full", "autotune": tune},
        "iterations_per_frame": float(np.mean(head["iters"])), "iterations_per_s": head["passes"] / head["seconds"],
        "plain": summary(plain),
        "roofline": roof,
        "gpu_launches": head["launches"],
        "e2e": {"value": head_e2e["frames_per_s"], "unit": UNIT, "h2d_bytes_per_step": int(bottom.size * 16),
                "d2h_bytes_per_step": int(N * 12)},
        "clocks": head["clocks"],
    }
    if warm is not None:
        line["warm"] = summary(warm)
        line["warm"]["learned_guess_kept"] = warm["ws_used"]
        line["warm"]["fallback_rate"] = 1.0 - warm["ws_used"] / max(len(warm["iters"]), 1)
        line["speedup_vs_plain"] = warm["frames_per_s"] / plain["frames_per_s"]
        line["clocks_plain"] = plain["clocks"]
    if not args.no_cpu_baseline:
        # whole frames W .. W+n-1 on the host, from the plain GPU arm's state at
        # the start of frame W
        x0, v0, vo0 = plain["state"]
        cpu = CpuFrames(m, bottom, length, threads=0, prec=args.cpu_prec, x=x0, v=v0, v_old=vo0)
        n = max(1, min(args.cpu_frames, args.steps))
        fr = [cpu.frame(args.warmup + j) for j in range(n)]
        secs = float(sum(t for t, _, _ in fr))
        line["cpu_baseline"] = {"value": n / secs, "unit": UNIT, "cores": cpu.threads, "kind": "port",
                                "sample": f"frames {args.warmup}..{args.warmup + n - 1} whole on the full mesh, from "
                                          f"the plain GPU arm's state at frame {args.warmup} (FP{args.cpu_prec} "
                                          f"restatement of DescentOptimize with the benchmark's control, per-tet "
                                          f"loops on {cpu.threads} threads)",
                                "iterations": [it for _, it, _ in fr], "converged": [c for _, _, c in fr],
                                "seconds": [round(t, 3) for t, _, _ in fr]}
        fsec, fthreads = cpu_force_comparator(m, x0, calls=3)
        line["cpu_force_eval"] = {
            "what": "the reference's OpenMP computeInnerForcesfromFhats2(nthreads) (IsotropicMaterial.cpp:411-453), "
                    "ported: stretch-based forces of all tets, FP32, one global lock around the node scatter",
            "ms_per_call": fsec * 1e3, "cores": fthreads, "tets": T,
            "gpu_stretch_pass_ms": stretch_pass_ms(args, m, x0, tune)}
    print(json.dumps(line))


def run_batch(args, rank, world):
    """Batched uneven instances: 256 independent 5-tet boxes (nx, ny in 4..16,
    nz in 8..32 cubes of 1 cm; E log-uniform in [1e4, 1e6] Pa, Poisson
    uniform in [0.3, 0.45]; the z = 0 end pinned; gravity from rest) packed
    into one handle and stepped together with the reference's GPU step
    semantics, doDescentOpt(h, 96) (CUDAInterface.cu:911-1007): 96
    iterations, its line search and Chebyshev profile, per instance.  The
    chunk shape is picked by pbs_autotune first.  A step is one time step of
    all 256 instances."""
    import torch

    from phybs_gb300 import meshes as M
    from phybs_gb300.solver import DescentSolver

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    from phybs_gb300.solver import make_params
    m = M.batch_of_boxes(256, seed=args.seed)
    # a fixed iteration count has no residual floor to respect: full FP32 stress
    s = DescentSolver(m, params=make_params("gpu_reference", h=1 / 30, max_iters=BATCH_ITERS, incremental_stress=0))
    tune = s.autotune(16)
    stream = torch.cuda.ExternalStream(s.stream())
    for _ in range(args.warmup):
        s.step(raise_on_error=False)
    sync_ranks(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters, passes, launches, statuses = [], 0, 0, []
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            it = s.step(raise_on_error=False)
            st = s.stats()
            iters.append(it)
            passes += st["passes"]
            launches += launches_per_frame(st["graph_launches"], False) - 1  # no boundary upload
            statuses.append(st["status"])
        e1.record(stream)
        sync_ranks(world)
    t = max_over_ranks(e0.elapsed_time(e1) / 1e3, world)
    prof, prof_err = None, None
    try:
        prof = s.profile_kernels(20)
    except Exception as exc:  # an instance stopped early: no valid per-kernel time
        prof_err = f"{exc}; {s.stats()}"
    s.close()
    if rank != 0:
        return
    T, N = m.n_tets, m.n_nodes
    line = {
        "metric": "batched frames/s, 256 uneven instances, 96 descent iterations per step, 1 GB300",
        "value": world * args.steps / t,
        "unit": "frames/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"256 boxes, nx,ny U{{4..16}}, nz U{{8..32}}, 5-tet split: {T} tets / {N} nodes; "
                               f"gravity from rest, z=0 pinned; doDescentOpt(h, 96) per instance",
                   "seed": args.seed, "h": 1 / 30, "iterations": BATCH_ITERS, "autotune": tune},
        "max_iterations_per_step": iters, "passes_per_s": passes / t, "tet_iterations_per_s": T * passes / t,
        "gpu_launches": launches, "status": statuses, "clocks": clk.summary(),
    }
    if prof is not None:
        alg = STATIC_BYTES_PER_TET * T + BYTES_PER_NODE * N
        peak, kind = measured_peak()
        a = alg / ((prof[0] + prof[1]) * 1e-3) / 1e9
        line["roofline"] = {"bound": "hbm", "kernel": "descent pass = k_tchunk + k_node", "achieved": a,
                            "peak": peak, "unit": "GB/s", "frac": a / peak, "peak_kind": kind,
                            "tet_ms": prof[0], "node_ms": prof[1], "algorithmic_bytes_per_pass": alg}
    else:
        line["roofline"] = {"error": prof_err}
    print(json.dumps(line))


def run_dynamics(args, rank, world, kind):
    """The reference's other integrators on the 1M-tet box (50 x 50 x 80
    cubes, 5-tet split, both end faces pinned at rest), twisted about its
    long axis by 0.3 rad sin(pi s) (s the height fraction) and stepped under
    gravity: `pbd` = strain-based PBD with the reference's
    5 sweeps, stretch 1, shear 0.8 (PosBaseDynamic.cpp), dt = 1/30; `pd` =
    projective dynamics with stiffness 1e6 and 5 local/global iterations
    (ProjDynamic.cpp), dt = 0.03, CG to 1e-6; `be` = the linearly implicit
    backward-Euler step (CUDAInterface::doBackEuler), dt = 0.03,
    alpha = beta = 0.02, CG to 1e-6.  A step is one call through the C ABI
    (synchronous; positions stay on the device)."""
    import torch

    from phybs_gb300 import meshes as M
    from phybs_gb300.solver import DescentSolver

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    m, _, _, _ = box_workload(args.seed, args.scale)
    # twisted 0.3 rad at mid-height, 0 at both pinned end faces (which stay at
    # rest: the backward-Euler step's pins are springs to the rest positions)
    x = M.twist_positions(m.rest, 0.3, axis=2, profile="sine").astype(np.float32)
    s = DescentSolver(m, positions=x)
    if kind == "pbd":
        step = lambda: s.pbd_step(1 / 30)
    elif kind == "pd":
        step = lambda: s.pd_step(0.03, tol=1e-6)
    else:
        step = lambda: s.backward_euler_step(dt=0.03, tol=1e-6, max_iters=20000)[0]
    for _ in range(args.warmup):
        step()
    stream = torch.cuda.ExternalStream(s.stream())
    sync_ranks(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    cg = []
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            r = step()
            if kind in ("pd", "be"):
                cg.append(r)
        e1.record(stream)
        sync_ranks(world)
    t = max_over_ranks(e0.elapsed_time(e1) / 1e3, world)
    s.close()
    if rank != 0:
        return
    line = {
        "metric": {"pbd": "strain-based PBD steps/s (5 sweeps)",
                   "pd": "projective-dynamics steps/s (5 local/global iterations)",
                   "be": "backward-Euler steps/s (CG to 1e-6)"}[kind] +
                  (", 1M-tet box, 1 GB300" if args.scale == 1.0 else f", {m.n_tets}-tet box, 1 GB300"),
        "value": world * args.steps / t, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"box, 5-tet split: {m.n_tets} tets / {m.n_nodes} nodes, both ends pinned, "
                               f"twisted 0.3 rad sin(pi s) along its height, gravity", "seed": args.seed,
                   "scale": args.scale},
        "clocks": clk.summary(),
    }
    if kind in ("pd", "be"):
        line["cg_iterations_per_step"] = cg
    else:
        L = M.pbd_levels(m.tets, m.n_nodes)
        line["roofline"] = {"bound": "latency", "levels": L, "level_sweeps_per_step": 5 * L,
                            "us_per_level": t / args.steps / (5 * L) * 1e6}
        if not args.no_cpu_baseline:
            from oracle import projective as P
            dinv, w, grav = P.rest_eigen32(m.rest, m.tets, m.pin_mask(), density=float(m.density))
            t0 = time.perf_counter()
            P.pbd_step(x, np.zeros_like(x), w, m.tets, dinv, grav, 1 / 30)
            cs = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": 1.0 / cs, "unit": "steps/s", "cores": 1, "kind": "port",
                                    "sample": "one step on the full mesh: the serial FP32 restatement of "
                                              "PosBaseDynamic (orc_pbd_step), bit-identical to the reference"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=27)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--scale", type=float, default=1.0, help="mesh resolution scale (1.0 = the 1M-tet box)")
    ap.add_argument("--max-iters", type=int, default=20000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-frames", type=int, default=3, help="whole frames the GPU arm's CPU baseline times")
    # FP64 by default: the FP32 restatement, like the reference, sums the
    # line search's energies in FP32, and on the 1M-tet box that noise rejects
    # good steps until alpha falls below 0.01 short of the 1e-4 bar (frame 0:
    # |g|/|g0| = 2.4e-4 after 1,719 iterations)
    ap.add_argument("--cpu-prec", type=int, choices=[32, 64], default=64,
                    help="arithmetic of the CPU restatement (the reference computes in FP32)")
    ap.add_argument("--plain-only", action="store_true", help="time the plain descent only")
    ap.add_argument("--stress", choices=["full", "incremental"], default=None,
                    help="pass stress evaluation (default: incremental)")
    ap.add_argument("--shape", default=None,
                    help="launch shapes 'threads,tets,nodes,staged,node_npt' instead of autotuning (profiling runs)")
    ap.add_argument("--workload", choices=["box1m", "batch", "pbd", "pd", "be"], default="box1m",
                    help="box1m: the 1M-tet pull (the headline); batch: 256 uneven instances; pbd / pd / be: the "
                         "strain-based PBD / projective-dynamics / backward-Euler steps on the 1M-tet box")
    args = ap.parse_args()
    if args.stress is not None:
        global INCREMENTAL_STRESS
        INCREMENTAL_STRESS = 1 if args.stress == "incremental" else 0
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("gloo")
    if args.workload == "batch":
        run_batch(args, rank, world)
    elif args.workload in ("pbd", "pd", "be"):
        run_dynamics(args, rank, world, args.workload)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
