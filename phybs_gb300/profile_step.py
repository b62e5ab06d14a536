"""Fixed launch sequence of the descent step's kernels, for profilers.

    python -m phybs_gb300.profile_step --scale 0.5 --passes 40 --warm --train-steps 20

On the pulled-box workload (50 x 50 x 80 cubes, 5-tet split, times --scale
per axis), with the bottom face at its frame --frame position:

1. pbs_profile_kernels(--passes): the step's prologue, guess check and base
   force (k_ref_tet, k_ref_gather), then --passes passes from k = 0 with the
   residual stop off.  Per-tet kernel launch j is pass k = j: launch 0 is a
   line-search pass that also refreshes the Jacobi diagonal, launches 1-7
   are plain passes, launch 8 a line-search pass (its check at k = 8 can
   reject and redo k; launch 8 is a line-search pass either way).
2. With --engine frame also pbs_profile_frame(--passes) (one k_frame launch).
3. With --warm: one warm-started step with the committed model (k_ws_*
   kernels once each, and a whole frame of passes).
4. With --train-steps N: N Adam steps of the warm-start network on random
   data (k_mlp_grad, k_mlp_reduce, k_mlp_adam per step).

Prints one JSON line with the CUDA-event times.  A profiler's kernel filter
and launch skip select the launches (for example `-k regex:k_tchunk -s 8 -c
1` for the line-search pass).
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=float, default=0.5)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--frame", type=int, default=0)
    ap.add_argument("--passes", type=int, default=40)
    ap.add_argument("--shape", default="256,512,256,0,2", help="threads,tets,nodes,staged,node_npt")
    ap.add_argument("--engine", choices=["graph", "frame"], default="graph")
    ap.add_argument("--warm", action="store_true")
    ap.add_argument("--train-steps", type=int, default=0)
    ap.add_argument("--stress", choices=["incremental", "full"], default="incremental")
    ap.add_argument("--l2", choices=["on", "off"], default="on", help="L2 residency window of the pass rows")
    args = ap.parse_args()

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    from .solver import DescentSolver

    m, bottom, length, young = bench.box_workload(args.seed, args.scale)
    s = DescentSolver(m, params=bench.solver_params(incremental=1 if args.stress == "incremental" else 0))
    s.set_chunk_shape(*[int(x) for x in args.shape.split(",")])
    if args.l2 == "off":
        s.set_l2_residency(False)
    s.set_node_positions(bottom, bench.bottom_positions(m, bottom, length, args.frame))
    out = {"tets": m.n_tets, "nodes": m.n_nodes, "shape": args.shape, "stress": args.stress, "l2": args.l2}
    tet, node = s.profile_kernels(args.passes)
    out["tet_us"], out["node_us"] = tet * 1e3, node * 1e3
    if args.engine == "frame":
        out["frame_pass_us"] = s.profile_frame(args.passes) * 1e3
    if args.warm:
        from .warmstart import DEFAULT_MODEL, WarmStartModel
        s.set_warm_start(WarmStartModel.load(DEFAULT_MODEL))
        it = s.step(raise_on_error=False)
        st = s.stats()
        out["warm_step"] = {"iterations": it, "passes": st["passes"], "device_ms": st["device_ms"],
                            "status": st["status"], "learned_guess_kept": st["warm_start_used"]}
    s.close()
    if args.train_steps > 0:
        import time

        from .warmstart import MLPTrainer
        rng = np.random.default_rng(args.seed)
        n = 65536
        X = rng.standard_normal((n, 24)).astype(np.float32)
        Y = (0.1 * rng.standard_normal((n, 3))).astype(np.float32)
        t = MLPTrainer(seed=args.seed)
        t.set_data(X, Y)
        t.train(2, batch=4096)
        t0 = time.perf_counter()
        t.train(args.train_steps, batch=4096)
        out["train_ms_per_step_host"] = (time.perf_counter() - t0) / args.train_steps * 1e3
        t.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
