"""The multi-rank path of bench.py on CPU (gloo, world size 2): the path is
replicas only (every rank steps its own copy of the workload, no data-path
collective), so what ranks share is the barrier around the timed region and
the job time, the slowest rank's.  The replicas themselves are the same
deterministic step: two ranks running the oracle's step on the same inputs
get the same bits."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys

    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import restated as O
    from phybs_gb300 import meshes as M
    # the job time is the slowest rank's, on every rank
    t = bench.max_over_ranks(1.0 + rank, world)
    # a replica: one restated FP32 step of the same small bar
    m = M.bar_mesh(6, 3, 3, edge=0.025, young=5e4, poisson=0.4)
    pm = m.pin_mask()
    mu, lam = O.lame(m.young, m.poisson)
    r = O.rest(m.rest, m.tets, pm, prec=32)
    st = O.StepState(m.rest)
    O.step(st, O.make_params(h=1 / 30, max_iters=32), m.tets, r, mu, lam, pm, prec=32)
    digest = torch.tensor(np.frombuffer(np.ascontiguousarray(st.x0, np.float64).tobytes(), np.int64)[:64].copy())
    gathered = [torch.zeros_like(digest) for _ in range(world)]
    dist.all_gather(gathered, digest)
    same = all(bool(torch.equal(gathered[0], g)) for g in gathered)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, same))


def test_two_gloo_ranks_share_job_time_and_step_alike():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(o[0] for o in out) == [0, 1]
    assert all(o[1] == 2.0 for o in out)  # max over ranks on both
    assert all(o[2] for o in out)         # replicas bit-identical
