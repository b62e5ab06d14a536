"""The softest body of the benchmark's seeds through the incremental stress.

Seed 3 of the 1M-tet pull draws E = 14.8 kPa: the body moves far within a
frame, so the increment of a node over the step's base is large and nearly
the same across a chunk.  When each node's increment was rounded to one FP32
word per pass, the differences the tets are made of were rounded away and
frames 4-6 stalled with |g| at 1.3-1.7e-4 of |g_0| until the 20,000-iteration
limit; the passes now hold the state as its increment over the base (an
exact split before the first pass) and a chunk stages it relative to one of
its nodes.  Every frame of the first eight must reach the 1e-4 bar, and the
pinned (prescribed) nodes must come back bit for bit from the increment form.
"""
import os
import sys

import numpy as np
import pytest

from phybs_gb300.solver import DescentSolver

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

FRAMES = 8


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


def test_soft_seed_frames_reach_the_bar():
    m, bottom, length, young = bench.box_workload(3)
    assert young < 2e4
    s = DescentSolver(m, params=bench.solver_params())
    iters = []
    for f in range(FRAMES):
        xb = bench.bottom_positions(m, bottom, length, f)
        s.set_node_positions(bottom, xb)
        it = s.step(raise_on_error=False)
        st = s.stats()
        iters.append(it)
        assert st["status"] == 0 and st["converged"] == 1, (f, it, st["residual_ratio"])
        assert st["residual_ratio"] <= 1e-4, (f, st["residual_ratio"])
        x = s.positions()
        # the prescribed face: exactly where it was put
        assert np.array_equal(x[bottom], xb.astype(np.float32)), f
    print(f"soft seed (E = {young:.0f} Pa) iterations per frame: {iters}")
    assert max(iters) < 5000, iters
    s.close()
