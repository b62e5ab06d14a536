"""Parity at the benchmarked solver settings, on a scaled copy of the
benchmark's mesh.

bench.py times the 1M-tet box pull (50 x 50 x 80 cubes, 5-tet split, nodes
jittered by 0.1 cell, top face pinned, bottom face pulled to 1.5x its length
over 30 frames, h = 1/30) with RESTART control, alpha0 0.45, alpha growth 1.2,
the three-stage Chebyshev schedule bench.PROFILE, incremental stress, the GPU energy
clamp and every frame iterated to |g| <= 1e-4 |g_0|.  This test runs the same
settings (bench.solver_params, bench.box_workload, bench.bottom_positions:
nothing re-typed) on the same box at 1/5 resolution (10 x 10 x 16 cubes,
8,000 tets, edge 2.5 cm), through its first frames, where the pull
accelerates the body and the step costs the most iterations, in both
benchmark arms: the plain descent and the descent warm-started by the learned
model.  Each frame is compared with the all-FP64 restatement of the same
step (same control, FP64 energies and residuals, converged to the same bar)
started from the GPU's state, so a frame's error is that frame's own: the
positions must agree within 1e-4 of the bounding-box diagonal, and the
errors are printed.
"""
import os
import sys

import numpy as np
import pytest

from oracle import restated as O
from phybs_gb300 import _lib as L
from phybs_gb300.solver import DescentSolver
from tests._util import bbox_diag

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

POS_TOL = 1e-4
FRAMES = 10


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


def _oracle_params():
    """bench.solver_params() as the restatement takes it."""
    return O.make_params(h=1 / 30, max_iters=20000, tol=1e-4, control=1, alpha0=bench.ALPHA0,
                         profile=bench.PROFILE, body_force_scale=1.0, energy_clamp=1, hessian_closed=1,
                         alpha_grow=bench.ALPHA_GROW)


@pytest.mark.parametrize("arm", ["plain", "warm"])
def test_benchmark_settings_frames_vs_fp64(arm):
    m, bottom, length, young = bench.box_workload(0, scale=0.2)
    assert (m.n_tets, m.n_nodes) == (8000, 11 * 11 * 17)
    p = bench.solver_params()
    assert p.incremental_stress == 1 and p.control == L.PBS_CONTROL_RESTART and p.tol == pytest.approx(1e-4)
    s = DescentSolver(m, params=p)
    if arm == "warm":
        from phybs_gb300.warmstart import DEFAULT_MODEL, WarmStartModel
        s.set_warm_start(WarmStartModel.load(DEFAULT_MODEL))
    mu, lam = O.lame(m.young, m.poisson)
    pm = m.pin_mask()
    r64 = O.rest(m.rest, m.tets, pm, prec=64)
    po = _oracle_params()
    diag = bbox_diag(m.rest)
    errs, iters, kept = [], [], 0
    for f in range(FRAMES):
        xb = bench.bottom_positions(m, bottom, length, f)
        x = s.positions()
        v, vo = s.velocities()
        st = O.StepState(x, v, vo)
        st.x0[bottom] = xb
        s.set_node_positions(bottom, xb)
        it = s.step()
        gs = s.stats()
        assert gs["status"] == 0 and gs["converged"] == 1, (f, gs)
        assert gs["residual_ratio"] <= 1e-4
        o = O.step(st, po, m.tets, r64, mu, lam, pm, prec=64)
        assert o.converged == 1, (f, o.k_final)
        err = float(np.abs(s.positions() - st.x0).max() / diag)
        errs.append(err)
        iters.append((it, o.k_final))
        kept += gs["warm_start_used"]
    print(f"{arm}: per-frame max |x - x_fp64| / diag = {[f'{e:.1e}' for e in errs]}; "
          f"iterations (GPU, FP64) = {iters}; learned guess kept on {kept} of {FRAMES} frames")
    assert max(errs) < POS_TOL, errs
    # the pull did move the body: the last frame's bottom sits well below rest
    assert np.abs(s.positions()[bottom, 2] - m.rest[bottom, 2]).max() > 0.1 * length * FRAMES / 30
    s.close()
