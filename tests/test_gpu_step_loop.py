"""The step graph's WHILE node runs exactly the pass bodies a step needs.

A step's passes run in bodies of 16 passes and a closing settle
(`CUDAInterface.cu:886-890` is the reference's host check every 8
iterations).  The graph's conditional node repeats the body while an instance
runs; the settle's last CTA sets the condition, so the loop ends after the body
in which the last instance finished and no body runs that only finds every
instance done.  The decisions and positions are those of the frame engine and
of the CPU reference (test_gpu_frame.py, test_gpu_parity.py); here the count of
bodies is pinned against the passes the step took.
"""
import numpy as np
import pytest

from phybs_gb300 import _lib as L
from phybs_gb300 import meshes as M
from phybs_gb300.solver import DescentSolver, make_params

pytestmark = pytest.mark.gpu

BODY = 16


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


def _bar():
    m = M.bar_mesh(16, 6, 6, edge=0.025, young=5e4, poisson=0.4)
    p = make_params("gpu_reference", h=1 / 30, max_iters=4000, tol=1e-3, control=L.PBS_CONTROL_RESTART,
                    alpha0=0.5, energy_slack=16.0, profile=((10, 0.995),))
    return m, p


def _boxes():
    """Six packed boxes that stop at different passes (incremental stress):
    some at the residual bar, others at the iteration limit (not an error)."""
    m = M.batch_of_boxes(6, seed=11, nxy=(4, 12), nz=(8, 24))
    p = make_params("gpu_reference", h=1 / 30, max_iters=3000, tol=1e-3, control=L.PBS_CONTROL_RESTART,
                    alpha0=0.3, energy_slack=16.0, alpha_grow=1.2, incremental_stress=1)
    return m, p


@pytest.mark.parametrize("case", [_bar, _boxes], ids=["bar", "packed boxes"])
def test_step_runs_no_extra_body(case):
    m, p = case()
    s = DescentSolver(m, params=p)
    for f in range(4):
        s.step()
        st = s.stats()
        assert st["status"] == 0 and st["converged"] >= 1, (f, st)
        n = st["graph_launches"]
        # the last instance finished in body n, not before it
        assert (n - 1) * BODY < st["passes"] <= n * BODY, (f, n, st["passes"])
        assert np.isfinite(s.positions()).all()
    s.close()


def test_pass_cap_ends_the_loop():
    """An instance that cannot converge stops at the pass cap: the loop runs
    the bodies the cap allows and no more."""
    m = M.bar_mesh(16, 6, 6, edge=0.025, young=5e4, poisson=0.4)
    p = make_params("gpu_reference", h=1 / 30, max_iters=40, tol=1e-12, control=L.PBS_CONTROL_RESTART,
                    alpha0=0.5, energy_slack=16.0, profile=((10, 0.995),))
    s = DescentSolver(m, params=p)
    s.step(raise_on_error=False)
    st = s.stats()
    assert st["converged"] == 0
    n = st["graph_launches"]
    assert (n - 1) * BODY < st["passes"] <= n * BODY, (n, st["passes"])
    s.close()
