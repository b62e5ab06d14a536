"""L2 residency of the pass rows (pbs_set_l2_residency) changes where the
per-tet kernels' rows are cached, not what they compute: steps with and
without the access-policy window are bit-identical, and a handle's own
toggling (which recaptures the step graph) is too."""
import numpy as np
import pytest

from phybs_gb300 import _lib as L
from phybs_gb300 import meshes as M
from phybs_gb300.solver import DescentSolver, make_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


def test_l2_window_changes_no_result():
    m = M.box_mesh(16, 16, 24, edge=0.01, seed=5, young=2e5, poisson=0.4, pin="both")
    p = make_params("gpu_reference", h=1 / 30, max_iters=2000, tol=1e-4, control=L.PBS_CONTROL_RESTART,
                    alpha0=0.3, energy_slack=16.0, profile=((10, 0.9999),), alpha_grow=1.2)
    a = DescentSolver(m, params=p)
    b = DescentSolver(m, params=p)
    b.set_l2_residency(False)
    z = m.rest[:, 2]
    bottom = np.nonzero(z <= z.min() + 1e-9)[0].astype(np.int32)
    for f in range(4):
        x = m.rest[bottom].copy()
        x[:, 2] -= np.float32(0.005 * (f + 1))
        for s in (a, b):
            s.set_node_positions(bottom, x)
            s.step()
        if f == 1:  # the same handle toggled: off, then back on
            a.set_l2_residency(False)
        if f == 2:
            a.set_l2_residency(True)
        sa, sb = a.stats(), b.stats()
        assert (sa["passes"], sa["rejections"], sa["converged"]) == (sb["passes"], sb["rejections"], sb["converged"])
        assert np.array_equal(a.positions(), b.positions()), f
    a.close()
    b.close()
