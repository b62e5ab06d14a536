"""GPU parity of the backward-Euler step (pbs_backward_euler_step) through the
C ABI against the FP64 restatement (oracle/implicit.py: the reference's
doBackEuler system, CUDAInterface.cu:784-884, with a direct sparse solve).

Bar: positions after a step within 1e-4 of the bounding-box diagonal of the
restatement's (the path's position bar), the CG residual below its tolerance,
bit-reproducible runs."""
import numpy as np
import pytest

from oracle import implicit as I
from oracle import restated as O
from phybs_gb300 import _lib as L
from phybs_gb300 import meshes as M
from phybs_gb300.solver import DescentSolver

pytestmark = pytest.mark.gpu

POS_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


def twisted_bar():
    m = M.bar_mesh(10, 4, 4, edge=0.025, young=5e4, poisson=0.4)
    x0 = M.twist_positions(m.rest, 0.5, axis=0)
    x0[m.pins] = m.rest[m.pins]
    return m, x0


@pytest.mark.parametrize("material", [L.PBS_MATERIAL_NEOHOOKEAN, L.PBS_MATERIAL_STRETCH])
def test_steps_match_restatement(material):
    """Five steps from a twisted bar (x = 0 pinned, gravity), each compared with
    one restated FP64 step from the GPU's state."""
    m, x0 = twisted_bar()
    mu, lam = O.lame(m.young, m.poisson)
    s = DescentSolver(m, positions=x0, material=material, mu=mu, lam=lam)
    diag = m.bbox_diagonal()
    x, v = s.positions(), s.velocities()[0]
    for k in range(5):
        xo, vo, _, _ = I.backward_euler_step(x, v, m.rest, m.tets, m.pin_mask(), mu, lam, material=material)
        it, res = s.backward_euler_step(tol=1e-6)
        assert res <= 1e-6 and it > 0
        x, v = s.positions(), s.velocities()[0]
        err = np.abs(x - xo).max() / diag
        assert err < POS_TOL, (k, err, it, res)
        assert np.abs(x[m.pins] - m.rest[m.pins]).max() < 1e-6
    # the bar untwists and sags
    assert np.abs(x - x0).max() > 1e-3 * diag
    s.close()


def test_box_step_with_external_forces():
    """A 12 x 12 x 20 box (14,400 tets), top pinned, gravity plus a lateral pull
    on the bottom face, against the restatement."""
    m = M.box_mesh(12, 12, 20, edge=0.01, seed=3, young=2e5, poisson=0.4)
    mu, lam = O.lame(m.young, m.poisson)
    ext = np.zeros_like(m.rest)
    bottom = m.rest[:, 2] <= m.rest[:, 2].min() + 1e-6
    ext[bottom, 0] = 0.02
    s = DescentSolver(m, mu=mu, lam=lam)
    x, v = s.positions(), s.velocities()[0]
    xo, vo, _, _ = I.backward_euler_step(x, v, m.rest, m.tets, m.pin_mask(), mu, lam, ext=ext, h=1 / 30)
    it, res = s.backward_euler_step(dt=1 / 30, ext=ext, tol=1e-6)
    assert res <= 1e-6
    assert np.abs(s.positions() - xo).max() / m.bbox_diagonal() < POS_TOL
    assert np.abs(s.velocities()[0] - vo).max() <= 1e-3 * np.abs(vo).max()
    s.close()


def test_bitwise_reproducible_and_iteration_cap():
    m, x0 = twisted_bar()
    out = []
    for _ in range(2):
        s = DescentSolver(m, positions=x0)
        for _ in range(2):
            s.backward_euler_step()
        out.append(s.positions())
        s.close()
    assert np.array_equal(out[0], out[1])
    s = DescentSolver(m, positions=x0)
    it, res = s.backward_euler_step(max_iters=2, raise_on_cap=False)
    assert s.last_status == L.PBS_E_ITER_CAP and it == 2 and res > 1e-6
    assert not np.array_equal(s.positions(), x0)  # the last iterate was applied
    with pytest.raises(L.PhybsError):
        s.backward_euler_step(dt=-1.0)
    s.close()
