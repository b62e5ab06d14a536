"""Pin the backward-Euler restatement's element stiffness (oracle/implicit.py:
the closed-form neo-Hookean Hessian) to the reference's own element matrices
(IsotropicMaterial::computeStiffnessMatrixFromPos, Xu et al.'s SVD-derivative
dP/dF; tests/golden/stiffness_*.npz), and check the restated step's system."""
import numpy as np
import pytest

from oracle import implicit as I
from oracle import restated as O
from phybs_gb300 import meshes as M
from tests._util import golden_names, load_golden

NAMES = golden_names("stiffness_")


@pytest.fixture(scope="module", params=NAMES)
def kg(request):
    return load_golden(request.param)


def test_fixture_set():
    assert NAMES == ["stiffness_bar_small", "stiffness_ellipsoid_small", "stiffness_model_bar"]


def test_element_stiffness_matches_reference(kg):
    """Per sampled tet, max-norm relative to the element matrix: the reference
    computes in FP32 through an SVD and perturbs near-equal stretches by 1e-6."""
    s = kg["sample"]
    K = I.element_stiffness(kg["x"], kg["tets"][s], kg["dminv"][s], kg["vol"][s], kg["mu"][s], kg["lam"][s])
    err = np.abs(K - kg["K"]).max(axis=(1, 2)) / np.abs(kg["K"]).max(axis=(1, 2))
    assert err.max() < 1e-5, err.max()
    assert np.abs(K - K.transpose(0, 2, 1)).max() <= 1e-9 * np.abs(K).max()  # symmetric


def test_restated_step_system():
    """The restated step's matrix is symmetric positive definite and its solve
    satisfies A v' = b; pinned nodes barely move."""
    m = M.bar_mesh(6, 3, 3, edge=0.025, young=5e4, poisson=0.4)
    mu, lam = O.lame(m.young, m.poisson)
    x0 = M.twist_positions(m.rest, 0.4, axis=0)
    x0[m.pins] = m.rest[m.pins]
    x1, v1, A, b = I.backward_euler_step(x0, np.zeros_like(x0), m.rest, m.tets, m.pin_mask(), mu, lam)
    assert abs(A - A.T).max() <= 1e-9 * abs(A).max()
    assert np.linalg.eigvalsh(A.toarray()).min() > 0
    assert np.abs(A @ v1.reshape(-1) - b).max() <= 1e-8 * np.abs(b).max()
    assert np.abs(x1[m.pins] - m.rest[m.pins]).max() < 1e-6
