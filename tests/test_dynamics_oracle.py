"""The strain-based PBD and projective-dynamics restatements (oracle/projective.py,
orc_pbd_step of oracle/phybs_oracle.cpp) against the reference's own outputs
(tests/golden/dynamics_*.npz, from PosBaseDynamic.cpp and ProjDynamic.cpp built
headless), on the reference's rest data.

Bars: PBD bit for bit (the same FP32 operations in the same order); projective
dynamics within 5e-5 of the bounding-box diagonal (the reference factorises
its matrix in FP32, the restatement solves in FP64), including a step from a
state with inverted tets (the SVD determinant fix flips the largest singular
direction)."""
import numpy as np
import pytest

from oracle import projective as P
from tests._util import bbox_diag, golden_names, load_golden

NAMES = golden_names("dynamics_")


@pytest.fixture(scope="module", params=NAMES)
def g(request):
    return load_golden(request.param)


def test_fixtures_present():
    assert len(NAMES) >= 3


def forces(g, k):
    f = g["gravity"].astype(np.float32).copy()
    if k == 0:
        f += g["ext"]
    return f


def test_pbd_matches_reference_bitwise(g):
    x, v = g["x0"], np.zeros_like(g["x0"])
    k = 0
    while f"x_pbd{k}" in g:
        x, v = P.pbd_step(x, v, g["inv_mass"], g["tets"], g["dminv"].reshape(-1, 9), forces(g, k), float(g["dt"]))
        assert np.array_equal(x, g[f"x_pbd{k}"]), k
        assert np.array_equal(v, g[f"v_pbd{k}"]), k
        k += 1
    assert k >= 3


def test_rest_data_matches_reference_bitwise(g):
    """The PBD step's rest data formed as TetMesh does in FP32 (Eigen's 3x3
    inverse, sequential lumped masses) equal the reference's bit for bit."""
    pm = np.zeros(len(g["rest"]), np.int32)
    pm[g["pins"]] = 1
    dinv, w, grav = P.rest_eigen32(g["rest"], g["tets"], pm)
    assert np.array_equal(dinv, g["dminv"].reshape(-1, 9))
    assert np.array_equal(w, g["inv_mass"])
    assert np.array_equal(grav, g["gravity"])


def test_pbd_planted_change_is_seen(g):
    """A 1e-5 relative change of one inverse mass changes the sweep's
    result: the bitwise comparison above is a real check."""
    w = g["inv_mass"].copy()
    i = int(np.argmax(w))
    w[i] = w[i] * np.float32(1 + 1e-5)
    x, _ = P.pbd_step(g["x0"], np.zeros_like(g["x0"]), w, g["tets"], g["dminv"].reshape(-1, 9), forces(g, 0),
                      float(g["dt"]))
    assert not np.array_equal(x, g["x_pbd0"])


def test_pd_matches_reference(g):
    diag = bbox_diag(g["rest"])
    x, v = g["x0"].astype(np.float64), np.zeros_like(g["x0"], dtype=np.float64)
    k = 0
    while f"x_pd{k}" in g:
        x_in = g[f"x_pd{k - 1}"] if k else g["x0"]
        v_in = g[f"v_pd{k - 1}"] if k else np.zeros_like(g["x0"])
        x, v = P.pd_step(x_in, v_in, g["mass"], g["inv_mass"], g["tets"], g["dminv"], g["vol"], forces(g, k),
                         dt=float(g["dt"]))
        assert np.abs(x - g[f"x_pd{k}"]).max() / diag < 5e-5, k
        moved = np.abs(g[f"x_pd{k}"] - x_in).max()
        assert np.abs(x - g[f"x_pd{k}"]).max() < 0.01 * moved, k
        k += 1
    assert k >= 2


def test_pd_inverted_tets_match_reference(g):
    diag = bbox_diag(g["rest"])
    x, _ = P.pd_step(g["x_inv"], np.zeros_like(g["x_inv"]), g["mass"], g["inv_mass"], g["tets"], g["dminv"],
                     g["vol"], g["gravity"], dt=float(g["dt"]))
    assert np.abs(x - g["x_pd_inv"]).max() / diag < 5e-5
    # flipping the smallest direction instead (the usual polar convention)
    # misses the reference's step by 2e-3 .. 4e-2 of the diagonal
    xs, _ = P.pd_step(g["x_inv"], np.zeros_like(g["x_inv"]), g["mass"], g["inv_mass"], g["tets"], g["dminv"],
                      g["vol"], g["gravity"], dt=float(g["dt"]), flip=2)
    assert np.abs(xs - g["x_pd_inv"]).max() / diag > 1e-3


def test_pd_split_time_step_matches_reference():
    """The reference forms its matrix with the integrator's time step
    (fvm.cpp:300-307) and steps with dt = 0.03 (fvm.cpp:169): with the two
    different, the restatement still follows the reference's own build."""
    from oracle import ref as R
    if not R.available():
        pytest.skip("reference build not available")
    g = load_golden("dynamics_bar_small")
    sim = R.RefSim(g["rest"], g["tets"], g["pins"], 5e5, 0.45)
    sim.set_nodes(g["x0"])
    sim.set_vel(np.zeros_like(g["x0"]))
    sim.set_ext(np.zeros_like(g["x0"]))
    sim.pd_step(0.03, dt_matrix=0.02)
    x, _ = P.pd_step(g["x0"], np.zeros_like(g["x0"]), g["mass"], g["inv_mass"], g["tets"], g["dminv"], g["vol"],
                     g["gravity"], dt=0.03, dt_matrix=0.02)
    diag = bbox_diag(g["rest"])
    assert np.abs(x - sim.nodes()).max() / diag < 5e-5
    same_dt, _ = P.pd_step(g["x0"], np.zeros_like(g["x0"]), g["mass"], g["inv_mass"], g["tets"], g["dminv"],
                           g["vol"], g["gravity"], dt=0.03)
    assert np.abs(x - same_dt).max() / diag > 1e-4  # the split changes the step
    sim.close()


def test_pbd_levels_count():
    """The dependency-level count of a Gauss-Seidel sweep: a chain of tets
    sharing a node has one level per tet; tets sharing no node, one level."""
    from phybs_gb300 import meshes as M
    chain = np.array([[0, 1, 2, 3], [3, 4, 5, 6], [6, 7, 8, 9]])
    assert M.pbd_levels(chain, 10) == 3
    apart = np.array([[0, 1, 2, 3], [4, 5, 6, 7], [8, 9, 10, 11]])
    assert M.pbd_levels(apart, 12) == 1
    m = M.box_mesh(10, 10, 40, edge=0.005, seed=0)
    assert M.pbd_levels(m.tets, m.n_nodes) == 920
