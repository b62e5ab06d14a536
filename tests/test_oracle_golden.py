"""Pin the restated CPU oracle to the reference's own outputs (tests/golden).

The fixtures were produced by the reference CPU solver compiled headless
(tests/golden/make_golden.py).  The restatement (oracle/phybs_oracle.cpp) is
the checker for the GPU tests, so it must reproduce the reference first.
"""
import numpy as np
import pytest

from oracle import restated as O
from tests._util import bbox_diag, elastic_from_ref, golden_names, load_golden, rel_max

NAMES = golden_names()


@pytest.fixture(scope="module", params=NAMES)
def g(request):
    d = load_golden(request.param)
    d["name"] = request.param
    return d


def pin_mask(g):
    m = np.zeros(g["rest"].shape[0], np.int32)
    m[g["pins"]] = 1
    return m


def test_fixture_set_complete():
    assert {"bar_small", "bar_config1", "ellipsoid_small", "model_bar", "model_dragon"} <= set(NAMES)


def test_rest_state(g):
    """TetMesh.cpp:186-216: volumes, lumped masses (pins 1e8), Dm^-1, AN, gravity."""
    for prec, tol in ((32, 2e-6), (64, 2e-6)):
        r = O.rest(g["rest"], g["tets"], pin_mask(g), prec=prec)
        assert rel_max(r.vol, g["vol"]) < tol
        assert rel_max(r.mass, g["mass"]) < tol
        assert rel_max(r.dinv, g["dminv"]) < 5e-6
        assert rel_max(r.an, g["an"]) < 5e-6
        assert rel_max(r.grav_y, g["gravity"][:, 1]) < tol
    r = O.rest(g["rest"], g["tets"], pin_mask(g), prec=64)
    # the area-weighted normals are -(det Dm / 6) Dm^-T exactly
    an = -r.svol[:, None, None] * np.transpose(r.dinv, (0, 2, 1))
    assert rel_max(an, r.an) < 1e-12


def test_lame_matches_reference(g):
    mu, lam = O.lame(np.full(g["tets"].shape[0], g["young"]), np.full(g["tets"].shape[0], g["poisson"]))
    assert np.array_equal(mu, g["mu"]) and np.array_equal(lam, g["lam"])


def _probe(g, material, prec):
    r = O.rest(g["rest"], g["tets"], pin_mask(g), prec=64)
    f, hd = O.node_eval(g["probe_x"], g["tets"], g["dminv"], g["an"], g["vol"], g["mu"], g["lam"],
                        material=material, hessian_closed=0, prec=prec)
    f[g["pins"]] = 0.0
    return r, f, hd


@pytest.mark.parametrize("prec", [32, 64])
def test_neohookean_forces(g, prec):
    """IsotropicNeohookeanMaterial::computeInnerForceFromPos at a deformed state."""
    _, f, _ = _probe(g, 0, prec)
    assert rel_max(f, elastic_from_ref(g, "probe_force_nh")) < 2e-5


@pytest.mark.parametrize("prec", [32, 64])
def test_stretch_forces(g, prec):
    """IsotropicMaterial::computeInnerForcesfromFhats2 (P = U P^ V^T)."""
    _, f, _ = _probe(g, 1, prec)
    assert rel_max(f, elastic_from_ref(g, "probe_force_stretch")) < 2e-5


def test_openmp_force_evaluation_port(g):
    """The port of the reference's OpenMP computeInnerForcesfromFhats2(nthreads)
    (the CPU comparator bench.py times) gives the reference's forces at any
    thread count: its locked scatter only reorders the FP32 sums."""
    ref = elastic_from_ref(g, "probe_force_stretch")
    for threads in (1, 3):
        f = O.forces_fhats2_omp(g["probe_x"], g["tets"], g["dminv"], g["an"], g["mu"], g["lam"], threads=threads)
        f = f.astype(np.float64)
        f[g["pins"]] = 0.0
        assert rel_max(f, ref) < 2e-5


def test_energy(g):
    _, e, _ = O.tet_eval(g["probe_x"], g["tets"], g["dminv"], g["an"], g["vol"], g["mu"], g["lam"], clamp=0,
                         forces=False, hdiag=False)
    assert rel_max(e, g["probe_energy"]) < 2e-5


def test_hessian_diagonal(g):
    """diag(computeGlobalStiffnessMatrixFromPos) at the deformed probe: the SVD
    (Xu et al.) route and the closed form agree with each other to FP64 and with
    the reference to its FP32 noise, which reaches ~1e-3 on nearly undeformed
    tets (see test_hessian_diagonal_at_rest)."""
    hds = []
    for closed in (0, 1):
        _, hd = O.node_eval(g["probe_x"], g["tets"], g["dminv"], g["an"], g["vol"], g["mu"], g["lam"],
                            hessian_closed=closed, prec=64)
        assert rel_max(hd, g["probe_hdiag"]) < 5e-3
        hds.append(hd)
    assert rel_max(hds[1], hds[0]) < 1e-5


def test_hessian_diagonal_at_rest(g):
    """At the rest shape all stretches are equal; the reference's FP32
    eps-perturbed SVD route carries percent-level noise there (the 2x2 solves
    divide by sigma_l^2 - sigma_k^2 ~ 2e-6).  Its error against the FP64 closed
    form is bounded, and the FP64 SVD route agrees with the closed form."""
    _, hd_closed = O.node_eval(g["rest"], g["tets"], g["dminv"], g["an"], g["vol"], g["mu"], g["lam"],
                               hessian_closed=1, prec=64)
    _, hd_svd = O.node_eval(g["rest"], g["tets"], g["dminv"], g["an"], g["vol"], g["mu"], g["lam"],
                            hessian_closed=0, prec=64)
    assert rel_max(hd_svd, hd_closed) < 1e-4
    assert rel_max(g["rest_hdiag"], hd_closed) < 0.05


def test_element_stiffness_diagonal(g):
    _, _, hd = O.tet_eval(g["probe_x"], g["tets"], g["dminv"], g["an"], g["vol"], g["mu"], g["lam"],
                          hessian_closed=1, forces=False, energy=False)
    k0 = np.diag(g["probe_k0"]).reshape(4, 3)
    assert rel_max(hd[0], k0) < 5e-3  # reference FP32 noise on near-rest tets


def test_trajectory_fp32(g):
    """DescentOptimize::doDescentOpt steps: positions within 1e-4 of the
    bounding-box diagonal (the spec bar) -- the FP32 restatement stays
    near 1e-5 -- and identical line-search outcomes (alpha)."""
    pm = pin_mask(g)
    r = O.rest(g["rest"], g["tets"], pm, prec=32)
    p = O.make_params(h=float(g["h"]), max_iters=int(g["iters"]))
    st = O.StepState(g["traj_x0"])
    diag = bbox_diag(g["rest"])
    for s in range(g["traj_x"].shape[0]):
        stats = O.step(st, p, g["tets"], r, g["mu"], g["lam"], pm, prec=32)
        err = np.abs(st.x0 - g["traj_x"][s]).max() / diag
        assert err < 1e-4, (g["name"], s, err)
        assert abs(stats.alpha - g["traj_scalars"][s, 0]) < 1e-6
        assert np.abs(st.v - g["traj_v"][s]).max() <= 1e-3 * max(np.abs(g["traj_v"][s]).max(), 1e-6) + 1e-4


def test_trajectory_fp64_error_is_stated(g):
    """The reference's FP32 step against the all-FP64 restatement: recorded, and
    far inside the parity bar."""
    pm = pin_mask(g)
    r = O.rest(g["rest"], g["tets"], pm, prec=64)
    p = O.make_params(h=float(g["h"]), max_iters=int(g["iters"]))
    st = O.StepState(g["traj_x0"])
    diag = bbox_diag(g["rest"])
    errs = []
    for s in range(g["traj_x"].shape[0]):
        O.step(st, p, g["tets"], r, g["mu"], g["lam"], pm, prec=64)
        errs.append(np.abs(st.x0 - g["traj_x"][s]).max() / diag)
    assert max(errs) < 5e-4, errs


def test_stiffness_pattern_restated(g):
    if "csr_row" not in g:
        pytest.skip("no CSR in this fixture")
    row, col, diag, kid = O.stiffness_pattern(g["tets"], g["rest"].shape[0])
    assert np.array_equal(row, g["csr_row"])
    assert np.array_equal(col, g["csr_col"])
    assert np.array_equal(diag, g["csr_diag"])
    assert np.array_equal(kid, g["csr_kid"])
