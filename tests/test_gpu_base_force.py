"""The per-step base force of the incremental stress, in double-float.

With incremental stress the passes evaluate P(F) - P(F_base) in FP32 and add
the elastic force at the base, formed once per step by k_ref_tet in the
double-float type (FP32 pairs, about 2^-44 relative per operation; FP64 only
for 1 / J and log1p per tet).  An error in that force is a floor under the
residual, so it must stay far below FP32's 6e-8: pbs_eval_base_force runs the
same kernels on given positions, and the node forces must match FP64 forces
of the same definition (the device's FP32 rest data: Dm^-1 rows, signed
volume, mu, lambda; F = I + Du Dm^-1) within 1e-11 of the largest force, on
the reference's deformed probe states and on a strongly stretched pull.  (The
restatement forms F = Ds Dm^-1 from absolute positions instead; with Dm^-1
rounded to FP32 the two differ by Dm (Dm^-1)_fp32 - I, about 1e-7, which is
why the FP64 forces here are formed in the device's own definition; they
agree with the restatement's to 2e-15 when Dm^-1 is not rounded.)
"""
import numpy as np
import pytest

from phybs_gb300 import _lib as L
from phybs_gb300 import meshes as M
from phybs_gb300.solver import DescentSolver, lame_arrays
from tests._util import load_golden, rel_max

pytestmark = pytest.mark.gpu

TOL = 1e-11


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


def _fp64_forces(s, mesh, x, mu, lam):
    """FP64 node forces in the device's convention: F = I + Du Dm^-1 with Du
    the displacements' FP32 hi words (as the step's base uses them) and the
    device's own FP32 rest data (Dm^-1 rows, signed volume); P = mu (F - F^-T)
    + lambda ln J F^-T (IsotropicNeohookeanMaterial.cpp:104); corner forces
    -svol P Dm^-T, corner 0 minus the others' sum, added per node."""
    dinv, svol, _, _ = s.rest_data()
    X = mesh.rest.astype(np.float32)
    hi = (x.astype(np.float32) - X).astype(np.float64)  # FP32 subtraction, as the device splits it
    d = dinv.astype(np.float64)
    sv = svol.astype(np.float64)
    t = np.asarray(mesh.tets, np.int64)
    du = np.stack([hi[t[:, c]] - hi[t[:, 0]] for c in (1, 2, 3)], axis=2)  # (T, xyz, corner)
    F = np.eye(3)[None] + du @ d
    J = np.linalg.det(F)
    FiT = np.transpose(np.linalg.inv(F), (0, 2, 1))
    mu = np.asarray(mu, np.float64)[:, None, None]
    lam = np.asarray(lam, np.float64)[:, None, None]
    P = mu * (F - FiT) + lam * np.log(J)[:, None, None] * FiT
    H = -sv[:, None, None] * (P @ np.transpose(d, (0, 2, 1)))  # columns: corners 1..3
    f = np.zeros((mesh.n_nodes, 3))
    for c in (1, 2, 3):
        np.add.at(f, t[:, c], H[:, :, c - 1])
    np.add.at(f, t[:, 0], -H.sum(axis=2))
    return f


def _check(s, mesh, x, mu, lam):
    fb = s.eval_base_force(x)
    f64 = _fp64_forces(s, mesh, x, mu, lam)
    pins = mesh.pin_mask() > 0
    f64[pins] = 0.0
    fb[pins] = 0.0
    err = rel_max(fb, f64)
    return err


@pytest.mark.parametrize("name", ["bar_small", "ellipsoid_small"])
def test_base_force_matches_fp64_on_reference_probes(name):
    g = load_golden(name)
    mesh = M.TetMeshData(g["rest"], g["tets"], g["pins"], g["young"], g["poisson"])
    s = DescentSolver(mesh, mu=g["mu"], lam=g["lam"])
    err = _check(s, mesh, g["probe_x"], g["mu"], g["lam"])
    print(f"{name}: max |f_base - f_fp64| / max |f_fp64| = {err:.2e}")
    assert err < TOL
    s.close()


def test_base_force_matches_fp64_on_a_stretched_pull():
    m = M.bar_mesh(12, 4, 4, edge=0.025, young=5e4, poisson=0.4)
    x = m.rest.astype(np.float64).copy()
    x[:, 0] *= 1.6  # 60% stretch along the bar
    x[:, 1] += 0.05 * np.sin(3.0 * x[:, 0])
    mu, lam = lame_arrays(m.young, m.poisson)
    s = DescentSolver(m)
    err = _check(s, m, x.astype(np.float32), mu, lam)
    print(f"stretched bar: max |f_base - f_fp64| / max |f_fp64| = {err:.2e}")
    assert err < TOL
    # the stretched state's forces are far from zero: the bar tests accuracy, not a null case
    assert np.abs(s.eval_base_force(x.astype(np.float32))).max() > 1.0
    s.close()


def test_base_force_rejects_the_stretch_material():
    m = M.bar_mesh(4, 2, 2, edge=0.025)
    s = DescentSolver(m, material=L.PBS_MATERIAL_STRETCH)
    with pytest.raises(L.PhybsError):
        s.eval_base_force(m.rest.astype(np.float32))
    s.close()
