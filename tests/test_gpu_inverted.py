"""Near-inverted tets: the FP64 stress branch against the FP64 restatement and
the reference's own forces.

The probe state (tests/golden/probe_inverted_bar.npz, made by
``make_golden.py inverted``) squeezes the 768-tet bar's y extent by up to
1e5 along its length, so det F runs from 1 down to ~1e-5 (216 tets between
1e-5 and 1e-3) with no tet inverted.  A tet with det F < 1e-3 (or, for the
stretch-based material, with smallest singular value below 0.3) takes its
stress in FP64, with F = Ds Dm^-1 formed from the absolute positions as the
reference defines it; the reference does the stretch-based material through
its modified SVD (IsotropicMaterial.cpp:16-60) in FP32 throughout.

Bars: the FP64-branch tets' corner forces within 1e-5 of the all-FP64
restatement, tet by tet (max-norm per tet, relative to the larger of the
tet's largest force and its force at unit strain, mu vol |Dm^-1|), on the
device's own rest data; every other tet within max(1e-5, 2^-19 / sigma_min)
of it per tet -- the conditioning of an FP32 evaluation, whose F carries an
absolute rounding of a few 2^-24, through a stress that varies as
1 / sigma_min; assembled node
forces within 1e-5 of the FP64 restatement, and no further from it than the
reference's FP32 forces are from the FP64 restatement on the reference's rest
data (both errors are printed); and the probe's count of FP64-branch tets
equals the tets the FP64 restatement puts below det F = 1e-3 (plus, for the
stretch material, those with sigma_3 < 0.3).
"""
import numpy as np
import pytest

from oracle import restated as O
from phybs_gb300 import _lib as L
from phybs_gb300 import meshes as M
from phybs_gb300.solver import DescentSolver
from tests._util import elastic_from_ref, load_golden, rel_max

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


@pytest.fixture(scope="module")
def g():
    return load_golden("probe_inverted_bar")


def _solver(g, material):
    m = M.TetMeshData(g["rest"], g["tets"], g["pins"], g["young"], g["poisson"], name="probe_inverted_bar")
    return DescentSolver(m, material=material, mu=g["mu"], lam=g["lam"])


def _device_rest(s):
    """The device's rest data as the restatement takes it: Dm^-1 (T, 3, 3)
    row-major, AN = -(det Dm / 6) Dm^-T, volumes."""
    dinv, svol, _, _ = s.rest_data()
    dinv = np.asarray(dinv, np.float64).reshape(-1, 3, 3)
    svol = np.asarray(svol, np.float64)
    an = -svol[:, None, None] * dinv.transpose(0, 2, 1)
    return dinv, an, np.abs(svol)


def _per_tet_rel(a, b, scale):
    """max |a - b| per tet over the larger of the tet's largest force and its
    stress scale: a nearly stress-free tet (a rigid turn) has forces near zero
    that no FP32 evaluation resolves relative to themselves."""
    a = np.asarray(a, np.float64).reshape(-1, 12)
    b = np.asarray(b, np.float64).reshape(-1, 12)
    return np.abs(a - b).max(1) / np.maximum(np.abs(b).max(1), scale)


def _stress_scale(g, dinv, vol):
    """Corner-force size of a tet at unit strain: mu vol |Dm^-1|_F."""
    return np.asarray(g["mu"], np.float64) * vol * np.linalg.norm(dinv.reshape(-1, 9), axis=1)


def _deformation(g, dinv):
    x = g["probe_x"].astype(np.float64)
    t = g["tets"]
    Ds = np.stack([x[t[:, 1]] - x[t[:, 0]], x[t[:, 2]] - x[t[:, 0]], x[t[:, 3]] - x[t[:, 0]]], axis=2)
    return Ds @ dinv


@pytest.mark.parametrize("material", [L.PBS_MATERIAL_STRETCH, L.PBS_MATERIAL_NEOHOOKEAN])
def test_near_inverted_tets_take_the_fp64_branch(g, material):
    s = _solver(g, material)
    dinv, an, vol = _device_rest(s)
    F = _deformation(g, dinv)
    J = np.linalg.det(F)
    assert (J > 0).all() and ((J > 1e-5) & (J < 1e-3)).sum() >= 200
    cf, _, _ = s.eval_tets(g["probe_x"])
    n64 = s.eval_fp64_svd_count()
    stretch = int(material == L.PBS_MATERIAL_STRETCH)
    f64, _, _ = O.tet_eval(g["probe_x"], g["tets"], dinv, an, vol, g["mu"], g["lam"], material=stretch, prec=64,
                           energy=False, hdiag=False)
    err = _per_tet_rel(cf, f64, _stress_scale(g, dinv, vol))
    sig_min = np.linalg.svd(F, compute_uv=False)[:, 2]
    near = J < 1e-3
    fp64 = (near | (sig_min < 0.3)) if stretch else near
    bound = np.maximum(TOL, 2.0 ** -19 / sig_min)
    print(f"material {material}: per-tet error vs FP64: FP64-branch tets {err[fp64].max():.2e}, "
          f"others {err[~fp64].max():.2e} (worst error / bound {(err[~fp64] / bound[~fp64]).max():.2f}); "
          f"FP64-branch tets {n64} of {len(J)}")
    assert err[fp64].max() < TOL, err[fp64].max()
    r = np.where(fp64, 0.0, err / bound)
    w = int(np.argmax(r))
    assert r[w] <= 1.0, dict(tet=w, err=err[w], bound=bound[w], detF=J[w], sigma_min=sig_min[w],
                             max_force=np.abs(f64[w]).max())
    if stretch:
        # the device classifies from its FP32 spectrum: a tet at the 0.3 edge
        # may fall on either side
        edge = int(((sig_min > 0.297) & (sig_min < 0.303) & ~near).sum())
        assert abs(n64 - int(fp64.sum())) <= edge, (n64, int(fp64.sum()), edge)
    else:
        assert n64 == int(near.sum()), (n64, int(near.sum()))
    s.close()


@pytest.mark.parametrize("material,key", [(L.PBS_MATERIAL_STRETCH, "probe_force_stretch"),
                                          (L.PBS_MATERIAL_NEOHOOKEAN, "probe_force_nh")])
def test_near_inverted_node_forces_vs_reference_and_fp64(g, material, key):
    s = _solver(g, material)
    dinv, an, vol = _device_rest(s)
    stretch = int(material == L.PBS_MATERIAL_STRETCH)
    f, _ = s.eval_nodes(g["probe_x"])
    f = f.astype(np.float64)
    f[g["pins"]] = 0.0
    f64, _ = O.node_eval(g["probe_x"], g["tets"], dinv, an, vol, g["mu"], g["lam"], material=stretch, prec=64)
    f64[g["pins"]] = 0.0
    # the reference against FP64 on its own rest data
    r64, _ = O.node_eval(g["probe_x"], g["tets"], g["dminv"], g["an"], g["vol"], g["mu"], g["lam"],
                         material=stretch, prec=64)
    r64[g["pins"]] = 0.0
    err_dev, err_ref = rel_max(f, f64), rel_max(elastic_from_ref(g, key), r64)
    print(f"material {material}: node forces vs FP64: device {err_dev:.2e}, reference (FP32) {err_ref:.2e}")
    assert err_dev < TOL
    assert err_dev <= max(err_ref, 2e-6)
    s.close()
