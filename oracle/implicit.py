"""FP64 restatement of the reference's GPU backward-Euler step.

TEST INFRASTRUCTURE ONLY: the checker for pbs_backward_euler_step.  The
reference runs the step as CUDAInterface::computeInnerforces +
computeGlobalStiffnessMatrix + doBackEuler (CUDAInterface.cu:784-884):

    f = elastic forces + gravity; a pinned node's force is replaced by the
        spring 1e8 (X - x) (addFixContraintsAndGravity, CUDAInterface.cu:327-344)
    b = h f + M v                                   (setRHSofLinearSystem, :418-433)
    A = M (1 + alpha h) + h (h + beta) K,  K = -df/dx
                                                    (scaleDeviceArray :848, setMassScaled :725)
    A v' = b (cuSOLVER Cholesky, :875),  x' = x + h v'

with M the lumped masses (1e8 at pinned nodes) and alpha = beta = 0.02.  Its
GPU code does not build with CUDA 13; the parity anchor is the reference's CPU
element stiffness (IsotropicMaterial::computeStiffnessMatrixFromPos, pinned by
tests/golden/implicit_*.npz) and its forces (already pinned by the solver
fixtures).  Here: the closed-form neo-Hookean element stiffness (the exact
Hessian of the energy both materials share), scipy sparse assembly and a
direct solve, all FP64.
"""
from __future__ import annotations

import numpy as np

from . import restated as O


def element_stiffness(x, tets, dinv, vol, mu, lam):
    """(T, 12, 12) K = -df/dx, row/column index 3 corner + dof.  With
    F = I + sum_c u_c w_c^T (w_1..3 the rows of Dm^-1, w_0 = -their sum),
    H = F^-T, a_c = H w_c:
        K[c d, c' e] = vol (mu (w_c . w_c') delta_de + lam a_c[d] a_c'[e]
                            + (mu - lam ln J) a_c[e] a_c'[d])."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    tets = np.asarray(tets, np.int64).reshape(-1, 4)
    dinv = np.asarray(dinv, np.float64).reshape(-1, 3, 3)
    w = np.concatenate([-dinv.sum(axis=1, keepdims=True), dinv], axis=1)  # (T, 4, 3)
    Ds = np.stack([x[tets[:, c]] - x[tets[:, 0]] for c in (1, 2, 3)], axis=2)  # columns x_c - x_0
    F = Ds @ dinv
    H = np.linalg.inv(F).transpose(0, 2, 1)
    lnJ = np.log(np.linalg.det(F))
    mu = np.asarray(mu, np.float64).reshape(-1)
    lam = np.asarray(lam, np.float64).reshape(-1)
    v = np.abs(np.asarray(vol, np.float64).reshape(-1))
    a = np.einsum("tde,tce->tcd", H, w)  # a[t, c, d] = (H w_c)_d
    ww = np.einsum("tce,tfe->tcf", w, w)
    K = (mu[:, None, None, None, None] * ww[:, :, None, :, None] * np.eye(3)[None, None, :, None, :]
         + lam[:, None, None, None, None] * np.einsum("tcd,tfe->tcdfe", a, a)
         + (mu - lam * lnJ)[:, None, None, None, None] * np.einsum("tce,tfd->tcdfe", a, a))
    return (v[:, None, None, None, None] * K).reshape(-1, 12, 12)


def assemble(n, tets, Ke):
    """Global 3n x 3n CSR of the element matrices (scipy)."""
    import scipy.sparse as sp
    tets = np.asarray(tets, np.int64).reshape(-1, 4)
    dof = (3 * tets[:, :, None] + np.arange(3)[None, None, :]).reshape(-1, 12)
    rows = np.repeat(dof, 12, axis=1).reshape(-1)
    cols = np.tile(dof, (1, 12)).reshape(-1)
    return sp.csr_matrix((Ke.reshape(-1), (rows, cols)), shape=(3 * n, 3 * n))


def backward_euler_step(x, v, rest, tets, pin_mask, mu, lam, h=0.03, alpha=0.02, beta=0.02, ext=None,
                        material=0, density=1000.0, gravity=9.8):
    """One step from (x, v): returns (x', v', A, b)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    x = np.asarray(x, np.float64).reshape(-1, 3)
    v = np.asarray(v, np.float64).reshape(-1, 3)
    rest = np.asarray(rest, np.float64).reshape(-1, 3)
    pm = np.asarray(pin_mask).reshape(-1) > 0
    n = x.shape[0]
    r = O.rest(rest, tets, pm.astype(np.int32), density=density, prec=64)
    f, _ = O.node_eval(x, tets, r.dinv, r.an, r.vol, mu, lam, material=material, hessian_closed=1, prec=64)
    f = f.copy()
    f[:, 1] += r.grav_y * (gravity / 9.8)
    if ext is not None:
        f += np.asarray(ext, np.float64).reshape(-1, 3)
    f[pm] = 1e8 * (rest[pm] - x[pm])
    m = r.mass
    b = (h * f + m[:, None] * v).reshape(-1)
    K = assemble(n, tets, element_stiffness(x, tets, r.dinv, r.vol, mu, lam))
    A = sp.diags(np.repeat(m * (1.0 + alpha * h), 3)) + (h * (h + beta)) * K
    vn = sla.spsolve(A.tocsc(), b).reshape(-1, 3)
    return x + h * vn, vn, A, b
