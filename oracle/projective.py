"""FP64 restatement of the reference's projective-dynamics integrator, and a
binding of the FP32 restatement of its strain-based PBD integrator.

TEST INFRASTRUCTURE ONLY: the checkers for pbs_pd_step and pbs_pbd_step.

Projective dynamics, ProjDynamic.cpp (driven by fvm.cpp:167-170, 300-307):

    s = (x + dt v + dt^2 w f) m / dt^2         (doProjDynamics, :442-465)
    A = M / dt_m^2 + sum_t k vol_t A_t^T A_t    (buildGlobalSolverMatrix, :48-100)
    repeat `iterations`:
        R_t = U V^T from JacobiSVD(F_t) with det U, det V made positive by
              negating their first columns         (projectLocalConstraints2, :351-434)
        b = s + sum_t k vol_t A_t^T vec(R_t)
        p = A^-1 b                                 (solveGlobalStep, :436-440)
    v = (p - x) / dt 0.99,  x = p

A_t maps a tet's corner positions to its deformation gradient, so
A_t^T A_t = (w_a . w_b) I_3 for corners a, b with w_1..3 the rows of Dm^-1 and
w_0 = -(w_1 + w_2 + w_3), and the corner-a block of A_t^T vec(R) is R w_a.
The reference factorises A with MKL Pardiso (FP32); here scipy's sparse LU in
FP64.  numpy's SVD, like Eigen's JacobiSVD, orders singular values
descending, so the determinant fix flips the same (largest) direction.

Strain-based PBD: ``pbd_step`` runs orc_pbd_step of phybs_oracle.cpp, the
serial Gauss-Seidel sweep of PosBaseDynamic.cpp:12-117 in FP32 and the
reference's operation order (pinned bit for bit to the reference's own build
by tests/golden/dynamics_*.npz).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import restated as O


def corner_gradients(dinv):
    """(T, 4, 3): w_0 = -(sum of the rows of Dm^-1), w_1..3 = its rows."""
    dinv = np.asarray(dinv, np.float64).reshape(-1, 3, 3)
    return np.concatenate([-dinv.sum(axis=1, keepdims=True), dinv], axis=1)


def pd_matrix(mass, tets, dinv, vol, dt_matrix, stiffness=1e6):
    """The N x N scalar matrix L with A = L (x) I_3 (scipy CSR, FP64)."""
    import scipy.sparse as sp
    tets = np.asarray(tets, np.int64).reshape(-1, 4)
    w = corner_gradients(dinv)
    wt = stiffness * np.asarray(vol, np.float64).reshape(-1)
    G = wt[:, None, None] * np.einsum("tad,tbd->tab", w, w)
    rows = np.repeat(tets, 4, axis=1).reshape(-1)
    cols = np.tile(tets, (1, 4)).reshape(-1)
    n = np.asarray(mass).shape[0]
    L = sp.csr_matrix((G.reshape(-1), (rows, cols)), shape=(n, n))
    return (L + sp.diags(np.asarray(mass, np.float64) / (dt_matrix * dt_matrix))).tocsc()


def rotations(x, tets, dinv, flip=0):
    """(T, 3, 3) R = U V^T with the reference's determinant fix (flip = 0:
    negate the first, largest-singular-value column of U or V when its
    determinant is negative; flip = 2 negates the last column instead, the
    usual polar-decomposition convention, for tests that tell them apart)."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    tets = np.asarray(tets, np.int64).reshape(-1, 4)
    dinv = np.asarray(dinv, np.float64).reshape(-1, 3, 3)
    Ds = np.stack([x[tets[:, c]] - x[tets[:, 0]] for c in (1, 2, 3)], axis=2)
    U, _, Vt = np.linalg.svd(Ds @ dinv)
    V = Vt.transpose(0, 2, 1).copy()
    U = U.copy()
    U[np.linalg.det(U) < 0, :, flip] *= -1.0
    V[np.linalg.det(V) < 0, :, flip] *= -1.0
    return U @ V.transpose(0, 2, 1)


def pd_step(x, v, mass, inv_mass, tets, dinv, vol, f, dt=0.03, dt_matrix=None, stiffness=1e6, iterations=5,
            flip=0):
    """One doProjDynamics step from (x, v) with forces f (gravity + external):
    returns (x', v')."""
    import scipy.sparse.linalg as sla
    x = np.asarray(x, np.float64).reshape(-1, 3)
    v = np.asarray(v, np.float64).reshape(-1, 3)
    f = np.asarray(f, np.float64).reshape(-1, 3)
    m = np.asarray(mass, np.float64).reshape(-1)
    im = np.asarray(inv_mass, np.float64).reshape(-1)
    tets = np.asarray(tets, np.int64).reshape(-1, 4)
    dtm = dt if dt_matrix is None else dt_matrix
    lu = sla.splu(pd_matrix(m, tets, dinv, vol, dtm, stiffness))
    s = (x + dt * v + (dt * dt * im)[:, None] * f) * (m / (dt * dt))[:, None]
    w = corner_gradients(dinv)
    wt = stiffness * np.asarray(vol, np.float64).reshape(-1)
    p = x.copy()
    for _ in range(iterations):
        R = rotations(p, tets, dinv, flip)
        c = wt[:, None, None] * np.einsum("tde,tae->tad", R, w)  # (T, 4, 3): k vol R w_a
        b = s.copy()
        for a in range(4):
            np.add.at(b, tets[:, a], c[:, a])
        p = lu.solve(b)
    return p, (p - x) / dt * 0.99


def rest_eigen32(pos, tets, pin_mask, density=1000.0, gravity=9.8):
    """(Dm^-1 row-major (T, 9), inverse masses, gravity (N, 3)) in FP32 exactly
    as the reference's TetMesh forms them (orc_rest_eigen32): the rest data
    of the strain-based PBD step."""
    lib = O.lib()
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    tets = np.ascontiguousarray(tets, np.int32).reshape(-1, 4)
    pm = np.ascontiguousarray(pin_mask, np.int32).reshape(-1)
    n, t = pos.shape[0], tets.shape[0]
    dinv, w, gy = np.zeros((t, 9), np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    lib.orc_rest_eigen32(C.c_int(n), p(pos), C.c_int(t), p(tets), C.c_float(density), C.c_float(gravity), p(pm),
                         p(dinv), p(w), p(gy))
    grav = np.zeros((n, 3), np.float32)
    grav[:, 1] = gy
    return dinv, w, grav


def pbd_step(x, v, inv_mass, tets, dinv, forces, dt, iterations=5, stretch=(1.0, 1.0, 1.0), shear=(0.8, 0.8, 0.8),
             eps=1e-6):
    """One strain-based PBD step in FP32 (orc_pbd_step): returns (x', v')."""
    lib = O.lib()
    pos = np.ascontiguousarray(x, np.float32).reshape(-1).copy()
    vel = np.ascontiguousarray(v, np.float32).reshape(-1).copy()
    tets = np.ascontiguousarray(tets, np.int32).reshape(-1, 4)
    dinv = np.ascontiguousarray(dinv, np.float32).reshape(-1, 9)
    im = np.ascontiguousarray(inv_mass, np.float32).reshape(-1)
    f = np.ascontiguousarray(forces, np.float32).reshape(-1)
    st = np.ascontiguousarray(stretch, np.float32)
    sh = np.ascontiguousarray(shear, np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    lib.orc_pbd_step(C.c_int(im.shape[0]), C.c_int(tets.shape[0]), p(tets), p(dinv), p(im), p(f), C.c_float(dt),
                     C.c_int(iterations), p(st), p(sh), C.c_float(eps), p(pos), p(vel))
    return pos.reshape(-1, 3), vel.reshape(-1, 3)
