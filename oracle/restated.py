"""ctypes binding of the restated CPU oracle (phybs_oracle.cpp) -- test infrastructure.

All arrays cross as float64; ``prec`` (32 or 64) selects the arithmetic the
C++ side evaluates in.  Layouts: positions (N, 3); tets (T, 4) int32; per-tet
3x3 blocks (Dm^-1, AN) row-major as (T, 3, 3).
"""
from __future__ import annotations

import ctypes as C
import os
import dataclasses

import numpy as np

from . import ORACLE_SO, build

_lib = None


def lib():
    global _lib
    if _lib is None:
        build(reference=False)
        _lib = C.CDLL(ORACLE_SO)
    return _lib


class OrcParams(C.Structure):
    _fields_ = [("h", C.c_float), ("max_iters", C.c_int), ("tol", C.c_float), ("control", C.c_int),
                ("alpha0", C.c_float), ("alpha_min", C.c_float), ("alpha_shrink", C.c_float),
                ("line_search_every", C.c_int), ("hessian_every", C.c_int), ("n_profile", C.c_int),
                ("profile_k", C.c_int * 4), ("profile_rho", C.c_float * 4), ("damping", C.c_float),
                ("warm_start", C.c_float), ("body_force_scale", C.c_float),
                ("energy_clamp", C.c_int), ("material", C.c_int), ("hessian_closed", C.c_int),
                ("alpha_grow", C.c_float)]


class OrcStats(C.Structure):
    _fields_ = [("passes", C.c_int), ("k_final", C.c_int), ("rejections", C.c_int), ("converged", C.c_int),
                ("alpha", C.c_double), ("energy", C.c_double), ("energy_old", C.c_double), ("rho", C.c_double),
                ("omega", C.c_double), ("residual_ratio", C.c_double), ("residual0", C.c_double)]


def set_threads(n: int = 0) -> int:
    """Threads of the per-tet loops (0 = all host cores); returns the count in
    effect.  Results do not depend on it."""
    if n <= 0:
        n = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    return int(lib().orc_set_threads(C.c_int(n)))


def make_params(h=0.03, max_iters=96, tol=0.0, control=0, alpha0=0.1, alpha_min=0.01, alpha_shrink=0.7,
                line_search_every=8, hessian_every=32, profile=((1, 0.96), (7, 0.991), (10, 0.999)),
                damping=0.99, warm_start=0.2, body_force_scale=2.0, energy_clamp=0, material=0,
                hessian_closed=0, alpha_grow=1.0) -> OrcParams:
    p = OrcParams()
    p.h, p.max_iters, p.tol, p.control = h, max_iters, tol, control
    p.alpha0, p.alpha_min, p.alpha_shrink = alpha0, alpha_min, alpha_shrink
    p.line_search_every, p.hessian_every = line_search_every, hessian_every
    p.n_profile = len(profile)
    for i, (k, r) in enumerate(profile):
        p.profile_k[i] = k
        p.profile_rho[i] = r
    p.damping, p.warm_start, p.body_force_scale = damping, warm_start, body_force_scale
    p.energy_clamp, p.material, p.hessian_closed = energy_clamp, material, hessian_closed
    p.alpha_grow = alpha_grow
    return p


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


@dataclasses.dataclass
class Rest:
    dinv: np.ndarray   # (T, 3, 3)
    an: np.ndarray     # (T, 3, 3)
    vol: np.ndarray    # (T,)
    svol: np.ndarray   # (T,)
    mass: np.ndarray   # (N,) pins = 1e8
    grav_y: np.ndarray  # (N,)


def rest(pos, tets, pin_mask, density=1000.0, prec=64) -> Rest:
    pos, tets, pm = _d(pos).reshape(-1, 3), _i(tets).reshape(-1, 4), _i(pin_mask)
    n, t = pos.shape[0], tets.shape[0]
    out = Rest(np.zeros((t, 3, 3)), np.zeros((t, 3, 3)), np.zeros(t), np.zeros(t), np.zeros(n), np.zeros(n))
    lib().orc_rest(C.c_int(prec), C.c_int(n), _p(pos), C.c_int(t), _p(tets), C.c_double(density), _p(pm),
                   _p(out.dinv), _p(out.an), _p(out.vol), _p(out.svol), _p(out.mass), _p(out.grav_y))
    return out


def lame(young, poisson, reference_lambda=True):
    """mu = E / (2 (1 + nu)); lambda = 2 mu / (1 - 2 nu) as the reference computes it
    (IsotropicNeohookeanMaterial.cpp:15-16), or the textbook 2 mu nu / (1 - 2 nu)."""
    e = np.asarray(young, np.float32)
    nu = np.asarray(poisson, np.float32)
    mu = (np.float32(0.5) * e / (np.float32(1) + nu)).astype(np.float32)
    lam = (mu * np.float32(2) / (np.float32(1) - np.float32(2) * nu)).astype(np.float32)
    if not reference_lambda:
        lam = (lam * nu).astype(np.float32)
    return mu, lam


def tet_eval(x, tets, dinv, an, vol, mu, lam, material=0, clamp=0, hessian_closed=0, prec=64,
             forces=True, energy=True, hdiag=True):
    x, tets = _d(x).reshape(-1, 3), _i(tets).reshape(-1, 4)
    t = tets.shape[0]
    cf = np.zeros((t, 4, 3)) if forces else None
    en = np.zeros(t) if energy else None
    hd = np.zeros((t, 4, 3)) if hdiag else None
    lib().orc_tet_eval(C.c_int(prec), C.c_int(material), C.c_int(clamp), C.c_int(hessian_closed),
                       C.c_int(x.shape[0]), _p(x), C.c_int(t), _p(tets), _p(_d(dinv)), _p(_d(an)), _p(_d(vol)),
                       _p(_d(mu)), _p(_d(lam)), _p(cf), _p(en), _p(hd))
    return cf, en, hd


def node_eval(x, tets, dinv, an, vol, mu, lam, material=0, hessian_closed=0, prec=64):
    x, tets = _d(x).reshape(-1, 3), _i(tets).reshape(-1, 4)
    f = np.zeros_like(x)
    hd = np.zeros_like(x)
    lib().orc_node_eval(C.c_int(prec), C.c_int(material), C.c_int(hessian_closed), C.c_int(x.shape[0]), _p(x),
                        C.c_int(tets.shape[0]), _p(tets), _p(_d(dinv)), _p(_d(an)), _p(_d(vol)), _p(_d(mu)),
                        _p(_d(lam)), _p(f), _p(hd))
    return f, hd


def forces_fhats2_omp(x, tets, dinv, an, mu, lam, threads=0):
    """The reference's OpenMP force evaluation computeInnerForcesfromFhats2
    (IsotropicMaterial.cpp:411-453) in FP32 on `threads` threads (0 = all host
    cores): node forces (N, 3) float32, started from zero.  The locked
    scatter adds in thread-timing order, so the sums vary in the last bits."""
    if threads <= 0:
        threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    x, tets = f32(x).reshape(-1, 3), _i(tets).reshape(-1, 4)
    n, t = x.shape[0], tets.shape[0]
    out = np.zeros((n, 3), np.float32)
    mu = f32(np.broadcast_to(mu, (t,)))
    lam = f32(np.broadcast_to(lam, (t,)))
    lib().orc_forces_fhats2_omp(C.c_int(threads), C.c_int(n), _p(x), C.c_int(t), _p(tets),
                                _p(f32(dinv).reshape(-1)), _p(f32(an).reshape(-1)), _p(mu), _p(lam), _p(out))
    return out


def svd(F, prec=64):
    F = _d(F).reshape(-1, 3, 3)
    U, V, S = np.zeros_like(F), np.zeros_like(F), np.zeros((F.shape[0], 3))
    lib().orc_svd(C.c_int(prec), C.c_int(F.shape[0]), _p(F), _p(U), _p(S), _p(V))
    return U, S, V


class StepState:
    """x0, v, v_old and the persistent Chebyshev (rho, omega) of one instance."""

    def __init__(self, x0, v=None, v_old=None):
        self.x0 = _d(x0).reshape(-1, 3).copy()
        self.v = np.zeros_like(self.x0) if v is None else _d(v).reshape(-1, 3).copy()
        self.v_old = np.zeros_like(self.x0) if v_old is None else _d(v_old).reshape(-1, 3).copy()
        self.cheb = np.zeros(2)


def step(state: StepState, params: OrcParams, tets, r: Rest, mu, lam, pin_mask, ext=None, prec=64) -> OrcStats:
    tets = _i(tets).reshape(-1, 4)
    st = OrcStats()
    ext_a = _d(ext).reshape(-1, 3) if ext is not None else None
    lib().orc_step(C.c_int(prec), C.byref(params), C.c_int(state.x0.shape[0]), C.c_int(tets.shape[0]), _p(tets),
                   _p(_d(r.dinv)), _p(_d(r.an)), _p(_d(r.vol)), _p(_d(mu)), _p(_d(lam)), _p(_d(r.mass)),
                   _p(_d(r.grav_y)), _p(_i(pin_mask)), _p(state.x0), _p(state.v), _p(state.v_old), _p(ext_a),
                   _p(state.cheb), C.byref(st))
    return st


def incidence(tets, n_nodes):
    """Node -> (tet, corner) gather lists in canonical order (per node: ascending
    tet id, then corner), entry = 4*tet + corner.  Plain loops; small meshes."""
    lists = [[] for _ in range(n_nodes)]
    for t, q in enumerate(np.asarray(tets).reshape(-1, 4).tolist()):
        for c, node in enumerate(q):
            lists[node].append(4 * t + c)
    row = [0]
    ent = []
    for li in lists:
        ent.extend(li)
        row.append(len(ent))
    return np.array(row, np.int32), np.array(ent, np.int32)


def stiffness_pattern(tets, n_nodes):
    """IsotropicMaterial::allocateGlobalStiffnessMatrix (IsotropicMaterial.cpp:554-644)
    restated with Python sets: rows 3n+d, sorted unique columns, the CSR slot of
    each diagonal and the 48 slots per tet."""
    tets = np.asarray(tets).reshape(-1, 4).tolist()
    nb = [set() for _ in range(n_nodes)]
    for q in tets:
        for a in q:
            nb[a].update(q)
    row = [0]
    col = []
    for n in range(n_nodes):
        cols = [3 * m + e for m in sorted(nb[n]) for e in range(3)]
        for _ in range(3):
            col.extend(cols)
            row.append(len(col))
    row = np.array(row, np.int32)
    col = np.array(col, np.int32)

    def slot(r, c):
        lo, hi = row[r], row[r + 1]
        return lo + int(np.searchsorted(col[lo:hi], c))

    diag = np.array([slot(r, r) for r in range(3 * n_nodes)], np.int32)
    kid = np.zeros(48 * len(tets), np.int32)
    for t, q in enumerate(tets):
        for fi in range(4):
            for fj in range(3):
                for ni in range(4):
                    kid[48 * t + (fi * 3 + fj) * 4 + ni] = slot(3 * q[fi] + fj, 3 * q[ni])
    return row, col, diag, kid
