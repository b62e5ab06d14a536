"""ctypes binding of the reference's own CPU solver (oracle/_ref) -- test infrastructure.

Available only where ``oracle/_ref/libphybs_ref.so`` was built from the
reference tree.  Arrays cross in the reference's layouts: positions (N, 3)
float32 (= Eigen 3 x N column-major), per-tet 3x3 blocks column-major.
"""
from __future__ import annotations

import ctypes as C
import os
import tempfile

import numpy as np

from . import REF_SO, build

_lib = None


def available() -> bool:
    try:
        lib()
        return True
    except OSError:
        return False


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(REF_SO):
            build(reference=True)
        _lib = C.CDLL(REF_SO)
        _lib.ref_create.restype = C.c_void_p
        _lib.ref_create_faces.restype = C.c_void_p
        _lib.ref_total_energy.restype = C.c_float
        _lib.ref_ext_energy.restype = C.c_float
        _lib.ref_pd_create.restype = C.c_void_p
        _lib.ref_pd_create.argtypes = [C.c_void_p, C.c_float, C.c_int]
        _lib.ref_pd_destroy.argtypes = [C.c_void_p]
        _lib.ref_pd_step.argtypes = [C.c_void_p, C.c_void_p, C.c_float]
        _lib.ref_pbd_step.argtypes = [C.c_void_p, C.c_float]
        for name in ["ref_destroy", "ref_set_h", "ref_set_profile", "ref_set_lame", "ref_get_lame", "ref_get_rest",
                     "ref_get_nodes", "ref_set_nodes", "ref_get_vel", "ref_set_vel", "ref_get_vel_old",
                     "ref_set_vel_old", "ref_set_ext", "ref_get_mass", "ref_get_gravity", "ref_get_vol",
                     "ref_get_dminv", "ref_get_an", "ref_force_nh", "ref_force_stretch", "ref_elastic_energy",
                     "ref_hessian_diag", "ref_element_stiffness", "ref_total_energy", "ref_csr_sizes", "ref_csr",
                     "ref_step", "ref_get_scalars", "ref_face_ring_size", "ref_face_ring", "ref_pick_face",
                     "ref_drag_face_ring", "ref_get_ext", "ref_get_inv_mass", "ref_load_model"]:
            getattr(_lib, name).argtypes = None
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def load_model(stem: str):
    """TetMesh's own loader (TetMesh.cpp:14-151) on ``<stem>.node/.ele/.face``:
    (rest (N, 3) float32 after its x0.1 scaling, tets (T, 4) int32 in file
    order, pins selected by its hard-coded rule (TetMesh.cpp:38-39))."""
    for ext in (".node", ".ele", ".face"):
        if not os.path.exists(stem + ext):  # the loader would exit the process
            raise FileNotFoundError(stem + ext)
    L = lib()
    n, t, p = C.c_int(), C.c_int(), C.c_int()
    L.ref_load_model(stem.encode(), C.byref(n), C.byref(t), C.byref(p), None, None, None)
    rest = np.zeros((n.value, 3), np.float32)
    tets = np.zeros((t.value, 4), np.int32)
    pins = np.zeros(p.value, np.int32)
    L.ref_load_model(stem.encode(), C.byref(n), C.byref(t), C.byref(p), _p(rest), _p(tets), _p(pins))
    return rest, tets, pins


def _p(a):
    return C.c_void_p(a.ctypes.data)


class RefSim:
    """One reference TetMesh + IsotropicNeohookeanMaterial + DescentOptimize."""

    def __init__(self, rest, tets, pins, young, poisson, density=1000.0, faces=None):
        self._tmp = tempfile.TemporaryDirectory(prefix="phybs_ref_")
        rest = _f(rest).reshape(-1, 3)
        tets = np.ascontiguousarray(tets, np.int32).reshape(-1, 4)
        pins = np.ascontiguousarray(pins, np.int32)
        faces = np.zeros((0, 3), np.int32) if faces is None else np.ascontiguousarray(faces, np.int32).reshape(-1, 3)
        self.n, self.t, self.nf = rest.shape[0], tets.shape[0], faces.shape[0]
        h = lib().ref_create_faces(self._tmp.name.encode(), C.c_int(self.n), _p(rest), C.c_int(self.t), _p(tets),
                                   C.c_int(pins.size), _p(pins), C.c_float(young), C.c_float(poisson),
                                   C.c_float(density), C.c_int(self.nf), _p(faces))
        if not h:
            raise RuntimeError("reference harness rejected the mesh")
        self.h = C.c_void_p(h)

    def close(self):
        self._pd_close()
        if self.h:
            lib().ref_destroy(self.h)
            self.h = None
            self._tmp.cleanup()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- getters / setters ---------------------------------------------------
    def _get(self, fn, shape, dtype=np.float32):
        out = np.zeros(shape, dtype)
        getattr(lib(), fn)(self.h, _p(out))
        return out

    def rest(self):
        return self._get("ref_get_rest", (self.n, 3))

    def nodes(self):
        return self._get("ref_get_nodes", (self.n, 3))

    def set_nodes(self, x):
        lib().ref_set_nodes(self.h, _p(_f(x).reshape(-1, 3)))

    def vel(self):
        return self._get("ref_get_vel", (self.n, 3))

    def set_vel(self, v):
        lib().ref_set_vel(self.h, _p(_f(v).reshape(-1, 3)))

    def vel_old(self):
        return self._get("ref_get_vel_old", (self.n, 3))

    def set_ext(self, f):
        lib().ref_set_ext(self.h, _p(_f(f).reshape(-1, 3)))

    def mass(self):
        return self._get("ref_get_mass", (self.n,))

    def gravity(self):
        return self._get("ref_get_gravity", (self.n, 3))

    def vol(self):
        return self._get("ref_get_vol", (self.t,))

    def dminv(self):
        """(T, 3, 3) row-major view of the reference's column-major blocks."""
        return self._get("ref_get_dminv", (self.t, 3, 3)).transpose(0, 2, 1).copy()

    def an(self):
        return self._get("ref_get_an", (self.t, 3, 3)).transpose(0, 2, 1).copy()

    def lame(self):
        mu, lam = np.zeros(self.t, np.float32), np.zeros(self.t, np.float32)
        lib().ref_get_lame(self.h, _p(mu), _p(lam))
        return mu, lam

    def set_lame(self, mu, lam):
        lib().ref_set_lame(self.h, _p(_f(mu)), _p(_f(lam)))

    def set_h(self, h):
        lib().ref_set_h(self.h, C.c_float(h))

    def set_profile(self, profile):
        ks = np.array([k for k, _ in profile], np.int32)
        vs = np.array([v for _, v in profile], np.float32)
        lib().ref_set_profile(self.h, C.c_int(len(profile)), _p(ks), _p(vs))

    # -- evaluations -----------------------------------------------------------
    def force_nh(self, x):
        out = np.zeros((self.n, 3), np.float32)
        lib().ref_force_nh(self.h, _p(_f(x).reshape(-1, 3)), _p(out))
        return out

    def force_stretch(self, x, nthreads=0):
        out = np.zeros((self.n, 3), np.float32)
        lib().ref_force_stretch(self.h, _p(_f(x).reshape(-1, 3)), C.c_int(nthreads), _p(out))
        return out

    def elastic_energy(self, x):
        out = np.zeros(self.t, np.float32)
        lib().ref_elastic_energy(self.h, _p(_f(x).reshape(-1, 3)), _p(out))
        return out

    def hessian_diag(self, x):
        out = np.zeros((self.n, 3), np.float32)
        lib().ref_hessian_diag(self.h, _p(_f(x).reshape(-1, 3)), _p(out))
        return out

    def element_stiffness(self, tet, x):
        out = np.zeros((12, 12), np.float32)
        lib().ref_element_stiffness(self.h, C.c_int(tet), _p(_f(x).reshape(-1, 3)), _p(out))
        return out

    def total_energy(self, x, xtilde):
        return float(lib().ref_total_energy(self.h, _p(_f(x).reshape(-1, 3)), _p(_f(xtilde).reshape(-1, 3))))

    def csr(self):
        nnz, rows = C.c_int(), C.c_int()
        lib().ref_csr_sizes(self.h, C.byref(nnz), C.byref(rows))
        rowptr = np.zeros(rows.value + 1, np.int32)
        col = np.zeros(nnz.value, np.int32)
        diag = np.zeros(rows.value, np.int32)
        kid = np.zeros(48 * self.t, np.int32)
        lib().ref_csr(self.h, _p(rowptr), _p(col), _p(diag), _p(kid))
        return rowptr, col, diag, kid

    def step(self, iters):
        lib().ref_step(self.h, C.c_int(iters))

    # -- surface picking and drag (TetMesh.cpp:229-277, 378-418, 446-470, 595-614)
    def face_ring(self, face):
        out = np.zeros(lib().ref_face_ring_size(self.h, C.c_int(face)), np.int32)
        lib().ref_face_ring(self.h, C.c_int(face), _p(out))
        return out

    def pick_face(self, orig, direction):
        normals, centers = np.zeros((self.nf, 3), np.float32), np.zeros((self.nf, 3), np.float32)
        face = lib().ref_pick_face(self.h, _p(_f(orig)), _p(_f(direction)), _p(normals), _p(centers))
        return face, normals, centers

    def drag_face_ring(self, face, drag):
        lib().ref_drag_face_ring(self.h, C.c_int(face), _p(_f(drag)))

    def ext(self):
        return self._get("ref_get_ext", (self.n, 3))

    def ext_energy(self, x):
        return float(lib().ref_ext_energy(self.h, _p(_f(x).reshape(-1, 3))))

    def scalars(self):
        out = np.zeros(5, np.float32)
        lib().ref_get_scalars(self.h, _p(out))
        return dict(zip(["alpha", "energy", "energy_old", "rho", "omega"], out.tolist()))

    # -- position-based and projective dynamics (PosBaseDynamic.cpp, ProjDynamic.cpp)
    def inv_mass(self):
        return self._get("ref_get_inv_mass", (self.n,))

    def pbd_step(self, dt):
        """One doStepStrainConstraints step on the mesh's nodes and velocities."""
        lib().ref_pbd_step(self.h, dt)

    def pd_step(self, dt, dt_matrix=None, iterations=5):
        """One doProjDynamics step; the integrator (and its factorised solver
        matrix) is built on first use for (dt_matrix, iterations)."""
        key = (dt if dt_matrix is None else dt_matrix, iterations)
        if getattr(self, "_pd_key", None) != key:
            self._pd_close()
            self._pd = C.c_void_p(lib().ref_pd_create(self.h, key[0], key[1]))
            self._pd_key = key
        lib().ref_pd_step(self._pd, self.h, dt)

    def _pd_close(self):
        if getattr(self, "_pd", None):
            lib().ref_pd_destroy(self._pd)
            self._pd = None
            self._pd_key = None
