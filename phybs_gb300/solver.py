"""Host-side mirror of PhyBS's descent-step classes over the C ABI.

* :class:`DescentSolver` - the general handle: one or many packed meshes,
  material, step parameters, step / read / update / reset, parity probes.
* :class:`CUDAInterface` - the constructor and ``doDescentOpt`` /
  ``updateNodePositions`` / ``reset`` of ``FVM/CUDAInterface.h:20-35`` with the
  GPU reference's semantics (gravity once in the gradient,
  ``CUDAInterface.cu:600-602``; ``max(e, 0)`` energy clamp, ``:549``).
* :class:`DescentOptimize` - ``FVM/DescentOptimize.h:11-18`` semantics
  (gravity and external forces twice in the gradient, ``e > 1e-6`` clamp),
  driving a mesh's node and velocity arrays in place as the CPU class does.

All compute runs in libphybs_gb300.so on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .meshes import TetMeshData

PRESETS = {
    # DescentOptimize (CPU) reference semantics: DescentOptimize.cpp:4-22,91-188
    "cpu_reference": dict(body_force_scale=2.0, energy_clamp=L.PBS_CLAMP_CPU),
    # CUDAInterface (GPU) reference semantics: CUDAInterface.cu:572-609, 911-1007
    "gpu_reference": dict(body_force_scale=1.0, energy_clamp=L.PBS_CLAMP_GPU),
}


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(shape) if shape is not None else a


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def make_params(preset: str = "cpu_reference", **kw) -> L.StepParams:
    """Reference preset (pbs_default_params) with overrides.  ``profile`` may be
    given as a sequence of (k, rho) pairs."""
    p = L.default_params()
    for k, v in PRESETS[preset].items():
        setattr(p, k, v)
    prof = kw.pop("profile", None)
    if prof is not None:
        p.n_profile = len(prof)
        for i, (k, r) in enumerate(prof):
            p.profile_k[i] = int(k)
            p.profile_rho[i] = float(r)
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


class DescentSolver:
    """One device-resident set of packed tet meshes advanced by descent steps."""

    def __init__(self, mesh: TetMeshData, positions=None, material: int = L.PBS_MATERIAL_NEOHOOKEAN, mu=None,
                 lam=None, reference_lambda: bool = True, params: L.StepParams | None = None, gravity: float = 9.8):
        self.mesh = mesh
        self._h = C.c_void_p()
        rest = _f32(mesh.rest, (-1, 3))
        pos = _f32(positions, (-1, 3)) if positions is not None else None
        tets = np.ascontiguousarray(mesh.tets, np.int32)
        pm = mesh.pin_mask()
        nptr = np.ascontiguousarray(mesh.instance_node_ptr, np.int32)
        tptr = np.ascontiguousarray(mesh.instance_tet_ptr, np.int32)
        d = L.MeshDesc(mesh.n_nodes, _ptr(rest).value, _ptr(pos).value if pos is not None else None, mesh.n_tets,
                       _ptr(tets).value, _ptr(pm).value, mesh.n_instances, _ptr(nptr).value, _ptr(tptr).value,
                       float(mesh.density), float(gravity))
        L.check(L.lib().pbs_create(C.byref(d), C.byref(self._h)), "pbs_create")
        self.n = mesh.n_nodes
        self.t = mesh.n_tets
        if mu is None:
            mu, lam = lame_arrays(mesh.young, mesh.poisson, reference_lambda)
        self.set_material(material, mu, lam)
        self.set_params(params if params is not None else make_params())

    # -- lifecycle -------------------------------------------------------------
    def close(self):
        if self._h:
            L.lib().pbs_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- configuration -----------------------------------------------------------
    def set_material(self, model: int, mu, lam):
        mu = np.atleast_1d(_f32(mu))
        lam = np.atleast_1d(_f32(lam))
        self.material = model
        L.check(L.lib().pbs_set_material(self._h, C.c_int(model), _ptr(mu), _ptr(lam), C.c_int(mu.size)),
                "pbs_set_material")

    def set_params(self, p: L.StepParams):
        self.params = p
        L.check(L.lib().pbs_set_params(self._h, C.byref(p)), "pbs_set_params")

    # -- stepping ---------------------------------------------------------------
    def step(self, ext=None, raise_on_error: bool = True) -> int:
        it = C.c_int()
        e = _f32(ext, (-1, 3)) if ext is not None else None
        rc = L.lib().pbs_step(self._h, _ptr(e), C.byref(it))
        if raise_on_error and rc not in (L.PBS_OK,):
            L.check(rc, "pbs_step")
        self.last_status = rc
        return it.value

    def positions(self, out=None) -> np.ndarray:
        out = np.empty((self.n, 3), np.float32) if out is None else out
        L.check(L.lib().pbs_read_positions(self._h, _ptr(out)), "pbs_read_positions")
        return out

    def update_positions(self, x):
        L.check(L.lib().pbs_update_positions(self._h, _ptr(_f32(x, (-1, 3)))), "pbs_update_positions")

    def set_guess(self, x):
        """Initial guess for the next step (kept only if its energy is lower)."""
        L.check(L.lib().pbs_set_guess(self._h, _ptr(_f32(x, (-1, 3)))), "pbs_set_guess")

    def set_node_positions(self, ids, xyz):
        ids = np.ascontiguousarray(ids, np.int32)
        xyz = _f32(xyz, (-1, 3))
        L.check(L.lib().pbs_set_node_positions(self._h, C.c_int(ids.size), _ptr(ids), _ptr(xyz)),
                "pbs_set_node_positions")

    def stream(self) -> int:
        s = C.c_void_p()
        L.check(L.lib().pbs_get_stream(self._h, C.byref(s)), "pbs_get_stream")
        return s.value or 0

    def profile_kernels(self, passes: int = 20):
        a, b = C.c_double(), C.c_double()
        L.check(L.lib().pbs_profile_kernels(self._h, C.c_int(passes), C.byref(a), C.byref(b)), "pbs_profile_kernels")
        return a.value, b.value

    def profile_frame(self, passes: int = 20) -> float:
        """Mean milliseconds per pass of one frame-engine launch of `passes` passes."""
        a = C.c_double()
        L.check(L.lib().pbs_profile_frame(self._h, C.c_int(passes), C.byref(a)), "pbs_profile_frame")
        return a.value

    def set_pass_engine(self, engine: str):
        """'graph' (per-pass kernels in captured graphs) or 'frame' (one
        persistent cooperative launch a step; one instance, unstaged shape)."""
        code = {"graph": L.PBS_ENGINE_GRAPH, "frame": L.PBS_ENGINE_FRAME}[engine]
        L.check(L.lib().pbs_set_pass_engine(self._h, C.c_int(code)), "pbs_set_pass_engine")

    def set_l2_residency(self, enable: bool):
        """Launch the per-tet kernels with (True, the default) or without an L2
        access-policy window that keeps the pass rows resident."""
        L.check(L.lib().pbs_set_l2_residency(self._h, C.c_int(1 if enable else 0)), "pbs_set_l2_residency")

    def pass_engine(self) -> str:
        e = C.c_int()
        L.check(L.lib().pbs_get_pass_engine(self._h, C.byref(e)), "pbs_get_pass_engine")
        return "frame" if e.value == L.PBS_ENGINE_FRAME else "graph"

    def autotune(self, passes: int = 32) -> dict:
        """Pick the pass kernels' chunk shape by timing candidates on this mesh."""
        r = L.TuneResult()
        L.check(L.lib().pbs_autotune(self._h, C.c_int(passes), C.byref(r)), "pbs_autotune")
        return {k: getattr(r, k) for k, _ in r._fields_}

    def set_chunk_shape(self, threads: int, chunk_tets: int, chunk_nodes: int, staged: int = 0, node_npt: int = 1):
        """Use launch shapes picked elsewhere (e.g. by autotune on another handle).
        staged: 0 = rows read in the tet loop, 1 = rows staged in shared memory,
        2 = the persistent double-buffered kernel (neo-Hookean, 128 or 256
        threads)."""
        L.check(L.lib().pbs_set_chunk_shape(self._h, C.c_int(threads), C.c_int(chunk_tets), C.c_int(chunk_nodes),
                                            C.c_int(staged), C.c_int(node_npt)), "pbs_set_chunk_shape")

    def warm_start_features(self, ext=None):
        """Raw 24 features per node for the next step, the plain initial
        guess, and each node's motion scale (features, x_init, scale)."""
        feats = np.empty((self.n, 24), np.float32)
        xin = np.empty((self.n, 3), np.float32)
        scale = np.empty(self.n, np.float32)
        e = _f32(ext, (-1, 3)) if ext is not None else None
        L.check(L.lib().pbs_warm_start_features(self._h, _ptr(e), _ptr(feats), _ptr(xin), _ptr(scale)),
                "pbs_warm_start_features")
        return feats, xin, scale

    def set_warm_start(self, model=None):
        """Install a WarmStartModel (or switch the warm start off with None)."""
        if model is None:
            L.check(L.lib().pbs_set_warm_start(self._h, None, None, None, None, C.c_int(0)), "pbs_set_warm_start")
            return
        th, fm, fs, os_ = (_f32(model.theta), _f32(model.feat_mean), _f32(model.feat_std), _f32(model.out_std))
        mode = 2 if getattr(model, "base", "inertial") == "extrapolation" else 1
        L.check(L.lib().pbs_set_warm_start(self._h, _ptr(th), _ptr(fm), _ptr(fs), _ptr(os_), C.c_int(mode)),
                "pbs_set_warm_start")

    def velocities(self):
        v = np.empty((self.n, 3), np.float32)
        vo = np.empty((self.n, 3), np.float32)
        L.check(L.lib().pbs_read_velocities(self._h, _ptr(v), _ptr(vo)), "pbs_read_velocities")
        return v, vo

    def write_velocities(self, v=None, v_old=None):
        L.check(L.lib().pbs_write_velocities(self._h, _ptr(_f32(v, (-1, 3)) if v is not None else None),
                                             _ptr(_f32(v_old, (-1, 3)) if v_old is not None else None)),
                "pbs_write_velocities")

    def reset(self):
        L.check(L.lib().pbs_reset(self._h), "pbs_reset")

    def backward_euler_step(self, dt: float = 0.03, alpha: float = 0.02, beta: float = 0.02, ext=None,
                            tol: float = 1e-6, max_iters: int = 4000, raise_on_cap: bool = True):
        """One linearly implicit Euler step (CUDAInterface::doBackEuler); returns
        (CG iterations, |r| / |b|)."""
        it, res = C.c_int(), C.c_double()
        e = _f32(ext, (-1, 3)) if ext is not None else None
        rc = L.lib().pbs_backward_euler_step(self._h, C.c_float(dt), C.c_float(alpha), C.c_float(beta), _ptr(e),
                                             C.c_float(tol), C.c_int(max_iters), C.byref(it), C.byref(res))
        if rc != L.PBS_OK and (raise_on_cap or rc != L.PBS_E_ITER_CAP):
            L.check(rc, "pbs_backward_euler_step")
        self.last_status = rc
        return it.value, res.value

    # -- strain-based PBD and projective dynamics (PosBaseDynamic.cpp, ProjDynamic.cpp) --
    def pbd_step(self, dt: float = 0.03, iterations: int = 5, stretch=None, shear=None, ext=None):
        """One PosBaseDynamic::doStepStrainConstraints step (defaults: the
        reference's 5 sweeps, stretch 1, shear 0.8), bit-identical to the
        serial CPU sweep on the same rest data."""
        st = _f32(stretch, (3,)) if stretch is not None else None
        sh = _f32(shear, (3,)) if shear is not None else None
        e = _f32(ext, (-1, 3)) if ext is not None else None
        L.check(L.lib().pbs_pbd_step(self._h, C.c_float(dt), C.c_int(iterations), _ptr(st), _ptr(sh), _ptr(e)),
                "pbs_pbd_step")

    def pd_step(self, dt: float = 0.03, dt_matrix: float = 0.0, stiffness: float = 1e6, iterations: int = 5,
                ext=None, tol: float = 1e-6, max_cg: int = 20000, raise_on_cap: bool = True) -> int:
        """One ProjDynamic::doProjDynamics step (defaults: the reference's
        stiffness 1e6, 5 local/global iterations, A formed with dt); returns
        the step's total CG iterations."""
        it = C.c_int()
        e = _f32(ext, (-1, 3)) if ext is not None else None
        rc = L.lib().pbs_pd_step(self._h, C.c_float(dt), C.c_float(dt_matrix), C.c_float(stiffness),
                                 C.c_int(iterations), _ptr(e), C.c_float(tol), C.c_int(max_cg), C.byref(it))
        if rc != L.PBS_OK and (raise_on_cap or rc != L.PBS_E_ITER_CAP):
            L.check(rc, "pbs_pd_step")
        self.last_status = rc
        return it.value

    # -- surface picking and drag forces (TetMesh.cpp:229-277, 378-418, 446-470) --
    def set_surface(self, faces):
        """Boundary triangles (F, 3) in caller node ids, e.g. load_tetgen_faces()."""
        f = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
        L.check(L.lib().pbs_set_surface(self._h, _ptr(f), C.c_int(f.shape[0])), "pbs_set_surface")

    def face_ring(self, face: int) -> np.ndarray:
        n = C.c_int()
        L.check(L.lib().pbs_get_face_ring(self._h, C.c_int(face), None, C.c_int(0), C.byref(n)), "pbs_get_face_ring")
        out = np.empty(n.value, np.int32)
        L.check(L.lib().pbs_get_face_ring(self._h, C.c_int(face), _ptr(out), C.c_int(n.value), C.byref(n)),
                "pbs_get_face_ring")
        return out

    def pick_face(self, orig, direction) -> int:
        """The face a ray picks at the current positions (-1: none)."""
        o, d = _f32(orig, (3,)), _f32(direction, (3,))
        face = C.c_int()
        L.check(L.lib().pbs_pick_face(self._h, _ptr(o), _ptr(d), C.byref(face)), "pbs_pick_face")
        return face.value

    def drag_face_ring(self, face: int, drag) -> np.ndarray:
        """External forces (N, 3) of dragging `face` along `drag`, for step(ext=...)."""
        d = _f32(drag, (3,))
        ext = np.empty((self.n, 3), np.float32)
        L.check(L.lib().pbs_drag_face_ring(self._h, C.c_int(face), _ptr(d), _ptr(ext)), "pbs_drag_face_ring")
        return ext

    def instance_stats(self, instance: int) -> dict:
        """The last step's figures of one packed instance."""
        s = L.Stats()
        L.check(L.lib().pbs_get_instance_stats(self._h, C.c_int(instance), C.byref(s)), "pbs_get_instance_stats")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def stats(self) -> dict:
        s = L.Stats()
        L.check(L.lib().pbs_get_stats(self._h, C.byref(s)), "pbs_get_stats")
        return {k: getattr(s, k) for k, _ in L.Stats._fields_}

    # -- parity probes ------------------------------------------------------------
    def eval_tets(self, x=None):
        cf = np.empty((self.t, 4, 3), np.float32)
        en = np.empty(self.t, np.float32)
        hd = np.empty((self.t, 4, 3), np.float32)
        xx = _f32(x, (-1, 3)) if x is not None else None
        L.check(L.lib().pbs_eval_tets(self._h, _ptr(xx), _ptr(cf), _ptr(en), _ptr(hd)), "pbs_eval_tets")
        return cf, en, hd

    def eval_fp64_svd_count(self) -> int:
        """Tets of the last eval_tets call whose stretch-based stress took the
        FP64 SVD (det F < 1e-3)."""
        n = C.c_int()
        L.check(L.lib().pbs_eval_fp64_svd_count(self._h, C.byref(n)), "pbs_eval_fp64_svd_count")
        return int(n.value)

    def eval_nodes(self, x=None):
        f = np.empty((self.n, 3), np.float32)
        hd = np.empty((self.n, 3), np.float32)
        xx = _f32(x, (-1, 3)) if x is not None else None
        L.check(L.lib().pbs_eval_nodes(self._h, _ptr(xx), _ptr(f), _ptr(hd)), "pbs_eval_nodes")
        return f, hd

    def eval_base_force(self, x) -> np.ndarray:
        """Elastic node forces (FP64 values, pins 0) at x from the incremental
        stress's per-step base-force kernels (double-float, neo-Hookean)."""
        f = np.empty((self.n, 3), np.float64)
        xx = _f32(x, (-1, 3))
        L.check(L.lib().pbs_eval_base_force(self._h, _ptr(xx), _ptr(f)), "pbs_eval_base_force")
        return f

    def incidence(self):
        row = np.empty(self.n + 1, np.int32)
        ent = np.empty(4 * self.t, np.int32)
        L.check(L.lib().pbs_get_incidence(self._h, _ptr(row), _ptr(ent)), "pbs_get_incidence")
        return row, ent

    def rest_data(self):
        dinv = np.empty((self.t, 3, 3), np.float32)
        svol = np.empty(self.t, np.float32)
        mass = np.empty(self.n, np.float32)
        gy = np.empty(self.n, np.float32)
        L.check(L.lib().pbs_get_rest_data(self._h, _ptr(dinv), _ptr(svol), _ptr(mass), _ptr(gy)),
                "pbs_get_rest_data")
        return dinv, svol, mass, gy


def lame_arrays(young, poisson, reference_lambda=True):
    """Per-tet Lame parameters, computed exactly as pbs_lame does."""
    e = np.asarray(young, np.float32)
    nu = np.asarray(poisson, np.float32)
    mu = (np.float32(0.5) * e / (np.float32(1.0) + nu)).astype(np.float32)
    lam = (mu * np.float32(2.0) / (np.float32(1.0) - np.float32(2.0) * nu)).astype(np.float32)
    if not reference_lambda:
        lam = (lam * nu).astype(np.float32)
    return mu, lam


def stiffness_pattern(n_nodes: int, tets):
    """IsotropicMaterial::allocateGlobalStiffnessMatrix's CSR pattern (host side)."""
    tets = np.ascontiguousarray(tets, np.int32).reshape(-1, 4)
    nnz = C.c_int()
    L.check(L.lib().pbs_stiffness_pattern(C.c_int(n_nodes), C.c_int(tets.shape[0]), _ptr(tets), C.byref(nnz),
                                          None, None, None, None), "pbs_stiffness_pattern")
    row = np.empty(3 * n_nodes + 1, np.int32)
    col = np.empty(nnz.value, np.int32)
    diag = np.empty(3 * n_nodes, np.int32)
    kid = np.empty(48 * tets.shape[0], np.int32)
    L.check(L.lib().pbs_stiffness_pattern(C.c_int(n_nodes), C.c_int(tets.shape[0]), _ptr(tets), C.byref(nnz),
                                          _ptr(row), _ptr(col), _ptr(diag), _ptr(kid)), "pbs_stiffness_pattern")
    return row, col, diag, kid


class CUDAInterface:
    """Drop-in for ``CUDAInterface`` (FVM/CUDAInterface.h:20-35).

    The CSR arguments of the reference constructor are accepted and ignored:
    the descent step needs no global matrix.  Unlike the reference, whose
    kernels always use h = 0.03 (CUDAInterface.cu:644), ``doDescentOpt``
    honours its ``h`` argument.
    """

    def __init__(self, num_nodes, nodes, restPoses, constraintsMask, num_tets, tets, youngs, nu, density,
                 csr_nnz=0, csr_m=0, csr_val=None, csr_row=None, csr_col=None, csr_diagonalIdx=None,
                 csr_kIDinCSRval=None):
        rest = _f32(restPoses, (-1, 3))[:num_nodes]
        mask = np.asarray(constraintsMask, np.int32)[:num_nodes]
        mesh = TetMeshData(rest, np.asarray(tets, np.int32).reshape(-1, 4)[:num_tets], np.nonzero(mask > 0)[0],
                           youngs, nu, density=density)
        self._solver = DescentSolver(mesh, positions=_f32(nodes, (-1, 3))[:num_nodes],
                                     params=make_params("gpu_reference"))
        self._h = None

    def doDescentOpt(self, h, iterations, hostExternForces, hostNode):
        if self._h != (h, iterations):
            self._solver.set_params(make_params("gpu_reference", h=float(h), max_iters=int(iterations)))
            self._h = (h, iterations)
        self._solver.step(hostExternForces)
        out = np.asarray(hostNode)
        res = self._solver.positions()
        out.reshape(-1)[:res.size] = res.reshape(-1)
        return out

    def updateNodePositions(self, hostNode):
        self._solver.update_positions(hostNode)

    def reset(self):
        self._solver.reset()


class DescentOptimize:
    """``DescentOptimize`` semantics on the GPU, advancing ``mesh_nodes`` /
    ``mesh_velocities`` (N x 3 float32 arrays) in place after each step."""

    def __init__(self, mesh: TetMeshData, h: float = 0.03, mu=None, lam=None):
        self._h = h
        self.nodes = np.array(mesh.rest, np.float32, copy=True)
        self.velocities = np.zeros_like(self.nodes)
        self._solver = DescentSolver(mesh, mu=mu, lam=lam, params=make_params("cpu_reference", h=h))

    def reset(self):
        self._solver.reset()
        self.nodes[:] = self._solver.mesh.rest
        self.velocities[:] = 0

    def doDescentOpt(self, iterations: int):
        p = self._solver.params
        if p.max_iters != iterations:
            p.max_iters = int(iterations)
            self._solver.set_params(p)
        self._solver.step(None)
        self.nodes[:] = self._solver.positions()
        self.velocities[:] = self._solver.velocities()[0]
