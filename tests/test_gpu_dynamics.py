"""GPU parity of strain-based PBD (pbs_pbd_step) and projective dynamics
(pbs_pd_step) through the C ABI.

PBD: bit for bit against the reference's own trajectories
(tests/golden/dynamics_*.npz, PosBaseDynamic built headless): the step forms
its rest data as TetMesh does in FP32 and sweeps in the serial order with the
same FP32 operations; and bit for bit against the serial restatement
(orc_pbd_step on orc_rest_eigen32's rest data) on a 64,000-tet box (910
dependency levels, several CTAs a level), with other stiffnesses, and on a
packed batch.

Projective dynamics: within 5e-6 of the bounding-box diagonal of the FP64
restatement (exact solves) given the device's rest data, including a state
with inverted tets and each instance of a packed batch away from the origin,
and within 1e-4 of the reference's trajectory (FP32 LDL^T)."""
import numpy as np
import pytest

from oracle import projective as P
from phybs_gb300 import _lib as L
from phybs_gb300 import meshes as M
from phybs_gb300.solver import DescentSolver
from tests._util import bbox_diag, golden_names, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


@pytest.fixture(scope="module", params=golden_names("dynamics_"))
def g(request):
    return load_golden(request.param)


def device_rest(s, mesh):
    """(Dm^-1 row-major (T, 9), inverse masses, body forces) as the device has them."""
    dinv, _, mass, gy = s.rest_data()
    pm = mesh.pin_mask() > 0
    w = np.where(pm, 0.0, 1.0 / mass.astype(np.float64)).astype(np.float32)
    grav = np.zeros((mesh.n_nodes, 3), np.float32)
    grav[:, 1] = gy
    return dinv.reshape(-1, 9), w, grav


def solver_of(g):
    m = M.TetMeshData(g["rest"], g["tets"], g["pins"], 5e5, 0.45)
    s = DescentSolver(m)
    return m, s


def pbd_rest(mesh):
    """The PBD step's rest data (Dm^-1 row-major, inverse masses, gravity)."""
    return P.rest_eigen32(mesh.rest, mesh.tets, mesh.pin_mask(), density=float(mesh.density), gravity=9.8)


def test_pbd_matches_reference_bitwise(g):
    m, s = solver_of(g)
    s.update_positions(g["x0"])
    s.write_velocities(np.zeros_like(g["x0"]), np.zeros_like(g["x0"]))
    assert np.array_equal(s.positions(), g["x0"])  # the exact position read-back
    for k in range(3):
        s.pbd_step(float(g["dt"]), ext=g["ext"] if k == 0 else None)
        assert np.array_equal(s.positions(), g[f"x_pbd{k}"]), k
        assert np.array_equal(s.velocities()[0], g[f"v_pbd{k}"]), k
    s.close()


@pytest.mark.parametrize("iterations,stretch,shear", [(5, None, None), (2, (0.5, 0.9, 1.0), (0.3, 0.6, 0.9)),
                                                      (0, None, None)])
def test_pbd_box_and_options_bitwise(iterations, stretch, shear):
    """A 20 x 20 x 32-cube box (64,000 tets, 910 levels), twisted, pulled by
    gravity, against the restatement; also other stiffnesses and zero sweeps
    (inertia only)."""
    m = M.box_mesh(20, 20, 32, edge=0.005, seed=4)
    x = M.twist_positions(m.rest, 0.3, axis=2).astype(np.float32)
    x[m.pins] = m.rest[m.pins]
    s = DescentSolver(m, positions=x)
    dinv, w, grav = pbd_rest(m)
    v = np.zeros_like(x)
    st = (1.0, 1.0, 1.0) if stretch is None else stretch
    sh = (0.8, 0.8, 0.8) if shear is None else shear
    for k in range(2):
        x, v = P.pbd_step(x, v, w, m.tets, dinv, grav, 1 / 60, iterations=iterations, stretch=st, shear=sh)
        s.pbd_step(1 / 60, iterations=iterations, stretch=stretch, shear=shear)
    assert np.array_equal(s.positions(), x)
    assert np.array_equal(s.velocities()[0], v)
    s.close()


@pytest.mark.parametrize("n_inst", [3, 6])
def test_pbd_packed_batch_bitwise(n_inst):
    """Uneven boxes packed in one handle: each instance's sweep (one cluster
    each: 16 CTAs for up to four instances, 8 beyond) equals the restatement
    of that instance alone."""
    m = M.batch_of_boxes(n_inst, seed=7, nxy=(3, 6), nz=(5, 12))
    x = M.twist_positions(m.rest, 0.05, axis=2).astype(np.float32)
    x[m.pins] = m.rest[m.pins]
    s = DescentSolver(m, positions=x)
    dinv, w, grav = pbd_rest(m)
    s.pbd_step(1 / 30)
    got = s.positions()
    for b in range(m.n_instances):
        n0, n1 = m.instance_node_ptr[b], m.instance_node_ptr[b + 1]
        t0, t1 = m.instance_tet_ptr[b], m.instance_tet_ptr[b + 1]
        xb, _ = P.pbd_step(x[n0:n1], np.zeros((n1 - n0, 3), np.float32), w[n0:n1], m.tets[t0:t1] - n0,
                           dinv[t0:t1], grav[n0:n1], 1 / 30)
        assert np.array_equal(got[n0:n1], xb), b
    s.close()


def test_pd_matches_restatement(g):
    m, s = solver_of(g)
    dinv, w, grav = device_rest(s, m)
    _, svol, mass, _ = s.rest_data()
    diag = bbox_diag(g["rest"])
    dt = float(g["dt"])
    for start in ("x0", "x_inv"):
        x0 = g[start]
        s.update_positions(x0)
        s.write_velocities(np.zeros_like(x0), np.zeros_like(x0))
        ext = g["ext"] if start == "x0" else None
        f = grav + (ext if ext is not None else 0.0)
        xo, vo = P.pd_step(x0, np.zeros_like(x0), mass, w, g["tets"], dinv.reshape(-1, 3, 3), np.abs(svol), f, dt=dt)
        it = s.pd_step(dt, ext=ext, tol=1e-7)
        assert it > 0
        err = np.abs(s.positions() - xo).max() / diag
        assert err < 5e-6, (start, err, it)
        assert np.abs(s.velocities()[0] - vo).max() <= 5e-6 * diag / dt
    s.close()


def test_pd_split_time_step():
    """A matrix formed with another time step than the step's (the
    reference's integrator step for A, 0.03 for the right-hand side): the
    residual's extra inertial term, against the restatement.  With the two
    steps different the system is no longer translation-invariant, and that
    term, (m / dt^2 - m / dt_m^2) x, carries the FP32 rounding of an absolute
    position: within 5e-5 of the diagonal (1.5e-5 measured), against 5e-6
    with one step."""
    g = load_golden("dynamics_bar_small")
    m, s = solver_of(g)
    dinv, w, grav = device_rest(s, m)
    _, svol, mass, _ = s.rest_data()
    s.update_positions(g["x0"])
    s.pd_step(0.03, dt_matrix=0.02, tol=1e-7)
    xo, _ = P.pd_step(g["x0"], np.zeros_like(g["x0"]), mass, w, g["tets"], dinv.reshape(-1, 3, 3), np.abs(svol),
                      grav, dt=0.03, dt_matrix=0.02)
    assert np.abs(s.positions() - xo).max() / bbox_diag(g["rest"]) < 5e-5
    s.close()


def test_pd_close_to_reference(g):
    m, s = solver_of(g)
    s.update_positions(g["x0"])
    diag = bbox_diag(g["rest"])
    for k in range(2):
        s.pd_step(float(g["dt"]), ext=g["ext"] if k == 0 else None, tol=1e-7)
        err = np.abs(s.positions() - g[f"x_pd{k}"]).max() / diag
        assert err < 1e-4, (k, err)
    s.close()


def test_pd_packed_batch():
    """Three uneven boxes in one handle (one block-diagonal system, one CG):
    each instance (0.5 and 1 m from the origin for the second and third)
    within 5e-6 of its bounding-box diagonal of the FP64 restatement of that
    instance alone."""
    m = M.batch_of_boxes(3, seed=9, nxy=(3, 6), nz=(5, 12))
    x = M.twist_positions(m.rest, 0.05, axis=2).astype(np.float32)
    x[m.pins] = m.rest[m.pins]
    s = DescentSolver(m, positions=x)
    dinv, w, grav = device_rest(s, m)
    _, svol, mass, _ = s.rest_data()
    s.pd_step(0.03, tol=1e-7)
    got = s.positions()
    for b in range(m.n_instances):
        n0, n1 = m.instance_node_ptr[b], m.instance_node_ptr[b + 1]
        t0, t1 = m.instance_tet_ptr[b], m.instance_tet_ptr[b + 1]
        xo, _ = P.pd_step(x[n0:n1], np.zeros((n1 - n0, 3)), mass[n0:n1], w[n0:n1], m.tets[t0:t1] - n0,
                          dinv[t0:t1].reshape(-1, 3, 3), np.abs(svol[t0:t1]), grav[n0:n1], dt=0.03)
        err = np.abs(got[n0:n1] - xo).max() / bbox_diag(m.rest[n0:n1])
        assert err < 5e-6, (b, err)
    s.close()


def test_pd_cap_and_arguments():
    m = M.bar_mesh(8, 3, 3, edge=0.025)
    s = DescentSolver(m)
    x0 = s.positions()
    it = s.pd_step(max_cg=2, raise_on_cap=False, iterations=1)
    assert s.last_status == L.PBS_E_ITER_CAP and it == 2
    assert not np.array_equal(s.positions(), x0)
    for kw in (dict(dt=-1.0), dict(stiffness=0.0), dict(tol=0.0), dict(max_cg=0), dict(iterations=-1)):
        with pytest.raises(L.PhybsError):
            s.pd_step(**kw)
    with pytest.raises(L.PhybsError):
        s.pbd_step(dt=0.0)
    with pytest.raises(L.PhybsError):
        s.pbd_step(stretch=(1.0, np.nan, 1.0))
    # the descent step still runs from the state the other integrators left
    s.pbd_step()
    s.step()
    assert s.stats()["status"] == L.PBS_OK
    s.close()


def test_cpp_wrapper_integrators(tmp_path):
    """The header-only CUDAInterface wrapper's doBackEuler, pbdStep and
    projectiveDynamicsStep run on the device and move the bar under gravity."""
    import subprocess

    from tests.test_host import build_cpp_demo
    exe = build_cpp_demo(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    vals = dict(zip(out[0::2], out[1::2]))
    for key in ("step", "backeuler", "pbd", "pd"):
        assert key in vals, out
        v = float(vals[key])
        assert np.isfinite(v) and 0.0 < v < 0.1, (key, v)


def test_pbd_handles_of_different_sizes_interleave():
    """Two live handles whose sweeps keep their positions in shared memory
    of different sizes: stepping the larger after the smaller was set up
    still runs and stays bit-identical to the restatement."""
    big = M.box_mesh(20, 20, 32, edge=0.005, seed=4)
    small = M.bar_mesh(6, 3, 3, edge=0.025)
    xb = M.twist_positions(big.rest, 0.2, axis=2).astype(np.float32)
    xb[big.pins] = big.rest[big.pins]
    a = DescentSolver(big, positions=xb)
    a.pbd_step(1 / 60)
    b = DescentSolver(small)
    b.pbd_step(1 / 60)
    a.pbd_step(1 / 60)
    dinv, w, grav = pbd_rest(big)
    x, v = xb, np.zeros_like(xb)
    for _ in range(2):
        x, v = P.pbd_step(x, v, w, big.tets, dinv, grav, 1 / 60)
    assert np.array_equal(a.positions(), x)
    a.close()
    b.close()
