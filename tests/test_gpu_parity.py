"""GPU parity: the sm_103a path through the C ABI against the restated oracle
and the reference's own outputs (tests/golden).

Bars (BASELINE the benchmark spec): per-tet forces within 1e-5 (max-norm relative),
positions after a step at a fixed iteration count within 1e-4 of the
bounding-box diagonal, the gather CSR and its order bit-exact.  Each test also
states the error against the all-FP64 oracle where it applies.
"""
import numpy as np
import pytest

from oracle import restated as O
from phybs_gb300 import _lib as L
from phybs_gb300 import meshes as M
from phybs_gb300.solver import CUDAInterface, DescentSolver, make_params
from tests._util import bbox_diag, elastic_from_ref, golden_names, load_golden, rel_max

pytestmark = pytest.mark.gpu

NAMES = golden_names()
FORCE_TOL = 1e-5       # per-tet corner forces, max-norm relative
POS_TOL = 1e-4         # positions / bounding-box diagonal


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


@pytest.fixture(scope="module", params=NAMES)
def g(request):
    d = load_golden(request.param)
    d["name"] = request.param
    return d


def mesh_of(g):
    return M.TetMeshData(g["rest"], g["tets"], g["pins"], g["young"], g["poisson"], name=g.get("name", "mesh"))


def solver_of(g, material=L.PBS_MATERIAL_NEOHOOKEAN, preset="cpu_reference", **kw):
    kw.setdefault("max_iters", int(g["iters"]))
    p = make_params(preset, h=float(g["h"]), **kw)
    return DescentSolver(mesh_of(g), positions=g["traj_x0"], material=material, mu=g["mu"], lam=g["lam"], params=p)


def pin_mask(g):
    m = np.zeros(g["rest"].shape[0], np.int32)
    m[g["pins"]] = 1
    return m


def test_rest_data(g):
    s = solver_of(g)
    dinv, svol, mass, gy = s.rest_data()
    assert rel_max(dinv, g["dminv"]) < 5e-6
    assert rel_max(np.abs(svol), g["vol"]) < 2e-6
    assert rel_max(mass, g["mass"]) < 2e-6
    assert rel_max(gy, g["gravity"][:, 1]) < 2e-6
    s.close()


def test_incidence_bit_exact(g):
    s = solver_of(g)
    row, ent = s.incidence()
    row_o, ent_o = O.incidence(g["tets"], g["rest"].shape[0])
    assert np.array_equal(row, row_o) and np.array_equal(ent, ent_o)
    s.close()


@pytest.mark.parametrize("material", [L.PBS_MATERIAL_NEOHOOKEAN, L.PBS_MATERIAL_STRETCH])
def test_per_tet_corner_forces(g, material):
    s = solver_of(g, material=material)
    cf, en, hd = s.eval_tets(g["probe_x"])
    ref = {}
    for prec in (32, 64):
        ref[prec], _, _ = O.tet_eval(g["probe_x"], g["tets"], g["dminv"], g["an"], g["vol"], g["mu"], g["lam"],
                                     material=material, prec=prec, energy=False, hdiag=False)
    err64 = rel_max(cf, ref[64])
    assert err64 < FORCE_TOL, err64
    # the oracle's own FP32 run sits at the same distance from FP64
    assert rel_max(ref[32], ref[64]) < FORCE_TOL
    s.close()


def test_node_forces_vs_reference(g):
    """Assembled node forces: within 1e-5 of the all-FP64 restatement (on the
    reference's rest data) and within 1e-5 of the reference's own FP32 forces,
    which carry FP32 rounding of their own (their distance from FP64 is
    printed beside the GPU's: up to 5e-6 for the stretch material's FP32 SVD
    route, against 2e-6 for the device)."""
    for material, key in ((L.PBS_MATERIAL_NEOHOOKEAN, "probe_force_nh"), (L.PBS_MATERIAL_STRETCH, "probe_force_stretch")):
        s = solver_of(g, material=material)
        f, _ = s.eval_nodes(g["probe_x"])
        f = f.astype(np.float64)
        f[g["pins"]] = 0.0
        f64, _ = O.node_eval(g["probe_x"], g["tets"], g["dminv"], g["an"], g["vol"], g["mu"], g["lam"],
                             material=material, prec=64)
        f64[g["pins"]] = 0.0
        ref = elastic_from_ref(g, key)
        e_gpu, e_ref, e_gr = rel_max(f, f64), rel_max(ref, f64), rel_max(f, ref)
        print(f"material {material}: node forces vs FP64 {e_gpu:.2e} (reference vs FP64 {e_ref:.2e}); "
              f"vs reference {e_gr:.2e}")
        assert e_gpu < 1e-5
        assert e_gr < 1e-5
        s.close()


def test_energy_and_hessian_diagonal(g):
    s = solver_of(g)
    _, en, _ = s.eval_tets(g["probe_x"])
    assert rel_max(en, g["probe_energy"]) < 2e-5
    _, hd = s.eval_nodes(g["probe_x"])
    _, hd64 = O.node_eval(g["probe_x"], g["tets"], g["dminv"], g["an"], g["vol"], g["mu"], g["lam"],
                          hessian_closed=1, prec=64)
    assert rel_max(hd, hd64) < 1e-5
    assert rel_max(hd, g["probe_hdiag"]) < 5e-3  # the reference's FP32 SVD-route noise
    s.close()


def test_trajectory_vs_reference(g):
    """DescentOptimize steps at the fixed iteration count: positions within 1e-4
    of the bbox diagonal of the reference's, the same line-search alpha."""
    s = solver_of(g)
    diag = bbox_diag(g["rest"])
    for k in range(g["traj_x"].shape[0]):
        s.step()
        x = s.positions()
        err = np.abs(x - g["traj_x"][k]).max() / diag
        assert err < POS_TOL, (g["name"], k, err)
        st = s.stats()
        assert abs(st["alpha"] - g["traj_scalars"][k, 0]) < 1e-6, (k, st)
    s.close()


def test_step_control_matches_oracle(g):
    """Same passes, rejections and final alpha as the FP32 restatement, and the
    error against the FP64 restatement stated."""
    s = solver_of(g)
    pm = pin_mask(g)
    r32 = O.rest(g["rest"], g["tets"], pm, prec=32)
    r64 = O.rest(g["rest"], g["tets"], pm, prec=64)
    p = O.make_params(h=float(g["h"]), max_iters=int(g["iters"]))
    s32, s64 = O.StepState(g["traj_x0"]), O.StepState(g["traj_x0"])
    diag = bbox_diag(g["rest"])
    for k in range(2):
        s.step()
        st = s.stats()
        o32 = O.step(s32, p, g["tets"], r32, g["mu"], g["lam"], pm, prec=32)
        O.step(s64, p, g["tets"], r64, g["mu"], g["lam"], pm, prec=64)
        assert (st["passes"], st["rejections"]) == (o32.passes, o32.rejections)
        x = s.positions()
        assert np.abs(x - s32.x0).max() / diag < POS_TOL
        assert np.abs(x - s64.x0).max() / diag < 5e-4
    s.close()


def test_bitwise_determinism():
    g = load_golden("ellipsoid_small")
    outs = []
    for _ in range(2):
        s = solver_of(g)
        for _ in range(2):
            s.step()
        outs.append(s.positions())
        s.close()
    assert np.array_equal(outs[0], outs[1])


def test_batched_instances_equal_single_runs():
    """Packing meshes of uneven size into one launch changes nothing: every
    instance's trajectory is bit-identical to its own single-mesh run."""
    gs = [load_golden(n) for n in ("bar_small", "model_bar", "ellipsoid_small")]
    h, iters = 1 / 30, 48
    rest, tets, pins, mu, lam, x0 = [], [], [], [], [], []
    nptr, tptr = [0], [0]
    for g in gs:
        off = nptr[-1]
        rest.append(g["rest"]); tets.append(g["tets"] + off); pins.append(g["pins"] + off)
        mu.append(g["mu"]); lam.append(g["lam"]); x0.append(g["traj_x0"])
        nptr.append(off + g["rest"].shape[0]); tptr.append(tptr[-1] + g["tets"].shape[0])
    mesh = M.TetMeshData(np.concatenate(rest), np.concatenate(tets), np.concatenate(pins), 1e5, 0.4,
                         instance_node_ptr=np.array(nptr), instance_tet_ptr=np.array(tptr))
    p = make_params(h=h, max_iters=iters)
    sb = DescentSolver(mesh, positions=np.concatenate(x0), mu=np.concatenate(mu), lam=np.concatenate(lam), params=p)
    for _ in range(2):
        sb.step()
    xb = sb.positions()
    for i, g in enumerate(gs):
        s = DescentSolver(mesh_of(g), positions=g["traj_x0"], mu=g["mu"], lam=g["lam"], params=p)
        for _ in range(2):
            s.step()
        assert np.array_equal(s.positions(), xb[nptr[i]:nptr[i + 1]]), i
        # the batch reports each instance's own control state
        si, sa = sb.instance_stats(i), s.stats()
        for key in ("passes", "iterations", "rejections", "converged", "status", "alpha", "residual_ratio"):
            assert si[key] == sa[key], (i, key, si[key], sa[key])
        s.close()
    sb.close()


def test_gpu_reference_preset_matches_oracle():
    """CUDAInterface semantics (gravity once, max(e,0) clamp) against the
    restatement run with the same switches."""
    g = load_golden("bar_small")
    s = solver_of(g, preset="gpu_reference")
    pm = pin_mask(g)
    r32 = O.rest(g["rest"], g["tets"], pm, prec=32)
    p = O.make_params(h=float(g["h"]), max_iters=int(g["iters"]), body_force_scale=1.0, energy_clamp=1)
    st = O.StepState(g["traj_x0"])
    for _ in range(3):
        s.step()
        O.step(st, p, g["tets"], r32, g["mu"], g["lam"], pm, prec=32)
    assert np.abs(s.positions() - st.x0).max() / bbox_diag(g["rest"]) < POS_TOL
    s.close()


@pytest.mark.parametrize("control", [L.PBS_CONTROL_REFERENCE, L.PBS_CONTROL_RESTART])
def test_residual_stop_matches_oracle(control):
    """Iterate to |g| <= 1e-4 |g_0| (FP64 norms): the GPU converges in about the
    iterations the FP64 restatement needs and lands on its solution."""
    g = load_golden("bar_small")
    prof = ((10, 0.995),)
    s = solver_of(g, preset="gpu_reference", max_iters=4000, tol=1e-4, profile=prof, control=control, alpha0=0.5,
                  energy_slack=16.0)
    pm = pin_mask(g)
    r64 = O.rest(g["rest"], g["tets"], pm, prec=64)
    p = O.make_params(h=float(g["h"]), max_iters=4000, tol=1e-4, profile=prof, control=control,
                      body_force_scale=1.0, energy_clamp=1, alpha0=0.5)
    st = O.StepState(g["traj_x0"])
    for _ in range(2):
        it = s.step()
        o = O.step(st, p, g["tets"], r64, g["mu"], g["lam"], pm, prec=64)
        stats = s.stats()
        assert stats["converged"] == 1 and o.converged == 1, (stats, o.k_final)
        assert stats["residual_ratio"] <= 1e-4
        assert abs(it - o.k_final) <= max(16, 0.1 * o.k_final), (it, o.k_final)
    assert np.abs(s.positions() - st.x0).max() / bbox_diag(g["rest"]) < POS_TOL
    s.close()


def test_stretch_material_step_matches_oracle():
    g = load_golden("ellipsoid_small")
    s = solver_of(g, material=L.PBS_MATERIAL_STRETCH)
    pm = pin_mask(g)
    r32 = O.rest(g["rest"], g["tets"], pm, prec=32)
    p = O.make_params(h=float(g["h"]), max_iters=int(g["iters"]), material=1)
    st = O.StepState(g["traj_x0"])
    for _ in range(2):
        s.step()
        O.step(st, p, g["tets"], r32, g["mu"], g["lam"], pm, prec=32)
    assert np.abs(s.positions() - st.x0).max() / bbox_diag(g["rest"]) < POS_TOL
    s.close()


def test_config1_bar_100_steps_vs_restatement():
    """Configuration 1 (40x10x10 cubes, 6-tet split, x = 0 pinned, gravity,
    h = 1/30, 96 iterations, 100 steps), compared step by step: each GPU step
    and one FP32-restatement step start from the same state (the GPU's).

    When both take the same line-search decisions (same passes and
    rejections) the positions agree within 1e-4 of the bbox diagonal.  The
    reference's accept test E > E_old is noise-driven when two energies tie
    to within FP32 rounding; a step where the two implementations break such a
    tie differently must stay within 1e-3, and such steps must be rare.  The
    first three steps are also checked against the reference's own trajectory."""
    g = load_golden("bar_config1")
    s = solver_of(g)
    pm = pin_mask(g)
    r32 = O.rest(g["rest"], g["tets"], pm, prec=32)
    p = O.make_params(h=float(g["h"]), max_iters=96)
    diag = bbox_diag(g["rest"])
    x, (v, vo) = g["traj_x0"].astype(np.float32), (np.zeros_like(g["rest"]), np.zeros_like(g["rest"]))
    flips, worst_same = [], 0.0
    for k in range(100):
        st = O.StepState(x, v, vo)
        o = O.step(st, p, g["tets"], r32, g["mu"], g["lam"], pm, prec=32)
        s.step()
        gs = s.stats()
        x = s.positions()
        v, vo = s.velocities()
        err = np.abs(x - st.x0).max() / diag
        if (gs["passes"], gs["rejections"]) == (o.passes, o.rejections):
            worst_same = max(worst_same, err)
            assert err < POS_TOL, (k, err)
        else:
            flips.append((k, err))
            assert err < 1e-3, (k, err, gs, o.passes, o.rejections)
        if k < g["traj_x"].shape[0]:
            assert np.abs(x - g["traj_x"][k]).max() / diag < POS_TOL
    assert len(flips) <= 5, flips
    s.close()


@pytest.mark.parametrize("material", [L.PBS_MATERIAL_STRETCH, L.PBS_MATERIAL_NEOHOOKEAN])
def test_ellipsoid_42k_twist_release_vs_restatement(material):
    """The 42K-tet ellipsoid (20x20x40-cube grid, 5-tet split, interior nodes
    jittered by +-0.15 cell, E = 1e5, nu = 0.45, lowest 5% of nodes pinned)
    released from a 90-degree twist about its long axis: h = 1/60, 64
    iterations per step, stretch-based and neo-Hookean.  Twelve steps compared
    step by step against the FP32 restatement, each pair starting from the
    GPU's state, with the tie rule of the bar test."""
    m = M.ellipsoid_mesh()
    x = M.twist_positions(m.rest, np.pi / 2, axis=2)
    mu, lam = O.lame(m.young, m.poisson)
    s = DescentSolver(m, positions=x, material=material, mu=mu, lam=lam,
                      params=make_params("cpu_reference", h=1 / 60, max_iters=64))
    pm = m.pin_mask()
    r32 = O.rest(m.rest, m.tets, pm, prec=32)
    p = O.make_params(h=1 / 60, max_iters=64, material=int(material == L.PBS_MATERIAL_STRETCH))
    diag = bbox_diag(m.rest)
    v = vo = np.zeros_like(m.rest)
    flips = []
    for k in range(12):
        st = O.StepState(x, v, vo)
        o = O.step(st, p, m.tets, r32, mu, lam, pm, prec=32)
        s.step()
        gs = s.stats()
        x = s.positions()
        v, vo = s.velocities()
        assert np.isfinite(x).all()
        err = np.abs(x - st.x0).max() / diag
        if (gs["passes"], gs["rejections"]) == (o.passes, o.rejections):
            assert err < POS_TOL, (k, err)
        else:
            flips.append((k, err))
            assert err < 1e-3, (k, err, gs, o.passes, o.rejections)
    assert len(flips) <= 2, flips
    # the body untwists: the top has turned back from 90 degrees
    top = m.rest[:, 2] >= m.rest[:, 2].max() - 1e-6
    assert np.abs(x[top] - M.twist_positions(m.rest, np.pi / 2, axis=2)[top]).max() > 1e-3 * diag
    s.close()


def test_state_roundtrip_and_reset():
    """Positions and velocities read back and written into a fresh handle
    continue the same trajectory (to FP32 rounding: the device carries a
    compensated displacement the FP32 read-back rounds)."""
    g = load_golden("bar_small")
    s = solver_of(g)
    s.step()
    x = s.positions()
    v, vo = s.velocities()
    s2 = solver_of(g)
    s2.update_positions(x)
    s2.write_velocities(v, vo)
    s.step()
    s2.step()
    assert np.abs(s.positions() - s2.positions()).max() / bbox_diag(g["rest"]) < 1e-6
    s.reset()
    assert np.array_equal(s.positions(), g["rest"])
    assert not s.velocities()[0].any()
    s.close()
    s2.close()


def test_nonfinite_input_reports_status():
    g = load_golden("bar_small")
    s = solver_of(g)
    ext = np.zeros_like(g["rest"])
    ext[5, 1] = np.nan
    s.step(ext, raise_on_error=False)
    assert s.last_status == L.PBS_E_NONFINITE
    s.close()


def test_pass_cap_reports_status():
    g = load_golden("bar_small")
    s = solver_of(g, pass_cap=5)
    s.step(raise_on_error=False)
    assert s.last_status == L.PBS_E_ITER_CAP and s.stats()["passes"] == 5
    s.close()


def test_bad_meshes_rejected():
    m = M.bar_mesh(2, 2, 2)
    bad = m.tets.copy()
    bad[0, [2, 3]] = bad[0, [3, 2]]  # inverted rest tet
    with pytest.raises(L.PhybsError) as e:
        DescentSolver(M.TetMeshData(m.rest, bad, m.pins, 1e5, 0.4))
    assert e.value.code == L.PBS_E_BAD_MESH
    bad = m.tets.copy()
    bad[1, 0] = m.n_nodes + 3  # index out of range
    with pytest.raises(L.PhybsError) as e:
        DescentSolver(M.TetMeshData(m.rest, bad, m.pins, 1e5, 0.4))
    assert e.value.code == L.PBS_E_BAD_MESH


def test_cuda_interface_wrapper():
    """CUDAInterface's call shape (fvm.cpp:44-47, 187-188)."""
    g = load_golden("model_bar")
    n, t = g["rest"].shape[0], g["tets"].shape[0]
    ci = CUDAInterface(n, g["traj_x0"].ravel(), g["rest"].ravel(), pin_mask(g), t, g["tets"].ravel(),
                       float(g["young"]), float(g["poisson"]), 1000.0)
    host = np.zeros(3 * n, np.float32)
    ci.doDescentOpt(0.03, 96, np.zeros(3 * n, np.float32), host)
    assert np.isfinite(host).all() and np.abs(host.reshape(-1, 3) - g["rest"]).max() > 0
    ci.reset()


def test_autotune_keeps_results():
    """pbs_autotune picks one of its chunk shapes by timing them on the mesh;
    a tuned handle steps to the same positions as an untuned one (the shape
    only changes the order corner forces are summed in)."""
    m = M.box_mesh(12, 12, 20, edge=0.01, seed=4, young=1e5, poisson=0.4)
    p = make_params("gpu_reference", h=1 / 30, max_iters=64)
    a = DescentSolver(m, params=p)
    b = DescentSolver(m, params=p)
    r = b.autotune(8)
    assert r["n_tried"] == 20 and r["chunk_threads"] in (128, 256, 512)
    assert 0.0 < r["pass_ms"] <= r["default_pass_ms"]
    for _ in range(3):
        a.step()
        b.step()
    assert np.abs(a.positions() - b.positions()).max() / m.bbox_diagonal() < 1e-5
    a.close()
    b.close()


def test_restart_control_recovers_from_nonfinite_iterates():
    """A step size far beyond the stable one (alpha0 = 3) inverts tets within
    six passes: the residual turns non-finite before the first scheduled
    energy check.  RESTART control then checks the energy at once (an inverted
    tet's energy counts as non-finite, not as the reference clamps' 0),
    rejects, restores the last accepted iterate with a smaller step, and the
    step still converges -- as the FP64 restatement does."""
    m = M.bar_mesh(8, 4, 4, edge=0.025, young=5e4, poisson=0.4)
    p = make_params("gpu_reference", h=1 / 30, max_iters=20000, tol=1e-4, control=L.PBS_CONTROL_RESTART,
                    alpha0=3.0, energy_slack=16.0, profile=((10, 0.995),))
    s = DescentSolver(m, params=p)
    s.step()
    st = s.stats()
    assert st["status"] == 0 and st["converged"] == 1 and st["rejections"] >= 1, st
    x = s.positions()
    assert np.isfinite(x).all()
    mu, lam = O.lame(m.young, m.poisson)
    r = O.rest(m.rest, m.tets, m.pin_mask(), prec=64)
    ref = O.StepState(m.rest)
    po = O.make_params(h=1 / 30, max_iters=20000, tol=1e-4, control=1, alpha0=3.0, body_force_scale=1.0,
                       energy_clamp=1, profile=((10, 0.995),), hessian_closed=1)
    so = O.step(ref, po, m.tets, r, mu, lam, m.pin_mask(), prec=64)
    assert so.converged == 1 and so.rejections >= 1
    # both stop at |g| <= 1e-4 |g0|: positions agree to well within the step
    assert np.abs(x - ref.x0).max() / m.bbox_diagonal() < 1e-4
    s.close()


def test_inverting_guess_falls_back_to_start_positions():
    """A bar pinned at both ends, its far face pulled 4 cm (1.6 cells) a frame
    for four frames, then held: in the first held frame the inertial guess
    carries the free nodes' momentum through the held face and inverts tets.
    RESTART control starts that step from the start positions instead; every
    frame converges, and positions follow the FP64 restatement, which does the
    same."""
    b = M.bar_mesh(8, 4, 4, edge=0.025, young=5e4, poisson=0.4)
    x = b.rest[:, 0]
    pins = np.nonzero((x <= x.min() + 1e-9) | (x >= x.max() - 1e-9))[0].astype(np.int32)
    far = np.nonzero(x >= x.max() - 1e-9)[0].astype(np.int32)
    m = M.TetMeshData(b.rest, b.tets, pins, 5e4, 0.4)
    h = 1 / 30
    p = make_params("gpu_reference", h=h, max_iters=20000, tol=1e-4, control=L.PBS_CONTROL_RESTART, alpha0=0.5,
                    energy_slack=16.0, profile=((10, 0.995),))
    s = DescentSolver(m, params=p)
    mu, lam = O.lame(m.young, m.poisson)
    r = O.rest(m.rest, m.tets, m.pin_mask(), prec=64)
    ref = O.StepState(m.rest)
    po = O.make_params(h=h, max_iters=20000, tol=1e-4, control=1, alpha0=0.5, body_force_scale=1.0, energy_clamp=1,
                       profile=((10, 0.995),), hessian_closed=1)
    fallbacks = []
    for f in range(7):
        tgt = m.rest[far].astype(np.float64).copy()
        tgt[:, 0] += 0.04 * min(f + 1, 4)
        s.set_node_positions(far, tgt.astype(np.float32))
        s.step()
        st = s.stats()
        assert st["status"] == 0 and st["converged"] == 1, (f, st)
        fallbacks.append(st["guess_fallbacks"])
        ref.x0[far] = tgt
        so = O.step(ref, po, m.tets, r, mu, lam, m.pin_mask(), prec=64)
        assert so.converged == 1, f
        assert np.abs(s.positions() - ref.x0).max() / m.bbox_diagonal() < 2e-4, f
    assert fallbacks[4] == 1 and sum(fallbacks) >= 1, fallbacks
    s.close()


@pytest.mark.parametrize("incremental", [0, 1])
def test_row_staged_chunk_kernel_matches_unstaged(incremental):
    """The row-staged pass kernel (per-tet rows copied into shared memory
    asynchronously) computes exactly what the unstaged one computes for the same
    chunk shape: same corner forces, same order of summation."""
    m = M.box_mesh(12, 12, 20, edge=0.01, seed=4, young=1e5, poisson=0.4)
    p = make_params("gpu_reference", h=1 / 30, max_iters=64, incremental_stress=incremental)
    a = DescentSolver(m, params=p)
    b = DescentSolver(m, params=p)
    a.set_chunk_shape(256, 512, 256, 0, 1)
    b.set_chunk_shape(256, 512, 256, 1, 2)
    for _ in range(3):
        a.step()
        b.step()
    # same corner forces; the node kernel's two-nodes-per-thread variant changes
    # only the order of the |g|^2 reduction
    assert np.abs(a.positions() - b.positions()).max() / m.bbox_diagonal() < 1e-6
    with pytest.raises(L.PhybsError):
        b.set_chunk_shape(512, 512, 256, 1, 1)  # no staged variant with 512 threads
    a.close()
    b.close()


@pytest.mark.parametrize("incremental", [0, 1])
@pytest.mark.parametrize("shape", [(256, 256, 160), (128, 128, 96)])
def test_persistent_chunk_kernel_matches_staged(incremental, shape):
    """The persistent chunk kernel (each CTA walks a strided list of chunks;
    rows and records arrive by bulk copies into two staging buffers while the
    previous chunk computes) is bit-identical to the one-CTA-per-chunk kernel
    of the same chunk shape.  The 264,000-tet box has more chunks than the
    device holds CTAs, so every CTA runs the pipeline over several chunks;
    64 iterations cover line-search checks and Jacobi refreshes."""
    m = M.box_mesh(30, 40, 44, edge=0.005, seed=6, young=3e5, poisson=0.4)
    assert m.n_tets == 264000
    p = make_params("gpu_reference", h=1 / 30, max_iters=64, incremental_stress=incremental)
    x0 = M.twist_positions(m.rest, 0.6, axis=2)
    a = DescentSolver(m, positions=x0, params=p)
    b = DescentSolver(m, positions=x0, params=p)
    a.set_chunk_shape(*shape, 1, 1)
    b.set_chunk_shape(*shape, 2, 1)
    for _ in range(3):
        a.step()
        b.step()
        sa, sb = a.stats(), b.stats()
        assert (sa["passes"], sa["rejections"], sa["energy"]) == (sb["passes"], sb["rejections"], sb["energy"])
    assert np.array_equal(a.positions(), b.positions())
    a.close()
    b.close()


def test_persistent_chunk_kernel_packed_batch():
    """A packed batch whose instances stop at different passes (residual
    tolerance, RESTART control with rejections): the persistent kernel skips
    the chunks of finished instances exactly as the one-CTA-per-chunk kernel
    does, instance by instance."""
    packed = M.batch_of_boxes(48, seed=11, nxy=(4, 12), nz=(8, 24))
    p = make_params("gpu_reference", h=1 / 30, max_iters=3000, tol=1e-3, control=L.PBS_CONTROL_RESTART,
                    alpha0=0.3, energy_slack=16.0, alpha_grow=1.2, incremental_stress=1)
    a = DescentSolver(packed, params=p)
    b = DescentSolver(packed, params=p)
    a.set_chunk_shape(128, 128, 96, 1, 1)
    b.set_chunk_shape(128, 128, 96, 2, 1)
    for _ in range(2):
        a.step()
        b.step()
    passes = set()
    for i in range(packed.n_instances):
        sa, sb = a.instance_stats(i), b.instance_stats(i)
        sa.pop("device_ms"), sb.pop("device_ms")  # wall time, not a result
        assert sa == sb, i
        passes.add(sa["passes"])
    assert len(passes) > 1  # the instances did stop at different passes
    assert np.array_equal(a.positions(), b.positions())
    a.close()
    b.close()


def test_alpha_growth_matches_oracle():
    """RESTART control with alpha_grow: the step size shrinks on a rejection and
    recovers by the growth factor on later accepted checks (never above
    alpha0); GPU and the FP64 restatement both converge to the same positions."""
    m = M.bar_mesh(8, 4, 4, edge=0.025, young=5e4, poisson=0.4)
    p = make_params("gpu_reference", h=1 / 30, max_iters=20000, tol=1e-4, control=L.PBS_CONTROL_RESTART,
                    alpha0=1.0, energy_slack=16.0, profile=((10, 0.995),), alpha_grow=1.2)
    s = DescentSolver(m, params=p)
    mu, lam = O.lame(m.young, m.poisson)
    r = O.rest(m.rest, m.tets, m.pin_mask(), prec=64)
    ref = O.StepState(m.rest)
    po = O.make_params(h=1 / 30, max_iters=20000, tol=1e-4, control=1, alpha0=1.0, body_force_scale=1.0,
                       energy_clamp=1, profile=((10, 0.995),), hessian_closed=1, alpha_grow=1.2)
    for f in range(3):
        s.step()
        st = s.stats()
        so = O.step(ref, po, m.tets, r, mu, lam, m.pin_mask(), prec=64)
        assert st["converged"] == 1 and so.converged == 1, (f, st)
        assert 0.0 < st["alpha"] <= 1.0
        assert np.abs(s.positions() - ref.x0).max() / m.bbox_diagonal() < 2e-4, f
    s.close()
