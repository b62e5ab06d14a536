"""Host-side tests that need no GPU: mesh generators, the C ABI's exports and
host-only entry points, and the canonical gather order."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from oracle import restated as O
from phybs_gb300 import _lib as L
from phybs_gb300 import meshes as M
from tests._util import golden_names, load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from phybs_gb300.build import build
    build()
    return L.lib()


def _faces_ok(tets):
    """Conformity: every triangle is shared by at most two tets."""
    f = np.sort(np.concatenate([tets[:, [0, 1, 2]], tets[:, [0, 1, 3]], tets[:, [0, 2, 3]], tets[:, [1, 2, 3]]]), 1)
    _, cnt = np.unique(f, axis=0, return_counts=True)
    return cnt.max() <= 2


def test_bar_config_sizes():
    m = M.bar_mesh()
    assert (m.n_tets, m.n_nodes, len(m.pins)) == (24000, 4961, 121)
    assert (M.signed_volumes(m.rest, m.tets) > 0).all()
    assert _faces_ok(m.tets)


def test_box_config_sizes_small_and_formula():
    m = M.box_mesh(6, 5, 8, edge=0.005, jitter=0.1, seed=3)
    assert m.n_tets == 5 * 6 * 5 * 8 and m.n_nodes == 7 * 6 * 9
    assert (M.signed_volumes(m.rest, m.tets) > 0).all()
    assert _faces_ok(m.tets)
    # 50 x 50 x 80 cubes: 1,000,000 tets and 210,681 nodes
    assert 5 * 50 * 50 * 80 == 1_000_000 and 51 * 51 * 81 == 210_681


def test_ellipsoid_config():
    m = M.ellipsoid_mesh()
    assert 40_000 < m.n_tets < 44_000 and 9_000 < m.n_nodes < 10_500
    assert (M.signed_volumes(m.rest, m.tets) > 0).all()
    assert _faces_ok(m.tets)
    assert abs(len(m.pins) - 0.05 * m.n_nodes) <= 1


def test_batch_packing():
    m = M.batch_of_boxes(8, seed=1)
    assert m.n_instances == 8
    for b in range(8):
        t = m.tets[m.instance_tet_ptr[b]:m.instance_tet_ptr[b + 1]]
        assert t.min() >= m.instance_node_ptr[b] and t.max() < m.instance_node_ptr[b + 1]
    assert (M.signed_volumes(m.rest, m.tets) > 0).all()


def test_twist_preserves_lengths_along_axis():
    m = M.bar_mesh(4, 2, 2)
    x = M.twist_positions(m.rest, np.pi / 2, axis=0)
    c = 0.5 * (m.rest.min(0) + m.rest.max(0))
    r0 = np.linalg.norm(m.rest[:, 1:] - c[1:], axis=1)
    r1 = np.linalg.norm(x[:, 1:] - c[1:], axis=1)
    assert np.allclose(r0, r1, atol=1e-6) and np.allclose(x[:, 0], m.rest[:, 0])


def test_incidence_canonical_order():
    m = M.ellipsoid_mesh(6, 6, 10)
    row, ent = M.incidence_csr(m.tets, m.n_nodes)
    row_o, ent_o = O.incidence(m.tets, m.n_nodes)
    assert np.array_equal(row, row_o) and np.array_equal(ent, ent_o)


def test_tetgen_roundtrip(tmp_path):
    m = M.bar_mesh(3, 2, 2)
    stem = str(tmp_path / "bar.1")
    M.write_tetgen_nodes(stem + ".node", m.rest)
    with open(stem + ".ele", "w") as f:
        f.write(f"{m.n_tets} 4 0\n")
        for i, t in enumerate(m.tets):
            f.write(f"{i} {t[0]} {t[1]} {t[2]} {t[3]}\n")
    m2 = M.load_tetgen(stem)
    assert np.array_equal(m2.tets, m.tets) and np.allclose(m2.rest, m.rest)


def test_library_exports_every_declared_symbol(lib):
    hdr = open(os.path.join(ROOT, "include", "phybs.h")).read()
    declared = set(re.findall(r"\b(pbs_[a-z_0-9]+)\s*\(", hdr))
    assert declared == set(L.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name


def test_default_params_are_reference_preset(lib):
    p = L.default_params()
    assert (p.h, p.max_iters, p.line_search_every, p.hessian_every) == (pytest.approx(0.03), 96, 8, 32)
    assert (p.alpha0, p.alpha_min, p.alpha_shrink) == (pytest.approx(0.1), pytest.approx(0.01), pytest.approx(0.7))
    assert [p.profile_k[i] for i in range(p.n_profile)] == [1, 7, 10]
    assert np.allclose([p.profile_rho[i] for i in range(3)], [0.96, 0.991, 0.999])
    assert p.body_force_scale == 2.0 and p.energy_clamp == L.PBS_CLAMP_CPU


def test_lame_matches_reference_formula(lib):
    for name in golden_names():
        g = load_golden(name)
        mu, lam = L.lame(float(g["young"]), float(g["poisson"]))
        assert np.float32(mu) == g["mu"][0] and np.float32(lam) == g["lam"][0]
    mu, lam = L.lame(1e5, 0.25, reference_formula=False)
    assert lam == pytest.approx(2 * mu * 0.25 / 0.5, rel=1e-6)


def test_error_strings(lib):
    for code in range(0, -9, -1):
        assert L.error_string(code) not in ("", "unknown error")


def test_stiffness_pattern_bit_exact(lib):
    """pbs_stiffness_pattern == IsotropicMaterial::allocateGlobalStiffnessMatrix."""
    from phybs_gb300.solver import stiffness_pattern
    n = 0
    for name in golden_names():
        g = load_golden(name)
        if "csr_row" not in g:
            continue
        row, col, diag, kid = stiffness_pattern(g["rest"].shape[0], g["tets"])
        assert np.array_equal(row, g["csr_row"]) and np.array_equal(col, g["csr_col"])
        assert np.array_equal(diag, g["csr_diag"]) and np.array_equal(kid, g["csr_kid"])
        n += 1
    assert n >= 3


def test_create_rejects_bad_input_without_device(lib):
    h = C.c_void_p()
    assert lib.pbs_create(None, C.byref(h)) == L.PBS_E_INVALID_ARG
    m = M.bar_mesh(2, 1, 1)
    rest = np.ascontiguousarray(m.rest, np.float32)
    tets = np.ascontiguousarray(m.tets, np.int32)
    d = L.MeshDesc(m.n_nodes, rest.ctypes.data, None, m.n_tets, tets.ctypes.data, None, 1, None, None, 1000.0, 9.8)
    rc = lib.pbs_create(C.byref(d), C.byref(h))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert rc == L.PBS_E_NO_DEVICE
    elif rc == L.PBS_OK:
        lib.pbs_destroy(h)
    d.density = -1.0
    assert lib.pbs_create(C.byref(d), C.byref(h)) == L.PBS_E_INVALID_ARG


def test_params_validation(lib):
    p = L.default_params()
    p.h = 0.0
    assert lib.pbs_set_params(None, C.byref(p)) == L.PBS_E_INVALID_ARG


def build_cpp_demo(tmp_path):
    import subprocess
    from phybs_gb300.build import LIB, build
    build()
    exe = str(tmp_path / "cuda_interface_demo")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "cuda_interface_demo.cpp"), LIB,
                    "-Wl,-rpath," + os.path.dirname(LIB), "-o", exe], check=True)
    return exe


def test_cpp_cuda_interface_wrapper_compiles_and_runs(tmp_path):
    """The header-only CUDAInterface wrapper builds against the C ABI; without
    a GB300 its constructor throws with PBS_E_NO_DEVICE."""
    import subprocess
    exe = build_cpp_demo(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    assert out[0] == "pattern" and int(out[1]) > 0
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert out[2:] == ["error", str(L.PBS_E_NO_DEVICE)]
