"""pbs_eval_nodes_static (forces with no device allocation in the call)
against pbs_eval_nodes, through the C ABI, on consecutive calls that share the
library's static scratch."""
import ctypes as C

import numpy as np
import pytest

from phybs_gb300 import _lib as L
from phybs_gb300 import meshes as M
from phybs_gb300.solver import DescentSolver

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

# the force tolerance of the other parity tests: 1e-5 of the largest force
RTOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


def _deformed(mesh, seed):
    """Rest positions stretched along x about each node's own coordinate
    origin and jittered by 5% of the mean edge: no tet inverts."""
    rng = np.random.default_rng(seed)
    edge = float(np.cbrt(6.0 * np.abs(M.signed_volumes(mesh.rest, mesh.tets)).mean()))
    x = mesh.rest.astype(np.float64) + rng.normal(0.0, 0.05 * edge, mesh.rest.shape)
    x[:, 0] += 0.05 * seed * (mesh.rest[:, 0] - np.floor(mesh.rest[:, 0]))  # a stretch that differs between calls
    x = x.astype(np.float32)
    assert (M.signed_volumes(x, mesh.tets) * M.signed_volumes(mesh.rest, mesh.tets) > 0).all()
    return x


def _static_forces(s, x):
    # the handle's stream does not wait for torch's: the inputs are written,
    # and the forces read, on that stream itself
    with torch.cuda.stream(torch.cuda.ExternalStream(s.stream())):
        xd = torch.from_numpy(np.ascontiguousarray(x.reshape(-1))).to("cuda")
        fd = torch.full_like(xd, float("nan"))
        rc = L.lib().pbs_eval_nodes_static(s._h, C.c_void_p(xd.data_ptr()), C.c_void_p(fd.data_ptr()))
        L.check(rc, "pbs_eval_nodes_static")
        out = fd.cpu().numpy().reshape(-1, 3)
    torch.cuda.synchronize()
    return out


@pytest.mark.parametrize("material", [L.PBS_MATERIAL_NEOHOOKEAN, L.PBS_MATERIAL_STRETCH])
def test_static_scratch_forces_match_eval_nodes(material):
    mesh = M.box_mesh(12, 10, 16, edge=0.01, seed=3, young=2e5, poisson=0.4)
    s = DescentSolver(mesh, material=material)
    for call in (1, 2):  # two calls in a row reuse the same scratch
        x = _deformed(mesh, call)
        ref, _ = s.eval_nodes(x)
        got = _static_forces(s, x)
        assert np.isfinite(got).all()
        scale = np.abs(ref).max()
        assert scale > 0
        assert np.abs(got - ref).max() <= RTOL * scale, (call, np.abs(got - ref).max() / scale)
    s.close()


def test_static_scratch_allocates_nothing():
    """After one call (which loads the library's device image, scratch
    included), further calls leave the device's free memory unchanged and the
    caller's current device as it was."""
    mesh = M.box_mesh(10, 8, 12, edge=0.01, seed=4, young=2e5, poisson=0.4)
    s = DescentSolver(mesh)
    x = _deformed(mesh, 1)
    with torch.cuda.stream(torch.cuda.ExternalStream(s.stream())):
        xd = torch.from_numpy(np.ascontiguousarray(x.reshape(-1))).to("cuda")
        fd = torch.empty_like(xd)
    torch.cuda.synchronize()
    lib = L.lib()
    args = (s._h, C.c_void_p(xd.data_ptr()), C.c_void_p(fd.data_ptr()))
    L.check(lib.pbs_eval_nodes_static(*args), "pbs_eval_nodes_static")
    torch.cuda.synchronize()
    dev = torch.cuda.current_device()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(8):
        L.check(lib.pbs_eval_nodes_static(*args), "pbs_eval_nodes_static")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert torch.cuda.current_device() == dev
    ref, _ = s.eval_nodes(x)
    got = fd.cpu().numpy().reshape(-1, 3)
    assert np.abs(got - ref).max() <= RTOL * np.abs(ref).max()
    s.close()


def test_static_scratch_packed_instances():
    packed = M.batch_of_boxes(12, seed=5, nxy=(3, 6), nz=(4, 9))
    s = DescentSolver(packed)
    for call in (1, 2):
        x = _deformed(packed, call)
        ref, _ = s.eval_nodes(x)
        got = _static_forces(s, x)
        assert np.abs(got - ref).max() <= RTOL * np.abs(ref).max()
    s.close()


def test_static_scratch_rejects_host_pointers_and_oversize():
    mesh = M.bar_mesh(4, 2, 2)
    s = DescentSolver(mesh)
    x = np.ascontiguousarray(mesh.rest.reshape(-1), dtype=np.float32)
    f = np.empty_like(x)
    rc = L.lib().pbs_eval_nodes_static(s._h, C.c_void_p(x.ctypes.data), C.c_void_p(f.ctypes.data))
    assert rc == L.PBS_E_INVALID_ARG
    s.close()
    big = M.box_mesh(50, 50, 42, edge=0.005)  # 525,000 tets > PBS_EVAL_STATIC_MAX_TETS
    assert big.n_tets > L.PBS_EVAL_STATIC_MAX_TETS
    s = DescentSolver(big)
    xd = torch.zeros(3 * big.n_nodes, device="cuda")
    fd = torch.zeros_like(xd)
    rc = L.lib().pbs_eval_nodes_static(s._h, C.c_void_p(xd.data_ptr()), C.c_void_p(fd.data_ptr()))
    assert rc == L.PBS_E_CAPACITY
    s.close()
