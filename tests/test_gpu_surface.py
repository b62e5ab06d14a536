"""GPU parity of surface picking and drag forces (pbs_set_surface,
pbs_get_face_ring, pbs_pick_face, pbs_drag_face_ring) through the C ABI,
against the reference's own outputs on its bar and dragon meshes
(tests/golden/surface_*.npz: rings and picks bit-exact, drag forces within the
lumped masses' 2e-6) and bit-exact against the restatement (oracle/surface.py)
given the device's masses, on a 25,600-face box whose pick runs as a
multi-block reduction."""
import numpy as np
import pytest

from oracle import restated as O
from oracle import surface as S
from phybs_gb300 import _lib as L
from phybs_gb300 import meshes as M
from phybs_gb300.solver import DescentSolver, make_params
from tests._util import golden_names, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from phybs_gb300.build import build
    build()


@pytest.fixture(scope="module", params=golden_names("surface_"))
def sg(request):
    return load_golden(request.param)


def solver_for(sg):
    m = M.TetMeshData(sg["rest"], sg["tets"], sg["pins"], 5e5, 0.45)
    s = DescentSolver(m)
    s.set_surface(sg["faces"])
    return s


def test_rings_match_reference(sg):
    s = solver_for(sg)
    ptr, ring = sg["ring_ptr"], sg["ring"]
    for f in range(len(ptr) - 1):
        assert np.array_equal(s.face_ring(f), ring[ptr[f]:ptr[f + 1]]), f
    s.close()


@pytest.mark.parametrize("k", [0, 1])
def test_picks_and_drags_match_reference(sg, k):
    """Picks and drag forces bit-exact against the restatement at the device's
    positions and lumped masses; picks equal the reference's where the
    positions round-trip exactly (the rest shape), drag forces are within 2e-6
    of the reference's (the device sums a node's corner masses in FP64, the
    reference in FP32)."""
    s = solver_for(sg)
    x = sg[f"x{k}"]
    s.update_positions(x)
    # the positions the kernels see: rest + (u hi + u lo), which can differ from
    # the uploaded FP32 positions in the last bit (the rest shape round-trips)
    xd = s.positions()
    assert np.abs(xd - x).max() <= 1e-6 * np.abs(x).max()
    exact = np.array_equal(xd, x)
    assert exact or k == 1
    for o, d, want in zip(sg[f"ray_orig{k}"], sg[f"ray_dir{k}"], sg[f"pick{k}"]):
        f = s.pick_face(o, d)
        assert f == S.pick_face(xd, sg["faces"], o, d)
        if exact:
            assert f == want
    mass = s.rest_data()[2]
    assert np.abs(mass - sg["mass"]).max() <= 2e-6 * np.abs(sg["mass"][sg["mass"] < 1e7]).max()
    rings = S.face_rings(sg["faces"], x.shape[0])
    for j, (f, d) in enumerate(zip(sg[f"drag_face{k}"], sg[f"drag{k}"])):
        got = s.drag_face_ring(int(f), d)
        assert np.array_equal(got, S.drag_face_ring(xd, mass, sg["faces"], rings, int(f), d)), j
        ref = sg[f"drag_ext{k}"][j]
        assert np.abs(got - ref).max() <= 2e-6 * np.abs(ref).max(), j
    s.close()


def test_large_surface_matches_restatement():
    """A 40 x 40 x 60-cube box: 25,600 surface triangles, picks over many
    blocks, on a twisted state, against the restatement."""
    m = M.box_mesh(40, 40, 60, edge=0.005, seed=2)
    faces = M.surface_faces(m.rest, m.tets)
    assert faces.shape[0] == 25600
    s = DescentSolver(m)
    s.set_surface(faces)
    x = M.twist_positions(m.rest, 0.5, axis=2)
    s.update_positions(x)
    x = s.positions()
    rings = S.face_rings(faces, x.shape[0])
    mass = s.rest_data()[2]
    rng = np.random.default_rng(5)
    hits = 0
    for _ in range(32):
        d = rng.normal(size=3).astype(np.float32)
        d /= np.linalg.norm(d)
        o = (x[rng.integers(len(x))] - 0.05 * d).astype(np.float32)
        f = s.pick_face(o, d)
        assert f == S.pick_face(x, faces, o, d)
        if f >= 0:
            hits += 1
            drag = rng.normal(0.0, 0.02, 3).astype(np.float32)
            assert np.array_equal(s.drag_face_ring(f, drag), S.drag_face_ring(x, mass, faces, rings, f, drag))
    assert hits >= 16
    s.close()


def test_drag_drives_a_step():
    """The drag field as a step's external forces: the dragged face moves
    along the drag, and the step equals the FP32 restatement's with the same
    forces."""
    m = M.bar_mesh(8, 4, 4, edge=0.025, young=5e4, poisson=0.4)
    faces = M.surface_faces(m.rest, m.tets)
    p = make_params("gpu_reference", h=1 / 30, max_iters=64)
    s = DescentSolver(m, params=p)
    s.set_surface(faces)
    tip = int(np.argmax(m.rest[:, 0]))
    f = next(i for i, q in enumerate(faces) if tip in q)
    ext = s.drag_face_ring(f, np.array([0.0, 0.05, 0.0], np.float32))
    assert (ext[:, 1] >= 0).all() and ext[:, 1].max() > 0
    pm = m.pin_mask()
    r32 = O.rest(m.rest, m.tets, pm, prec=32)
    mu, lam = O.lame(m.young, m.poisson)
    st = O.StepState(m.rest)
    o = O.step(st, O.make_params(h=1 / 30, max_iters=64, body_force_scale=1.0, energy_clamp=1),
               m.tets, r32, mu, lam, pm, ext=ext, prec=32)
    s.step(ext=ext)
    x = s.positions()
    ring = s.face_ring(f)
    assert (x[ring, 1] - m.rest[ring, 1]).mean() > (x[:, 1] - m.rest[:, 1]).mean()
    assert np.abs(x - st.x0).max() / m.bbox_diagonal() < 1e-4, (s.stats(), o)
    s.close()


def test_surface_argument_checks():
    m = M.bar_mesh(4, 2, 2)
    s = DescentSolver(m)
    with pytest.raises(L.PhybsError):
        s.pick_face([0, 0, 1], [0, 0, -1])  # no surface yet
    faces = M.surface_faces(m.rest, m.tets)
    with pytest.raises(L.PhybsError):
        s.set_surface(np.array([[0, 1, m.n_nodes]]))  # node id out of range
    s.set_surface(faces)
    with pytest.raises(L.PhybsError):
        s.drag_face_ring(len(faces), [0, 1, 0])
    with pytest.raises(L.PhybsError):
        s.pick_face([0, 0, np.nan], [0, 0, -1])
    s.set_surface(np.zeros((0, 3), np.int32))  # clears it
    with pytest.raises(L.PhybsError):
        s.drag_face_ring(0, [0, 1, 0])
    s.close()
