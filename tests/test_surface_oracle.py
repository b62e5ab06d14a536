"""Pin the surface restatement (oracle/surface.py) to the reference's own
outputs (tests/golden/surface_*.npz: TetMesh's rings, picks, normals, centres,
drag forces and drag energies on its shipped bar and dragon meshes), bit for
bit, and check the host-side boundary extraction against the shipped .face
files' triangles."""
import numpy as np
import pytest

from oracle import surface as S
from phybs_gb300 import meshes as M
from tests._util import golden_names, load_golden

NAMES = golden_names("surface_")


@pytest.fixture(scope="module", params=NAMES)
def sg(request):
    return load_golden(request.param)


def test_fixture_set():
    assert NAMES == ["surface_model_bar", "surface_model_dragon"]


def test_rings(sg):
    """TetMesh::computeBoundfaceRingIndices (TetMesh.cpp:229-277)."""
    rings = S.face_rings(sg["faces"], sg["rest"].shape[0])
    ptr, ring = sg["ring_ptr"], sg["ring"]
    assert len(rings) == len(ptr) - 1
    for f, r in enumerate(rings):
        assert np.array_equal(r, ring[ptr[f]:ptr[f + 1]]), f


@pytest.mark.parametrize("k", [0, 1])
def test_normals_centres_and_picks(sg, k):
    """computeBoundfaceNormals + pickFacebyRay (TetMesh.cpp:378-418), hits and misses."""
    x = sg[f"x{k}"]
    n, c = S.normals_centers(x, sg["faces"])
    assert np.array_equal(n, sg[f"normals{k}"]) and np.array_equal(c, sg[f"centers{k}"])
    picks = [S.pick_face(x, sg["faces"], o, d) for o, d in zip(sg[f"ray_orig{k}"], sg[f"ray_dir{k}"])]
    assert np.array_equal(picks, sg[f"pick{k}"])
    assert (sg[f"pick{k}"] < 0).sum() == 4 and (sg[f"pick{k}"] >= 0).sum() == 20


@pytest.mark.parametrize("k", [0, 1])
def test_drag_forces_and_energy(sg, k):
    """dragFaceRing and computeExternalForcesEnergy (TetMesh.cpp:443-470, 595-614)."""
    x = sg[f"x{k}"]
    rings = S.face_rings(sg["faces"], x.shape[0])
    for j, (f, d) in enumerate(zip(sg[f"drag_face{k}"], sg[f"drag{k}"])):
        ext = S.drag_face_ring(x, sg["mass"], sg["faces"], rings, int(f), d)
        assert np.array_equal(ext, sg[f"drag_ext{k}"][j]), j
        assert np.float32(S.ext_energy(x, ext, rings[f])) == sg[f"drag_energy{k}"][j], j


def test_surface_extraction_matches_face_files(sg):
    """Boundary triangles extracted from the tets equal the shipped .face file's,
    with tetgen's orientation (each up to a cyclic rotation)."""
    got = M.surface_faces(sg["rest"], sg["tets"])
    canon = lambda q: min((q[i], q[(i + 1) % 3], q[(i + 2) % 3]) for i in range(3))
    assert sorted(map(canon, map(tuple, got.tolist()))) == sorted(map(canon, map(tuple, sg["faces"].tolist())))


def test_surface_extraction_of_a_box():
    """A 4 x 5 x 6 cube box: 2 (20 + 30 + 24) squares, two triangles each, all
    with outward picking normals (x2 - x0) x (x1 - x0)."""
    m = M.box_mesh(4, 5, 6)
    f = M.surface_faces(m.rest, m.tets)
    assert f.shape == (296, 3)
    n, c = S.normals_centers(m.rest, f)
    assert (np.einsum("ij,ij->i", n, c - m.rest.mean(0)) > 0).all()
