"""CPU restatement of the reference's surface picking and drag forces.

TEST INFRASTRUCTURE ONLY: the checker for the library's pbs_set_surface /
pbs_pick_face / pbs_drag_face_ring, pinned to the reference's own outputs
(tests/golden/surface_*.npz, made by tests/golden/make_golden.py from the
reference's TetMesh compiled headless).  Nothing in the product imports it.

Every float operation is FP32 in the reference's order, so results match bit
for bit.  Eigen 3.2 sums the three terms of dot() and squaredNorm() as
x0 + (x1 + x2) when the size is fixed at compile time (its unrolled halving
reduction: Vector3f operands) and as (x0 + x1) + x2 when it is not (columns
of a MatrixXf on both sides).

* face_rings         TetMesh::computeBoundfaceRingIndices  TetMesh.cpp:229-277
* normals_centers    TetMesh::computeBoundfaceNormals      TetMesh.cpp:378-393
* pick_face          TetMesh::pickFacebyRay                TetMesh.cpp:395-418
* drag_face_ring     TetMesh::dragFaceRing                 TetMesh.cpp:443-470
* ext_energy         TetMesh::computeExternalForcesEnergy  TetMesh.cpp:595-614
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def face_rings(faces, n_nodes: int):
    """Per face: its three nodes, then every other node sharing a surface edge
    with one of them, ascending (std::set order)."""
    faces = np.asarray(faces, np.int64).reshape(-1, 3)
    nbr = [set() for _ in range(n_nodes)]
    for a, b, c in faces:
        nbr[a].update((b, c))
        nbr[b].update((a, c))
        nbr[c].update((a, b))
    rings = []
    for a, b, c in faces:
        rest = (nbr[a] | nbr[b] | nbr[c]) - {a, b, c}
        rings.append(np.array([a, b, c] + sorted(rest), np.int64))
    return rings


def _dot(u, v):
    """Row-wise u0 v0 + (u1 v1 + u2 v2) in FP32: a fixed-size Eigen dot."""
    return u[..., 0] * v[..., 0] + (u[..., 1] * v[..., 1] + u[..., 2] * v[..., 2])


def _dot_dyn(u, v):
    """Row-wise (u0 v0 + u1 v1) + u2 v2 in FP32: a dot of MatrixXf columns."""
    return (u[..., 0] * v[..., 0] + u[..., 1] * v[..., 1]) + u[..., 2] * v[..., 2]


def _norm(u):
    return np.sqrt(_dot(u, u))


def normals_centers(x, faces):
    """normal = ((x2 - x0) x (x1 - x0)) / |.|, centre = ((x0 + x1) + x2) / 3."""
    x = np.asarray(x, f32).reshape(-1, 3)
    faces = np.asarray(faces, np.int64).reshape(-1, 3)
    x0, x1, x2 = x[faces[:, 0]], x[faces[:, 1]], x[faces[:, 2]]
    v1, v2 = x1 - x0, x2 - x0
    n = np.stack([v2[:, 1] * v1[:, 2] - v2[:, 2] * v1[:, 1],
                  v2[:, 2] * v1[:, 0] - v2[:, 0] * v1[:, 2],
                  v2[:, 0] * v1[:, 1] - v2[:, 1] * v1[:, 0]], axis=1).astype(f32)
    with np.errstate(invalid="ignore", divide="ignore"):
        n = (n / _norm(n)[:, None]).astype(f32)
    c = ((x0 + x1) + x2) / f32(3.0)
    return n, c.astype(f32)


def _first_edge(x, faces):
    """|x[f0.1] - x[f0.0]|: the reference's length scale for picking and drag."""
    e = x[faces[0, 1]] - x[faces[0, 0]]  # a difference of two MatrixXf columns
    return f32(np.sqrt(_dot_dyn(e, e)))


def pick_face(x, faces, orig, direction) -> int:
    """Among faces whose normal opposes the ray, the first one whose centre's
    squared distance from the ray is smallest and below the first face's first
    edge length squared; -1 if none."""
    x = np.asarray(x, f32).reshape(-1, 3)
    faces = np.asarray(faces, np.int64).reshape(-1, 3)
    orig = np.asarray(orig, f32)
    d = np.asarray(direction, f32)
    n, c = normals_centers(x, faces)
    r = _first_edge(x, faces)
    r2 = f32(r * r)
    ov = (orig[None, :] - c).astype(f32)
    a = _dot(ov, ov)
    b = _dot(ov, d[None, :])
    d2 = (a - b * b).astype(f32)
    with np.errstate(invalid="ignore"):
        cand = (_dot(n, d[None, :]) < f32(0)) & (d2 < r2) & (d2 < f32(1e8))
    if not cand.any():
        return -1
    idx = np.nonzero(cand)[0]
    return int(idx[np.argmin(d2[idx])])  # argmin returns the first of equal minima


def drag_force_scale(x, faces, drag, cap=800.0):
    """factor = min(|drag| / r * 100, cap) and the unit drag direction."""
    x = np.asarray(x, f32).reshape(-1, 3)
    drag = np.asarray(drag, f32)
    r = _first_edge(x, np.asarray(faces, np.int64).reshape(-1, 3))
    nd = f32(_norm(drag))
    factor = f32(f32(nd / r) * f32(100))
    if factor > f32(cap):
        factor = f32(cap)
    return factor, (drag / nd).astype(f32)


def drag_face_ring(x, mass, faces, rings, face: int, drag):
    """External forces (n, 3): factor m dir on the face's three nodes and
    (0.5 factor m) dir on the rest of its ring (0.5 * factor * m in FP64,
    rounded once to FP32, as the reference's double literal makes it)."""
    x = np.asarray(x, f32).reshape(-1, 3)
    mass = np.asarray(mass, f32)
    factor, dvec = drag_force_scale(x, faces, drag)
    ext = np.zeros_like(x)
    ring = rings[face]
    for j, node in enumerate(ring):
        s = f32(factor * mass[node]) if j < 3 else f32(0.5 * float(factor) * float(mass[node]))
        ext[node] = ext[node] + s * dvec
    return ext


def ext_energy(x, ext, ring) -> float:
    """-sum over the picked face's ring of x . f_ext, accumulated in FP32 in ring order."""
    x = np.asarray(x, f32).reshape(-1, 3)
    ext = np.asarray(ext, f32).reshape(-1, 3)
    e = f32(0)
    for node in ring:
        e = f32(e - f32(_dot_dyn(x[node], ext[node])))
    return float(e)
