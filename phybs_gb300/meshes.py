"""Procedural tet meshes and tetgen I/O for the descent time step.

Every generator returns a :class:`TetMeshData` whose arrays use the layouts the
reference passes across its GPU boundary (``CUDAInterface.h:23-25``):
positions are interleaved ``xyz`` float32 (Eigen ``3 x N`` column-major),
tets are 4 consecutive int32 node ids per tet, 0-based.

Tets are emitted positively oriented (``det[x1-x0, x2-x0, x3-x0] > 0``).  The
reference forms corner forces as ``P * AN`` with area-weighted normals taken
from cross products of rest edges (``TetMesh.cpp:279-294``); for a negatively
oriented tet that product has the wrong sign, so orientation is part of the
mesh contract.

Workloads (sizes as stated by the benchmark configurations):

* :func:`bar_mesh` - structured box, 6-tet (Kuhn) split, e.g. 40x10x10 cubes
  of edge 0.025 m (24,000 tets, 4,961 nodes), x = 0 face pinned.
* :func:`ellipsoid_mesh` - voxelised ellipsoid from a 20x20x40 cube grid,
  5-tet split with parity alternation, interior nodes jittered.
* :func:`box_mesh` - structured box, 5-tet split, e.g. 50x50x80 cubes
  (1,000,000 tets, 210,681 nodes) with interior jitter.
* :func:`batch_of_boxes` - many uneven 5-tet boxes packed into one mesh.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

__all__ = [
    "TetMeshData", "bar_mesh", "box_mesh", "ellipsoid_mesh", "batch_of_boxes", "load_tetgen_faces", "surface_faces",
    "load_tetgen", "write_tetgen_nodes", "orient_positive", "signed_volumes",
    "twist_positions", "incidence_csr",
]


@dataclasses.dataclass
class TetMeshData:
    """A tet mesh plus the per-node and per-tet inputs of one simulation.

    ``instance_node_ptr``/``instance_tet_ptr`` delimit packed independent
    instances (a single mesh has one instance).  ``young``/``poisson`` are per
    tet.  ``pins`` are sorted node ids held fixed within a step.
    """

    rest: np.ndarray                  # (N, 3) float32
    tets: np.ndarray                  # (T, 4) int32
    pins: np.ndarray                  # (P,) int32, sorted
    young: np.ndarray                 # (T,) float32
    poisson: np.ndarray               # (T,) float32
    density: float = 1000.0
    instance_node_ptr: np.ndarray | None = None
    instance_tet_ptr: np.ndarray | None = None
    name: str = "mesh"

    def __post_init__(self):
        self.rest = np.ascontiguousarray(self.rest, dtype=np.float32).reshape(-1, 3)
        self.tets = np.ascontiguousarray(self.tets, dtype=np.int32).reshape(-1, 4)
        self.pins = np.ascontiguousarray(np.unique(np.asarray(self.pins, dtype=np.int64)), dtype=np.int32)
        t = self.tets.shape[0]
        self.young = np.ascontiguousarray(np.broadcast_to(np.asarray(self.young, np.float32), (t,)))
        self.poisson = np.ascontiguousarray(np.broadcast_to(np.asarray(self.poisson, np.float32), (t,)))
        if self.instance_node_ptr is None:
            self.instance_node_ptr = np.array([0, self.rest.shape[0]], np.int32)
        if self.instance_tet_ptr is None:
            self.instance_tet_ptr = np.array([0, t], np.int32)
        self.instance_node_ptr = np.ascontiguousarray(self.instance_node_ptr, np.int32)
        self.instance_tet_ptr = np.ascontiguousarray(self.instance_tet_ptr, np.int32)

    @property
    def n_nodes(self) -> int:
        return int(self.rest.shape[0])

    @property
    def n_tets(self) -> int:
        return int(self.tets.shape[0])

    @property
    def n_instances(self) -> int:
        return int(self.instance_node_ptr.shape[0] - 1)

    def pin_mask(self) -> np.ndarray:
        m = np.zeros(self.n_nodes, np.int32)
        m[self.pins] = 1
        return m

    def bbox_diagonal(self) -> float:
        return float(np.linalg.norm(self.rest.max(0).astype(np.float64) - self.rest.min(0)))


# ----------------------------------------------------------------------------
# geometry helpers

def signed_volumes(pos: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """det[x1-x0, x2-x0, x3-x0] / 6 per tet, in float64."""
    p = np.asarray(pos, np.float64).reshape(-1, 3)
    t = np.asarray(tets).reshape(-1, 4)
    e1 = p[t[:, 1]] - p[t[:, 0]]
    e2 = p[t[:, 2]] - p[t[:, 0]]
    e3 = p[t[:, 3]] - p[t[:, 0]]
    return np.einsum("ij,ij->i", e1, np.cross(e2, e3)) / 6.0


def orient_positive(pos: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """Swap corners 2 and 3 of every negatively oriented tet."""
    t = np.array(tets, np.int32, copy=True).reshape(-1, 4)
    neg = signed_volumes(pos, t) < 0
    t[neg, 2], t[neg, 3] = t[neg, 3].copy(), t[neg, 2].copy()
    return t


def _grid_nodes(nx: int, ny: int, nz: int, h: float) -> np.ndarray:
    # x fastest: node(i, j, k) = i + (nx+1) * (j + (ny+1) * k)
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    return np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64) * h


def _cube_corner_ids(nx: int, ny: int, cells: np.ndarray) -> np.ndarray:
    """(C, 8) node ids of each cell's corners; corner bit 0 = +x, 1 = +y, 2 = +z."""
    sx, sy = 1, nx + 1
    sz = (nx + 1) * (ny + 1)
    base = cells[:, 0] * sx + cells[:, 1] * sy + cells[:, 2] * sz
    off = np.array([((b & 1) * sx + ((b >> 1) & 1) * sy + ((b >> 2) & 1) * sz) for b in range(8)])
    return base[:, None] + off[None, :]


# Kuhn split: 6 tets around the 0 -> 7 diagonal, one per axis permutation.
_KUHN = np.array([[0, 1, 3, 7], [0, 1, 5, 7], [0, 2, 3, 7], [0, 2, 6, 7], [0, 4, 5, 7], [0, 4, 6, 7]])
# 5-tet split.  Parity 0: central tet on the even corners {000,110,101,011},
# one corner tet per odd corner.  Parity 1 mirrors it.  Alternating the parity
# with (i+j+k) makes shared face diagonals agree, so the mesh is conforming.
_FIVE = {
    0: np.array([[0, 3, 5, 6], [1, 0, 3, 5], [2, 0, 3, 6], [4, 0, 5, 6], [7, 3, 5, 6]]),
    1: np.array([[1, 2, 4, 7], [0, 1, 2, 4], [3, 1, 2, 7], [5, 1, 4, 7], [6, 2, 4, 7]]),
}


def _split_cells(nx: int, ny: int, cells: np.ndarray, split: int) -> np.ndarray:
    cid = _cube_corner_ids(nx, ny, cells)
    if split == 6:
        return cid[:, _KUHN].reshape(-1, 4)
    if split != 5:
        raise ValueError("split must be 5 or 6")
    par = (cells.sum(axis=1) & 1)
    out = np.empty((cells.shape[0], 5, 4), np.int64)
    for p in (0, 1):
        sel = par == p
        out[sel] = cid[sel][:, _FIVE[p]]
    return out.reshape(-1, 4)


def _compact(pos: np.ndarray, tets: np.ndarray):
    used = np.zeros(pos.shape[0], bool)
    used[tets.ravel()] = True
    remap = -np.ones(pos.shape[0], np.int64)
    remap[used] = np.arange(int(used.sum()))
    return pos[used], remap[tets], used


def _interior_mask(n_nodes: int, tets_cells_corners: np.ndarray, valence_full: int) -> np.ndarray:
    cnt = np.bincount(tets_cells_corners.ravel(), minlength=n_nodes)
    return cnt == valence_full


def _jitter(pos: np.ndarray, interior: np.ndarray, amp: float, h: float, seed: int) -> np.ndarray:
    if amp <= 0:
        return pos
    rng = np.random.default_rng(seed)
    d = rng.uniform(-amp, amp, size=pos.shape) * h
    out = pos.copy()
    out[interior] += d[interior]
    return out


# ----------------------------------------------------------------------------
# generators

def bar_mesh(nx: int = 40, ny: int = 10, nz: int = 10, edge: float = 0.025, young: float = 5e4,
             poisson: float = 0.4, pin_x0: bool = True, name: str = "bar") -> TetMeshData:
    """Structured box of nx*ny*nz cubes, 6-tet Kuhn split; x is the long axis.

    With the defaults: 24,000 tets, 4,961 nodes; the x = 0 face (121 nodes) is
    pinned.
    """
    pos = _grid_nodes(nx, ny, nz, edge)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cells = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)
    tets = orient_positive(pos, _split_cells(nx, ny, cells, 6))
    pins = np.nonzero(pos[:, 0] == 0.0)[0] if pin_x0 else np.zeros(0, np.int64)
    return TetMeshData(pos.astype(np.float32), tets, pins, young, poisson, name=name)


def box_mesh(nx: int = 50, ny: int = 50, nz: int = 80, edge: float = 0.005, jitter: float = 0.1,
             seed: int = 0, young: float = 1e5, poisson: float = 0.4, pin: str = "top",
             name: str = "box") -> TetMeshData:
    """Structured box, 5-tet split with parity alternation; z is the long axis.

    Defaults: 50x50x80 cubes of 0.005 m -> 1,000,000 tets and 210,681 nodes.
    Interior nodes are jittered uniformly by +-jitter*edge per axis.
    ``pin``: "top" pins z = max, "bottom" pins z = 0, "both" pins both ends
    (the bottom face is then driven by a prescribed motion), "none".
    """
    pos = _grid_nodes(nx, ny, nz, edge)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cells = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)
    tets = _split_cells(nx, ny, cells, 5)
    ii = np.rint(pos / edge).astype(np.int64)
    interior = ((ii[:, 0] > 0) & (ii[:, 0] < nx) & (ii[:, 1] > 0) & (ii[:, 1] < ny)
                & (ii[:, 2] > 0) & (ii[:, 2] < nz))
    pos = _jitter(pos, interior, jitter, edge, seed)
    tets = orient_positive(pos, tets)
    top = np.nonzero(ii[:, 2] == nz)[0]
    bot = np.nonzero(ii[:, 2] == 0)[0]
    pins = {"top": top, "bottom": bot, "both": np.concatenate([top, bot]),
            "none": np.zeros(0, np.int64)}[pin]
    return TetMeshData(pos.astype(np.float32), tets, pins, young, poisson, name=name)


def ellipsoid_mesh(gx: int = 20, gy: int = 20, gz: int = 40, cell: float = 0.01, jitter: float = 0.15,
                   seed: int = 2, young: float = 1e5, poisson: float = 0.45, pin_fraction: float = 0.05,
                   name: str = "ellipsoid") -> TetMeshData:
    """Voxelised ellipsoid from a gx*gy*gz cube grid, 5-tet split.

    Keeps cubes whose centres satisfy (x/(gx/2))^2 + (y/(gy/2))^2 +
    (z/(gz/2))^2 <= 1 in cell units about the grid centre.  Interior nodes
    (all 8 surrounding cubes kept) are jittered by +-jitter*cell; surface nodes
    are not.  The lowest ``pin_fraction`` of nodes by z are pinned.
    """
    k, j, i = np.meshgrid(np.arange(gz), np.arange(gy), np.arange(gx), indexing="ij")
    cells = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)
    c = cells + 0.5 - np.array([gx / 2, gy / 2, gz / 2])
    keep = (c[:, 0] / (gx / 2)) ** 2 + (c[:, 1] / (gy / 2)) ** 2 + (c[:, 2] / (gz / 2)) ** 2 <= 1.0
    cells = cells[keep]
    pos = _grid_nodes(gx, gy, gz, cell)
    corner_ids = _cube_corner_ids(gx, gy, cells)
    interior_full = np.bincount(corner_ids.ravel(), minlength=pos.shape[0]) == 8
    tets = _split_cells(gx, gy, cells, 5)
    pos, tets, used = _compact(pos, tets)
    interior = interior_full[used]
    pos = _jitter(pos, interior, jitter, cell, seed)
    tets = orient_positive(pos, tets)
    n_pin = max(1, int(round(pin_fraction * pos.shape[0])))
    order = np.lexsort((np.arange(pos.shape[0]), pos[:, 2]))
    pins = np.sort(order[:n_pin])
    return TetMeshData(pos.astype(np.float32), tets, pins, young, poisson, name=name)


def batch_of_boxes(n_instances: int = 256, seed: int = 0, edge: float = 0.01, spacing: float = 0.5,
                   nxy=(4, 16), nz=(8, 32), young=(1e4, 1e6), poisson=(0.3, 0.45),
                   name: str = "batch") -> TetMeshData:
    """Independent 5-tet boxes packed into one mesh (disjoint node/tet ranges).

    Per instance: nx, ny ~ U{nxy}, nz ~ U{nz}; E log-uniform in ``young``;
    Poisson uniform in ``poisson``; its z = 0 end pinned.  Instances are laid
    out on a line ``spacing`` metres apart so they never touch.
    """
    rng = np.random.default_rng(seed)
    rests, tetss, pinss, ys, ps = [], [], [], [], []
    node_ptr, tet_ptr = [0], [0]
    for b in range(n_instances):
        bx = int(rng.integers(nxy[0], nxy[1] + 1))
        by = int(rng.integers(nxy[0], nxy[1] + 1))
        bz = int(rng.integers(nz[0], nz[1] + 1))
        e = float(10.0 ** rng.uniform(np.log10(young[0]), np.log10(young[1])))
        nu = float(rng.uniform(poisson[0], poisson[1]))
        m = box_mesh(bx, by, bz, edge=edge, jitter=0.0, young=e, poisson=nu, pin="bottom")
        off = node_ptr[-1]
        r = m.rest.astype(np.float64)
        r[:, 0] += b * spacing
        rests.append(r)
        tetss.append(m.tets.astype(np.int64) + off)
        pinss.append(m.pins.astype(np.int64) + off)
        ys.append(np.full(m.n_tets, e, np.float32))
        ps.append(np.full(m.n_tets, nu, np.float32))
        node_ptr.append(off + m.n_nodes)
        tet_ptr.append(tet_ptr[-1] + m.n_tets)
    return TetMeshData(np.concatenate(rests).astype(np.float32), np.concatenate(tetss),
                       np.concatenate(pinss), np.concatenate(ys), np.concatenate(ps),
                       instance_node_ptr=np.array(node_ptr, np.int32),
                       instance_tet_ptr=np.array(tet_ptr, np.int32), name=name)


def twist_positions(rest: np.ndarray, angle: float, axis: int = 2, profile: str = "linear") -> np.ndarray:
    """Rotate each node about the long axis through the mesh centre by an angle
    growing linearly from 0 at the lowest coordinate to ``angle`` at the top
    (``profile="sine"``: angle * sin(pi s), s in [0, 1] along the axis, zero at
    both ends, for meshes pinned at both ends)."""
    p = np.asarray(rest, np.float64).reshape(-1, 3)
    a, b = [d for d in range(3) if d != axis]
    c = 0.5 * (p.min(0) + p.max(0))
    z = p[:, axis]
    s = (z - z.min()) / max(z.max() - z.min(), 1e-30)
    t = (np.sin(np.pi * s) if profile == "sine" else s) * angle
    x, y = p[:, a] - c[a], p[:, b] - c[b]
    out = p.copy()
    out[:, a] = c[a] + np.cos(t) * x - np.sin(t) * y
    out[:, b] = c[b] + np.sin(t) * x + np.cos(t) * y
    return out.astype(np.float32)


# ----------------------------------------------------------------------------
# node -> (tet, corner) incidence

def incidence_csr(tets: np.ndarray, n_nodes: int):
    """Node -> incident (tet, corner) lists in canonical order.

    Canonical order: per node ascending tet id, then ascending corner.  Entry
    value = ``4 * tet + corner``.  Returns ``(row_ptr[N+1], entries[4T])`` as
    int32.  This is the gather order the device uses, so per-node force sums
    are reproducible bit for bit.
    """
    t = np.asarray(tets, np.int64).reshape(-1, 4)
    node = t.ravel()
    slot = np.arange(node.size, dtype=np.int64)       # = 4*tet + corner, already ascending
    order = np.argsort(node, kind="stable")
    counts = np.bincount(node, minlength=n_nodes)
    row = np.zeros(n_nodes + 1, np.int64)
    np.cumsum(counts, out=row[1:])
    return row.astype(np.int32), slot[order].astype(np.int32)


# ----------------------------------------------------------------------------
# tetgen I/O (TetMesh.cpp:14-151 reads the same text formats)

def _read_table(path: str):
    with open(path) as f:
        lines = [ln.split("#", 1)[0].split() for ln in f]
    lines = [ln for ln in lines if ln]
    return lines[0], lines[1:]


def load_tetgen(stem: str, scale: float = 1.0, young: float = 5e5, poisson: float = 0.45,
                pins=None, orient: bool = True) -> TetMeshData:
    """Load ``<stem>.node`` and ``<stem>.ele`` (tetgen text).

    Coordinates are formed as TetMesh::initNodesFromFile forms them
    (TetMesh.cpp:36-37): each decimal read into an FP32 float, then the column
    multiplied by the scale rounded to FP32, in FP32; with ``scale`` = 0.1 the
    positions equal the reference loader's bit for bit.  Index base follows
    the files (the reference meshes are 0-based).  Unlike the reference
    loader, no scaling or pin rule is hard-coded: ``scale`` and ``pins`` are
    arguments.  ``orient``: swap corners 2 and 3 of every negatively oriented
    tet (the device path wants positive orientation); False keeps the file's
    corner order, as the reference loader does (TetMesh.cpp:93-114).
    """
    head, rows = _read_table(stem + ".node")
    n = int(head[0])
    ids = np.array([int(r[0]) for r in rows[:n]], np.int64)
    pos = np.array([[float(r[1]), float(r[2]), float(r[3])] for r in rows[:n]], np.float64).astype(np.float32)
    if scale != 1.0:
        pos = (pos * np.float32(scale)).astype(np.float32)
    base = int(ids.min()) if n else 0
    head, rows = _read_table(stem + ".ele")
    t = int(head[0])
    tets = np.array([[int(r[1]), int(r[2]), int(r[3]), int(r[4])] for r in rows[:t]], np.int64) - base
    tets = orient_positive(pos, tets) if orient else tets.astype(np.int32)
    return TetMeshData(pos, tets, np.zeros(0, np.int32) if pins is None else pins,
                       young, poisson, name=os.path.basename(stem))


def load_tetgen_faces(stem: str) -> np.ndarray:
    """Boundary triangles of ``<stem>.face`` (tetgen text) as (F, 3) node ids,
    in the index base of ``<stem>.node`` (the file TetMesh.cpp:130-151 reads)."""
    head, rows = _read_table(stem + ".node")
    base = min(int(r[0]) for r in rows[:int(head[0])]) if int(head[0]) else 0
    head, rows = _read_table(stem + ".face")
    f = int(head[0])
    return (np.array([[int(r[1]), int(r[2]), int(r[3])] for r in rows[:f]], np.int64) - base).astype(np.int32)


def surface_faces(pos: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """Boundary triangles of a tet mesh (faces that belong to one tet), in
    tetgen's orientation: (x1 - x0) x (x2 - x0) points into the mesh, so the
    picking normal (x2 - x0) x (x1 - x0) points out.  Ordered by tet, then by
    the corner each face is opposite to."""
    p = np.asarray(pos, np.float64).reshape(-1, 3)
    t = np.asarray(tets, np.int64).reshape(-1, 4)
    tri = np.concatenate([t[:, [1, 2, 3]], t[:, [0, 2, 3]], t[:, [0, 1, 3]], t[:, [0, 1, 2]]], axis=0)
    opp = np.concatenate([t[:, 0], t[:, 1], t[:, 2], t[:, 3]])
    order = np.concatenate([np.arange(t.shape[0]) * 4 + k for k in range(4)])
    key = np.sort(tri, axis=1)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    inv = inv.reshape(-1)
    keep = cnt[inv] == 1
    tri, opp, order = tri[keep], opp[keep], order[keep]
    tri = tri[np.argsort(order, kind="stable")]
    opp = opp[np.argsort(order, kind="stable")]
    n = np.cross(p[tri[:, 1]] - p[tri[:, 0]], p[tri[:, 2]] - p[tri[:, 0]])
    flip = np.einsum("ij,ij->i", n, p[opp] - p[tri[:, 0]]) < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    return tri.astype(np.int32)


def write_tetgen_nodes(path: str, pos: np.ndarray) -> None:
    """Write positions as a tetgen ``.node`` file (the format TetMesh.cpp:558 exports)."""
    p = np.asarray(pos, np.float32).reshape(-1, 3)
    with open(path, "w") as f:
        f.write(f"{p.shape[0]} 3 0 0\n")
        for i, (x, y, z) in enumerate(p):
            f.write(f"{i} {x:.9g} {y:.9g} {z:.9g}\n")


def pbd_levels(tets: np.ndarray, n_nodes: int) -> int:
    """Number of dependency levels of a Gauss-Seidel sweep over the tets in
    their order (a tet's level is one more than the highest level of the
    earlier tets sharing a node with it): the length of the chain the
    strain-based PBD step runs level by level."""
    last = np.full(n_nodes, -1, np.int64)
    top = -1
    for q in np.asarray(tets, np.int64).reshape(-1, 4):
        lv = max(last[q[0]], last[q[1]], last[q[2]], last[q[3]]) + 1
        last[q] = lv
        top = max(top, lv)
    return int(top + 1)
