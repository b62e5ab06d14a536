"""Generate tests/golden/*.npz from the reference's own CPU solver.

Run where the reference tree exists (it is compiled headless into
oracle/_ref by oracle/ref_build/Makefile):

    python tests/golden/make_golden.py

Each fixture freezes, for one mesh, the reference's outputs: the rest state it
loaded (TetMesh.cpp:186-216), forces / energies / Hessian diagonal at a
deformed probe state (IsotropicNeohookeanMaterial.cpp:93-131,
IsotropicMaterial.cpp:360-409, 503-682), the stiffness CSR pattern
(IsotropicMaterial.cpp:554-644) for small meshes, and the node positions and
velocities after successive DescentOptimize::doDescentOpt steps
(DescentOptimize.cpp:91-188); and, in separate fixtures, the surface
picking / drag, element stiffness and PBD / projective-dynamics outputs.
Meshes are the procedural workloads of the
benchmark configurations, at fixture-friendly sizes, plus two of the
reference's own tetgen meshes.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

if not os.environ.get("PHYBS_REFERENCE") and os.path.isdir("/root/reference/FVM"):
    os.environ["PHYBS_REFERENCE"] = "/root/reference"
import oracle  # noqa: E402
from oracle import ref as REF  # noqa: E402

REFERENCE_TREE = oracle.reference_tree()
if REFERENCE_TREE is None:
    raise SystemExit("make_golden.py reads the reference checkout: set PHYBS_REFERENCE")
from phybs_gb300 import meshes as M  # noqa: E402


def reference_mesh(name, stem, pin_axis, pin_side, young=5e5, poisson=0.45):
    m = M.load_tetgen(os.path.join(REFERENCE_TREE, "model", stem), scale=0.1, young=young, poisson=poisson)
    c = m.rest[:, pin_axis].astype(np.float64)
    sel = c <= c.min() + 0.05 * (c.max() - c.min()) if pin_side == "min" else c >= c.max() - 0.05 * (c.max() - c.min())
    return M.TetMeshData(m.rest, m.tets, np.nonzero(sel)[0], young, poisson, name=name)


def cases():
    return {
        "bar_small": dict(mesh=M.bar_mesh(8, 4, 4, edge=0.025, young=5e4, poisson=0.4), h=1 / 30, iters=96,
                          steps=5, init_twist=0.0, probe_twist=np.pi / 4, csr=True),
        "bar_config1": dict(mesh=M.bar_mesh(40, 10, 10, edge=0.025, young=5e4, poisson=0.4), h=1 / 30, iters=96,
                            steps=3, init_twist=0.0, probe_twist=np.pi / 6, csr=False),
        "ellipsoid_small": dict(mesh=M.ellipsoid_mesh(8, 8, 16, cell=0.01, jitter=0.15, seed=2, young=1e5,
                                                      poisson=0.45), h=1 / 60, iters=64, steps=3,
                                init_twist=np.pi / 2, probe_twist=np.pi / 2, csr=True),
        "model_bar": dict(mesh=reference_mesh("model_bar", "bar/bar.1", 0, "min"), h=0.03, iters=96, steps=3,
                          init_twist=0.0, probe_twist=np.pi / 4, csr=True),
        "model_dragon": dict(mesh=reference_mesh("model_dragon", "asiandragon/asiandragon.1", 1, "min"), h=0.03,
                             iters=96, steps=2, init_twist=0.0, probe_twist=np.pi / 8, csr=True),
    }


def twist_axis(rest):
    ext = rest.max(0) - rest.min(0)
    return int(np.argmax(ext))


def make(name, cfg, rng):
    m = cfg["mesh"]
    sim = REF.RefSim(m.rest, m.tets, m.pins, float(m.young[0]), float(m.poisson[0]), density=m.density)
    sim.set_h(cfg["h"])
    rest = sim.rest()
    mu, lam = sim.lame()
    out = dict(rest=rest, tets=m.tets, pins=m.pins, mu=mu, lam=lam, h=np.float32(cfg["h"]),
               iters=np.int32(cfg["iters"]), young=np.float32(m.young[0]), poisson=np.float32(m.poisson[0]),
               dminv=sim.dminv(), an=sim.an(), vol=sim.vol(), mass=sim.mass(), gravity=sim.gravity())
    ax = twist_axis(rest)
    xp = M.twist_positions(rest, cfg["probe_twist"], axis=ax)
    e = rest[m.tets[:, 1]] - rest[m.tets[:, 0]]
    edge = float(np.median(np.linalg.norm(e, axis=1)))
    xp = (xp + rng.normal(0.0, 0.02 * edge, xp.shape)).astype(np.float32)
    assert (M.signed_volumes(xp, m.tets) > 0).all(), "probe state must not invert tets"
    out.update(probe_x=xp, probe_force_nh=sim.force_nh(xp), probe_force_stretch=sim.force_stretch(xp),
               probe_energy=sim.elastic_energy(xp), probe_hdiag=sim.hessian_diag(xp),
               probe_k0=sim.element_stiffness(0, xp), probe_total_energy=np.float32(sim.total_energy(xp, rest)),
               rest_hdiag=sim.hessian_diag(rest))
    if cfg["csr"]:
        row, col, diag, kid = sim.csr()
        out.update(csr_row=row, csr_col=col, csr_diag=diag, csr_kid=kid)
    x0 = rest.copy()
    if cfg["init_twist"]:
        x0 = M.twist_positions(rest, cfg["init_twist"], axis=ax)
        x0[m.pins] = rest[m.pins]
        sim.set_nodes(x0)
    out["traj_x0"] = x0
    xs, vs, sc = [], [], []
    for _ in range(cfg["steps"]):
        sim.step(cfg["iters"])
        xs.append(sim.nodes())
        vs.append(sim.vel())
        s = sim.scalars()
        sc.append([s["alpha"], s["energy"], s["energy_old"], s["rho"], s["omega"]])
    out.update(traj_x=np.stack(xs), traj_v=np.stack(vs), traj_scalars=np.array(sc, np.float32))
    sim.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, m.n_nodes, m.n_tets, len(m.pins), os.path.getsize(os.path.join(HERE, name + ".npz")))


def surface_cases():
    """The reference's shipped meshes with their own .face files."""
    return {"surface_model_bar": ("model_bar", "bar/bar.1", 0, "min"),
            "surface_model_dragon": ("model_dragon", "asiandragon/asiandragon.1", 1, "min")}


def make_surface(name, spec, rng, n_rays=24, n_drags=12):
    """Face rings, picks, normals / centres, drag forces and drag energies
    from TetMesh (TetMesh.cpp:229-277, 378-418, 446-470, 595-614) at the rest
    shape and at a perturbed shape."""
    mesh_name, stem, axis, side = spec
    m = reference_mesh(mesh_name, stem, axis, side)
    faces = M.load_tetgen_faces(os.path.join(REFERENCE_TREE, "model", stem))
    sim = REF.RefSim(m.rest, m.tets, m.pins, float(m.young[0]), float(m.poisson[0]), density=m.density, faces=faces)
    rest = sim.rest()
    rings = [sim.face_ring(f) for f in range(faces.shape[0])]
    out = dict(rest=rest, tets=m.tets, pins=m.pins, faces=faces, mass=sim.mass(),
               ring_ptr=np.cumsum([0] + [len(r) for r in rings]).astype(np.int32),
               ring=np.concatenate(rings).astype(np.int32))
    edge = float(np.median(np.linalg.norm(rest[m.tets[:, 1]] - rest[m.tets[:, 0]], axis=1)))
    states = [rest, (rest + rng.normal(0.0, 0.3 * edge, rest.shape)).astype(np.float32)]
    states[1][m.pins] = rest[m.pins]
    for k, x in enumerate(states):
        sim.set_nodes(x)
        orig = np.zeros((n_rays, 3), np.float32)
        dirs = np.zeros((n_rays, 3), np.float32)
        picks = np.zeros(n_rays, np.int32)
        extent = float(np.linalg.norm(x.max(0) - x.min(0)))
        for j in range(n_rays):
            d = rng.normal(size=3)
            d = (d / np.linalg.norm(d)).astype(np.float32)
            dirs[j] = d
            if j < n_rays - 4:  # aimed at a node
                target = x[rng.integers(len(x))]
                orig[j] = (target - 3.0 * edge * d + rng.normal(0.0, 0.2 * edge, 3)).astype(np.float32)
            else:  # a line far off the mesh: no face is picked
                side = np.cross(d, [0.0, 0.0, 1.0] if abs(d[2]) < 0.9 else [1.0, 0.0, 0.0])
                orig[j] = (x.mean(0) + 5.0 * extent * side / np.linalg.norm(side)).astype(np.float32)
            picks[j], normals, centers = sim.pick_face(orig[j], dirs[j])
        drag_face = np.array([p if p >= 0 else rng.integers(len(faces)) for p in picks[:n_drags]], np.int32)
        drags = rng.normal(0.0, 10.0 * edge, (n_drags, 3)).astype(np.float32)
        ext = np.zeros((n_drags, len(x), 3), np.float32)
        energy = np.zeros(n_drags, np.float32)
        for j in range(n_drags):
            sim.drag_face_ring(int(drag_face[j]), drags[j])
            ext[j] = sim.ext()
            energy[j] = sim.ext_energy(x)
        out.update({f"x{k}": x, f"ray_orig{k}": orig, f"ray_dir{k}": dirs, f"pick{k}": picks,
                    f"normals{k}": normals, f"centers{k}": centers, f"drag_face{k}": drag_face,
                    f"drag{k}": drags, f"drag_ext{k}": ext, f"drag_energy{k}": energy})
    sim.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, len(rest), len(faces), os.path.getsize(os.path.join(HERE, name + ".npz")))


def make_stiffness(name, cfg, rng, n_sample=64):
    """Element stiffness matrices K = -df/dx of a sample of tets
    (IsotropicMaterial::computeStiffnessMatrixFromPos, IsotropicMaterial.cpp:503-552:
    Xu et al.'s SVD-derivative dP/dF), at a twisted and jittered state, with the
    reference's rest data; the checker of the backward-Euler step's matrix."""
    m = cfg["mesh"]
    sim = REF.RefSim(m.rest, m.tets, m.pins, float(m.young[0]), float(m.poisson[0]), density=m.density)
    rest = sim.rest()
    mu, lam = sim.lame()
    edge = float(np.median(np.linalg.norm(rest[m.tets[:, 1]] - rest[m.tets[:, 0]], axis=1)))
    x = M.twist_positions(rest, cfg["probe_twist"], axis=twist_axis(rest))
    x = (x + rng.normal(0.0, 0.05 * edge, x.shape)).astype(np.float32)
    assert (M.signed_volumes(x, m.tets) > 0).all()
    sample = np.sort(rng.choice(m.tets.shape[0], size=min(n_sample, m.tets.shape[0]), replace=False)).astype(np.int32)
    K = np.stack([sim.element_stiffness(int(t), x) for t in sample])
    out = dict(rest=rest, tets=m.tets, pins=m.pins, mu=mu, lam=lam, dminv=sim.dminv(), vol=sim.vol(),
               mass=sim.mass(), gravity=sim.gravity(), x=x, sample=sample, K=K)
    sim.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, len(sample), os.path.getsize(os.path.join(HERE, name + ".npz")))


def inverted_positions(rest, tets, pins, rng, n_nodes=3):
    """Rest positions with a few interior free nodes moved 2 edge lengths in
    random directions: the incident tets on that side invert (det F < 0)."""
    x = rest.astype(np.float64).copy()
    edge = float(np.median(np.linalg.norm(rest[tets[:, 1]] - rest[tets[:, 0]], axis=1)))
    pinned = set(int(p) for p in pins)
    counts = np.bincount(tets.reshape(-1), minlength=len(rest))
    cand = [i for i in np.argsort(-counts) if int(i) not in pinned][: 4 * n_nodes]
    for i in rng.choice(cand, size=n_nodes, replace=False):
        d = rng.normal(size=3)
        x[i] += 2.0 * edge * d / np.linalg.norm(d)
    return x.astype(np.float32)


def make_dynamics(name, cfg, rng, pbd_steps=3, pd_steps=2, dt=0.03):
    """The reference's strain-based PBD (PosBaseDynamic.cpp:12-117) and
    projective dynamics (ProjDynamic.cpp:48-100, 351-480, with Eigen's
    SimplicialLDLT standing in for MKL Pardiso) trajectories from a twisted
    state, the first step with external forces on a few nodes, plus one
    projective step from a state with inverted tets; with the reference's rest
    data (Dm^-1 row-major, inverse masses, volumes)."""
    m = cfg["mesh"]
    sim = REF.RefSim(m.rest, m.tets, m.pins, float(m.young[0]), float(m.poisson[0]), density=m.density)
    rest = sim.rest()
    edge = float(np.median(np.linalg.norm(rest[m.tets[:, 1]] - rest[m.tets[:, 0]], axis=1)))
    x0 = M.twist_positions(rest, cfg["probe_twist"] / 2, axis=twist_axis(rest))
    x0 = (x0 + rng.normal(0.0, 0.02 * edge, x0.shape)).astype(np.float32)
    x0[m.pins] = rest[m.pins]
    free = np.setdiff1d(np.arange(len(rest)), m.pins)
    ext = np.zeros_like(rest)
    pull = rng.choice(free, size=min(6, len(free)), replace=False)
    ext[pull] = rng.normal(0.0, 0.05, (len(pull), 3)).astype(np.float32)
    out = dict(rest=rest, tets=m.tets, pins=m.pins, dminv=sim.dminv(), inv_mass=sim.inv_mass(), mass=sim.mass(),
               vol=sim.vol(), gravity=sim.gravity(), x0=x0, ext=ext, dt=np.float32(dt))
    zero = np.zeros_like(rest)
    for kind, steps in (("pbd", pbd_steps), ("pd", pd_steps)):
        sim.set_nodes(x0)
        sim.set_vel(zero)
        for k in range(steps):
            sim.set_ext(ext if k == 0 else zero)
            if kind == "pbd":
                sim.pbd_step(dt)
            else:
                sim.pd_step(dt)
            out[f"x_{kind}{k}"], out[f"v_{kind}{k}"] = sim.nodes(), sim.vel()
    xi = inverted_positions(rest, m.tets, m.pins, rng)
    assert (M.signed_volumes(xi, m.tets) < 0).any()
    sim.set_nodes(xi)
    sim.set_vel(zero)
    sim.set_ext(zero)
    sim.pd_step(dt)
    out.update(x_inv=xi, x_pd_inv=sim.nodes(), v_pd_inv=sim.vel())
    sim.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, len(rest), len(m.tets), os.path.getsize(os.path.join(HERE, name + ".npz")))


def compressed_probe(rest, edge, rng):
    """A state with near-inverted tets: the bar's y extent is scaled by
    c(s) = 10^(-5 (s - 1/4) / (3/4)) beyond a quarter of its length s (1 down
    to 1e-5), x and z jittered by 1% of the edge, then the bar turned 30
    degrees about y (so F is not diagonal).  det F spans 1 .. ~1e-5, no tet
    inverts."""
    x = np.asarray(rest, np.float64).copy()
    s = (x[:, 0] - x[:, 0].min()) / (x[:, 0].max() - x[:, 0].min())
    c = 10.0 ** np.where(s < 0.25, 0.0, -5.0 * (s - 0.25) / 0.75)
    x[:, 1] = x[:, 1] * c
    x[:, 0] += rng.normal(0.0, 0.01 * edge, x.shape[0])
    x[:, 2] += rng.normal(0.0, 0.01 * edge, x.shape[0])
    th = np.deg2rad(30.0)
    x0, z0 = x[:, 0].copy(), x[:, 2].copy()
    x[:, 0] = np.cos(th) * x0 - np.sin(th) * z0
    x[:, 2] = np.sin(th) * x0 + np.cos(th) * z0
    return x.astype(np.float32)


def make_inverted(name="probe_inverted_bar"):
    """probe_inverted_bar.npz: the reference's node forces (both materials;
    the stretch-based one through its modified SVD, IsotropicMaterial.cpp:16-60)
    at a state whose tets have det F from 1 down to ~1e-5
    (compressed_probe), for the near-inversion parity test
    (tests/test_gpu_inverted.py)."""
    m = M.bar_mesh(8, 4, 4, edge=0.025, young=5e4, poisson=0.4)
    sim = REF.RefSim(m.rest, m.tets, m.pins, float(m.young[0]), float(m.poisson[0]), density=m.density)
    rest = sim.rest()
    mu, lam = sim.lame()
    x = compressed_probe(rest, 0.025, np.random.default_rng(20261207))
    J = M.signed_volumes(x, m.tets) / M.signed_volumes(rest, m.tets)
    assert (J > 0).all() and ((J > 1e-5) & (J < 1e-3)).sum() >= 100
    out = dict(rest=rest, tets=m.tets, pins=m.pins, mu=mu, lam=lam, young=np.float32(m.young[0]),
               poisson=np.float32(m.poisson[0]), dminv=sim.dminv(), an=sim.an(), vol=sim.vol(), mass=sim.mass(),
               gravity=sim.gravity(), probe_x=x, probe_force_nh=sim.force_nh(x),
               probe_force_stretch=sim.force_stretch(x))
    sim.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, m.n_nodes, m.n_tets, int((J < 1e-3).sum()), "tets below det F 1e-3")


def make_reference_lines():
    """reference_lines.json: the line count of every C/C++/CUDA source under
    the reference's FVM/ and 3rd/CUDA_helper/, by file name, so that the
    file:line citations of this repository can be checked without the
    reference checkout (tests/test_citations.py)."""
    import json
    out = {}
    for sub in ("FVM", os.path.join("3rd", "CUDA_helper")):
        d = os.path.join(REFERENCE_TREE, sub)
        for f in sorted(os.listdir(d)):
            if f.endswith((".cpp", ".cu", ".h", ".hpp", ".cuh")):
                with open(os.path.join(d, f), "rb") as fh:
                    out[f] = len(fh.read().splitlines())
    with open(os.path.join(HERE, "reference_lines.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
        fh.write("\n")
    print("reference_lines.json", len(out), "files")


def make_loader_digests():
    """loader_models.json: for every tetgen mesh the reference ships
    (model/*/*.node with .ele and .face), what TetMesh's own loader
    (TetMesh.cpp:14-151) makes of it -- node and tet counts, the nodes its
    hard-coded rule pins, and SHA-256 digests of its FP32 rest positions
    (after the x0.1 scaling) and int32 tets in file order -- so that
    meshes.load_tetgen can be checked against it bit for bit
    (tests/test_loader_parity.py)."""
    import glob
    import hashlib
    import json
    out = {}
    for node in sorted(glob.glob(os.path.join(REFERENCE_TREE, "model", "*", "*.node"))):
        stem = node[:-len(".node")]
        if not all(os.path.exists(stem + e) for e in (".ele", ".face")):
            continue
        rest, tets, pins = REF.load_model(stem)
        rel = os.path.relpath(stem, os.path.join(REFERENCE_TREE, "model"))
        out[rel] = dict(n_nodes=int(rest.shape[0]), n_tets=int(tets.shape[0]), pins=pins.tolist(),
                        rest_sha256=hashlib.sha256(np.ascontiguousarray(rest, np.float32).tobytes()).hexdigest(),
                        tets_sha256=hashlib.sha256(np.ascontiguousarray(tets, np.int32).tobytes()).hexdigest())
    with open(os.path.join(HERE, "loader_models.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
        fh.write("\n")
    print("loader_models.json", len(out), "meshes")


if __name__ == "__main__":
    # `make_golden.py surface|stiffness|dynamics|lines|loader|inverted` write
    # only those fixtures
    only = sys.argv[1] if len(sys.argv) > 1 else None
    if only in (None, "lines"):
        make_reference_lines()
    if only in (None, "loader"):
        make_loader_digests()
    if only in (None, "inverted"):
        make_inverted()
    rng = np.random.default_rng(20261203)
    if only is None:
        for n, c in cases().items():
            make(n, c, rng)
    if only in (None, "surface"):
        srng = np.random.default_rng(20261204)
        for n, spec in surface_cases().items():
            make_surface(n, spec, srng)
    if only in (None, "stiffness"):
        krng = np.random.default_rng(20261205)
        all_cases = cases()
        for n in ("bar_small", "model_bar", "ellipsoid_small"):
            make_stiffness("stiffness_" + n, all_cases[n], krng)
    if only in (None, "dynamics"):
        drng = np.random.default_rng(20261206)
        all_cases = cases()
        for n in ("bar_small", "model_bar", "ellipsoid_small"):
            make_dynamics("dynamics_" + n, all_cases[n], drng)
