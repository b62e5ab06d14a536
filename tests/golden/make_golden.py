"""Generate tests/golden/*.npz from the reference's own CPU solver.

Run where the reference tree exists (it is compiled headless into
oracle/_ref by oracle/ref_build/Makefile):

    python tests/golden/make_golden.py

Each fixture freezes, for one mesh, the reference's outputs: the rest state it
loaded (TetMesh.cpp:186-216), forces / energies / Hessian diagonal at a
deformed probe state (IsotropicNeohookeanMaterial.cpp:135-173,
IsotropicMaterial.cpp:360-409, 503-682), the stiffness CSR pattern
(IsotropicMaterial.cpp:554-644) for small meshes, and the node positions and
velocities after successive DescentOptimize::doDescentOpt steps
(DescentOptimize.cpp:146-243).  Meshes are the procedural workloads of the
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

from oracle import REFERENCE_TREE  # noqa: E402
from oracle import ref as REF  # noqa: E402
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


if __name__ == "__main__":
    rng = np.random.default_rng(20261203)
    for n, c in cases().items():
        make(n, c, rng)
