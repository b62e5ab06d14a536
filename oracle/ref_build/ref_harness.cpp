// C-ABI harness over the reference's own CPU solver, built headless.
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled together with the
// unmodified reference sources FVM/TetMesh.cpp, FVM/IsotropicMaterial.cpp,
// FVM/IsotropicNeohookeanMaterial.cpp, FVM/DescentOptimize.cpp,
// FVM/PosBaseDynamic.cpp and FVM/ProjDynamic.cpp (read in place from the
// reference tree by oracle/ref_build/Makefile) into
// oracle/_ref/libphybs_ref.so.  It is the parity anchor for the restated
// oracle (oracle/phybs_oracle.cpp) and the generator of tests/golden fixtures.
//
// Mesh injection: TetMesh() loads "..\\model\\armadillo\\armadillo.1.*" and
// scales coordinates by 0.1 (TetMesh.cpp:36-38,179-181).  The harness writes
// the caller's mesh as tetgen text with coordinates x10 and redirects the
// shim's QFile to it.  The reference's post-load rest positions
// (ref_get_rest) are therefore the canonical inputs for every comparison.
// Pins: the loader's own rule (z>0 && y>8.5 after scaling, TetMesh.cpp:39)
// must select nothing; the caller's pins are then applied exactly as
// TetMesh.cpp:212-216 does (mass 1e8, inverse mass 0), after gravity was
// formed from the lumped masses (TetMesh.cpp:205).
#include <vector>
#include <memory>
#include <array>
#include <set>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <iostream>
#include <string>
#include <Eigen/Dense>
#include <Eigen/Sparse>
#include <Eigen/SVD>
#include <omp.h>
#include "phybs_qt_shim.h"

// Reach the reference classes' private state (h, Chebyshev profile, pins).
#define private public
#define protected public
#include "TetMesh.h"
#include "IsotropicNeohookeanMaterial.h"
#include "DescentOptimize.h"
#include "PosBaseDynamic.h"
#include "ProjDynamic.h"
#undef private
#undef protected

static std::string g_stem;
void phybs_shim_set_mesh_stem(const std::string &stem) { g_stem = stem; }
const std::string &phybs_shim_mesh_stem() { return g_stem; }

struct RefSim {
    std::shared_ptr<TetMesh> mesh;
    std::shared_ptr<IsotropicNeohookeanMaterial> mat;
    std::shared_ptr<DescentOptimize> opt;
};

static Eigen::MatrixXf as_pos(const float *p, int n) {
    Eigen::MatrixXf m(3, n);
    std::memcpy(m.data(), p, sizeof(float) * 3 * (size_t)n);
    return m;
}

extern "C" {

// Returns nullptr on failure (unwritable work dir, density other than the
// loader's 1000, or the loader's own pin rule selecting nodes).  faces: the
// mesh's boundary triangles for TetMesh's .face file (n_faces = 0 writes an
// empty one); the loader builds their rings (TetMesh.cpp:150).
void *ref_create_faces(const char *workdir, int n_nodes, const float *pos, int n_tets, const int *tets,
                       int n_pins, const int *pins, float E, float nu, float density, int n_faces,
                       const int *faces) {
    if (density != 1000.0f) return nullptr;  // TetMesh.cpp:185 fixes the loader's density
    std::string stem = std::string(workdir) + "/mesh";
    {
        FILE *f = std::fopen((stem + ".node").c_str(), "w");
        if (!f) return nullptr;
        std::fprintf(f, "%d  3  0  0\n", n_nodes);
        for (int i = 0; i < n_nodes; ++i)
            std::fprintf(f, "%d %.9g %.9g %.9g\n", i, 10.0 * (double)pos[3 * i], 10.0 * (double)pos[3 * i + 1],
                         10.0 * (double)pos[3 * i + 2]);
        std::fclose(f);
        f = std::fopen((stem + ".ele").c_str(), "w");
        if (!f) return nullptr;
        std::fprintf(f, "%d  4  0\n", n_tets);
        for (int i = 0; i < n_tets; ++i)
            std::fprintf(f, "%d %d %d %d %d\n", i, tets[4 * i], tets[4 * i + 1], tets[4 * i + 2], tets[4 * i + 3]);
        std::fclose(f);
        f = std::fopen((stem + ".face").c_str(), "w");
        if (!f) return nullptr;
        std::fprintf(f, "%d  0\n", n_faces);
        for (int i = 0; i < n_faces; ++i)
            std::fprintf(f, "%d %d %d %d\n", i, faces[3 * i], faces[3 * i + 1], faces[3 * i + 2]);
        std::fclose(f);
    }
    phybs_shim_set_mesh_stem(stem);
    RefSim *s = new RefSim();
    s->mesh = std::make_shared<TetMesh>();
    if (!s->mesh->m_constraintIDs.empty()) { delete s; return nullptr; }
    s->mesh->setTetMaterial(E, nu, density);
    std::vector<int> p(pins, pins + n_pins);
    std::sort(p.begin(), p.end());
    s->mesh->m_constraintIDs = p;
    for (size_t i = 0; i < p.size(); ++i) {
        s->mesh->m_nodes_invMass(p[i]) = 0.0;
        s->mesh->m_nodes_mass(p[i]) = 1e8;
    }
    s->mat = std::make_shared<IsotropicNeohookeanMaterial>(s->mesh);
    s->opt = std::make_shared<DescentOptimize>(s->mesh, s->mat);
    return s;
}

void *ref_create(const char *workdir, int n_nodes, const float *pos, int n_tets, const int *tets,
                 int n_pins, const int *pins, float E, float nu, float density) {
    return ref_create_faces(workdir, n_nodes, pos, n_tets, tets, n_pins, pins, E, nu, density, 0, nullptr);
}

void ref_destroy(void *h) { delete static_cast<RefSim *>(h); }

static RefSim *S(void *h) { return static_cast<RefSim *>(h); }

void ref_set_h(void *h, float dt) { S(h)->opt->m_h = dt; }

void ref_set_profile(void *h, int n, const int *ks, const float *vs) {
    DescentOptimize *o = S(h)->opt.get();
    o->m_profile_n = n;
    for (int i = 0; i < n && i < 3; ++i) { o->m_profile_k[i] = ks[i]; o->m_profile_v[i] = vs[i]; }
}

void ref_set_lame(void *h, const float *mu, const float *lambda) {
    RefSim *s = S(h);
    for (size_t i = 0; i < s->mat->m_mus.size(); ++i) { s->mat->m_mus[i] = mu[i]; s->mat->m_lambdas[i] = lambda[i]; }
}

void ref_get_lame(void *h, float *mu, float *lambda) {
    RefSim *s = S(h);
    for (size_t i = 0; i < s->mat->m_mus.size(); ++i) { mu[i] = s->mat->m_mus[i]; lambda[i] = s->mat->m_lambdas[i]; }
}

void ref_get_rest(void *h, float *out) {
    auto &m = S(h)->mesh->getRestPosition();
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}
void ref_get_nodes(void *h, float *out) {
    auto &m = S(h)->mesh->getNodes();
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}
void ref_set_nodes(void *h, const float *in) {
    auto &m = S(h)->mesh->getNodes();
    std::memcpy(m.data(), in, sizeof(float) * m.size());
}
void ref_get_vel(void *h, float *out) {
    auto &m = S(h)->mesh->getVelocities();
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}
void ref_set_vel(void *h, const float *in) {
    auto &m = S(h)->mesh->getVelocities();
    std::memcpy(m.data(), in, sizeof(float) * m.size());
}
void ref_get_vel_old(void *h, float *out) {
    auto &m = S(h)->opt->m_vel_old;
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}
void ref_set_vel_old(void *h, const float *in) {
    auto &m = S(h)->opt->m_vel_old;
    std::memcpy(m.data(), in, sizeof(float) * m.size());
}
void ref_set_ext(void *h, const float *in) {
    auto &m = S(h)->mesh->getExternalForces();
    std::memcpy(m.data(), in, sizeof(float) * m.size());
}
void ref_get_mass(void *h, float *out) {
    auto &m = S(h)->mesh->getMasses();
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}
void ref_get_gravity(void *h, float *out) {
    auto &m = S(h)->mesh->getGravities();
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}
void ref_get_vol(void *h, float *out) {
    auto &m = S(h)->mesh->getTetVolumes();
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}
// 3 x 3T column-major: tet i's 3x3 block starts at 9*i and is column-major.
void ref_get_dminv(void *h, float *out) {
    auto &m = S(h)->mesh->m_Dm_inverses;
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}
void ref_get_an(void *h, float *out) {
    auto &m = S(h)->mesh->m_ANs;
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}

// IsotropicNeohookeanMaterial::computeInnerForceFromPos: gravity + external +
// elastic, with pinned nodes overwritten by the 1e8 spring (TetMesh.cpp:580).
void ref_force_nh(void *h, const float *pos, float *out) {
    RefSim *s = S(h);
    Eigen::MatrixXf f = s->mat->computeInnerForceFromPos(as_pos(pos, s->mesh->getNodesNum()));
    std::memcpy(out, f.data(), sizeof(float) * f.size());
}

// IsotropicMaterial::computeInnerForcesfromFhats2 (stretch-based P = U P^ V^T);
// it reads the mesh's current nodes, so they are swapped in and restored.
// nthreads <= 0 selects the serial variant (IsotropicMaterial.cpp:360),
// otherwise the OpenMP one (IsotropicMaterial.cpp:411).
void ref_force_stretch(void *h, const float *pos, int nthreads, float *out) {
    RefSim *s = S(h);
    Eigen::MatrixXf saved = s->mesh->getNodes();
    s->mesh->getNodes() = as_pos(pos, s->mesh->getNodesNum());
    Eigen::MatrixXf f = nthreads > 0 ? s->mat->computeInnerForcesfromFhats2(nthreads) : s->mat->computeInnerForcesfromFhats2();
    s->mesh->getNodes() = saved;
    std::memcpy(out, f.data(), sizeof(float) * f.size());
}

// Per-tet clamped elastic energy (IsotropicNeohookeanMaterial.cpp:116-131).
void ref_elastic_energy(void *h, const float *pos, float *out) {
    RefSim *s = S(h);
    s->mat->computeElasticEnergyFromPos(as_pos(pos, s->mesh->getNodesNum()));
    auto &e = s->mat->getElasticEnergys();
    std::memcpy(out, e.data(), sizeof(float) * e.size());
}

// diag(K(pos)) as DescentOptimize.cpp:133 forms it (before adding M/h^2).
void ref_hessian_diag(void *h, const float *pos, float *out) {
    RefSim *s = S(h);
    Eigen::SparseMatrix<float, Eigen::RowMajor> K =
        s->mat->computeGlobalStiffnessMatrixFromPos(as_pos(pos, s->mesh->getNodesNum()));
    Eigen::VectorXf d = K.diagonal();
    std::memcpy(out, d.data(), sizeof(float) * d.size());
}

// Full 12x12 element stiffness of one tet (IsotropicMaterial.cpp:503), row-major.
void ref_element_stiffness(void *h, int tet, const float *pos, float *out144) {
    RefSim *s = S(h);
    Eigen::MatrixXf K = s->mat->computeStiffnessMatrixFromPos(tet, as_pos(pos, s->mesh->getNodesNum()));
    for (int r = 0; r < 12; ++r)
        for (int c = 0; c < 12; ++c) out144[r * 12 + c] = K(r, c);
}

// DescentOptimize::computeTotalEnergy(pos) with the inertial target x~ given.
float ref_total_energy(void *h, const float *pos, const float *xtilde) {
    RefSim *s = S(h);
    int n = s->mesh->getNodesNum();
    s->opt->m_pos = as_pos(xtilde, n);
    return s->opt->computeTotalEnergy(as_pos(pos, n));
}

void ref_csr_sizes(void *h, int *nnz, int *rows) {
    auto &K = S(h)->mat->getGlobalK();
    *nnz = (int)K.nonZeros();
    *rows = (int)K.rows();
}
void ref_csr(void *h, int *rowptr, int *colidx, int *diag_idx, int *kid48) {
    RefSim *s = S(h);
    auto &K = s->mat->getGlobalK();
    std::memcpy(rowptr, K.outerIndexPtr(), sizeof(int) * (K.rows() + 1));
    std::memcpy(colidx, K.innerIndexPtr(), sizeof(int) * K.nonZeros());
    auto &d = s->mat->getDiagonalIdx();
    std::memcpy(diag_idx, d.data(), sizeof(int) * d.size());
    auto &k = s->mat->getKIDinCSRval();
    std::memcpy(kid48, k.data(), sizeof(int) * k.size());
}

// One DescentOptimize::doDescentOpt(iters) step (DescentOptimize.cpp:91).
void ref_step(void *h, int iters) { S(h)->opt->doDescentOpt(iters); }

// The solver's scalar state after a step: alpha, energy, energy_old, rho, omega.
void ref_get_scalars(void *h, float *out5) {
    DescentOptimize *o = S(h)->opt.get();
    out5[0] = o->m_alpha; out5[1] = o->m_energy; out5[2] = o->m_energy_old; out5[3] = o->m_rho; out5[4] = o->m_omega;
}

int ref_num_threads() { return omp_get_max_threads(); }

// Surface picking and drag (TetMesh.cpp:229-277, 378-418, 446-470, 595-614),
// on the mesh's current nodes (ref_set_nodes).
int ref_face_ring_size(void *h, int face) { return (int)S(h)->mesh->m_faceRingIndices[face].size(); }
void ref_face_ring(void *h, int face, int *out) {
    const auto &r = S(h)->mesh->m_faceRingIndices[face];
    std::copy(r.begin(), r.end(), out);
}
// computeBoundfaceNormals, then pickFacebyRay; normals / centers: 3 x faces
int ref_pick_face(void *h, const float *orig, const float *dir, float *normals, float *centers) {
    TetMesh *m = S(h)->mesh.get();
    m->computeBoundfaceNormals();
    std::memcpy(normals, m->m_bound_normals.data(), sizeof(float) * m->m_bound_normals.size());
    std::memcpy(centers, m->m_face_centers.data(), sizeof(float) * m->m_face_centers.size());
    return m->pickFacebyRay(Eigen::Vector3f(orig[0], orig[1], orig[2]), Eigen::Vector3f(dir[0], dir[1], dir[2]));
}
void ref_drag_face_ring(void *h, int face, const float *drag) {
    S(h)->mesh->dragFaceRing(face, Eigen::Vector3f(drag[0], drag[1], drag[2]));
}
void ref_get_ext(void *h, float *out) {
    auto &m = S(h)->mesh->getExternalForces();
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}
float ref_ext_energy(void *h, const float *pos) {
    RefSim *s = S(h);
    return s->mesh->computeExternalForcesEnergy(as_pos(pos, s->mesh->getNodesNum()));
}

// Inverse lumped masses (0 at a pinned node; TetMesh.cpp:207-215).
void ref_get_inv_mass(void *h, float *out) {
    auto &m = S(h)->mesh->getInvMasses();
    std::memcpy(out, m.data(), sizeof(float) * m.size());
}

// One strain-based PBD step as the viewer runs it (fvm.cpp:162-165): forces =
// TetMesh::computeExternalForces() (gravity + external + pin springs), then
// PosBaseDynamic::doStepStrainConstraints on the mesh's nodes and velocities.
void ref_pbd_step(void *h, float dt) {
    TetMesh *m = S(h)->mesh.get();
    PosBaseDynamic pbd(m->getNodes(), m->getTetsNum());
    Eigen::MatrixXf f = m->computeExternalForces();
    pbd.doStepStrainConstraints(m->getNodes(), m->getVelocities(), f, m->getDmInvs(), m->getTets(),
                                m->getInvMasses(), dt);
}

// Projective dynamics (ProjDynamic.cpp): the integrator object, its solver
// matrix for time step dt_matrix (FVM::SetTypeComputing, fvm.cpp:300-307) and
// one doProjDynamics step at dt with `iterations` local/global iterations
// (the reference's 5; fvm.cpp:167-170 passes dt = 0.03).
void *ref_pd_create(void *h, float dt_matrix, int iterations) {
    TetMesh *m = S(h)->mesh.get();
    ProjDynamic *pd = new ProjDynamic(S(h)->mesh);
    pd->m_iterations = iterations;
    pd->buildGlobalSolverMatrix(m->getMasses(), m->getTets(), dt_matrix, m->getDmInvs());
    return pd;
}
// TetMesh's own loader (TetMesh.cpp:14-151, run by its constructor) on the
// tetgen files <stem>.node/.ele/.face: rest positions after its x0.1 scaling
// (3 x n_nodes, column-major), tets in file order (4 x n_tets) and the nodes its
// hard-coded rule pins (TetMesh.cpp:38-39).  Pass NULL outputs to read the
// sizes only.  The caller checks that the three files exist: the loader exits
// the process when one is missing.
void ref_load_model(const char *stem, int *n_nodes, int *n_tets, int *n_pins, float *rest, int *tets, int *pins) {
    phybs_shim_set_mesh_stem(stem);
    TetMesh m;
    phybs_shim_set_mesh_stem("");
    *n_nodes = m.getNodesNum();
    *n_tets = m.getTetsNum();
    *n_pins = (int)m.m_constraintIDs.size();
    if (rest) std::memcpy(rest, m.getRestPosition().data(), sizeof(float) * 3 * (size_t)*n_nodes);
    if (tets) std::memcpy(tets, m.getTets().data(), sizeof(int) * 4 * (size_t)*n_tets);
    if (pins) std::memcpy(pins, m.m_constraintIDs.data(), sizeof(int) * (size_t)*n_pins);
}

void ref_pd_destroy(void *pd) { delete static_cast<ProjDynamic *>(pd); }
void ref_pd_step(void *pd, void *h, float dt) {
    TetMesh *m = S(h)->mesh.get();
    static_cast<ProjDynamic *>(pd)->doProjDynamics(m->getNodes(), m->getVelocities(), m->getMasses(),
                                                   m->getInvMasses(), m->getTets(), dt, m->getDmInvs(),
                                                   m->computeExternalForces());
}

}  // extern "C"
