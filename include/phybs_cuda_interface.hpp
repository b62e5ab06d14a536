// phybs_cuda_interface.hpp - header-only C++ drop-in for PhyBS's
// CUDAInterface (FVM/CUDAInterface.h:20-102), built on the C ABI of phybs.h.
//
// It keeps the constructor and the step-loop calls that FVM/fvm.cpp makes
// (fvm.cpp:44-47 construct, :187 doDescentOpt, :101 updateNodePositions,
// :217 reset), so replacing
//     #include "CUDAInterface.h"
// with
//     #include "phybs_cuda_interface.hpp"
//     using CUDAInterface = phybs::CUDAInterface;
// is the whole change on the caller's side.  The CSR arguments the reference
// constructor takes for its backward-Euler solver are accepted and ignored:
// the descent step needs no global matrix (phybs::stiffness_pattern rebuilds
// the same pattern when a caller wants it).
//
// Differences from the reference, all documented in phybs.h:
//   - doDescentOpt honours its h argument (the reference's kernels always use
//     0.03, CUDAInterface.cu:644);
//   - errors are reported: every call throws phybs::Error on a PBS_E_* code
//     (the reference ignores CUDA errors);
//   - the backward-Euler path (fvm.cpp:179-183) keeps its three calls:
//     computeInnerforces and computeGlobalStiffnessMatrix are no-ops and
//     doBackEuler runs the whole step (pbs_backward_euler_step assembles the
//     forces and the matrix itself);
//   - pbdStep and projectiveDynamicsStep run the viewer's other two
//     integrators (PosBaseDynamic / ProjDynamic, fvm.cpp:162-171) on the same
//     state.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "phybs.h"

namespace phybs {

class Error : public std::runtime_error {
public:
    Error(int code, const char *what)
        : std::runtime_error(std::string(what) + ": " + pbs_error_string(code)), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc, const char *what) {
    if (rc != PBS_OK) throw Error(rc, what);
}

class CUDAInterface {
public:
    CUDAInterface(int num_nodes, const float *nodes, const float *restPoses, const int *constraintsMask, int num_tets,
                  const int *tets, const float youngs, const float nu, const float density, int /*csr_nnz*/ = 0,
                  int /*csr_m*/ = 0, float * /*csr_val*/ = nullptr, int * /*csr_row*/ = nullptr,
                  int * /*csr_col*/ = nullptr, int * /*csr_diagonalIdx*/ = nullptr,
                  int * /*csr_kIDinCSRval*/ = nullptr)
        : n_nodes_(num_nodes) {
        pbs_mesh_desc d{};
        d.n_nodes = num_nodes;
        d.rest = restPoses;
        d.positions = nodes;
        d.n_tets = num_tets;
        d.tets = tets;
        d.pin_mask = constraintsMask;
        d.n_instances = 1;
        d.density = density;
        d.gravity = 9.8f;
        check(pbs_create(&d, &h_), "pbs_create");
        float mu, lambda;
        pbs_lame(youngs, nu, 1, &mu, &lambda);  // CUDAInterface.cu:704-705
        check(pbs_set_material(h_, PBS_MATERIAL_NEOHOOKEAN, &mu, &lambda, 1), "pbs_set_material");
        pbs_default_params(&params_);
        params_.body_force_scale = 1.0f;        // gravity once (CUDAInterface.cu:600-602)
        params_.energy_clamp = PBS_CLAMP_GPU;   // max(e, 0) (CUDAInterface.cu:549)
        check(pbs_set_params(h_, &params_), "pbs_set_params");
    }
    ~CUDAInterface() { pbs_destroy(h_); }
    CUDAInterface(const CUDAInterface &) = delete;
    CUDAInterface &operator=(const CUDAInterface &) = delete;

    // CUDAInterface::doDescentOpt (CUDAInterface.cu:911-1007)
    void doDescentOpt(float h, int iterations, float *hostExternForces, float *hostNode) {
        if (h != params_.h || iterations != params_.max_iters) {
            params_.h = h;
            params_.max_iters = iterations;
            check(pbs_set_params(h_, &params_), "pbs_set_params");
        }
        int rc = pbs_step(h_, hostExternForces, nullptr);
        if (rc != PBS_OK && rc != PBS_E_ITER_CAP) throw Error(rc, "pbs_step");
        check(pbs_read_positions(h_, hostNode), "pbs_read_positions");
    }
    // CUDAInterface::updateNodePositions (CUDAInterface.cu:771)
    void updateNodePositions(const float *hostNode) { check(pbs_update_positions(h_, hostNode), "pbs_update_positions"); }
    // CUDAInterface::reset (CUDAInterface.cu:776)
    void reset() { check(pbs_reset(h_), "pbs_reset"); }

    // CUDAInterface::computeInnerforces / computeGlobalStiffnessMatrix /
    // doBackEuler (CUDAInterface.cu:784-884): h = 0.03, alpha = beta = 0.02.
    void computeInnerforces() {}
    void computeGlobalStiffnessMatrix() {}
    void doBackEuler(float *hostNode, float h = 0.03f, float tol = 1e-6f, int max_iters = 4000) {
        int rc = pbs_backward_euler_step(h_, h, 0.02f, 0.02f, nullptr, tol, max_iters, nullptr, nullptr);
        if (rc != PBS_OK && rc != PBS_E_ITER_CAP) throw Error(rc, "pbs_backward_euler_step");
        check(pbs_read_positions(h_, hostNode), "pbs_read_positions");
    }

    // PosBaseDynamic::doStepStrainConstraints (fvm.cpp:162-165): 5 sweeps,
    // stretch 1, shear 0.8; hostExternForces 3N floats or nullptr.
    void pbdStep(float t, const float *hostExternForces, float *hostNode, int sweeps = 5) {
        check(pbs_pbd_step(h_, t, sweeps, nullptr, nullptr, hostExternForces), "pbs_pbd_step");
        check(pbs_read_positions(h_, hostNode), "pbs_read_positions");
    }

    // ProjDynamic::doProjDynamics (fvm.cpp:167-170, matrix at fvm.cpp:305):
    // t = 0.03 for the step, tMatrix the integrator's time step for A.
    void projectiveDynamicsStep(float t, float tMatrix, const float *hostExternForces, float *hostNode,
                                float tol = 1e-6f, int max_cg = 20000) {
        int rc = pbs_pd_step(h_, t, tMatrix, 1e6f, 5, hostExternForces, tol, max_cg, nullptr);
        if (rc != PBS_OK && rc != PBS_E_ITER_CAP) throw Error(rc, "pbs_pd_step");
        check(pbs_read_positions(h_, hostNode), "pbs_read_positions");
    }

    pbs_handle *handle() const { return h_; }
    pbs_step_params &params() { return params_; }

private:
    pbs_handle *h_ = nullptr;
    int n_nodes_ = 0;
    pbs_step_params params_{};
};

// IsotropicMaterial::allocateGlobalStiffnessMatrix's CSR pattern.
struct StiffnessPattern {
    std::vector<int> row_ptr, col, diag_idx, kid48;
};
inline StiffnessPattern stiffness_pattern(int n_nodes, int n_tets, const int *tets) {
    StiffnessPattern p;
    int nnz = 0;
    check(pbs_stiffness_pattern(n_nodes, n_tets, tets, &nnz, nullptr, nullptr, nullptr, nullptr), "pbs_stiffness_pattern");
    p.row_ptr.resize(3 * (size_t)n_nodes + 1);
    p.col.resize(nnz);
    p.diag_idx.resize(3 * (size_t)n_nodes);
    p.kid48.resize(48 * (size_t)n_tets);
    check(pbs_stiffness_pattern(n_nodes, n_tets, tets, &nnz, p.row_ptr.data(), p.col.data(), p.diag_idx.data(),
                                p.kid48.data()),
          "pbs_stiffness_pattern");
    return p;
}

}  // namespace phybs
