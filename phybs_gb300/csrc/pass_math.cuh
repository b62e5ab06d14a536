// Per-tet force evaluation shared by the pass kernels and the warm start.
#pragma once
#include "../../include/phybs.h"
#include "phybs_internal.cuh"
#include "tet_math.cuh"

namespace pbs {

// Corner forces of a tet in a descent pass.  Neo-Hookean with p.incremental:
// the increment dP = P(F) - P(F0) against the base displacement U0 (the
// step's initial guess; the node kernel adds the FP64 force at the base held
// in bh/bl), so the summed corner terms scale with the guess's error rather
// than with the stress and the residual has no FP32 floor above ~1e-6 of its
// initial value; otherwise the full stress.  kin returns the current
// kinematics (energy, Jacobi diagonal).
template <int MATERIAL>
__device__ __forceinline__ void pass_forces(const DevParams &p, const float4 *U, const float4 *U0, const int4 &q,
                                            const float dinv[9], float svol, float mu, float lambda, Kin<float> &kin,
                                            float f[12]) {
    const float4 x0 = U[q.x], x1 = U[q.y], x2 = U[q.z], x3 = U[q.w];
    disp_gradient<float>(x0, x1, x2, x3, dinv, kin.G);
    kinematics(kin);
    float P[9];
    if (MATERIAL == PBS_MATERIAL_STRETCH) {
        pk1_stretch(kin, mu, lambda, P);
    } else if (p.incremental) {
        const float4 a0 = U0[q.x], a1 = U0[q.y], a2 = U0[q.z], a3 = U0[q.w];
        Kin<float> k0;
        disp_gradient<float>(a0, a1, a2, a3, dinv, k0.G);
        kinematics(k0);
        const float4 d0 = make_float4(x0.x - a0.x, x0.y - a0.y, x0.z - a0.z, 0.f);
        const float4 d1 = make_float4(x1.x - a1.x, x1.y - a1.y, x1.z - a1.z, 0.f);
        const float4 d2 = make_float4(x2.x - a2.x, x2.y - a2.y, x2.z - a2.z, 0.f);
        const float4 d3 = make_float4(x3.x - a3.x, x3.y - a3.y, x3.z - a3.z, 0.f);
        float dG[9];
        disp_gradient<float>(d0, d1, d2, d3, dinv, dG);
        pk1_neohookean_delta<float>(k0, kin, dG, mu, lambda, P);
    } else {
        pk1_neohookean<float>(kin, mu, lambda, P);
    }
    corner_forces(P, dinv, svol, f);
}

}  // namespace pbs
