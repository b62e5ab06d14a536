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
//
// Displacement differences are formed from the state's full (hi, lo) pair:
// forces from the hi word alone would see u quantised to ulp(|u|), and
// K * ulp(|u|) summed over the mesh is a residual floor that grows with the
// accumulated displacement (5e-4 of the initial residual by the third frame
// of the 1M-tet pull).
__device__ __forceinline__ float4 f4sub(const float4 &a, const float4 &b) {
    return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, 0.f);
}
__device__ __forceinline__ float4 f4add(const float4 &a, const float4 &b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, 0.f);
}

template <int MATERIAL>
__device__ __forceinline__ void pass_forces(const DevParams &p, const float4 *U, const float4 *UL, const float4 *U0,
                                            const int4 &q, const float dinv[9], float svol, float mu, float lambda,
                                            Kin<float> &kin, float f[12]) {
    const float4 x0 = U[q.x], x1 = U[q.y], x2 = U[q.z], x3 = U[q.w];
    const float4 l0 = UL[q.x], l1 = UL[q.y], l2 = UL[q.z], l3 = UL[q.w];
    float P[9];
    if (MATERIAL != PBS_MATERIAL_STRETCH && p.incremental) {
        disp_gradient<float>(x0, x1, x2, x3, dinv, kin.G);
        kinematics(kin);
        const float4 a0 = U0[q.x], a1 = U0[q.y], a2 = U0[q.z], a3 = U0[q.w];
        Kin<float> k0;
        disp_gradient<float>(a0, a1, a2, a3, dinv, k0.G);
        kinematics(k0);
        // increments from the base: (u_hi - base) + u_lo
        float dG[9];
        disp_gradient<float>(f4add(f4sub(x0, a0), l0), f4add(f4sub(x1, a1), l1), f4add(f4sub(x2, a2), l2),
                             f4add(f4sub(x3, a3), l3), dinv, dG);
        pk1_neohookean_delta<float>(k0, kin, dG, mu, lambda, P);
    } else {
        // Du = (u_j,hi - u_0,hi) + (u_j,lo - u_0,lo)
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        disp_gradient<float>(z, f4add(f4sub(x1, x0), f4sub(l1, l0)), f4add(f4sub(x2, x0), f4sub(l2, l0)),
                             f4add(f4sub(x3, x0), f4sub(l3, l0)), dinv, kin.G);
        kinematics(kin);
        if (MATERIAL == PBS_MATERIAL_STRETCH) pk1_stretch(kin, mu, lambda, P);
        else pk1_neohookean<float>(kin, mu, lambda, P);
    }
    corner_forces(P, dinv, svol, f);
}

}  // namespace pbs
