// The per-instance decisions of a descent pass, on a copy of the instance's
// control block: the line-search accept / reject of a check pass and the
// residual test, Chebyshev state, parity and caps after the node update.  The
// graph path takes them in the last CTA of a pass kernel (chunks.cu,
// kernels.cu); the persistent frame kernel (chunks.cu) takes them in every CTA
// from the same sums, so every CTA's copy stays the same.
#pragma once
#include <math.h>

#include "../../include/phybs.h"
#include "phybs_internal.cuh"

namespace pbs {

// Line-search decision of a check pass at iteration k (DescentOptimize.cpp:
// 107-128) from the instance's energy E and the sum of its squared terms E2.
// Sets ci.action for the node update of the same pass.
__device__ __forceinline__ void decide_line_search(InstCtl &ci, const DevParams &p, int k, double E, double E2) {
    ci.energy = E;
    // rounding-noise allowance: the FP64 sum of FP32 terms e_i carries a random
    // error of order 2^-24 sqrt(sum e_i^2); slack 0 is the reference's strict test
    const double tau = (double)p.energy_slack * 5.9604644775390625e-8 * sqrt(E2);
    // RESTART control also treats a non-finite energy (a step that inverted
    // tets) as a rejection; the reference control accepts it (NaN > E_old is
    // false), and the step then ends with PBS_E_NONFINITE below
    const bool bad = !isfinite(E) && p.control == PBS_CONTROL_RESTART;
    if ((k != 0 && E > ci.energy_old + tau) || (bad && k != 0)) {
        ci.action = ACT_RESTORE;
        ci.alpha = (float)((double)ci.alpha * (double)p.alpha_shrink);
        ci.rejections += 1;
        if (p.control == PBS_CONTROL_REFERENCE) ci.iters -= k - p.ls_every;
    } else {
        ci.action = ACT_SAVE_STEP;
        ci.energy_old = E;
        // grow only after real steps since the last restore (not on the re-check
        // of a restored iterate, whose energy is the accepted one)
        if (p.control == PBS_CONTROL_RESTART && k != 0 && k > ci.k_restart)
            ci.alpha = fminf(ci.alpha * p.alpha_grow, p.alpha0);
    }
    // force_check stays set: the node update of this pass reads it to apply the
    // decision, and the pass decision clears it
    if (!isfinite(E) && !(bad && k != 0)) {
        ci.status = PBS_E_NONFINITE;
        ci.done = 1;
    }
}

// The pass decision after the node update of iteration k, which took `action`
// with the schedule's (rho, omega) and left |g(x_k)|^2 = R2.  No FP64 square
// root or division: the stop test compares |g|^2 with (tol g0)^2; the ratio is
// formed on the host.
__device__ __forceinline__ void decide_pass(InstCtl &ci, const DevParams &p, int k, int action, float rho,
                                            float omega, double R2) {
    int passes = ci.passes + 1, par_c = ci.par, kk = k, done = 0, converged = 0, status = ci.status;
    int force_check = 0, k_restart = ci.k_restart;
    double g0 = ci.g0;
    float rho_n = ci.rho, omega_n = ci.omega;
    if (action == ACT_RESTORE) {
        par_c = 1 - par_c;  // the restored state; k is redone
        if (p.control == PBS_CONTROL_RESTART) k_restart = k;  // rerun the rho schedule from here
    } else {
        if (k == 0 && !ci.g0_fixed) g0 = sqrt(R2);
        ci.r2 = R2;
        const double lim = (double)p.tol * g0;
        if (p.tol > 0.f && k > 0 && R2 <= lim * lim) {
            converged = 1;  // keep x_k (the current parity)
            done = 1;
        } else {
            rho_n = rho;
            omega_n = omega;
            par_c = 1 - par_c;
            kk = k + 1;
        }
        if (!isfinite(R2)) {
            if (p.control == PBS_CONTROL_RESTART && kk > 0) {
                force_check = 1;  // the next pass measures the energy and restores
                converged = 0;
                done = 0;
            } else {
                status = PBS_E_NONFINITE;
                done = 1;
            }
        }
    }
    if (!done) {
        if (kk >= ci.iters || ci.alpha < p.alpha_min) done = 1;
        else if (passes >= p.pass_cap) { done = 1; status = PBS_E_ITER_CAP; }
    }
    ci.counter_n = 0;
    ci.passes = passes;
    ci.force_check = force_check;  // a forced line-search check was applied in this pass
    ci.par = par_c;
    ci.k_restart = k_restart;
    ci.g0 = g0;
    ci.rho = rho_n;
    ci.omega = omega_n;
    ci.k = kk;
    ci.converged = converged;
    ci.status = status;
    ci.done = done;
}

}  // namespace pbs
