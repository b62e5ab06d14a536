// The per-instance decisions of a descent pass, on a copy of the instance's
// control block: the line-search accept / reject of a check pass and the
// residual test, Chebyshev state, parity and caps after the node update.  The
// graph path takes the line search in the last CTA of the pass's tet kernel
// and the pass decision in the first chunk CTA of the next pass's tet kernel
// (settle_pass, chunks.cu) or in k_settle after the last pass of a run
// (kernels.cu); the persistent frame kernel (chunks.cu) takes them in every
// CTA from the same sums, so every CTA's copy stays the same.
#pragma once
#include <math.h>

#include "../../include/phybs.h"
#include "pass_math.cuh"
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

// What a pass's tet kernel works from: the control block of its instance as
// the last pass left it, whose pass decision may still be pending.  That
// decision moves k on by one unless the last node update restored the saved
// iterate (k is then redone) or the instance stops (this pass's work is then
// unused: nothing reads it).  The one outcome the tet CTAs cannot foresee, a
// residual that turned non-finite and forces an energy check at a k without
// one, makes the pass void (settle_pass).
struct PassView {
    int k;
    bool skip, check, do_h;
};

__device__ __forceinline__ PassView pass_view(const InstCtl *c, const DevParams &p) {
    PassView v;
    const int k = c->k, fc = c->force_check;
    v.skip = c->done != 0;
    if (c->pending) {
        const int act = ((k % p.ls_every) == 0 || fc) ? c->action : ACT_STEP;
        v.k = act == ACT_RESTORE ? k : k + 1;
        v.check = (v.k % p.ls_every) == 0;
    } else {
        v.k = k;
        v.check = (k % p.ls_every) == 0 || fc;
    }
    v.do_h = (v.k % p.hd_every) == 0;
    return v;
}

// A control block read around L1: written by another CTA of the running
// kernel.
__device__ __forceinline__ InstCtl load_ctl_cg(const InstCtl *p) {
    static_assert(sizeof(InstCtl) % 16 == 0, "InstCtl is read as 16-byte words");
    InstCtl c;
    const int4 *s = reinterpret_cast<const int4 *>(p);
    int4 *d = reinterpret_cast<int4 *>(&c);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(InstCtl) / 16); ++i) d[i] = __ldcg(s + i);
    return c;
}

// The pass decision of the instance's last node update, taken by one CTA from
// the control block src into dst: |g|^2 summed in double-float from the node
// blocks' partials (each thread its blocks in ascending order, then the block
// tree), then decide_pass with the action, rho and omega that update used.
// in_pass: the first chunk CTA of a pass that already runs on the outcome
// (pass_view); dst is then the copy this pass's line search and node kernel
// read, its decision pending again, and a forced energy check at a k without
// one makes this pass void.  Otherwise (k_settle, after the last pass of a
// run) the decision is left settled.  A device wait that gave up (active[1])
// stops the instance with PBS_E_DEVICE_TIMEOUT.  Called by every thread.
template <int THREADS>
__device__ __forceinline__ void settle_pass(const DevParams &p, const DevState &st, const InstCtl *src,
                                            InstCtl *dst, bool in_pass) {
    __shared__ float2 shf[THREADS / 32];
    const bool pend = src->pending && !src->done;
    const int nb0 = src->nblk_begin, nb1 = src->nblk_end;
    DFloat acc{0.f, 0.f};
    if (pend) {
        // eight partials in flight a thread ahead of their additions
        constexpr int U = 8;
        for (int j0 = nb0 + (int)threadIdx.x; j0 < nb1; j0 += U * THREADS) {
            float v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) v[u] = j0 + u * THREADS < nb1 ? __ldcg(st.npartf + j0 + u * THREADS) : 0.f;
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (j0 + u * THREADS < nb1) acc = df_add(acc, v[u]);
        }
    }
    // (its barriers also order every thread's reads of src before the store)
    const DFloat R = block_sum_df(acc, shf);
    if (threadIdx.x != 0) return;
    InstCtl ci = *src;
    const bool was_done = ci.done != 0;
    if (!ci.done) {
        if (ci.void_pass) {
            // the void pass copied the state to the other parity
            ci.void_pass = 0;
            ci.par = 1 - ci.par;
            ci.passes += 1;
            if (ci.passes >= p.pass_cap) {
                ci.done = 1;
                ci.status = PBS_E_ITER_CAP;
            }
        } else if (ci.pending) {
            const int k = ci.k;
            const int action = ((k % p.ls_every) == 0 || ci.force_check) ? ci.action : ACT_STEP;
            float rho = ci.rho, omega = ci.omega;
            chebyshev_schedule(p, k - ci.k_restart, rho, omega);
            decide_pass(ci, p, k, action, rho, omega, df_double(R));
            if (in_pass && !ci.done && ci.force_check && (ci.k % p.ls_every) != 0) ci.void_pass = 1;
        }
        if (!ci.done && __ldcg(st.active + 1) != 0) {
            ci.status = PBS_E_DEVICE_TIMEOUT;
            ci.done = 1;
        }
    }
    ci.pending = in_pass && !ci.done && !ci.void_pass;
    *dst = ci;
    if (ci.done && !was_done) atomicSub(st.active, 1);
}

}  // namespace pbs
