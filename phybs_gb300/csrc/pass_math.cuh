// Per-tet force evaluation shared by the pass kernels and the warm start.
#pragma once
#include "../../include/phybs.h"
#include "phybs_internal.cuh"
#include "tet_math.cuh"

namespace pbs {

// Programmatic dependent launch between the two kernels of a pass (and from
// one pass to the next) inside the step graph.  A kernel lets its successor
// launch as soon as all of its own CTAs are running, so the successor's CTAs
// fill the SMs the tail wave leaves idle and issue their state-independent
// loads; pdl_wait() then blocks until this grid's predecessor has completed and
// its writes are visible.  Every read of the predecessor's outputs and every
// write comes after pdl_wait().  Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Asynchronous global -> shared copies (completion waited for by the hardware:
// no polling loop).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
// One 128-bit shared-memory access for a float4 whose .w may be unused: a
// node word or a corner-force slot is then one LSU request, not two or three.
__device__ __forceinline__ float4 lds128(const float4 *p) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "r"((unsigned)__cvta_generic_to_shared(p)));
    return v;
}
__device__ __forceinline__ void sts128(float4 *p, float x, float y, float z, float w = 0.f) {
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"((unsigned)__cvta_generic_to_shared(p)), "f"(x),
                 "f"(y), "f"(z), "f"(w)
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Deterministic block sum: fixed shuffle tree per warp, then warp 0 sums the
// warp totals in warp order.  Result valid in thread 0; sh holds one double
// per warp.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// Energy terms of one free node: 1/2 m |u - u~|^2 / h^2 - g_y u_y - f_ext . u
// (DescentOptimize.cpp:73-87 / CUDAInterface.cu:589-597), measured from the
// rest shape so that no large constant rides along in the sum.
__device__ __forceinline__ double node_energy(const DevState &st, const float4 &info, const float4 &uh,
                                              const float4 &ul, int i, float h2inv) {
    const float4 th = st.th[i], tl = st.tl[i], ex = st.ext[i];
    const float dx = (uh.x - th.x) + (ul.x - tl.x);
    const float dy = (uh.y - th.y) + (ul.y - tl.y);
    const float dz = (uh.z - th.z) + (ul.z - tl.z);
    const double uy = (double)uh.y + ul.y;
    return 0.5 * (double)info.x * ((double)dx * dx + (double)dy * dy + (double)dz * dz) * (double)h2inv -
           (double)info.y * uy - ((double)ex.x * ((double)uh.x + ul.x) + (double)ex.y * uy + (double)ex.z * ((double)uh.z + ul.z));
}

// Deterministic FP32 block sum (fixed shuffle tree, then warp 0 over the warp
// totals); result valid in thread 0.
__device__ __forceinline__ float block_sum_f(float v, float *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    float r = 0.f;
    if (w == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;
}

// Deterministic double-float block sum (fixed shuffle tree, then warp 0 over
// the warp totals in warp order); result valid in thread 0.  sh: 2 floats a
// warp.
__device__ __forceinline__ DFloat block_sum_df(DFloat v, float2 *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h = __shfl_down_sync(0xffffffffu, v.hi, o), l = __shfl_down_sync(0xffffffffu, v.lo, o);
        v = df_add(v, DFloat{h, l});
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = make_float2(v.hi, v.lo);
    __syncthreads();
    DFloat r{0.f, 0.f};
    if (w == 0) {
        if (lane < (int)(blockDim.x >> 5)) r = DFloat{sh[lane].x, sh[lane].y};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float h = __shfl_down_sync(0xffffffffu, r.hi, o), l = __shfl_down_sync(0xffffffffu, r.lo, o);
            r = df_add(r, DFloat{h, l});
        }
    }
    return r;
}

// node_energy in double-float: the same terms, FP32 operations only.  With
// base (incremental stress) (uh, ul) is the increment w over it: u = base +
// w, u - u~ = (base - u~hi) + (w hi + (w lo - u~lo)).
__device__ __forceinline__ DFloat node_energy_df(const DevState &st, const float4 &info, const float4 &uh,
                                                 const float4 &ul, int i, float h2inv,
                                                 const float4 *base = nullptr) {
    const float4 th = st.th[i], tl = st.tl[i], ex = st.ext[i];
    float dx, dy, dz;
    DFloat ux{uh.x, ul.x}, uy{uh.y, ul.y}, uz{uh.z, ul.z};
    if (base) {
        const float4 b = base[i];
        dx = (b.x - th.x) + (uh.x + (ul.x - tl.x));
        dy = (b.y - th.y) + (uh.y + (ul.y - tl.y));
        dz = (b.z - th.z) + (uh.z + (ul.z - tl.z));
        ux = df_add(DFloat{b.x, 0.f}, ux);
        uy = df_add(DFloat{b.y, 0.f}, uy);
        uz = df_add(DFloat{b.z, 0.f}, uz);
    } else {
        dx = (uh.x - th.x) + (ul.x - tl.x);
        dy = (uh.y - th.y) + (ul.y - tl.y);
        dz = (uh.z - th.z) + (ul.z - tl.z);
    }
    const DFloat sq = df_add(df_add(df_prod(dx, dx), df_prod(dy, dy)), df_prod(dz, dz));
    DFloat k = df_prod(info.x, h2inv);
    k.hi *= 0.5f;  // exact
    k.lo *= 0.5f;
    DFloat e = df_mul(k, sq);
    e = df_add(e, df_mul(uy, -info.y));
    e = df_add(e, df_mul(ux, -ex.x));
    e = df_add(e, df_mul(uy, -ex.y));
    e = df_add(e, df_mul(uz, -ex.z));
    return e;
}

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

// Corner values: x = u hi word, l = u lo word, a = base (hi) of the 4 corners.
// INC (compile time): the incremental neo-Hookean form, where l carries the
// corner's increment u - base less a reference common to the tet, formed once
// per node (increment_rel from the passes' increment state in the chunk
// kernels, node_increment_rel from a (hi, lo) state elsewhere), and x is
// unused; without INC, a is unused.  cr locates the corners' rest positions
// for the FP64 stress of a near-inverted tet (full stress only).  DEFER:
// leave that stress out (f is then not the tet's) and return whether the tet
// needs it, for a caller that forms it after its loop.  KIN = false: with
// INC, kin holds only d and lnJ (a pass that needs neither the energy nor the
// Jacobi diagonal; a loop without them also needs fewer registers).
template <int MATERIAL, bool INC, bool DEFER = false, bool KIN = true>
__device__ __forceinline__ bool pass_forces_c(const float4 &x0, const float4 &x1, const float4 &x2, const float4 &x3,
                                              const float4 &l0, const float4 &l1, const float4 &l2, const float4 &l3,
                                              const float4 &a0, const float4 &a1, const float4 &a2, const float4 &a3,
                                              const float dinv[9], float svol, float mu, float lambda, Kin<float> &kin,
                                              float f[12], const CornerRest &cr) {
    float P[9];
    bool exact = false;
    if (MATERIAL != PBS_MATERIAL_STRETCH && INC) {
        Kin<float> k0;
        disp_gradient<float>(a0, a1, a2, a3, dinv, k0.G);
        kinematics(k0);
        float dG[9];
        disp_gradient<float>(l0, l1, l2, l3, dinv, dG);
        pk1_neohookean_inc<KIN>(k0, dG, mu, lambda, kin, P);
    } else {
        // Du = (u_j,hi - u_0,hi) + (u_j,lo - u_0,lo)
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        disp_gradient<float>(z, f4add(f4sub(x1, x0), f4sub(l1, l0)), f4add(f4sub(x2, x0), f4sub(l2, l0)),
                             f4add(f4sub(x3, x0), f4sub(l3, l0)), dinv, kin.G);
        kinematics(kin);
        // near inversion (det F < 1e-3, or a stretch-material tet whose FP32
        // spectrum has sigma_3 < 0.3): the FP64 stress from the absolute positions
        exact = 1.0f + kin.d < 1e-3f;
        if (!exact) {
            if (MATERIAL == PBS_MATERIAL_STRETCH) exact = !stretch_pk1<float>(kin.G, mu, lambda, P);
            else pk1_neohookean<float>(kin, mu, lambda, P);
        }
        if (exact && !DEFER)
            pk1_exact_fp64(MATERIAL, cr, x0, x1, x2, x3, l0, l1, l2, l3,
                           make_float4(dinv[0], dinv[1], dinv[2], 0.f), make_float4(dinv[3], dinv[4], dinv[5], 0.f),
                           make_float4(dinv[6], dinv[7], dinv[8], 0.f), mu, lambda, P);
    }
    corner_forces(P, dinv, svol, f);
    return exact;
}

// The staged increment of a node in a pass: the state holds w = u - base as
// (w hi, w lo) (k_to_increment), and a chunk stages (w hi - r) + w lo with r
// the w hi of its local node 0.  The tets use only differences of
// increments, which r leaves unchanged; w hi - r is exact wherever the two
// are within a factor 2 of each other, so an increment that is large and
// nearly the same across a chunk (a soft body that moves far in one frame)
// keeps the small differences dG is made of.  (One rounded FP32 increment
// (u hi - base) + u lo a node lost them there, and the residual of such
// frames stalled near 1.5e-4 of its initial value.)
__device__ __forceinline__ float4 increment_rel(const float4 &wh, const float4 &wl, const float4 &r) {
    return make_float4(__fadd_rn(__fsub_rn(wh.x, r.x), wl.x), __fadd_rn(__fsub_rn(wh.y, r.y), wl.y),
                       __fadd_rn(__fsub_rn(wh.z, r.z), wl.z), 0.f);
}

// Outside the passes (the state as u = (hi, lo)): a reference for
// node_increment_rel, fl(u hi - base) of one node (a tet's corner 0).  Its
// rounding does not matter: any constant common to the nodes would do.
__device__ __forceinline__ float4 increment_ref(const float4 &uh, const float4 &ub) {
    return make_float4(__fsub_rn(uh.x, ub.x), __fsub_rn(uh.y, ub.y), __fsub_rn(uh.z, ub.z), 0.f);
}

// One component: (s - r) + (e + lo), s + e = hi - base exactly (TwoSum).
__device__ __forceinline__ float increment_rel1(float hi, float lo, float base, float r) {
    float s, e;
    two_sum(hi, -base, s, e);
    return __fadd_rn(__fsub_rn(s, r), __fadd_rn(e, lo));
}

// The increment u - base = (u hi - base) + u lo of a node, less a reference
// r common to the nodes that are differenced together (increment_ref), and
// rounded once.  The tets evaluate only differences of increments, which r
// leaves unchanged.  An increment that is large and nearly the same across a
// chunk (a soft body that moves far in one frame) then keeps the small
// differences dG is made of: u hi - base is split exactly into s + e, and
// s - r is exact wherever the two are within a factor 2 of each other, which
// is where the cancellation is.  With one rounded FP32 increment a node the
// residual of such frames stalled near 1.5e-4 of its initial value.
__device__ __forceinline__ float4 node_increment_rel(const float4 &uh, const float4 &ul, const float4 &ub,
                                                     const float4 &r) {
    return make_float4(increment_rel1(uh.x, ul.x, ub.x, r.x), increment_rel1(uh.y, ul.y, ub.y, r.y),
                       increment_rel1(uh.z, ul.z, ub.z, r.z), 0.f);
}

template <int MATERIAL>
__device__ __forceinline__ void pass_forces_v(const DevParams &p, const float4 &x0, const float4 &x1, const float4 &x2,
                                              const float4 &x3, const float4 &l0, const float4 &l1, const float4 &l2,
                                              const float4 &l3, const float4 &a0, const float4 &a1, const float4 &a2,
                                              const float4 &a3, const float dinv[9], float svol, float mu,
                                              float lambda, Kin<float> &kin, float f[12], const CornerRest &cr) {
    if (MATERIAL != PBS_MATERIAL_STRETCH && p.incremental)
        pass_forces_c<MATERIAL, true>(x0, x1, x2, x3, l0, l1, l2, l3, a0, a1, a2, a3, dinv, svol, mu, lambda, kin, f,
                                      cr);
    else
        pass_forces_c<MATERIAL, false>(x0, x1, x2, x3, l0, l1, l2, l3, a0, a1, a2, a3, dinv, svol, mu, lambda, kin, f,
                                       cr);
}

// rest: the rest positions by padded node id (q's ids)
template <int MATERIAL>
__device__ __forceinline__ void pass_forces(const DevParams &p, const float4 *U, const float4 *UL, const float4 *U0,
                                            const int4 &q, const float dinv[9], float svol, float mu, float lambda,
                                            Kin<float> &kin, float f[12], const float4 *rest) {
    const CornerRest cr{rest, nullptr, {q.x, q.y, q.z, q.w}};
    const bool inc = MATERIAL != PBS_MATERIAL_STRETCH && p.incremental;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 x0 = U[q.x], x1 = U[q.y], x2 = U[q.z], x3 = U[q.w];
    const float4 l0 = UL[q.x], l1 = UL[q.y], l2 = UL[q.z], l3 = UL[q.w];
    const float4 a0 = inc ? U0[q.x] : z, a1 = inc ? U0[q.y] : z, a2 = inc ? U0[q.z] : z, a3 = inc ? U0[q.w] : z;
    if (inc) {
        // increments relative to corner 0's
        const float4 r = increment_ref(x0, a0);
        pass_forces_v<MATERIAL>(p, x0, x1, x2, x3, node_increment_rel(x0, l0, a0, r),
                                node_increment_rel(x1, l1, a1, r), node_increment_rel(x2, l2, a2, r),
                                node_increment_rel(x3, l3, a3, r), a0, a1, a2, a3, dinv, svol, mu, lambda, kin, f, cr);
    }
    else
        pass_forces_v<MATERIAL>(p, x0, x1, x2, x3, l0, l1, l2, l3, a0, a1, a2, a3, dinv, svol, mu, lambda, kin, f,
                                cr);
}

}  // namespace pbs
