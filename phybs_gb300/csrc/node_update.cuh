// The per-node update of a descent pass (the Jacobi step with Chebyshev
// extrapolation, or the line search's restore / save), shared by the node
// kernel of the graph path (kernels.cu) and the persistent frame kernel
// (chunks.cu).
#pragma once
#include "../../include/phybs.h"
#include "pass_math.cuh"
#include "phybs_internal.cuh"
#include "tet_math.cuh"

namespace pbs {

// One component of g = M/h^2 (u_hi + u_lo) - (c_hi + c_lo) - f.
__device__ __forceinline__ float node_gradient(float uh, float ul, float mh, float ch, float cl, float f) {
    const float ph = __fmul_rn(uh, mh);
    const float pl = __fmaf_rn(uh, mh, -ph);  // ph + pl = uh * mh exactly
    return __fsub_rn(__fadd_rn(__fsub_rn(ph, ch), __fsub_rn(__fmaf_rn(ul, mh, pl), cl)), f);
}

// The inputs of one node: the state-independent ones loaded before the
// grid-dependency wait, the state words right after it.
struct NodeIn {
    int pa, pe;
    float4 uh, ul, dd, diag;
};

// Per-step node constants staged in shared memory before the grid-dependency
// wait: c = (M / h^2) x~ + b as (hi, lo) -- with incremental stress, where the
// state u is the increment over the step's base, c = (M / h^2)(x~ - base) + b
// -- with M / h^2 in ch.w and the node's state (0 free, 1 pinned, 2 padding)
// in cl.w.
struct NodeConst {
    float4 ch, cl;
};

// The instance's pass state as the node update needs it.
struct PassCtx {
    int action;
    bool do_h;
    float alpha, omega;
    size_t cur, nxt;
};

// Jacobi step with Chebyshev extrapolation (or restore / save) of node i;
// returns its |g|^2 (FP32: three positive squares).
// NPRE: partials of the node loaded together with its state words (a node of
// the 1M box touches 2-4 chunks of 256 tets; the rest cost one more round
// trip).
template <int NPRE>
__device__ __forceinline__ float node_update(const DevMesh &m, const DevParams &p, const DevState &st, int i,
                                             const NodeConst &in, const NodeIn &nn, const float4 (&f)[NPRE],
                                             const PassCtx &c) {
    float r2 = 0.f;
    const float state = in.cl.w;
    if (state == 2.f) return r2;
    const size_t nxt = c.nxt;
    const float4 uh = nn.uh, ul = nn.ul, dd = nn.dd;
    float4 nh = uh, nl = ul, nd = make_float4(0.f, 0.f, 0.f, 0.f);
    if (c.action == ACT_RESTORE) {
        // x <- x_old (DescentOptimize.cpp:116); the Chebyshev history keeps
        // x_last = x_{k-1} = u - d (the reference does not restore it), or
        // restarts it under PBS_CONTROL_RESTART
        nh = st.oh[i];
        nl = st.ol[i];
        if (state == 0.f && p.control == PBS_CONTROL_REFERENCE)
            nd = make_float4(((nh.x - uh.x) + (nl.x - ul.x)) + dd.x, ((nh.y - uh.y) + (nl.y - ul.y)) + dd.y,
                             ((nh.z - uh.z) + (nl.z - ul.z)) + dd.z, 0.f);
    } else {
        if (c.action == ACT_SAVE_STEP) {  // x_old <- x (DescentOptimize.cpp:126)
            st.oh[i] = uh;
            st.ol[i] = ul;
        }
        if (state == 0.f) {
            float fx = 0.f, fy = 0.f, fz = 0.f, hx = 0.f, hy = 0.f, hz = 0.f;
            // this node's per-chunk partial sums, in chunk order (the first
            // NPRE loaded with the state words, the rest here)
#pragma unroll
            for (int j = 0; j < NPRE; ++j) {
                fx += f[j].x;
                fy += f[j].y;
                fz += f[j].z;
            }
            for (int j = nn.pa + NPRE; j < nn.pe; ++j) {
                const float4 q = st.part[j];
                fx += q.x;
                fy += q.y;
                fz += q.z;
            }
            if (c.do_h) {
                for (int j = nn.pa; j < nn.pe; ++j) {
                    const float4 q = st.parth[j];
                    hx += q.x;
                    hy += q.y;
                    hz += q.z;
                }
            }
            const float mh = in.ch.w;  // M / h^2
            float4 D;
            if (c.do_h) {
                D = make_float4(hx + mh, hy + mh, hz + mh, 0.f);
                st.diag[i] = D;
            } else {
                D = nn.diag;
            }
            // g = M/h^2 (u - u~) - (b + sum of corner forces), b = step-start elastic
            // force (incremental mode) + body_force_scale (external + gravity),
            // formed as M/h^2 u - c - f with the per-step c = M/h^2 u~ + b (u
            // and c relative to the base with incremental stress): the
            // product M/h^2 u_hi exactly (fma), its large part cancelled
            // against c hi, the small terms added after
            const float4 ch = in.ch, cl = in.cl;
            const float gx = node_gradient(uh.x, ul.x, mh, ch.x, cl.x, fx);
            const float gy = node_gradient(uh.y, ul.y, mh, ch.y, cl.y, fy);
            const float gz = node_gradient(uh.z, ul.z, mh, ch.z, cl.z, fz);
            r2 = fmaf(gx, gx, fmaf(gy, gy, gz * gz));
            // Jacobi step delta = alpha * (g / -H) (DescentOptimize.cpp:142-150), then the
            // Chebyshev extrapolation x' = omega (x + delta - x_last) + x_last written as
            // d' = (omega - 1) d + omega delta
            const float alpha = c.alpha, omega = c.omega;
            const float dx = alpha * (gx / -D.x), dy = alpha * (gy / -D.y), dz = alpha * (gz / -D.z);
            if (omega != 1.0f)
                nd = make_float4((omega - 1.f) * dd.x + omega * dx, (omega - 1.f) * dd.y + omega * dy,
                                 (omega - 1.f) * dd.z + omega * dz, 0.f);
            else
                nd = make_float4(dx, dy, dz, 0.f);
            add_comp(nh.x, nl.x, nd.x);
            add_comp(nh.y, nl.y, nd.y);
            add_comp(nh.z, nl.z, nd.z);
        }
    }
    st.uh[nxt + i] = nh;
    st.ul[nxt + i] = nl;
    st.dd[nxt + i] = nd;
    return r2;
}

}  // namespace pbs
