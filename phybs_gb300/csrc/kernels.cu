// Device kernels of the descent time step (sm_103a).
//
// One descent iteration ("pass") is two launches:
//   k_tchunk (chunks.cu) one CTA per chunk of tets: forms G, the first
//           Piola-Kirchhoff stress and the 12 corner forces of every tet; on
//           Hessian-refresh passes the 12 Jacobi-diagonal terms; on
//           line-search passes the clamped tet energies plus the node energy
//           terms, reduced in FP64.  Corner terms are summed per node in
//           shared memory into one partial per (node, chunk).  The instance's
//           last chunk to finish decides accept / reject
//           (DescentOptimize.cpp:107-128) before any node moves.  Replaces
//           computeForceKd (CUDAInterface.cu:495-568) and its 13-25 atomics
//           per tet.
//   k_node  one thread per node: adds its partials in chunk order -- no
//           atomics, so forces are bit-reproducible -- forms the gradient, takes the Jacobi step with
//           Chebyshev extrapolation (updateNodesNextIter + updateChebyshev,
//           CUDAInterface.cu:572-623) in step form, d' = (omega-1) d +
//           omega alpha delta, u' = u + d' in compensated FP32, or restores the
//           saved state after a rejection.  |g|^2 is summed per block; the
//           stopping / Chebyshev / iteration-count logic on the FP64 total
//           runs in the next pass's first chunk CTA while the other chunks
//           already evaluate their tets (or in k_settle after a run of
//           passes), so a step needs no host round trip (the reference syncs
//           every 8 iterations, CUDAInterface.cu:886-890) and no pass waits
//           on a one-CTA tail.
#include "../../include/phybs.h"
#include "node_update.cuh"
#include "pass_ctl.cuh"
#include "pass_math.cuh"
#include "phybs_internal.cuh"
#include "tet_math.cuh"

namespace pbs {

// ------------------------------------------------------------ rest state
// Dm^-1 and det Dm / 6 in FP64 from the rest positions (TetMesh.cpp:190-204,
// CUDAInterface.cu:273-325); per-tet lumped-mass share density*|vol|/4.
__global__ void k_rest(DevMesh m, const double *rest, float density, float4 *row0, float4 *row1, float4 *row2,
                       double *tmass, int *bad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.Tp) return;
    const int4 q = m.tets[t];
    if (q.x < 0) {
        row0[t] = row1[t] = row2[t] = make_float4(0.f, 0.f, 0.f, 0.f);
        tmass[t] = 0.0;
        return;
    }
    const int id[4] = {q.x, q.y, q.z, q.w};
    double p[4][3];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) p[c][d] = rest[3 * (size_t)id[c] + d];
    double Dm[9];
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int c = 0; c < 3; ++c) Dm[3 * d + c] = p[c + 1][d] - p[0][d];
    double C[9];
    cofactor3<double>(Dm, C);
    const double det = Dm[0] * C[0] + Dm[1] * C[1] + Dm[2] * C[2];
    if (!(det > 0.0) || !isfinite(det)) atomicOr(bad, 1);
    const double inv = 1.0 / det;  // Dm^-1 = C^T / det
    row0[t] = make_float4((float)(C[0] * inv), (float)(C[3] * inv), (float)(C[6] * inv), (float)(det / 6.0));
    row1[t] = make_float4((float)(C[1] * inv), (float)(C[4] * inv), (float)(C[7] * inv), 0.f);
    row2[t] = make_float4((float)(C[2] * inv), (float)(C[5] * inv), (float)(C[8] * inv), 0.f);
    tmass[t] = (double)density * fabs(det) / 6.0 * 0.25;
}

// Lumped mass by the deterministic gather (FP64), gravity = -g * mass before
// pinning (TetMesh.cpp:205), pinned mass 1e8 (TetMesh.cpp:212-216).
__global__ void k_mass(DevMesh m, const double *tmass, const int *state, float gravity, float4 *info) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    double s = 0.0;
    for (int j = m.inc_ptr[i]; j < m.inc_ptr[i + 1]; ++j) s += tmass[m.inc[j] >> 2];
    const int st = state[i];
    const float mass = (float)s;
    info[i] = make_float4(st == 1 ? 1e8f : mass, (float)(-(double)gravity * s), (float)st, mass);
}

__global__ void k_set_lame(int Tp, const float *mu, const float *lambda, int count, float4 *row1, float4 *row2,
                           const int *tet_user) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Tp) return;
    const int u = tet_user[t];
    if (u < 0) return;
    const int src = count == 1 ? 0 : u;
    row1[t].w = mu[src];
    row2[t].w = lambda[src];
}

// ------------------------------------------------------------ step control
__global__ void k_init_ctl(int n_inst, DevParams p, DevState st) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_inst) return;
    st.tcount[b] = 0;
    InstCtl c = st.ctl[b];
    c.k = 0;
    c.iters = p.max_iters;
    c.done = (c.tet_end == c.tet_begin || p.max_iters <= 0) ? 1 : 0;
    c.passes = 0;
    c.rejections = 0;
    c.converged = 0;
    c.status = PBS_OK;
    c.par = 0;
    c.action = ACT_STEP;
    c.k_restart = 0;
    c.force_check = 0;
    c.g0_fixed = 0;
    c.ws_used = 0;
    c.guess_bad = 0;
    c.counter_t = 0;
    c.counter_n = 0;
    c.pending = 0;
    c.void_pass = 0;
    c.alpha = p.alpha0;
    c.energy = 0.0;
    c.energy_old = 0.0;
    c.g0 = -1.0;
    c.r2 = -1.0;
    st.ctl[b] = c;
    st.ctl2[b] = c;  // an instance without chunks is never settled into it
    if (!c.done) atomicAdd(st.active, 1);
}

__device__ __forceinline__ const InstCtl &node_ctl(const DevMesh &m, const DevState &st, int i) {
    return st.ctl[m.nblk_inst[i / BLOCK]];
}

// DescentOptimize::initialization (DescentOptimize.cpp:35-41) /
// initDescentOpt (CUDAInterface.cu:482-493) in displacement form:
// u~ = u0 + h v, u_init = u~ + warm_start h (v - v_old); plus the external-
// force upload.  Writes parity 0 (k_init_ctl resets it).
__global__ void k_prologue(DevMesh m, DevParams p, DevState st, const float *ext_user, const int *pad2user) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const int u = pad2user[i];
    if (u < 0) return;
    const float4 hi = st.u0h[i], lo = st.u0l[i], v = st.v[i], vo = st.vold[i];
    float th[3] = {hi.x, hi.y, hi.z}, tl[3] = {lo.x, lo.y, lo.z};
    const float vv[3] = {v.x, v.y, v.z}, dv[3] = {v.x - vo.x, v.y - vo.y, v.z - vo.z};
    const float w = p.warm_start * p.h;
#pragma unroll
    for (int d = 0; d < 3; ++d) add_comp(th[d], tl[d], p.h * vv[d]);
    float xh[3] = {th[0], th[1], th[2]}, xl[3] = {tl[0], tl[1], tl[2]};
#pragma unroll
    for (int d = 0; d < 3; ++d) add_comp(xh[d], xl[d], w * dv[d]);
    st.th[i] = make_float4(th[0], th[1], th[2], 0.f);
    st.tl[i] = make_float4(tl[0], tl[1], tl[2], 0.f);
    st.uh[i] = make_float4(xh[0], xh[1], xh[2], 0.f);
    st.ul[i] = make_float4(xl[0], xl[1], xl[2], 0.f);
    st.ub[i] = make_float4(xh[0], xh[1], xh[2], 0.f);
    st.dd[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ext_user) e = make_float4(ext_user[3 * (size_t)u], ext_user[3 * (size_t)u + 1], ext_user[3 * (size_t)u + 2], 0.f);
    st.ext[i] = e;
}

// RESTART control: a guess that inverts a tet.  When prescribed nodes stop or
// reverse, x~ = x0 + h v carries the free nodes' momentum into the held layer
// and can turn tets inside out before the solve starts; the reference then
// iterates on NaN forces (its energy clamps hide the NaN).  k_guess_check
// flags an instance whose guess has a tet with det F <= 0 (or a non-finite
// one), k_guess_fallback starts it from the step's start positions instead --
// the last accepted state -- with the same residual bar.
__global__ void k_guess_check(DevMesh m, DevState st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;  // one instance per 256-tet block
    const int4 q = m.tets[t];
    if (q.x < 0) return;
    const float4 r0 = m.row0[t], r1 = m.row1[t], r2 = m.row2[t];
    const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
    Kin<float> kin;
    disp_gradient<float>(st.uh[q.x], st.uh[q.y], st.uh[q.z], st.uh[q.w], dinv, kin.G);
    kinematics(kin);
    if (!(1.0f + kin.d > 0.0f)) atomicOr(&st.ctl[m.tblk_inst[blockIdx.x]].guess_bad, 1);
}

__global__ void k_guess_fallback(DevMesh m, DevState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    if (!node_ctl(m, st, i).guess_bad) return;
    const float4 h0 = st.u0h[i], l0 = st.u0l[i];
    st.uh[i] = h0;
    st.ul[i] = l0;
    st.ub[i] = h0;
}

// v_old <- v; v = damping (u - u0) / h; u0 <- u  (DescentOptimize.cpp:183-185)
__global__ void k_epilogue(DevMesh m, DevParams p, DevState st, const int *pad2user) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    if (pad2user[i] < 0) return;
    const size_t off = (size_t)node_ctl(m, st, i).par * m.Np + i;
    const float4 hi = st.uh[off], lo = st.ul[off];
    const float4 h0 = st.u0h[i], l0 = st.u0l[i];
    const float dx = (hi.x - h0.x) + (lo.x - l0.x);
    const float dy = (hi.y - h0.y) + (lo.y - l0.y);
    const float dz = (hi.z - h0.z) + (lo.z - l0.z);
    st.vold[i] = st.v[i];
    st.v[i] = make_float4(__fdiv_rn(p.damping * dx, p.h), __fdiv_rn(p.damping * dy, p.h), __fdiv_rn(p.damping * dz, p.h),
                          0.f);
    st.hist2[i] = st.hist1[i];
    st.hist1[i] = make_float4(dx, dy, dz, 0.f);
    st.u0h[i] = hi;
    st.u0l[i] = lo;
}

// Incremental stress: the passes hold the state as its increment over the
// step's base, w = u - base as a pair (hi, lo), so that a tet's increments
// need no exact subtraction each pass (pass_math.cuh, increment_rel).  Before
// the first pass the parity-0 state u = (hi, lo) becomes (s, e + lo) with
// s + e = hi - base exactly (TwoSum); a node whose hi word is its base (a
// pinned node, or any node of the plain guess) gets (0, lo) exactly.  After
// the last pass each node's final state goes back to u = base + w, hi =
// fl(base + w hi), lo = that rounding error + w lo: bit for bit the state of
// a node that did not move.
__global__ void k_to_increment(DevMesh m, DevState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np || m.info[i].z == 2.f) return;
    const float4 uh = st.uh[i], ul = st.ul[i], ub = st.ub[i];
    float4 wh, wl;
    float e;
    two_sum(uh.x, -ub.x, wh.x, e);
    wl.x = __fadd_rn(e, ul.x);
    two_sum(uh.y, -ub.y, wh.y, e);
    wl.y = __fadd_rn(e, ul.y);
    two_sum(uh.z, -ub.z, wh.z, e);
    wl.z = __fadd_rn(e, ul.z);
    wh.w = wl.w = 0.f;
    st.uh[i] = wh;
    st.ul[i] = wl;
}

__global__ void k_from_increment(DevMesh m, DevState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np || m.info[i].z == 2.f) return;
    const size_t off = (size_t)node_ctl(m, st, i).par * m.Np + i;
    const float4 wh = st.uh[off], wl = st.ul[off], ub = st.ub[i];
    float4 uh, ul;
    float e;
    two_sum(ub.x, wh.x, uh.x, e);
    ul.x = __fadd_rn(e, wl.x);
    two_sum(ub.y, wh.y, uh.y, e);
    ul.y = __fadd_rn(e, wl.y);
    two_sum(ub.z, wh.z, uh.z, e);
    ul.z = __fadd_rn(e, wl.z);
    uh.w = ul.w = 0.f;
    st.uh[off] = uh;
    st.ul[off] = ul;
}

// ------------------------------------------------------------ one pass
// (the per-node update itself is node_update.cuh's, shared with the frame
// kernel)

// One CTA per 256-node block (one instance); NPT nodes per thread.  The
// per-step constants go to shared memory by cp.async before the
// grid-dependency wait, so no registers hold them across it.  With two nodes
// a thread the kernel is held to 85 registers: six 128-thread CTAs fit an SM,
// and the 1M-tet box's 823 node blocks run as one wave.  |g|^2 is summed in
// FP32 within the block (256 positive terms: relative error < 1e-6); the
// pass decision on the block sums (FP64 over the blocks) is taken by the
// next pass's tet kernel or by k_settle, so the kernel ends with its blocks
// and no CTA waits for the instance's last one.
template <int NPT>
__global__ void __launch_bounds__(BLOCK / NPT, NPT == 2 ? 6 : 0) k_node(DevMesh m, DevParams p, DevState st, int par) {
    constexpr int TH = BLOCK / NPT;
    __shared__ float sh[TH / 32];
    __shared__ __align__(16) float4 s_c[2][BLOCK];  // c hi (.w = M/h^2), c lo (.w = state) of the block's nodes
    const int b = blockIdx.x;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    NodeIn in[NPT];
#pragma unroll
    for (int j = 0; j < NPT; ++j) {
        const int l = threadIdx.x + j * TH, i = b * BLOCK + l;  // < Np: the grid covers the padded nodes exactly
        cp_async16(&s_c[0][l], st.ch + i);
        cp_async16(&s_c[1][l], st.cl + i);
        in[j].pa = m.pptr[i];
        in[j].pe = m.pptr[i + 1];
    }
    cp_async_commit();
    const int inst = m.nblk_inst[b];
    const size_t cur = (size_t)par * m.Np;
    pdl_launch_dependents();
    pdl_wait();  // the chunk kernel's partials and decisions are visible from here
    // the state words and the first partials go out together with the
    // instance's control block: the pass's parity is known at launch
    constexpr int NPRE = NPT == 1 ? 4 : 2;  // two nodes a thread: registers are short
    float4 fp[NPT][NPRE];
#pragma unroll
    for (int j = 0; j < NPT; ++j) {
        const int i = b * BLOCK + threadIdx.x + j * TH;
#pragma unroll
        for (int q = 0; q < NPRE; ++q) fp[j][q] = in[j].pa + q < in[j].pe ? st.part[in[j].pa + q] : z4;
        in[j].uh = st.uh[cur + i];
        in[j].ul = st.ul[cur + i];
        in[j].dd = st.dd[cur + i];
        in[j].diag = st.diag[i];
    }
    // the copy of the control block this pass's tet kernel settled
    const InstCtl *cp = ctl_buf(st, par ^ 1) + inst;
    cp_async_wait_all();  // this thread's own constants
    if (cp->done) return;
    const size_t nxt = (size_t)(1 - par) * m.Np;
    if (cp->void_pass) {
        // a forced energy check this pass did not make: the state goes on
        // unchanged to the next pass, which makes it
#pragma unroll
        for (int j = 0; j < NPT; ++j) {
            const int l = threadIdx.x + j * TH, i = b * BLOCK + l;
            if (s_c[1][l].w == 2.f) continue;
            st.uh[nxt + i] = in[j].uh;
            st.ul[nxt + i] = in[j].ul;
            st.dd[nxt + i] = in[j].dd;
        }
        return;
    }
    const int k = cp->k;
    const bool check = (k % p.ls_every) == 0 || cp->force_check;
    const int action = check ? cp->action : ACT_STEP;
    const bool do_h = (k % p.hd_every) == 0;
    float rho = cp->rho, omega = cp->omega;
    chebyshev_schedule(p, k - cp->k_restart, rho, omega);
    PassCtx ctx;
    ctx.action = action;
    ctx.do_h = do_h;
    ctx.alpha = cp->alpha;
    ctx.omega = omega;
    ctx.cur = cur;
    ctx.nxt = nxt;
    float r2 = 0.f;
#pragma unroll
    for (int j = 0; j < NPT; ++j) {
        const int l = threadIdx.x + j * TH;
        NodeConst nc;
        nc.ch = s_c[0][l];
        nc.cl = s_c[1][l];
        r2 += node_update<NPRE>(m, p, st, b * BLOCK + l, nc, in[j], fp[j], ctx);
    }
    const float sr = block_sum_f(r2, sh);
    if (threadIdx.x == 0) st.npartf[b] = sr;
}

// The pending pass decisions after the last pass of a run, one CTA an
// instance; par: the parity the next pass would have (the copy they are in).
// The result goes to st.ctl.
template <bool LOOP>
__global__ void __launch_bounds__(BLOCK) k_settle(DevParams p, DevState st, int par, LoopCtl lc) {
    pdl_wait();
    settle_pass<BLOCK>(p, st, ctl_buf(st, par) + blockIdx.x, st.ctl + blockIdx.x, false);
    if (!LOOP || threadIdx.x != 0) return;
    // each CTA's atomicSub of active[0] comes before its ticket, so the last
    // ticket sees every instance's outcome of this run
    __threadfence();
    if (atomicAdd(st.active + 3, 1) != (int)gridDim.x - 1) return;
    __threadfence();
    st.active[3] = 0;
    const int runs = __ldcg(st.active + 2) + 1;
    st.active[2] = runs;
    const int live = atomicAdd(st.active, 0);
    cudaGraphSetConditional(lc.cond, (live > 0 && runs < lc.max_runs) ? 1u : 0u);
}

// Per-step node constant b = f_el(u_base) (incremental mode, double-float /
// FP64) + body_force_scale (external + gravity), split into FP32 (hi, lo).
// k_ref_tet evaluates each tet's full neo-Hookean stress at the base (the
// step's initial guess, whose increments the passes evaluate) once, in the
// double-float type DD (about 2^-44 relative per operation; FP64 only for
// 1 / J and log1p(d)), and writes its 4 corner forces into FP64 gather slots;
// k_ref_gather sums each node's slots in FP64 in the canonical (tet, corner)
// order.
__global__ void k_ref_tet(DevMesh m, DevParams p, DevState st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.Tp) return;
    const int4 q = m.tets[t];
    if (q.x < 0) return;
    const int id[4] = {q.x, q.y, q.z, q.w};
    // the base displacements are FP32 words: their differences are exact in
    // the double-float type
    DD u[4][3];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const float4 hh = st.ub[id[a]];
        u[a][0] = DD(hh.x);
        u[a][1] = DD(hh.y);
        u[a][2] = DD(hh.z);
    }
    const float4 r0 = m.row0[t], r1 = m.row1[t], r2 = m.row2[t];
    const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
    Kin<DD> k;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
            k.G[3 * r + cc] = (u[1][r] - u[0][r]) * DD(dinv[cc]) + (u[2][r] - u[0][r]) * DD(dinv[3 + cc]) +
                              (u[3][r] - u[0][r]) * DD(dinv[6 + cc]);
    kinematics(k);
    DD P[9];
    pk1_neohookean<DD>(k, DD(r1.w), DD(r2.w), P);
    const DD sv(r0.w);
    const int4 sl = m.tslot[t];
    const int slot[4] = {sl.x, sl.y, sl.z, sl.w};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        // corner c: -svol P w_c (w_c = row c-1 of Dm^-1, w_0 = -sum of rows)
        DD w[3];
#pragma unroll
        for (int qq = 0; qq < 3; ++qq)
            w[qq] = c == 0 ? -(DD(dinv[qq]) + DD(dinv[3 + qq]) + DD(dinv[6 + qq])) : DD(dinv[3 * (c - 1) + qq]);
        double *o = st.rslot + 3 * (size_t)slot[c];
#pragma unroll
        for (int d = 0; d < 3; ++d)
            o[d] = (-sv * (P[3 * d] * w[0] + P[3 * d + 1] * w[1] + P[3 * d + 2] * w[2])).value();
    }
}

__global__ void k_ref_gather(DevMesh m, DevParams p, DevState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const float4 info = m.info[i];
    if (info.z == 2.f) {  // padding: only the node update's state word
        st.ch[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        st.cl[i] = make_float4(0.f, 0.f, 0.f, 2.f);
        return;
    }
    const float4 ex = st.ext[i];
    double b[3] = {(double)p.body_scale * ex.x, (double)p.body_scale * ((double)ex.y + info.y),
                   (double)p.body_scale * ex.z};
    if (p.incremental && info.z == 0.f) {
        for (int j = m.inc_ptr[i]; j < m.inc_ptr[i + 1]; ++j) {
            const double *o = st.rslot + 3 * (size_t)j;
#pragma unroll
            for (int d = 0; d < 3; ++d) b[d] += o[d];
        }
    }
    float hi[3], lo[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        hi[d] = (float)b[d];
        lo[d] = (float)(b[d] - (double)hi[d]);
    }
    st.bh[i] = make_float4(hi[0], hi[1], hi[2], 0.f);
    st.bl[i] = make_float4(lo[0], lo[1], lo[2], 0.f);
    // c = (M / h^2) x~ + b with the node update's FP32 M / h^2, in FP64,
    // split into (hi, lo); .w carries M / h^2 and the node's state, so that
    // the node update reads these two words and no other per-step constant.
    // Incremental stress: the passes hold u - base (k_to_increment), so
    // c = (M / h^2) (x~ - base) + b
    const float mh = info.x * p.h2inv;
    const float4 th = st.th[i], tl = st.tl[i];
    double t[3] = {(double)th.x + (double)tl.x, (double)th.y + (double)tl.y, (double)th.z + (double)tl.z};
    if (p.incremental) {
        const float4 ub = st.ub[i];
        t[0] -= (double)ub.x;
        t[1] -= (double)ub.y;
        t[2] -= (double)ub.z;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double c = (double)mh * t[d] + b[d];
        hi[d] = (float)c;
        lo[d] = (float)(c - (double)hi[d]);
    }
    st.ch[i] = make_float4(hi[0], hi[1], hi[2], mh);
    st.cl[i] = make_float4(lo[0], lo[1], lo[2], info.z);
}

// ------------------------------------------------------------ helpers
// x = X + u (u as hi + lo)
__global__ void k_pack_positions(DevMesh m, const float4 *uh, const float4 *ul, const int *pad2user, float *dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const int u = pad2user[i];
    if (u < 0) return;
    const float4 X = m.rest[i], h = uh[i], l = ul[i];
    dst[3 * (size_t)u] = state_position(X.x, h.x, l.x);
    dst[3 * (size_t)u + 1] = state_position(X.y, h.y, l.y);
    dst[3 * (size_t)u + 2] = state_position(X.z, h.z, l.z);
}

// u = x - X exactly as (hi, lo)
__device__ __forceinline__ void split_disp(float x, float X, float &hi, float &lo) { two_sum(x, -X, hi, lo); }

__global__ void k_unpack_positions(DevMesh m, const float *src, const int *pad2user, float4 *uh, float4 *ul) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const int u = pad2user[i];
    if (u < 0) {
        uh[i] = ul[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float4 X = m.rest[i];
    float h[3], l[3];
    split_disp(src[3 * (size_t)u], X.x, h[0], l[0]);
    split_disp(src[3 * (size_t)u + 1], X.y, h[1], l[1]);
    split_disp(src[3 * (size_t)u + 2], X.z, h[2], l[2]);
    uh[i] = make_float4(h[0], h[1], h[2], 0.f);
    ul[i] = make_float4(l[0], l[1], l[2], 0.f);
}

__global__ void k_scatter_positions(DevMesh m, int count, const int *ids, const float *xyz, float4 *uh, float4 *ul) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= count) return;
    const int i = ids[j];
    const float4 X = m.rest[i];
    float h[3], l[3];
    split_disp(xyz[3 * (size_t)j], X.x, h[0], l[0]);
    split_disp(xyz[3 * (size_t)j + 1], X.y, h[1], l[1]);
    split_disp(xyz[3 * (size_t)j + 2], X.z, h[2], l[2]);
    uh[i] = make_float4(h[0], h[1], h[2], 0.f);
    ul[i] = make_float4(l[0], l[1], l[2], 0.f);
}

__global__ void k_pack(int Np, const float4 *src, const int *pad2user, float *dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Np) return;
    const int u = pad2user[i];
    if (u < 0) return;
    const float4 x = src[i];
    dst[3 * (size_t)u] = x.x;
    dst[3 * (size_t)u + 1] = x.y;
    dst[3 * (size_t)u + 2] = x.z;
}

__global__ void k_unpack(int Np, const float *src, const int *pad2user, float4 *dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Np) return;
    const int u = pad2user[i];
    if (u < 0) {
        dst[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    dst[i] = make_float4(src[3 * (size_t)u], src[3 * (size_t)u + 1], src[3 * (size_t)u + 2], 0.f);
}

template <int MATERIAL>
__global__ void k_eval_tets(DevMesh m, const float4 *U, const float4 *UL, int clamp_cpu, float *tf, float *energy,
                            float *hd, unsigned int *n_fp64_svd) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.Tp) return;
    const int4 q = m.tets[t];
    float f[12] = {0}, kd[12] = {0}, e = 0.f;
    if (q.x >= 0) {
        const float4 r0 = m.row0[t], r1 = m.row1[t], r2 = m.row2[t];
        const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
        Kin<float> kin;
        disp_gradient<float>(U[q.x], U[q.y], U[q.z], U[q.w], dinv, kin.G);
        kinematics(kin);
        float P[9];
        // near inversion: the FP64 gradient from the absolute positions
        const CornerRest cr{m.rest, nullptr, {q.x, q.y, q.z, q.w}};
        auto exact = [&](double G64[9]) {
            position_gradient_exact(cr, U[q.x], U[q.y], U[q.z], U[q.w], UL[q.x], UL[q.y], UL[q.z], UL[q.w], dinv,
                                    G64);
        };
        if (MATERIAL == PBS_MATERIAL_STRETCH) {
            if (UL)
                pk1_stretch_x(kin, r1.w, r2.w, P, n_fp64_svd, exact);
            else
                pk1_stretch(kin, r1.w, r2.w, P, n_fp64_svd);
        } else if (UL) {
            pk1_neohookean_x(kin, r1.w, r2.w, P, n_fp64_svd, exact);
        } else {
            pk1_neohookean<float>(kin, r1.w, r2.w, P);
        }
        corner_forces(P, dinv, r0.w, f);
        e = clamp_energy(energy_density<float>(kin, r1.w, r2.w) * fabsf(r0.w), clamp_cpu);
        hessian_diag(kin, r1.w, r2.w, dinv, r0.w, kd);
    }
    for (int j = 0; j < 12; ++j) {
        if (tf) tf[12 * (size_t)t + j] = f[j];
        if (hd) hd[12 * (size_t)t + j] = kd[j];
    }
    if (energy) energy[t] = e;
}

__global__ void k_gather(DevMesh m, const float *tf, const float *hd, const int *pad2user, float *fo, float *ho) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const int u = pad2user[i];
    if (u < 0) return;
    float s[6] = {0, 0, 0, 0, 0, 0};
    for (int j = m.inc_ptr[i]; j < m.inc_ptr[i + 1]; ++j) {
        const int ent = m.inc[j];
        const size_t o = 12 * (size_t)(ent >> 2) + 3 * (ent & 3);
        for (int d = 0; d < 3; ++d) {
            s[d] += tf[o + d];
            s[3 + d] += hd[o + d];
        }
    }
    for (int d = 0; d < 3; ++d) {
        if (fo) fo[3 * (size_t)u + d] = s[d];
        if (ho) ho[3 * (size_t)u + d] = s[3 + d];
    }
}

// ------------------------------------------------------------ launchers
static inline int nblk(int n, int b) { return (n + b - 1) / b; }

cudaError_t launch_rest(cudaStream_t s, const DevMesh &m, const double *rest_pad, float density, float4 *row0,
                        float4 *row1, float4 *row2, double *tmass, int *bad) {
    k_rest<<<nblk(m.Tp, 128), 128, 0, s>>>(m, rest_pad, density, row0, row1, row2, tmass, bad);
    return cudaGetLastError();
}
cudaError_t launch_mass(cudaStream_t s, const DevMesh &m, const double *tmass, const int *state, float gravity,
                        float4 *info) {
    k_mass<<<nblk(m.Np, 128), 128, 0, s>>>(m, tmass, state, gravity, info);
    return cudaGetLastError();
}
cudaError_t launch_set_lame(cudaStream_t s, int Tp, const int4 *, const float *mu, const float *lambda, int count,
                            float4 *row1, float4 *row2, const int *tet_user) {
    k_set_lame<<<nblk(Tp, 256), 256, 0, s>>>(Tp, mu, lambda, count, row1, row2, tet_user);
    return cudaGetLastError();
}
cudaError_t launch_init_ctl(cudaStream_t s, int n_inst, const DevParams &p, const DevState &st) {
    k_init_ctl<<<nblk(n_inst, 128), 128, 0, s>>>(n_inst, p, st);
    return cudaGetLastError();
}
cudaError_t launch_prologue(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, const float *ext_user,
                            const int *pad2user) {
    k_prologue<<<nblk(m.Np, BLOCK), BLOCK, 0, s>>>(m, p, st, ext_user, pad2user);
    return cudaGetLastError();
}
template <int NPT>
static cudaError_t launch_node_t(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int par, bool pdl) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(m.n_nblk);
    cfg.blockDim = dim3(BLOCK / NPT);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_node<NPT>, m, p, st, par);
}
cudaError_t launch_node_only(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int par, bool pdl) {
    return m.node_npt == 2 ? launch_node_t<2>(s, m, p, st, par, pdl) : launch_node_t<1>(s, m, p, st, par, pdl);
}
cudaError_t launch_settle(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int par, bool pdl,
                          const LoopCtl *loop) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(m.n_inst);
    cfg.blockDim = dim3(BLOCK);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    if (loop) return cudaLaunchKernelEx(&cfg, k_settle<true>, p, st, par, *loop);
    return cudaLaunchKernelEx(&cfg, k_settle<false>, p, st, par, LoopCtl{});
}
// One pass of the step graph: both kernels with programmatic dependent launch.
cudaError_t launch_pass(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int material, int par) {
    cudaError_t e = launch_tet_only(s, m, p, st, material, par, true);
    if (e != cudaSuccess) return e;
    return launch_node_only(s, m, p, st, par, true);
}
cudaError_t launch_to_increment(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st) {
    if (!p.incremental) return cudaSuccess;
    k_to_increment<<<nblk(m.Np, BLOCK), BLOCK, 0, s>>>(m, st);
    return cudaGetLastError();
}
cudaError_t launch_from_increment(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st) {
    if (!p.incremental) return cudaSuccess;
    k_from_increment<<<nblk(m.Np, BLOCK), BLOCK, 0, s>>>(m, st);
    return cudaGetLastError();
}
cudaError_t launch_ref_force(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st) {
    if (p.incremental) k_ref_tet<<<nblk(m.Tp, 128), 128, 0, s>>>(m, p, st);
    k_ref_gather<<<nblk(m.Np, 128), 128, 0, s>>>(m, p, st);
    return cudaGetLastError();
}
cudaError_t launch_guess_check(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st) {
    if (p.control != PBS_CONTROL_RESTART) return cudaSuccess;
    k_guess_check<<<m.n_tblk, BLOCK, 0, s>>>(m, st);
    k_guess_fallback<<<nblk(m.Np, BLOCK), BLOCK, 0, s>>>(m, st);
    return cudaGetLastError();
}
cudaError_t launch_epilogue(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, const int *pad2user) {
    k_epilogue<<<nblk(m.Np, BLOCK), BLOCK, 0, s>>>(m, p, st, pad2user);
    return cudaGetLastError();
}
cudaError_t launch_pack_positions(cudaStream_t s, const DevMesh &m, const float4 *uh, const float4 *ul,
                                  const int *pad2user, float *dst_user) {
    k_pack_positions<<<nblk(m.Np, 256), 256, 0, s>>>(m, uh, ul, pad2user, dst_user);
    return cudaGetLastError();
}
cudaError_t launch_unpack_positions(cudaStream_t s, const DevMesh &m, const float *src_user, const int *pad2user,
                                    float4 *uh, float4 *ul) {
    k_unpack_positions<<<nblk(m.Np, 256), 256, 0, s>>>(m, src_user, pad2user, uh, ul);
    return cudaGetLastError();
}
cudaError_t launch_pack(cudaStream_t s, int Np, const float4 *src, const int *pad2user, float *dst_user) {
    k_pack<<<nblk(Np, 256), 256, 0, s>>>(Np, src, pad2user, dst_user);
    return cudaGetLastError();
}
cudaError_t launch_unpack(cudaStream_t s, int Np, const float *src_user, const int *pad2user, float4 *dst) {
    k_unpack<<<nblk(Np, 256), 256, 0, s>>>(Np, src_user, pad2user, dst);
    return cudaGetLastError();
}
cudaError_t launch_scatter_positions(cudaStream_t s, const DevMesh &m, int count, const int *ids_pad,
                                     const float *xyz, float4 *uh, float4 *ul) {
    if (count <= 0) return cudaSuccess;
    k_scatter_positions<<<nblk(count, 256), 256, 0, s>>>(m, count, ids_pad, xyz, uh, ul);
    return cudaGetLastError();
}
cudaError_t launch_eval_tets(cudaStream_t s, const DevMesh &m, const float4 *uh, int material, int clamp_cpu,
                             float *tf, float *energy, float *hd, unsigned int *n_fp64_svd, const float4 *ul) {
    if (material == PBS_MATERIAL_STRETCH)
        k_eval_tets<PBS_MATERIAL_STRETCH><<<nblk(m.Tp, 128), 128, 0, s>>>(m, uh, ul, clamp_cpu, tf, energy, hd,
                                                                          n_fp64_svd);
    else
        k_eval_tets<PBS_MATERIAL_NEOHOOKEAN><<<nblk(m.Tp, 128), 128, 0, s>>>(m, uh, ul, clamp_cpu, tf, energy, hd,
                                                                             n_fp64_svd);
    return cudaGetLastError();
}
cudaError_t launch_gather(cudaStream_t s, const DevMesh &m, const float *tf, const float *hd, const int *pad2user,
                          float *force_user, float *hd_user) {
    k_gather<<<nblk(m.Np, 128), 128, 0, s>>>(m, tf, hd, pad2user, force_user, hd_user);
    return cudaGetLastError();
}

}  // namespace pbs
