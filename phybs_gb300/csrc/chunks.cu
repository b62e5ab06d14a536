// The per-tet kernel of a descent pass, on chunks of tets.
//
// A chunk is a run of at most chunk_tets tets of one instance, consecutive in
// the Morton order of their centroids, that touches at most chunk_nodes nodes
// (the handle's chunk shape: CHUNK_TETS / CHUNK_NODES / CHUNK_THREADS, or what
// pbs_autotune picked).  One CTA per chunk:
//   1. stages the chunk's nodes (u hi, u lo and the force base) in shared
//      memory: each node is read once per chunk instead of once per corner;
//   2. evaluates its tets (one thread per tet, chunk tets / CTA threads tets
//      a thread), streaming the per-tet rows in chunk order, and writes the 12
//      corner forces to shared-memory slots, where a node's slots are
//      contiguous in (tet, corner) order;
//   3. sums each node's slots in that order into one partial per (node,
//      chunk), written to part[] at the node's place for this chunk.
// The node kernel adds a node's partials in chunk order.  No atomics touch a
// force, so results are bit-reproducible run to run, and instances are
// chunked on their own, so a packed batch gives each instance the bits it gets
// alone.  Against one thread per tet writing 4 global slots, this moves the
// corner forces through shared memory instead of HBM (64 B written and read
// back per tet per pass) and replaces 4 gathers of 3 node words per tet with
// one staged read per touched node.
//
// On line-search passes the CTA also adds the clamped tet energies and its
// share of the instance's node energy terms (FP64, fixed order); the
// instance's last chunk to finish decides accept / reject
// (DescentOptimize.cpp:107-128) before any node moves.
//
// The pass decision of the previous node update (residual test, Chebyshev
// state, caps) is taken by the instance's first chunk CTA (settle_pass) from
// one control-block copy into the other, while every CTA runs on its
// foreseen outcome (pass_view): the next k, or work that goes unused when the
// instance stopped.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <utility>
#include <vector>

#include "../../include/phybs.h"
#include "node_update.cuh"
#include "pass_ctl.cuh"
#include "pass_math.cuh"
#include "phybs_internal.cuh"
#include "tet_math.cuh"

namespace pbs {

// ------------------------------------------------------------ host: layout
namespace {

uint32_t spread10(uint32_t v) {  // 10 bits -> every third bit of 30
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

}  // namespace

void build_chunks(int Np, const std::vector<int4> &tets, const std::vector<double> &rest, std::vector<InstCtl> &ctl,
                  int chunk_tets, int chunk_nodes, ChunkLayout &out) {
    out = ChunkLayout();
    std::vector<int> stamp(Np, -1), lidx(Np, 0), n_part(Np, 0);
    std::vector<std::pair<uint32_t, int>> order;
    std::vector<int> ctets, lnodes, scount, lnode_all, lsptr_all, lsend_all;
    int tq = 0;
    for (size_t b = 0; b < ctl.size(); ++b) {
        InstCtl &C = ctl[b];
        C.cblk_begin = (int)out.chunk.size();
        double lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::numeric_limits<double>::max();
            hi[d] = -std::numeric_limits<double>::max();
        }
        auto centroid = [&](int t, double c[3]) {
            const int *q = &tets[t].x;
            for (int d = 0; d < 3; ++d)
                c[d] = 0.25 * (rest[3 * (size_t)q[0] + d] + rest[3 * (size_t)q[1] + d] + rest[3 * (size_t)q[2] + d] +
                               rest[3 * (size_t)q[3] + d]);
        };
        for (int t = C.tet_begin; t < C.tet_end; ++t) {
            double c[3];
            centroid(t, c);
            for (int d = 0; d < 3; ++d) {
                lo[d] = std::min(lo[d], c[d]);
                hi[d] = std::max(hi[d], c[d]);
            }
        }
        order.clear();
        for (int t = C.tet_begin; t < C.tet_end; ++t) {
            double c[3];
            centroid(t, c);
            uint32_t code = 0;
            for (int d = 0; d < 3; ++d) {
                const double ext = hi[d] - lo[d];
                const double f = ext > 0.0 ? (c[d] - lo[d]) / ext : 0.0;
                const uint32_t v = (uint32_t)std::min(1023.0, std::max(0.0, std::floor(f * 1024.0)));
                code |= spread10(v) << d;
            }
            order.emplace_back(code, t);
        }
        std::sort(order.begin(), order.end());
        if (order.empty()) {  // an instance without tets still needs a CTA for its line-search decisions
            out.chunk.push_back(make_int4(tq, 0, (int)lnode_all.size(), 0));
            out.chunk_inst.push_back((int)b);
        }
        size_t pos = 0;
        while (pos < order.size()) {
            const int cid = (int)out.chunk.size();
            ctets.clear();
            lnodes.clear();
            while (pos < order.size() && (int)ctets.size() < chunk_tets) {
                const int t = order[pos].second;
                const int *q = &tets[t].x;
                int add = 0;
                for (int c = 0; c < 4; ++c) {
                    bool seen = stamp[q[c]] == cid;
                    for (int c2 = 0; c2 < c && !seen; ++c2) seen = q[c2] == q[c];
                    add += !seen;
                }
                if ((int)lnodes.size() + add > chunk_nodes) break;
                for (int c = 0; c < 4; ++c)
                    if (stamp[q[c]] != cid) {
                        stamp[q[c]] = cid;
                        lnodes.push_back(q[c]);
                    }
                ctets.push_back(t);
                ++pos;
            }
            // local nodes in ascending id order: a warp's node gathers then
            // share sectors (ordering them by corner count, which evens out the
            // partial-sum loops, measured slower)
            std::sort(lnodes.begin(), lnodes.end());
            const int nl = (int)lnodes.size(), nt = (int)ctets.size();
            for (int j = 0; j < nl; ++j) lidx[lnodes[j]] = j;
            scount.assign(nl + 1, 0);
            for (int t : ctets)
                for (int c = 0; c < 4; ++c) scount[lidx[(&tets[t].x)[c]] + 1]++;
            for (int j = 0; j < nl; ++j) scount[j + 1] += scount[j];
            const int l0 = (int)lnode_all.size();
            for (int j = 0; j < nl; ++j) {
                lnode_all.push_back(lnodes[j]);
                lsptr_all.push_back(scount[j]);
                lsend_all.push_back(scount[j + 1]);
                n_part[lnodes[j]]++;
            }
            for (int lt = 0; lt < nt; ++lt) {
                const int *q = &tets[ctets[lt]].x;
                unsigned loc[4], sl[4];
                for (int c = 0; c < 4; ++c) {
                    loc[c] = (unsigned)lidx[q[c]];
                    sl[c] = (unsigned)scount[loc[c]]++;
                }
                out.qcor.push_back(make_uint4(loc[0] | loc[1] << 16, loc[2] | loc[3] << 16, sl[0] | sl[1] << 16,
                                              sl[2] | sl[3] << 16));
                out.qperm.push_back(ctets[lt]);
            }
            out.chunk.push_back(make_int4(tq, nt, l0, nl));
            out.chunk_inst.push_back((int)b);
            out.max_local = std::max(out.max_local, nl);
            tq += nt;
        }
        C.cblk_end = (int)out.chunk.size();
    }
    // node -> partials, in chunk order
    out.pptr.assign(Np + 1, 0);
    for (int i = 0; i < Np; ++i) out.pptr[i + 1] = out.pptr[i] + n_part[i];
    std::vector<int> fill(out.pptr.begin(), out.pptr.end() - 1);
    out.lmeta.resize(lnode_all.size());
    for (size_t j = 0; j < lnode_all.size(); ++j)
        out.lmeta[j] = make_int4(lnode_all[j], lsptr_all[j], lsend_all[j], fill[lnode_all[j]]++);
}

// ------------------------------------------------------------ device
__global__ void k_pass_rows(int T, const int *qperm, const float4 *row0, const float4 *row1, const float4 *row2,
                            float4 *q0, float4 *q1, float4 *q2) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= T) return;
    const int t = qperm[j];
    q0[j] = row0[t];
    q1[j] = row1[t];
    q2[j] = row2[t];
}

// Corner ids of a pass tet from its packed record.
__device__ __forceinline__ void unpack_cor(const uint4 &w, int loc[4], int slot[4]) {
    loc[0] = (int)(w.x & 0xffffu);
    loc[1] = (int)(w.x >> 16);
    loc[2] = (int)(w.y & 0xffffu);
    loc[3] = (int)(w.y >> 16);
    slot[0] = (int)(w.z & 0xffffu);
    slot[1] = (int)(w.z >> 16);
    slot[2] = (int)(w.w & 0xffffu);
    slot[3] = (int)(w.w >> 16);
}

// One chunk as its tet loop reads it: node words staged in shared memory;
// per-tet rows and corner records in shared memory or at the chunk's place in
// the pass arrays.
struct ChunkView {
    const float4 *uh, *ul, *ub;
    const float4 *r0, *r1, *r2;
    const uint4 *cor;
    const int4 *meta;    // local-node records (their global ids locate the rest positions)
    const float4 *rest;  // rest positions, for the FP64 stress of a near-inverted tet
};

// Corner forces of the chunk's tets into the slots; on line-search passes
// returns the thread's sum of clamped tet energies.
// The node words of a tet's four corners from the chunk's shared-memory
// staging (one 128-bit access each): x = u hi (full stress) or nothing (the
// incremental form), l = u lo or the increment relative to the chunk's
// reference node, a = the base (incremental).
template <bool INC>
__device__ __forceinline__ void corner_words(const ChunkView &v, const int lc[4], float4 x[4], float4 l[4],
                                             float4 a[4]) {
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        x[c] = INC ? z4 : lds128(v.uh + lc[c]);
        l[c] = lds128(v.ul + lc[c]);
        a[c] = INC ? lds128(v.ub + lc[c]) : z4;
    }
}

// A near-inverted tet (full stress) gets its FP32 forces here and a mark in
// its corner-0 slot's .w; *any_exact tells whether the thread marked one.
// CHECK: a line-search pass (the tet energies too); the loop is compiled once
// with and once without them.
template <int MATERIAL, int THREADS, bool INC, bool CHECK>
__device__ __forceinline__ DFloat chunk_forces(const DevParams &p, const ChunkView &v, int nt, float4 *sf,
                                               bool *any_exact) {
    DFloat e{0.f, 0.f};
    bool any = false;
    for (int lt = threadIdx.x; lt < nt; lt += THREADS) {
        const float4 r0 = v.r0[lt], r1 = v.r1[lt], r2 = v.r2[lt];
        int lc[4], sl[4];
        unpack_cor(v.cor[lt], lc, sl);
        const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
        Kin<float> kin;
        float f[12];
        float4 x[4], l[4], a[4];
        corner_words<INC>(v, lc, x, l, a);
        const bool ex = pass_forces_c<MATERIAL, INC, true, CHECK>(
            x[0], x[1], x[2], x[3], l[0], l[1], l[2], l[3], a[0], a[1], a[2], a[3], dinv, r0.w, r1.w, r2.w, kin, f,
            CornerRest{v.rest, v.meta, {lc[0], lc[1], lc[2], lc[3]}});
        any |= ex;
#pragma unroll
        for (int cc = 0; cc < 4; ++cc)
            sts128(sf + sl[cc], f[3 * cc], f[3 * cc + 1], f[3 * cc + 2], cc == 0 && ex ? 1.f : 0.f);
        if (CHECK)
            e = df_add(e, search_energy(energy_density<float>(kin, r1.w, r2.w) * fabsf(r0.w), p.clamp_cpu,
                                        p.control == PBS_CONTROL_RESTART));
    }
    *any_exact = any;
    return e;
}

// The FP64 stress of the chunk's marked (near-inverted) tets, into their
// slots.  After the tet loop rather than inside it: the loop then carries no
// call, and keeps its registers.
template <int MATERIAL, int THREADS>
__device__ __forceinline__ void chunk_exact(const ChunkView &v, int nt, float4 *sf) {
    for (int lt = threadIdx.x; lt < nt; lt += THREADS) {
        int lc[4], sl[4];
        unpack_cor(v.cor[lt], lc, sl);
        if (lds128(sf + sl[0]).w == 0.f) continue;
        const float4 r0 = v.r0[lt], r1 = v.r1[lt], r2 = v.r2[lt];
        const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
        float4 x[4], l[4], a[4];
        corner_words<false>(v, lc, x, l, a);
        float P[9], f[12];
        pk1_exact_fp64(MATERIAL, CornerRest{v.rest, v.meta, {lc[0], lc[1], lc[2], lc[3]}}, x[0], x[1], x[2], x[3],
                       l[0], l[1], l[2], l[3], r0, r1, r2, r1.w, r2.w, P);
        corner_forces(P, dinv, r0.w, f);
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) sts128(sf + sl[cc], f[3 * cc], f[3 * cc + 1], f[3 * cc + 2]);
    }
}

// chunk_forces, then the FP64 stress of a chunk that has a near-inverted tet;
// every thread sees the finished slots on return.
template <int MATERIAL, int THREADS, bool INC>
__device__ __forceinline__ DFloat chunk_forces_all(const DevParams &p, const ChunkView &v, int nt, bool check,
                                                   float4 *sf) {
    bool ex;
    const DFloat e = check ? chunk_forces<MATERIAL, THREADS, INC, true>(p, v, nt, sf, &ex)
                           : chunk_forces<MATERIAL, THREADS, INC, false>(p, v, nt, sf, &ex);
    if (INC) {
        __syncthreads();
    } else if (__syncthreads_or(ex)) {
        chunk_exact<MATERIAL, THREADS>(v, nt, sf);
        __syncthreads();
    }
    return e;
}

// Jacobi-diagonal refresh: the same slots carry the 12 diagonal terms.
template <int MATERIAL, int THREADS, bool INC>
__device__ __forceinline__ void chunk_hdiag(const ChunkView &v, int nt, float4 *sf) {
    for (int lt = threadIdx.x; lt < nt; lt += THREADS) {
        const float4 r0 = v.r0[lt], r1 = v.r1[lt], r2 = v.r2[lt];
        int lc[4], sl[4];
        unpack_cor(v.cor[lt], lc, sl);
        const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
        Kin<float> kin;
        float f[12], kd[12];
        float4 x[4], l[4], a[4];
        corner_words<INC>(v, lc, x, l, a);
        // only the kinematics are used here (no FP64 stress needed)
        pass_forces_c<MATERIAL, INC, true>(x[0], x[1], x[2], x[3], l[0], l[1], l[2], l[3], a[0], a[1], a[2], a[3],
                                           dinv, r0.w, r1.w, r2.w, kin, f,
                                           CornerRest{v.rest, v.meta, {lc[0], lc[1], lc[2], lc[3]}});
        hessian_diag(kin, r1.w, r2.w, dinv, r0.w, kd);
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) sts128(sf + sl[cc], kd[3 * cc], kd[3 * cc + 1], kd[3 * cc + 2]);
    }
}

// Sums every local node's slots (in slot order) into its partial for this
// chunk.  meta: the chunk's local-node records (shared or global memory).
template <int THREADS>
__device__ __forceinline__ void chunk_partials(const int4 *meta, int nl, const float4 *sf, float4 *out) {
    for (int j = threadIdx.x; j < nl; j += THREADS) {
        const int4 md = meta[j];
        float fx = 0.f, fy = 0.f, fz = 0.f;
        for (int s = md.y; s < md.z; ++s) {
            const float4 q = lds128(sf + s);
            fx += q.x;
            fy += q.y;
            fz += q.z;
        }
        out[md.w] = make_float4(fx, fy, fz, 0.f);
    }
}

// Line-search pass: adds the chunk's share of the instance's node energy terms
// to the thread's tet energies e, stores the chunk's {sum e, sum e^2}, and in
// the instance's last chunk to finish sums the chunks in order and decides
// accept / reject (DescentOptimize.cpp:107-128) on dst, the control-block copy
// the pass's node kernel reads (its first chunk settled the last pass into
// it before counting itself in).  The sums run in double-float (e) and FP32
// (e^2, a noise scale), the chunk totals and their sum in FP64.  Called by
// every thread of the CTA; *is_last is a shared word.
template <int THREADS>
__device__ __forceinline__ void chunk_line_search(const DevMesh &m, const DevParams &p, const DevState &st, int c,
                                                  int inst, int par, int k, size_t cur, DFloat e, double *sh,
                                                  int *is_last) {
    __shared__ float2 shf[THREADS / 32];
    // (formed here, not carried through the tet loop: registers are short)
    const InstCtl *src = ctl_buf(st, par) + inst;
    InstCtl *dst = ctl_buf(st, par ^ 1) + inst;
    unsigned int *cnt = st.tcount + inst;
    __shared__ float shs[THREADS / 32];
    float e2 = e.hi * e.hi;
    const int cb = src->cblk_begin, ce = src->cblk_end;
    {
        const int nb = ce - cb;
        const float4 *U = st.uh + cur;
        for (int i = src->node_begin + (c - cb) * THREADS + threadIdx.x; i < src->node_end; i += nb * THREADS) {
            const float4 info = m.info[i];
            if (info.z != 0.f) continue;
            const DFloat en = node_energy_df(st, info, U[i], st.ul[cur + i], i, p.h2inv, p.incremental ? st.ub : nullptr);
            e = df_add(e, en);
            e2 = fmaf(en.hi, en.hi, e2);
        }
    }
    const DFloat se = block_sum_df(e, shf);
    const float se2 = block_sum_f(e2, shs);
    if (threadIdx.x == 0) {
        st.cpart[c] = make_double2(df_double(se), (double)se2);
        __threadfence();
        const unsigned int prev = atomicAdd(cnt, 1u);
        *is_last = (prev == (unsigned int)(ce - cb - 1));
    }
    __syncthreads();
    if (!*is_last) return;
    __threadfence();
    // the instance's last chunk: fixed-order sums (each thread adds its chunks
    // in ascending order, then the block tree), then accept / reject.  The
    // partials are loaded eight at a time ahead of their additions: this tail
    // runs on one CTA while the rest of the GPU waits, and one load round trip
    // per partial made it several microseconds
    constexpr int U = 8;
    double ea = 0.0, eb = 0.0;
    for (int j0 = cb + threadIdx.x; j0 < ce; j0 += U * THREADS) {
        double2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = j0 + u * THREADS;
            v[u] = j < ce ? __ldcg(st.cpart + j) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            ea += v[u].x;
            eb += v[u].y;
        }
    }
    const double E = block_sum(ea, sh);
    const double E2 = block_sum(eb, sh);
    if (threadIdx.x != 0) return;
    *cnt = 0;
    // one load, updates in registers, one store; an instance the settled
    // decision stopped keeps its control block (this pass ran on speculation)
    InstCtl ci = load_ctl_cg(dst);
    if (ci.done) return;
    decide_line_search(ci, p, k, E, E2);
    *dst = ci;
    if (ci.done) atomicSub(st.active, 1);
}

// The whole of one chunk once its node words (and, with STAGE, its rows and
// records) are in shared memory: forces, partials, the Jacobi diagonal every
// hd_every passes, and the line-search tail.
template <int MATERIAL, int THREADS, bool INC>
__device__ __forceinline__ void chunk_body(const DevMesh &m, const DevParams &p, const DevState &st, int c,
                                           int inst, int par, const PassView &pv, size_t cur, const ChunkView &v,
                                           const int4 *meta, int nt, int nl, float4 *sf, double *sh,
                                           int *is_last) {
    const DFloat e = chunk_forces_all<MATERIAL, THREADS, INC>(p, v, nt, pv.check, sf);
    chunk_partials<THREADS>(meta, nl, sf, st.part);
    if (pv.do_h) {
        __syncthreads();
        chunk_hdiag<MATERIAL, THREADS, INC>(v, nt, sf);
        __syncthreads();
        chunk_partials<THREADS>(meta, nl, sf, st.parth);
    }
    // the instance's first chunk takes the last pass's pending decision after
    // its own tets (the other chunks run on its foreseen outcome without
    // waiting), and before it counts itself into a line search
    const InstCtl *src = ctl_buf(st, par) + inst;
    if (c == src->cblk_begin) settle_pass<THREADS>(p, st, src, ctl_buf(st, par ^ 1) + inst, true);
    if (pv.check) chunk_line_search<THREADS>(m, p, st, c, inst, par, pv.k, cur, e, sh, is_last);
}

// One CTA per chunk.  STAGE: every thread first issues asynchronous copies of
// its tets' rows and corner records and of the chunk's local-node records into
// shared memory -- before the grid-dependency wait, since they are constant --
// and of the chunk's node words after it; one wait then covers all of them,
// instead of one global round trip per tet inside the loop.
#ifndef PBS_INC_THREADS_PER_SM
#define PBS_INC_THREADS_PER_SM 1024
#endif
// Register budget of the neo-Hookean variants: 64 a thread (1024 threads a
// SM; with the incremental stress a few registers spill, and the extra
// resident warps pay for them: 44.9 against 49.7 us a pass on the 1M-tet box
// at 85 registers).  The full stress needs 64 on its tet loop; the bound
// keeps the out-of-line FP64 call of a near-inverted tet, after the loop,
// from raising it.
template <int MATERIAL, int THREADS, bool INC, bool STAGE>
__global__ void __launch_bounds__(THREADS,
                                  MATERIAL == PBS_MATERIAL_NEOHOOKEAN ? PBS_INC_THREADS_PER_SM / THREADS : 0)
    k_tchunk(DevMesh m, DevParams p, DevState st, int par) {
    extern __shared__ float4 smem4[];
    const int CN = m.chunk_nodes, CT = m.chunk_tets;
    // node words: u hi, u lo (without INC) or the increment (with INC), base
    // (INC only); corner slots; with STAGE the rows and records
    float4 *s_uh = smem4, *s_ul = smem4 + CN, *s_ub = smem4 + 2 * CN;
    float4 *s_f = smem4 + (INC ? 3 : 2) * CN;  // corner slots, 4 a tet
    float4 *s_r0 = s_f + 4 * CT, *s_r1 = s_r0 + CT, *s_r2 = s_r1 + CT;  // STAGE only
    uint4 *s_cor = reinterpret_cast<uint4 *>(s_r2 + CT);
    int4 *s_meta = reinterpret_cast<int4 *>(s_cor + CT);
    __shared__ double sh[THREADS / 32];
    __shared__ int is_last;
    const int c = blockIdx.x;
    // the chunk table and the per-tet rows are constant: read them before
    // waiting for the node kernel
    const int4 cd = m.chunk[c];
    const int inst = m.chunk_inst[c];
    const int tq0 = cd.x, nt = cd.y, l0 = cd.z, nl = cd.w;
    // the chunk's reference node for the increments (incremental form)
    const int g_ref = INC && !STAGE ? m.lmeta[l0].x : 0;
    if (STAGE) {
        for (int lt = threadIdx.x; lt < nt; lt += THREADS) {
            const int q = tq0 + lt;
            cp_async16(s_r0 + lt, m.qrow0 + q);
            cp_async16(s_r1 + lt, m.qrow1 + q);
            cp_async16(s_r2 + lt, m.qrow2 + q);
            cp_async16(s_cor + lt, m.qcor + q);
        }
        for (int j = threadIdx.x; j < nl; j += THREADS) cp_async16(s_meta + j, m.lmeta + l0 + j);
        cp_async_commit();
    }
    const size_t cur = (size_t)par * m.Np;
    pdl_launch_dependents();
    pdl_wait();
    const InstCtl *src = ctl_buf(st, par) + inst;
    InstCtl *dst = ctl_buf(st, par ^ 1) + inst;
    const int4 *meta = STAGE ? s_meta : m.lmeta + l0;
    if (STAGE) {
        // each thread stages the node words of the records it copied itself;
        // the gathers need no control word (the pass's parity is known at
        // launch) and run while it is read
        cp_async_wait_all();
        for (int j = threadIdx.x; j < nl; j += THREADS) {
            const int g = s_meta[j].x;
            cp_async16(s_uh + j, st.uh + cur + g);
            cp_async16(s_ul + j, st.ul + cur + g);
            if (INC) cp_async16(s_ub + j, st.ub + g);
        }
        cp_async_commit();
    }
    const PassView pv = pass_view(src, p);
    if (pv.skip) {
        // an instance that stopped: its first chunk carries the control block
        // over to the copy the node kernel reads
        if (c == src->cblk_begin) settle_pass<THREADS>(p, st, src, dst, true);
        if (STAGE) cp_async_wait_all();
        return;
    }
    if (STAGE) {
        cp_async_wait_all();
        if (INC) {
            // the increments of the nodes this thread staged, relative to the
            // chunk's local node 0 (staged by thread 0)
            __syncthreads();
            const float4 r = s_uh[0];
            __syncthreads();
            for (int j = threadIdx.x; j < nl; j += THREADS) s_ul[j] = increment_rel(s_uh[j], s_ul[j], r);
        }
    } else {
        // (the increments relative to the chunk's local node 0)
        float4 r;
        if (INC) r = st.uh[cur + g_ref];
        for (int j = threadIdx.x; j < nl; j += THREADS) {
            const int g = meta[j].x;
            const float4 uh = st.uh[cur + g], ul = st.ul[cur + g];
            if (INC) {
                const float4 ub = st.ub[g];
                s_ul[j] = increment_rel(uh, ul, r);
                s_ub[j] = ub;
            } else {
                s_uh[j] = uh;
                s_ul[j] = ul;
            }
        }
    }
    __syncthreads();
    ChunkView v;
    v.uh = s_uh;
    v.ul = s_ul;
    v.ub = s_ub;
    v.r0 = STAGE ? s_r0 : m.qrow0 + tq0;
    v.r1 = STAGE ? s_r1 : m.qrow1 + tq0;
    v.r2 = STAGE ? s_r2 : m.qrow2 + tq0;
    v.cor = STAGE ? s_cor : m.qcor + tq0;
    v.meta = meta;
    v.rest = m.rest;
    chunk_body<MATERIAL, THREADS, INC>(m, p, st, c, inst, par, pv, cur, v, meta, nt, nl, s_f, sh, &is_last);
}

// ------------------------------------------------------------ persistent, TMA-fed variant
// mbarrier and bulk-copy (TMA) primitives.  A bulk copy moves a contiguous
// global range into shared memory and reports its bytes to an mbarrier; the
// phase completes when the expected byte count has arrived.
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for phase `parity` of *bar for at most limit_ns; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity, unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer_ns();
    while (!mbar_try_wait(bar, parity))
        if (globaltimer_ns() - t0 > limit_ns) return false;
    return true;
}

// A wait on a bulk copy that has not completed in a second means the copy
// engine or the pipeline bookkeeping is broken: the kernel records
// PBS_E_DEVICE_TIMEOUT in the instance and returns instead of spinning on.
constexpr unsigned long long STREAM_WAIT_NS = 1000000000ull;

// One staging buffer of the persistent kernel.
struct StageBuf {
    float4 *r0, *r1, *r2;
    uint4 *cor;
    int4 *meta;
    float4 *uh, *ul, *ub;
};

// Buffer b of the persistent kernel's shared memory: [buffer 0][buffer 1]
// [slots]; a buffer holds rows 0..2 and corner records (16 B a tet each),
// then local-node records and node words (16 B a node each).
__device__ __forceinline__ StageBuf stage_buf(float4 *smem4, int b, int CT, int CN, int stride) {
    float4 *q = smem4 + b * stride;
    StageBuf s;
    s.r0 = q;
    s.r1 = q + CT;
    s.r2 = q + 2 * CT;
    s.cor = reinterpret_cast<uint4 *>(q + 3 * CT);
    s.meta = reinterpret_cast<int4 *>(q + 4 * CT);
    s.uh = q + 4 * CT + CN;
    s.ul = q + 4 * CT + 2 * CN;
    s.ub = q + 4 * CT + 3 * CN;  // with incremental stress only
    return s;
}

// Thread 0: the chunk's rows, corner records and local-node records by bulk
// copies, completing on *bar.
__device__ __forceinline__ void stage_chunk_bulk(const DevMesh &m, int c, const StageBuf &b, uint64_t *bar) {
    const int4 cd = m.chunk[c];
    const unsigned nt = (unsigned)cd.y, nl = (unsigned)cd.w;
    mbar_expect_tx(bar, 64u * nt + 16u * nl);
    if (nt) {
        bulk_g2s(b.r0, m.qrow0 + cd.x, 16u * nt, bar);
        bulk_g2s(b.r1, m.qrow1 + cd.x, 16u * nt, bar);
        bulk_g2s(b.r2, m.qrow2 + cd.x, 16u * nt, bar);
        bulk_g2s(b.cor, m.qcor + cd.x, 16u * nt, bar);
    }
    if (nl) bulk_g2s(b.meta, m.lmeta + cd.z, 16u * nl, bar);
}

// What a chunk's pass needs from its instance's control blocks.
struct StreamCtx {
    const InstCtl *src;
    InstCtl *dst;
    int inst, nt, nl;
    bool first, skip;
    PassView pv;
    size_t cur;
};

__device__ __forceinline__ StreamCtx stream_ctx(const DevMesh &m, const DevParams &p, const DevState &st, int c,
                                                int par, size_t cur) {
    StreamCtx x;
    const int4 cd = m.chunk[c];
    x.nt = cd.y;
    x.nl = cd.w;
    x.inst = m.chunk_inst[c];
    x.src = ctl_buf(st, par) + x.inst;
    x.dst = ctl_buf(st, par ^ 1) + x.inst;
    x.first = c == x.src->cblk_begin;
    x.pv = pass_view(x.src, p);
    x.skip = x.pv.skip;
    x.cur = cur;
    return x;
}

// Node words of a chunk (local-node records already in b.meta) by cp.async.
template <int THREADS, bool INC>
__device__ __forceinline__ void stage_nodes(const DevState &st, const StageBuf &b, int nl, size_t cur) {
    for (int j = threadIdx.x; j < nl; j += THREADS) {
        const int g = b.meta[j].x;
        cp_async16(b.uh + j, st.uh + cur + g);
        cp_async16(b.ul + j, st.ul + cur + g);
        if (INC) cp_async16(b.ub + j, st.ub + g);
    }
}

// Persistent chunk kernel: CTA b walks chunks b, b + G, b + 2G, ... (G =
// gridDim.x, a whole number of resident CTAs per SM) through two staging
// buffers.  While chunk j computes, chunk j+1's node words are in flight by
// cp.async and chunk j+2's rows and records by bulk copies, so the global
// round trips of the one-CTA-per-chunk kernel (control block, records, node
// gather) leave the critical path.  Chunk for chunk, the arithmetic and its
// order are those of k_tchunk with the same shape: results are bit-identical.
template <int MATERIAL, int THREADS, bool INC>
__global__ void __launch_bounds__(THREADS, 768 / THREADS) k_tstream(DevMesh m, DevParams p, DevState st, int par) {
    extern __shared__ float4 smem4[];
    const int CN = m.chunk_nodes, CT = m.chunk_tets;
    const int stride = 4 * CT + (INC ? 4 : 3) * CN;  // float4 words of one staging buffer
    float4 *s_f = smem4 + 2 * stride;  // corner slots, 4 a tet
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ double sh[THREADS / 32];
    __shared__ int is_last;
    const int G = gridDim.x, c0 = blockIdx.x;
    const int nj = c0 < m.n_chunks ? (m.n_chunks - c0 + G - 1) / G : 0;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
    }
    __syncthreads();
    // the first two chunks' rows and records are constant: they go out before
    // the grid-dependency wait
    if (threadIdx.x == 0) {
        if (nj > 0) stage_chunk_bulk(m, c0, stage_buf(smem4, 0, CT, CN, stride), &bar[0]);
        if (nj > 1) stage_chunk_bulk(m, c0 + G, stage_buf(smem4, 1, CT, CN, stride), &bar[1]);
    }
    pdl_launch_dependents();
    pdl_wait();
    if (nj == 0) return;
    StreamCtx cur, nxt;
    nxt.skip = true;
    // chunk 0: its records, then its node words
    bool ok = mbar_wait_bounded(&bar[0], 0u, STREAM_WAIT_NS);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicExch(st.active + 1, 1);  // the instances stop with PBS_E_DEVICE_TIMEOUT
        if (nj > 1) mbar_wait_bounded(&bar[1], 0u, STREAM_WAIT_NS);
        return;
    }
    const size_t pcur = (size_t)par * m.Np;
    cur = stream_ctx(m, p, st, c0, par, pcur);
    if (!cur.skip) stage_nodes<THREADS, INC>(st, stage_buf(smem4, 0, CT, CN, stride), cur.nl, cur.cur);
    cp_async_commit();
    for (int j = 0; j < nj; ++j) {
        const int b = j & 1, c = c0 + j * G;
        if (j + 1 < nj) {
            // chunk j+1: wait for its records, start its node words
            ok = mbar_wait_bounded(&bar[b ^ 1], (unsigned)((j + 1) >> 1) & 1u, STREAM_WAIT_NS);
            if (__syncthreads_or(!ok)) {
                if (threadIdx.x == 0) atomicExch(st.active + 1, 1);
                cp_async_wait_all();
                mbar_wait_bounded(&bar[b ^ 1], (unsigned)((j + 1) >> 1) & 1u, STREAM_WAIT_NS);
                return;
            }
            nxt = stream_ctx(m, p, st, c + G, par, pcur);
            if (!nxt.skip) stage_nodes<THREADS, INC>(st, stage_buf(smem4, b ^ 1, CT, CN, stride), nxt.nl, nxt.cur);
            cp_async_commit();
            asm volatile("cp.async.wait_group 1;" ::: "memory");  // chunk j's node words (this thread's)
        } else {
            cp_async_wait_all();
        }
        const StageBuf sb = stage_buf(smem4, b, CT, CN, stride);
        if (INC && !cur.skip) {
            // the increments of the nodes this thread staged, relative to the
            // chunk's local node 0 (staged by thread 0)
            __syncthreads();
            const float4 r = sb.uh[0];
            __syncthreads();
            for (int i = threadIdx.x; i < cur.nl; i += THREADS) sb.ul[i] = increment_rel(sb.uh[i], sb.ul[i], r);
        }
        __syncthreads();
        if (cur.first && cur.skip) settle_pass<THREADS>(p, st, cur.src, cur.dst, true);
        if (!cur.skip) {
            ChunkView v;
            v.uh = sb.uh;
            v.ul = sb.ul;
            v.ub = sb.ub;
            v.r0 = sb.r0;
            v.r1 = sb.r1;
            v.r2 = sb.r2;
            v.cor = sb.cor;
            v.meta = sb.meta;
            v.rest = m.rest;
            chunk_body<MATERIAL, THREADS, INC>(m, p, st, c, cur.inst, par, cur.pv, cur.cur, v, sb.meta, cur.nt,
                                               cur.nl, s_f, sh, &is_last);
        }
        __syncthreads();  // buffer b and the slots are free again
        if (threadIdx.x == 0 && j + 2 < nj) stage_chunk_bulk(m, c + 2 * G, sb, &bar[b]);
        cur = nxt;
    }
}

// ------------------------------------------------------------ launchers
template <int MATERIAL, int THREADS, bool INC, bool STAGE> static cudaError_t allow_smem() {
    return cudaFuncSetAttribute(k_tchunk<MATERIAL, THREADS, INC, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                CHUNK_MAX_SMEM);
}

template <int MATERIAL, int THREADS, bool INC> static cudaError_t allow_smem_stream() {
    return cudaFuncSetAttribute(k_tstream<MATERIAL, THREADS, INC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                CHUNK_MAX_SMEM);
}

template <int MATERIAL, bool INC> static cudaError_t allow_smem_all() {
    const cudaError_t e[] = {allow_smem<MATERIAL, 128, INC, false>(), allow_smem<MATERIAL, 256, INC, false>(),
                             allow_smem<MATERIAL, 512, INC, false>()};
    for (cudaError_t x : e)
        if (x != cudaSuccess) return x;
    return cudaSuccess;
}

cudaError_t prepare_chunk_kernels() {
    const cudaError_t e[] = {allow_smem_all<PBS_MATERIAL_NEOHOOKEAN, true>(),
                             allow_smem_all<PBS_MATERIAL_NEOHOOKEAN, false>(),
                             allow_smem_all<PBS_MATERIAL_STRETCH, false>(),
                             allow_smem<PBS_MATERIAL_NEOHOOKEAN, 128, false, true>(),
                             allow_smem<PBS_MATERIAL_NEOHOOKEAN, 256, false, true>(),
                             allow_smem<PBS_MATERIAL_NEOHOOKEAN, 128, true, true>(),
                             allow_smem<PBS_MATERIAL_NEOHOOKEAN, 256, true, true>(),
                             allow_smem_stream<PBS_MATERIAL_NEOHOOKEAN, 128, false>(),
                             allow_smem_stream<PBS_MATERIAL_NEOHOOKEAN, 256, false>(),
                             allow_smem_stream<PBS_MATERIAL_NEOHOOKEAN, 128, true>(),
                             allow_smem_stream<PBS_MATERIAL_NEOHOOKEAN, 256, true>()};
    for (cudaError_t x : e)
        if (x != cudaSuccess) return x;
    return cudaSuccess;
}

cudaError_t launch_pass_rows(cudaStream_t s, int T, const int *qperm, const float4 *row0, const float4 *row1,
                             const float4 *row2, float4 *q0, float4 *q1, float4 *q2) {
    if (T <= 0) return cudaSuccess;
    k_pass_rows<<<(T + 255) / 256, 256, 0, s>>>(T, qperm, row0, row1, row2, q0, q1, q2);
    return cudaGetLastError();
}

// Launch of a per-tet pass kernel: programmatic dependent launch (pdl), and
// the mesh's L2 access-policy window over the pass rows when it has one.  at:
// room for two attributes.
static cudaLaunchConfig_t chunk_config(cudaStream_t s, int grid, int threads, size_t smem, bool pdl,
                                       cudaLaunchAttribute *at, const DevMesh &m) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    int n = 0;
    if (pdl) {
        at[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[n].val.programmaticStreamSerializationAllowed = 1;
        ++n;
    }
    if (m.l2_base) {
        at[n].id = cudaLaunchAttributeAccessPolicyWindow;
        at[n].val.accessPolicyWindow.base_ptr = const_cast<void *>(m.l2_base);
        at[n].val.accessPolicyWindow.num_bytes = m.l2_bytes;
        at[n].val.accessPolicyWindow.hitRatio = m.l2_hit;
        at[n].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        at[n].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        ++n;
    }
    cfg.attrs = at;
    cfg.numAttrs = n;
    return cfg;
}

template <int MATERIAL, int THREADS, bool INC, bool STAGE>
static cudaError_t launch_tchunk_t(cudaStream_t s, const DevMesh &m, const DevParams &p, const DevState &st, int par,
                                   bool pdl) {
    cudaLaunchAttribute at[2];
    cudaLaunchConfig_t cfg = chunk_config(s, m.n_chunks, THREADS,
                                          chunk_smem(m.chunk_tets, m.chunk_nodes, INC, STAGE ? 1 : 0), pdl, at, m);
    return cudaLaunchKernelEx(&cfg, k_tchunk<MATERIAL, THREADS, INC, STAGE>, m, p, st, par);
}

template <int MATERIAL, int THREADS, bool INC>
static cudaError_t launch_tstream_t(cudaStream_t s, const DevMesh &m, const DevParams &p, const DevState &st, int par,
                                    bool pdl) {
    if (m.stream_grid <= 0) return cudaErrorInvalidConfiguration;
    cudaLaunchAttribute at[2];
    cudaLaunchConfig_t cfg =
        chunk_config(s, m.stream_grid, THREADS, chunk_smem(m.chunk_tets, m.chunk_nodes, INC, 2), pdl, at, m);
    return cudaLaunchKernelEx(&cfg, k_tstream<MATERIAL, THREADS, INC>, m, p, st, par);
}

template <int MATERIAL, bool INC>
static cudaError_t launch_tchunk(cudaStream_t s, const DevMesh &m, const DevParams &p, const DevState &st, int par,
                                 bool pdl) {
    if (m.chunk_threads == 128) return launch_tchunk_t<MATERIAL, 128, INC, false>(s, m, p, st, par, pdl);
    if (m.chunk_threads == 512) return launch_tchunk_t<MATERIAL, 512, INC, false>(s, m, p, st, par, pdl);
    return launch_tchunk_t<MATERIAL, 256, INC, false>(s, m, p, st, par, pdl);
}

cudaError_t launch_tet_only(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int material, int par,
                            bool pdl) {
    if (m.n_chunks <= 0) return cudaSuccess;
    if (material == PBS_MATERIAL_STRETCH) return launch_tchunk<PBS_MATERIAL_STRETCH, false>(s, m, p, st, par, pdl);
    // staged shapes: neo-Hookean, 128 or 256 threads
    const bool t128 = m.chunk_threads == 128, t256 = m.chunk_threads == 256;
    if (m.chunk_stage == 2) {
        if (p.incremental) {
            if (t128) return launch_tstream_t<PBS_MATERIAL_NEOHOOKEAN, 128, true>(s, m, p, st, par, pdl);
            if (t256) return launch_tstream_t<PBS_MATERIAL_NEOHOOKEAN, 256, true>(s, m, p, st, par, pdl);
        } else {
            if (t128) return launch_tstream_t<PBS_MATERIAL_NEOHOOKEAN, 128, false>(s, m, p, st, par, pdl);
            if (t256) return launch_tstream_t<PBS_MATERIAL_NEOHOOKEAN, 256, false>(s, m, p, st, par, pdl);
        }
    }
    const bool st128 = m.chunk_stage == 1 && t128, st256 = m.chunk_stage == 1 && t256;
    if (p.incremental) {
        if (st128) return launch_tchunk_t<PBS_MATERIAL_NEOHOOKEAN, 128, true, true>(s, m, p, st, par, pdl);
        if (st256) return launch_tchunk_t<PBS_MATERIAL_NEOHOOKEAN, 256, true, true>(s, m, p, st, par, pdl);
        return launch_tchunk<PBS_MATERIAL_NEOHOOKEAN, true>(s, m, p, st, par, pdl);
    }
    if (st128) return launch_tchunk_t<PBS_MATERIAL_NEOHOOKEAN, 128, false, true>(s, m, p, st, par, pdl);
    if (st256) return launch_tchunk_t<PBS_MATERIAL_NEOHOOKEAN, 256, false, true>(s, m, p, st, par, pdl);
    return launch_tchunk<PBS_MATERIAL_NEOHOOKEAN, false>(s, m, p, st, par, pdl);
}

// CTAs of the persistent chunk kernel for the mesh's shape: as many as fit on
// the device at once, at most one per chunk.  0 when the shape has no
// persistent variant.
template <int MATERIAL, int THREADS, bool INC> static int stream_fit(const DevMesh &m, int sms) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tstream<MATERIAL, THREADS, INC>, THREADS,
                                                      chunk_smem(m.chunk_tets, m.chunk_nodes, INC, 2)) != cudaSuccess)
        return 0;
    return std::min(m.n_chunks, per_sm * sms);
}

int stream_grid(const DevMesh &m, int material, bool inc, int sms) {
    if (m.chunk_stage != 2 || material != PBS_MATERIAL_NEOHOOKEAN || m.n_chunks <= 0) return 0;
    if (m.chunk_threads == 128)
        return inc ? stream_fit<PBS_MATERIAL_NEOHOOKEAN, 128, true>(m, sms)
                   : stream_fit<PBS_MATERIAL_NEOHOOKEAN, 128, false>(m, sms);
    if (m.chunk_threads == 256)
        return inc ? stream_fit<PBS_MATERIAL_NEOHOOKEAN, 256, true>(m, sms)
                   : stream_fit<PBS_MATERIAL_NEOHOOKEAN, 256, false>(m, sms);
    return 0;
}

// ------------------------------------------------------------ persistent frame kernel
// One cooperative launch runs a whole step's passes for a one-instance handle.
// Every CTA stays resident (the launch fails otherwise) and walks the chunks
// b, b + G, ... of each pass's tet phase, then the nodes b * THREADS + t,
// + G * THREADS, ... of its node phase; grid barriers separate the phases.
// After each barrier every CTA takes the line-search and pass decisions
// itself, from the same per-CTA sums in the same order, on its own
// shared-memory copy of the control block: the copies stay equal, and no
// "last CTA" tail, kernel launch or host poll sits between passes.  The
// arithmetic of a tet, a chunk's slot sums and a node's update is the pass
// kernels' (chunk_forces_all, chunk_partials, node_update); the instance's
// sums are grouped by CTA instead of by chunk and node block, so results
// agree with the pass kernels' to rounding, and are bit-reproducible run to
// run.

// Release / acquire accesses of the barrier words (device scope).
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// A barrier wait that has not ended in half a second means a CTA is gone (a
// fault elsewhere) or the launch was not co-resident: the kernel records
// PBS_E_DEVICE_TIMEOUT and every CTA returns instead of spinning on.
constexpr unsigned long long FRAME_WAIT_NS = 500000000ull;

// Grid-wide barrier: every CTA's writes before it are visible to every CTA
// after it.  Thread 0 arrives on the counter; the last to arrive resets it and
// advances the generation (release); the others wait for the generation
// (acquire), at most FRAME_WAIT_NS, and stop waiting as soon as any CTA has
// recorded a failure.  gen: the generation this CTA last passed (thread 0).
__device__ bool frame_barrier(FrameSync *fs, unsigned G, unsigned &gen) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        const unsigned target = gen + 1;
        __threadfence();
        const unsigned arrived = atomicAdd(&fs->count, 1u) + 1u;
        if (arrived == G) {
            fs->count = 0u;
            __threadfence();
            st_release_u32(&fs->gen, target);
        } else {
            const unsigned long long t0 = globaltimer_ns();
            while (ld_acquire_u32(&fs->gen) != target) {
                if (*(volatile int *)&fs->err) {
                    ok = 0;
                    break;
                }
                if (globaltimer_ns() - t0 > FRAME_WAIT_NS) {
                    atomicExch(&fs->err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        gen = target;
    }
    __syncthreads();
    return ok != 0;
}

// Fixed-order FP64 sum of n per-CTA values (ascending per thread, then the
// block tree): every CTA gets the same bits.
template <int THREADS>
__device__ __forceinline__ double2 frame_sum2(const double2 *v, int n, double *sh) {
    double a = 0.0, b = 0.0;
    for (int j = threadIdx.x; j < n; j += THREADS) {
        const double2 x = __ldcg(v + j);
        a += x.x;
        b += x.y;
    }
    const double A = block_sum(a, sh);
    const double B = block_sum(b, sh);
    return make_double2(A, B);
}

// Register budget of the neo-Hookean frame kernels: the pass loop keeps its
// control values live across both phases, so they get 896 threads a SM
// (73 registers) where the pass kernel gets 1024.
#ifndef PBS_FRAME_THREADS_PER_SM
#define PBS_FRAME_THREADS_PER_SM 896
#endif
template <int MATERIAL, int THREADS, bool INC>
__global__ void __launch_bounds__(THREADS,
                                  MATERIAL == PBS_MATERIAL_NEOHOOKEAN ? PBS_FRAME_THREADS_PER_SM / THREADS : 0)
    k_frame(DevMesh m, DevParams p, DevState st, FrameAux fx) {
    extern __shared__ float4 smem4[];
    const int CN = m.chunk_nodes;
    float4 *s_uh = smem4, *s_ul = smem4 + CN, *s_ub = smem4 + 2 * CN;
    float4 *s_f = smem4 + (INC ? 3 : 2) * CN;  // corner slots, 4 a tet
    __shared__ InstCtl sc;                      // this CTA's copy of the control block
    __shared__ double sh[THREADS / 32];
    __shared__ float2 shf[THREADS / 32];
    __shared__ float shs[THREADS / 32];
    const unsigned G = gridDim.x;
    const int b = blockIdx.x;
    unsigned gen = 0;
    if (threadIdx.x == 0) {
        sc = st.ctl[0];
        gen = ld_acquire_u32(&fx.sync->gen);
    }
    __syncthreads();
    bool ok = true;
    for (int pass = 0; pass < fx.max_passes; ++pass) {
        if (sc.done) break;
        const int k = sc.k;
        const bool check = (k % p.ls_every) == 0 || sc.force_check;
        const bool do_h = (k % p.hd_every) == 0;
        const size_t cur = (size_t)sc.par * m.Np;
        // ---- tet phase: the chunks b, b + G, ...
        DFloat e{0.f, 0.f};
        float e2 = 0.f;
        for (int c = b; c < m.n_chunks; c += (int)G) {
            const int4 cd = m.chunk[c];
            const int nt = cd.y, nl = cd.w;
            const int4 *meta = m.lmeta + cd.z;
            // (the increments relative to the chunk's local node 0)
            float4 r;
            if (INC) {
                const int g0 = meta[0].x;
                r = st.uh[cur + g0];
            }
            for (int j = threadIdx.x; j < nl; j += THREADS) {
                const int g = meta[j].x;
                const float4 uh = st.uh[cur + g], ul = st.ul[cur + g];
                if (INC) {
                    const float4 ub = st.ub[g];
                    s_ul[j] = increment_rel(uh, ul, r);
                    s_ub[j] = ub;
                } else {
                    s_uh[j] = uh;
                    s_ul[j] = ul;
                }
            }
            __syncthreads();
            ChunkView v;
            v.uh = s_uh;
            v.ul = s_ul;
            v.ub = s_ub;
            v.r0 = m.qrow0 + cd.x;
            v.r1 = m.qrow1 + cd.x;
            v.r2 = m.qrow2 + cd.x;
            v.cor = m.qcor + cd.x;
            v.meta = meta;
            v.rest = m.rest;
            const DFloat ec = chunk_forces_all<MATERIAL, THREADS, INC>(p, v, nt, check, s_f);
            chunk_partials<THREADS>(meta, nl, s_f, st.part);
            if (do_h) {
                __syncthreads();
                chunk_hdiag<MATERIAL, THREADS, INC>(v, nt, s_f);
                __syncthreads();
                chunk_partials<THREADS>(meta, nl, s_f, st.parth);
            }
            if (check) {
                e = df_add(e, ec);
                e2 = fmaf(ec.hi, ec.hi, e2);
            }
            __syncthreads();  // the slots and node words are free for the next chunk
        }
        if (check) {
            // this CTA's share of the node energy terms
            const float4 *U = st.uh + cur;
            for (int i = b * THREADS + threadIdx.x; i < m.Np; i += (int)G * THREADS) {
                const float4 info = m.info[i];
                if (info.z != 0.f) continue;
                const DFloat en =
                    node_energy_df(st, info, U[i], st.ul[cur + i], i, p.h2inv, INC ? st.ub : nullptr);
                e = df_add(e, en);
                e2 = fmaf(en.hi, en.hi, e2);
            }
            const DFloat se = block_sum_df(e, shf);
            const float se2 = block_sum_f(e2, shs);
            if (threadIdx.x == 0) fx.ce[b] = make_double2(df_double(se), (double)se2);
        }
        ok = frame_barrier(fx.sync, G, gen);
        if (!ok) break;
        // ---- the line-search decision (every CTA, the same sums)
        if (check) {
            const double2 E = frame_sum2<THREADS>(fx.ce, (int)G, sh);
            if (threadIdx.x == 0) decide_line_search(sc, p, k, E.x, E.y);
            __syncthreads();
            if (sc.done) break;
        }
        // ---- node phase: the nodes b * THREADS + t, + G * THREADS, ...
        const int action = check ? sc.action : ACT_STEP;
        float rho = sc.rho, omega = sc.omega;
        chebyshev_schedule(p, k - sc.k_restart, rho, omega);
        PassCtx ctx;
        ctx.action = action;
        ctx.do_h = do_h;
        ctx.alpha = sc.alpha;
        ctx.omega = omega;
        ctx.cur = cur;
        ctx.nxt = (size_t)(1 - sc.par) * m.Np;
        float r2 = 0.f;
        for (int i = b * THREADS + threadIdx.x; i < m.Np; i += (int)G * THREADS) {
            NodeConst nc;
            nc.ch = st.ch[i];
            nc.cl = st.cl[i];
            NodeIn nn;
            nn.pa = m.pptr[i];
            nn.pe = m.pptr[i + 1];
            float4 fp[2];  // a node touches 1.7 chunks on average: two prefetched partials
#pragma unroll
            for (int q = 0; q < 2; ++q)
                fp[q] = nn.pa + q < nn.pe ? st.part[nn.pa + q] : make_float4(0.f, 0.f, 0.f, 0.f);
            nn.uh = st.uh[cur + i];
            nn.ul = st.ul[cur + i];
            nn.dd = st.dd[cur + i];
            nn.diag = st.diag[i];
            r2 += node_update<2>(m, p, st, i, nc, nn, fp, ctx);
        }
        const float sr = block_sum_f(r2, shs);
        if (threadIdx.x == 0) fx.cr[b] = make_double2((double)sr, 0.0);
        ok = frame_barrier(fx.sync, G, gen);
        if (!ok) break;
        // ---- the pass decision (every CTA, the same sums)
        const double2 R = frame_sum2<THREADS>(fx.cr, (int)G, sh);
        if (threadIdx.x == 0) decide_pass(sc, p, k, action, rho, omega, R.x);
        __syncthreads();
    }
    if (b == 0 && threadIdx.x == 0) {
        if (!ok) {
            sc.status = PBS_E_DEVICE_TIMEOUT;
            sc.done = 1;
        }
        st.ctl[0] = sc;
        if (sc.done) atomicSub(st.active, 1);
    }
}

template <int MATERIAL, int THREADS, bool INC> static cudaError_t allow_smem_frame() {
    return cudaFuncSetAttribute(k_frame<MATERIAL, THREADS, INC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                CHUNK_MAX_SMEM);
}

template <int MATERIAL, int THREADS, bool INC> static int frame_fit(const DevMesh &m, int sms) {
    if (allow_smem_frame<MATERIAL, THREADS, INC>() != cudaSuccess) return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_frame<MATERIAL, THREADS, INC>, THREADS,
                                                      chunk_smem(m.chunk_tets, m.chunk_nodes, INC, 0)) != cudaSuccess)
        return 0;
    return std::min(m.n_chunks, per_sm * sms);
}

int frame_grid(const DevMesh &m, int material, bool inc, int sms) {
    if (m.n_inst != 1 || m.chunk_stage != 0 || m.n_chunks <= 0) return 0;
    const bool nh_inc = material == PBS_MATERIAL_NEOHOOKEAN && inc;
    if (material == PBS_MATERIAL_STRETCH) {
        if (m.chunk_threads == 128) return frame_fit<PBS_MATERIAL_STRETCH, 128, false>(m, sms);
        if (m.chunk_threads == 256) return frame_fit<PBS_MATERIAL_STRETCH, 256, false>(m, sms);
        return 0;
    }
    if (m.chunk_threads == 128)
        return nh_inc ? frame_fit<PBS_MATERIAL_NEOHOOKEAN, 128, true>(m, sms)
                      : frame_fit<PBS_MATERIAL_NEOHOOKEAN, 128, false>(m, sms);
    if (m.chunk_threads == 256)
        return nh_inc ? frame_fit<PBS_MATERIAL_NEOHOOKEAN, 256, true>(m, sms)
                      : frame_fit<PBS_MATERIAL_NEOHOOKEAN, 256, false>(m, sms);
    return 0;
}

template <int MATERIAL, int THREADS, bool INC>
static cudaError_t launch_frame_t(cudaStream_t s, const DevMesh &m, const DevParams &p, const DevState &st,
                                  const FrameAux &fx, int grid) {
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = chunk_smem(m.chunk_tets, m.chunk_nodes, INC, 0);
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_frame<MATERIAL, THREADS, INC>, m, p, st, fx);
}

cudaError_t launch_frame(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int material,
                         const FrameAux &fx, int grid) {
    if (grid <= 0) return cudaErrorInvalidConfiguration;
    const bool inc = material == PBS_MATERIAL_NEOHOOKEAN && p.incremental;
    if (material == PBS_MATERIAL_STRETCH) {
        if (m.chunk_threads == 128) return launch_frame_t<PBS_MATERIAL_STRETCH, 128, false>(s, m, p, st, fx, grid);
        return launch_frame_t<PBS_MATERIAL_STRETCH, 256, false>(s, m, p, st, fx, grid);
    }
    if (m.chunk_threads == 128)
        return inc ? launch_frame_t<PBS_MATERIAL_NEOHOOKEAN, 128, true>(s, m, p, st, fx, grid)
                   : launch_frame_t<PBS_MATERIAL_NEOHOOKEAN, 128, false>(s, m, p, st, fx, grid);
    return inc ? launch_frame_t<PBS_MATERIAL_NEOHOOKEAN, 256, true>(s, m, p, st, fx, grid)
               : launch_frame_t<PBS_MATERIAL_NEOHOOKEAN, 256, false>(s, m, p, st, fx, grid);
}

}  // namespace pbs
