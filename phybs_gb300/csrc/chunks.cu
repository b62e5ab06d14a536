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
// (DescentOptimize.cpp:162-183) before any node moves.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <utility>
#include <vector>

#include "../../include/phybs.h"
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
    std::vector<int> ctets, lnodes, scount;
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
            out.chunk.push_back(make_int4(tq, 0, (int)out.lnode.size(), 0));
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
            std::sort(lnodes.begin(), lnodes.end());
            const int nl = (int)lnodes.size(), nt = (int)ctets.size();
            for (int j = 0; j < nl; ++j) lidx[lnodes[j]] = j;
            scount.assign(nl + 1, 0);
            for (int t : ctets)
                for (int c = 0; c < 4; ++c) scount[lidx[(&tets[t].x)[c]] + 1]++;
            for (int j = 0; j < nl; ++j) scount[j + 1] += scount[j];
            const int l0 = (int)out.lnode.size();
            for (int j = 0; j < nl; ++j) {
                out.lnode.push_back(lnodes[j]);
                out.lsptr.push_back(scount[j]);
                n_part[lnodes[j]]++;
            }
            for (int lt = 0; lt < nt; ++lt) {
                const int *q = &tets[ctets[lt]].x;
                unsigned short loc[4], sl[4];
                for (int c = 0; c < 4; ++c) {
                    loc[c] = (unsigned short)lidx[q[c]];
                    sl[c] = (unsigned short)scount[loc[c]]++;
                }
                out.qloc.push_back(make_ushort4(loc[0], loc[1], loc[2], loc[3]));
                out.qslot.push_back(make_ushort4(sl[0], sl[1], sl[2], sl[3]));
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
    out.lpidx.resize(out.lnode.size());
    for (size_t j = 0; j < out.lnode.size(); ++j) out.lpidx[j] = fill[out.lnode[j]]++;
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

// Sums every local node's slots (in slot order) into its partial for this
// chunk.
template <int THREADS>
__device__ __forceinline__ void chunk_partials(const DevMesh &m, int l0, int nl, int nt, const float *sx,
                                               const float *sy, const float *sz, float4 *out) {
    for (int j = threadIdx.x; j < nl; j += THREADS) {
        const int s0 = m.lsptr[l0 + j];
        const int s1 = j + 1 < nl ? m.lsptr[l0 + j + 1] : 4 * nt;
        float fx = 0.f, fy = 0.f, fz = 0.f;
        for (int s = s0; s < s1; ++s) {
            fx += sx[s];
            fy += sy[s];
            fz += sz[s];
        }
        out[m.lpidx[l0 + j]] = make_float4(fx, fy, fz, 0.f);
    }
}

// STAGE: the row-staged variant.  Every thread first issues asynchronous
// copies of its tets' rows and corner ids into shared memory -- before the
// grid-dependency wait, since they are constant -- and of the chunk's node
// words after it; one wait then covers all of them, instead of one global
// round trip per tet inside the loop.
template <int MATERIAL, int THREADS, bool INC, bool STAGE>
__global__ void __launch_bounds__(THREADS) k_tchunk(DevMesh m, DevParams p, DevState st) {
    extern __shared__ float4 smem4[];
    const int CN = m.chunk_nodes, CT = m.chunk_tets;
    float4 *s_uh = smem4, *s_ul = smem4 + CN, *s_ub = smem4 + 2 * CN;  // s_ub only with INC
    float *s_x = reinterpret_cast<float *>(smem4 + (INC ? 3 : 2) * CN);
    float *s_y = s_x + 4 * CT, *s_z = s_y + 4 * CT;
    float4 *s_r0 = reinterpret_cast<float4 *>(s_z + 4 * CT), *s_r1 = s_r0 + CT, *s_r2 = s_r1 + CT;  // STAGE only
    ushort4 *s_lc = reinterpret_cast<ushort4 *>(s_r2 + CT), *s_sl = s_lc + CT;
    __shared__ double sh[THREADS / 32];
    __shared__ int is_last;
    const int c = blockIdx.x;
    // the chunk table and the per-tet rows are constant: read them before
    // waiting for the node kernel
    const int4 cd = m.chunk[c];
    const int inst = m.chunk_inst[c];
    const int tq0 = cd.x, nt = cd.y, l0 = cd.z, nl = cd.w;
    if (STAGE) {
        for (int lt = threadIdx.x; lt < nt; lt += THREADS) {
            const int q = tq0 + lt;
            cp_async16(s_r0 + lt, m.qrow0 + q);
            cp_async16(s_r1 + lt, m.qrow1 + q);
            cp_async16(s_r2 + lt, m.qrow2 + q);
            cp_async8(s_lc + lt, m.qloc + q);
            cp_async8(s_sl + lt, m.qslot + q);
        }
        cp_async_commit();
    }
    pdl_launch_dependents();
    pdl_wait();
    InstCtl *cp = st.ctl + inst;
    if (cp->done) {
        if (STAGE) cp_async_wait_all();
        return;
    }
    const int k = cp->k;
    const bool check = (k % p.ls_every) == 0 || cp->force_check;
    const bool do_h = (k % p.hd_every) == 0;
    const size_t cur = (size_t)cp->par * m.Np;
    for (int j = threadIdx.x; j < nl; j += THREADS) {
        const int g = m.lnode[l0 + j];
        if (STAGE) {
            cp_async16(s_uh + j, st.uh + cur + g);
            cp_async16(s_ul + j, st.ul + cur + g);
            if (INC) cp_async16(s_ub + j, st.ub + g);
        } else {
            s_uh[j] = st.uh[cur + g];
            s_ul[j] = st.ul[cur + g];
            if (INC) s_ub[j] = st.ub[g];
        }
    }
    if (STAGE) cp_async_wait_all();
    __syncthreads();
    double e = 0.0;
    for (int lt = threadIdx.x; lt < nt; lt += THREADS) {
        const int q = tq0 + lt;
        const float4 r0 = STAGE ? s_r0[lt] : m.qrow0[q], r1 = STAGE ? s_r1[lt] : m.qrow1[q],
                     r2 = STAGE ? s_r2[lt] : m.qrow2[q];
        const ushort4 lc = STAGE ? s_lc[lt] : m.qloc[q], sl = STAGE ? s_sl[lt] : m.qslot[q];
        const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
        Kin<float> kin;
        float f[12];
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        pass_forces_c<MATERIAL, INC>(s_uh[lc.x], s_uh[lc.y], s_uh[lc.z], s_uh[lc.w], s_ul[lc.x], s_ul[lc.y],
                                     s_ul[lc.z], s_ul[lc.w], INC ? s_ub[lc.x] : z4, INC ? s_ub[lc.y] : z4,
                                     INC ? s_ub[lc.z] : z4, INC ? s_ub[lc.w] : z4, dinv, r0.w, r1.w, r2.w, kin, f);
        const int slot[4] = {sl.x, sl.y, sl.z, sl.w};
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
            s_x[slot[cc]] = f[3 * cc];
            s_y[slot[cc]] = f[3 * cc + 1];
            s_z[slot[cc]] = f[3 * cc + 2];
        }
        if (check)
            e += (double)search_energy(energy_density<float>(kin, r1.w, r2.w) * fabsf(r0.w), p.clamp_cpu,
                                       p.control == PBS_CONTROL_RESTART);
    }
    __syncthreads();
    chunk_partials<THREADS>(m, l0, nl, nt, s_x, s_y, s_z, st.part);
    if (do_h) {  // Jacobi-diagonal refresh: the same slots carry the 12 diagonal terms
        __syncthreads();
        for (int lt = threadIdx.x; lt < nt; lt += THREADS) {
            const int q = tq0 + lt;
            const float4 r0 = STAGE ? s_r0[lt] : m.qrow0[q], r1 = STAGE ? s_r1[lt] : m.qrow1[q],
                         r2 = STAGE ? s_r2[lt] : m.qrow2[q];
            const ushort4 lc = STAGE ? s_lc[lt] : m.qloc[q], sl = STAGE ? s_sl[lt] : m.qslot[q];
            const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
            Kin<float> kin;
            float f[12], kd[12];
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            pass_forces_c<MATERIAL, INC>(s_uh[lc.x], s_uh[lc.y], s_uh[lc.z], s_uh[lc.w], s_ul[lc.x], s_ul[lc.y],
                                         s_ul[lc.z], s_ul[lc.w], INC ? s_ub[lc.x] : z4, INC ? s_ub[lc.y] : z4,
                                         INC ? s_ub[lc.z] : z4, INC ? s_ub[lc.w] : z4, dinv, r0.w, r1.w, r2.w, kin,
                                         f);
            hessian_diag(kin, r1.w, r2.w, dinv, r0.w, kd);
            const int slot[4] = {sl.x, sl.y, sl.z, sl.w};
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
                s_x[slot[cc]] = kd[3 * cc];
                s_y[slot[cc]] = kd[3 * cc + 1];
                s_z[slot[cc]] = kd[3 * cc + 2];
            }
        }
        __syncthreads();
        chunk_partials<THREADS>(m, l0, nl, nt, s_x, s_y, s_z, st.parth);
    }
    if (!check) return;
    // line-search pass: add this chunk's share of the instance's node terms
    double e2 = e * e;
    {
        const int nb = cp->cblk_end - cp->cblk_begin;
        const float4 *U = st.uh + cur;
        for (int i = cp->node_begin + (c - cp->cblk_begin) * THREADS + threadIdx.x; i < cp->node_end;
             i += nb * THREADS) {
            const float4 info = m.info[i];
            if (info.z != 0.f) continue;
            const double en = node_energy(st, info, U[i], st.ul[cur + i], i, p.h2inv);
            e += en;
            e2 += en * en;
        }
    }
    const double se = block_sum(e, sh);
    const double se2 = block_sum(e2, sh);
    if (threadIdx.x == 0) {
        st.cpart[c] = make_double2(se, se2);
        __threadfence();
        const unsigned int prev = atomicAdd(&cp->counter_t, 1u);
        is_last = (prev == (unsigned int)(cp->cblk_end - cp->cblk_begin - 1));
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // the instance's last chunk: fixed-order sums, then accept / reject
    double E = 0.0, E2 = 0.0;
    for (int j = cp->cblk_begin + threadIdx.x; j < cp->cblk_end; j += THREADS) {
        const double2 v = __ldcg(st.cpart + j);
        E += v.x;
        E2 += v.y;
    }
    E = block_sum(E, sh);
    E2 = block_sum(E2, sh);
    if (threadIdx.x != 0) return;
    InstCtl &ci = *cp;  // in place, as in the node kernel
    ci.counter_t = 0;
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
    // force_check stays set: the node kernel of this pass reads it to apply the
    // decision, and clears it
    if (!isfinite(E) && !(bad && k != 0)) {
        ci.status = PBS_E_NONFINITE;
        ci.done = 1;
    }
    if (ci.done) atomicSub(st.active, 1);
}

// ------------------------------------------------------------ launchers
template <int MATERIAL, int THREADS, bool INC, bool STAGE> static cudaError_t allow_smem() {
    return cudaFuncSetAttribute(k_tchunk<MATERIAL, THREADS, INC, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
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
                             allow_smem<PBS_MATERIAL_NEOHOOKEAN, 256, true, true>()};
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

template <int MATERIAL, int THREADS, bool INC, bool STAGE>
static cudaError_t launch_tchunk_t(cudaStream_t s, const DevMesh &m, const DevParams &p, const DevState &st, bool pdl) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(m.n_chunks);
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = chunk_smem(m.chunk_tets, m.chunk_nodes, INC, STAGE);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_tchunk<MATERIAL, THREADS, INC, STAGE>, m, p, st);
}

template <int MATERIAL, bool INC>
static cudaError_t launch_tchunk(cudaStream_t s, const DevMesh &m, const DevParams &p, const DevState &st, bool pdl) {
    if (m.chunk_threads == 128) return launch_tchunk_t<MATERIAL, 128, INC, false>(s, m, p, st, pdl);
    if (m.chunk_threads == 512) return launch_tchunk_t<MATERIAL, 512, INC, false>(s, m, p, st, pdl);
    return launch_tchunk_t<MATERIAL, 256, INC, false>(s, m, p, st, pdl);
}

cudaError_t launch_tet_only(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int material, bool pdl) {
    if (m.n_chunks <= 0) return cudaSuccess;
    if (material == PBS_MATERIAL_STRETCH) return launch_tchunk<PBS_MATERIAL_STRETCH, false>(s, m, p, st, pdl);
    // row-staged shapes: neo-Hookean, 128 or 256 threads
    const bool st128 = m.chunk_stage && m.chunk_threads == 128, st256 = m.chunk_stage && m.chunk_threads == 256;
    if (p.incremental) {
        if (st128) return launch_tchunk_t<PBS_MATERIAL_NEOHOOKEAN, 128, true, true>(s, m, p, st, pdl);
        if (st256) return launch_tchunk_t<PBS_MATERIAL_NEOHOOKEAN, 256, true, true>(s, m, p, st, pdl);
        return launch_tchunk<PBS_MATERIAL_NEOHOOKEAN, true>(s, m, p, st, pdl);
    }
    if (st128) return launch_tchunk_t<PBS_MATERIAL_NEOHOOKEAN, 128, false, true>(s, m, p, st, pdl);
    if (st256) return launch_tchunk_t<PBS_MATERIAL_NEOHOOKEAN, 256, false, true>(s, m, p, st, pdl);
    return launch_tchunk<PBS_MATERIAL_NEOHOOKEAN, false>(s, m, p, st, pdl);
}

}  // namespace pbs
