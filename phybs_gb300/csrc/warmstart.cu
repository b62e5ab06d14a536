// Learned warm start of the descent step (device side).
//
// Before the first iteration of a step, when a network is installed:
//   k_ws_force     corner forces at the plain guess u_plain (into the gather slots)
//   k_ws_gref      |g(u_plain)| per instance -> ctl.g0: the residual reference of
//                  the step, the same with or without the warm start
//   k_ws_tet_F     per-tet F - I and det F - 1 at the inertial target x~,
//                  and the tet's log10 E and Poisson's ratio
//   k_ws_infer     per 32 nodes and warp: node features (velocity history,
//                  inertial offset, material, mean incident F and J), the
//                  standardised 24-vector, the tensor-core MLP, and the
//                  candidate guess u_plain + s * out_std * output (free nodes;
//                  s the node's motion scale)
//   k_ws_judge     energies of both guesses (tets + node terms, FP64 sums);
//                  the instance keeps the candidate only if its energy is not
//                  higher (the plain descent is the fallback and the judge)
//   k_ws_select    copies the chosen guess into the pass state.  The base of
//                  the incremental stress stays at the plain guess, whose
//                  elastic force the step already formed: the increments are
//                  exact from any base, so a kept guess needs no second base
//                  force
#include <algorithm>

#include "../../include/phybs.h"
#include "mlp.cuh"
#include "pass_math.cuh"
#include "phybs_internal.cuh"
#include "tet_math.cuh"

namespace pbs {

// Corner forces at displacement U into the gather slots (as k_tet, no energy).
template <int MATERIAL>
__global__ void __launch_bounds__(BLOCK) k_ws_force(DevMesh m, DevParams p, DevState st, const float4 *U) {
    const int t = blockIdx.x * BLOCK + threadIdx.x;
    if (t >= m.Tp) return;
    const int4 q = m.tets[t];
    if (q.x < 0) return;
    const float4 r0 = m.row0[t], r1 = m.row1[t], r2 = m.row2[t];
    const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
    Kin<float> kin;
    float f[12];
    pass_forces<MATERIAL>(p, U, st.ul, st.ub, q, dinv, r0.w, r1.w, r2.w, kin, f, m.rest);
    const int4 sl = m.tslot[t];
    float4 *tf4 = reinterpret_cast<float4 *>(st.tf);
    tf4[sl.x] = make_float4(f[0], f[1], f[2], 0.f);
    tf4[sl.y] = make_float4(f[3], f[4], f[5], 0.f);
    tf4[sl.z] = make_float4(f[6], f[7], f[8], 0.f);
    tf4[sl.w] = make_float4(f[9], f[10], f[11], 0.f);
}

// |g|^2 at the learned candidate (parity 1), with its elastic forces gathered
// from the slots k_ws_force filled (incremental mode: the increment from the
// plain guess, whose force is in b), reduced per instance into ctl.g1.
__global__ void __launch_bounds__(BLOCK) k_ws_gcand(DevMesh m, DevParams p, DevState st) {
    __shared__ double sh[BLOCK / 32];
    __shared__ int is_last;
    const int b = blockIdx.x;
    InstCtl *cp = st.ctl + m.nblk_inst[b];
    if (cp->done) return;
    const int i = b * BLOCK + threadIdx.x;
    const float4 info = m.info[i];
    double r2 = 0.0;
    if (info.z == 0.f) {
        float fx = 0.f, fy = 0.f, fz = 0.f;
        const float4 *tf4 = reinterpret_cast<const float4 *>(st.tf);
        for (int j = m.inc_ptr[i]; j < m.inc_ptr[i + 1]; ++j) {
            const float4 f = tf4[j];
            fx += f.x;
            fy += f.y;
            fz += f.z;
        }
        const float4 uh = st.uh[m.Np + i], ul = st.ul[m.Np + i], th = st.th[i], tl = st.tl[i], bh = st.bh[i],
                     bl = st.bl[i];
        const float mh = info.x * p.h2inv;
        const float gx = ((((uh.x - th.x) + (ul.x - tl.x)) * mh - bh.x) - bl.x) - fx;
        const float gy = ((((uh.y - th.y) + (ul.y - tl.y)) * mh - bh.y) - bl.y) - fy;
        const float gz = ((((uh.z - th.z) + (ul.z - tl.z)) * mh - bh.z) - bl.z) - fz;
        r2 = (double)gx * gx + (double)gy * gy + (double)gz * gz;
    }
    const double s = block_sum(r2, sh);
    if (threadIdx.x == 0) {
        st.npart[b] = s;
        __threadfence();
        const unsigned int prev = atomicAdd(&cp->counter_n, 1u);
        is_last = (prev == (unsigned int)(cp->nblk_end - cp->nblk_begin - 1));
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double R2 = 0.0;
    for (int j = cp->nblk_begin + threadIdx.x; j < cp->nblk_end; j += BLOCK) R2 += __ldcg(st.npart + j);
    R2 = block_sum(R2, sh);
    if (threadIdx.x == 0) {
        cp->counter_n = 0;
        cp->g1 = sqrt(R2);
    }
}

// |g|^2 at the plain guess (parity 0), reduced per instance into ctl.g0.
__global__ void __launch_bounds__(BLOCK) k_ws_gref(DevMesh m, DevParams p, DevState st) {
    __shared__ double sh[BLOCK / 32];
    __shared__ int is_last;
    const int b = blockIdx.x;
    InstCtl *cp = st.ctl + m.nblk_inst[b];
    if (cp->done) return;
    const int i = b * BLOCK + threadIdx.x;
    const float4 info = m.info[i];
    double r2 = 0.0;
    if (info.z == 0.f) {
        // incremental mode: the plain guess is the base, so its elastic force is
        // all in b; otherwise sum the full corner forces of k_ws_force
        float fx = 0.f, fy = 0.f, fz = 0.f;
        if (!p.incremental) {
            const float4 *tf4 = reinterpret_cast<const float4 *>(st.tf);
            for (int j = m.inc_ptr[i]; j < m.inc_ptr[i + 1]; ++j) {
                const float4 f = tf4[j];
                fx += f.x;
                fy += f.y;
                fz += f.z;
            }
        }
        const float4 uh = st.uh[i], ul = st.ul[i], th = st.th[i], tl = st.tl[i], bh = st.bh[i], bl = st.bl[i];
        const float mh = info.x * p.h2inv;
        const float gx = ((((uh.x - th.x) + (ul.x - tl.x)) * mh - bh.x) - bl.x) - fx;
        const float gy = ((((uh.y - th.y) + (ul.y - tl.y)) * mh - bh.y) - bl.y) - fy;
        const float gz = ((((uh.z - th.z) + (ul.z - tl.z)) * mh - bh.z) - bl.z) - fz;
        r2 = (double)gx * gx + (double)gy * gy + (double)gz * gz;
    }
    const double s = block_sum(r2, sh);
    if (threadIdx.x == 0) {
        st.npart[b] = s;
        __threadfence();
        const unsigned int prev = atomicAdd(&cp->counter_n, 1u);
        is_last = (prev == (unsigned int)(cp->nblk_end - cp->nblk_begin - 1));
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double R2 = 0.0;
    for (int j = cp->nblk_begin + threadIdx.x; j < cp->nblk_end; j += BLOCK) R2 += __ldcg(st.npart + j);
    R2 = block_sum(R2, sh);
    if (threadIdx.x == 0) {
        cp->counter_n = 0;
        cp->g0 = sqrt(R2);
        cp->g0_fixed = 1;
    }
}

// Per tet at the inertial target: F - I (9 values) and det F - 1, then the
// tet's material features log10 E and Poisson's ratio (constant, but formed
// here once a tet rather than once per incident node), into a [Tp][12]
// scratch array that the node features read as three 128-bit words.
__global__ void k_ws_tet_F(DevMesh m, DevState st, float *tetF) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.Tp) return;
    const int4 q = m.tets[t];
    float *o = tetF + 12 * (size_t)t;
    if (q.x < 0) return;
    const float4 r0 = m.row0[t], r1 = m.row1[t], r2 = m.row2[t];
    const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
    Kin<float> kin;
    disp_gradient<float>(st.th[q.x], st.th[q.y], st.th[q.z], st.th[q.w], dinv, kin.G);
    kinematics(kin);
    const float mu = r1.w, lam = r2.w;
    const float nu = 0.5f - mu / lam;  // lambda = 2 mu / (1 - 2 nu)
    float4 *o4 = reinterpret_cast<float4 *>(o);
    o4[0] = make_float4(kin.G[0], kin.G[1], kin.G[2], kin.G[3]);
    o4[1] = make_float4(kin.G[4], kin.G[5], kin.G[6], kin.G[7]);
    o4[2] = make_float4(kin.G[8], kin.d, log10f(2.0f * mu * (1.0f + nu)), nu);
}

// The 24 raw features of node i (see phybs_gb300/warmstart.py for the list)
// and its motion scale s = (1 - damping) |d1| + |d1 - d2| + 1e-4 l (d1, d2:
// the last two displacements, l: the mean edge length): the size of the plain
// guess's error when the node moves with constant acceleration.  It divides
// every length feature and the predicted correction, so the network's target
// is O(1) in smooth motion, where the guess is worth most.
__device__ __forceinline__ void node_features(const DevMesh &m, const DevState &st, const DevParams &p,
                                              const float *tetF, float ell, int i, float f[24], float &scale) {
    const float4 v = st.v[i], vo = st.vold[i], h1 = st.hist1[i], h2 = st.hist2[i];
    const float ax = h1.x - h2.x, ay = h1.y - h2.y, az = h1.z - h2.z;
    scale = (1.0f - p.damping) * sqrtf(h1.x * h1.x + h1.y * h1.y + h1.z * h1.z) + sqrtf(ax * ax + ay * ay + az * az) +
            1e-4f * ell;
    const float il = 1.0f / scale, ivl = p.h / scale, wo = p.warm_start * p.h / scale;
    f[0] = v.x * ivl; f[1] = v.y * ivl; f[2] = v.z * ivl;
    f[3] = h1.x * il; f[4] = h1.y * il; f[5] = h1.z * il;
    f[6] = h2.x * il; f[7] = h2.y * il; f[8] = h2.z * il;
    f[9] = (v.x - vo.x) * wo; f[10] = (v.y - vo.y) * wo; f[11] = (v.z - vo.z) * wo;
    float acc[12] = {0};
    const int a = m.inc_ptr[i], e = m.inc_ptr[i + 1];
    for (int j = a; j < e; ++j) {
        const int t = m.inc[j] >> 2;
        const float4 *F = reinterpret_cast<const float4 *>(tetF + 12 * (size_t)t);
        const float4 f0 = F[0], f1 = F[1], f2 = F[2];
        acc[0] += f0.x; acc[1] += f0.y; acc[2] += f0.z; acc[3] += f0.w;
        acc[4] += f1.x; acc[5] += f1.y; acc[6] += f1.z; acc[7] += f1.w;
        acc[8] += f2.x; acc[9] += f2.y;
        acc[10] += f2.z;  // log10 E
        acc[11] += f2.w;  // Poisson's ratio
    }
    const float inv = e > a ? 1.0f / (float)(e - a) : 0.f;
    f[12] = acc[10] * inv;
    f[13] = acc[11] * inv;
#pragma unroll
    for (int k = 0; k < 10; ++k) f[14 + k] = acc[k] * inv;
}

__global__ void k_ws_features(DevMesh m, DevParams p, DevState st, const float *tetF, const int *pad2user, float *out,
                              float *scale_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const int u = pad2user[i];
    if (u < 0) return;
    float f[24], sc;
    node_features(m, st, p, tetF, node_ell(m, st, i), i, f, sc);
    for (int k = 0; k < 24; ++k) out[24 * (size_t)u + k] = f[k];
    if (scale_out) scale_out[u] = sc;
}

struct WsNet {
    const float *theta;
    const float *feat_mean, *feat_std, *out_std;  // 24, 24, 3
    int base;  // 0: the correction is added to the plain guess; 1: to u0 + 2 d1 - d2
};

// Features -> standardised BF16 fragments -> MLP -> candidate guess in
// (uh, ul)[parity 1] (free nodes; others copy the plain guess).
__global__ void __launch_bounds__(128) k_ws_infer(DevMesh m, DevParams p, DevState st, const float *tetF, WsNet net) {
    __shared__ mlp::SmemWeights sw;
    __shared__ float tile[4][32][25];
    __shared__ float tscale[4][32];
    __shared__ float fm[24], fs[24], os[3];
    mlp::stage_weights(net.theta, sw);
    if (threadIdx.x < 24) {
        fm[threadIdx.x] = net.feat_mean[threadIdx.x];
        fs[threadIdx.x] = 1.0f / net.feat_std[threadIdx.x];
    }
    if (threadIdx.x < 3) os[threadIdx.x] = net.out_std[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const int nwarps = gridDim.x * 4;
    // 32 nodes a warp and iteration (Np is a multiple of 256): every lane
    // gathers one node's features, then the MLP runs on two 16-row tiles
    for (int row0 = (blockIdx.x * 4 + w) * 32; row0 < m.Np; row0 += nwarps * 32) {
        {
            const int i = row0 + lane;
            float f[24], sc = 0.f;
            const float4 info = m.info[i];
            if (info.z == 0.f) {
                node_features(m, st, p, tetF, node_ell(m, st, i), i, f, sc);
#pragma unroll
                for (int k = 0; k < 24; ++k) f[k] = (f[k] - fm[k]) * fs[k];
            } else {
#pragma unroll
                for (int k = 0; k < 24; ++k) f[k] = 0.f;
            }
#pragma unroll
            for (int k = 0; k < 24; ++k) tile[w][lane][k] = f[k];
            tscale[w][lane] = sc;
        }
        __syncwarp();
#pragma unroll 1
        for (int half = 0; half < 2; ++half) {
            float(*tl)[25] = tile[w] + 16 * half;
            uint32_t x[2][4];
#pragma unroll
            for (int kb = 0; kb < 2; ++kb) {
                float v[4][2];
#pragma unroll
                for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                    for (int e2 = 0; e2 < 2; ++e2) {
                        const int col = 16 * kb + 8 * hh + 2 * t + e2;
                        v[2 * hh][e2] = col < 24 ? tl[g][col] : 0.f;
                        v[2 * hh + 1][e2] = col < 24 ? tl[g + 8][col] : 0.f;
                    }
                x[kb][0] = mlp::pack_bf16(v[0][0], v[0][1]);
                x[kb][1] = mlp::pack_bf16(v[1][0], v[1][1]);
                x[kb][2] = mlp::pack_bf16(v[2][0], v[2][1]);
                x[kb][3] = mlp::pack_bf16(v[3][0], v[3][1]);
            }
            float out[4];
            mlp::forward_tile(sw, x, out);
            __syncwarp();
            // corrections of rows g and g+8, columns 2t, 2t+1 -> shared tile
#pragma unroll
            for (int e2 = 0; e2 < 2; ++e2) {
                const int col = 2 * t + e2;
                if (col < 3) {
                    tl[g][col] = out[e2];
                    tl[g + 8][col] = out[2 + e2];
                }
            }
            __syncwarp();
        }
        {
            const int i = row0 + lane;
            const float4 info = m.info[i];
            if (info.z != 2.f) {
                float hx = st.uh[i].x, hy = st.uh[i].y, hz = st.uh[i].z;
                float lx = st.ul[i].x, ly = st.ul[i].y, lz = st.ul[i].z;
                if (info.z == 0.f && net.base == 1) {
                    // the constant-acceleration extrapolation of the last two
                    // displacements: u0 + d1 + (d1 - d2)
                    const float4 h0 = st.u0h[i], l0 = st.u0l[i], d1 = st.hist1[i], d2 = st.hist2[i];
                    hx = h0.x; hy = h0.y; hz = h0.z;
                    lx = l0.x; ly = l0.y; lz = l0.z;
                    add_comp(hx, lx, d1.x + (d1.x - d2.x));
                    add_comp(hy, ly, d1.y + (d1.y - d2.y));
                    add_comp(hz, lz, d1.z + (d1.z - d2.z));
                }
                if (info.z == 0.f) {
                    const float sc = tscale[w][lane];
                    add_comp(hx, lx, tile[w][lane][0] * os[0] * sc);
                    add_comp(hy, ly, tile[w][lane][1] * os[1] * sc);
                    add_comp(hz, lz, tile[w][lane][2] * os[2] * sc);
                }
                st.uh[m.Np + i] = make_float4(hx, hy, hz, 0.f);
                st.ul[m.Np + i] = make_float4(lx, ly, lz, 0.f);
            }
        }
        __syncwarp();
    }
}

// Energies of the plain guess (parity 0) and the candidate (parity 1).
// residual: also require the candidate's |g| below the plain guess's (the
// extrapolation base, whose energy can undercut the plain guess's while its
// gradient, which the stop test measures, is larger).
__global__ void __launch_bounds__(BLOCK) k_ws_judge(DevMesh m, DevParams p, DevState st, int residual) {
    __shared__ double sh[BLOCK / 32];
    __shared__ int is_last;
    const int b = blockIdx.x;
    InstCtl *cp = st.ctl + m.tblk_inst[b];
    if (cp->done) return;
    const int t = b * BLOCK + threadIdx.x;
    double e0 = 0.0, e1 = 0.0;
    const int4 q = m.tets[t];
    if (q.x >= 0) {
        const float4 r0 = m.row0[t], r1 = m.row1[t], r2 = m.row2[t];
        const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
        for (int s = 0; s < 2; ++s) {
            const float4 *U = st.uh + (size_t)s * m.Np;
            Kin<float> kin;
            disp_gradient<float>(U[q.x], U[q.y], U[q.z], U[q.w], dinv, kin.G);
            kinematics(kin);
            const double e =
                (double)search_energy(energy_density<float>(kin, r1.w, r2.w) * fabsf(r0.w), p.clamp_cpu, true);
            if (s == 0) e0 = e; else e1 = e;
        }
    }
    const int nb = cp->tblk_end - cp->tblk_begin;
    for (int i = cp->node_begin + (b - cp->tblk_begin) * BLOCK + threadIdx.x; i < cp->node_end; i += nb * BLOCK) {
        const float4 info = m.info[i];
        if (info.z != 0.f) continue;
        e0 += node_energy(st, info, st.uh[i], st.ul[i], i, p.h2inv);
        e1 += node_energy(st, info, st.uh[m.Np + i], st.ul[m.Np + i], i, p.h2inv);
    }
    const double s0 = block_sum(e0, sh);
    const double s1 = block_sum(e1, sh);
    if (threadIdx.x == 0) {
        st.tpart[b] = make_double2(s0, s1);
        __threadfence();
        const unsigned int prev = atomicAdd(&cp->counter_t, 1u);
        is_last = (prev == (unsigned int)(nb - 1));
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double E0 = 0.0, E1 = 0.0;
    for (int j = cp->tblk_begin + threadIdx.x; j < cp->tblk_end; j += BLOCK) {
        const double2 v = __ldcg(st.tpart + j);
        E0 += v.x;
        E1 += v.y;
    }
    E0 = block_sum(E0, sh);
    E1 = block_sum(E1, sh);
    if (threadIdx.x == 0) {
        cp->counter_t = 0;
        // a finite candidate also wins over a plain guess whose energy is not finite
        cp->ws_used = (isfinite(E1) && (E1 <= E0 || !isfinite(E0)) && (!residual || cp->g1 < cp->g0)) ? 1 : 0;
    }
}

__global__ void k_ws_select(DevMesh m, DevState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    if (!node_ctl_ws(m, st, i)) return;
    st.uh[i] = st.uh[m.Np + i];
    st.ul[i] = st.ul[m.Np + i];
}

// A caller-supplied candidate (parity 1) keeps the prescribed positions of
// pinned nodes, as the plain guess (parity 0) has them.
__global__ void k_ws_guess_pins(DevMesh m, DevState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    if (m.info[i].z == 0.f) return;
    st.uh[m.Np + i] = st.uh[i];
    st.ul[m.Np + i] = st.ul[i];
}

static inline int nblk(int n, int b) { return (n + b - 1) / b; }

cudaError_t launch_ws_choose(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st) {
    k_ws_guess_pins<<<nblk(m.Np, 256), 256, 0, s>>>(m, st);
    k_ws_judge<<<m.n_tblk, BLOCK, 0, s>>>(m, p, st, 0);
    k_ws_select<<<nblk(m.Np, 256), 256, 0, s>>>(m, st);
    return cudaGetLastError();
}

cudaError_t launch_ws_gref(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, int material) {
    // without incremental stress the elastic force at the plain guess is not in b
    if (material == PBS_MATERIAL_STRETCH)
        k_ws_force<PBS_MATERIAL_STRETCH><<<m.n_tblk, BLOCK, 0, s>>>(m, p, st, st.uh);
    else if (!p.incremental)
        k_ws_force<PBS_MATERIAL_NEOHOOKEAN><<<m.n_tblk, BLOCK, 0, s>>>(m, p, st, st.uh);
    k_ws_gref<<<m.n_nblk, BLOCK, 0, s>>>(m, p, st);
    return cudaGetLastError();
}

cudaError_t launch_ws_predict(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, const float *theta,
                              const float *feat_mean, const float *feat_std, const float *out_std, float *tetF,
                              int sms, int base, int material) {
    k_ws_tet_F<<<nblk(m.Tp, 256), 256, 0, s>>>(m, st, tetF);
    WsNet net{theta, feat_mean, feat_std, out_std, base};
    const int rows32 = nblk(m.Np, 32);  // 32 nodes a warp and iteration
    const int blocks = std::min(nblk(rows32, 4), 8 * sms);
    k_ws_infer<<<blocks, 128, 0, s>>>(m, p, st, tetF, net);
    if (base == 1) {  // the candidate's gradient for the residual test
        DevState s1 = st;
        s1.ul = st.ul + m.Np;
        if (material == PBS_MATERIAL_STRETCH)
            k_ws_force<PBS_MATERIAL_STRETCH><<<m.n_tblk, BLOCK, 0, s>>>(m, p, s1, st.uh + m.Np);
        else
            k_ws_force<PBS_MATERIAL_NEOHOOKEAN><<<m.n_tblk, BLOCK, 0, s>>>(m, p, s1, st.uh + m.Np);
        k_ws_gcand<<<m.n_nblk, BLOCK, 0, s>>>(m, p, st);
    }
    k_ws_judge<<<m.n_tblk, BLOCK, 0, s>>>(m, p, st, base == 1);
    k_ws_select<<<nblk(m.Np, 256), 256, 0, s>>>(m, st);
    return cudaGetLastError();
}

cudaError_t launch_ws_features(cudaStream_t s, const DevMesh &m, const DevParams &p, DevState st, float *tetF,
                               const int *pad2user, float *out, float *scale_out) {
    k_ws_tet_F<<<nblk(m.Tp, 256), 256, 0, s>>>(m, st, tetF);
    k_ws_features<<<nblk(m.Np, 128), 128, 0, s>>>(m, p, st, tetF, pad2user, out, scale_out);
    return cudaGetLastError();
}

}  // namespace pbs
