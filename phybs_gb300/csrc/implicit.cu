// Linearly implicit (backward) Euler step: the reference's second GPU
// integrator, CUDAInterface::computeInnerforces + computeGlobalStiffnessMatrix
// + doBackEuler (CUDAInterface.cu:784-884):
//
//   f = elastic forces + gravity (+ external); a pinned node's force is the
//       spring 1e8 (X - x)                       (addFixContraintsAndGravity :327)
//   A v' = b,  A = M (1 + alpha h) + h (h + beta) K,  b = h f + M v
//   x' = x + h v'
//
// K = -df/dx is the closed-form Hessian of the neo-Hookean energy (the energy
// both materials share; the reference's Xu et al. SVD-derivative dP/dF is the
// same derivative for an uninverted tet):
//   K[c d, c' e] = vol (mu (w_c . w_c') delta_de + lam a_c[d] a_c'[e]
//                       + (mu - lam ln J) a_c[e] a_c'[d]),   a_c = F^-T w_c.
//
// GB300 design instead of the reference's atomics into a scalar CSR and a
// cuSOLVER Cholesky:
//   * 3x3 block-CSR (BSR) over padded nodes; one thread owns a block row and
//     adds its incident (tet, corner) terms in the incidence order (ascending
//     tet): no atomics, bit-reproducible;
//   * block-Jacobi preconditioned conjugate gradients (3x3 diagonal blocks
//     inverted in FP64), FP32 vectors as float4, FP64 dot products reduced in
//     a fixed order; the solve stops on |r| <= tol |b|.
#include <cuda_runtime.h>

#include "../../include/phybs.h"
#include "phybs_internal.cuh"
#include "tet_math.cuh"

namespace pbs {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float4 f4(float x, float y, float z) { return make_float4(x, y, z, 0.f); }

// index of padded node col in block row i (columns ascending)
__device__ __forceinline__ int bsr_find(const int *col, int b, int e, int target) {
    while (b < e) {
        const int mid = (b + e) >> 1;
        if (col[mid] < target) b = mid + 1;
        else e = mid;
    }
    return b;
}

__device__ __forceinline__ void add_block(float *v, float s, const float K[9]) {
#pragma unroll
    for (int k = 0; k < 9; ++k) v[k] += s * K[k];
}

// Row i of A, b, the block-Jacobi inverse and the initial guess (v).
template <int MATERIAL>
__global__ void __launch_bounds__(128) k_be_assemble(DevMesh m, DevState st, BsrView A, float dt, float alpha,
                                                     float beta, const float4 *ext, float4 *b, float4 *x,
                                                     float *dinv9) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const int rb = A.ptr[i], re = A.ptr[i + 1];
    float *row = A.val + 9 * (size_t)rb;
    for (int k = 0; k < 9 * (re - rb); ++k) row[k] = 0.f;
    const float4 info = m.info[i];
    const int dslot = bsr_find(A.col, rb, re, i) - rb;
    if (info.z == 2.f) {  // padding node: identity row, zero right-hand side
        float *d = row + 9 * dslot;
        d[0] = d[4] = d[8] = 1.f;
        b[i] = x[i] = f4(0.f, 0.f, 0.f);
        for (int k = 0; k < 9; ++k) dinv9[9 * (size_t)i + k] = (k % 4 == 0) ? 1.f : 0.f;
        return;
    }
    const float sK = dt * (dt + beta);
    float fx = 0.f, fy = 0.f, fz = 0.f;
    for (int j = m.inc_ptr[i]; j < m.inc_ptr[i + 1]; ++j) {
        const int ent = m.inc[j], t = ent >> 2, c = ent & 3;
        const int4 q = m.tets[t];
        const int qn[4] = {q.x, q.y, q.z, q.w};
        const float4 r0 = m.row0[t], r1 = m.row1[t], r2 = m.row2[t];
        const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
        const float svol = r0.w, mu = r1.w, lam = r2.w;
        // G from the full (hi, lo) displacements, differences first
        const float4 h0 = st.u0h[q.x], l0 = st.u0l[q.x];
        float4 du[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float4 hk = st.u0h[qn[k + 1]], lk = st.u0l[qn[k + 1]];
            du[k] = f4((hk.x - h0.x) + (lk.x - l0.x), (hk.y - h0.y) + (lk.y - l0.y), (hk.z - h0.z) + (lk.z - l0.z));
        }
        Kin<float> kin;
        disp_gradient<float>(f4(0.f, 0.f, 0.f), du[0], du[1], du[2], dinv, kin.G);
        kinematics(kin);
        float P[9];
        if (MATERIAL == PBS_MATERIAL_STRETCH) pk1_stretch(kin, mu, lam, P);
        else pk1_neohookean<float>(kin, mu, lam, P);
        // corner shape gradients w_0..3 (w_1..3 = rows of Dm^-1)
        float w[4][3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            w[k + 1][0] = dinv[3 * k];
            w[k + 1][1] = dinv[3 * k + 1];
            w[k + 1][2] = dinv[3 * k + 2];
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) w[0][d] = -(w[1][d] + w[2][d] + w[3][d]);
        // the corner force -svol P w_c (corner_forces' rows for this corner)
        float wc[3] = {w[c][0], w[c][1], w[c][2]};
        fx -= svol * (P[0] * wc[0] + P[1] * wc[1] + P[2] * wc[2]);
        fy -= svol * (P[3] * wc[0] + P[4] * wc[1] + P[5] * wc[2]);
        fz -= svol * (P[6] * wc[0] + P[7] * wc[1] + P[8] * wc[2]);
        float H[9];
        inv_transpose<float>(kin, H);
        float ac[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) ac[d] = H[3 * d] * wc[0] + H[3 * d + 1] * wc[1] + H[3 * d + 2] * wc[2];
        const float cm = mu - lam * kin.lnJ;
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
            float a2[3];
#pragma unroll
            for (int d = 0; d < 3; ++d)
                a2[d] = H[3 * d] * w[cc][0] + H[3 * d + 1] * w[cc][1] + H[3 * d + 2] * w[cc][2];
            const float ww = wc[0] * w[cc][0] + wc[1] * w[cc][1] + wc[2] * w[cc][2];
            float K[9];
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int e = 0; e < 3; ++e)
                    K[3 * d + e] = svol * ((d == e ? mu * ww : 0.f) + lam * ac[d] * a2[e] + cm * ac[e] * a2[d]);
            const int slot = bsr_find(A.col, rb, re, qn[cc]) - rb;
            add_block(row + 9 * slot, sK, K);
        }
    }
    // the diagonal block's mass term and the right-hand side
    const float mass = info.x, ms = mass * (1.f + alpha * dt);
    float *d = row + 9 * dslot;
    d[0] += ms;
    d[4] += ms;
    d[8] += ms;
    const float4 uh = st.u0h[i], ul = st.u0l[i];
    if (info.z == 1.f) {  // pinned: the spring 1e8 (X - x)
        fx = -1e8f * (uh.x + ul.x);
        fy = -1e8f * (uh.y + ul.y);
        fz = -1e8f * (uh.z + ul.z);
    } else {
        fy += info.y;  // gravity
        if (ext) {
            const float4 e = ext[i];
            fx += e.x;
            fy += e.y;
            fz += e.z;
        }
    }
    const float4 v = st.v[i];
    b[i] = f4(dt * fx + mass * v.x, dt * fy + mass * v.y, dt * fz + mass * v.z);
    x[i] = v;
    // block-Jacobi: the diagonal block's inverse, in FP64
    double D[9], C[9];
    for (int k = 0; k < 9; ++k) D[k] = d[k];
    cofactor3<double>(D, C);
    const double det = D[0] * C[0] + D[1] * C[1] + D[2] * C[2];
    for (int r = 0; r < 3; ++r)
        for (int cl = 0; cl < 3; ++cl) dinv9[9 * (size_t)i + 3 * r + cl] = (float)(C[3 * cl + r] / det);
}

__device__ __forceinline__ float4 bsr_row_mul(const BsrView &A, int i, const float4 *p) {
    float sx = 0.f, sy = 0.f, sz = 0.f;
    if (A.scalar) {  // blocks a I3: one value a block
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            const float a = A.val[k];
            const float4 v = p[A.col[k]];
            sx += a * v.x;
            sy += a * v.y;
            sz += a * v.z;
        }
        return f4(sx, sy, sz);
    }
    for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
        const float *a = A.val + 9 * (size_t)k;
        const float4 v = p[A.col[k]];
        sx += a[0] * v.x + a[1] * v.y + a[2] * v.z;
        sy += a[3] * v.x + a[4] * v.y + a[5] * v.z;
        sz += a[6] * v.x + a[7] * v.y + a[8] * v.z;
    }
    return f4(sx, sy, sz);
}

__device__ __forceinline__ float4 block_apply(const float *D, const float4 &r) {
    return f4(D[0] * r.x + D[1] * r.y + D[2] * r.z, D[3] * r.x + D[4] * r.y + D[5] * r.z,
              D[6] * r.x + D[7] * r.y + D[8] * r.z);
}

__device__ __forceinline__ double dot4(const float4 &a, const float4 &b) {
    return (double)a.x * b.x + (double)a.y * b.y + (double)a.z * b.z;
}

// Fixed-order block sums of up to three doubles into part[k * nblk + block].
__device__ __forceinline__ void block_sums(double a0, double a1, double a2, int nv, double *part, int nblk) {
    __shared__ double sh[3][kThreads / 32];
    double v[3] = {a0, a1, a2};
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < nv; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        if (lane == 0) sh[k][w] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < nv) {
        double s = 0.0;
        for (int j = 0; j < (int)(blockDim.x >> 5); ++j) s += sh[threadIdx.x][j];
        part[threadIdx.x * nblk + blockIdx.x] = s;
    }
}

// r = b - A x, z = D^-1 r, p = z; partial r.z, r.r and b.b (pnorm = 0) or
// b.D^-1 b (pnorm = 1, the preconditioned norm)
__global__ void __launch_bounds__(kThreads) k_cg_init(int Np, BsrView A, const float *dinv9, const float4 *b,
                                                      const float4 *x, float4 *r, float4 *z, float4 *p,
                                                      double *part, int pnorm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rz = 0.0, rr = 0.0, bb = 0.0;
    if (i < Np) {
        const float4 ax = bsr_row_mul(A, i, x), bi = b[i];
        const float4 ri = f4(bi.x - ax.x, bi.y - ax.y, bi.z - ax.z);
        const float4 zi = block_apply(dinv9 + 9 * (size_t)i, ri);
        r[i] = ri;
        z[i] = zi;
        p[i] = zi;
        rz = dot4(ri, zi);
        rr = dot4(ri, ri);
        bb = pnorm ? dot4(bi, block_apply(dinv9 + 9 * (size_t)i, bi)) : dot4(bi, bi);
    }
    block_sums(rz, rr, bb, 3, part, gridDim.x);
}

// q = A p; partial p.q
__global__ void __launch_bounds__(kThreads) k_cg_spmv(int Np, BsrView A, const float4 *p, float4 *q, double *part,
                                                      const CgState *cs) {
    if (cs->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double pq = 0.0;
    if (i < Np) {
        const float4 qi = bsr_row_mul(A, i, p);
        q[i] = qi;
        pq = dot4(p[i], qi);
    }
    block_sums(pq, 0.0, 0.0, 1, part, gridDim.x);
}

// x += alpha p, r -= alpha q, z = D^-1 r; partial r.z, r.r
__global__ void __launch_bounds__(kThreads) k_cg_update(int Np, const float *dinv9, const float4 *p, const float4 *q,
                                                        float4 *x, float4 *r, float4 *z, double *part,
                                                        const CgState *cs) {
    if (cs->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rz = 0.0, rr = 0.0;
    if (i < Np) {
        const float a = (float)cs->alpha;
        const float4 pi = p[i], qi = q[i], xi = x[i], ri0 = r[i];
        x[i] = f4(xi.x + a * pi.x, xi.y + a * pi.y, xi.z + a * pi.z);
        const float4 ri = f4(ri0.x - a * qi.x, ri0.y - a * qi.y, ri0.z - a * qi.z);
        const float4 zi = block_apply(dinv9 + 9 * (size_t)i, ri);
        r[i] = ri;
        z[i] = zi;
        rz = dot4(ri, zi);
        rr = dot4(ri, ri);
    }
    block_sums(rz, rr, 0.0, 2, part, gridDim.x);
}

// p = z + beta p
__global__ void __launch_bounds__(kThreads) k_cg_direction(int Np, const float4 *z, float4 *p, const CgState *cs) {
    if (cs->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Np) return;
    const float bt = (float)cs->beta;
    const float4 zi = z[i], pi = p[i];
    p[i] = f4(zi.x + bt * pi.x, zi.y + bt * pi.y, zi.z + bt * pi.z);
}

// The scalars of one CG stage from the block partials, summed in block order
// by one CTA.  stage 0: after init; 1: alpha = rz / pq; 2: beta, convergence
// (|r|^2 <= tol2 |b|^2, or r.D^-1 r <= tol2 b.D^-1 b when pnorm).
__global__ void __launch_bounds__(kThreads) k_cg_scalars(int nblk, const double *part, CgState *cs, int stage,
                                                         double tol2, int max_iters, int pnorm) {
    __shared__ double sh[3][kThreads / 32];
    const int nv = stage == 1 ? 1 : (stage == 0 ? 3 : 2);
    if (cs->done && stage != 0) return;
    double v[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < nv; ++k)
        for (int j = threadIdx.x; j < nblk; j += blockDim.x) v[k] += part[k * nblk + j];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < nv; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        if (lane == 0) sh[k][w] = v[k];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double s[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < nv; ++k)
        for (int j = 0; j < (int)(blockDim.x >> 5); ++j) s[k] += sh[k][j];
    CgState &c = *cs;
    if (stage == 0) {
        c.rz = s[0];
        c.rr = s[1];
        c.bb = s[2];
        c.iters = 0;
        c.status = PBS_OK;
        c.done = 0;
        if (!((pnorm ? s[0] : s[1]) <= tol2 * s[2])) {
            if (!isfinite(s[1])) { c.status = PBS_E_NONFINITE; c.done = 1; }
        } else {
            c.done = 1;  // the initial guess already solves it
        }
    } else if (stage == 1) {
        c.alpha = s[0] != 0.0 ? c.rz / s[0] : 0.0;
        if (!isfinite(c.alpha) || s[0] <= 0.0) { c.status = PBS_E_NONFINITE; c.done = 1; }
    } else {
        c.iters += 1;
        c.beta = c.rz != 0.0 ? s[0] / c.rz : 0.0;
        c.rz = s[0];
        c.rr = s[1];
        if (!isfinite(s[1])) { c.status = PBS_E_NONFINITE; c.done = 1; }
        else if ((pnorm ? s[0] : s[1]) <= tol2 * c.bb) c.done = 1;
        else if (c.iters >= max_iters) { c.status = PBS_E_ITER_CAP; c.done = 1; }
    }
}

// v_old <- v, v <- v', u += dt v' (compensated)
__global__ void k_be_finish(DevMesh m, DevState st, const float4 *x, float dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np || m.info[i].z == 2.f) return;
    const float4 vn = x[i];
    float4 hi = st.u0h[i], lo = st.u0l[i];
    add_comp(hi.x, lo.x, dt * vn.x);
    add_comp(hi.y, lo.y, dt * vn.y);
    add_comp(hi.z, lo.z, dt * vn.z);
    st.u0h[i] = hi;
    st.u0l[i] = lo;
    st.vold[i] = st.v[i];
    st.v[i] = vn;
}

}  // namespace

int cg_blocks(int Np) { return (Np + kThreads - 1) / kThreads; }

cudaError_t launch_be_assemble(cudaStream_t s, const DevMesh &m, const DevState &st, int material, const BsrView &A,
                               float dt, float alpha, float beta, const float4 *ext, float4 *b, float4 *x,
                               float *dinv9) {
    const int g = (m.Np + 127) / 128;
    if (material == PBS_MATERIAL_STRETCH)
        k_be_assemble<PBS_MATERIAL_STRETCH><<<g, 128, 0, s>>>(m, st, A, dt, alpha, beta, ext, b, x, dinv9);
    else
        k_be_assemble<PBS_MATERIAL_NEOHOOKEAN><<<g, 128, 0, s>>>(m, st, A, dt, alpha, beta, ext, b, x, dinv9);
    return cudaGetLastError();
}

cudaError_t launch_cg_init(cudaStream_t s, int Np, const BsrView &A, const float *dinv9, const float4 *b,
                           const float4 *x, float4 *r, float4 *z, float4 *p, double *part, CgState *cs, double tol2,
                           int pnorm) {
    const int g = cg_blocks(Np);
    k_cg_init<<<g, kThreads, 0, s>>>(Np, A, dinv9, b, x, r, z, p, part, pnorm);
    k_cg_scalars<<<1, kThreads, 0, s>>>(g, part, cs, 0, tol2, 0, pnorm);
    return cudaGetLastError();
}

cudaError_t launch_cg_iteration(cudaStream_t s, int Np, const BsrView &A, const float *dinv9, float4 *x, float4 *r,
                                float4 *z, float4 *p, float4 *q, double *part, CgState *cs, double tol2,
                                int max_iters, int pnorm) {
    const int g = cg_blocks(Np);
    k_cg_spmv<<<g, kThreads, 0, s>>>(Np, A, p, q, part, cs);
    k_cg_scalars<<<1, kThreads, 0, s>>>(g, part, cs, 1, tol2, max_iters, pnorm);
    k_cg_update<<<g, kThreads, 0, s>>>(Np, dinv9, p, q, x, r, z, part, cs);
    k_cg_scalars<<<1, kThreads, 0, s>>>(g, part, cs, 2, tol2, max_iters, pnorm);
    k_cg_direction<<<g, kThreads, 0, s>>>(Np, z, p, cs);
    return cudaGetLastError();
}

cudaError_t launch_be_finish(cudaStream_t s, const DevMesh &m, const DevState &st, const float4 *x, float dt) {
    k_be_finish<<<(m.Np + 255) / 256, 256, 0, s>>>(m, st, x, dt);
    return cudaGetLastError();
}

}  // namespace pbs
