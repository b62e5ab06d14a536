// The reference's two other CPU integrators, on the device:
//
// Strain-based position-based dynamics (PosBaseDynamic.cpp:12-117, Mueller et
// al. 2014): Gauss-Seidel sweeps over the tets in the caller's order.  A
// serial sweep is reproduced exactly by dependency levels: a tet's level is
// one more than the highest level of the earlier tets that share one of its
// nodes, so a level's tets share no node and each reads exactly the updates of
// the tets before it in the serial order.  One thread-block cluster sweeps an
// instance level by level (16 CTAs when the handle holds few instances, else
// 8), the cluster barrier ordering the levels (its arrive/wait carry
// release/acquire semantics for the global positions):
// 2,320 levels of ~430 tets for the 1M-tet box, 920 for the 24K bar.  The
// arithmetic is FP32 with every product and sum rounded separately (no
// contraction) in Eigen 3.2's order, so a sweep is the CPU's bit for bit.
//
// Projective dynamics (ProjDynamic.cpp:48-100, 351-480): per-tet polar
// rotations from the modified SVD and the constant global matrix A = L (x) I3.
// A p and b are of the size of the positions times the stiffness, and an
// FP32 A's rows do not sum to zero exactly, so applied to absolute positions
// it would add forces proportional to the distance from the origin.  Each
// global solve is therefore a correction from a residual formed without
// absolute coordinates: r = b - A p = M / dt^2 ((x - p) + q) +
// sum_t k vol (R - F) w_a (edge differences only), A d = r by the
// block-Jacobi conjugate gradients of the backward-Euler step, p += d.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "../../include/phybs.h"
#include "phybs_internal.cuh"
#include "tet_math.cuh"

namespace cg = cooperative_groups;

namespace pbs {

namespace {

// CTAs a PBD cluster sweeps an instance with: 16 (the non-portable maximum,
// opted into at launch) when a handle holds few instances, else 8
constexpr int kPbdClusterMax = 16;
constexpr int kPbdThreads = 128;

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
// Eigen 3.2's 3-vector dot / squaredNorm: x0 + (x1 + x2)
__device__ __forceinline__ float dot3e(const float a[3], const float b[3]) {
    return fadd(fmul(a[0], b[0]), fadd(fmul(a[1], b[1]), fmul(a[2], b[2])));
}

// float(((double)S - 1.0) / (double)lam * (double)k): the reference's stretch
// multiplier, whose double literal makes it FP64 (PosBaseDynamic.cpp:100).
// GB300's FP64 pipe is narrow, so the value is formed in double-float FP32
// (error below 2^-44 relative) and rounded; the FP64 expression is evaluated
// only when that value lies within 2^-40 relative of a float rounding
// boundary, where the two roundings could differ (or for zero, non-finite or
// tiny values).  Published methods used: the quotient is Markstein's
// correction of an approximate reciprocal by its exact FMA remainder
// r = a - q b (P. Markstein, "IA-64 and Elementary Functions", 2000, ch. 8);
// S - 1 and the product by k use the error-free transformations TwoSum
// (Knuth, TAOCP vol. 2, 4.2.2) and the FMA form of TwoProduct (Ogita, Rump
// and Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005),
// and the final renormalisation is Dekker's FastTwoSum (Dekker, Numer. Math.
// 18, 1971).  The boundary test then decides whether the double-float value
// determines the FP32 rounding of the exact FP64 quotient.
__device__ __forceinline__ float pbd_stretch_mult(float S, float lam, float k) {
    float ah, al;
    two_sum(S, -1.0f, ah, al);  // S - 1 = ah + al exactly
    if (ah == 0.0f && al == 0.0f) return fmul(0.0f, k);
    // (ah + al) / lam as q1 + q2 from one approximate reciprocal: q1 is within
    // a few ulp, the remainder ah - q1 lam is formed by one fma (exact, or
    // rounded at 2^-24 of itself) and corrected by q2; |error| < 2^-45 of the
    // quotient, well inside the boundary test's 2^-40 margin below
    float inv;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(lam));
    const float q1 = fmul(ah, inv);
    const float r = fadd(__fmaf_rn(-q1, lam, ah), al);
    const float q2 = fmul(r, inv);
    const float p1 = fmul(q1, k);
    const float p2 = __fmaf_rn(q2, k, __fmaf_rn(q1, k, -p1));  // q1 k - p1 is exact
    const float c = fadd(p1, p2);
    const float d = fadd(fsub(p1, c), p2);  // (p1 + p2) - c
    const float ac = fabsf(c);
    if (ac < 1e-30f || ac > 1e30f || !isfinite(ac))
        return __double2float_rn(__dmul_rn(__ddiv_rn(__dsub_rn((double)S, 1.0), (double)lam), (double)k));
    // the float boundary on d's side of c: half the gap to the neighbour
    const float away = __int_as_float(__float_as_int(ac) + 1), toward = __int_as_float(__float_as_int(ac) - 1);
    const float half = ((d >= 0.0f) == (c >= 0.0f)) ? 0.5f * (away - ac) : 0.5f * (ac - toward);
    if (fabsf(d) + ac * 0x1p-40f < half) return c;
    return __double2float_rn(__dmul_rn(__ddiv_rn(__dsub_rn((double)S, 1.0), (double)lam), (double)k));
}

struct PbdConst {
    float stretch[3], shear[3], eps;
};

// solveStrainConstraints (PosBaseDynamic.cpp:55-117) for one tet: p[c].xyz
// the corner positions, p[c].w the inverse masses, D = Dm^-1 row-major.
__device__ __forceinline__ void pbd_project(const float4 p[4], const float D[9], const PbdConst &k, float dp[4][3]) {
    const float pw[4] = {p[0].w, p[1].w, p[2].w, p[3].w};
#pragma unroll
    for (int c = 0; c < 4; ++c) dp[c][0] = dp[c][1] = dp[c][2] = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            const float x0[3] = {fadd(p[0].x, dp[0][0]), fadd(p[0].y, dp[0][1]), fadd(p[0].z, dp[0][2])};
            float P[3][3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float4 &q = p[c + 1];
                P[0][c] = fsub(fadd(q.x, dp[c + 1][0]), x0[0]);
                P[1][c] = fsub(fadd(q.y, dp[c + 1][1]), x0[1]);
                P[2][c] = fsub(fadd(q.z, dp[c + 1][2]), x0[2]);
            }
            float fi[3], fj[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                fi[r] = fadd(fadd(fmul(P[r][0], D[i]), fmul(P[r][1], D[3 + i])), fmul(P[r][2], D[6 + i]));
                fj[r] = fadd(fadd(fmul(P[r][0], D[j]), fmul(P[r][1], D[3 + j])), fmul(P[r][2], D[6 + j]));
            }
            const float S = dot3e(fi, fj);
            float d[4][3];
#pragma unroll
            for (int r = 0; r < 3; ++r) d[0][r] = 0.f;
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    d[kk + 1][r] = fadd(fmul(fj[r], D[3 * kk + i]), fmul(fi[r], D[3 * kk + j]));
                    d[0][r] = fsub(d[0][r], d[kk + 1][r]);
                }
            float lam = fmul(pw[0], dot3e(d[0], d[0]));
            lam = fadd(lam, fmul(pw[1], dot3e(d[1], d[1])));
            lam = fadd(lam, fmul(pw[2], dot3e(d[2], d[2])));
            lam = fadd(lam, fmul(pw[3], dot3e(d[3], d[3])));
            if (lam < k.eps) continue;
            if (i == j) lam = pbd_stretch_mult(S, lam, k.stretch[i]);
            else lam = fmul(__fdiv_rn(S, lam), k.shear[i + j - 1]);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float s = fmul(lam, pw[c]);
#pragma unroll
                for (int r = 0; r < 3; ++r) dp[c][r] = fsub(dp[c][r], fmul(s, d[c][r]));
            }
        }
    }
}

// A level-ordered tet's static record (ids, Dm^-1 rows).
struct PbdTet {
    int4 q;
    float4 r0, r1, r2;
};

__device__ __forceinline__ PbdTet pbd_load(const PbdView &v, int j) {
    PbdTet t;
    t.q = __ldg(v.tet + j);
    t.r0 = __ldg(v.d0 + j);
    t.r1 = __ldg(v.d1 + j);
    t.r2 = __ldg(v.d2 + j);
    return t;
}

__device__ __forceinline__ void pbd_apply(const PbdView &v, const PbdTet &t, const PbdConst &k) {
    const float D[9] = {t.r0.x, t.r0.y, t.r0.z, t.r1.x, t.r1.y, t.r1.z, t.r2.x, t.r2.y, t.r2.z};
    const int id[4] = {t.q.x, t.q.y, t.q.z, t.q.w};
    float4 p[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) p[c] = __ldcg(v.px + id[c]);
    float dp[4][3];
    pbd_project(p, D, k, dp);
#pragma unroll
    for (int c = 0; c < 4; ++c)
        v.px[id[c]] = make_float4(fadd(p[c].x, dp[c][0]), fadd(p[c].y, dp[c][1]), fadd(p[c].z, dp[c][2]), p[c].w);
}

// One cluster per group of levels (an instance): `iterations` sweeps over its
// levels; a level's tets are split into one contiguous run per CTA of the
// cluster.  Positions are read through L2 (ld.global.cg); the cluster barrier
// orders one level's writes before the next level's reads.  A thread's first
// static record of the next level is loaded before the barrier, so a level's
// dependent chain starts at the position loads.
__global__ void __launch_bounds__(kPbdThreads) k_pbd_sweep(PbdView v, int iterations, PbdConst k) {
    cg::cluster_group cl = cg::this_cluster();
    const int csize = (int)cl.num_blocks();
    const int g = blockIdx.x / csize;
    const int rank = (int)cl.block_rank();
    const int l0 = v.grp[g], l1 = v.grp[g + 1];
    if (l0 == l1 || iterations <= 0) return;  // uniform over the cluster
    // this thread's run [j, b1) of level l
    auto run_of = [&](int l, int &j, int &b1) {
        const int a = v.lvl[l], e = v.lvl[l + 1];
        const int chunk = (e - a + csize - 1) / csize;
        const int b0 = a + rank * chunk;
        b1 = min(b0 + chunk, e);
        j = b0 + (int)threadIdx.x;
    };
    int j, b1;
    run_of(l0, j, b1);
    PbdTet cur = pbd_load(v, j < b1 ? j : v.lvl[l0]);
    const int total = iterations * (l1 - l0);
    for (int s = 0; s < total; ++s) {
        const int l = l0 + s % (l1 - l0);
        // next level's first record (for the last level of the last sweep: none)
        int jn = 0, bn = 0;
        PbdTet nxt = cur;
        if (s + 1 < total) {
            const int ln = l + 1 < l1 ? l + 1 : l0;
            run_of(ln, jn, bn);
            if (jn < bn) nxt = pbd_load(v, jn);
        }
        if (j < b1) pbd_apply(v, cur, k);
        for (int jj = j + kPbdThreads; jj < b1; jj += kPbdThreads) pbd_apply(v, pbd_load(v, jj), k);
        cl.sync();
        cur = nxt;
        j = jn;
        b1 = bn;
    }
}

// The same sweep with the instance's positions held in the cluster's
// distributed shared memory: CTA r of the 16 keeps nodes [r S, (r + 1) S) of
// the instance, and a tet corner is addressed by its code (owner CTA << 16 |
// offset), so every level's position loads and stores go SM to SM instead of
// through L2, and the cluster barrier releases shared-memory writes only.
// Used when an instance's nodes fit (S * 16 B of dynamic shared memory a CTA).
__device__ __forceinline__ float4 *dsm_node(cg::cluster_group &cl, float4 *s_px, int code) {
    return cl.map_shared_rank(s_px, (unsigned)code >> 16) + (code & 0xffff);
}

__global__ void __launch_bounds__(kPbdThreads)
    k_pbd_sweep_dsmem(PbdView v, const int4 *codes, const int4 *gnode, int iterations, PbdConst k) {
    extern __shared__ float4 s_px[];
    cg::cluster_group cl = cg::this_cluster();
    const int csize = (int)cl.num_blocks();
    const int g = blockIdx.x / csize;
    const int rank = (int)cl.block_rank();
    const int4 gn = gnode[g];  // {first padded node, slice S, node count}
    const int nb = gn.x, S = gn.y, cnt = gn.z;
    for (int j = threadIdx.x; j < S; j += kPbdThreads) {
        const int n = rank * S + j;
        if (n < cnt) s_px[j] = v.px[nb + n];
    }
    cl.sync();
    const int l0 = v.grp[g], l1 = v.grp[g + 1];
    const int total = iterations > 0 ? iterations * (l1 - l0) : 0;
    auto run_of = [&](int l, int &j, int &b1) {
        const int a = v.lvl[l], e = v.lvl[l + 1];
        const int chunk = (e - a + csize - 1) / csize;
        const int b0 = a + rank * chunk;
        b1 = min(b0 + chunk, e);
        j = b0 + (int)threadIdx.x;
    };
    auto apply = [&](const PbdTet &t) {
        const float D[9] = {t.r0.x, t.r0.y, t.r0.z, t.r1.x, t.r1.y, t.r1.z, t.r2.x, t.r2.y, t.r2.z};
        float4 *ptr[4] = {dsm_node(cl, s_px, t.q.x), dsm_node(cl, s_px, t.q.y), dsm_node(cl, s_px, t.q.z),
                          dsm_node(cl, s_px, t.q.w)};
        float4 p[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) p[c] = *ptr[c];
        float dp[4][3];
        pbd_project(p, D, k, dp);
#pragma unroll
        for (int c = 0; c < 4; ++c)
            *ptr[c] = make_float4(fadd(p[c].x, dp[c][0]), fadd(p[c].y, dp[c][1]), fadd(p[c].z, dp[c][2]), p[c].w);
    };
    PbdView vc = v;  // the static records with corner codes in place of node ids
    vc.tet = codes;
    int j = 0, b1 = 0;
    PbdTet cur;
    if (total > 0) {
        run_of(l0, j, b1);
        cur = pbd_load(vc, j < b1 ? j : v.lvl[l0]);
    }
    for (int st = 0; st < total; ++st) {
        const int l = l0 + st % (l1 - l0);
        // the next level's first record before this level's chain
        int jn = 0, bn = 0;
        PbdTet nxt = cur;
        if (st + 1 < total) {
            run_of(l + 1 < l1 ? l + 1 : l0, jn, bn);
            if (jn < bn) nxt = pbd_load(vc, jn);
        }
        if (j < b1) apply(cur);
        for (int jj = j + kPbdThreads; jj < b1; jj += kPbdThreads) apply(pbd_load(vc, jj));
        cl.sync();
        cur = nxt;
        j = jn;
        b1 = bn;
    }
    for (int j = threadIdx.x; j < S; j += kPbdThreads) {
        const int n = rank * S + j;
        if (n < cnt) v.px[nb + n] = s_px[j];
    }
}

// slot of column `target` in block row [b, e) (columns ascending), e if absent
__device__ __forceinline__ int col_slot(const int *col, int b, int e, int target) {
    int lo = b, hi = e;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (col[mid] < target) lo = mid + 1;
        else hi = mid;
    }
    return (lo < e && col[lo] == target) ? lo : e;
}

// 1 / lumped mass as the reference forms it (1.0 / m: an FP64 quotient
// rounded to FP32, TetMesh.cpp:209), 0 at a pinned node
__device__ __forceinline__ float inv_mass_of(const float4 &info) {
    return info.z == 1.f ? 0.f : __double2float_rn(__ddiv_rn(1.0, (double)info.x));
}

__device__ __forceinline__ float4 state_pos4(const DevMesh &m, const DevState &st, int i) {
    const float4 X = m.rest[i], h = st.u0h[i], l = st.u0l[i];
    return make_float4(state_position(X.x, h.x, l.x), state_position(X.y, h.y, l.y), state_position(X.z, h.z, l.z),
                       0.f);
}

// f = gravity + ext of a node (the caller's forces; the pin spring that
// TetMesh::computeExternalForces puts on a pinned node is multiplied by its
// zero inverse mass in both integrators)
__device__ __forceinline__ float3 node_force(const float4 &info, const float4 *ext, int i) {
    float3 f = make_float3(0.f, info.y, 0.f);
    if (ext) {
        const float4 e = ext[i];
        f = make_float3(fadd(f.x, e.x), fadd(f.y, e.y), fadd(f.z, e.z));
    }
    return f;
}

// ---- the PBD step's rest data, formed exactly as TetMesh::initModel does in
// FP32 (TetMesh.cpp:186-216) with Eigen 3.2's 3x3 determinant (row-0
// cofactor expansion) and inverse (adjugate of the column-0 cofactors times
// 1 / det): the sweeps then see the reference's own Dm^-1 and masses.
__device__ __forceinline__ float eig_cof(const float m[3][3], int i, int j) {
    const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
    return fsub(fmul(m[i1][j1], m[i2][j2]), fmul(m[i1][j2], m[i2][j1]));
}

// level-ordered tet j (padded tet order[j]): Dm^-1 rows, and its lumped-mass
// share vol / 4 * density by padded tet
__global__ void k_pbd_rest(DevMesh m, const int *order, int n, float density, float4 *d0, float4 *d1, float4 *d2,
                           float *share) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int tp = order[j];
    const int4 q = m.tets[tp];
    const float4 X0 = m.rest[q.x], X1 = m.rest[q.y], X2 = m.rest[q.z], X3 = m.rest[q.w];
    const float m_[3][3] = {{fsub(X1.x, X0.x), fsub(X2.x, X0.x), fsub(X3.x, X0.x)},
                            {fsub(X1.y, X0.y), fsub(X2.y, X0.y), fsub(X3.y, X0.y)},
                            {fsub(X1.z, X0.z), fsub(X2.z, X0.z), fsub(X3.z, X0.z)}};
    const float det = fadd(fsub(fmul(m_[0][0], fsub(fmul(m_[1][1], m_[2][2]), fmul(m_[1][2], m_[2][1]))),
                                fmul(m_[0][1], fsub(fmul(m_[1][0], m_[2][2]), fmul(m_[1][2], m_[2][0])))),
                           fmul(m_[0][2], fsub(fmul(m_[1][0], m_[2][1]), fmul(m_[1][1], m_[2][0]))));
    const float vol = __double2float_rn(__ddiv_rn((double)fabsf(det), 6.0));
    share[tp] = __double2float_rn(__dmul_rn(__ddiv_rn((double)vol, 4.0), (double)density));
    const float c0[3] = {eig_cof(m_, 0, 0), eig_cof(m_, 1, 0), eig_cof(m_, 2, 0)};
    const float d = fadd(fmul(c0[0], m_[0][0]), fadd(fmul(c0[1], m_[1][0]), fmul(c0[2], m_[2][0])));
    const float inv = __fdiv_rn(1.0f, d);
    d0[j] = make_float4(fmul(c0[0], inv), fmul(c0[1], inv), fmul(c0[2], inv), 0.f);
    d1[j] = make_float4(fmul(eig_cof(m_, 0, 1), inv), fmul(eig_cof(m_, 1, 1), inv), fmul(eig_cof(m_, 2, 1), inv), 0.f);
    d2[j] = make_float4(fmul(eig_cof(m_, 0, 2), inv), fmul(eig_cof(m_, 1, 2), inv), fmul(eig_cof(m_, 2, 2), inv), 0.f);
}

// per node: lumped mass summed in tet order, {1 / mass (FP64 quotient
// rounded; 0 when pinned), -gravity * mass}
__global__ void k_pbd_mass(DevMesh m, const float *share, float gravity, float2 *node) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const float4 info = m.info[i];
    if (info.z == 2.f) { node[i] = make_float2(0.f, 0.f); return; }
    float s = 0.f;
    for (int j = m.inc_ptr[i]; j < m.inc_ptr[i + 1]; ++j) s = fadd(s, share[m.inc[j] >> 2]);
    node[i] = make_float2(info.z == 1.f ? 0.f : __double2float_rn(__ddiv_rn(1.0, (double)s)), fmul(-gravity, s));
}

// p = x + dt (v + (dt w) f), px = (p, w), x0 = x (PosBaseDynamic.cpp:24-30);
// node = {w, gravity_y} of the PBD rest data
__global__ void k_pbd_begin(DevMesh m, DevState st, const float2 *node, const float4 *ext, float dt, float4 *px,
                            float4 *x0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const float4 info = m.info[i];
    if (info.z == 2.f) { px[i] = x0[i] = make_float4(0.f, 0.f, 0.f, 0.f); return; }
    const float4 x = state_pos4(m, st, i), v = st.v[i];
    const float2 nd = node[i];
    const float w = nd.x, s = fmul(dt, w);
    float3 f = make_float3(0.f, nd.y, 0.f);
    if (ext) {
        const float4 e = ext[i];
        f = make_float3(fadd(f.x, e.x), fadd(f.y, e.y), fadd(f.z, e.z));
    }
    px[i] = make_float4(fadd(x.x, fmul(dt, fadd(v.x, fmul(s, f.x)))), fadd(x.y, fmul(dt, fadd(v.y, fmul(s, f.y)))),
                        fadd(x.z, fmul(dt, fadd(v.z, fmul(s, f.z)))), w);
    x0[i] = x;
}

// x = p and v = ((p - x) 0.99) / dt (PosBaseDynamic.cpp:51-52), or, with
// divide_first, ((p - x) / dt) 0.99 (ProjDynamic.cpp:477-478); the state keeps
// p - X exactly as (hi, lo)
__global__ void k_dyn_end(DevMesh m, DevState st, const float4 *px, const float4 *x0, float dt, int divide_first) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np || m.info[i].z == 2.f) return;
    const float4 p = px[i], x = x0[i], X = m.rest[i];
    const float c = 0.99f;
    float3 v;
    if (divide_first)
        v = make_float3(fmul(__fdiv_rn(fsub(p.x, x.x), dt), c), fmul(__fdiv_rn(fsub(p.y, x.y), dt), c),
                        fmul(__fdiv_rn(fsub(p.z, x.z), dt), c));
    else
        v = make_float3(__fdiv_rn(fmul(fsub(p.x, x.x), c), dt), __fdiv_rn(fmul(fsub(p.y, x.y), c), dt),
                        __fdiv_rn(fmul(fsub(p.z, x.z), c), dt));
    float h[3], l[3];
    two_sum(p.x, -X.x, h[0], l[0]);
    two_sum(p.y, -X.y, h[1], l[1]);
    two_sum(p.z, -X.z, h[2], l[2]);
    st.u0h[i] = make_float4(h[0], h[1], h[2], 0.f);
    st.u0l[i] = make_float4(l[0], l[1], l[2], 0.f);
    st.v[i] = make_float4(v.x, v.y, v.z, 0.f);
}

// ---------------------------------------------------------------- projective dynamics
// Row i of A = M / dt_m^2 + sum_t k vol_t (w_a . w_b) I3, one value a block
// (A.scalar), in the node's incidence order; D^-1 = 1 / a_ii.
__global__ void __launch_bounds__(128) k_pd_assemble(DevMesh m, BsrView A, float inv_dt2, float stiffness,
                                                     float *dinv9) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const int rb = A.ptr[i], re = A.ptr[i + 1];
    float *row = A.val + rb;
    for (int k = 0; k < re - rb; ++k) row[k] = 0.f;
    const float4 info = m.info[i];
    if (info.z != 2.f) {
        for (int j = m.inc_ptr[i]; j < m.inc_ptr[i + 1]; ++j) {
            const int ent = m.inc[j], t = ent >> 2, c = ent & 3;
            const int4 q = m.tets[t];
            const int qn[4] = {q.x, q.y, q.z, q.w};
            const float4 r0 = m.row0[t], r1 = m.row1[t], r2 = m.row2[t];
            const float w[4][3] = {{-(r0.x + r1.x + r2.x), -(r0.y + r1.y + r2.y), -(r0.z + r1.z + r2.z)},
                                   {r0.x, r0.y, r0.z},
                                   {r1.x, r1.y, r1.z},
                                   {r2.x, r2.y, r2.z}};
            const float kv = stiffness * fabsf(r0.w);
            for (int cc = 0; cc < 4; ++cc) {
                const int sl = col_slot(A.col, rb, re, qn[cc]);
                if (sl == re) continue;  // (the pattern holds every tet's node pairs)
                row[sl - rb] += kv * (w[c][0] * w[cc][0] + w[c][1] * w[cc][1] + w[c][2] * w[cc][2]);
            }
        }
    }
    const int dsl = col_slot(A.col, rb, re, i);
    float inv = 0.f;
    if (dsl < re) {
        row[dsl - rb] += info.z == 2.f ? 1.f : info.x * inv_dt2;
        inv = 1.f / row[dsl - rb];
    }
    for (int k = 0; k < 9; ++k) dinv9[9 * (size_t)i + k] = (k % 4 == 0) ? inv : 0.f;
}

// q = dt v + (dt^2 w) f, the inertial target's offset from x (the reference's
// s = (x + dt v + dt^2 w f) m / dt^2, ProjDynamic.cpp:447-463, is
// m / dt^2 (x + q)); p = x0 = x
__global__ void k_pd_begin(DevMesh m, DevState st, const float4 *ext, float dt, float4 *q, float4 *px, float4 *x0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    const float4 info = m.info[i];
    if (info.z == 2.f) {
        q[i] = px[i] = x0[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float4 x = state_pos4(m, st, i), v = st.v[i];
    const float dt2 = fmul(dt, dt), a = fmul(dt2, inv_mass_of(info));
    const float3 f = node_force(info, ext, i);
    q[i] = make_float4(fadd(fmul(dt, v.x), fmul(a, f.x)), fadd(fmul(dt, v.y), fmul(a, f.y)),
                       fadd(fmul(dt, v.z), fmul(a, f.z)), 0.f);
    px[i] = x;
    x0[i] = x;
}

// Per tet: R = U V^T with JacobiSVD's determinant fix (first, largest
// columns negated), i.e. U diag(sg, 1, sg) V^T of the modified SVD
// (sg = sign of the smallest singular value).  Corner a's share of the
// global step's residual, k vol (R - F) w_a (its projection k vol R w_a
// less its share of A p, both from edge differences: no absolute coordinate
// enters), goes into its gather slot.
__global__ void __launch_bounds__(128) k_pd_local(DevMesh m, const float4 *px, float stiffness, float4 *slot) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.Tp) return;
    const int4 q = m.tets[t];
    if (q.x < 0) return;
    const float4 r0 = m.row0[t], r1 = m.row1[t], r2 = m.row2[t];
    const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
    const float4 x0 = px[q.x], x1 = px[q.y], x2 = px[q.z], x3 = px[q.w];
    const float ds[3][3] = {{x1.x - x0.x, x2.x - x0.x, x3.x - x0.x},
                            {x1.y - x0.y, x2.y - x0.y, x3.y - x0.y},
                            {x1.z - x0.z, x2.z - x0.z, x3.z - x0.z}};
    float G[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            G[3 * r + c] = ds[r][0] * dinv[c] + ds[r][1] * dinv[3 + c] + ds[r][2] * dinv[6 + c] - (r == c ? 1.f : 0.f);
    float U[9], sv[3], V[9], sign3;
    svd_disp<float, 4>(G, U, sv, V, sign3);
    const float sg = sign3 < 0.f ? -1.f : 1.f;
    float E[9];  // R - F = R - I - G
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            E[3 * r + c] = (sg * U[3 * r] * V[3 * c] + U[3 * r + 1] * V[3 * c + 1] + sg * U[3 * r + 2] * V[3 * c + 2] -
                            (r == c ? 1.f : 0.f)) - G[3 * r + c];
    const float kv = stiffness * fabsf(r0.w);
    const float w[4][3] = {{-(r0.x + r1.x + r2.x), -(r0.y + r1.y + r2.y), -(r0.z + r1.z + r2.z)},
                           {r0.x, r0.y, r0.z},
                           {r1.x, r1.y, r1.z},
                           {r2.x, r2.y, r2.z}};
    const int4 sl = m.tslot[t];
    const int sls[4] = {sl.x, sl.y, sl.z, sl.w};
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        slot[sls[a]] = make_float4(kv * (E[0] * w[a][0] + E[1] * w[a][1] + E[2] * w[a][2]),
                                   kv * (E[3] * w[a][0] + E[4] * w[a][1] + E[5] * w[a][2]),
                                   kv * (E[6] * w[a][0] + E[7] * w[a][1] + E[8] * w[a][2]), 0.f);
    }
}

// The global step's residual r = b - A p = m / dt_m^2 (x - p) + m / dt^2 q
// + (m / dt^2 - m / dt_m^2) x (zero unless A was formed with another time
// step) + the node's (R - F) slots in incidence order (ascending tet, as the
// reference's m_proj_idx lists them); the correction d = 0
__global__ void k_pd_rhs(DevMesh m, const float4 *q, const float4 *x0, const float4 *px, const float4 *slot,
                         float inv_dt2, float inv_dtm2, float4 *r, float4 *d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.Np) return;
    d[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 info = m.info[i];
    if (info.z == 2.f) { r[i] = d[i]; return; }
    const float4 qq = q[i], x = x0[i], p = px[i];
    const float mb = info.x * inv_dt2, mm = info.x * inv_dtm2, mx = mb - mm;
    float4 a = make_float4(mm * (x.x - p.x) + mb * qq.x, mm * (x.y - p.y) + mb * qq.y, mm * (x.z - p.z) + mb * qq.z, 0.f);
    if (mx != 0.f) {
        a.x += mx * x.x;
        a.y += mx * x.y;
        a.z += mx * x.z;
    }
    for (int j = m.inc_ptr[i]; j < m.inc_ptr[i + 1]; ++j) {
        const float4 c = slot[j];
        a.x += c.x;
        a.y += c.y;
        a.z += c.z;
    }
    r[i] = a;
}

__global__ void k_pd_apply(int Np, float4 *p, const float4 *d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Np) return;
    const float4 a = p[i], c = d[i];
    p[i] = make_float4(a.x + c.x, a.y + c.y, a.z + c.z, a.w);
}

}  // namespace

cudaError_t launch_pd_apply(cudaStream_t s, int Np, float4 *p, const float4 *d) {
    k_pd_apply<<<(Np + 255) / 256, 256, 0, s>>>(Np, p, d);
    return cudaGetLastError();
}

cudaError_t launch_pbd_rest(cudaStream_t s, const DevMesh &m, const int *order, int n, float density, float gravity,
                            float4 *d0, float4 *d1, float4 *d2, float *share, float2 *node) {
    if (n > 0) k_pbd_rest<<<(n + 127) / 128, 128, 0, s>>>(m, order, n, density, d0, d1, d2, share);
    k_pbd_mass<<<(m.Np + 255) / 256, 256, 0, s>>>(m, share, gravity, node);
    return cudaGetLastError();
}

cudaError_t launch_pbd_begin(cudaStream_t s, const DevMesh &m, const DevState &st, const float2 *node,
                             const float4 *ext, float dt, float4 *px, float4 *x0) {
    k_pbd_begin<<<(m.Np + 255) / 256, 256, 0, s>>>(m, st, node, ext, dt, px, x0);
    return cudaGetLastError();
}

cudaError_t launch_pbd_sweeps(cudaStream_t s, const PbdView &v, int n_groups, int iterations, const float stretch[3],
                              const float shear[3]) {
    PbdConst k;
    for (int i = 0; i < 3; ++i) { k.stretch[i] = stretch[i]; k.shear[i] = shear[i]; }
    k.eps = 1e-6f;
    static int big_ok = -1;  // whether 16-CTA clusters of this kernel can be resident
    if (big_ok < 0) {
        big_ok = 0;
        if (cudaFuncSetAttribute(k_pbd_sweep, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
            cudaLaunchConfig_t q = {};
            q.gridDim = dim3(kPbdClusterMax);
            q.blockDim = dim3(kPbdThreads);
            cudaLaunchAttribute qa;
            qa.id = cudaLaunchAttributeClusterDimension;
            qa.val.clusterDim.x = kPbdClusterMax;
            qa.val.clusterDim.y = 1;
            qa.val.clusterDim.z = 1;
            q.attrs = &qa;
            q.numAttrs = 1;
            int n = 0;
            if (cudaOccupancyMaxActiveClusters(&n, k_pbd_sweep, &q) == cudaSuccess && n > 0) big_ok = 1;
        }
        cudaGetLastError();  // a refused query leaves no error behind
    }
    const int csize = (big_ok && n_groups <= 4) ? kPbdClusterMax : 8;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(n_groups * csize);
    cfg.blockDim = dim3(kPbdThreads);
    cfg.stream = s;
    cudaLaunchAttribute at;
    at.id = cudaLaunchAttributeClusterDimension;
    at.val.clusterDim.x = csize;
    at.val.clusterDim.y = 1;
    at.val.clusterDim.z = 1;
    cfg.attrs = &at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_pbd_sweep, v, iterations, k);
}

bool pbd_dsmem_fits(int smem_bytes) {
    if (smem_bytes > 227 * 1024) return false;
    if (cudaFuncSetAttribute(k_pbd_sweep_dsmem, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(k_pbd_sweep_dsmem, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes) !=
            cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t q = {};
    q.gridDim = dim3(kPbdClusterMax);
    q.blockDim = dim3(kPbdThreads);
    q.dynamicSmemBytes = smem_bytes;
    cudaLaunchAttribute qa;
    qa.id = cudaLaunchAttributeClusterDimension;
    qa.val.clusterDim.x = kPbdClusterMax;
    qa.val.clusterDim.y = 1;
    qa.val.clusterDim.z = 1;
    q.attrs = &qa;
    q.numAttrs = 1;
    int n = 0;
    const bool ok = cudaOccupancyMaxActiveClusters(&n, k_pbd_sweep_dsmem, &q) == cudaSuccess && n > 0;
    cudaGetLastError();
    return ok;
}

cudaError_t launch_pbd_sweeps_dsmem(cudaStream_t s, const PbdView &v, const int4 *codes, const int4 *gnode,
                                    int n_groups, int smem_bytes, int iterations, const float stretch[3],
                                    const float shear[3]) {
    PbdConst k;
    for (int i = 0; i < 3; ++i) { k.stretch[i] = stretch[i]; k.shear[i] = shear[i]; }
    k.eps = 1e-6f;
    // the kernel's shared-memory limit is per function, not per handle: set
    // it for this launch (another handle may have set a smaller one)
    cudaError_t e = cudaFuncSetAttribute(k_pbd_sweep_dsmem, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(n_groups * kPbdClusterMax);
    cfg.blockDim = dim3(kPbdThreads);
    cfg.dynamicSmemBytes = smem_bytes;
    cfg.stream = s;
    cudaLaunchAttribute at;
    at.id = cudaLaunchAttributeClusterDimension;
    at.val.clusterDim.x = kPbdClusterMax;
    at.val.clusterDim.y = 1;
    at.val.clusterDim.z = 1;
    cfg.attrs = &at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_pbd_sweep_dsmem, v, codes, gnode, iterations, k);
}

cudaError_t launch_dyn_end(cudaStream_t s, const DevMesh &m, const DevState &st, const float4 *px, const float4 *x0,
                           float dt, int divide_first) {
    k_dyn_end<<<(m.Np + 255) / 256, 256, 0, s>>>(m, st, px, x0, dt, divide_first);
    return cudaGetLastError();
}

cudaError_t launch_pd_assemble(cudaStream_t s, const DevMesh &m, const BsrView &A, float dt_matrix, float stiffness,
                               float *dinv9) {
    k_pd_assemble<<<(m.Np + 127) / 128, 128, 0, s>>>(m, A, 1.f / (dt_matrix * dt_matrix), stiffness, dinv9);
    return cudaGetLastError();
}

cudaError_t launch_pd_begin(cudaStream_t s, const DevMesh &m, const DevState &st, const float4 *ext, float dt,
                            float4 *q, float4 *px, float4 *x0) {
    k_pd_begin<<<(m.Np + 255) / 256, 256, 0, s>>>(m, st, ext, dt, q, px, x0);
    return cudaGetLastError();
}

cudaError_t launch_pd_residual(cudaStream_t s, const DevMesh &m, const float4 *px, float stiffness, float dt,
                               float dt_matrix, float4 *slot, const float4 *q, const float4 *x0, float4 *r, float4 *d) {
    k_pd_local<<<(m.Tp + 127) / 128, 128, 0, s>>>(m, px, stiffness, slot);
    k_pd_rhs<<<(m.Np + 255) / 256, 256, 0, s>>>(m, q, x0, px, slot, 1.f / (dt * dt),
                                                1.f / (dt_matrix * dt_matrix), r, d);
    return cudaGetLastError();
}

}  // namespace pbs
