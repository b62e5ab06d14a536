// Per-tet constitutive math for the descent step (device side).
//
// The device keeps node state as displacements u = x - X from the rest shape,
// so every tet works with the displacement gradient G = Du * Dm^-1
// (F = I + G).  All quantities below are written in terms of G so that none
// of them is a difference of O(1) numbers: in FP32 the reference's
// F - F^-T, I1 - 3 and ln det F lose ~|G| relative digits to cancellation,
// which puts the line-search energy's rounding noise above the energy changes
// of late iterations and stalls the solve short of a 1e-4 relative residual.
//
// Identities used (exact for 3x3):
//   det(I + G) = 1 + d,  d = tr G + c2 + c3,  c2 = sum of principal 2x2 minors
//                        of G (= tr cof G), c3 = det G
//   cof(I + G) = (1 + tr G) I - G^T + cof G,   F^-T = cof(F) / J
//   F - F^-T   = [(c2 + c3) I + J G + G^T - cof G] / J
//   I1 - 3 - 2 ln J = |G|^2 + 2 (tr G - ln(1 + d))
//                   = |G|^2 - 2 (c2 + c3) + 2 phi(d),  phi(d) = d - log1p(d)
//
// Reference semantics reproduced:
//   F = Ds * Dm^-1                                      TetMesh.cpp:307-316
//   neo-Hookean P = mu (F - F^-T) + lambda ln J F^-T     IsotropicNeohookeanMaterial.cpp:104
//   stretch-based P = U diag(P^) V^T,
//       P^_i = mu s_i + (lambda sum_j ln s_j - mu) / s_i  IsotropicNeohookeanMaterial.cpp:50-60
//       with the modified SVD of IsotropicMaterial.cpp:16-60 (U, V rotations,
//       an inversion's sign on the smallest singular value)
//   corner forces H = P * AN, AN = -(det Dm / 6) Dm^-T   TetMesh.cpp:279-294
//       (computeANs' cross-product normals equal -(det Dm/6) Dm^-T exactly),
//       corners 1..3 = H's columns, corner 0 = minus their sum
//   energy vol * (mu/2 (I1-3) - mu ln J + lambda/2 ln^2 J), clamped
//                                                        IsotropicNeohookeanMaterial.cpp:122-130
//   Jacobi diagonal: diagonal of K = -df/dx (IsotropicMaterial.cpp:503-552,
//       which builds the full 12x12 element matrix from Xu et al.'s
//       SVD-derivative dP/dF).  For this energy, restricted to one row d of F,
//       dP_dj/dF_dq = mu delta_jq + (mu + lambda - lambda ln J) G'_dj G'_dq with
//       G' = F^-T, hence the closed form
//         K_cc,dd = svol [mu |w_c|^2 + (mu + lambda - lambda ln J) (G'_d . w_c)^2]
//       w_c = row c-1 of Dm^-1 (w_0 = -sum of rows), svol = det Dm / 6.
//
// SVD (stretch material): own implementation of the classic route of
// McAdams et al. 2011 -- cyclic Jacobi eigen-analysis of a symmetric 3x3 with
// exact rotations, sorting (det V kept +1), Givens QR for U -- applied to
// S = F^T F - I = G + G^T + G^T G, whose eigenvalues s_i give sigma_i - 1
// without cancellation (sigma_i^2 = 1 + s_i, ln sigma_i = log1p(s_i) / 2).
// Near-inverted tets (det F < 1e-3, or smallest singular value below 0.3 from
// the FP32 spectrum) redo the SVD in FP64 with F formed from the absolute
// positions (position_gradient_exact); neo-Hookean tets with det F < 1e-3 take
// their stress in FP64 the same way.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace pbs {

template <typename T> __device__ __forceinline__ T log1p_t(T x);
template <> __device__ __forceinline__ float log1p_t<float>(float x) { return log1pf(x); }
template <> __device__ __forceinline__ double log1p_t<double>(double x) { return log1p(x); }
template <typename T> __device__ __forceinline__ T rsqrt_t(T x);
template <> __device__ __forceinline__ float rsqrt_t<float>(float x) { return rsqrtf(x); }
template <> __device__ __forceinline__ double rsqrt_t<double>(double x) { return rsqrt(x); }
template <typename T> __device__ __forceinline__ T sqrt_t(T x);
template <> __device__ __forceinline__ float sqrt_t<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double sqrt_t<double>(double x) { return sqrt(x); }

// Cofactor matrix of a 3x3 (row-major): cof(A) = det(A) A^-T.
template <typename T> __device__ __forceinline__ void cofactor3(const T m[9], T c[9]) {
    c[0] = m[4] * m[8] - m[5] * m[7];
    c[1] = m[5] * m[6] - m[3] * m[8];
    c[2] = m[3] * m[7] - m[4] * m[6];
    c[3] = m[2] * m[7] - m[1] * m[8];
    c[4] = m[0] * m[8] - m[2] * m[6];
    c[5] = m[1] * m[6] - m[0] * m[7];
    c[6] = m[1] * m[5] - m[2] * m[4];
    c[7] = m[2] * m[3] - m[0] * m[5];
    c[8] = m[0] * m[4] - m[1] * m[3];
}

// G = Du * Dinv with Du columns u1-u0, u2-u0, u3-u0.
template <typename T>
__device__ __forceinline__ void disp_gradient(const float4 &u0, const float4 &u1, const float4 &u2, const float4 &u3,
                                              const float dinv[9], T G[9]) {
    const T du[9] = {(T)u1.x - (T)u0.x, (T)u2.x - (T)u0.x, (T)u3.x - (T)u0.x,
                     (T)u1.y - (T)u0.y, (T)u2.y - (T)u0.y, (T)u3.y - (T)u0.y,
                     (T)u1.z - (T)u0.z, (T)u2.z - (T)u0.z, (T)u3.z - (T)u0.z};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            G[3 * r + c] = du[3 * r] * (T)dinv[c] + du[3 * r + 1] * (T)dinv[3 + c] + du[3 * r + 2] * (T)dinv[6 + c];
}

// Everything a tet needs about F = I + G.
template <typename T> struct Kin {
    T G[9], cofG[9];
    T tr, c2, c3, d;  // det F = 1 + d
    T lnJ;            // log1p(d)
};

template <typename T> __device__ __forceinline__ void kinematics(Kin<T> &k) {
    cofactor3<T>(k.G, k.cofG);
    k.tr = k.G[0] + k.G[4] + k.G[8];
    k.c2 = k.cofG[0] + k.cofG[4] + k.cofG[8];
    k.c3 = k.G[0] * k.cofG[0] + k.G[1] * k.cofG[1] + k.G[2] * k.cofG[2];
    k.d = k.tr + k.c2 + k.c3;
    k.lnJ = log1p_t<T>(k.d);
}

// F^-T = [(1 + tr G) I - G^T + cof G] / J
template <typename T> __device__ __forceinline__ void inv_transpose(const Kin<T> &k, T FiT[9]) {
    const T invJ = T(1) / (T(1) + k.d);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            FiT[3 * i + j] = ((i == j ? T(1) + k.tr : T(0)) - k.G[3 * j + i] + k.cofG[3 * i + j]) * invJ;
}

// Neo-Hookean P = mu (F - F^-T) + lambda ln J F^-T, cancellation-free.
template <typename T> __device__ __forceinline__ void pk1_neohookean(const Kin<T> &k, T mu, T lambda, T P[9]) {
    const T J = T(1) + k.d;
    const T invJ = T(1) / J;
    const T lg = lambda * k.lnJ;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const T diag = (i == j) ? T(1) : T(0);
            const T fmf = (diag * (k.c2 + k.c3) + J * k.G[3 * i + j] + k.G[3 * j + i] - k.cofG[3 * i + j]) * invJ;
            const T fit = (diag * (T(1) + k.tr) - k.G[3 * j + i] + k.cofG[3 * i + j]) * invJ;
            P[3 * i + j] = mu * fmf + lg * fit;
        }
}

// log1p(x) of a volume increment.  For |x| < 1/32 its Taylor series
// x - x^2/2 + x^3/3 - ... to the x^6 term by Horner's rule (the first term
// left out is below 2^-26 |x| there: a few FP32 ulp in all); otherwise log1pf.
// The increments of a descent pass against its step's base are almost always
// in the series' range.
__device__ __forceinline__ float log1p_increment(float x) {
    if (fabsf(x) < 0.03125f) {
        float s = -1.0f / 6.0f;
        s = fmaf(x, s, 0.2f);
        s = fmaf(x, s, -0.25f);
        s = fmaf(x, s, 1.0f / 3.0f);
        s = fmaf(x, s, -0.5f);
        s = fmaf(x, s, 1.0f);
        return x * s;
    }
    return log1pf(x);
}

// dP = P(F0 + dG) - P(F0) of the neo-Hookean stress, from the base kinematics
// k0 (the step's start, with ln J0) and the increment dG.  With
// P = mu F + (lambda ln J - mu) F^-T:
//   dP = mu dG + (lambda ln J - mu) (F^-T - F0^-T) + lambda (ln J - ln J0) F0^-T
// where, with cof(F) = cof(F0) + L(F0, dG) + cof(dG) (L: the part of the
// cofactor bilinear in F0 and dG) and dJ = cof(F0) : dG + F0 : cof(dG) +
// det dG,
//   F^-T - F0^-T = (L(F0, dG) + cof(dG) - F0^-T dJ) / J
// and ln J - ln J0 = log1p(dJ / J0) -- no term subtracts the two states'
// O(1) quantities, so dP is accurate to FP32 relative to itself rather than
// to P.  The scale factors 1/J0 and 1/J multiply only O(|dG|) terms and use
// the fast reciprocal (a few ulp).  Returns in k the current det F - 1 =
// d0 + dJ and ln J = ln J0 + log1p(dJ / J0), and with FULL_KIN the rest of
// the current kinematics (G = G0 + dG, its cofactor and invariants: the
// energy and the Jacobi diagonal need them, the forces do not).
template <bool FULL_KIN>
__device__ __forceinline__ void pk1_neohookean_inc(const Kin<float> &k0, const float dG[9], float mu, float lambda,
                                                   Kin<float> &k, float dP[9]) {
    float F0iT[9];
    const float rJ0 = __fdividef(1.0f, 1.0f + k0.d);
    // F0 = I + G0 and cof(F0) = (1 + tr G0) I - G0^T + cof(G0), entry by entry
    auto F0 = [&](int r, int c) { return ((r == c) ? 1.0f : 0.0f) + k0.G[3 * r + c]; };
    float dJ = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int a = (i + 1) % 3, b = (i + 2) % 3;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int c = (j + 1) % 3, d = (j + 2) % 3;
            const float cofdG = dG[3 * a + c] * dG[3 * b + d] - dG[3 * a + d] * dG[3 * b + c];
            const float cof0 = ((i == j) ? 1.0f + k0.tr : 0.0f) - k0.G[3 * j + i] + k0.cofG[3 * i + j];
            // dJ = cof(F0) : dG + F0 : cof(dG) + det dG (det dG = dG row 0 . cof(dG) row 0)
            dJ += cof0 * dG[3 * i + j] + (F0(i, j) + ((i == 0) ? dG[j] : 0.0f)) * cofdG;
            F0iT[3 * i + j] = cof0 * rJ0;
        }
    }
    const float dl = log1p_increment(dJ * rJ0);
    k.d = k0.d + dJ;
    k.lnJ = k0.lnJ + dl;
    const float rJ = __fdividef(1.0f, 1.0f + k.d);
    const float c1 = lambda * k.lnJ - mu, c2 = lambda * dl;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int a = (i + 1) % 3, b = (i + 2) % 3;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int c = (j + 1) % 3, d = (j + 2) % 3;
            // cof(F)_ij - cof(F0)_ij = L(F0, dG)_ij + cof(dG)_ij
            //   = F_ac dG_bd + dG_ac F0_bd - F_ad dG_bc - dG_ad F0_bc  (F = F0 + dG)
            const float Fac = F0(a, c) + dG[3 * a + c], Fad = F0(a, d) + dG[3 * a + d];
            const float dcof = Fac * dG[3 * b + d] + dG[3 * a + c] * F0(b, d) - Fad * dG[3 * b + c] -
                               dG[3 * a + d] * F0(b, c);
            const float t = (dcof - F0iT[3 * i + j] * dJ) * rJ;  // F^-T - F0^-T
            dP[3 * i + j] = mu * dG[3 * i + j] + c1 * t + c2 * F0iT[3 * i + j];
        }
    }
    if (FULL_KIN) {
#pragma unroll
        for (int i = 0; i < 9; ++i) k.G[i] = k0.G[i] + dG[i];
        cofactor3<float>(k.G, k.cofG);
        k.tr = k.G[0] + k.G[4] + k.G[8];
        k.c2 = k.cofG[0] + k.cofG[4] + k.cofG[8];
        k.c3 = k.G[0] * k.cofG[0] + k.G[1] * k.cofG[1] + k.G[2] * k.cofG[2];
    }
}

// phi(d) = d - log1p(d) >= 0, by its Taylor series where that is exact to FP32.
template <typename T> __device__ __forceinline__ T phi_log1p(T d) {
    if (fabs(d) < T(0.1)) {
        T s = T(0.125);
        s = T(-1.0 / 7.0) + d * s;
        s = T(1.0 / 6.0) + d * s;
        s = T(-0.2) + d * s;
        s = T(0.25) + d * s;
        s = T(-1.0 / 3.0) + d * s;
        s = T(0.5) + d * s;
        return d * d * s;
    }
    return d - log1p_t<T>(d);
}

// Psi / vol = mu (|G|^2/2 - c2 - c3 + phi(d)) + lambda/2 ln^2 J
template <typename T> __device__ __forceinline__ T energy_density(const Kin<T> &k, T mu, T lambda) {
    T g2 = T(0);
#pragma unroll
    for (int i = 0; i < 9; ++i) g2 += k.G[i] * k.G[i];
    return mu * (T(0.5) * g2 - k.c2 - k.c3 + phi_log1p<T>(k.d)) + T(0.5) * lambda * k.lnJ * k.lnJ;
}

__device__ __forceinline__ float clamp_energy(float e, int clamp_cpu) {
    if (clamp_cpu) return e > 1e-6f ? e : 0.0f;  // IsotropicNeohookeanMaterial.cpp:129
    return fmaxf(e, 0.0f);                       // CUDAInterface.cu:549
}

// Tet energy as a line search compares it.  Both reference clamps map the NaN
// energy of an inverted tet (log J of J <= 0) to 0, which makes an inverted
// state look cheaper; with keep_nan (RESTART control, the warm-start judge) a
// NaN stays NaN so that the state is rejected.
__device__ __forceinline__ float search_energy(float e, int clamp_cpu, bool keep_nan) {
    return (keep_nan && e != e) ? e : clamp_energy(e, clamp_cpu);
}

// ---------------------------------------------------------------- SVD
// One Jacobi rotation annihilating a_pq of a symmetric 3x3 (r = third index),
// accumulated into V's columns p and q.
template <typename T>
__device__ __forceinline__ void jacobi_rotate(T &app, T &aqq, T &apq, T &arp, T &arq, T V[9], int p, int q) {
    const T off = apq;
    const T scale = fabs(app) + fabs(aqq);
    if (fabs(off) <= T(1e-37) + scale * (sizeof(T) == 4 ? T(1e-9) : T(1e-18))) { apq = T(0); return; }
    const T theta = (aqq - app) / (T(2) * off);
    T t = T(1) / (fabs(theta) + sqrt_t<T>(theta * theta + T(1)));
    t = theta < T(0) ? -t : t;
    const T c = rsqrt_t<T>(t * t + T(1));
    const T s = t * c;
    app -= t * off;
    aqq += t * off;
    apq = T(0);
    const T rp = arp, rq = arq;
    arp = c * rp - s * rq;
    arq = s * rp + c * rq;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const T vp = V[3 * k + p], vq = V[3 * k + q];
        V[3 * k + p] = c * vp - s * vq;
        V[3 * k + q] = s * vp + c * vq;
    }
}

// Zero B[i][j] with a rotation of rows j and i; U <- U * G^T.
template <typename T> __device__ __forceinline__ void givens_qr_step(T B[9], T U[9], int j, int i) {
    const T a = B[3 * j + j], b = B[3 * i + j];
    const T r2 = a * a + b * b;
    T c = T(1), s = T(0);
    if (r2 > T(1e-37)) {
        const T inv = rsqrt_t<T>(r2);
        c = a * inv;
        s = b * inv;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const T bj = B[3 * j + k], bi = B[3 * i + k];
        B[3 * j + k] = c * bj + s * bi;
        B[3 * i + k] = -s * bj + c * bi;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const T uj = U[3 * k + j], ui = U[3 * k + i];
        U[3 * k + j] = c * uj + s * ui;
        U[3 * k + i] = -s * uj + c * ui;
    }
}

// Modified SVD of F = I + G: rotations U, V; s_i = sigma_i^2 - 1 (descending);
// sign = sign of the smallest singular value (-1 for an inverted tet).
template <typename T, int SWEEPS>
__device__ __forceinline__ void svd_disp(const T G[9], T U[9], T s[3], T V[9], T &sign3) {
    // S = G + G^T + G^T G
    T a00 = T(2) * G[0] + G[0] * G[0] + G[3] * G[3] + G[6] * G[6];
    T a11 = T(2) * G[4] + G[1] * G[1] + G[4] * G[4] + G[7] * G[7];
    T a22 = T(2) * G[8] + G[2] * G[2] + G[5] * G[5] + G[8] * G[8];
    T a01 = G[1] + G[3] + G[0] * G[1] + G[3] * G[4] + G[6] * G[7];
    T a02 = G[2] + G[6] + G[0] * G[2] + G[3] * G[5] + G[6] * G[8];
    T a12 = G[5] + G[7] + G[1] * G[2] + G[4] * G[5] + G[7] * G[8];
#pragma unroll
    for (int k = 0; k < 9; ++k) V[k] = (k % 4 == 0) ? T(1) : T(0);
    for (int sweep = 0; sweep < SWEEPS; ++sweep) {
        jacobi_rotate<T>(a00, a11, a01, a02, a12, V, 0, 1);
        jacobi_rotate<T>(a00, a22, a02, a01, a12, V, 0, 2);
        jacobi_rotate<T>(a11, a22, a12, a01, a02, V, 1, 2);
    }
    T e0 = a00, e1 = a11, e2 = a22;
    auto swap_cols = [&](int i, int j) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const T t = V[3 * r + i];
            V[3 * r + i] = -V[3 * r + j];
            V[3 * r + j] = t;
        }
    };
    if (e0 < e1) { swap_cols(0, 1); T t = e0; e0 = e1; e1 = t; }
    if (e0 < e2) { swap_cols(0, 2); T t = e0; e0 = e2; e2 = t; }
    if (e1 < e2) { swap_cols(1, 2); T t = e1; e1 = e2; e2 = t; }
    s[0] = e0; s[1] = e1; s[2] = e2;
    // B = F V = V + G V, then QR for U
    T B[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            B[3 * r + c] = V[3 * r + c] + G[3 * r] * V[c] + G[3 * r + 1] * V[3 + c] + G[3 * r + 2] * V[6 + c];
#pragma unroll
    for (int k = 0; k < 9; ++k) U[k] = (k % 4 == 0) ? T(1) : T(0);
    givens_qr_step<T>(B, U, 0, 1);
    givens_qr_step<T>(B, U, 0, 2);
    givens_qr_step<T>(B, U, 1, 2);
    sign3 = B[8] < T(0) ? T(-1) : T(1);
}

// Smallest singular value below which the FP32 eigen-analysis of
// F^T F - I is redone in FP64 (the SVD of a near-inverted tet): sigma_3^2 =
// 1 + s_3 carries the FP32 rounding of s_3 (about 2^-24 absolute), a relative
// 2^-25 / sigma_3^2 on sigma_3, and the stress's (lambda ln J - mu) / sigma_3
// term scales that by up to 1 / sigma_3 in the corner forces: about 1e-6 at
// sigma_3 = 0.3, 3e-5 at 0.1.
constexpr float STRETCH_FP32_MIN_SIGMA2 = 0.09f;

// The stretch-based P from G; returns false (P untouched) when the FP32
// spectrum is too ill-conditioned to use (T = float and sigma_3 < 0.3).
template <typename T> __device__ __forceinline__ bool stretch_pk1(const T G[9], T mu, T lambda, float P[9]) {
    T U[9], s[3], V[9], sign3;
    svd_disp<T, sizeof(T) == 4 ? 4 : 8>(G, U, s, V, sign3);
    if (sizeof(T) == 4 && T(1) + s[2] < T(STRETCH_FP32_MIN_SIGMA2)) return false;
    T sig[3], ph[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) sig[i] = sqrt_t<T>(T(1) + s[i]);
    sig[2] *= sign3;
    // sum_j ln sigma_j; an inverted tet (sigma_3 < 0) gives NaN as in the reference
    const T L = T(0.5) * (log1p_t<T>(s[0]) + log1p_t<T>(s[1]) + log1p_t<T>(s[2])) +
                (sign3 < T(0) ? T(NAN) : T(0));
    // P^_i = mu sigma_i + (lambda L - mu) / sigma_i = (mu s_i + lambda L) / sigma_i
#pragma unroll
    for (int i = 0; i < 3; ++i) ph[i] = (mu * s[i] + lambda * L) / sig[i];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            P[3 * i + j] = (float)(U[3 * i] * ph[0] * V[3 * j] + U[3 * i + 1] * ph[1] * V[3 * j + 1] +
                                   U[3 * i + 2] * ph[2] * V[3 * j + 2]);
    return true;
}

// Where a tet's four rest positions are: rest[meta[id[c]].x] (chunk-local
// ids) or rest[id[c]] (padded node ids, meta null).
struct CornerRest {
    const float4 *rest;
    const int4 *meta;
    int id[4];
    __device__ __forceinline__ float4 get(int c) const { return rest[meta ? meta[id[c]].x : id[c]]; }
};

// F - I in FP64 with F = Ds Dm^-1 formed from the corners' absolute
// positions x = X + (u hi + u lo), as the reference defines F
// (TetMesh.cpp:307-316).  Near inversion the FP32 displacement form loses
// 2^-24 / sigma_min of the stress: det F = 1 + d carries the rounding of d, and
// F = I + Du Dm^-1 also differs from Ds Dm^-1 by Dm (Dm^-1)_fp32 - I, an
// O(2^-24) perturbation that is a relative 2^-24 / sigma_min change of the
// smallest singular value.  A near-inverted tet therefore takes this form.
__device__ __forceinline__ void position_gradient_exact(const CornerRest &cr, const float4 &h0, const float4 &h1,
                                                        const float4 &h2, const float4 &h3, const float4 &l0,
                                                        const float4 &l1, const float4 &l2, const float4 &l3,
                                                        const float dinv[9], double G[9]) {
    const float4 X0 = cr.get(0), X1 = cr.get(1), X2 = cr.get(2), X3 = cr.get(3);
    const double x0[3] = {(double)X0.x + h0.x + l0.x, (double)X0.y + h0.y + l0.y, (double)X0.z + h0.z + l0.z};
    const double x1[3] = {(double)X1.x + h1.x + l1.x, (double)X1.y + h1.y + l1.y, (double)X1.z + h1.z + l1.z};
    const double x2[3] = {(double)X2.x + h2.x + l2.x, (double)X2.y + h2.y + l2.y, (double)X2.z + h2.z + l2.z};
    const double x3[3] = {(double)X3.x + h3.x + l3.x, (double)X3.y + h3.y + l3.y, (double)X3.z + h3.z + l3.z};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const double d1 = x1[r] - x0[r], d2 = x2[r] - x0[r], d3 = x3[r] - x0[r];
#pragma unroll
        for (int c = 0; c < 3; ++c)
            G[3 * r + c] = d1 * (double)dinv[c] + d2 * (double)dinv[3 + c] + d3 * (double)dinv[6 + c] -
                           (r == c ? 1.0 : 0.0);
    }
}

// Stretch-based P (IsotropicMaterial.cpp:370-384).  The SVD runs in FP64 for
// near-inverted tets: det F < 1e-3, and also any tet whose FP32 spectrum
// gives sigma_3 < 0.3 (see STRETCH_FP32_MIN_SIGMA2).  exact(double G[9])
// fills the FP64 gradient for that case (from the corners' exact displacement
// pairs where the caller has them).  n_fp64: when not null, counts the tets
// that took the FP64 SVD (a parity probe's evidence that the branch ran).
template <class Exact>
__device__ __forceinline__ void pk1_stretch_x(const Kin<float> &k, float mu, float lambda, float P[9],
                                              unsigned int *n_fp64, Exact exact) {
    if (1.0f + k.d < 1e-3f || !stretch_pk1<float>(k.G, mu, lambda, P)) {
        if (n_fp64) atomicAdd(n_fp64, 1u);
        double Gd[9];
        exact(Gd);
        stretch_pk1<double>(Gd, (double)mu, (double)lambda, P);
    }
}

// Neo-Hookean P with the same near-inversion rule: below det F = 1e-3 the
// FP32 gradient's rounding (2^-24 absolute on J) is a relative 2^-24 / J on
// F^-T, so the stress is formed in FP64 from exact(G) and rounded.
template <class Exact>
__device__ __forceinline__ void pk1_neohookean_x(const Kin<float> &k, float mu, float lambda, float P[9],
                                                 unsigned int *n_fp64, Exact exact) {
    if (1.0f + k.d < 1e-3f) {
        if (n_fp64) atomicAdd(n_fp64, 1u);
        Kin<double> kd;
        exact(kd.G);
        kinematics(kd);
        double Pd[9];
        pk1_neohookean<double>(kd, (double)mu, (double)lambda, Pd);
#pragma unroll
        for (int i = 0; i < 9; ++i) P[i] = (float)Pd[i];
    } else {
        pk1_neohookean<float>(k, mu, lambda, P);
    }
}

// The FP64 stress of a near-inverted tet (either material) from its corners'
// absolute positions (rest + exact displacement pair h + l) and the rows of
// Dm^-1; out of line, so the pass kernels' common path keeps its registers.
// Returns P rounded to FP32.
static __device__ __noinline__ void pk1_exact_fp64(int material, CornerRest cr, float4 h0, float4 h1, float4 h2,
                                                   float4 h3, float4 l0, float4 l1, float4 l2, float4 l3, float4 r0,
                                                   float4 r1, float4 r2, float mu, float lambda, float *P) {
    const float dinv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
    Kin<double> kd;
    position_gradient_exact(cr, h0, h1, h2, h3, l0, l1, l2, l3, dinv, kd.G);
    if (material == 1) {  // PBS_MATERIAL_STRETCH
        stretch_pk1<double>(kd.G, (double)mu, (double)lambda, P);
        return;
    }
    kinematics(kd);
    double Pd[9];
    pk1_neohookean<double>(kd, (double)mu, (double)lambda, Pd);
#pragma unroll
    for (int i = 0; i < 9; ++i) P[i] = (float)Pd[i];
}

// The same with the FP64 gradient taken from the FP32 one.
__device__ __forceinline__ void pk1_stretch(const Kin<float> &k, float mu, float lambda, float P[9],
                                            unsigned int *n_fp64 = nullptr) {
    pk1_stretch_x(k, mu, lambda, P, n_fp64, [&](double Gd[9]) {
#pragma unroll
        for (int i = 0; i < 9; ++i) Gd[i] = (double)k.G[i];
    });
}

// Corner forces f[3c + d]: H = -svol * P * Dinv^T; corner 0 = -(sum of 1..3).
__device__ __forceinline__ void corner_forces(const float P[9], const float dinv[9], float svol, float f[12]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float s0 = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float h = -svol * (P[3 * d] * dinv[3 * c] + P[3 * d + 1] * dinv[3 * c + 1] + P[3 * d + 2] * dinv[3 * c + 2]);
            f[3 * (c + 1) + d] = h;
            s0 += h;
        }
        f[d] = -s0;
    }
}

// 12 Jacobi-diagonal entries (corner-major) from the closed form above.
__device__ __forceinline__ void hessian_diag(const Kin<float> &k, float mu, float lambda, const float dinv[9],
                                             float svol, float kd[12]) {
    float FiT[9];
    inv_transpose<float>(k, FiT);
    const float beta = mu + lambda - lambda * k.lnJ;
    float w[4][3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        w[1][q] = dinv[q];
        w[2][q] = dinv[3 + q];
        w[3][q] = dinv[6 + q];
        w[0][q] = -(dinv[q] + dinv[3 + q] + dinv[6 + q]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float ww = w[c][0] * w[c][0] + w[c][1] * w[c][1] + w[c][2] * w[c][2];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float gw = FiT[3 * d] * w[c][0] + FiT[3 * d + 1] * w[c][1] + FiT[3 * d + 2] * w[c][2];
            kd[3 * c + d] = svol * (mu * ww + beta * gw * gw);
        }
    }
}

// ---------------------------------------------------------------- compensated sums
// Error-free transformation a + b = s + e (Knuth's TwoSum); the _rn
// intrinsics keep the compiler from contracting or reassociating it.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// The FP32 position of a node whose state is rest X plus displacement
// hi + lo, rounded once (the three terms summed in FP64 first): exactly the
// position a caller uploaded, whose displacement was split exactly.
__device__ __forceinline__ float state_position(float X, float hi, float lo) {
    return __double2float_rn(__dadd_rn(__dadd_rn((double)X, (double)hi), (double)lo));
}
// (hi, lo) + b, renormalised so that |lo| <= ulp(hi) / 2.
__device__ __forceinline__ void add_comp(float &hi, float &lo, float b) {
    float s, e;
    two_sum(hi, b, s, e);
    lo = __fadd_rn(lo, e);
    const float s2 = __fadd_rn(s, lo);
    lo = __fsub_rn(lo, __fsub_rn(s2, s));
    hi = s2;
}

// Double-float value hi + lo (|lo| <= ulp(hi) / 2) with FP32 operations only:
// products exact through fma, sums through TwoSum, about 2^-44 relative.  The
// line search's energy sums use it: in FP64 they ran on GB300's narrow
// double-precision pipe and made a check pass 60% dearer than a plain one.
struct DFloat {
    float hi, lo;
};
__device__ __forceinline__ DFloat df_norm(float s, float e) {
    const float h = __fadd_rn(s, e);
    return DFloat{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ DFloat df_add(DFloat a, float b) {
    float s, e;
    two_sum(a.hi, b, s, e);
    return df_norm(s, __fadd_rn(e, a.lo));
}
__device__ __forceinline__ DFloat df_add(DFloat a, DFloat b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    return df_norm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DFloat df_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return DFloat{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ DFloat df_mul(DFloat a, float b) {
    const float p = __fmul_rn(a.hi, b);
    return df_norm(p, __fmaf_rn(a.lo, b, __fmaf_rn(a.hi, b, -p)));
}
__device__ __forceinline__ DFloat df_mul(DFloat a, DFloat b) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.hi, -p);
    return df_norm(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e)));
}
__device__ __forceinline__ double df_double(DFloat a) { return (double)a.hi + (double)a.lo; }

// The same double-float arithmetic as a number type, so that the templated
// tet math above (disp-gradient, kinematics, stress) runs in it unchanged:
// about 2^-44 relative per operation on the FP32 pipes, against GB300's
// double-precision pipe, which ran the per-step base force at 0.5 ms on the
// 1M-tet box.  The two scalar functions of a tet, 1 / J and log1p(d), are
// taken in FP64 from the pair's value (one of each per tet).
struct DD {
    float hi, lo;
    DD() = default;
    __device__ __forceinline__ DD(float h) : hi(h), lo(0.f) {}
    __device__ __forceinline__ DD(int v) : hi((float)v), lo(0.f) {}
    __device__ __forceinline__ DD(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ explicit DD(double v) {
        hi = __double2float_rn(v);
        lo = __double2float_rn(v - (double)hi);
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ DD operator+(DD a, DD b) {
    const DFloat r = df_add(DFloat{a.hi, a.lo}, DFloat{b.hi, b.lo});
    return DD(r.hi, r.lo);
}
__device__ __forceinline__ DD operator-(DD a) { return DD(-a.hi, -a.lo); }
__device__ __forceinline__ DD operator-(DD a, DD b) { return a + (-b); }
__device__ __forceinline__ DD operator*(DD a, DD b) {
    const DFloat r = df_mul(DFloat{a.hi, a.lo}, DFloat{b.hi, b.lo});
    return DD(r.hi, r.lo);
}
__device__ __forceinline__ DD operator/(DD a, DD b) { return DD(a.value() / b.value()); }
template <> __device__ __forceinline__ DD log1p_t<DD>(DD x) { return DD(log1p(x.value())); }

}  // namespace pbs
