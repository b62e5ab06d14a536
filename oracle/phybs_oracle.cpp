// CPU restatement of PhyBS's descent time step — TEST INFRASTRUCTURE ONLY.
//
// This is the parity checker for the CUDA path.  Only tests/, the smoke entry
// point and bench.py's CPU-baseline leg load it.  It restates, templated on
// the arithmetic type (float = the reference's FP32, double = the all-FP64
// reference every result is measured against), the reference CPU solver:
//
//   rest state          TetMesh.cpp:186-216, computeANs TetMesh.cpp:279-294
//   Lame parameters     IsotropicNeohookeanMaterial.cpp:15-16 (lambda = 2mu/(1-2nu))
//   NH forces           IsotropicNeohookeanMaterial.cpp:93-114
//   stretch forces      IsotropicMaterial.cpp:360-409 with the modified SVD
//                       IsotropicMaterial.cpp:16-60 and the principal-stretch
//                       gradient IsotropicNeohookeanMaterial.cpp:50-60
//   energy              IsotropicNeohookeanMaterial.cpp:116-131
//   Hessian diagonal    IsotropicMaterial.cpp:503-552 + 872-1019 (Xu et al. 2015
//                       dP/dF through SVD derivatives, eps-perturbed spectrum),
//                       stretch Hessian IsotropicNeohookeanMaterial.cpp:63-91
//   descent step        DescentOptimize.cpp:35-188
//
// The SVD is a cyclic Jacobi eigen-solve of F^T F (converged to the working
// precision) with sigma_i = |F v_i|, followed by the reference's sign fix-ups;
// Eigen's JacobiSVD (what the reference calls) is not used.  The perturbed
// spectrum is used directly instead of re-running the SVD of
// U diag(sigma~) V^T (IsotropicMaterial.cpp:921-928); both give the same
// factors up to rounding.
//
// Parity of this restatement is pinned against the reference itself
// (oracle/_ref, built by oracle/ref_build) through tests/golden fixtures.
#include <cmath>
#include <cstring>
#include <cstdint>
#include <vector>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename R> struct M3 {
    R a[3][3];
    R &operator()(int r, int c) { return a[r][c]; }
    const R &operator()(int r, int c) const { return a[r][c]; }
};

template <typename R> M3<R> zero3() { M3<R> m; std::memset(&m, 0, sizeof(m)); return m; }
template <typename R> M3<R> mul(const M3<R> &A, const M3<R> &B) {
    M3<R> C;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            R s = 0;
            for (int k = 0; k < 3; ++k) s += A(i, k) * B(k, j);
            C(i, j) = s;
        }
    return C;
}
template <typename R> M3<R> transpose(const M3<R> &A) {
    M3<R> T;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T(i, j) = A(j, i);
    return T;
}
template <typename R> R det3(const M3<R> &A) {
    return A(0, 0) * (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) - A(0, 1) * (A(1, 0) * A(2, 2) - A(1, 2) * A(2, 0)) +
           A(0, 2) * (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0));
}
// Inverse by the adjugate (Eigen's 3x3 inverse is the cofactor formula too).
template <typename R> M3<R> inv3(const M3<R> &A) {
    M3<R> C;
    C(0, 0) = A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1);
    C(0, 1) = A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2);
    C(0, 2) = A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1);
    C(1, 0) = A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2);
    C(1, 1) = A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0);
    C(1, 2) = A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2);
    C(2, 0) = A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0);
    C(2, 1) = A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1);
    C(2, 2) = A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0);
    R d = A(0, 0) * C(0, 0) + A(0, 1) * C(1, 0) + A(0, 2) * C(2, 0);
    R inv = R(1) / d;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C(i, j) *= inv;
    return C;
}

// ---------------------------------------------------------------- SVD
// Cyclic Jacobi on the symmetric A (in place); V accumulates the rotations.
template <typename R> void sym_eig3(M3<R> &A, M3<R> &V) {
    V = zero3<R>();
    V(0, 0) = V(1, 1) = V(2, 2) = 1;
    const R eps = std::numeric_limits<R>::epsilon();
    for (int sweep = 0; sweep < 60; ++sweep) {
        R off = std::fabs(A(0, 1)) + std::fabs(A(0, 2)) + std::fabs(A(1, 2));
        R diag = std::fabs(A(0, 0)) + std::fabs(A(1, 1)) + std::fabs(A(2, 2));
        if (off <= eps * eps * diag || off == R(0)) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                R apq = A(p, q);
                if (apq == R(0)) continue;
                R theta = (A(q, q) - A(p, p)) / (R(2) * apq);
                R t = (theta >= 0 ? R(1) : R(-1)) / (std::fabs(theta) + std::sqrt(theta * theta + R(1)));
                R c = R(1) / std::sqrt(t * t + R(1));
                R s = t * c;
                for (int k = 0; k < 3; ++k) {  // A <- J^T A J
                    R akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - s * akq;
                    A(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    R apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - s * aqk;
                    A(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    R vkp = V(k, p), vkq = V(k, q);
                    V(k, p) = c * vkp - s * vkq;
                    V(k, q) = s * vkp + c * vkq;
                }
            }
    }
}

template <typename R> void cross3(const R *a, const R *b, R *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
template <typename R> R norm3(const R *a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// IsotropicMaterial::computeSVD33modified (IsotropicMaterial.cpp:16-60):
// U, V rotations, S descending with the sign of an inversion carried by S[2].
template <typename R> void svd_modified(const M3<R> &F, M3<R> &U, R S[3], M3<R> &V) {
    const R eps_sv = R(1e-8);
    M3<R> A = mul(transpose(F), F);
    M3<R> W;
    sym_eig3(A, W);
    M3<R> B = mul(F, W);
    R sig[3];
    for (int i = 0; i < 3; ++i) {
        R col[3] = {B(0, i), B(1, i), B(2, i)};
        sig[i] = norm3(col);
    }
    int ord[3] = {0, 1, 2};
    std::sort(ord, ord + 3, [&](int a, int b) { return sig[a] > sig[b]; });
    for (int c = 0; c < 3; ++c) {
        S[c] = sig[ord[c]];
        for (int r = 0; r < 3; ++r) V(r, c) = W(r, ord[c]);
    }
    if (det3(V) < 0)
        for (int r = 0; r < 3; ++r) V(r, 0) = -V(r, 0);
    M3<R> FV = mul(F, V);
    for (int c = 0; c < 3; ++c) {
        R inv = S[c] > eps_sv ? R(1) / S[c] : R(0);
        for (int r = 0; r < 3; ++r) U(r, c) = FV(r, c) * inv;
    }
    if (S[0] < eps_sv) {
        U = zero3<R>();
        U(0, 0) = U(1, 1) = U(2, 2) = 1;
    } else if (S[1] < eps_sv) {
        R u0[3] = {U(0, 0), U(1, 0), U(2, 0)};
        // a unit vector orthogonal to u0 (Eigen's unitOrthogonal picks the
        // same family: zero the smallest-magnitude coordinate)
        R v1[3];
        if (std::fabs(u0[0]) <= std::fabs(u0[1]) && std::fabs(u0[0]) <= std::fabs(u0[2])) {
            R n = std::sqrt(u0[1] * u0[1] + u0[2] * u0[2]);
            v1[0] = 0; v1[1] = -u0[2] / n; v1[2] = u0[1] / n;
        } else {
            R n = std::sqrt(u0[0] * u0[0] + u0[1] * u0[1]);
            v1[0] = -u0[1] / n; v1[1] = u0[0] / n; v1[2] = 0;
        }
        R v2[3];
        cross3(u0, v1, v2);
        R n2 = norm3(v2);
        for (int r = 0; r < 3; ++r) { U(r, 1) = v1[r]; U(r, 2) = v2[r] / n2; }
    } else if (S[2] < eps_sv) {
        R u0[3] = {U(0, 0), U(1, 0), U(2, 0)}, u1[3] = {U(0, 1), U(1, 1), U(2, 1)}, u2[3];
        cross3(u0, u1, u2);
        R n = norm3(u2);
        for (int r = 0; r < 3; ++r) U(r, 2) = u2[r] / n;
    }
    if (det3(U) < 0) {
        for (int r = 0; r < 3; ++r) U(r, 2) = -U(r, 2);
        S[2] = -S[2];
    }
}

// ---------------------------------------------------------------- materials
template <typename R> struct TetIn {
    M3<R> Dinv;   // Dm^-1
    M3<R> AN;     // columns = area-weighted normals of corners 1..3
    R vol, mu, lambda;
};

template <typename R> M3<R> deformation_gradient(const R *x, const int *t, const M3<R> &Dinv) {
    M3<R> Ds;
    for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) Ds(d, c) = x[3 * t[c + 1] + d] - x[3 * t[0] + d];
    return mul(Ds, Dinv);
}

// IsotropicNeohookeanMaterial.cpp:104: P = mu (F - F^-T) + lambda ln(det F) F^-T
template <typename R> M3<R> pk1_nh(const M3<R> &F, R mu, R lambda) {
    M3<R> FiT = transpose(inv3(F));
    R lj = std::log(det3(F));
    M3<R> P;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) P(i, j) = (F(i, j) - FiT(i, j)) * mu + lambda * lj * FiT(i, j);
    return P;
}

// IsotropicNeohookeanMaterial.cpp:50-60
template <typename R> void stretch_gradient(const R s[3], R mu, R lambda, R g[3]) {
    R tmp = lambda * (std::log(s[0]) + std::log(s[1]) + std::log(s[2])) - mu;
    for (int i = 0; i < 3; ++i) g[i] = mu * s[i] + tmp / s[i];
}
// IsotropicNeohookeanMaterial.cpp:63-91 (row-major 3x3)
template <typename R> void stretch_hessian(const R s[3], R mu, R lambda, R h[9]) {
    R tmp = lambda * (std::log(s[0]) + std::log(s[1]) + std::log(s[2]));
    R tmp1 = mu + lambda - tmp, tmp2 = tmp - mu;
    R i1 = R(1) / s[0], i2 = R(1) / s[1], i3 = R(1) / s[2];
    h[0] = mu + tmp1 * i1 * i1;
    h[4] = mu + tmp1 * i2 * i2;
    h[8] = mu + tmp1 * i3 * i3;
    h[1] = h[3] = (tmp1 + tmp2) * i1 * i2;
    h[2] = h[6] = (tmp1 + tmp2) * i1 * i3;
    h[5] = h[7] = (tmp1 + tmp2) * i2 * i3;
}

// IsotropicMaterial.cpp:374-384: P = U diag(P^(sigma)) V^T
template <typename R> M3<R> pk1_stretch(const M3<R> &F, R mu, R lambda) {
    M3<R> U, V;
    R S[3], Ph[3];
    svd_modified(F, U, S, V);
    stretch_gradient(S, mu, lambda, Ph);
    M3<R> P;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) P(i, j) = U(i, 0) * Ph[0] * V(j, 0) + U(i, 1) * Ph[1] * V(j, 1) + U(i, 2) * Ph[2] * V(j, 2);
    return P;
}

// Corner forces: H = P * AN; corners 1..3 take H's columns, corner 0 takes
// minus their sum (IsotropicNeohookeanMaterial.cpp:105-110).
template <typename R> void corner_forces(const M3<R> &P, const M3<R> &AN, R out[12]) {
    M3<R> H = mul(P, AN);
    for (int d = 0; d < 3; ++d) {
        out[3 + d] = H(d, 0);
        out[6 + d] = H(d, 1);
        out[9 + d] = H(d, 2);
        out[d] = -(H(d, 0) + H(d, 1) + H(d, 2));
    }
}

// IsotropicNeohookeanMaterial.cpp:122-130; clamp 0: e > 1e-6 ? e : 0 (CPU),
// clamp 1: max(e, 0) (CUDAInterface.cu:549).
// keep_nan: an inverted tet's NaN energy stays NaN (RESTART control) instead of
// the reference clamps' 0.
template <typename R> R tet_energy(const M3<R> &F, R mu, R lambda, R vol, int clamp, int keep_nan = 0) {
    R I1 = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) I1 += F(i, j) * F(i, j);
    R lj = std::log(det3(F));
    R e = (R(0.5) * mu * (I1 - 3) - mu * lj + R(0.5) * lambda * lj * lj) * vol;
    if (keep_nan && e != e) return e;
    if (clamp == 0) return e > R(1e-6) ? e : R(0);
    return e > R(0) ? e : R(0);
}

// IsotropicMaterial::computeDPDFij (IsotropicMaterial.cpp:963-1019), with U, V
// passed as matrices (U_ik = U(i,k)).
template <typename R> M3<R> dPdFij(const M3<R> &U, const R s[3], const M3<R> &V, const R Ph[3], const R h[9], int i, int j) {
    M3<R> wU = zero3<R>(), wVT = zero3<R>();
    const int kl[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int q = 0; q < 3; ++q) {
        int k = kl[q][0], l = kl[q][1];
        // [[s_l, s_k], [s_k, s_l]] [a; b] = [U_ik V_jl; -U_il V_jk]
        R b0 = U(i, k) * V(j, l), b1 = -U(i, l) * V(j, k);
        R det = s[l] * s[l] - s[k] * s[k];
        R a = (s[l] * b0 - s[k] * b1) / det;
        R b = (s[l] * b1 - s[k] * b0) / det;
        wU(k, l) = a; wU(l, k) = -a;
        wVT(k, l) = b; wVT(l, k) = -b;
    }
    M3<R> dU = mul(U, wU);
    M3<R> dVT = mul(wVT, transpose(V));
    R dPh[3];
    for (int k = 0; k < 3; ++k) dPh[k] = h[k] * U(i, 0) * V(j, 0) + h[k + 3] * U(i, 1) * V(j, 1) + h[k + 6] * U(i, 2) * V(j, 2);
    M3<R> out;
    for (int m = 0; m < 3; ++m)
        for (int n = 0; n < 3; ++n) {
            R acc = 0;
            for (int c = 0; c < 3; ++c)
                acc += dU(m, c) * Ph[c] * V(n, c) + U(m, c) * dPh[c] * V(n, c) + U(m, c) * Ph[c] * dVT(c, n);
            out(m, n) = acc;
        }
    return out;
}

// The 12 diagonal entries of the element stiffness K = -df/dx
// (IsotropicMaterial.cpp:503-552), ordered corner-major: [3*corner + dof].
template <typename R> void hessian_diag_svd(const M3<R> &F, const TetIn<R> &tin, R out[12]) {
    M3<R> U, V;
    R S[3];
    svd_modified(F, U, S, V);
    const R eps = R(1e-6);
    R St[3];
    if (S[0] - S[2] < 2 * eps) { St[2] = S[2]; St[1] = St[2] + eps; St[0] = St[1] + eps; }
    else if (S[0] - S[1] < eps && S[1] - S[2] >= eps) { St[2] = S[2]; St[1] = S[0] - eps; St[0] = S[0]; }
    else if (S[0] - S[1] >= eps && S[1] - S[2] < eps) { St[2] = S[2]; St[1] = S[2] + eps; St[0] = S[0]; }
    else { St[0] = S[0]; St[1] = S[1]; St[2] = S[2]; }
    R Ph[3], h[9];
    stretch_gradient(St, tin.mu, tin.lambda, Ph);
    stretch_hessian(St, tin.mu, tin.lambda, h);
    // C[f][p] = dP_p / dF_f, both row-major 3x3 indices
    R C[9][9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            M3<R> d = dPdFij(U, St, V, Ph, h, i, j);
            for (int m = 0; m < 3; ++m)
                for (int n = 0; n < 3; ++n) C[3 * i + j][3 * m + n] = d(m, n);
        }
    // w_c: dF_{a q}/dx_{c,a} = w_c[q]; AN_c: corner c's normal (corner 0 = -sum).
    R w[4][3], an[4][3];
    for (int q = 0; q < 3; ++q) {
        w[0][q] = -(tin.Dinv(0, q) + tin.Dinv(1, q) + tin.Dinv(2, q));
        an[0][q] = -(tin.AN(q, 0) + tin.AN(q, 1) + tin.AN(q, 2));
        for (int c = 1; c < 4; ++c) { w[c][q] = tin.Dinv(c - 1, q); an[c][q] = tin.AN(q, c - 1); }
    }
    // dH_{a r}/dF_f = sum_s AN(s, r) C[f][3a + s]; K_diag(c, a) = -sum_{q} w_c[q] * dH_{a c}/dF_{3a+q}
    for (int c = 0; c < 4; ++c)
        for (int a = 0; a < 3; ++a) {
            R acc = 0;
            for (int q = 0; q < 3; ++q) {
                R dH = 0;
                for (int s = 0; s < 3; ++s) dH += an[c][s] * C[3 * a + q][3 * a + s];
                acc += w[c][q] * dH;
            }
            out[3 * c + a] = -acc;
        }
}

// Closed form of the same diagonal for the neo-Hookean energy (no SVD):
// dP_{dj}/dF_{dq} = mu delta_jq + (mu + lambda - lambda ln J) G_dj G_dq with
// G = F^-T, so K_diag(c, d) = -[mu (w_c . AN_c) + (mu + lambda - lambda lnJ)
// (G_d . AN_c)(G_d . w_c)].  This is what the device kernel evaluates.
template <typename R> void hessian_diag_closed(const M3<R> &F, const TetIn<R> &tin, R out[12]) {
    M3<R> G = transpose(inv3(F));
    R lj = std::log(det3(F));
    R beta = tin.mu + tin.lambda - tin.lambda * lj;
    R w[4][3], an[4][3];
    for (int q = 0; q < 3; ++q) {
        w[0][q] = -(tin.Dinv(0, q) + tin.Dinv(1, q) + tin.Dinv(2, q));
        an[0][q] = -(tin.AN(q, 0) + tin.AN(q, 1) + tin.AN(q, 2));
        for (int c = 1; c < 4; ++c) { w[c][q] = tin.Dinv(c - 1, q); an[c][q] = tin.AN(q, c - 1); }
    }
    for (int c = 0; c < 4; ++c) {
        R wa = w[c][0] * an[c][0] + w[c][1] * an[c][1] + w[c][2] * an[c][2];
        for (int d = 0; d < 3; ++d) {
            R ga = G(d, 0) * an[c][0] + G(d, 1) * an[c][1] + G(d, 2) * an[c][2];
            R gw = G(d, 0) * w[c][0] + G(d, 1) * w[c][1] + G(d, 2) * w[c][2];
            out[3 * c + d] = -(tin.mu * wa + beta * ga * gw);
        }
    }
}

// ---------------------------------------------------------------- mesh state
template <typename R> struct Mesh {
    int n, t;
    const int *tets;
    std::vector<TetIn<R>> tin;
    std::vector<R> mass, grav_y;   // mass: pinned = 1e8; grav_y = -9.8 * lumped mass (pre-pin)
    std::vector<int> pinned;
    std::vector<int> iptr, ient;   // node -> 4 * tet + corner, ascending tet
    // per-tet scratch reused by every pass (a fresh 12T buffer per pass cost
    // more in page faults than the arithmetic on a 1M-tet mesh)
    mutable std::vector<R> all, e;
};

template <typename R> Mesh<R> load_mesh(int n, int t, const int *tets, const double *dinv9, const double *an9,
                                        const double *vol, const double *mu, const double *lambda,
                                        const double *mass, const double *grav_y, const int *pin_mask) {
    Mesh<R> m;
    m.n = n; m.t = t; m.tets = tets;
    m.tin.resize(t);
    for (int i = 0; i < t; ++i) {
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) { m.tin[i].Dinv(r, c) = (R)dinv9[9 * i + 3 * r + c]; m.tin[i].AN(r, c) = (R)an9[9 * i + 3 * r + c]; }
        m.tin[i].vol = (R)vol[i]; m.tin[i].mu = (R)mu[i]; m.tin[i].lambda = (R)lambda[i];
    }
    m.mass.assign(mass, mass + n);
    m.grav_y.assign(grav_y, grav_y + n);
    m.pinned.assign(pin_mask, pin_mask + n);
    m.iptr.assign(n + 1, 0);
    for (int i = 0; i < 4 * t; ++i) m.iptr[tets[i] + 1]++;
    for (int i = 0; i < n; ++i) m.iptr[i + 1] += m.iptr[i];
    m.ient.resize(4 * (size_t)t);
    std::vector<int> fill(m.iptr.begin(), m.iptr.end() - 1);
    for (int i = 0; i < 4 * t; ++i) m.ient[fill[tets[i]]++] = i;
    return m;
}

// Per-node sums of per-tet 12-vectors, each node adding its incident (tet,
// corner) terms in ascending tet order: the order in which a serial scatter
// over tets adds them, so the result is the scatter's, bit for bit.
template <typename R> void gather_nodes(const Mesh<R> &m, const std::vector<R> &all, std::vector<R> &out) {
    out.assign(3 * (size_t)m.n, R(0));
#pragma omp parallel for schedule(static)
    for (int v = 0; v < m.n; ++v) {
        R s[3] = {0, 0, 0};
        for (int j = m.iptr[v]; j < m.iptr[v + 1]; ++j) {
            const R *c = &all[3 * (size_t)m.ient[j]];
            for (int d = 0; d < 3; ++d) s[d] += c[d];
        }
        for (int d = 0; d < 3; ++d) out[3 * (size_t)v + d] = s[d];
    }
}

// Per-tet terms are evaluated in parallel (OpenMP, when built with it) into a
// per-tet buffer, then gathered per node in tet order: the sums are the
// serial scatter's, bit for bit, whatever the thread count.

// Per-node elastic force in tet order (the reference's scatter order).
template <typename R> void elastic_forces(const Mesh<R> &m, const std::vector<R> &x, int material, std::vector<R> &f) {
    f.assign(3 * (size_t)m.n, R(0));
    std::vector<R> &all = m.all;
    all.resize(12 * (size_t)m.t);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m.t; ++i) {
        const int *t = m.tets + 4 * i;
        M3<R> F = deformation_gradient(x.data(), t, m.tin[i].Dinv);
        M3<R> P = material == 1 ? pk1_stretch(F, m.tin[i].mu, m.tin[i].lambda) : pk1_nh(F, m.tin[i].mu, m.tin[i].lambda);
        corner_forces(P, m.tin[i].AN, &all[12 * (size_t)i]);
    }
    gather_nodes(m, all, f);
}

template <typename R> void hessian_diag_nodes(const Mesh<R> &m, const std::vector<R> &x, int closed, std::vector<R> &hd) {
    hd.assign(3 * (size_t)m.n, R(0));
    std::vector<R> &all = m.all;
    all.resize(12 * (size_t)m.t);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m.t; ++i) {
        const int *t = m.tets + 4 * i;
        M3<R> F = deformation_gradient(x.data(), t, m.tin[i].Dinv);
        if (closed) hessian_diag_closed(F, m.tin[i], &all[12 * (size_t)i]);
        else hessian_diag_svd(F, m.tin[i], &all[12 * (size_t)i]);
    }
    gather_nodes(m, all, hd);
}

// Sum of the clamped tet energies, added in tet order.
template <typename R> R elastic_energy(const Mesh<R> &m, const std::vector<R> &x, int clamp, int keep_nan) {
    std::vector<R> &e = m.e;
    e.resize(m.t);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m.t; ++i) {
        M3<R> F = deformation_gradient(x.data(), m.tets + 4 * i, m.tin[i].Dinv);
        e[i] = tet_energy(F, m.tin[i].mu, m.tin[i].lambda, m.tin[i].vol, clamp, keep_nan);
    }
    R Ee = 0;
    for (int i = 0; i < m.t; ++i) Ee += e[i];
    return Ee;
}

}  // namespace

// ============================================================== C ABI
extern "C" {

// Threads of the per-tet loops (1 = serial; ignored without OpenMP).  Returns
// the count in effect.
int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// Step parameters (mirrors pbs_step_params of include/phybs.h field by field).
typedef struct orc_params {
    float h;
    int max_iters;
    float tol;
    int control;            // 0: reference (iterations -= k-8; k -= 1), 1: restart
    float alpha0, alpha_min, alpha_shrink;
    int line_search_every, hessian_every;
    int n_profile;
    int profile_k[4];
    float profile_rho[4];
    float damping, warm_start;
    float body_force_scale;  // times gravity + external forces enter the gradient (2: DescentOptimize.cpp:52 with
                             // IsotropicNeohookeanMaterial.cpp:98; 1: CUDAInterface.cu:600-602)
    int energy_clamp;
    int material;           // 0 NH invariants, 1 stretch-based
    int hessian_closed;     // 1: closed-form diagonal, 0: SVD (Xu et al.) path
    float alpha_grow;        // RESTART: alpha <- min(alpha * alpha_grow, alpha0) on an accepted check
} orc_params;

typedef struct orc_stats {
    int passes, k_final, rejections, converged;
    double alpha, energy, energy_old, rho, omega, residual_ratio, residual0;
} orc_stats;

// Rest state (TetMesh.cpp:186-216, 279-294), computed in precision `prec`
// (32 or 64).  Outputs: Dm^-1 and AN row-major per tet (9T), |det|/6 (T),
// signed det/6 (T), lumped mass with pins = 1e8 (N), gravity_y = -9.8 * lumped
// mass (N, before pinning).
int orc_rest(int prec, int n, const double *pos, int t, const int *tets, double density, const int *pin_mask,
             double *dinv9, double *an9, double *vol, double *svol, double *mass, double *grav_y) {
    auto run = [&](auto zero) {
        using R = decltype(zero);
        std::vector<R> m(n, R(0));
        const int edge[3][4] = {{1, 0, 2, 3}, {2, 0, 3, 1}, {3, 0, 1, 2}};
        for (int i = 0; i < t; ++i) {
            const int *q = tets + 4 * i;
            M3<R> Dm;
            for (int c = 0; c < 3; ++c)
                for (int d = 0; d < 3; ++d) Dm(d, c) = (R)pos[3 * q[c + 1] + d] - (R)pos[3 * q[0] + d];
            R det = det3(Dm);
            R v = std::fabs(det) / R(6);
            vol[i] = v;
            svol[i] = det / R(6);
            R w = v / R(4) * (R)density;
            for (int c = 0; c < 4; ++c) m[q[c]] += w;
            M3<R> Di = inv3(Dm);
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) dinv9[9 * i + 3 * r + c] = Di(r, c);
            for (int k = 0; k < 3; ++k) {
                R a[3], b[3], c3[3];
                for (int d = 0; d < 3; ++d) {
                    a[d] = (R)pos[3 * q[edge[k][1]] + d] - (R)pos[3 * q[edge[k][0]] + d];
                    b[d] = (R)pos[3 * q[edge[k][2]] + d] - (R)pos[3 * q[edge[k][0]] + d];
                    c3[d] = (R)pos[3 * q[edge[k][3]] + d] - (R)pos[3 * q[edge[k][0]] + d];
                }
                R x1[3], x2[3], x3[3];
                cross3(a, b, x1); cross3(b, c3, x2); cross3(c3, a, x3);
                for (int d = 0; d < 3; ++d) an9[9 * i + 3 * d + k] = -(x1[d] + x2[d] + x3[d]) / R(6);
            }
        }
        for (int i = 0; i < n; ++i) {
            grav_y[i] = (R)(-9.8) * m[i];
            mass[i] = pin_mask[i] ? 1e8 : (double)m[i];
        }
    };
    if (prec == 64) run(0.0); else run(0.0f);
    return 0;
}

// Per-tet corner forces (12 per tet: corner-major xyz), energy and the 12
// Hessian-diagonal entries, at positions x.
int orc_tet_eval(int prec, int material, int clamp, int hessian_closed, int n, const double *x, int t, const int *tets,
                 const double *dinv9, const double *an9, const double *vol, const double *mu, const double *lambda,
                 double *corner12, double *energy, double *hdiag12) {
    auto run = [&](auto zero) {
        using R = decltype(zero);
        std::vector<R> xr(x, x + 3 * (size_t)n);
        for (int i = 0; i < t; ++i) {
            TetIn<R> tin;
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) { tin.Dinv(r, c) = (R)dinv9[9 * i + 3 * r + c]; tin.AN(r, c) = (R)an9[9 * i + 3 * r + c]; }
            tin.vol = (R)vol[i]; tin.mu = (R)mu[i]; tin.lambda = (R)lambda[i];
            M3<R> F = deformation_gradient(xr.data(), tets + 4 * i, tin.Dinv);
            R out[12];
            if (corner12) {
                M3<R> P = material == 1 ? pk1_stretch(F, tin.mu, tin.lambda) : pk1_nh(F, tin.mu, tin.lambda);
                corner_forces(P, tin.AN, out);
                for (int k = 0; k < 12; ++k) corner12[12 * i + k] = out[k];
            }
            if (energy) energy[i] = tet_energy(F, tin.mu, tin.lambda, tin.vol, clamp);
            if (hdiag12) {
                if (hessian_closed) hessian_diag_closed(F, tin, out); else hessian_diag_svd(F, tin, out);
                for (int k = 0; k < 12; ++k) hdiag12[12 * i + k] = out[k];
            }
        }
    };
    if (prec == 64) run(0.0); else run(0.0f);
    return 0;
}

// Modified SVD of a batch of 3x3 matrices (row-major in and out).
int orc_svd(int prec, int count, const double *F9, double *U9, double *S3, double *V9) {
    auto run = [&](auto zero) {
        using R = decltype(zero);
        for (int i = 0; i < count; ++i) {
            M3<R> F, U, V;
            R S[3];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) F(r, c) = (R)F9[9 * i + 3 * r + c];
            svd_modified(F, U, S, V);
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) { U9[9 * i + 3 * r + c] = U(r, c); V9[9 * i + 3 * r + c] = V(r, c); }
            for (int k = 0; k < 3; ++k) S3[3 * i + k] = S[k];
        }
    };
    if (prec == 64) run(0.0); else run(0.0f);
    return 0;
}

// One descent time step of one instance (DescentOptimize.cpp:91-188), in
// precision `prec`.  State in/out: x0 (node positions at step start ->
// end), v, v_old (the reference's m_vel_old).  ext: external forces (3N).
// The Chebyshev scalars rho/omega persist across steps in *cheb (2 values)
// exactly as DescentOptimize's members do.
int orc_step(int prec, const orc_params *p, int n, int t, const int *tets, const double *dinv9, const double *an9,
             const double *vol, const double *mu, const double *lambda, const double *mass, const double *grav_y,
             const int *pin_mask, double *x0_io, double *v_io, double *vold_io, const double *ext, double *cheb,
             orc_stats *st) {
    auto run = [&](auto zero) {
        using R = decltype(zero);
        Mesh<R> m = load_mesh<R>(n, t, tets, dinv9, an9, vol, mu, lambda, mass, grav_y, pin_mask);
        const size_t N3 = 3 * (size_t)n;
        std::vector<R> x0(x0_io, x0_io + N3), v(v_io, v_io + N3), vold(vold_io, vold_io + N3);
        std::vector<R> ex(N3);
        for (size_t i = 0; i < N3; ++i) ex[i] = ext ? (R)ext[i] : R(0);
        const R h = (R)p->h;
        const R h2inv = R(1) / (h * h);
        // DescentOptimize::initialization (DescentOptimize.cpp:35-41)
        std::vector<R> xt(N3), x(N3), xlast(N3), xold(N3), xnext(N3), g(N3), hq(N3, R(0)), fel;
        for (size_t i = 0; i < N3; ++i) {
            xt[i] = x0[i] + h * v[i];
            x[i] = xt[i] + (R)p->warm_start * h * (v[i] - vold[i]);
        }
        // RESTART control: a guess that inverts a tet (det F <= 0) starts the
        // step from x0 instead, as the device's k_guess_check / k_guess_fallback do
        if (p->control == 1) {
            bool bad = false;
            for (int i = 0; i < m.t && !bad; ++i) {
                M3<R> F = deformation_gradient(x.data(), m.tets + 4 * i, m.tin[i].Dinv);
                if (!(det3(F) > R(0))) bad = true;
            }
            if (bad) x = x0;
        }
        xlast = x;  // only read once omega != 1, i.e. after it was set below
        R rho = (R)cheb[0], omega = (R)cheb[1];
        R alpha = (R)p->alpha0;
        R E = 0, Eold = 0;
        int iters = p->max_iters;
        int passes = 0, rejections = 0, converged = 0;
        double g0 = -1, ratio = -1;
        int k, k_restart = 0;  // RESTART control runs the rho schedule from the last restart
        // RESTART control: a non-finite residual makes the next iteration a
        // line-search check, and a non-finite energy is a rejection
        bool force_check = false;
        const bool restart = p->control == 1;
        for (k = 0; k < iters; ++k) {
            if (alpha < (R)p->alpha_min) break;
            ++passes;
            if (k % p->line_search_every == 0 || force_check) {
                force_check = false;
                // DescentOptimize::computeTotalEnergy (DescentOptimize.cpp:63-89): the
                // gravity term 0.5 m 2 g y is -gravity_y . y; plus the external work
                // -f_ext . x over free nodes.
                const R Ee = elastic_energy(m, x, p->energy_clamp, restart ? 1 : 0);
                R En = 0;
                for (int i = 0; i < n; ++i) {
                    if (m.pinned[i]) continue;
                    R d2 = 0, w = 0;
                    for (int d = 0; d < 3; ++d) { R dd = x[3 * i + d] - xt[3 * i + d]; d2 += dd * dd; w += ex[3 * i + d] * x[3 * i + d]; }
                    En += R(0.5) * m.mass[i] * d2 * h2inv - m.grav_y[i] * x[3 * i + 1] - w;
                }
                E = Ee + En;
                if (!std::isfinite(E) && (k == 0 || !restart)) break;  // a non-finite step start: give up
                if (k != 0 && (E > Eold || !std::isfinite(E))) {
                    alpha *= (R)p->alpha_shrink;
                    ++rejections;
                    if (p->control == 0) iters -= k - p->line_search_every;
                    k -= 1;
                    x = xold;
                    if (p->control == 1) { xlast = xold; k_restart = k + 1; }
                    continue;
                }
                Eold = E;
                if (restart && k != 0 && k > k_restart) alpha = std::min(alpha * (R)p->alpha_grow, (R)p->alpha0);
                xold = x;
            }
            if (k % p->hessian_every == 0) {
                hessian_diag_nodes(m, x, p->hessian_closed, hq);
                for (int i = 0; i < n; ++i)
                    for (int d = 0; d < 3; ++d) hq[3 * i + d] += (R)m.mass[i] * h2inv;
            }
            // DescentOptimize::computeGradient (DescentOptimize.cpp:43-61).
            elastic_forces(m, x, p->material, fel);
            // the gradient in parallel (elementwise), |g|^2 summed in node order
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; ++i)
                for (int d = 0; d < 3; ++d) {
                    size_t id = 3 * (size_t)i + d;
                    R body = ex[id] + (d == 1 ? m.grav_y[i] : R(0));
                    R gv = (x[id] - xt[id]) * m.mass[i] * h2inv - fel[id] - (R)p->body_force_scale * body;
                    if (m.pinned[i]) gv = 0;
                    g[id] = gv;
                }
            double r2 = 0;
            for (size_t id = 0; id < N3; ++id) r2 += (double)g[id] * (double)g[id];
            if (!std::isfinite(r2)) {
                if (!restart) break;  // the device stops with PBS_E_NONFINITE
                force_check = true;   // the next iteration measures the energy and restores
            }
            double r = std::sqrt(r2);
            if (k == 0) g0 = r;
            ratio = g0 > 0 ? r / g0 : 0.0;
            if (p->tol > 0 && k > 0 && r <= (double)p->tol * g0) { converged = 1; break; }
#pragma omp parallel for schedule(static)
            for (long long id = 0; id < (long long)N3; ++id) xnext[id] = x[id] + alpha * (g[id] / -hq[id]);
            // Chebyshev schedule (DescentOptimize.cpp:156-178)
            const int ks = k - k_restart;
            if (ks == 0) { rho = 0; omega = 1; }
            omega = R(4) / (R(4) - rho * rho * omega);
            for (int i = 0; i < p->n_profile; i++) {
                if (ks == p->profile_k[i] - 1) { rho = 0; omega = 1; }
                if (ks == p->profile_k[i]) { rho = (R)p->profile_rho[i]; omega = R(2) / (R(2) - rho * rho); break; }
            }
            if (omega != R(1)) {
#pragma omp parallel for schedule(static)
                for (long long id = 0; id < (long long)N3; ++id) xnext[id] = omega * (xnext[id] - xlast[id]) + xlast[id];
            }
            // xlast <- x, x <- xnext (xnext is rewritten before it is read again)
            std::swap(xlast, x);
            std::swap(x, xnext);
        }
        // DescentOptimize.cpp:183-185
        for (size_t i = 0; i < N3; ++i) {
            vold[i] = v[i];
            v[i] = (R)p->damping * (x[i] - x0[i]) / h;
            x0[i] = x[i];
        }
        for (size_t i = 0; i < N3; ++i) { x0_io[i] = x0[i]; v_io[i] = v[i]; vold_io[i] = vold[i]; }
        cheb[0] = rho; cheb[1] = omega;
        if (st) {
            st->passes = passes; st->k_final = k; st->rejections = rejections; st->converged = converged;
            st->alpha = alpha; st->energy = E; st->energy_old = Eold; st->rho = rho; st->omega = omega;
            st->residual_ratio = ratio; st->residual0 = g0;
        }
    };
    if (prec == 64) run(0.0); else run(0.0f);
    return 0;
}

// Assembled per-node elastic force (tet-order scatter) and Hessian diagonal.
int orc_node_eval(int prec, int material, int hessian_closed, int n, const double *x, int t, const int *tets,
                  const double *dinv9, const double *an9, const double *vol, const double *mu, const double *lambda,
                  double *force3, double *hd3) {
    auto run = [&](auto zero) {
        using R = decltype(zero);
        std::vector<double> ones(n, 1.0), zeros(n, 0.0);
        std::vector<int> nop(n, 0);
        Mesh<R> m = load_mesh<R>(n, t, tets, dinv9, an9, vol, mu, lambda, ones.data(), zeros.data(), nop.data());
        std::vector<R> xr(x, x + 3 * (size_t)n), out;
        if (force3) {
            elastic_forces(m, xr, material, out);
            for (size_t i = 0; i < out.size(); ++i) force3[i] = out[i];
        }
        if (hd3) {
            hessian_diag_nodes(m, xr, hessian_closed, out);
            for (size_t i = 0; i < out.size(); ++i) hd3[i] = out[i];
        }
    };
    if (prec == 64) run(0.0); else run(0.0f);
    return 0;
}

// Rest data in FP32 exactly as TetMesh::initModel forms it (TetMesh.cpp:186-216)
// with Eigen 3.2's 3x3 determinant (row-0 cofactor expansion, Determinant.h)
// and inverse (adjugate of the column-0 cofactors times 1 / det,
// Inverse.h:117-159): Dm^-1 row-major (9T), inverse masses (N; 0 when
// pinned) and gravity_y = -gravity * lumped mass (N).
static inline float eig_cof(const float m[3][3], int i, int j) {
    const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
    return m[i1][j1] * m[i2][j2] - m[i1][j2] * m[i2][j1];
}

int orc_rest_eigen32(int n, const float *pos, int t, const int *tets, float density, float gravity,
                     const int *pin_mask, float *dinv9, float *inv_mass, float *grav_y) {
    std::vector<float> mass(n, 0.0f);
    for (int i = 0; i < t; ++i) {
        const int *q = tets + 4 * (size_t)i;
        float m[3][3];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) m[r][c] = pos[3 * (size_t)q[c + 1] + r] - pos[3 * (size_t)q[0] + r];
        const float det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                          m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                          m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
        const float vol = (float)((double)std::fabs(det) / 6.0);
        const float w = (float)((double)vol / 4.0 * (double)density);
        for (int c = 0; c < 4; ++c) mass[q[c]] += w;
        const float c0[3] = {eig_cof(m, 0, 0), eig_cof(m, 1, 0), eig_cof(m, 2, 0)};
        const float d = c0[0] * m[0][0] + (c0[1] * m[1][0] + c0[2] * m[2][0]);
        const float inv = 1.0f / d;
        float *o = dinv9 + 9 * (size_t)i;
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) o[3 * r + k] = (r == 0 ? c0[k] : eig_cof(m, k, r)) * inv;
    }
    for (int i = 0; i < n; ++i) {
        grav_y[i] = -gravity * mass[i];
        inv_mass[i] = pin_mask[i] ? 0.0f : (float)(1.0 / (double)mass[i]);
    }
    return 0;
}

// Strain-based position-based dynamics, FP32 in the reference's operation
// order (this file is built with -ffp-contract=off):
// PosBaseDynamic::doStepStrainConstraints (PosBaseDynamic.cpp:12-53) and
// solveStrainConstraints (:55-117).  Eigen 3.2 evaluates a 3x3 * 3x1 product
// as ((a0 b0 + a1 b1) + a2 b2) (CoeffBasedProduct.h) and a 3-vector dot or
// squaredNorm as x0 + (x1 + x2) (redux_novec_unroller's halving).
// dinv9: Dm^-1 row-major per tet; pos, vel: 3n in/out.
static inline float pbd_dot3(const float *a, const float *b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }

static void pbd_tet(const float *p[4], const float w[4], const float *D, const float *stretch, const float *shear,
                    float eps, float dp[4][3]) {
    std::memset(dp, 0, sizeof(float) * 12);
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j <= i; ++j) {
            float P[3][3];  // P(r, c): column c = (p_{c+1} + dp_{c+1}) - (p_0 + dp_0)
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) P[r][c] = (p[c + 1][r] + dp[c + 1][r]) - (p[0][r] + dp[0][r]);
            float fi[3], fj[3];
            for (int r = 0; r < 3; ++r) {
                fi[r] = (P[r][0] * D[3 * 0 + i] + P[r][1] * D[3 * 1 + i]) + P[r][2] * D[3 * 2 + i];
                fj[r] = (P[r][0] * D[3 * 0 + j] + P[r][1] * D[3 * 1 + j]) + P[r][2] * D[3 * 2 + j];
            }
            const float Sij = pbd_dot3(fi, fj);
            float d[4][3] = {{0.f, 0.f, 0.f}};
            for (int k = 0; k < 3; ++k) {
                for (int r = 0; r < 3; ++r) {
                    d[k + 1][r] = fj[r] * D[3 * k + i] + fi[r] * D[3 * k + j];
                    d[0][r] -= d[k + 1][r];
                }
            }
            float lambda = w[0] * pbd_dot3(d[0], d[0]) + w[1] * pbd_dot3(d[1], d[1]) + w[2] * pbd_dot3(d[2], d[2]) +
                           w[3] * pbd_dot3(d[3], d[3]);
            if (lambda < eps) continue;
            if (i == j)
                lambda = (float)(((double)Sij - 1.0) / (double)lambda * (double)stretch[i]);
            else
                lambda = Sij / lambda * shear[i + j - 1];
            for (int c = 0; c < 4; ++c) {
                const float s = lambda * w[c];
                for (int r = 0; r < 3; ++r) dp[c][r] -= s * d[c][r];
            }
        }
    }
}

int orc_pbd_step(int n, int t, const int *tets, const float *dinv9, const float *inv_mass, const float *forces,
                 float dt, int iters, const float *stretch, const float *shear, float eps, float *pos, float *vel) {
    std::vector<float> p(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        const float s = dt * inv_mass[i];
        for (int r = 0; r < 3; ++r) {
            const size_t k = 3 * (size_t)i + r;
            p[k] = pos[k] + dt * (vel[k] + s * forces[k]);
        }
    }
    for (int it = 0; it < iters; ++it) {
        for (int j = 0; j < t; ++j) {
            const int *q = tets + 4 * (size_t)j;
            float cp[4][3];
            const float *pp[4];
            float w[4];
            for (int c = 0; c < 4; ++c) {
                for (int r = 0; r < 3; ++r) cp[c][r] = p[3 * (size_t)q[c] + r];
                pp[c] = cp[c];
                w[c] = inv_mass[q[c]];
            }
            float dp[4][3];
            pbd_tet(pp, w, dinv9 + 9 * (size_t)j, stretch, shear, eps, dp);
            for (int c = 0; c < 4; ++c)
                for (int r = 0; r < 3; ++r) p[3 * (size_t)q[c] + r] += dp[c][r];
        }
    }
    for (size_t k = 0; k < 3 * (size_t)n; ++k) {
        vel[k] = (p[k] - pos[k]) * 0.99f / dt;
        pos[k] = p[k];
    }
    return 0;
}

// The reference's OpenMP force evaluation,
// IsotropicMaterial::computeInnerForcesfromFhats2(num_Threads)
// (IsotropicMaterial.cpp:411-453), in FP32 on `nthreads` threads with its
// structure: computeFhats (the modified SVD of every tet's F, in parallel,
// into per-tet Fhat / U / V arrays), then a parallel loop that forms
// P^ (IsotropicNeohookeanMaterial.cpp:50-60), P = U diag(P^) V^T and
// H = P AN, and adds the four corner forces to the node array under one
// global lock.  Forces start at zero (the reference starts from gravity +
// external forces).  The scatter's order follows the threads' timing, so the
// sums are not reproducible to the last bit; this is the CPU comparator of
// the force evaluation, not a parity reference.
int orc_forces_fhats2_omp(int nthreads, int n, const float *x, int t, const int *tets, const float *dinv9,
                          const float *an9, const float *mu, const float *lambda, float *forces3) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    std::vector<float> fhat(3 * (size_t)t), Us(9 * (size_t)t), Vs(9 * (size_t)t);
    // computeFhats(num_Threads)
#pragma omp parallel for
    for (int i = 0; i < t; ++i) {
        M3<float> Dinv, U, V;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Dinv(r, c) = dinv9[9 * (size_t)i + 3 * r + c];
        const M3<float> F = deformation_gradient(x, tets + 4 * (size_t)i, Dinv);
        float S[3];
        svd_modified(F, U, S, V);
        for (int k = 0; k < 3; ++k) fhat[3 * (size_t)i + k] = S[k];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                Us[9 * (size_t)i + 3 * r + c] = U(r, c);
                Vs[9 * (size_t)i + 3 * r + c] = V(r, c);
            }
    }
    for (size_t k = 0; k < 3 * (size_t)n; ++k) forces3[k] = 0.0f;
#ifdef _OPENMP
    omp_lock_t lck;
    omp_init_lock(&lck);
#endif
#pragma omp parallel for
    for (int i = 0; i < t; ++i) {
        float ph[3];
        stretch_gradient(&fhat[3 * (size_t)i], mu[i], lambda[i], ph);
        M3<float> P, AN;
        const float *U = &Us[9 * (size_t)i], *V = &Vs[9 * (size_t)i];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                P(r, c) = U[3 * r] * ph[0] * V[3 * c] + U[3 * r + 1] * ph[1] * V[3 * c + 1] +
                          U[3 * r + 2] * ph[2] * V[3 * c + 2];
                AN(r, c) = an9[9 * (size_t)i + 3 * r + c];
            }
        float f[12];
        corner_forces(P, AN, f);
        const int *q = tets + 4 * (size_t)i;
#ifdef _OPENMP
        omp_set_lock(&lck);
#endif
        for (int c = 0; c < 4; ++c)
            for (int d = 0; d < 3; ++d) forces3[3 * (size_t)q[c] + d] += f[3 * c + d];
#ifdef _OPENMP
        omp_unset_lock(&lck);
#endif
    }
#ifdef _OPENMP
    omp_destroy_lock(&lck);
#endif
    return 0;
}

}  // extern "C"
