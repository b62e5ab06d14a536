// Drives the CUDAInterface-shaped wrapper the way FVM/fvm.cpp does
// (construct from a mesh, doDescentOpt, updateNodePositions, reset, and the
// backward-Euler, PBD and projective-dynamics steps) on a 2x1x1-cube bar.
// Prints "pattern <nnz>" (host-only), then either "step <max |x - rest|>"
// followed by "backeuler", "pbd" and "pd" lines of the same form, or
// "error <code>" when no GB300 is present.
#include <cmath>
#include <cstdio>
#include <vector>

#include "phybs_cuda_interface.hpp"

int main() {
    // 3x2x2 grid nodes, x fastest; 2 cubes along x, 6 tets each (Kuhn split)
    const int nx = 2, ny = 1, nz = 1;
    std::vector<float> rest;
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                rest.push_back(0.1f * i);
                rest.push_back(0.1f * j);
                rest.push_back(0.1f * k);
            }
    const int n = (int)rest.size() / 3;
    auto id = [&](int i, int j, int k) { return i + (nx + 1) * (j + (ny + 1) * k); };
    const int kuhn[6][4] = {{0, 1, 3, 7}, {0, 1, 5, 7}, {0, 2, 3, 7}, {0, 2, 6, 7}, {0, 4, 5, 7}, {0, 4, 6, 7}};
    std::vector<int> tets;
    for (int i = 0; i < nx; ++i) {
        int c[8];
        for (int b = 0; b < 8; ++b) c[b] = id(i + (b & 1), (b >> 1) & 1, (b >> 2) & 1);
        for (auto &t : kuhn) {
            int q[4] = {c[t[0]], c[t[1]], c[t[2]], c[t[3]]};
            // orient positively
            float e[3][3];
            for (int a = 0; a < 3; ++a)
                for (int d = 0; d < 3; ++d) e[a][d] = rest[3 * q[a + 1] + d] - rest[3 * q[0] + d];
            float det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) - e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
                        e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
            if (det < 0) { int s = q[2]; q[2] = q[3]; q[3] = s; }
            tets.insert(tets.end(), q, q + 4);
        }
    }
    const int t = (int)tets.size() / 4;
    std::vector<int> mask(n, 0);
    for (int v = 0; v < n; ++v) mask[v] = rest[3 * v] == 0.0f ? 1 : 0;  // x = 0 face pinned
    phybs::StiffnessPattern p = phybs::stiffness_pattern(n, t, tets.data());
    std::printf("pattern %zu\n", p.col.size());
    try {
        phybs::CUDAInterface ci(n, rest.data(), rest.data(), mask.data(), t, tets.data(), 5e4f, 0.4f, 1000.f);
        std::vector<float> ext(3 * n, 0.f), out(3 * n, 0.f);
        ci.doDescentOpt(1.0f / 30, 96, ext.data(), out.data());
        float dmax = 0.f;
        for (int i = 0; i < 3 * n; ++i) dmax = std::fmax(dmax, std::fabs(out[i] - rest[i]));
        ci.updateNodePositions(out.data());
        ci.reset();
        std::printf("step %g\n", dmax);
        // the viewer's other integrators on the same handle (fvm.cpp:162-183)
        auto moved = [&]() {
            float d = 0.f;
            for (int i = 0; i < 3 * n; ++i) d = std::fmax(d, std::fabs(out[i] - rest[i]));
            return d;
        };
        ci.computeInnerforces();
        ci.computeGlobalStiffnessMatrix();
        ci.doBackEuler(out.data());
        std::printf("backeuler %g\n", moved());
        ci.reset();
        ci.pbdStep(1.0f / 30, ext.data(), out.data());
        std::printf("pbd %g\n", moved());
        ci.reset();
        ci.projectiveDynamicsStep(0.03f, 0.03f, ext.data(), out.data());
        std::printf("pd %g\n", moved());
    } catch (const phybs::Error &e) {
        std::printf("error %d\n", e.code());
    }
    return 0;
}
