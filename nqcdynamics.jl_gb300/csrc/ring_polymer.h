// Ring-polymer primitives, evaluated once per run on the host and shared by
// the engine's set-up code and the CPU oracle.
//
//  * Normal-mode transformation (RingPolymerArrays.NormalModeTransformation,
//    used at src/DynamicsMethods/IntegrationAlgorithms/bcb_electronics.jl:67-71):
//    orthogonal U[j,k] for bead j and mode k (0-based),
//        k = 0          : 1/sqrt(n)
//        0 < k < n/2    : sqrt(2/n) cos(2 pi j k / n)
//        k = n/2        : (-1)^j / sqrt(n)
//        k > n/2        : sqrt(2/n) sin(2 pi j k / n)
//    to normal modes q = U^T x, back x = U q; the centroid is q_0 / sqrt(n).
//    This arrangement reproduces the reference documentation's n = 4 values
//    (docs/src/api/RingPolymerArrays/ringpolymerarrays.md:93-133).
//  * Cayley propagator of the free ring polymer (cayley_propagator,
//    src/RingPolymers/ring_polymer.jl:71-82, full step as used at
//    bcb_electronics.jl:36): for mode frequency w_k = 2 w_n sin(k pi / n),
//    w_n = n / beta, cay(dt A) = (I - dt A/2)^-1 (I + dt A/2) with
//    A = [[0, 1], [-w^2, 0]], in closed form
//        [[1 - dt^2 w^2 / 4, dt], [-dt w^2, 1 - dt^2 w^2 / 4]] / (1 + dt^2 w^2 / 4).
//  * Bead-space free step of the deviations from the centroid (fast path):
//    M = sum_{k >= 1} u_k cay_k u_k^T, i.e. the normal-mode step with the
//    centroid mode projected out, as one 2n x 2n matrix.  Functions of the
//    cyclic ring's Laplacian are circulant (the degenerate cos/sin pairs share
//    one frequency), so M[j][m] = c[(j - m) mod n] and four coefficient
//    vectors (x<-x, x<-v, v<-x, v<-v) describe it.
#pragma once
#include <math.h>
#include <vector>

namespace nqcd {

// U column-major: U[j + n*k]
inline void nm_transform_matrix(int n, double* U) {
    const double pi = 3.14159265358979323846;
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) {
            double val;
            if (k == 0)
                val = 1.0 / sqrt((double)n);
            else if (2 * k < n)
                val = sqrt(2.0 / n) * cos(2.0 * pi * j * k / n);
            else if (2 * k == n)
                val = ((j % 2) ? -1.0 : 1.0) / sqrt((double)n);
            else
                val = sqrt(2.0 / n) * sin(2.0 * pi * j * k / n);
            U[j + n * k] = val;
        }
}

// prop[4*k + (0..3)] = (c11, c12, c21, c22) for mode k
inline void cayley_matrices(int n, double beta, double dt, double* prop) {
    const double pi = 3.14159265358979323846;
    const double wn = (double)n / beta;
    for (int k = 0; k < n; ++k) {
        double w = 2.0 * wn * sin(k * pi / n);
        double x = dt * dt * w * w / 4.0;
        double det = 1.0 + x;
        prop[4 * k + 0] = (1.0 - x) / det;
        prop[4 * k + 1] = dt / det;
        prop[4 * k + 2] = -dt * w * w / det;
        prop[4 * k + 3] = (1.0 - x) / det;
    }
}

// out[4*d + (0..3)] = (cxx, cxv, cvx, cvv)[d] for d = 0..n-1, in FP32 from an
// FP64 evaluation.  Returns false if M is not circulant to 1e-12 (which the
// normal-mode basis above rules out; the check guards the derivation).
inline bool circulant_free_step(int n, double beta, double dt, float* out) {
    std::vector<double> U((size_t)n * n), cay(4 * (size_t)n), M(4 * (size_t)n * n, 0.0);
    nm_transform_matrix(n, U.data());
    cayley_matrices(n, beta, dt, cay.data());
    for (int j = 0; j < n; ++j)
        for (int m = 0; m < n; ++m)
            for (int k = 1; k < n; ++k) {
                const double uu = U[j + n * k] * U[m + n * k];
                for (int q = 0; q < 4; ++q) M[((size_t)q * n + j) * n + m] += uu * cay[4 * k + q];
            }
    for (int q = 0; q < 4; ++q)
        for (int j = 0; j < n; ++j)
            for (int m = 0; m < n; ++m) {
                const double a = M[((size_t)q * n + j) * n + m], b = M[((size_t)q * n + (j - m + n) % n) * n];
                if (fabs(a - b) > 1e-12 * (1.0 + fabs(b))) return false;
            }
    for (int d = 0; d < n; ++d)
        for (int q = 0; q < 4; ++q) out[4 * d + q] = (float)M[((size_t)q * n + d) * n];
    return true;
}

}  // namespace nqcd
