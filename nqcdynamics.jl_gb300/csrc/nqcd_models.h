// Model Hamiltonians of the ensemble hot path, restated from their published
// definitions (the reference takes them from the un-vendored NQCModels
// package; call sites: src/DynamicsMethods/SurfaceHoppingMethods/fssh.jl:67-74,
// src/DynamicsMethods/ClassicalMethods/mdef.jl:110, iesh.jl:192).
//
//  * Tully's models 1-3: J. C. Tully, J. Chem. Phys. 93, 1061 (1990).
//  * Spin-boson with an Ohmic bath discretised as in the reference's model
//    documentation (docs/src/NQCModels/systembathmodels.md:20-26,54-59):
//      V = [[eps + c.R, Delta], [Delta, -eps - c.R]] + 1/2 R^T Omega^2 R.
//
// These functions are shared by the CUDA kernels and by the CPU oracle so
// that the plain FP64 path and the oracle evaluate identical operation
// sequences.  Their correctness is checked separately (finite differences,
// closed-form values) in the test suite.
#pragma once

#include <type_traits>

#include "nqcd_math.h"

namespace nqcd {

enum ModelKind : int32_t {
    MODEL_TULLY1 = 1,
    MODEL_TULLY2 = 2,
    MODEL_TULLY3 = 3,
    MODEL_SPINBOSON = 10,
    MODEL_NEWNS_ANDERSON = 20,
};

// Default parameters (Tully 1990, Table I of the paper).
//   Tully 1: A=0.01, B=1.6, C=0.005, D=1.0
//   Tully 2: A=0.1, B=0.28, C=0.015, D=0.06, E0=0.05
//   Tully 3: A=6e-4, B=0.1, C=0.9
// Symmetric 2x2 matrices are stored as (m00, m01, m11).

template <typename T>
NQCD_HD T model_exp(T x);

template <>
NQCD_HD double model_exp<double>(double x) { return nqcd_exp(x); }

template <>
NQCD_HD float model_exp<float>(float x) {
#if defined(__CUDA_ARCH__)
    return __expf(x);
#else
    return expf(x);
#endif
}

template <typename T>
NQCD_HD void tully_potential(int kind, const T* p, T x, T V[3]) {
    if (kind == MODEL_TULLY1) {
        T A = p[0], B = p[1], C = p[2], D = p[3];
        T v11 = x > T(0) ? A * (T(1) - model_exp<T>(-B * x)) : -A * (T(1) - model_exp<T>(B * x));
        V[0] = v11;
        V[1] = C * model_exp<T>(-D * (x * x));
        V[2] = -v11;
    } else if (kind == MODEL_TULLY2) {
        T A = p[0], B = p[1], C = p[2], D = p[3], E0 = p[4];
        V[0] = T(0);
        V[1] = C * model_exp<T>(-D * (x * x));
        V[2] = -A * model_exp<T>(-B * (x * x)) + E0;
    } else {  // MODEL_TULLY3
        T A = p[0], B = p[1], C = p[2];
        V[0] = A;
        V[1] = x < T(0) ? B * model_exp<T>(C * x) : B * (T(2) - model_exp<T>(-C * x));
        V[2] = -A;
    }
}

template <typename T>
NQCD_HD void tully_derivative(int kind, const T* p, T x, T D[3]) {
    if (kind == MODEL_TULLY1) {
        T A = p[0], B = p[1], C = p[2], Dp = p[3];
        T d11 = x > T(0) ? (A * B) * model_exp<T>(-B * x) : (A * B) * model_exp<T>(B * x);
        D[0] = d11;
        D[1] = -T(2) * C * Dp * x * model_exp<T>(-Dp * (x * x));
        D[2] = -d11;
    } else if (kind == MODEL_TULLY2) {
        T A = p[0], B = p[1], C = p[2], Dp = p[3];
        D[0] = T(0);
        D[1] = -T(2) * C * Dp * x * model_exp<T>(-Dp * (x * x));
        D[2] = T(2) * A * B * x * model_exp<T>(-B * (x * x));
    } else {  // MODEL_TULLY3
        T B = p[1], C = p[2];
        D[0] = T(0);
        D[1] = x < T(0) ? (B * C) * model_exp<T>(C * x) : (B * C) * model_exp<T>(-C * x);
        D[2] = T(0);
    }
}

// ---------------------------------------------------------------------------
// Symmetric 2x2 eigen-decomposition (ascending eigenvalues), with the
// eigenvector sign fixed by continuity with the previous step's eigenvectors
// (a column whose overlap with its predecessor is negative is negated; the
// first call of a trajectory compares with the identity).
// Z is column-major: Z[0]=Z00, Z[1]=Z10, Z[2]=Z01, Z[3]=Z11.
// ---------------------------------------------------------------------------
template <typename T>
NQCD_HD void eigen2_phase(const T H[3], const T Zprev[4], T w[2], T Z[4]) {
    T a = H[0], b = H[1], c = H[2];
    T m = T(0.5) * (a + c);
    T h = T(0.5) * (a - c);
    T rad = sqrt(h * h + b * b);
    w[0] = m - rad;
    w[1] = m + rad;
    T v1x, v1y;
    if (rad == T(0)) {
        v1x = T(0);
        v1y = T(1);
    } else {
        if (h >= T(0)) {
            v1x = h + rad;
            v1y = b;
        } else {
            v1x = b;
            v1y = rad - h;
        }
#if defined(__CUDA_ARCH__)
        if constexpr (std::is_same<T, float>::value) {
            // fast paths: normalise with the hardware reciprocal square root
            const float rn = rsqrtf(v1x * v1x + v1y * v1y);
            v1x = v1x * rn;
            v1y = v1y * rn;
        } else
#endif
        {
            T n = sqrt(v1x * v1x + v1y * v1y);
            v1x = v1x / n;
            v1y = v1y / n;
        }
    }
    // column 0 = (-v1y, v1x), column 1 = (v1x, v1y)
    T z00 = -v1y, z10 = v1x, z01 = v1x, z11 = v1y;
    if (z00 * Zprev[0] + z10 * Zprev[1] < T(0)) {
        z00 = -z00;
        z10 = -z10;
    }
    if (z01 * Zprev[2] + z11 * Zprev[3] < T(0)) {
        z01 = -z01;
        z11 = -z11;
    }
    Z[0] = z00;
    Z[1] = z10;
    Z[2] = z01;
    Z[3] = z11;
}

// Z^T dH Z for a symmetric 2x2 dH = (d00, d01, d11).  Evaluated as
// T = dH Z followed by Z^T T, summing over the inner index in ascending
// order; the (0,1) element is computed and mirrored to (1,0).
// Output (A00, A01, A11).
template <typename T>
NQCD_HD void adiabatic_derivative2(const T dH[3], const T Z[4], T A[3]) {
    T d00 = dH[0], d01 = dH[1], d11 = dH[2];
    // T = dH * Z (column-major Z)
    T t00 = d00 * Z[0] + d01 * Z[1];
    T t10 = d01 * Z[0] + d11 * Z[1];
    T t01 = d00 * Z[2] + d01 * Z[3];
    T t11 = d01 * Z[2] + d11 * Z[3];
    A[0] = Z[0] * t00 + Z[1] * t10;
    A[1] = Z[0] * t01 + Z[1] * t11;
    A[2] = Z[2] * t01 + Z[3] * t11;
}

}  // namespace nqcd
