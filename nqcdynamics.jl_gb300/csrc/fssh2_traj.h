// Per-trajectory fewest-switches surface hopping for two-state models
// (Tully 1-3, spin-boson), written as host+device code.  The CUDA kernels in
// fssh2_kernels.cuh run one trajectory per thread through these functions;
// the same functions compile on the host for the bit-exactness self-check.
//
// Reference algorithm (NQCDynamics.jl):
//   BABwithTsit5.perform_step!      src/DynamicsMethods/IntegrationAlgorithms/bab_electronics.jl:61-91
//   step_B!/step_A!                 src/DynamicsMethods/IntegrationAlgorithms/steps.jl:3-8
//   DoubleBuffer/update_parameters! src/DynamicsMethods/electronic_dynamics.jl:15-53
//   DensityMatrixODEProblem f!      src/DynamicsMethods/electronic_dynamics.jl:104-130
//   commutator!                     src/DynamicsUtils/density_matrix_dynamics.jl:29-33
//   FSSH acceleration!              src/DynamicsMethods/SurfaceHoppingMethods/fssh.jl:67-74
//   fewest_switches_probability!    src/DynamicsMethods/SurfaceHoppingMethods/fssh.jl:86-108
//   select_new_state                src/DynamicsMethods/SurfaceHoppingMethods/fssh.jl:110-121
//   rescale_velocity!               src/DynamicsMethods/SurfaceHoppingMethods/surface_hopping.jl:64-168
//
// Two precisions share the code:
//   * double (plain path): every operation in the oracle's order; translation
//     units are built with -fmad=false, so results match the oracle bit for
//     bit (hop sequences identical).
//   * float (fast path): Hamiltonian, eigen, couplings and the Tsit5
//     density-matrix propagation in FP32 with energies shifted by the
//     eigenvalue mean; positions and velocities accumulate in FP64; a macro
//     step whose adiabatic gap is below gap_fp64 is propagated in FP64.
//
// The density matrix is Hermitian and stays so exactly under these updates,
// so only (p, q, x, y) = (sigma00, sigma11, Re sigma01, Im sigma01) are
// carried.  The reduced commutator below is the oracle's full complex
// product with its exactly-zero terms removed (derivation in comments).
#pragma once

#include "nqcd_math.h"
#include "nqcd_models.h"

namespace nqcd {

enum Rescaling : int32_t { RESCALE_STANDARD = 0, RESCALE_VINVERSION = 1, RESCALE_OFF = 2 };
enum InitKind : int32_t { INIT_GIVEN = 0, INIT_ADIABATIC_PURE = 1, INIT_DIABATIC_PURE = 2 };

template <typename R>
struct Sig2 {
    R p, q, x, y;
};

// DoubleBuffer of the electronic parameters: eigenvalues, dynamical
// coupling D01 = sum_I d_I,01 v_I and time, at the start (c) and end (n) of
// the current nuclear step.  Both start zeroed at t = 0, as the reference's
// DensityMatrixODEProblem does.
template <typename R>
struct EBuf {
    R E0c, E1c, Dc;
    double tc;
    R E0n, E1n, Dn;
    double tn;
};

// -d sigma/dt = i [A, sigma],  A = diag(E(t)) - i D(t) sigma_y-like coupling.
// Oracle order (complex 2x2 products, then times -i):
//   C00.im = (-(D x)) - (x D)              -> dp = -m - m,  m = D*x
//   C11.im = (D x) - (-(x D))              -> dq =  m + m
//   C01    = (E0 x - x E1, (E0 y - D q) - (y E1 - p D))
//   du01   = (C01.im, -C01.re)
template <typename R>
NQCD_HD Sig2<R> rhs2(R E0, R E1, R D, const Sig2<R>& u) {
    Sig2<R> d;
    R m = D * u.x;
    d.p = -m - m;
    d.q = m + m;
    d.x = (E0 * u.y - D * u.q) - (u.y * E1 - u.p * D);
    d.y = -(E0 * u.x - u.x * E1);
    return d;
}

// Plain path: interpolation exactly as interpolate_eigenvalues! /
// interpolate_dynamical_coupling! (electronic_dynamics.jl:55-79).
struct Interp64 {
    double E0c, E1c, Dc, dE0, dE1, dD, tc, den;
    NQCD_HD Interp64(const EBuf<double>& b)
        : E0c(b.E0c), E1c(b.E1c), Dc(b.Dc), dE0(b.E0n - b.E0c), dE1(b.E1n - b.E1c), dD(b.Dn - b.Dc),
          tc(b.tc), den(b.tn - b.tc) {}
    NQCD_HD Sig2<double> f(double t, const Sig2<double>& u) const {
        double s = (t - tc) / den;
        if (s != s) s = 0.0;
        double D = Dc + dD * s;
        double E0 = E0c + dE0 * s;
        double E1 = E1c + dE1 * s;
        return rhs2<double>(E0, E1, D, u);
    }
};

// Fast path: FP32 interpolation from a precomputed reciprocal.
struct Interp32 {
    float E0c, E1c, Dc, dE0, dE1, dD;
    double tc, inv;
    NQCD_HD Interp32(const EBuf<float>& b)
        : E0c(b.E0c), E1c(b.E1c), Dc(b.Dc), dE0(b.E0n - b.E0c), dE1(b.E1n - b.E1c), dD(b.Dn - b.Dc),
          tc(b.tc), inv(b.tn != b.tc ? 1.0 / (b.tn - b.tc) : 0.0) {}
    NQCD_HD Sig2<float> f(double t, const Sig2<float>& u) const {
        float s = (float)((t - tc) * inv);
        float D = Dc + dD * s;
        float E0 = E0c + dE0 * s;
        float E1 = E1c + dE1 * s;
        return rhs2<float>(E0, E1, D, u);
    }
};

#define NQCD_TS_COMB(dst, EXPR)                        \
    {                                                  \
        dst.p = u.p + h * (EXPR(p));                   \
        dst.q = u.q + h * (EXPR(q));                   \
        dst.x = u.x + h * (EXPR(x));                   \
        dst.y = u.y + h * (EXPR(y));                   \
    }

// One fixed Tsit5 step (first-same-as-last: k1 in, k7 out through k1).
template <typename R, typename F>
NQCD_HD void tsit5_step2(const F& fn, double t, double hd, Sig2<R>& u, Sig2<R>& k1) {
    typedef Tsit5 TS;
    const R h = (R)hd;
    Sig2<R> tmp, k2, k3, k4, k5, k6;
#define E2(c) ((R)TS::a21 * k1.c)
    NQCD_TS_COMB(tmp, E2);
#undef E2
    k2 = fn.f(t + TS::c2 * hd, tmp);
#define E3(c) ((R)TS::a31 * k1.c + (R)TS::a32 * k2.c)
    NQCD_TS_COMB(tmp, E3);
#undef E3
    k3 = fn.f(t + TS::c3 * hd, tmp);
#define E4(c) ((R)TS::a41 * k1.c + (R)TS::a42 * k2.c + (R)TS::a43 * k3.c)
    NQCD_TS_COMB(tmp, E4);
#undef E4
    k4 = fn.f(t + TS::c4 * hd, tmp);
#define E5(c) ((R)TS::a51 * k1.c + (R)TS::a52 * k2.c + (R)TS::a53 * k3.c + (R)TS::a54 * k4.c)
    NQCD_TS_COMB(tmp, E5);
#undef E5
    k5 = fn.f(t + TS::c5 * hd, tmp);
#define E6(c) ((R)TS::a61 * k1.c + (R)TS::a62 * k2.c + (R)TS::a63 * k3.c + (R)TS::a64 * k4.c + (R)TS::a65 * k5.c)
    NQCD_TS_COMB(tmp, E6);
#undef E6
    k6 = fn.f(t + hd, tmp);
#define E7(c)                                                                                            \
    ((R)TS::a71 * k1.c + (R)TS::a72 * k2.c + (R)TS::a73 * k3.c + (R)TS::a74 * k4.c + (R)TS::a75 * k5.c + \
     (R)TS::a76 * k6.c)
    NQCD_TS_COMB(tmp, E7);
#undef E7
    k1 = fn.f(t + hd, tmp);
    u = tmp;
}
#undef NQCD_TS_COMB

// SciMLBase.step!(electronic_integrator, dt, true) at fixed sub-step dt/5
// (bab_electronics.jl:40-43, 87-90).
template <typename R, typename F>
NQCD_HD void electronic_macro_step2(const F& fn, double t, double h, double dtsub, Sig2<R>& u) {
    double tend = t + h;
    Sig2<R> k1 = fn.f(t, u);
    double tc = t;
    for (int guard = 0; tc < tend && guard < 64; ++guard) {
        double hs = (tend - tc) < dtsub ? (tend - tc) : dtsub;
        tsit5_step2<R>(fn, tc, hs, u, k1);
        tc = snap_time(tc + hs, tend);
    }
}

// Fast path, FP32 only.  rhs2 changes p and q by opposite amounts
// (dq/dt = -dp/dt = 2 D x exactly, a negation), so a Tsit5 stage needs three
// derivative components, (dp, dx, dy), and the q update subtracts the p
// stage sum: the same values as integrating q on its own (negation is exact),
// with a quarter fewer stage sums.  With G = E0 - E1 the derivative is
//   dp/dt = -2 D x,   dx/dt = G y + D (p - q),   dy/dt = -G x.
//
// The macro step [t, t + h] lies inside the DoubleBuffer interval [tc, tn]
// (equal to it except in the first step of a run that does not start at
// t = 0), so a stage at position sigma in [0, 1] of the macro step reads the
// buffer at s = sa + sb * sigma, with sa = (t - tc) / (tn - tc) and
// sb = h / (tn - tc) formed on the host.  G and D are linear in s: a sub-step
// starting at sigma0 forms G = Gb + c Gs for its stage at c once (Gb, Gs) are
// known, one FMA per stage and quantity, and no FP64.
struct Deriv3 {
    float p, x, y;  // dq = -p
};

NQCD_HD Deriv3 rhs_fast(float G, float D, const Sig2<float>& u) {
    const float m = D * u.x;
    return {-m - m, fmaf(G, u.y, D * (u.p - u.q)), -(G * u.x)};
}

// One Tsit5 sub-step of length hs (time) whose stage at c reads
// G = Gb + c Gs, D = Db + c Ds (FSAL: k1 in, the end point's derivative out).
NQCD_HD void tsit5_step_fast(float Gb, float Gs, float Db, float Ds, float hs, Sig2<float>& u, Deriv3& k1) {
    typedef Tsit5 TS;
    Sig2<float> t;
    Deriv3 k2, k3, k4, k5, k6;
#define NQCD_TS_COMB_F(EXPR)              \
    {                                     \
        const float sp = (EXPR(p));       \
        t.p = fmaf(hs, sp, u.p);          \
        t.q = fmaf(hs, -sp, u.q);         \
        t.x = fmaf(hs, (EXPR(x)), u.x);   \
        t.y = fmaf(hs, (EXPR(y)), u.y);   \
    }
#define NQCD_TS_STAGE(c) rhs_fast(fmaf((float)(c), Gs, Gb), fmaf((float)(c), Ds, Db), t)
#define E2(c) ((float)TS::a21 * k1.c)
    NQCD_TS_COMB_F(E2);
#undef E2
    k2 = NQCD_TS_STAGE(TS::c2);
#define E3(c) ((float)TS::a31 * k1.c + (float)TS::a32 * k2.c)
    NQCD_TS_COMB_F(E3);
#undef E3
    k3 = NQCD_TS_STAGE(TS::c3);
#define E4(c) ((float)TS::a41 * k1.c + (float)TS::a42 * k2.c + (float)TS::a43 * k3.c)
    NQCD_TS_COMB_F(E4);
#undef E4
    k4 = NQCD_TS_STAGE(TS::c4);
#define E5(c) ((float)TS::a51 * k1.c + (float)TS::a52 * k2.c + (float)TS::a53 * k3.c + (float)TS::a54 * k4.c)
    NQCD_TS_COMB_F(E5);
#undef E5
    k5 = NQCD_TS_STAGE(TS::c5);
#define E6(c)                                                                                                  \
    ((float)TS::a61 * k1.c + (float)TS::a62 * k2.c + (float)TS::a63 * k3.c + (float)TS::a64 * k4.c + \
     (float)TS::a65 * k5.c)
    NQCD_TS_COMB_F(E6);
#undef E6
    k6 = rhs_fast(Gb + Gs, Db + Ds, t);
#define E7(c)                                                                                                  \
    ((float)TS::a71 * k1.c + (float)TS::a72 * k2.c + (float)TS::a73 * k3.c + (float)TS::a74 * k4.c + \
     (float)TS::a75 * k5.c + (float)TS::a76 * k6.c)
    NQCD_TS_COMB_F(E7);
#undef E7
#undef NQCD_TS_STAGE
#undef NQCD_TS_COMB_F
    k1 = rhs_fast(Gb + Gs, Db + Ds, t);
    u = t;
}

// Fast-path macro step: sub-steps of dtsub (the last one shortened), in FP32,
// on the buffer weights (sa, sb) of this step.
NQCD_HD void electronic_macro_step2_fast(const EBuf<float>& b, float sa, float sb, float h, float dtsub,
                                         Sig2<float>& u) {
    const float Gc = b.E0c - b.E1c, dG = (b.E0n - b.E1n) - Gc;
    const float Dc = b.Dc, dD = b.Dn - b.Dc;
#ifdef __CUDA_ARCH__
    // the sub-step count does not hang on the last bits of fs (the snap below)
    const float fs = __fdividef(dtsub, h);
#else
    const float fs = dtsub / h;
#endif
    Deriv3 k1 = rhs_fast(fmaf(dG, sa, Gc), fmaf(dD, sa, Dc), u);
    float s0 = 0.f;
    for (int guard = 0; s0 < 1.f && guard < 64; ++guard) {
        const float hr = (1.f - s0) < fs ? (1.f - s0) : fs;
        const float base = fmaf(sb, s0, sa), scale = sb * hr;
        tsit5_step_fast(fmaf(dG, base, Gc), dG * scale, fmaf(dD, base, Dc), dD * scale, hr * h, u, k1);
        s0 = s0 + hr;
        if (1.f - s0 < 1e-6f) s0 = 1.f;
    }
}

// 24-bit uniform in [0, 1) from the same Philox block as rng_uniform (the
// fast path compares in FP32; it differs from the 53-bit draw only below 2^-24).
NQCD_HD float rng_uniform_f(uint64_t seed, uint64_t traj, uint32_t step, uint32_t stream) {
    u32x4 b = rng_block(seed, traj, step, stream);
#ifdef __CUDA_ARCH__
    // (float)(b.x >> 8) without a conversion instruction (conversions issue on this GPU's FP64
    // unit): the top 23 bits through the exponent bias 2^23, exact, doubled, plus the last bit
    const uint32_t x = b.x >> 8;
    const float hi = __uint_as_float(0x4B000000u | (x >> 1)) - 8388608.0f;
    return fmaf(2.0f, hi, (x & 1u) ? 1.0f : 0.0f) * 0x1.0p-24f;
#else
    return (float)(b.x >> 8) * 0x1.0p-24f;
#endif
}

// clamp(x, 0, 1) with the reference's NaN propagation.
template <typename R>
NQCD_HD R clamp01(R x) {
    return x > R(1) ? R(1) : (x < R(0) ? R(0) : x);
}

}  // namespace nqcd
