// Numeric primitives shared by the CUDA kernels and the CPU oracle.
//
// Everything here must produce bit-identical results on the host (gcc,
// -ffp-contract=off) and on the device (nvcc, FP64 translation units built
// with -fmad=false), because the plain FP64 engine path is required to
// reproduce the oracle's hop sequences exactly.  Only IEEE-754 basic
// operations (+ - * / sqrt), floor and ldexp are used; all of them are
// correctly rounded on both sides.
//
//  * Philox4x32-10 counter RNG (Salmon, Moraes, Dror, Shaw, "Parallel random
//    numbers: as easy as 1, 2, 3", SC'11).  Keyed by the run seed, counter =
//    (trajectory, step, stream, 0), so every random draw is addressable and a
//    trajectory's stream does not depend on how trajectories are mapped to
//    threads, warps or devices.
//  * nqcd_exp: Cody-Waite range reduction x = k ln2 + r, |r| <= ln2/2, then
//    the degree-13 Taylor polynomial of e^r in Horner form, then 2^k scaling
//    with ldexp.  The ln2 split (32 significant bits in the high part) and the
//    Taylor coefficients 1/n! were derived for this project with exact
//    rational arithmetic.  Tested against the C library to <= 2 ulp.
//  * Tsit5 tableau (Ch. Tsitouras, "Runge-Kutta pairs of order 5(4)
//    satisfying only the first column simplifying assumption", Comput. Math.
//    Appl. 62 (2011) 770-775), the electronic sub-integrator the reference
//    runs at dt/5 (src/DynamicsMethods/IntegrationAlgorithms/bab_electronics.jl:40-43).
#pragma once

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define NQCD_HD __host__ __device__ __forceinline__
#else
#define NQCD_HD inline
#endif

namespace nqcd {

// ---------------------------------------------------------------------------
// Philox4x32-10
// ---------------------------------------------------------------------------
struct u32x4 { uint32_t x, y, z, w; };

NQCD_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

NQCD_HD u32x4 philox4x32_10(u32x4 ctr, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int round = 0; round < 10; ++round) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(M0, ctr.x, hi0, lo0);
        mulhilo32(M1, ctr.z, hi1, lo1);
        u32x4 n;
        n.x = hi1 ^ ctr.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ ctr.w ^ k1;
        n.w = lo0;
        ctr = n;
        k0 += W0;
        k1 += W1;
    }
    return ctr;
}

// Random-number streams of one trajectory step.  Each stream is one Philox
// block, so one draw per (trajectory, step, stream) costs one block.
enum RngStream : uint32_t {
    RNG_HOP = 1,        // uniform for the hop test (fssh.jl:112, iesh.jl:393)
    RNG_INIT_STATE = 2, // uniform for sampling the initial adiabatic state (fssh.jl:54)
    RNG_NOISE = 3,      // Gaussian Wiener increments for MDEF (mdef_baoab.jl:164)
    RNG_INIT_FD = 4,    // Fermi-Dirac occupation sampling (DynamicsUtils.jl:194-208)
    RNG_INIT_POSITION = 5, // device-side initial positions (selections.jl:24-101); counter z = degree of freedom
    RNG_INIT_VELOCITY = 6, // device-side initial velocities
};

// 53-bit uniform in [0, 1) from the two high words of one Philox block.
NQCD_HD double u01_from_words(uint32_t hi, uint32_t lo) {
    uint64_t bits = ((uint64_t)hi << 32) | (uint64_t)lo;
    return (double)(bits >> 11) * 0x1.0p-53;
}

NQCD_HD u32x4 rng_block(uint64_t seed, uint64_t traj, uint32_t step, uint32_t stream) {
    u32x4 c;
    c.x = (uint32_t)traj;
    c.y = (uint32_t)(traj >> 32);
    c.z = step;
    c.w = stream;
    return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

NQCD_HD double rng_uniform(uint64_t seed, uint64_t traj, uint32_t step, uint32_t stream) {
    u32x4 b = rng_block(seed, traj, step, stream);
    return u01_from_words(b.x, b.y);
}

// ---------------------------------------------------------------------------
// exp (own implementation, see header comment)
// ---------------------------------------------------------------------------
NQCD_HD double nqcd_exp(double x) {
    const double INV_LN2 = 0x1.71547652b82fep+0;
    const double LN2_HI = 0x1.62e42ff000000p-1;   // 32 significant bits
    const double LN2_LO = -0x1.718432a1b0e26p-35; // ln2 - LN2_HI
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
    double kd = floor(x * INV_LN2 + 0.5);
    double r = (x - kd * LN2_HI) - kd * LN2_LO;
    // Taylor coefficients 1/n!, n = 13 ... 2
    double p = 0x1.6124613a86d09p-33;
    p = p * r + 0x1.1eed8eff8d898p-29;
    p = p * r + 0x1.ae64567f544e4p-26;
    p = p * r + 0x1.27e4fb7789f5cp-22;
    p = p * r + 0x1.71de3a556c734p-19;
    p = p * r + 0x1.a01a01a01a01ap-16;
    p = p * r + 0x1.a01a01a01a01ap-13;
    p = p * r + 0x1.6c16c16c16c17p-10;
    p = p * r + 0x1.1111111111111p-7;
    p = p * r + 0x1.5555555555555p-5;
    p = p * r + 0x1.5555555555555p-3;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    return ldexp(p, (int)kd);
}

// ---------------------------------------------------------------------------
// Tsit5 tableau (Tsitouras 2011).  Stage abscissae c2..c7 and the rows of A;
// the solution weights equal row 7 (first-same-as-last).
// ---------------------------------------------------------------------------
struct Tsit5 {
    static constexpr double c2 = 0.161;
    static constexpr double c3 = 0.327;
    static constexpr double c4 = 0.9;
    static constexpr double c5 = 0.9800255409045097;
    static constexpr double a21 = 0.161;
    static constexpr double a31 = -0.008480655492356989;
    static constexpr double a32 = 0.335480655492357;
    static constexpr double a41 = 2.897153057105493;
    static constexpr double a42 = -6.359448489975075;
    static constexpr double a43 = 4.3622954328695815;
    static constexpr double a51 = 5.325864828439257;
    static constexpr double a52 = -11.748883564062828;
    static constexpr double a53 = 7.4955393428898365;
    static constexpr double a54 = -0.09249506636175525;
    static constexpr double a61 = 5.86145544294642;
    static constexpr double a62 = -12.92096931784711;
    static constexpr double a63 = 8.159367898576159;
    static constexpr double a64 = -0.071584973281401;
    static constexpr double a65 = -0.028269050394068383;
    static constexpr double a71 = 0.09646076681806523;
    static constexpr double a72 = 0.01;
    static constexpr double a73 = 0.4798896504144996;
    static constexpr double a74 = 1.379008574103742;
    static constexpr double a75 = -3.290069515436081;
    static constexpr double a76 = 2.324710524099774;
};

// ---------------------------------------------------------------------------
// Real part of the complex quotient (a + ib) / (c + id), rounded as Julia's
// `/` for Complex{Float64} rounds it.  That operator is the robust complex
// division of Baudin and Smith ("A Robust Complex Division in Scilab",
// arXiv:1210.4539, 2012), restated here from the paper:
//   1. scale (a, b) and (c, d) by powers of two when the larger magnitude of
//      a pair is at or above half the largest double, or at or below
//      2 * (smallest normal) / eps; the scale factor s undoes it at the end;
//   2. pivot on the larger of |c|, |d|: r = d/c, t = 1/(c + d r) when
//      |d| <= |c|, else the roles of (a, b) and (c, d) are swapped;
//   3. the real part is (a + b r) t, with b r split as a t + (b t) r when it
//      underflows to zero, and (a + d (b/c)) t when r itself is zero.
// The reference's fewest-switches probability uses it as
// real(sigma[m, s] / sigma[s, s]) (fssh.jl:96-108).  With d = 0 (the
// diagonal of a two-state density matrix, whose imaginary part stays exactly
// zero) it reduces to a * (1/c) for normal operands.
// ---------------------------------------------------------------------------
NQCD_HD double cdiv_real_part(double A, double B, double C, double D, double r, double t) {
    if (r != 0.0) {
        double br = B * r;
        return br != 0.0 ? (A + br) * t : A * t + (B * t) * r;
    }
    return (A + D * (B / C)) * t;
}

NQCD_HD double cdiv_real(double a, double b, double c, double d) {
    const double halfov = 0x1.fffffffffffffp+1022;  // largest double / 2
    const double twoun = 0x1p-969;                  // 2 * smallest normal / eps
    const double bs = 0x1p+105;                     // 2 / eps^2
    double absa = fabs(a), absb = fabs(b), absc = fabs(c), absd = fabs(d);
    double ab = absa >= absb ? absa : absb;
    double cd = absc >= absd ? absc : absd;
    double s = 1.0;
    if (ab >= halfov || ab <= twoun || cd >= halfov || cd <= twoun) {
        if (ab >= halfov) { a = 0.5 * a; b = 0.5 * b; s = 2.0; }
        if (cd >= halfov) { c = 0.5 * c; d = 0.5 * d; s = s * 0.5; }
        if (ab <= twoun) { a = a * bs; b = b * bs; s = s / bs; }
        if (cd <= twoun) { c = c * bs; d = d * bs; s = s * bs; }
    }
    double re;
    if (fabs(d) <= fabs(c)) {
        double r = d / c;
        double t = 1.0 / (c + d * r);
        re = cdiv_real_part(a, b, c, d, r, t);
    } else {
        double r = c / d;
        double t = 1.0 / (d + c * r);
        re = cdiv_real_part(b, a, d, c, r, t);
    }
    return re * s;
}

// Time snapping used by the reference's ODE integrator after each step:
// a time within 100 eps of the stop time is set to the stop time.
NQCD_HD double snap_time(double t, double tstop) {
    double m = fabs(t) > fabs(tstop) ? fabs(t) : fabs(tstop);
    // eps(m) for normal m: 2^(exponent(m) - 52)
    int e;
    frexp(m, &e);
    double eps = ldexp(1.0, e - 53);
    if (m == 0.0) eps = 4.9406564584124654e-324;
    return fabs(t - tstop) < 100.0 * eps ? tstop : t;
}

}  // namespace nqcd
