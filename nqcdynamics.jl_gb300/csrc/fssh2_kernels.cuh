// Ensemble kernels for two-state fewest-switches surface hopping.
// One trajectory per thread, the whole time loop inside one launch.
//
//   fssh2_tully_kernel<R>     Tully models 1-3 (1 DoF): r, v, k, sigma and the
//                             electronic cache live in registers.
//   fssh2_spinboson_kernel<R> spin-boson (N bath modes): bath coordinates and
//                             velocities in HBM as [mode][trajectory] (coalesced);
//                             the 2x2 electronic problem in registers.
//
// R = double is the plain path (bit-identical to the oracle; its translation
// unit is compiled with -fmad=false); R = float is the fast path.
// Algorithm and reference citations: fssh2_traj.h.
#pragma once

#include <cuda_runtime.h>
#include <type_traits>

#include "engine_params.h"
#include "fssh2_traj.h"

namespace nqcd {

constexpr int kFsshBlock = 128;

// Per-warp partial sums of the diabatic population correlation at one save
// point (TimeCorrelationFunctions.jl:61-88); reduced over warps afterwards in
// a fixed order, so the ensemble mean is deterministic.
__device__ __forceinline__ void warp_save_popcorr(const FsshParams& p, int isave, bool active, const double pop0[2],
                                                  const double pop[2]) {
    double c[4];
    c[0] = active ? pop0[0] * pop[0] : 0.0;
    c[1] = active ? pop0[0] * pop[1] : 0.0;
    c[2] = active ? pop0[1] * pop[0] : 0.0;
    c[3] = active ? pop0[1] * pop[1] : 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) c[q] += __shfl_xor_sync(0xffffffffu, c[q], off);
    if ((threadIdx.x & 31) == 0 && isave < p.nsave) {
        int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        double* dst = p.popcorr_partial + (warp * p.nsave + isave) * 4;
#pragma unroll
        for (int q = 0; q < 4; ++q) dst[q] = c[q];
    }
}

// diag(U sigma' U^T), sigma' = Re(sigma) with diagonal replaced by the
// occupied state (fssh.jl:132-142).
// Ehrenfest (ehrenfest.jl:75-83): the density matrix itself on the diagonal.
template <typename R>
__device__ __forceinline__ void diabatic_pop2(const Sig2<R>& sg, int s, const R Z[4], double pop[2],
                                              bool ehrenfest = false) {
    double sp00 = ehrenfest ? (double)sg.p : (s == 0 ? 1.0 : 0.0);
    double sp11 = ehrenfest ? (double)sg.q : (s == 1 ? 1.0 : 0.0);
    double sp01 = (double)sg.x;
    double U00 = Z[0], U10 = Z[1], U01 = Z[2], U11 = Z[3];
    double M00 = U00 * sp00 + U01 * sp01;
    double M01 = U00 * sp01 + U01 * sp11;
    double M10 = U10 * sp00 + U11 * sp01;
    double M11 = U10 * sp01 + U11 * sp11;
    pop[0] = M00 * U00 + M01 * U01;
    pop[1] = M10 * U10 + M11 * U11;
}

// Ehrenfest force weight (ehrenfest.jl:50-68): sum_m sum_n A_nm Re sigma_nm
// for a symmetric 2x2 A = (A00, A01, A11), in the reference's loop order
// (m outer, n inner); Re sigma_10 = Re sigma_01 = x.
template <typename R>
__device__ __forceinline__ R ehrenfest_weight(R A00, R A01, R A11, const Sig2<R>& sg) {
    return ((A00 * sg.p + A01 * sg.x) + A01 * sg.x) + A11 * sg.q;
}

// Ehrenfest potential energy (ehrenfest.jl:85-95): sum_i Re sigma_ii E_i.
template <typename R>
__device__ __forceinline__ double ehrenfest_potential(const Sig2<R>& sg, const R w[2]) {
    return (double)sg.p * (double)w[0] + (double)sg.q * (double)w[1];
}

// Initial electronic variables: adiabatic pure state, or a diabatic pure
// state rotated to the adiabatic basis with the occupied state sampled from
// its populations (fssh.jl:47-65; density_matrix_dynamics.jl:37-75).
template <typename R>
__device__ __forceinline__ void init_electronics2(const FsshParams& p, int64_t i, int64_t gid, const R Z[4],
                                                  Sig2<R>& sg, int& state) {
    if (p.init_kind == INIT_GIVEN) {
        sg.p = (R)p.sigma[0 * p.ntraj + i];
        sg.x = (R)p.sigma[2 * p.ntraj + i];
        sg.y = (R)p.sigma[3 * p.ntraj + i];
        sg.q = (R)p.sigma[6 * p.ntraj + i];
        state = p.state[i];
        return;
    }
    if (p.init_kind == INIT_ADIABATIC_PURE) {
        sg.p = p.init_state == 0 ? R(1) : R(0);
        sg.q = p.init_state == 1 ? R(1) : R(0);
        sg.x = R(0);
        sg.y = R(0);
        state = p.init_state;
        return;
    }
    // sigma = U^T rho U with rho = e_k e_k^T: sigma_ij = U_ki U_kj (evaluated as the oracle's products)
    double U[2][2] = {{(double)Z[0], (double)Z[2]}, {(double)Z[1], (double)Z[3]}};
    double rho[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    rho[p.init_state][p.init_state] = 1.0;
    double T[2][2], S[2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) T[a][b] = U[0][a] * rho[0][b] + U[1][a] * rho[1][b];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) S[a][b] = T[a][0] * U[0][b] + T[a][1] * U[1][b];
    sg.p = (R)S[0][0];
    sg.q = (R)S[1][1];
    sg.x = (R)S[0][1];
    sg.y = R(0);
    double wsum = S[0][0] + S[1][1];
    double tt = rng_uniform(p.seed, (uint64_t)gid, 0u, RNG_INIT_STATE) * wsum;
    state = (S[0][0] < tt) ? 1 : 0;
}

// One electronic macro step of the plain path (FP64, the reference's
// fixed sub-steps of dt/5 on the FP64 clock).
__device__ __forceinline__ void electronics2(const FsshParams& p, const EBuf<double>& buf, double t, double h,
                                             Sig2<double>& sg) {
    const double dtsub = p.dt / 5.0;
    Interp64 fn(buf);
    electronic_macro_step2<double>(fn, t, h, dtsub, sg);
}

// Fast-path electronic step on the host-computed schedule: interpolation
// weights (sa, sb) = (sa1, sb1) on the first step (the buffer starts at
// t = 0) and (0, 1) afterwards, which is what the FP64 clock gives; below the
// gap threshold the FP64 sub-integrator runs on the same relative times.
// The FP64 sub-integration of a near-degenerate step.  Not inlined, so that
// none of its conversions to and from FP64 is scheduled into the FP32 path of
// the steps that do not take it (the FP64 pipe of this GPU runs at 1/64 of
// the FP32 rate).
// (Arguments and result by value: an address passed to a call that is not inlined would keep the
// caller's density matrix in local memory for the whole step loop.)
static __device__ __noinline__ Sig2<float> electronics2_fp64_step(const EBuf<float> buf, bool first, float h, double t0,
                                                                 double dt, const Sig2<float> sg) {
    const double hd = h;
    const double tn = first ? t0 + hd : hd, t = first ? t0 : 0.0;
    EBuf<double> b64 = {buf.E0c, buf.E1c, buf.Dc, 0.0, buf.E0n, buf.E1n, buf.Dn, tn};
    Sig2<double> s64 = {sg.p, sg.q, sg.x, sg.y};
    Interp64 fn(b64);
    electronic_macro_step2<double>(fn, t, hd, dt / 5.0, s64);
    return {(float)s64.p, (float)s64.q, (float)s64.x, (float)s64.y};
}

template <typename P>  // FsshParams or RpshParams
__device__ __forceinline__ void electronics2_sched(const P& p, const EBuf<float>& buf, bool first, float h, float gap,
                                                   Sig2<float>& sg, int& nfp64) {
    const float dtsub = p.dtsub;
    if (gap < p.gap_fp64) {
        ++nfp64;  // steps integrated with the FP64 electronics (per-trajectory status)
        sg = electronics2_fp64_step(buf, first, h, p.t0, p.dt, sg);
    } else {
        electronic_macro_step2_fast(buf, first ? p.sa1 : 0.f, first ? p.sb1 : 1.f, h, dtsub, sg);
    }
}

// Position / velocity accumulators of the fast paths:
//   AccF64   FP64 accumulator (one FP64 add per update),
//   AccKahan FP32 value + FP32 compensation (Kahan summation, four FP32 ops
//            per update), used where the FP64 pipe (1/73 of the FP32 rate on
//            this GPU, measured) would bound the step.
struct AccF64 {
    double x;
    __device__ __forceinline__ void load(double d) { x = d; }
    __device__ __forceinline__ double get() const { return x; }
    __device__ __forceinline__ float f() const { return (float)x; }
    __device__ __forceinline__ void add(float inc) { x += (double)inc; }
    __device__ __forceinline__ void add_prod(float a, float b) { add(a * b); }
};

struct AccKahan {
    float s, c;  // value ~ s - c
    __device__ __forceinline__ void load(double d) {
        s = (float)d;
        c = -(float)(d - (double)s);
    }
    __device__ __forceinline__ double get() const { return (double)s - (double)c; }
    __device__ __forceinline__ float f() const { return s; }
    __device__ __forceinline__ void add(float inc) {
        float y = __fsub_rn(inc, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    // add(a * b) with the product and the compensation in one rounding (one FMA fewer)
    __device__ __forceinline__ void add_prod(float a, float b) {
        float y = __fmaf_rn(a, b, -c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
};

// FP32 form of diabatic_pop2 and of the warp sum of the population products
// (fast paths): no FP64 arithmetic in the step loop.
__device__ __forceinline__ void diabatic_pop2_f(const Sig2<float>& sg, int s, const float Z[4], float pop[2],
                                                bool ehrenfest = false) {
    const float sp00 = ehrenfest ? sg.p : (s == 0 ? 1.f : 0.f), sp11 = ehrenfest ? sg.q : (s == 1 ? 1.f : 0.f);
    const float sp01 = sg.x;
    const float M00 = Z[0] * sp00 + Z[2] * sp01, M01 = Z[0] * sp01 + Z[2] * sp11;
    const float M10 = Z[1] * sp00 + Z[3] * sp01, M11 = Z[1] * sp01 + Z[3] * sp11;
    pop[0] = M00 * Z[0] + M01 * Z[2];
    pop[1] = M10 * Z[1] + M11 * Z[3];
}

__device__ __forceinline__ void warp_save_popcorr_f(const FsshParams& p, int isave, bool active, const float pop0[2],
                                                    const float pop[2]) {
    float c[4];
    c[0] = active ? pop0[0] * pop[0] : 0.f;
    c[1] = active ? pop0[0] * pop[1] : 0.f;
    c[2] = active ? pop0[1] * pop[0] : 0.f;
    c[3] = active ? pop0[1] * pop[1] : 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) c[q] += __shfl_xor_sync(0xffffffffu, c[q], off);
    if ((threadIdx.x & 31) == 0 && isave < p.nsave) {
        // FP32 partial sums, one 16-byte store (the fast paths' buffer holds floats; the host
        // reduction sums them in FP64): no FP32-to-FP64 conversion in the step loop
        int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        reinterpret_cast<float4*>(p.popcorr_partial)[warp * p.nsave + isave] = make_float4(c[0], c[1], c[2], c[3]);
    }
}

template <typename R>
__device__ __forceinline__ void write_sigma(const FsshParams& p, int64_t i, const Sig2<R>& sg) {
    const int64_t N = p.ntraj;
    p.sigma[0 * N + i] = sg.p;
    p.sigma[1 * N + i] = 0.0;
    p.sigma[2 * N + i] = sg.x;
    p.sigma[3 * N + i] = sg.y;
    p.sigma[4 * N + i] = sg.x;
    p.sigma[5 * N + i] = -(double)sg.y;
    p.sigma[6 * N + i] = sg.q;
    p.sigma[7 * N + i] = 0.0;
}

__device__ __forceinline__ void log_hop(const FsshParams& p, bool active, int64_t i, int nh, int step, int from,
                                        int to) {
    if (active && p.hop_log && nh < p.max_hops) {
        const int64_t N = p.ntraj;
        p.hop_log[((int64_t)nh * 3 + 0) * N + i] = step;
        p.hop_log[((int64_t)nh * 3 + 1) * N + i] = from;
        p.hop_log[((int64_t)nh * 3 + 2) * N + i] = to;
    }
}

// ---------------------------------------------------------------------------
// Tully models (1 DoF)
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kFsshBlock) fssh2_tully_kernel(const FsshParams p) {
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i0 < p.ntraj;
    const int64_t i = active ? i0 : p.ntraj - 1;
    const int64_t gid = p.traj_offset + i;

    R mp[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) mp[q] = (R)p.mp[q];
    const double mass = p.mass[0];
    double x = p.r[i], v = p.v[i];

    R Z[4] = {R(1), R(0), R(0), R(1)};
    R w[2], A[3], nac;
    auto update_cache = [&](double xx) {
        R V[3], D[3], Zn[4];
        tully_potential<R>(p.model, mp, (R)xx, V);
        eigen2_phase<R>(V, Z, w, Zn);
#pragma unroll
        for (int q = 0; q < 4; ++q) Z[q] = Zn[q];
        tully_derivative<R>(p.model, mp, (R)xx, D);
        adiabatic_derivative2<R>(D, Z, A);
        nac = A[1] / (w[1] - w[0]);
    };
    Sig2<R> sg;
    int state;
    const bool ehr = p.ehrenfest != 0;
    // FSSH: force of the occupied state; Ehrenfest: of the current density matrix
    auto accel = [&](int s) -> double {
        R a = ehr ? ehrenfest_weight<R>(A[0], A[1], A[2], sg) : (s == 0 ? A[0] : A[2]);
        return (double)(-a / (R)mass);
    };
    auto pot = [&]() { return ehr ? ehrenfest_potential<R>(sg, w) : (double)(state == 0 ? w[0] : w[1]); };

    update_cache(x);
    init_electronics2<R>(p, i, gid, Z, sg, state);
    double k = accel(state);

    double e0 = (0.0 + mass * (v * v)) / 2.0 + pot();
    double pop0[2] = {0.0, 0.0};
    int isave = 0;
    if (p.save_stride > 0) {
        diabatic_pop2<R>(sg, state, Z, pop0, ehr);
        warp_save_popcorr(p, isave++, active, pop0, pop0);
    }

    EBuf<R> buf = {R(0), R(0), R(0), 0.0, R(0), R(0), R(0), 0.0};
    int nh = 0, nf = 0, step = 0;
    double t = p.t0;
    const R dtR = (R)p.dt;
    // the reference's FP64 clock
    while (t < p.t1) {
        double h = (p.t1 - t) < p.dt ? (p.t1 - t) : p.dt;
        double half = h / 2.0;
        double vtmp = v + half * k;
        x = x + h * vtmp;
        update_cache(x);
        k = accel(state);
        v = vtmp + half * k;
        buf.E0c = buf.E0n;
        buf.E1c = buf.E1n;
        buf.Dc = buf.Dn;
        buf.E0n = w[0];
        buf.E1n = w[1];
        buf.Dn = R(0) + nac * (R)v;
        {
            buf.tc = buf.tn;
            buf.tn = t + h;
            electronics2(p, buf, t, h, sg);
            t = snap_time(t + h, p.t1);
        }
        step += 1;

        // hop test
        // real(sigma[m, s] / sigma[s, s]) by Julia's complex division; the
        // imaginary part of sigma[s, s] is exactly zero for two states
        const int s = state;
        R re = cdiv_real(sg.x, s == 0 ? -sg.y : sg.y, s == 0 ? sg.p : sg.q, 0.0);
        R nsm = s == 0 ? nac : -nac;
        R prob = clamp01<R>(R(0) + R(2) * (R)v * re * nsm * dtR);
        double u = rng_uniform(p.seed, (uint64_t)gid, (uint32_t)step, RNG_HOP);
        if (!ehr && (double)prob > u) {  // Ehrenfest: no hopping
            const int ns = 1 - s;
            bool accept = true;
            if (p.rescaling != RESCALE_OFF) {
                double d = (double)(ns < s ? nac : -nac);
                double aa = (0.0 + d * d / mass) / 2.0;
                double bb = 0.0 + d * v;
                double cc = ns == 1 ? (double)w[1] - (double)w[0] : (double)w[0] - (double)w[1];
                double disc = bb * bb - 4.0 * aa * cc;
                if (disc < 0.0) {
                    accept = false;
                    if (p.rescaling == RESCALE_VINVERSION) {
                        double nrm = sqrt(0.0 + d * d);
                        double g = 0.0 + v * (d / nrm);
                        v = v - 2.0 * g * (d / nrm);
                    }
                } else {
                    double root = sqrt(disc);
                    double gamma = bb < 0.0 ? (bb + root) / (2.0 * aa) : (bb - root) / (2.0 * aa);
                    v = v - gamma * d / mass;
                }
            }
            if (accept) {
                log_hop(p, active, i, nh, step, s, ns);
                nh += 1;
                state = ns;
            } else {
                nf += 1;
            }
        }
        // save points are the multiples of save_stride: a product, not an integer division per step
        if (p.save_stride > 0 && step == isave * p.save_stride) {
            double pop[2];
            diabatic_pop2<R>(sg, state, Z, pop, ehr);
            warp_save_popcorr(p, isave++, active, pop0, pop);
        }
    }

    if (!active) return;
    p.r[i] = x;
    p.v[i] = v;
    write_sigma<R>(p, i, sg);
    p.state[i] = state;
    if (p.nhops) p.nhops[i] = nh;
    if (p.nfrustrated) p.nfrustrated[i] = nf;
    if (p.nsteps) p.nsteps[i] = step;
    if (p.energy) {
        p.energy[i] = e0;
        p.energy[p.ntraj + i] = (0.0 + mass * (v * v)) / 2.0 + pot();
    }
    if (p.scatter) atomicAdd(p.scatter + (x > 0.0 ? 2 : 0) + state, 1ull);
}

// Fast one-dimensional Tully kernel: the steps of fssh2_tully_kernel<float>
// with no FP64 arithmetic in the step loop.  Position and velocity are
// Kahan-compensated FP32 accumulators (AccKahan), the force, step lengths and
// hop test are FP32; FP64 remains in the set-up, the rare momentum rescaling
// and the FP64 electronics below the gap threshold.  With one trajectory per
// thread and few trajectories per SM this kernel is bound by the latency of
// one step, to which every FP64 operation (1/73 of the FP32 rate) adds.
// (R = float; a template so that only the FP32 translation unit emits it.)
template <typename R>
__global__ void __launch_bounds__(kFsshBlock) fssh2_tully_fast_kernel(const FsshParams p) {
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i0 < p.ntraj;
    const int64_t i = active ? i0 : p.ntraj - 1;
    const int64_t gid = p.traj_offset + i;

    float mp[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) mp[q] = (float)p.mp[q];
    const double mass = p.mass[0];
    const float inv_mass = (float)(1.0 / mass);
    AccKahan x, v;
    x.load(p.r[i]);
    v.load(p.v[i]);

    float Z[4] = {1.f, 0.f, 0.f, 1.f};
    float w[2], A[3], nac;
    auto update_cache = [&](float xx) {
        float V[3], D[3], Zn[4];
        tully_potential<float>(p.model, mp, xx, V);
        eigen2_phase<float>(V, Z, w, Zn);
#pragma unroll
        for (int q = 0; q < 4; ++q) Z[q] = Zn[q];
        tully_derivative<float>(p.model, mp, xx, D);
        adiabatic_derivative2<float>(D, Z, A);
        nac = A[1] / (w[1] - w[0]);
    };
    Sig2<float> sg;
    int state;
    const bool ehr = p.ehrenfest != 0;
    // FSSH: force of the occupied state; Ehrenfest: of the current density matrix
    auto accel = [&](int s) -> float {
        return -(ehr ? ehrenfest_weight<float>(A[0], A[1], A[2], sg) : (s == 0 ? A[0] : A[2])) * inv_mass;
    };
    auto pot = [&]() { return ehr ? ehrenfest_potential<float>(sg, w) : (double)(state == 0 ? w[0] : w[1]); };

    update_cache(x.f());
    init_electronics2<float>(p, i, gid, Z, sg, state);
    float k = accel(state);
    const double v0 = v.get();
    const double e0 = (0.0 + mass * (v0 * v0)) / 2.0 + pot();
    float pop0[2] = {0.f, 0.f};
    int isave = 0;
    if (p.save_stride > 0) {
        diabatic_pop2_f(sg, state, Z, pop0, ehr);
        warp_save_popcorr_f(p, isave++, active, pop0, pop0);
    }

    EBuf<float> buf = {0.f, 0.f, 0.f, 0.0, 0.f, 0.f, 0.f, 0.0};
    int nh = 0, nf = 0, step = 0, nfp64 = 0;
    const float dtf = (float)p.dt;
    while (step < p.nsteps_total) {
        const float h = step == 0 ? p.h_first : (step + 1 == p.nsteps_total ? p.h_last : p.h_mid);
        const float half = 0.5f * h;
        v.add(half * k);
        x.add(h * v.f());
        update_cache(x.f());
        k = accel(state);
        v.add(half * k);
        buf.E0c = buf.E0n;
        buf.E1c = buf.E1n;
        buf.Dc = buf.Dn;
        buf.E0n = w[0];
        buf.E1n = w[1];
        buf.Dn = nac * v.f();
        electronics2_sched(p, buf, step == 0, h, w[1] - w[0], sg, nfp64);
        step += 1;

        // hop test
        const int s = state;
        const float re = sg.x / (s == 0 ? sg.p : sg.q);
        const float nsm = s == 0 ? nac : -nac;
        const float prob = clamp01<float>(2.0f * v.f() * re * nsm * dtf);
        const float u = rng_uniform_f(p.seed, (uint64_t)gid, (uint32_t)step, RNG_HOP);
        if (!ehr && prob > u) {  // Ehrenfest: no hopping
            const int ns = 1 - s;
            bool accept = true;
            if (p.rescaling != RESCALE_OFF) {
                const double vd = v.get();
                const double d = (double)(ns < s ? nac : -nac);
                const double aa = (0.0 + d * d / mass) / 2.0;
                const double bb = 0.0 + d * vd;
                const double cc = ns == 0 ? (double)w[0] - (double)w[1] : (double)w[1] - (double)w[0];
                const double disc = bb * bb - 4.0 * aa * cc;
                if (disc < 0.0) {
                    accept = false;
                    if (p.rescaling == RESCALE_VINVERSION) {  // one degree of freedom: v -> -v
                        v.s = -v.s;
                        v.c = -v.c;
                    }
                } else {
                    const double root = sqrt(disc);
                    const double gamma = bb < 0.0 ? (bb + root) / (2.0 * aa) : (bb - root) / (2.0 * aa);
                    v.load(vd - gamma * d / mass);
                }
            }
            if (accept) {
                log_hop(p, active, i, nh, step, s, ns);
                nh += 1;
                state = ns;
            } else {
                nf += 1;
            }
        }
        // save points are the multiples of save_stride: a product, not an integer division per step
        if (p.save_stride > 0 && step == isave * p.save_stride) {
            float pf[2];
            diabatic_pop2_f(sg, state, Z, pf, ehr);
            warp_save_popcorr_f(p, isave++, active, pop0, pf);
        }
    }

    if (!active) return;
    const double xf = x.get(), vf = v.get();
    p.r[i] = xf;
    p.v[i] = vf;
    if (p.fp64_steps) p.fp64_steps[i] = nfp64;
    write_sigma<float>(p, i, sg);
    p.state[i] = state;
    if (p.nhops) p.nhops[i] = nh;
    if (p.nfrustrated) p.nfrustrated[i] = nf;
    if (p.nsteps) p.nsteps[i] = step;
    if (p.energy) {
        p.energy[i] = e0;
        p.energy[p.ntraj + i] = (0.0 + mass * (vf * vf)) / 2.0 + pot();
    }
    if (p.scatter) atomicAdd(p.scatter + (xf > 0.0 ? 2 : 0) + state, 1ull);
}

// ---------------------------------------------------------------------------
// Spin-boson (N bath modes, unit or given masses)
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kFsshBlock) fssh2_spinboson_kernel(const FsshParams p) {
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i0 < p.ntraj;
    const int64_t i = active ? i0 : p.ntraj - 1;
    const int64_t gid = p.traj_offset + i;
    const int64_t N = p.ntraj;
    const int nd = p.ndof;
    const double* __restrict__ cj = p.bath_c;
    const double* __restrict__ w2j = p.bath_w2;
    const double* __restrict__ mj = p.mass;
    // inactive lanes (tail of the last warp) follow trajectory i on private
    // copies only through registers: they never store to r or v.
    double* __restrict__ r = p.r + i;
    double* __restrict__ v = p.v + i;
    double* __restrict__ nacs = p.scratch ? p.scratch + i : nullptr;
    const R eps = (R)p.mp[0], Delta = (R)p.mp[1];

    R Z[4] = {R(1), R(0), R(0), R(1)};
    R w[2];
    // Hamiltonian from the sums s0 = sum w2 r^2 and cr = c.r
    auto set_eigen = [&](double s0, double cr) {
        R V[3], Zn[4];
        double V0 = 0.5 * s0;
        V[0] = (V0 + cr) + eps;
        V[1] = Delta;
        V[2] = (V0 - cr) - eps;
        eigen2_phase<R>(V, Z, w, Zn);
#pragma unroll
        for (int q = 0; q < 4; ++q) Z[q] = Zn[q];
    };
    // (Z^T dH_I Z)_ss with dH_I = diag(w2 r + c, w2 r - c), oracle order
    auto adi_ss = [&](const R Zk[4], int s, double rI, int I) -> R {
        R d0 = (R)(w2j[I] * rI);
        R d00 = d0 + (R)cj[I], d11 = d0 - (R)cj[I];
        R z0 = Zk[2 * s], z1 = Zk[2 * s + 1];
        return z0 * (d00 * z0) + z1 * (d11 * z1);
    };
    // Ehrenfest: sum_nm (Z^T dH_I Z)_nm Re sigma_nm, elements in oracle order
    auto adi_ehr = [&](const R Zk[4], const Sig2<R>& sgk, double rI, int I) -> R {
        R d0 = (R)(w2j[I] * rI);
        R d00 = d0 + (R)cj[I], d11 = d0 - (R)cj[I];
        R A00 = Zk[0] * (d00 * Zk[0]) + Zk[1] * (d11 * Zk[1]);
        R A11 = Zk[2] * (d00 * Zk[2]) + Zk[3] * (d11 * Zk[3]);
        R A01 = Zk[0] * (d00 * Zk[2]) + Zk[1] * (d11 * Zk[3]);
        return ehrenfest_weight<R>(A00, A01, A11, sgk);
    };
    const bool ehr = p.ehrenfest != 0;

    double s0 = 0.0, cr = 0.0, ke = 0.0;
    for (int I = 0; I < nd; ++I) {
        double rI = r[(int64_t)I * N];
        double vI = v[(int64_t)I * N];
        s0 = s0 + w2j[I] * (rI * rI);
        cr = cr + cj[I] * rI;
        ke = ke + mj[I] * (vI * vI);
    }
    set_eigen(s0, cr);
    Sig2<R> sg;
    int state;
    init_electronics2<R>(p, i, gid, Z, sg, state);
    double e0 = ke / 2.0 + (ehr ? ehrenfest_potential<R>(sg, w) : (double)(state == 0 ? w[0] : w[1]));
    R Zk[4] = {Z[0], Z[1], Z[2], Z[3]};  // eigenvectors the cached force was computed with
    int sk = state;                      // state the cached force was computed for
    Sig2<R> sgk = sg;                    // Ehrenfest: density matrix the cached force was computed with

    double pop0[2] = {0.0, 0.0};
    int isave = 0;
    if (p.save_stride > 0) {
        diabatic_pop2<R>(sg, state, Z, pop0, ehr);
        warp_save_popcorr(p, isave++, active, pop0, pop0);
    }

    EBuf<R> buf = {R(0), R(0), R(0), 0.0, R(0), R(0), R(0), 0.0};
    int nh = 0, nf = 0, step = 0;
    double t = p.t0;
    while (t < p.t1) {
        double h = (p.t1 - t) < p.dt ? (p.t1 - t) : p.dt;
        double half = h / 2.0;
        // B then A with the cached force (recomputed from r, Zk, sk)
        s0 = 0.0;
        cr = 0.0;
        for (int I = 0; I < nd; ++I) {
            double rI = r[(int64_t)I * N];
            double vI = v[(int64_t)I * N];
            double kI = (double)(-(ehr ? adi_ehr(Zk, sgk, rI, I) : adi_ss(Zk, sk, rI, I)) / (R)mj[I]);
            double vt = vI + half * kI;
            double rn = rI + h * vt;
            if (active) {
                r[(int64_t)I * N] = rn;
                v[(int64_t)I * N] = vt;
            }
            s0 = s0 + w2j[I] * (rn * rn);
            cr = cr + cj[I] * rn;
        }
        set_eigen(s0, cr);
        // B with the new force; couplings
        R Dn;
        {
            double acc = 0.0;
            for (int I = 0; I < nd; ++I) {
                double rI = r[(int64_t)I * N];
                double vt = v[(int64_t)I * N];
                double d0 = w2j[I] * rI;
                double d00 = d0 + cj[I], d11 = d0 - cj[I];
                double a00 = Z[0] * (d00 * Z[0]) + Z[1] * (d11 * Z[1]);
                double a11 = Z[2] * (d00 * Z[2]) + Z[3] * (d11 * Z[3]);
                double a01 = Z[0] * (d00 * Z[2]) + Z[1] * (d11 * Z[3]);
                double ass = ehr ? ehrenfest_weight<double>(a00, a01, a11, sg) : (state == 0 ? a00 : a11);
                double kI = -ass / mj[I];
                double vn = vt + half * kI;
                double nI = a01 / (w[1] - w[0]);
                if (active) {
                    v[(int64_t)I * N] = vn;
                    nacs[(int64_t)I * N] = nI;
                }
                acc = acc + nI * vn;
            }
            Dn = 0.0 + acc;
        }
        Zk[0] = Z[0];
        Zk[1] = Z[1];
        Zk[2] = Z[2];
        Zk[3] = Z[3];
        sk = state;
        sgk = sg;
        buf.E0c = buf.E0n;
        buf.E1c = buf.E1n;
        buf.Dc = buf.Dn;
        buf.tc = buf.tn;
        buf.E0n = w[0];
        buf.E1n = w[1];
        buf.Dn = Dn;
        buf.tn = t + h;
        electronics2(p, buf, t, h, sg);
        t = snap_time(t + h, p.t1);
        step += 1;

        // hop test
        // real(sigma[m, s] / sigma[s, s]) by Julia's complex division; the
        // imaginary part of sigma[s, s] is exactly zero for two states
        const int s = state;
        R re = cdiv_real(sg.x, s == 0 ? -sg.y : sg.y, s == 0 ? sg.p : sg.q, 0.0);
        R prob;
        {
            double acc = 0.0;
            for (int I = 0; I < nd; ++I) {
                double nI = nacs[(int64_t)I * N];
                double nsm = s == 0 ? nI : -nI;
                acc = acc + 2.0 * v[(int64_t)I * N] * re * nsm * p.dt;
            }
            prob = clamp01<double>(acc);
        }
        double u = rng_uniform(p.seed, (uint64_t)gid, (uint32_t)step, RNG_HOP);
        if (!ehr && (double)prob > u) {  // Ehrenfest: no hopping
            const int ns = 1 - s;
            const double sgn = ns < s ? 1.0 : -1.0;  // d(new, old) = sgn * d01
            bool accept = true;
            if (p.rescaling != RESCALE_OFF) {
                double aa = 0.0, bb = 0.0;
                for (int I = 0; I < nd; ++I) {
                    double d = sgn * nacs[(int64_t)I * N];
                    aa = aa + d * d / mj[I];
                    bb = bb + d * v[(int64_t)I * N];
                }
                aa = aa / 2.0;
                double cc = ns == 1 ? (double)w[1] - (double)w[0] : (double)w[0] - (double)w[1];
                double disc = bb * bb - 4.0 * aa * cc;
                if (disc < 0.0) {
                    accept = false;
                    if (p.rescaling == RESCALE_VINVERSION) {
                        double nrm = 0.0;
                        for (int I = 0; I < nd; ++I) {
                            double d = sgn * nacs[(int64_t)I * N];
                            nrm = nrm + d * d;
                        }
                        nrm = sqrt(nrm);
                        double g = 0.0;
                        for (int I = 0; I < nd; ++I) {
                            double d = sgn * nacs[(int64_t)I * N];
                            g = g + v[(int64_t)I * N] * (d / nrm);
                        }
                        for (int I = 0; I < nd; ++I) {
                            double d = sgn * nacs[(int64_t)I * N];
                            double vn = v[(int64_t)I * N] - 2.0 * g * (d / nrm);
                            if (active) v[(int64_t)I * N] = vn;
                        }
                    }
                } else {
                    double root = sqrt(disc);
                    double gamma = bb < 0.0 ? (bb + root) / (2.0 * aa) : (bb - root) / (2.0 * aa);
                    for (int I = 0; I < nd; ++I) {
                        double d = sgn * nacs[(int64_t)I * N];
                        double vn = v[(int64_t)I * N] - gamma * d / mj[I];
                        if (active) v[(int64_t)I * N] = vn;
                    }
                }
            }
            if (accept) {
                log_hop(p, active, i, nh, step, s, ns);
                nh += 1;
                state = ns;
            } else {
                nf += 1;
            }
        }
        // save points are the multiples of save_stride: a product, not an integer division per step
        if (p.save_stride > 0 && step == isave * p.save_stride) {
            double pop[2];
            diabatic_pop2<R>(sg, state, Z, pop, ehr);
            warp_save_popcorr(p, isave++, active, pop0, pop);
        }
    }

    if (!active) return;
    write_sigma<R>(p, i, sg);
    p.state[i] = state;
    if (p.nhops) p.nhops[i] = nh;
    if (p.nfrustrated) p.nfrustrated[i] = nf;
    if (p.nsteps) p.nsteps[i] = step;
    if (p.energy) {
        double ke1 = 0.0;
        for (int I = 0; I < nd; ++I) {
            double vI = v[(int64_t)I * N];
            ke1 = ke1 + mj[I] * (vI * vI);
        }
        p.energy[i] = e0;
        p.energy[N + i] = ke1 / 2.0 + (ehr ? ehrenfest_potential<R>(sg, w) : (double)(state == 0 ? w[0] : w[1]));
    }
    if (p.scatter) atomicAdd(p.scatter + (r[0] > 0.0 ? 2 : 0) + state, 1ull);
}

// Plain path (R = double): one thread per trajectory, both model families.
template <typename R>
cudaError_t launch_fssh2(const FsshParams& p, cudaStream_t s) {
    static_assert(std::is_same<R, double>::value, "the fast paths have their own kernels");
    if (p.ntraj <= 0) return cudaSuccess;
    int64_t blocks = (p.ntraj + kFsshBlock - 1) / kFsshBlock;
    if (p.model == MODEL_SPINBOSON)
        fssh2_spinboson_kernel<R><<<(unsigned)blocks, kFsshBlock, 0, s>>>(p);
    else
        fssh2_tully_kernel<R><<<(unsigned)blocks, kFsshBlock, 0, s>>>(p);
    return cudaGetLastError();
}

// Fast one-dimensional Tully path.
inline cudaError_t launch_tully_fast(const FsshParams& p, cudaStream_t s) {
    if (p.ntraj <= 0) return cudaSuccess;
    int64_t blocks = (p.ntraj + kFsshBlock - 1) / kFsshBlock;
    fssh2_tully_fast_kernel<float><<<(unsigned)blocks, kFsshBlock, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace nqcd
