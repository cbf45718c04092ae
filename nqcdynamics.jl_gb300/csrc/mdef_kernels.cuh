// MDEF (electronic-friction Langevin dynamics) on the Newns-Anderson model,
// one warp per trajectory.
//
// Reference algorithm (NQCDynamics.jl):
//   MDEF_BAOAB.perform_step!    src/DynamicsMethods/IntegrationAlgorithms/mdef_baoab.jl:163-180
//   step_O! (friction eigenbasis) src/DynamicsMethods/IntegrationAlgorithms/steps.jl:41-69
//   DiabaticMDEF acceleration!  src/DynamicsMethods/ClassicalMethods/mdef.jl:102-124
//   friction! (Lambda / sqrt(m)sqrt(m)^T) src/DynamicsMethods/ClassicalMethods/mdef.jl:131-140
// The reference diagonalises the (1 + M)-state one-electron Hamiltonian
//     H = [[h(x), V_k], [V_k, diag(e_k)]]     (AndersonHolstein)
// with LAPACK at every force and friction evaluation.  This Hamiltonian is
// an arrowhead matrix with x-independent border, so its eigenvalues are the
// roots of the secular function
//     f(l) = l - h - sum_k V_k^2 / (l - e_k),
// one in each interval between consecutive bath levels plus one on each side,
// and the impurity weights of the eigenvectors are z0_i^2 = 1 / f'(l_i).
// Because dH/dx = h'(x) e0 e0^T, the Fermi-weighted force and the broadened
// friction need only (l_i, z0_i^2):
//     F = U0'(x) + h' sum_i z0_i^2 (f_i + f'_i l_i),
//     Lambda = -pi h'^2 sum_nm z0_n^2 z0_m^2 g_sigma(l_n - l_m) f'(l_n).
// So each of the 32 lanes owns roots i = lane, lane + 32, ... and solves them
// by bracketed Newton measured from the nearer pole (accurate next to a pole),
// warm-started from the previous evaluation.
//
// R = double: plain FP64 (all terms of the friction double sum).
// R = float : fast path; Fermi factors below 1e-12 of their maximum and
//             Gaussian factors beyond 8 sigma are skipped; optional friction
//             surrogate network (BF16 weights, FP32 arithmetic) in place of the
//             midpoint electronic evaluation.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "nqcd_math.h"
#include "secular.h"

namespace nqcd {

constexpr int kMdefMaxBath = 512;
constexpr int kMdefRootsPerLane = (kMdefMaxBath + 1 + 31) / 32;
constexpr int kMdefWarps = 4;  // trajectories per block

struct MlpWeights {
    // 1-64-64-1 network, SiLU activations, output = softplus -> Cholesky factor L, Lambda = L^2
    const __nv_bfloat16* W1;  // [64]
    const __nv_bfloat16* b1;  // [64]
    const __nv_bfloat16* W2;  // [64][64] row-major (out, in)
    const __nv_bfloat16* b2;  // [64]
    const __nv_bfloat16* W3;  // [64]
    const __nv_bfloat16* b3;  // [1]
    float x_shift, x_scale;   // input normalisation
    float lo, hi;             // training domain (outside: exact friction)
    float floor;              // judge: relative errors are taken against max(|exact|, floor)
};

struct MdefParams {
    int32_t nbath;
    const double* eps;   // [nbath] ascending
    const double* V2;    // [nbath] V_k^2
    double k, g, delta;  // impurity: U0 = k x^2/2, h = k g (g/2 - x) + delta
    // model3d = 1: the three-dimensional adsorbate (one atom, x, y, z; state [3][ntraj]):
    // U0 = kxy (x^2 + y^2)/2 + A exp(-a z), h = delta - B exp(-b z).  Its friction tensor
    // F grad h grad h^T has the one nonzero eigenvalue F (dh/dz)^2 along z.
    int32_t model3d;
    double kxy, A, a, B, b;
    double mu, beta, sigma;
    double mass;
    int64_t ntraj, traj_offset;
    double dt;
    double h_last;          // length of the last step (dt unless the span is not a whole number of steps)
    int32_t nsteps;
    uint64_t seed;
    int32_t save_stride, nsave;
    int32_t use_mlp;        // fast path: friction from the surrogate inside its domain
    int32_t exact_friction_every;    // fast path with surrogate: exact friction every k steps (0 = never)
    double judge_tol;       // relative error of a judged network value that retires the network for the trajectory
    MlpWeights mlp;
    double* x;              // [ntraj] in/out
    double* v;              // [ntraj] in/out
    double* energy;         // [2][ntraj] (initial, final) or null
    double* obs_partial;    // [nwarps_total][nsave][4] (<x>, <x^2>, <KE>, <Lambda>)
    unsigned long long* counters;  // [0] exact friction evaluations, [1] surrogate evaluations, [2] non-converged roots,
                                   // [8] judged steps, [9] rejected trajectories, [10] largest judged relative
                                   // error (bits of a non-negative double), [11] sum of judged relative errors (double)
    double* friction_out;   // optional: exact friction at x (single evaluation mode), [ntraj]
    double* force_out;      // optional: force at x, [ntraj]
    // ring polymers (RingPolymerSimulation{DiabaticMDEF}, rpmdef_kernel): x, v are [bead][ntraj]
    int32_t nbeads;         // 0 or 1: classical nuclei (mdef_kernel)
    const double* rp_U;     // [nbeads * nbeads] normal-mode matrix, column-major U[j + n k]
    const double* rp_half;  // [nbeads][4] half-step Cayley matrices (c11, c12, c21, c22)
};

template <typename R>
struct MdefShared {
    R eps[kMdefMaxBath];
    R V2[kMdefMaxBath];
    R lam[kMdefWarps][kMdefMaxBath + 1];
    R z2[kMdefWarps][kMdefMaxBath + 1];
};

template <typename R>
__device__ __forceinline__ R mdef_exp(R x) {
    if constexpr (std::is_same<R, float>::value)
        return __expf(x);
    else
        return nqcd_exp(x);
}

// Fermi function and its derivative, f = 1/(1+e^{b(e-mu)}), f' = -b f (1-f).
template <typename R>
__device__ __forceinline__ void fermi_pair(R e, R mu, R beta, R& f, R& df) {
    R z = beta * (e - mu);
    if (z > R(0)) {
        R ez = mdef_exp<R>(-z);
        f = ez / (R(1) + ez);
    } else {
        R ez = mdef_exp<R>(z);
        f = R(1) / (R(1) + ez);
    }
    df = -beta * f * (R(1) - f);
}

// Electronic structure at x for the warp's trajectory: all roots, force and
// (optionally) friction.  Roots and weights are also left in shared memory.
template <typename R, bool D3 = false>
__device__ void mdef_electronic(const MdefParams& p, MdefShared<R>& sh, int wib, R lam[kMdefRootsPerLane],
                                double x, bool want_friction, double& force, double& friction) {
    const int lane = threadIdx.x & 31;
    const int M = p.nbath;
    // x is the height z for the three-dimensional adsorbate; dU0 its derivative of U0
    R h, dh;
    double dU0;
    if constexpr (D3) {
        if constexpr (std::is_same<R, float>::value) {
            const float e = expf(-(float)p.b * (float)x);
            h = (float)p.delta - (float)p.B * e;
            dh = (float)p.B * (float)p.b * e;
            dU0 = -p.A * p.a * (double)expf(-(float)p.a * (float)x);
        } else {
            const double e = nqcd_exp(-p.b * x);
            h = p.delta - p.B * e;
            dh = p.B * p.b * e;
            dU0 = -p.A * p.a * nqcd_exp(-p.a * x);
        }
    } else {
        h = (R)(p.k * p.g * (p.g / 2.0 - x) + p.delta);
        dh = (R)(-p.k * p.g);
        dU0 = p.k * x;
    }
    const R mu = (R)p.mu, beta = (R)p.beta;
    R Lb = fabs(h) + R(2);
    R accF = R(0);
    // the root's Fermi weight in the force, and its eigenpair for the friction
    auto finish = [&](int q, int i, R l, R z2) {
        lam[q] = l;
        R f, df;
        fermi_pair<R>(l, mu, beta, f, df);
        accF += z2 * (f + df * l);
        sh.lam[wib][i] = l;
        sh.z2[wib][i] = z2;
    };
    unsigned long long* nonconv = p.counters ? p.counters + 2 : nullptr;
    if constexpr (std::is_same<R, float>::value) {
        // A lane's seven roots one evaluation of f at a time: a lane whose root has converged
        // starts its next one while the others still iterate (each lane finishes its roots in
        // the same order and with the same arithmetic as one solve after the other).  One copy
        // of the solver in the step loop; the warm starts live in local memory.
        SecularSolve<R> st;
        int q = 0, i = lane;
        bool act = i <= M;
        if (act) secular_begin<R>(sh.eps, M, i, Lb, lam[0], st);
        while (__any_sync(0xffffffffu, act)) {
            if (act && secular_eval<R>(sh.eps, sh.V2, M, h, lam[q], st, nonconv)) {
                finish(q, i, st.o + st.d, R(1) / st.fp);
                ++q;
                i = lane + 32 * q;
                act = q < kMdefRootsPerLane && i <= M;
                if (act) secular_begin<R>(sh.eps, M, i, Lb, lam[q], st);
            }
        }
    } else {
        // one copy of the root solve, not one per root of the lane: the unrolled copies of both
        // electronic evaluations of a step outgrew the instruction cache (the warm starts then
        // live in local memory, two accesses per solve)
#pragma unroll 1
        for (int q = 0; q < kMdefRootsPerLane; ++q) {
            int i = lane + 32 * q;
            if (i <= M) {
                R l = lam[q], z2;
                secular_root<R>(sh.eps, sh.V2, M, i, h, Lb, l, z2, nonconv);
                finish(q, i, l, z2);
            }
        }
    }
    // warp sum in the working precision (no FP64 shuffle-adds on the fast path)
    for (int off = 16; off > 0; off >>= 1) accF += __shfl_xor_sync(0xffffffffu, accF, off);
    force = dU0 + (double)dh * (double)accF;
    friction = 0.0;
    if (!want_friction) return;
    __syncwarp();
    const R inv_s2 = R(0.5) / (R)(p.sigma * p.sigma);
    const R norm = R(1) / ((R)p.sigma * R(2.5066282746310002));  // 1/(sigma sqrt(2 pi))
    R acc = R(0);
    for (int n = lane; n <= M; n += 32) {
        R ln = sh.lam[wib][n];
        R f, df;
        fermi_pair<R>(ln, mu, beta, f, df);
        if constexpr (std::is_same<R, float>::value) {
            if (fabsf(df) < 1e-12f * beta) continue;  // negligible Fermi derivative
        }
        R zn = sh.z2[wib][n];
        R inner = R(0);
        for (int m = 0; m <= M; ++m) {
            R de = ln - sh.lam[wib][m];
            if constexpr (std::is_same<R, float>::value) {
                if (fabsf(de) > 8.0f * (float)p.sigma) continue;
            }
            inner += sh.z2[wib][m] * mdef_exp<R>(-de * de * inv_s2);
        }
        acc += zn * inner * df;
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    friction = -3.14159265358979323846 * (double)dh * (double)dh * (double)norm * (double)acc;
    __syncwarp();
}

// Surrogate friction: 1-64-64-1 network, BF16 weights, FP32 arithmetic; each
// lane computes two hidden units per layer.
__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

__device__ inline float mlp_friction(const MlpWeights& w, float x) {
    const int lane = threadIdx.x & 31;
    float u = (x - w.x_shift) * w.x_scale;
    // hidden layer 1 rounded to BF16, as the tensor-core training kernel sees it
    float h1a = __bfloat162float(__float2bfloat16(silu(__bfloat162float(w.W1[lane]) * u + __bfloat162float(w.b1[lane]))));
    float h1b = __bfloat162float(
        __float2bfloat16(silu(__bfloat162float(w.W1[lane + 32]) * u + __bfloat162float(w.b1[lane + 32]))));
    float za = __bfloat162float(w.b2[lane]), zb = __bfloat162float(w.b2[lane + 32]);
#pragma unroll 8
    for (int j = 0; j < 32; ++j) {
        float hj0 = __shfl_sync(0xffffffffu, h1a, j);
        float hj1 = __shfl_sync(0xffffffffu, h1b, j);
        za += __bfloat162float(w.W2[lane * 64 + j]) * hj0 + __bfloat162float(w.W2[lane * 64 + 32 + j]) * hj1;
        zb += __bfloat162float(w.W2[(lane + 32) * 64 + j]) * hj0 + __bfloat162float(w.W2[(lane + 32) * 64 + 32 + j]) * hj1;
    }
    float o = __bfloat162float(w.W3[lane]) * silu(za) + __bfloat162float(w.W3[lane + 32]) * silu(zb);
    for (int off = 16; off > 0; off >>= 1) o += __shfl_xor_sync(0xffffffffu, o, off);
    o += __bfloat162float(w.b3[0]);
    float L = o > 20.f ? o : log1pf(__expf(o));  // softplus
    return L * L;
}

// Standard normal of (trajectory, step): Box-Muller on one Philox block.
__device__ __forceinline__ double noise_normal(uint64_t seed, uint64_t traj, uint32_t step, uint32_t dof = 0) {
    u32x4 b = rng_block(seed, traj, step, RNG_NOISE + 16u * dof);
    double u1 = 1.0 - u01_from_words(b.x, b.y);
    double u2 = u01_from_words(b.z, b.w);
    return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

// Fast path: the same Box-Muller transform of the same Philox block with
// 24-bit uniforms in FP32.
__device__ __forceinline__ float noise_normal_f(uint64_t seed, uint64_t traj, uint32_t step, uint32_t dof = 0) {
    u32x4 b = rng_block(seed, traj, step, RNG_NOISE + 16u * dof);
    const float u1 = 1.f - (float)(b.x >> 8) * 0x1.0p-24f;
    const float u2 = (float)(b.z >> 8) * 0x1.0p-24f;
    return sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
}

// D3: the three-dimensional adsorbate (p.model3d), a separate instantiation so that the
// one-dimensional kernel keeps its registers
template <typename R, bool D3>
__global__ void __launch_bounds__(32 * kMdefWarps) mdef_kernel(const MdefParams p) {
    __shared__ MdefShared<R> sh;
    for (int k = threadIdx.x; k < p.nbath; k += blockDim.x) {
        sh.eps[k] = (R)p.eps[k];
        sh.V2[k] = (R)p.V2[k];
    }
    __syncthreads();
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t w0 = (int64_t)blockIdx.x * kMdefWarps + wib;
    const bool active = w0 < p.ntraj;
    const int64_t i = active ? w0 : p.ntraj - 1;
    const uint64_t gid = (uint64_t)(p.traj_offset + i);
    const int M = p.nbath;
    R lam[kMdefRootsPerLane];
#pragma unroll
    for (int q = 0; q < kMdefRootsPerLane; ++q) {  // initial guesses: just above each pole
        int idx = lane + 32 * q;
        lam[q] = idx == 0 ? sh.eps[0] - R(1e-3) : (idx <= M ? sh.eps[idx - 1] + R(1e-9) : R(0));
    }
    // x, v: the coordinate the electronic structure depends on (z of the three-dimensional
    // adsorbate, whose x, y move in the harmonic U0 alone: rx, ry, vx, vy); single-evaluation
    // mode reads p.x as a list of those coordinates
    const bool single = p.force_out || p.friction_out;
    const bool d3 = D3 && !single;
    const int64_t NT = p.ntraj;
    double x = p.x[d3 ? 2 * NT + i : i], v = p.v[d3 ? 2 * NT + i : i];
    double rx = d3 ? p.x[i] : 0.0, ry = d3 ? p.x[NT + i] : 0.0;
    double vx = d3 ? p.v[i] : 0.0, vy = d3 ? p.v[NT + i] : 0.0;
    const double m = p.mass, T = 1.0 / p.beta, dt = p.dt, half = 0.5;
    const float inv_m_f = (float)(1.0 / m), sig_f = (float)sqrt(T / m);
    const uint32_t zdof = d3 ? 2u : 0u;  // noise stream of the friction's direction
    double F, fr;
    mdef_electronic<R, D3>(p, sh, wib, lam, x, p.friction_out != nullptr, F, fr);
    if (single) {  // single-evaluation mode (force/friction tables, training data)
        if (active && lane == 0) {
            if (p.force_out) p.force_out[i] = F;
            if (p.friction_out) p.friction_out[i] = fr;
        }
        return;
    }
    double k = -F / m;
    // total energy with the potential of DiabaticMDEF, U0 + sum_i l_i f_i
    // (mdef.jl:162-175), from the roots of the last electronic evaluation at x
    auto total_energy = [&]() {
        R acc = R(0);
        for (int n = lane; n <= M; n += 32) {
            R f, df;
            fermi_pair<R>(sh.lam[wib][n], (R)p.mu, (R)p.beta, f, df);
            acc += sh.lam[wib][n] * f;
        }
        double s = (double)acc;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (d3)
            return 0.5 * m * (vx * vx + vy * vy + v * v) + 0.5 * p.kxy * (rx * rx + ry * ry) +
                   p.A * (std::is_same<R, float>::value ? (double)expf(-(float)p.a * (float)x) : nqcd_exp(-p.a * x)) + s;
        return 0.5 * m * v * v + 0.5 * p.k * x * x + s;
    };
    const double e0 = p.energy ? total_energy() : 0.0;
    int isave = 0;
    auto save = [&](double lamv) {
        if (p.save_stride <= 0) return;
        if (lane == 0 && active && isave < p.nsave) {
            double* dst = p.obs_partial + ((int64_t)(blockIdx.x * kMdefWarps + wib) * p.nsave + isave) * 4;
            dst[0] = x;
            dst[1] = x * x;
            dst[2] = 0.5 * m * (vx * vx + vy * vy + v * v);
            dst[3] = lamv;
        }
        ++isave;
    };
    save(0.0);
    unsigned long long n_exact = 0, n_mlp = 0, n_judged = 0;
    bool net_on = p.use_mlp != 0;  // the judge retires the network for this trajectory
    double err_max = 0.0, err_sum = 0.0;
    for (int step = 1; step <= p.nsteps; ++step) {
        // the integrator's dt: the shortened last step reaches t1 (mdef_baoab.jl:163-180)
        const double hs = step == p.nsteps ? p.h_last : dt;
        v = v + (half * hs) * k;  // B
        x = x + (half * hs) * v;  // A
        if (d3) {  // x, y: harmonic U0, no friction (the O step leaves them)
            vx = vx + (half * hs) * (-(p.kxy * rx) / m);
            vy = vy + (half * hs) * (-(p.kxy * ry) / m);
            rx = rx + (half * hs) * vx;
            ry = ry + (half * hs) * vy;
        }
        double lamv;
        bool in_domain = false, judge = false;
        if constexpr (std::is_same<R, float>::value) {
            in_domain = net_on && (float)x >= p.mlp.lo && (float)x <= p.mlp.hi;
            judge = in_domain && p.exact_friction_every > 0 && step % p.exact_friction_every == 0;
        }
        // x is the same in every lane of the warp, so these branches are warp-uniform
        if (in_domain && !judge) {
            lamv = (double)mlp_friction(p.mlp, (float)x);
            ++n_mlp;
        } else {
            double Fm;
            mdef_electronic<R, D3>(p, sh, wib, lam, x, true, Fm, lamv);
            ++n_exact;
            if (judge) {  // the exact friction (mdef.jl:131-140) judges the network at this step
                const double net = (double)mlp_friction(p.mlp, (float)x);
                const double ref = fabs(lamv) > (double)p.mlp.floor ? fabs(lamv) : (double)p.mlp.floor;
                const double err = fabs(net - lamv) / ref;
                ++n_judged;
                err_sum += err;
                err_max = err > err_max ? err : err_max;
                if (!(err <= p.judge_tol)) net_on = false;
            }
        }
        if constexpr (std::is_same<R, float>::value) {
            // O step in FP32: c2 = sqrt(1 - c1^2) as sqrt(-expm1(-2 gamma dt)), accurate for small gamma dt
            float gdt = (float)lamv * inv_m_f * (float)hs;
            if (gdt < 0.f) gdt = 0.f;
            const float c1 = expf(-gdt);
            const float c2 = sqrtf(-expm1f(-2.f * gdt));
            const float xi = noise_normal_f(p.seed, gid, (uint32_t)step, zdof);
            v = (double)c1 * v + (double)(c2 * sig_f * xi);
        } else {
            double gam = lamv / m;  // friction / (sqrt m sqrt m)
            if (gam < 0.0) gam = 0.0;
            double c1 = exp(-gam * hs);
            double c2 = sqrt(1.0 - c1 * c1);
            double xi = noise_normal(p.seed, gid, (uint32_t)step, zdof);
            v = c1 * v + c2 * (sqrt(T / m) * xi);  // O
        }
        x = x + (half * hs) * v;                // A
        double Fn, dummy;
        mdef_electronic<R, D3>(p, sh, wib, lam, x, false, Fn, dummy);
        k = -Fn / m;
        v = v + (half * hs) * k;  // B
        if (d3) {
            rx = rx + (half * hs) * vx;
            ry = ry + (half * hs) * vy;
            vx = vx + (half * hs) * (-(p.kxy * rx) / m);
            vy = vy + (half * hs) * (-(p.kxy * ry) / m);
        }
        // save points are the multiples of save_stride: a product, not an integer division per step
        if (p.save_stride > 0 && step == isave * p.save_stride) {
            save(lamv);
        }
    }
    const double e1 = p.energy ? total_energy() : 0.0;
    if (!active || lane != 0) return;
    p.x[d3 ? 2 * NT + i : i] = x;
    p.v[d3 ? 2 * NT + i : i] = v;
    if (d3) {
        p.x[i] = rx;
        p.x[NT + i] = ry;
        p.v[i] = vx;
        p.v[NT + i] = vy;
    }
    if (p.energy) {
        p.energy[i] = e0;
        p.energy[p.ntraj + i] = e1;
    }
    if (p.counters) {
        atomicAdd(p.counters + 0, n_exact);
        atomicAdd(p.counters + 1, n_mlp);
        if (n_judged) {
            atomicAdd(p.counters + 8, n_judged);
            if (p.use_mlp && !net_on) atomicAdd(p.counters + 9, 1ull);
            // non-negative doubles order as their bit patterns
            atomicMax(p.counters + 10, (unsigned long long)__double_as_longlong(err_max));
            atomicAdd(reinterpret_cast<double*>(p.counters + 11), err_sum);
        }
    }
}

// ---------------------------------------------------------------------------
// Ring-polymer MDEF (RingPolymerSimulation{DiabaticMDEF}, rpmdef.jl) with the
// BCOCB integrator (bcocb.jl:79-105): per step B (each bead's Fermi-weighted
// force, rpmdef.jl:30-55), half Cayley step of the free ring polymer in
// normal modes, O in bead space with each bead's own broadened friction and
// noise at the ring-polymer temperature n T (steps.jl:71-107), half Cayley
// step, B.  One CTA per trajectory: its kMdefWarps warps take the beads in
// turn (bead j on warp j mod kMdefWarps; a warp's secular roots start from its
// previous bead's, which lies close by), and warp 0 does the ring-polymer
// algebra on the bead arrays in shared memory.  The per-bead noise is the
// Philox normal of (trajectory, step, dof = bead).
// ---------------------------------------------------------------------------
constexpr int kRpMdefMaxBeads = 32;

template <typename R>
__global__ void __launch_bounds__(32 * kMdefWarps) rpmdef_kernel(const MdefParams p) {
    __shared__ MdefShared<R> sh;
    __shared__ double bx[kRpMdefMaxBeads], bv[kRpMdefMaxBeads], bk[kRpMdefMaxBeads];
    __shared__ double qx[kRpMdefMaxBeads], qv[kRpMdefMaxBeads];
    for (int k = threadIdx.x; k < p.nbath; k += blockDim.x) {
        sh.eps[k] = (R)p.eps[k];
        sh.V2[k] = (R)p.V2[k];
    }
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t i = blockIdx.x;
    const uint64_t gid = (uint64_t)(p.traj_offset + i);
    const int64_t N = p.ntraj;
    const int B = p.nbeads, M = p.nbath;
    const double m = p.mass, dt = p.dt, half = 0.5;
    const double sig_rp = sqrt((double)B / p.beta / m);  // sqrt(T_rp / m), T_rp = n T
    for (int j = threadIdx.x; j < B; j += blockDim.x) {
        bx[j] = p.x[(int64_t)j * N + i];
        bv[j] = p.v[(int64_t)j * N + i];
    }
    R lam[kMdefRootsPerLane];
#pragma unroll
    for (int q = 0; q < kMdefRootsPerLane; ++q) {
        int idx = lane + 32 * q;
        lam[q] = R(0);
        if (idx <= M) lam[q] = idx == 0 ? (R)p.eps[0] - R(1e-3) : (R)p.eps[idx - 1] + R(1e-9);
    }
    __syncthreads();
    // forces of all beads (warp w: beads w, w + kMdefWarps, ...)
    auto forces = [&]() {
        for (int j = wib; j < B; j += kMdefWarps) {
            double F, fr;
            mdef_electronic<R>(p, sh, wib, lam, bx[j], false, F, fr);
            if (lane == 0) bk[j] = -F / m;
        }
        __syncthreads();
    };
    // half Cayley step of the free ring polymer: to normal modes, rotate, back (warp 0)
    auto free_half = [&]() {
        if (wib == 0) {
            if (lane < B) {
                double a = 0.0, b = 0.0;
                for (int j = 0; j < B; ++j) {
                    const double u = p.rp_U[j + B * lane];
                    a = a + u * bx[j];
                    b = b + u * bv[j];
                }
                const double* c = p.rp_half + 4 * lane;
                qx[lane] = c[0] * a + c[1] * b;
                qv[lane] = c[2] * a + c[3] * b;
            }
            __syncwarp();
            if (lane < B) {
                double a = 0.0, b = 0.0;
                for (int k = 0; k < B; ++k) {
                    const double u = p.rp_U[lane + B * k];
                    a = a + u * qx[k];
                    b = b + u * qv[k];
                }
                bx[lane] = a;
                bv[lane] = b;
            }
        }
        __syncthreads();
    };
    forces();
    unsigned long long n_exact = 0;
    for (int step = 1; step <= p.nsteps; ++step) {
        if (threadIdx.x < B) bv[threadIdx.x] = bv[threadIdx.x] + (half * dt) * bk[threadIdx.x];  // B
        __syncthreads();
        free_half();  // C
        for (int j = wib; j < B; j += kMdefWarps) {  // O
            double F, lamv;
            mdef_electronic<R>(p, sh, wib, lam, bx[j], true, F, lamv);
            ++n_exact;
            if (lane == 0) {
                if constexpr (std::is_same<R, float>::value) {
                    float gdt = (float)lamv / (float)m * (float)dt;
                    if (gdt < 0.f) gdt = 0.f;
                    const float c1 = expf(-gdt), c2 = sqrtf(-expm1f(-2.f * gdt));
                    const float xi = noise_normal_f(p.seed, gid, (uint32_t)step, (uint32_t)j);
                    bv[j] = (double)c1 * bv[j] + (double)(c2 * (float)sig_rp * xi);
                } else {
                    double gam = lamv / m;
                    if (gam < 0.0) gam = 0.0;
                    const double c1 = exp(-gam * dt), c2 = sqrt(1.0 - c1 * c1);
                    bv[j] = c1 * bv[j] + c2 * (sig_rp * noise_normal(p.seed, gid, (uint32_t)step, (uint32_t)j));
                }
            }
        }
        __syncthreads();
        free_half();  // C
        forces();     // B (new forces)
        if (threadIdx.x < B) bv[threadIdx.x] = bv[threadIdx.x] + (half * dt) * bk[threadIdx.x];
        __syncthreads();
    }
    for (int j = threadIdx.x; j < B; j += blockDim.x) {
        p.x[(int64_t)j * N + i] = bx[j];
        p.v[(int64_t)j * N + i] = bv[j];
    }
    if (p.counters && lane == 0) atomicAdd(p.counters + 0, n_exact);
}

template <typename R>
cudaError_t launch_rpmdef(const MdefParams& p, cudaStream_t s) {
    if (p.ntraj <= 0) return cudaSuccess;
    if (p.nbath > kMdefMaxBath || p.nbath < 1 || p.nbeads < 1 || p.nbeads > kRpMdefMaxBeads) return cudaErrorInvalidValue;
    rpmdef_kernel<R><<<(unsigned)p.ntraj, 32 * kMdefWarps, 0, s>>>(p);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_mdef(const MdefParams& p, cudaStream_t s) {
    if (p.nbeads > 1) return launch_rpmdef<R>(p, s);
    if (p.ntraj <= 0) return cudaSuccess;
    if (p.nbath > kMdefMaxBath || p.nbath < 1) return cudaErrorInvalidValue;
    int64_t blocks = (p.ntraj + kMdefWarps - 1) / kMdefWarps;
    if (p.model3d)
        mdef_kernel<R, true><<<(unsigned)blocks, 32 * kMdefWarps, 0, s>>>(p);
    else
        mdef_kernel<R, false><<<(unsigned)blocks, 32 * kMdefWarps, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace nqcd
