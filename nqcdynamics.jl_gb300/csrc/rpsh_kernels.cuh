// Ring-polymer surface hopping (RPSH) ensemble kernels, two-state Tully models.
//
// Reference algorithm (NQCDynamics.jl):
//   BCBwithTsit5.perform_step!   src/DynamicsMethods/IntegrationAlgorithms/bcb_electronics.jl:53-97
//   step_C! (Cayley free step)   src/DynamicsMethods/IntegrationAlgorithms/steps.jl:10-17
//   cayley_propagator            src/RingPolymers/ring_polymer.jl:71-82
//   RPSH rescaling / inversion   src/DynamicsMethods/SurfaceHoppingMethods/rpsh.jl:127-147
//   hopping with centroid data   SurfaceHoppingMethods.jl:403-425, fssh.jl:254-289
//   TerminatingCallback          src/DynamicsUtils/callbacks.jl:29
//
// Uneven ensembles: trajectories carry their own bead count (one of the
// instantiated counts 1, 2, 4, 5, 8, 10, 16, 32).  The host sorts them
// into bead-count classes; one persistent launch serves all classes.  Each
// thread takes a trajectory from its class's atomic queue, integrates it
// until the termination test or the end time, then refills its slot with the
// next trajectory; when its class is drained it moves on to the other
// classes, so threads never idle while work is left.  The queues are plain
// atomic counters: there is no spin-wait anywhere.
//
//   R = double: plain path, every operation in the CPU oracle's order
//               (translation unit built with -fmad=false): bit-identical.
//   R = float : fast path.  Bead coordinates are split into the centroid
//               (FP64) and deviations from it (FP32); the normal-mode
//               transform, Cayley step, bead forces and the electronics run
//               in FP32.  Since the rescaling shifts every bead by the same
//               amount, hops change only the FP64 centroid velocity.
#pragma once

#include <cuda_runtime.h>

#include "fssh2_kernels.cuh"
#include "fssh2_traj.h"

namespace nqcd {

constexpr int kRpshMaxClasses = 24;  // (Tully model, bead count) pairs
constexpr int kRpshBlock = 128;

struct RpshParams {
    int32_t class_model[kRpshMaxClasses];   // Tully model of each class
    double class_mp[kRpshMaxClasses][8];    // its parameters
    double mass;
    double beta;
    int32_t rescaling;
    int32_t init_kind;
    int32_t init_state;
    float gap_fp64;
    int64_t ntraj;
    int64_t traj_offset;
    double t0, t1, dt;
    // step schedule for the fast path (see FsshParams)
    int32_t nsteps_total;
    float h_first, h_mid, h_last;
    float sa1, sb1;
    float dtsub;
    uint64_t seed;
    double terminate_x;
    int32_t max_hops;
    int32_t nclass;
    int32_t class_beads[kRpshMaxClasses];   // bead count of each class
    int64_t class_begin[kRpshMaxClasses + 1];
    const int32_t* class_traj;              // trajectory indices grouped by class
    const double* U[kRpshMaxClasses];       // per class: n*n column-major U[j + n*k]
    const double* cay[kRpshMaxClasses];     // per class: [n][4]
    const float* Uf[kRpshMaxClasses];       // FP32 copies for the fast path
    const float* cayf[kRpshMaxClasses];
    unsigned long long* queue;              // [nclass] next index within each class
    int32_t first_class_of_block_stride;    // blocks per class assignment stride (see host)
    const int32_t* block_class;             // [gridDim.x] preferred class of each block
    // state SoA
    double* r;      // [bead][ntraj]
    double* v;      // [bead][ntraj]
    double* sigma;  // [8][ntraj]
    int32_t* state;
    int32_t* nhops;
    int32_t* nfrustrated;
    int32_t* nsteps;
    int32_t* hop_log;  // [max_hops][3][ntraj]
    double* energy;    // [2][ntraj]
    unsigned long long* scatter;  // [4]
    // plain path: bead-array scratch, [6 * bead count][scratch_stride] doubles
    double* scratch;
    int64_t scratch_stride;  // threads in the launch
};

__device__ __forceinline__ void rp_log_hop(const RpshParams& p, int64_t i, int nh, int step, int from, int to) {
    if (p.hop_log && nh < p.max_hops) {
        const int64_t N = p.ntraj;
        p.hop_log[((int64_t)nh * 3 + 0) * N + i] = step;
        p.hop_log[((int64_t)nh * 3 + 1) * N + i] = from;
        p.hop_log[((int64_t)nh * 3 + 2) * N + i] = to;
    }
}

template <typename R>
__device__ __forceinline__ void rp_init_sigma(const RpshParams& p, int64_t i, Sig2<R>& sg, int& state) {
    if (p.init_kind == INIT_GIVEN) {
        sg.p = (R)p.sigma[0 * p.ntraj + i];
        sg.x = (R)p.sigma[2 * p.ntraj + i];
        sg.y = (R)p.sigma[3 * p.ntraj + i];
        sg.q = (R)p.sigma[6 * p.ntraj + i];
        state = p.state[i];
    } else {  // adiabatic pure state (diabatic initial states are rejected on the host for RPSH)
        sg.p = p.init_state == 0 ? R(1) : R(0);
        sg.q = p.init_state == 1 ? R(1) : R(0);
        sg.x = R(0);
        sg.y = R(0);
        state = p.init_state;
    }
}

template <typename R>
__device__ __forceinline__ void rp_write_final(const RpshParams& p, int64_t i, const Sig2<R>& sg, int state, int nh,
                                               int nf, int step, double e0, double e1, double x0) {
    const int64_t N = p.ntraj;
    p.sigma[0 * N + i] = sg.p;
    p.sigma[1 * N + i] = 0.0;
    p.sigma[2 * N + i] = sg.x;
    p.sigma[3 * N + i] = sg.y;
    p.sigma[4 * N + i] = sg.x;
    p.sigma[5 * N + i] = -(double)sg.y;
    p.sigma[6 * N + i] = sg.q;
    p.sigma[7 * N + i] = 0.0;
    p.state[i] = state;
    if (p.nhops) p.nhops[i] = nh;
    if (p.nfrustrated) p.nfrustrated[i] = nf;
    if (p.nsteps) p.nsteps[i] = step;
    if (p.energy) {
        p.energy[i] = e0;
        p.energy[N + i] = e1;
    }
    // OutputStateResolvedScattering1D reads the first bead's position
    if (p.scatter) atomicAdd(p.scatter + (x0 > 0.0 ? 2 : 0) + state, 1ull);
}

// Per-bead FSSH force on the active state (sign-invariant, so no phase
// tracking): -(Z^T dH Z)_ss / m, oracle order.  Optionally the bead's
// eigenvalue of the active state.
template <typename R>
__device__ __forceinline__ R rp_bead_accel(int model, const R* mp, R x, int s, R mass, R* ws) {
    R V[3], D[3], w[2], Z[4];
    const R I2[4] = {R(1), R(0), R(0), R(1)};
    tully_potential<R>(model, mp, x, V);
    eigen2_phase<R>(V, I2, w, Z);
    tully_derivative<R>(model, mp, x, D);
    R z0 = Z[2 * s], z1 = Z[2 * s + 1];
    R T0 = D[0] * z0 + D[1] * z1;
    R T1 = D[1] * z0 + D[2] * z1;
    R a = z0 * T0 + z1 * T1;
    if (ws) *ws = w[s];
    return -a / mass;
}

// ---------------------------------------------------------------------------
// plain FP64 trajectory (oracle order)
// ---------------------------------------------------------------------------
// One column of the launch's scratch block: element j of a per-thread bead
// array, stride = threads in the launch (coalesced across a warp).
struct BeadCol {
    double* base;
    int64_t stride;
    __device__ __forceinline__ double& operator[](int j) const { return base[(int64_t)j * stride]; }
};

// The six bead arrays of a plain trajectory (r, v, k, vt and the normal-mode
// q, p) live in the launch's global scratch block, one column per thread,
// instead of in per-thread local arrays: with 16 and 32 beads the local-array
// form of this FP64 code gave wrong results on sm_103a while the identical
// source compiled for the host reproduces the oracle bit for bit (cause not
// identified).  The arithmetic and its order are unchanged.
template <int B>
__device__ __noinline__ void rpsh_traj_plain(const RpshParams& p, int cls, int64_t i) {
    const int64_t N = p.ntraj;
    const int64_t gid = p.traj_offset + i;
    const double mass = p.mass;
    const double* __restrict__ U = p.U[cls];
    const double* __restrict__ cay = p.cay[cls];
    const int model = p.class_model[cls];
    double mp[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) mp[q] = p.class_mp[cls][q];
    const int64_t T = p.scratch_stride;
    double* col = p.scratch + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const BeadCol r{col, T}, v{col + (int64_t)B * T, T}, k{col + (int64_t)2 * B * T, T},
        vt{col + (int64_t)3 * B * T, T}, qm{col + (int64_t)4 * B * T, T}, pm{col + (int64_t)5 * B * T, T};
    for (int j = 0; j < B; ++j) {
        r[j] = p.r[(int64_t)j * N + i];
        v[j] = p.v[(int64_t)j * N + i];
    }
    auto centroid = [&](const BeadCol& x) {
        double acc = 0.0;
        for (int j = 0; j < B; ++j) acc = acc + x[j];
        return acc / B;
    };
    double Zc[4] = {1.0, 0.0, 0.0, 1.0}, w[2], A[3], nac;
    auto update_centroid = [&](double xc) {
        double V[3], D[3], Zn[4];
        tully_potential<double>(model, mp, xc, V);
        eigen2_phase<double>(V, Zc, w, Zn);
#pragma unroll
        for (int q = 0; q < 4; ++q) Zc[q] = Zn[q];
        tully_derivative<double>(model, mp, xc, D);
        adiabatic_derivative2<double>(D, Zc, A);
        nac = A[1] / (w[1] - w[0]);
    };
    auto rp_energy = [&](int s) {
        double wn = B / p.beta;
        double spring = 0.0;
        if (B > 1) {
            spring = spring + mass * ((r[B - 1] - r[0]) * (r[B - 1] - r[0]));
            for (int j = 0; j < B - 1; ++j) spring = spring + mass * ((r[j] - r[j + 1]) * (r[j] - r[j + 1]));
        }
        spring = spring * (wn * wn) / 2.0;
        double ke = 0.0, pe = 0.0;
        for (int j = 0; j < B; ++j) ke = ke + mass * (v[j] * v[j]);
        for (int j = 0; j < B; ++j) {
            double ws;
            rp_bead_accel<double>(model, mp, r[j], s, mass, &ws);
            pe = pe + ws;
        }
        return spring + ke / 2.0 + pe;
    };

    double xc = centroid(r);
    update_centroid(xc);
    Sig2<double> sg;
    int state;
    rp_init_sigma<double>(p, i, sg, state);
    for (int j = 0; j < B; ++j) k[j] = rp_bead_accel<double>(model, mp, r[j], state, mass, nullptr);
    const double e0 = p.energy ? rp_energy(state) : 0.0;

    EBuf<double> buf = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    int nh = 0, nf = 0, step = 0;
    double t = p.t0;
    const double dtsub = p.dt / 5.0;
    while (t < p.t1) {
        double h = (p.t1 - t) < p.dt ? (p.t1 - t) : p.dt;
        double half = h / 2.0;
        for (int j = 0; j < B; ++j) vt[j] = v[j] + half * k[j];
        // to normal modes: q_k = sum_j U[j,k] x_j
        for (int kk = 0; kk < B; ++kk) {
            double a = U[0 + B * kk] * r[0], b = U[0 + B * kk] * vt[0];
            for (int j = 1; j < B; ++j) {
                a = a + U[j + B * kk] * r[j];
                b = b + U[j + B * kk] * vt[j];
            }
            qm[kk] = a;
            pm[kk] = b;
        }
        for (int kk = 0; kk < B; ++kk) {  // step_C!
            const double* c = cay + 4 * kk;
            double rn = c[0] * qm[kk] + c[1] * pm[kk];
            double vn = c[2] * qm[kk] + c[3] * pm[kk];
            qm[kk] = rn;
            pm[kk] = vn;
        }
        // from normal modes: x_j = sum_k U[j,k] q_k
        for (int j = 0; j < B; ++j) {
            double a = U[j] * qm[0], b = U[j] * pm[0];
            for (int kk = 1; kk < B; ++kk) {
                a = a + U[j + B * kk] * qm[kk];
                b = b + U[j + B * kk] * pm[kk];
            }
            r[j] = a;
            vt[j] = b;
        }
        for (int j = 0; j < B; ++j) k[j] = rp_bead_accel<double>(model, mp, r[j], state, mass, nullptr);
        for (int j = 0; j < B; ++j) v[j] = vt[j] + half * k[j];
        xc = centroid(r);
        update_centroid(xc);
        double vc = centroid(v);
        buf.E0c = buf.E0n;
        buf.E1c = buf.E1n;
        buf.Dc = buf.Dn;
        buf.tc = buf.tn;
        buf.E0n = w[0];
        buf.E1n = w[1];
        buf.Dn = 0.0 + nac * vc;
        buf.tn = t + h;
        {
            Interp64 fn(buf);
            electronic_macro_step2<double>(fn, t, h, dtsub, sg);
        }
        t = snap_time(t + h, p.t1);
        step += 1;

        const int s = state;
        double inv = 1.0 / (s == 0 ? sg.p : sg.q);
        double re = sg.x * inv;
        double nsm = s == 0 ? nac : -nac;
        double prob = clamp01<double>(0.0 + 2.0 * vc * re * nsm * p.dt);
        double u = rng_uniform(p.seed, (uint64_t)gid, (uint32_t)step, RNG_HOP);
        if (prob > u) {
            const int ns = 1 - s;
            bool accept = true;
            if (p.rescaling != RESCALE_OFF) {
                double d = ns < s ? nac : -nac;
                double aa = (0.0 + d * d / mass) / 2.0;
                double bb = 0.0 + d * vc;
                double cc = w[ns] - w[s];
                double disc = bb * bb - 4.0 * aa * cc;
                if (disc < 0.0) {
                    accept = false;
                    if (p.rescaling == RESCALE_VINVERSION) {
                        double nrm = sqrt(0.0 + d * d);
                        double dn = d / nrm;
                        double vcom = 0.0;
                        for (int j = 0; j < B; ++j) vcom = vcom + v[j];
                        vcom = vcom / B;
                        double g = 0.0 + vcom * dn;
                        for (int j = 0; j < B; ++j) v[j] = v[j] - 2.0 * g * dn;
                    }
                } else {
                    double root = sqrt(disc);
                    double gamma = bb < 0.0 ? (bb + root) / (2.0 * aa) : (bb - root) / (2.0 * aa);
                    double dv = gamma * d / mass;
                    for (int j = 0; j < B; ++j) v[j] = v[j] - dv;
                }
            }
            if (accept) {
                rp_log_hop(p, i, nh, step, s, ns);
                nh += 1;
                state = ns;
            } else {
                nf += 1;
            }
        }
        if (p.terminate_x > 0.0 && fabs(centroid(r)) > p.terminate_x) break;
    }
    for (int j = 0; j < B; ++j) {
        p.r[(int64_t)j * N + i] = r[j];
        p.v[(int64_t)j * N + i] = v[j];
    }
    const double e1 = p.energy ? rp_energy(state) : 0.0;
    rp_write_final<double>(p, i, sg, state, nh, nf, step, e0, e1, r[0]);
}

// ---------------------------------------------------------------------------
// fast trajectory: FP64 centroid, FP32 internal modes and electronics
// ---------------------------------------------------------------------------
template <int B>
__device__ __noinline__ void rpsh_traj_fast(const RpshParams& p, int cls, int64_t i) {
    const int64_t N = p.ntraj;
    const int64_t gid = p.traj_offset + i;
    const double mass = p.mass;
    const float massf = (float)mass;
    const float* __restrict__ U = p.Uf[cls];
    const float* __restrict__ cay = p.cayf[cls];
    float mp[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) mp[q] = (float)p.class_mp[cls][q];
    const int model = p.class_model[cls];
    // centroid (FP64) and deviations (FP32)
    double xc = 0.0, vc = 0.0;
    float dx[B], dv[B], k[B], qm[B], pm[B];
    {
        double rr[B], vv[B];
#pragma unroll
        for (int j = 0; j < B; ++j) {
            rr[j] = p.r[(int64_t)j * N + i];
            vv[j] = p.v[(int64_t)j * N + i];
            xc += rr[j];
            vc += vv[j];
        }
        xc /= B;
        vc /= B;
#pragma unroll
        for (int j = 0; j < B; ++j) {
            dx[j] = (float)(rr[j] - xc);
            dv[j] = (float)(vv[j] - vc);
        }
    }
    float Zc[4] = {1.f, 0.f, 0.f, 1.f}, w[2], A[3], nac;
    auto update_centroid = [&](double x) {
        float V[3], D[3], Zn[4];
        tully_potential<float>(model, mp, (float)x, V);
        eigen2_phase<float>(V, Zc, w, Zn);
#pragma unroll
        for (int q = 0; q < 4; ++q) Zc[q] = Zn[q];
        tully_derivative<float>(model, mp, (float)x, D);
        adiabatic_derivative2<float>(D, Zc, A);
        nac = A[1] / (w[1] - w[0]);
    };
    auto rp_energy = [&](int s) {
        double wn = B / p.beta;
        double spring = 0.0, ke = 0.0, pe = 0.0;
        for (int j = 0; j < B; ++j) {
            int jn = (j + 1) % B;
            double d = (double)dx[j] - (double)dx[jn];
            if (B > 1) spring += mass * d * d;
            double vj = vc + (double)dv[j];
            ke += mass * vj * vj;
            float ws;
            rp_bead_accel<float>(model, mp, (float)(xc + (double)dx[j]), s, massf, &ws);
            pe += ws;
        }
        return spring * (wn * wn) / 2.0 + ke / 2.0 + pe;
    };
    update_centroid(xc);
    Sig2<float> sg;
    int state;
    rp_init_sigma<float>(p, i, sg, state);
#pragma unroll
    for (int j = 0; j < B; ++j) k[j] = rp_bead_accel<float>(model, mp, (float)(xc + (double)dx[j]), state, massf, nullptr);
    const double e0 = p.energy ? rp_energy(state) : 0.0;

    EBuf<float> buf = {0.f, 0.f, 0.f, 0.0, 0.f, 0.f, 0.f, 0.0};
    int nh = 0, nf = 0, step = 0;
    const float dtf = (float)p.dt;
    // the host's step schedule replaces the reference's FP64 clock
    while (step < p.nsteps_total) {
        const float h = step == 0 ? p.h_first : (step + 1 == p.nsteps_total ? p.h_last : p.h_mid);
        const double hd = h;
        const float half = 0.5f * h;
        // B kick: centroid part in FP64, deviations in FP32
        float kbar = 0.f;
#pragma unroll
        for (int j = 0; j < B; ++j) kbar += k[j];
        kbar *= 1.0f / B;
        double vct = vc + (double)(half * kbar);
#pragma unroll
        for (int j = 0; j < B; ++j) dv[j] += half * (k[j] - kbar);
        // free ring polymer: centroid mode is a free particle, internal modes rotate (Cayley)
        xc = xc + hd * vct;
#pragma unroll
        for (int kk = 1; kk < B; ++kk) {
            float a = 0.f, b = 0.f;
#pragma unroll
            for (int j = 0; j < B; ++j) {
                float u = U[j + B * kk];
                a += u * dx[j];
                b += u * dv[j];
            }
            const float* c = cay + 4 * kk;
            qm[kk] = c[0] * a + c[1] * b;
            pm[kk] = c[2] * a + c[3] * b;
        }
#pragma unroll
        for (int j = 0; j < B; ++j) {
            float a = 0.f, b = 0.f;
#pragma unroll
            for (int kk = 1; kk < B; ++kk) {
                float u = U[j + B * kk];
                a += u * qm[kk];
                b += u * pm[kk];
            }
            dx[j] = a;
            dv[j] = b;
        }
        // bead forces, B kick
        kbar = 0.f;
        const float xcf = (float)xc;
#pragma unroll
        for (int j = 0; j < B; ++j) {
            k[j] = rp_bead_accel<float>(model, mp, xcf + dx[j], state, massf, nullptr);
            kbar += k[j];
        }
        kbar *= 1.0f / B;
        vc = vct + (double)(half * kbar);
#pragma unroll
        for (int j = 0; j < B; ++j) dv[j] += half * (k[j] - kbar);
        update_centroid(xc);
        const float gap = w[1] - w[0];
        buf.E0c = buf.E0n;
        buf.E1c = buf.E1n;
        buf.Dc = buf.Dn;
        buf.E0n = w[0];
        buf.E1n = w[1];
        buf.Dn = nac * (float)vc;
        electronics2_sched(p, buf, step == 0, h, gap, sg);
        step += 1;

        const int s = state;
        float re = sg.x / (s == 0 ? sg.p : sg.q);
        float nsm = s == 0 ? nac : -nac;
        float prob = clamp01<float>(2.0f * (float)vc * re * nsm * dtf);
        float u = rng_uniform_f(p.seed, (uint64_t)gid, (uint32_t)step, RNG_HOP);
        if (prob > u) {
            const int ns = 1 - s;
            bool accept = true;
            if (p.rescaling != RESCALE_OFF) {
                double d = ns < s ? (double)nac : -(double)nac;
                double aa = d * d / mass / 2.0;
                double bb = d * vc;
                double cc = (double)w[ns] - (double)w[s];
                double disc = bb * bb - 4.0 * aa * cc;
                if (disc < 0.0) {
                    accept = false;
                    if (p.rescaling == RESCALE_VINVERSION) vc = -vc;  // only the centroid moves along d (1 DoF)
                } else {
                    double root = sqrt(disc);
                    double gamma = bb < 0.0 ? (bb + root) / (2.0 * aa) : (bb - root) / (2.0 * aa);
                    vc = vc - gamma * d / mass;
                }
            }
            if (accept) {
                rp_log_hop(p, i, nh, step, s, ns);
                nh += 1;
                state = ns;
            } else {
                nf += 1;
            }
        }
        if (p.terminate_x > 0.0 && fabs(xc) > p.terminate_x) break;
    }
    double x0 = 0.0;
#pragma unroll
    for (int j = 0; j < B; ++j) {
        double xj = xc + (double)dx[j];
        if (j == 0) x0 = xj;
        p.r[(int64_t)j * N + i] = xj;
        p.v[(int64_t)j * N + i] = vc + (double)dv[j];
    }
    const double e1 = p.energy ? rp_energy(state) : 0.0;
    rp_write_final<float>(p, i, sg, state, nh, nf, step, e0, e1, x0);
}

template <typename R, int B>
__device__ __forceinline__ void rpsh_traj(const RpshParams& p, int cls, int64_t i) {
    if constexpr (std::is_same<R, double>::value)
        rpsh_traj_plain<B>(p, cls, i);
    else
        rpsh_traj_fast<B>(p, cls, i);
}

// Persistent launch: refill-on-finish work queues per bead-count class.
template <typename R>
__global__ void __launch_bounds__(kRpshBlock) rpsh_persistent_kernel(const RpshParams p) {
    int cls = p.block_class[blockIdx.x];
    for (int visited = 0; visited < p.nclass;) {
        const int64_t begin = p.class_begin[cls], count = p.class_begin[cls + 1] - begin;
        unsigned long long idx = count > 0 ? atomicAdd(p.queue + cls, 1ull) : (unsigned long long)count;
        if ((int64_t)idx >= count) {  // class drained: help the next one
            cls = (cls + 1) % p.nclass;
            ++visited;
            continue;
        }
        const int64_t i = p.class_traj[begin + idx];
        switch (p.class_beads[cls]) {
            case 1: rpsh_traj<R, 1>(p, cls, i); break;
            case 2: rpsh_traj<R, 2>(p, cls, i); break;
            case 4: rpsh_traj<R, 4>(p, cls, i); break;
            case 5: rpsh_traj<R, 5>(p, cls, i); break;
            case 8: rpsh_traj<R, 8>(p, cls, i); break;
            case 10: rpsh_traj<R, 10>(p, cls, i); break;
            case 16: rpsh_traj<R, 16>(p, cls, i); break;
            case 32: rpsh_traj<R, 32>(p, cls, i); break;
            default: break;  // the host admits only the instantiated bead counts
        }
    }
}

template <typename R>
cudaError_t launch_rpsh(const RpshParams& p, int blocks, cudaStream_t s) {
    rpsh_persistent_kernel<R><<<blocks, kRpshBlock, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace nqcd
