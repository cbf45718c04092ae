// Ring-polymer surface hopping (RPSH) ensemble kernels, two-state Tully models.
//
// Reference algorithm (NQCDynamics.jl):
//   BCBwithTsit5.perform_step!   src/DynamicsMethods/IntegrationAlgorithms/bcb_electronics.jl:53-97
//   step_C! (Cayley free step)   src/DynamicsMethods/IntegrationAlgorithms/steps.jl:10-17
//   cayley_propagator            src/RingPolymers/ring_polymer.jl:71-82
//   RPSH rescaling / inversion   src/DynamicsMethods/SurfaceHoppingMethods/rpsh.jl:30-50
//   hopping with centroid data   SurfaceHoppingMethods.jl:81-103, fssh.jl:86-121
//   TerminatingCallback          src/DynamicsUtils/callbacks.jl:29
//
// Uneven ensembles: trajectories carry their own bead count (one of the
// instantiated counts 1, 2, 4, 5, 8, 10, 16, 32).  The host sorts them
// into bead-count classes; one persistent launch serves all classes.  A
// worker takes a trajectory from its class's atomic queue, integrates it
// until the termination test or the end time, then refills its slot with the
// next trajectory; when its class is drained it moves on to the other
// classes, so workers never idle while work is left.  The queues are plain
// atomic counters: there is no spin-wait anywhere.
//
//   plain path (rpsh_persistent_kernel): one thread per trajectory, FP64,
//               every operation in the CPU oracle's order (translation unit
//               built with -fmad=false): bit-identical.
//   fast path (rpsh_group_kernel): one lane per bead.  Bead coordinates are
//               split into the centroid (FP64) and deviations from it (FP32);
//               the free ring-polymer step, bead forces and the electronics
//               run in FP32.  Since the rescaling shifts every bead by the
//               same amount, hops change only the FP64 centroid velocity.
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
    const float4* circf[kRpshMaxClasses];   // fast path: per class [B] circulant free-step coefficients
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
    int32_t* fp64_steps;          // [ntraj] fast path: steps with FP64 electronics (gap below gap_fp64)
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
    R z0 = s == 0 ? Z[0] : Z[2], z1 = s == 0 ? Z[1] : Z[3];  // selects keep Z in registers
    R T0 = D[0] * z0 + D[1] * z1;
    R T1 = D[1] * z0 + D[2] * z1;
    R a = z0 * T0 + z1 * T1;
    if (ws) *ws = s == 0 ? w[0] : w[1];
    return -a / mass;
}

// Fast-path form: the same force with the reciprocal mass precomputed.
__device__ __forceinline__ float rp_bead_accel_f(int model, const float* mp, float x, int s, float inv_mass) {
    float V[3], D[3], w[2], Z[4];
    const float I2[4] = {1.f, 0.f, 0.f, 1.f};
    tully_potential<float>(model, mp, x, V);
    eigen2_phase<float>(V, I2, w, Z);
    tully_derivative<float>(model, mp, x, D);
    const float z0 = s == 0 ? Z[0] : Z[2], z1 = s == 0 ? Z[1] : Z[3];
    const float T0 = D[0] * z0 + D[1] * z1;
    const float T1 = D[1] * z0 + D[2] * z1;
    return -(z0 * T0 + z1 * T1) * inv_mass;
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
        // real(sigma[m, s] / sigma[s, s]) by Julia's complex division
        double re = cdiv_real(sg.x, s == 0 ? -sg.y : sg.y, s == 0 ? sg.p : sg.q, 0.0);
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
                double cc = ns == 1 ? w[1] - w[0] : w[0] - w[1];
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
// ---------------------------------------------------------------------------
// fast path: a group of GL lanes per trajectory, Q beads per lane
// ---------------------------------------------------------------------------
// A warp serves one bead-count class at a time, split into 32/GL groups of GL
// lanes; lane j of a group holds beads jQ .. jQ+Q-1 (B = GL Q exactly:
// B = 1, 2, 4, 8, 16, 32 -> GL = 1, 2, 4, 4, 4, 4; B = 5, 10 -> GL = 1, 2).
// The per-trajectory state (centroid position and velocity, electronic
// density matrix, active state, hop test) is computed redundantly by the GL
// lanes of the group and is bitwise the same on all of them: group sums are
// per-lane sums followed by xor butterflies, and at every level a lane and its
// partner add the same two operands.  Four lanes per trajectory keep the
// redundant electronics (five Tsit5 sub-steps per nuclear step) shared by
// eight trajectories per warp, while the bead work is split four ways.  The
// centroid is accumulated in Kahan-compensated FP32 (AccKahan): FP64
// arithmetic in the step (1/73 of the FP32 rate) would bound it.
//
// The free ring-polymer step acts on the bead deviations through the
// bead-space propagator M = sum_{k >= 1} u_k cay_k u_k^T (normal modes u_k,
// Cayley blocks cay_k; the centroid mode is left out exactly as in the
// normal-mode form, bcb_electronics.jl:67-71).  The cyclic ring's normal
// modes are Fourier modes whose degenerate pairs share one frequency, so M
// is circulant: M[b][m] = c[(b - m) mod B], four coefficient vectors
// (x<-x, x<-v, v<-x, v<-v) per class, computed on the host in FP64.  Lane j
// forms out[jQ + q] = sum_d c[d] in[jQ + q - d] by offsets d = d1 Q + d0:
// the inputs of one d1 are the bead blocks of lanes j - d1 and j - d1 - 1,
// so a step costs each lane GL block shuffles and 4 B Q multiply-adds.
//
// A group whose trajectory ends (termination test or end of the schedule)
// writes it out and takes the class queue's next trajectory before the next
// step; the warp moves to another class once every group found the queue
// empty.

struct RpLanes {
    int j, base;    // lane within the group, first lane of the group
    unsigned mask;  // the group's lanes
};

template <int GL, typename T>
__device__ __forceinline__ T rp_group_sum(const RpLanes& g, T x) {
#pragma unroll
    for (int off = GL >> 1; off > 0; off >>= 1) x += __shfl_xor_sync(g.mask, x, off);
    return x;
}

// State of the trajectory a group is integrating.
template <int Q>
struct RpTraj {
    int64_t i;
    AccKahan xc, vc;          // centroid
    float dx[Q], dv[Q], k[Q]; // this lane's beads: deviations from the centroid, accelerations
    float Zc[4], w[2], nac;
    Sig2<float> sg;
    EBuf<float> buf;
    int state, nh, nf, step, nfp64;
    double e0;
};

// Ring-polymer energy of the group's trajectory on state s (the plain path's
// rp_energy, summed over the group's beads).
template <int Q, int GL>
__device__ __forceinline__ double rp_group_energy(const RpshParams& p, const RpLanes& g, int model, const float* mp,
                                                  double xc, double vc, const float (&dx)[Q], const float (&dv)[Q],
                                                  int s) {
    constexpr int B = Q * GL;
    const double mass = p.mass;
    const float next = GL == 1 ? dx[0] : __shfl_sync(g.mask, dx[0], g.base + ((g.j + 1) & (GL - 1)));
    double spring = 0.0, ke = 0.0, pe = 0.0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const double d = (double)dx[q] - (double)(q + 1 < Q ? dx[q + 1] : next);
        if (B > 1) spring += mass * d * d;
        const double vj = vc + (double)dv[q];
        ke += mass * vj * vj;
        float ws;
        rp_bead_accel<float>(model, mp, (float)(xc + (double)dx[q]), s, (float)mass, &ws);
        pe += ws;
    }
    spring = rp_group_sum<GL>(g, spring);
    ke = rp_group_sum<GL>(g, ke);
    pe = rp_group_sum<GL>(g, pe);
    const double wn = B / p.beta;
    return spring * (wn * wn) / 2.0 + ke / 2.0 + pe;
}

template <int Q>
__device__ __forceinline__ void rp_update_centroid(int model, const float* mp, RpTraj<Q>& t) {
    float V[3], D[3], Zn[4], A[3];
    tully_potential<float>(model, mp, t.xc.f(), V);
    eigen2_phase<float>(V, t.Zc, t.w, Zn);
#pragma unroll
    for (int q = 0; q < 4; ++q) t.Zc[q] = Zn[q];
    tully_derivative<float>(model, mp, t.xc.f(), D);
    adiabatic_derivative2<float>(D, t.Zc, A);
    t.nac = A[1] / (t.w[1] - t.w[0]);
}

template <int Q, int GL>
__device__ __forceinline__ void rp_group_begin(const RpshParams& p, const RpLanes& g, int model, const float* mp,
                                               int64_t i, RpTraj<Q>& t) {
    constexpr int B = Q * GL;
    const int64_t N = p.ntraj;
    t.i = i;
    double r[Q], v[Q], sr = 0.0, sv = 0.0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        r[q] = p.r[(int64_t)(g.j * Q + q) * N + i];
        v[q] = p.v[(int64_t)(g.j * Q + q) * N + i];
        sr += r[q];
        sv += v[q];
    }
    const double xc = rp_group_sum<GL>(g, sr) / B, vc = rp_group_sum<GL>(g, sv) / B;
    t.xc.load(xc);
    t.vc.load(vc);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        t.dx[q] = (float)(r[q] - xc);
        t.dv[q] = (float)(v[q] - vc);
    }
    t.Zc[0] = 1.f;
    t.Zc[1] = 0.f;
    t.Zc[2] = 0.f;
    t.Zc[3] = 1.f;
    rp_update_centroid(model, mp, t);
    rp_init_sigma<float>(p, i, t.sg, t.state);
#pragma unroll
    for (int q = 0; q < Q; ++q)
        t.k[q] = rp_bead_accel_f(model, mp, (float)(xc + (double)t.dx[q]), t.state, (float)(1.0 / p.mass));
    t.e0 = p.energy ? rp_group_energy<Q, GL>(p, g, model, mp, xc, vc, t.dx, t.dv, t.state) : 0.0;
    t.buf = {0.f, 0.f, 0.f, 0.0, 0.f, 0.f, 0.f, 0.0};
    t.nh = t.nf = t.step = t.nfp64 = 0;
}

template <int Q, int GL>
__device__ __forceinline__ void rp_group_finish(const RpshParams& p, const RpLanes& g, int model, const float* mp,
                                                const RpTraj<Q>& t) {
    const int64_t N = p.ntraj;
    const double xc = t.xc.get(), vc = t.vc.get();
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        p.r[(int64_t)(g.j * Q + q) * N + t.i] = xc + (double)t.dx[q];
        p.v[(int64_t)(g.j * Q + q) * N + t.i] = vc + (double)t.dv[q];
    }
    const double x0 = __shfl_sync(g.mask, xc + (double)t.dx[0], g.base);
    const double e1 = p.energy ? rp_group_energy<Q, GL>(p, g, model, mp, xc, vc, t.dx, t.dv, t.state) : 0.0;
    if (g.j == 0) {
        rp_write_final<float>(p, t.i, t.sg, t.state, t.nh, t.nf, t.step, t.e0, e1, x0);
        if (p.fp64_steps) p.fp64_steps[t.i] = t.nfp64;
    }
}

// Free ring-polymer step of the deviations: (dx, dv) <- M (dx, dv), M circulant.
template <int Q, int GL>
__device__ __forceinline__ void rp_free_step(const RpLanes& g, const float4* __restrict__ circ, float (&dx)[Q],
                                             float (&dv)[Q]) {
    float nx[Q], nv[Q], ax[Q], av[Q], bx[Q], bv[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        nx[q] = nv[q] = 0.f;
        ax[q] = dx[q];
        av[q] = dv[q];
    }
#pragma unroll
    for (int d1 = 0; d1 < GL; ++d1) {
        // bead block of lane j - d1 - 1 (the wrap-around part of this d1's window)
        const int src = g.base + ((g.j - d1 - 1) & (GL - 1));
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            bx[q] = GL == 1 ? dx[q] : __shfl_sync(g.mask, dx[q], src);
            bv[q] = GL == 1 ? dv[q] : __shfl_sync(g.mask, dv[q], src);
        }
#pragma unroll
        for (int d0 = 0; d0 < Q; ++d0) {
            const float4 c = __ldg(circ + d1 * Q + d0);
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const float xs = q >= d0 ? ax[q - d0] : bx[Q + q - d0];
                const float vs = q >= d0 ? av[q - d0] : bv[Q + q - d0];
                nx[q] = fmaf(c.x, xs, fmaf(c.y, vs, nx[q]));
                nv[q] = fmaf(c.z, xs, fmaf(c.w, vs, nv[q]));
            }
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            ax[q] = bx[q];
            av[q] = bv[q];
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        dx[q] = nx[q];
        dv[q] = nv[q];
    }
}

// One step of the group's trajectory; returns true when it has ended.
template <int Q, int GL>
__device__ __forceinline__ bool rp_group_step(const RpshParams& p, const RpLanes& g, int model, const float* mp,
                                              const float4* __restrict__ circ, RpTraj<Q>& t) {
    constexpr float invB = 1.0f / (Q * GL);
    const float inv_mass = (float)(1.0 / p.mass);
    const int step = t.step;
    const float h = step == 0 ? p.h_first : (step + 1 == p.nsteps_total ? p.h_last : p.h_mid);
    const float half = 0.5f * h;
    // B kick: centroid and deviations
    float ks = 0.f;
#pragma unroll
    for (int q = 0; q < Q; ++q) ks += t.k[q];
    float kbar = rp_group_sum<GL>(g, ks) * invB;
    AccKahan vct = t.vc;
    vct.add(half * kbar);
#pragma unroll
    for (int q = 0; q < Q; ++q) t.dv[q] += half * (t.k[q] - kbar);
    // free ring polymer: centroid drifts, deviations through the circulant propagator
    t.xc.add(h * vct.f());
    rp_free_step<Q, GL>(g, circ, t.dx, t.dv);
    // bead forces, B kick
    const float xcf = t.xc.f();
    ks = 0.f;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        t.k[q] = rp_bead_accel_f(model, mp, xcf + t.dx[q], t.state, inv_mass);
        ks += t.k[q];
    }
    kbar = rp_group_sum<GL>(g, ks) * invB;
    t.vc = vct;
    t.vc.add(half * kbar);
#pragma unroll
    for (int q = 0; q < Q; ++q) t.dv[q] += half * (t.k[q] - kbar);
    rp_update_centroid(model, mp, t);
    const float gap = t.w[1] - t.w[0];
    t.buf.E0c = t.buf.E0n;
    t.buf.E1c = t.buf.E1n;
    t.buf.Dc = t.buf.Dn;
    t.buf.E0n = t.w[0];
    t.buf.E1n = t.w[1];
    t.buf.Dn = t.nac * t.vc.f();
    electronics2_sched(p, t.buf, step == 0, h, gap, t.sg, t.nfp64);
    t.step = step + 1;

    const int s = t.state;
    const float re = t.sg.x / (s == 0 ? t.sg.p : t.sg.q);
    const float nsm = s == 0 ? t.nac : -t.nac;
    const float prob = clamp01<float>(2.0f * t.vc.f() * re * nsm * (float)p.dt);
    const float u = rng_uniform_f(p.seed, (uint64_t)(p.traj_offset + t.i), (uint32_t)t.step, RNG_HOP);
    if (prob > u) {
        const int ns = 1 - s;
        bool accept = true;
        if (p.rescaling != RESCALE_OFF) {
            const double d = ns < s ? (double)t.nac : -(double)t.nac;
            const double aa = d * d / p.mass / 2.0;
            const double vc = t.vc.get();
            const double bb = d * vc;
            const double cc = ns == 0 ? (double)t.w[0] - (double)t.w[1] : (double)t.w[1] - (double)t.w[0];
            const double disc = bb * bb - 4.0 * aa * cc;
            if (disc < 0.0) {
                accept = false;
                if (p.rescaling == RESCALE_VINVERSION) {  // only the centroid moves along d (1 DoF)
                    t.vc.s = -t.vc.s;
                    t.vc.c = -t.vc.c;
                }
            } else {
                const double root = sqrt(disc);
                const double gamma = bb < 0.0 ? (bb + root) / (2.0 * aa) : (bb - root) / (2.0 * aa);
                t.vc.load(vc - gamma * d / p.mass);
            }
        }
        if (accept) {
            if (g.j == 0) rp_log_hop(p, t.i, t.nh, t.step, s, ns);
            t.nh += 1;
            t.state = ns;
        } else {
            t.nf += 1;
        }
    }
    return t.step >= p.nsteps_total || (p.terminate_x > 0.0 && fabsf(t.xc.f()) > (float)p.terminate_x);
}

// All trajectories of class cls, groups of GL lanes refilled from its queue.
template <int Q, int GL>
__device__ __forceinline__ void rp_serve_class(const RpshParams& p, int cls) {
    const int lane = threadIdx.x & 31;
    RpLanes g;
    g.j = lane & (GL - 1);
    g.base = lane & ~(GL - 1);
    g.mask = GL == 32 ? 0xffffffffu : ((1u << GL) - 1u) << g.base;
    const int model = p.class_model[cls];
    float mp[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) mp[q] = (float)p.class_mp[cls][q];
    const float4* circ = p.circf[cls];
    const int64_t begin = p.class_begin[cls], count = p.class_begin[cls + 1] - begin;
    RpTraj<Q> t;
    bool has = false, drained = count <= 0;
    while (true) {
        if (!has && !drained) {  // uniform within the group
            unsigned long long idx = 0ull;
            if (g.j == 0) idx = atomicAdd(p.queue + cls, 1ull);
            idx = __shfl_sync(g.mask, idx, g.base);
            if ((int64_t)idx < count) {
                rp_group_begin<Q, GL>(p, g, model, mp, p.class_traj[begin + (int64_t)idx], t);
                has = true;
            } else {
                drained = true;
            }
        }
        if (__all_sync(0xffffffffu, drained)) break;
        if (has && rp_group_step<Q, GL>(p, g, model, mp, circ, t)) {
            rp_group_finish<Q, GL>(p, g, model, mp, t);
            has = false;
        }
    }
}

// Persistent fast kernel of one bead count B = Q GL: warps over the classes
// with B beads (the Tully models), groups over their trajectories.  The
// shapes are separate kernels because one kernel holding all of them needs
// the register budget of the largest everywhere; the host launches them
// concurrently on forked streams (instantiated in the FP32 translation unit).
template <int Q, int GL>
__global__ void __launch_bounds__(kRpshBlock) rpsh_group_kernel(const RpshParams p) {
    int cls = p.block_class[blockIdx.x];
    for (int visited = 0; visited < p.nclass; ++visited, cls = (cls + 1) % p.nclass)
        if (p.class_beads[cls] == Q * GL) rp_serve_class<Q, GL>(p, cls);
}

// Plain path persistent launch: refill-on-finish work queues per bead-count
// class, one thread per trajectory (R = double, instantiated in the FP64
// translation unit only).
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
            case 1: rpsh_traj_plain<1>(p, cls, i); break;
            case 2: rpsh_traj_plain<2>(p, cls, i); break;
            case 4: rpsh_traj_plain<4>(p, cls, i); break;
            case 5: rpsh_traj_plain<5>(p, cls, i); break;
            case 8: rpsh_traj_plain<8>(p, cls, i); break;
            case 10: rpsh_traj_plain<10>(p, cls, i); break;
            case 16: rpsh_traj_plain<16>(p, cls, i); break;
            case 32: rpsh_traj_plain<32>(p, cls, i); break;
            default: break;  // the host admits only the instantiated bead counts
        }
    }
}

template <typename R>
cudaError_t launch_rpsh_plain(const RpshParams& p, int blocks, cudaStream_t s) {
    rpsh_persistent_kernel<R><<<blocks, kRpshBlock, 0, s>>>(p);
    return cudaGetLastError();
}

// Persistent grid of a lane-group kernel: SMs x resident blocks.
template <int Q, int GL>
int rpsh_group_grid_t() {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, rpsh_group_kernel<Q, GL>, kRpshBlock, 0);
    return sms * (per > 0 ? per : 1);
}

// Lane-group shapes: lanes = 0 takes the default of the bead count; another
// power of two dividing it (at most 32) selects that shape.  0 when no
// kernel exists for the shape.
int rpsh_group_grid(int beads, int lanes);
cudaError_t launch_rpsh_group(int beads, int lanes, const RpshParams& p, int blocks, cudaStream_t s);
int rpsh_group_grid_tuned(int beads, int lanes);
// One persistent launch serving every bead count (kernels_tune.cu).
int rpsh_one_launch_grid();
cudaError_t launch_rpsh_one(const RpshParams& p, int blocks, cudaStream_t s);
cudaError_t launch_rpsh_group_tuned(int beads, int lanes, const RpshParams& p, int blocks, cudaStream_t s);

// Lane-group shape (beads per lane Q, lanes per trajectory GL) of a bead count.
inline void rpsh_group_shape(int beads, int& Q, int& GL) {
    switch (beads) {
        case 1: Q = 1, GL = 1; break;
        case 2: Q = 1, GL = 2; break;
        case 5: Q = 5, GL = 1; break;
        case 10: Q = 5, GL = 2; break;
        default: Q = beads / 4, GL = 4; break;  // 4, 8, 16, 32
    }
}

}  // namespace nqcd
