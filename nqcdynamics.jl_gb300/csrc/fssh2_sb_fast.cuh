// Fast spin-boson FSSH kernel: G lanes per trajectory, bath modes in registers.
//
// The spin-boson Hamiltonian V = [[eps + c.R, Delta], [Delta, -eps - c.R]]
// + R^T W^2 R / 2 makes every per-mode quantity of the reference step a
// function of two group sums (c.R, R^T W^2 R) and of the 2x2 eigenvectors:
//   force on mode I on state s:  -(w_I^2 R_I + c_I M_ss) / m_I,
//     M = Z^T diag(1, -1) Z  (the common part of Z^T dH_I Z),
//   coupling d_I,01 = c_I M_01 / (E1 - E0),  so  D01 = (c.v) M_01 / gap,
//   hop probability and momentum rescaling need only c.v and
//   sum_I c_I^2 / m_I.
// So each of the G lanes of a trajectory integrates ceil(N/G) modes in
// registers, the group reduces three sums per step with shuffles, and all
// G lanes carry the identical 2x2 electronic problem (FP32 Tsit5, FP64 below
// the gap threshold).  Nothing per step touches HBM.
//
// Accumulation of positions and velocities (template Acc):
//   AccF64  FP64 accumulators (one DFMA per update),
//   AccKahan FP32 value + FP32 compensation (Kahan summation, four FP32 ops
//            per update), used because the FP64 pipe of this GPU runs at
//            1/73 of the FP32 rate (measured).
// Reference algorithm: fssh2_traj.h (same steps, same random stream).
#pragma once

#include <type_traits>

#include "fssh2_kernels.cuh"

namespace nqcd {

// AccF64 and AccKahan are defined in fssh2_kernels.cuh.

template <int G>
__device__ __forceinline__ float group_sum(float x) {
#pragma unroll
    for (int off = 1; off < G; off <<= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    return x;
}

constexpr int kSbFastBlock = 128;   // default threads per block
constexpr int kSbFastBlockMax = 256;
constexpr int kSbGroup = 4;         // default lanes per trajectory

// G lanes per trajectory (4, or 8 in the variants the autotuner may pick).
// Ehr = true: Ehrenfest (mean-field force from the density matrix, no
// hopping); a template parameter so that the surface-hopping instantiation
// keeps its register allocation.
template <typename Acc, int G, int NPL, bool Ehr>
__global__ void __launch_bounds__(kSbFastBlockMax) fssh2_sb_fast_kernel(const FsshParams p) {
    extern __shared__ float4 bath[];  // (c, w2, 1/m, c^2/m) per mode
    const int nd = p.ndof;
    for (int I = threadIdx.x; I < G * NPL; I += blockDim.x) {
        if (I < nd) {
            double m = p.mass[I];
            bath[I] = make_float4((float)p.bath_c[I], (float)p.bath_w2[I], (float)(1.0 / m),
                                  (float)(p.bath_c[I] * p.bath_c[I] / m));
        } else {
            bath[I] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    __syncthreads();

    // trajectories [0, traj_hi) of the (launch wrapper's shifted) per-trajectory arrays
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane_g = (int)(gt % G);
    const int64_t i0 = gt / G;
    const bool active = i0 < p.traj_hi;
    const int64_t i = active ? i0 : p.traj_hi - 1;  // (the launch's last trajectory: pointers may be shifted)
    const int64_t gid = p.traj_offset + i;
    const int64_t N = p.ntraj;
    const float eps = (float)p.mp[0], Delta = (float)p.mp[1];

    // this lane's modes: I = lane_g + G * j
    Acc r[NPL], v[NPL];
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        int I = lane_g + G * j;
        r[j].load(I < nd ? p.r[(int64_t)I * N + i] : 0.0);
        v[j].load(I < nd ? p.v[(int64_t)I * N + i] : 0.0);
    }

    float Z[4] = {1.f, 0.f, 0.f, 1.f};
    float w[2];
    float vmean = 0.f;  // eigenvalue mean (energies are shifted by it for the electronics)
    auto set_eigen = [&](float s0, float cr) {
        float V0 = 0.5f * s0;
        float Vs[3] = {(V0 + cr) + eps, Delta, (V0 - cr) - eps};
        float Zn[4];
        eigen2_phase<float>(Vs, Z, w, Zn);
#pragma unroll
        for (int q = 0; q < 4; ++q) Z[q] = Zn[q];
        vmean = V0;
    };

    float s0 = 0.f, cr = 0.f, ke = 0.f;
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        float4 b = bath[lane_g + G * j];
        float x = r[j].f(), vv = v[j].f();
        s0 += b.y * x * x;
        cr += b.x * x;
        ke += vv * vv / b.z;
    }
    s0 = group_sum<G>(s0);
    cr = group_sum<G>(cr);
    ke = group_sum<G>(ke);
    set_eigen(s0, cr);
    Sig2<float> sg;
    int state;
    init_electronics2<float>(p, i, gid, Z, sg, state);
    constexpr bool ehr = Ehr;
    // weight of the coupling force c_I in the cached force: M_ss (FSSH) or
    // sum_nm M_nm Re sigma_nm (Ehrenfest), M = Z^T sigma_z Z
    auto force_weight = [&]() {
        const float M00 = Z[0] * Z[0] - Z[1] * Z[1], M11 = Z[2] * Z[2] - Z[3] * Z[3];
        return ehr ? ehrenfest_weight<float>(M00, Z[0] * Z[2] - Z[1] * Z[3], M11, sg) : (state == 0 ? M00 : M11);
    };
    auto pot = [&]() { return ehr ? ehrenfest_potential<float>(sg, w) : (double)w[state]; };
    double e0 = 0.5 * (double)ke + pot();
    float Mk = force_weight();

    float pop0[2] = {0.f, 0.f};
    int isave = 0;
    const bool lead = lane_g == 0;
    if (p.save_stride > 0) {
        diabatic_pop2_f(sg, state, Z, pop0, ehr);
        warp_save_popcorr_f(p, isave++, active && lead, pop0, pop0);
    }

    EBuf<float> buf = {0.f, 0.f, 0.f, 0.0, 0.f, 0.f, 0.f, 0.0};
    int nh = 0, nf = 0, step = 0, nfp64 = 0;
    float cv = 0.f;
    float u_pack = 0.f;  // hop uniform of step (batch start + lane_g), see the hop test
    const float dtf = (float)p.dt;
    // the host's step schedule replaces the reference's FP64 clock (no FP64 in the loop)
    while (step < p.nsteps_total) {
        const float h = step == 0 ? p.h_first : (step + 1 == p.nsteps_total ? p.h_last : p.h_mid);
        const float half = 0.5f * h;
        // B (cached force) and A
        s0 = 0.f;
        cr = 0.f;
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
            float4 b = bath[lane_g + G * j];
            float x = r[j].f();
            const float mk = (b.y * x + b.x * Mk) * b.z;  // minus the force
            v[j].add_prod(-half, mk);
            r[j].add_prod(h, v[j].f());
            float xn = r[j].f();
            s0 += b.y * xn * xn;
            cr += b.x * xn;
        }
        s0 = group_sum<G>(s0);
        cr = group_sum<G>(cr);
        float Eold0 = w[0], Eold1 = w[1];
        (void)Eold0;
        (void)Eold1;
        set_eigen(s0, cr);
        const float gap = w[1] - w[0];
        const float M01 = Z[0] * Z[2] - Z[1] * Z[3];
        Mk = force_weight();
        // B with the new force; c.v
        cv = 0.f;
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
            float4 b = bath[lane_g + G * j];
            float x = r[j].f();
            const float mk = (b.y * x + b.x * Mk) * b.z;
            v[j].add_prod(-half, mk);
            cv += b.x * v[j].f();
        }
        cv = group_sum<G>(cv);
        const float dscale = __fdividef(M01, gap);  // d_I,01 = c_I * dscale
        buf.E0c = buf.E0n;
        buf.E1c = buf.E1n;
        buf.Dc = buf.Dn;
        buf.E0n = w[0] - vmean;
        buf.E1n = w[1] - vmean;
        buf.Dn = cv * dscale;
        electronics2_sched(p, buf, step == 0, h, gap, sg, nfp64);
        step += 1;

        // hop test (identical in all G lanes of the group)
        const int s = state;
        float re = __fdividef(sg.x, s == 0 ? sg.p : sg.q);
        float nsm = (s == 0 ? 1.0f : -1.0f) * cv * dscale;
        float prob = clamp01<float>(2.0f * re * nsm * dtf);
        // hop uniforms: every G steps lane g of the group draws the Philox block of step + g, and
        // a shuffle hands each step its own (the same values as one draw per step, a quarter of
        // the Philox work)
        const int kq = (step - 1) & (G - 1);
        if (kq == 0) u_pack = rng_uniform_f(p.seed, (uint64_t)gid, (uint32_t)(step + lane_g), RNG_HOP);
        const float u = __shfl_sync(0xffffffffu, u_pack, ((int)threadIdx.x & 31 & ~(G - 1)) | kq);
        if (!ehr && prob > u) {  // Ehrenfest: no hopping
            const int ns = 1 - s;
            const float sgn = ns < s ? 1.0f : -1.0f;  // d(new, old) = sgn * c_I * dscale
            bool accept = true;
            if (p.rescaling != RESCALE_OFF) {
                // rescale_velocity! (surface_hopping.jl:64-99) in FP32, the precision of this path:
                // a = |d|^2/(2m) summed, b = d.v, c = E_new - E_old, disc = b^2 - 4ac.  (FP64 here
                // cost about ten FP64-pipe instructions per warp and step on average: a warp takes
                // the branch whenever one of its eight trajectories attempts a hop.)
                const float aa = 0.5f * dscale * dscale * p.sum_c2_over_m_f;
                const float bb = sgn * dscale * cv;
                const float cc = w[ns] - w[s];
                const float disc = fmaf(bb, bb, -4.0f * aa * cc);
                if (disc < 0.f) {
                    accept = false;
                    if (p.rescaling == RESCALE_VINVERSION) {
                        // v -= 2 (v.n) n with n = d/|d|, |d|^2 = dscale^2 sum c^2; v.d = sgn dscale c.v
                        float c2 = 0.f;
                        for (int I = 0; I < nd; ++I) c2 = fmaf(bath[I].x, bath[I].x, c2);
                        const float coef = 2.0f * cv / c2;  // 2 (v.d) d_I / |d|^2 = coef * c_I
#pragma unroll
                        for (int j = 0; j < NPL; ++j) v[j].add(-coef * bath[lane_g + G * j].x);
                    }
                } else {
                    const float root = sqrtf(disc);
                    const float gamma = bb < 0.f ? (bb + root) / (2.0f * aa) : (bb - root) / (2.0f * aa);
                    const float coef = gamma * sgn * dscale;  // gamma d_I / m_I = coef c_I / m_I
#pragma unroll
                    for (int j = 0; j < NPL; ++j) {
                        float4 b = bath[lane_g + G * j];
                        v[j].add(-coef * b.x * b.z);
                    }
                }
            }
            if (accept) {
                log_hop(p, active && lead, i, nh, step, s, ns);
                nh += 1;
                state = ns;
            } else {
                nf += 1;
            }
        }
        // save points are the multiples of save_stride: a product, not an integer division per step
        if (p.save_stride > 0 && step == isave * p.save_stride) {
            float pop[2];
            diabatic_pop2_f(sg, state, Z, pop, ehr);
            warp_save_popcorr_f(p, isave++, active && lead, pop0, pop);
        }
    }

    // final state
    ke = 0.f;
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        float vv = v[j].f();
        ke += vv * vv / bath[lane_g + G * j].z;
    }
    ke = group_sum<G>(ke);
    if (!active) return;
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        int I = lane_g + G * j;
        if (I < nd) {
            p.r[(int64_t)I * N + i] = r[j].get();
            p.v[(int64_t)I * N + i] = v[j].get();
        }
    }
    if (!lead) return;
    if (p.fp64_steps) p.fp64_steps[i] = nfp64;
    write_sigma<float>(p, i, sg);
    p.state[i] = state;
    if (p.nhops) p.nhops[i] = nh;
    if (p.nfrustrated) p.nfrustrated[i] = nf;
    if (p.nsteps) p.nsteps[i] = step;
    if (p.energy) {
        p.energy[i] = e0;
        p.energy[N + i] = 0.5 * (double)ke + pot();
    }
    if (p.scatter) atomicAdd(p.scatter + (p.r[i] > 0.0 ? 2 : 0) + state, 1ull);
}

template <typename Acc, int G, int NPL>
cudaError_t launch_sb_fast_npl(const FsshParams& p0, cudaStream_t s) {
    FsshParams p = p0;
    const int block = p.sb_block > 0 ? p.sb_block : kSbFastBlock;
    const int64_t lo = p.traj_lo, n = p.traj_hi - p.traj_lo;
    if ((lo * G) % block != 0 || p.traj_hi > p.ntraj || n < 0) return cudaErrorInvalidValue;
    if (lo > 0) {
        // trajectories [lo, traj_hi): every per-trajectory array (stride ntraj) from column lo, the
        // random stream from trajectory traj_offset + lo, the partial sums from the launch's first
        // warp row (lo is a whole number of blocks: each warp keeps its trajectories and its row)
        p.r += lo;
        p.v += lo;
        p.sigma += lo;
        p.state += lo;
        if (p.nhops) p.nhops += lo;
        if (p.nfrustrated) p.nfrustrated += lo;
        if (p.nsteps) p.nsteps += lo;
        if (p.hop_log) p.hop_log += lo;
        if (p.energy) p.energy += lo;
        if (p.fp64_steps) p.fp64_steps += lo;
        if (p.popcorr_partial)  // rows of nsave float4
            p.popcorr_partial = reinterpret_cast<double*>(reinterpret_cast<float4*>(p.popcorr_partial) +
                                                          lo * G / 32 * (int64_t)p.nsave);
        p.traj_offset += lo;
        p.traj_lo = 0;
        p.traj_hi = n;
    }
    int64_t threads = n * G;
    int64_t blocks = (threads + block - 1) / block;
    if (blocks == 0) return cudaSuccess;
    size_t shmem = sizeof(float4) * G * NPL;
    if (p.ehrenfest)
        fssh2_sb_fast_kernel<Acc, G, NPL, true><<<(unsigned)blocks, block, shmem, s>>>(p);
    else
        fssh2_sb_fast_kernel<Acc, G, NPL, false><<<(unsigned)blocks, block, shmem, s>>>(p);
    return cudaGetLastError();
}

// Lane group of 8 (Kahan accumulators), instantiated in their own translation unit.
cudaError_t launch_sb_fast_g8_kahan(const FsshParams& p, cudaStream_t s);

// modes per lane rounded up to an instantiated size
template <typename Acc>
cudaError_t launch_sb_fast(const FsshParams& p, cudaStream_t s) {
    if (p.ntraj <= 0 || p.traj_hi <= p.traj_lo) return cudaSuccess;
    if (p.sb_group == 8) {
        if constexpr (std::is_same<Acc, AccKahan>::value) return launch_sb_fast_g8_kahan(p, s);
        return cudaErrorInvalidValue;
    }
    int need = (p.ndof + kSbGroup - 1) / kSbGroup;
    if (need <= 1) return launch_sb_fast_npl<Acc, 4, 1>(p, s);
    if (need <= 2) return launch_sb_fast_npl<Acc, 4, 2>(p, s);
    if (need <= 4) return launch_sb_fast_npl<Acc, 4, 4>(p, s);
    if (need <= 8) return launch_sb_fast_npl<Acc, 4, 8>(p, s);
    if (need <= 16) return launch_sb_fast_npl<Acc, 4, 16>(p, s);
    if (need <= 25) return launch_sb_fast_npl<Acc, 4, 25>(p, s);
    if (need <= 32) return launch_sb_fast_npl<Acc, 4, 32>(p, s);
    if (need <= 64) return launch_sb_fast_npl<Acc, 4, 64>(p, s);
    return cudaErrorInvalidValue;
}

}  // namespace nqcd
