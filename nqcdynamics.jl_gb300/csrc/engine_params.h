// Launch parameters of the ensemble kernels (device pointers only).
// Layout in HBM: structure-of-arrays with the trajectory index fastest, so
// that consecutive threads (one trajectory each) touch consecutive words.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace nqcd {

struct FsshParams {
    // model
    int32_t model;
    double mp[8];
    int32_t ndof;             // degrees of freedom per trajectory (spin-boson: bath modes)
    const double* mass;       // [ndof]
    const double* bath_c;     // [ndof] (spin-boson)
    const double* bath_w2;    // [ndof] (spin-boson)
    double sum_c2_over_m;     // sum_j c_j^2 / m_j (spin-boson fast path)
    float sum_c2_over_m_f;    // the same in FP32 (the fast kernel's hop rescaling)
    // method
    int32_t rescaling;
    int32_t ehrenfest;        // 1: Ehrenfest (mean-field force from sigma, no hopping), 0: FSSH
    int32_t init_kind;
    int32_t init_state;
    float gap_fp64;           // fast path: FP64 electronics below this adiabatic gap
    // run
    int64_t ntraj;
    int64_t traj_offset;
    double t0, t1, dt;
    // step schedule of [t0, t1] (the reference integrator's: steps of dt, a
    // shorter last step, times snapped to t1), precomputed on the host for the
    // fast kernels, which keep no FP64 clock
    int32_t nsteps_total;
    float h_first, h_mid, h_last;  // step lengths: first, interior, last
    float sa1, sb1;                // first step's interpolation weights (the buffer starts at t = 0)
    float dtsub;                   // Tsit5 sub-step dt/5 (FP32)
    uint64_t seed;
    int32_t save_stride;
    int32_t nsave;
    int32_t max_hops;
    // state, SoA [component][ntraj]
    double* r;                // [ndof][ntraj]
    double* v;                // [ndof][ntraj]
    double* scratch;          // plain spin-boson: per-DoF couplings [ndof][ntraj]
    double* sigma;            // [8][ntraj]
    int32_t* state;           // [ntraj]
    // outputs
    int32_t* nhops;           // [ntraj]
    int32_t* nfrustrated;     // [ntraj]
    int32_t* nsteps;          // [ntraj]
    int32_t* hop_log;         // [max_hops][3][ntraj]
    double* energy;           // [2][ntraj]
    double* popcorr_partial;  // [nwarps][nsave][4] doubles (plain paths) or floats (fast paths)
    unsigned long long* scatter;  // [4]
    int32_t* fp64_steps;      // [ntraj] fast paths: steps whose electronics ran in FP64 (gap below gap_fp64)
    // launch shape of the fast spin-boson kernel (nqcd_set_mapping; 0 = default)
    int32_t sb_group;         // lanes per trajectory: 4 or 8
    int32_t sb_block;         // threads per block: 64, 128 or 256
    // trajectories [traj_lo, traj_hi) of this launch (the fast spin-boson kernel; the others run
    // [0, ntraj)); traj_lo is a whole number of blocks, so that every warp keeps the trajectories
    // and the partial-sum row it has in a launch of all of them.  The launch wrapper shifts the
    // per-trajectory pointers by traj_lo: the kernel sees trajectories [0, traj_hi).
    int64_t traj_lo, traj_hi;
};

// Host launchers (one translation unit per precision).
cudaError_t launch_fssh2_fp64(const FsshParams& p, cudaStream_t s);
cudaError_t launch_fssh2_fp32(const FsshParams& p, cudaStream_t s);
cudaError_t launch_fssh2_fp32_kahan(const FsshParams& p, cudaStream_t s);

// Threads per trajectory of the kernel that runs (model, precision): the
// fast spin-boson kernel spreads the bath over a group of sb_group lanes (4
// unless the mapping says 8).
inline int fssh2_lanes_per_traj(int model, int precision, int sb_group = 4) {
    return (model == 10 /* MODEL_SPINBOSON */ && precision != 0 /* FP64 */) ? (sb_group == 8 ? 8 : 4) : 1;
}
// out[k] = sum over rows p of partial[p][k], deterministic: rows are summed in
// fixed chunks in parallel (tmp: [reduce_chunks(nparts, width)][width]) and the
// chunk sums in ascending order.
int64_t reduce_chunks(int64_t nparts, int64_t width);
cudaError_t launch_reduce_partials(const float* partial, int64_t nparts, int64_t width, double* tmp, double* out,
                                   cudaStream_t s);
cudaError_t launch_reduce_partials(const double* partial, int64_t nparts, int64_t width, double* tmp, double* out,
                                   cudaStream_t s);

}  // namespace nqcd
