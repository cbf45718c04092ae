// C ABI of the GB300 ensemble trajectory engine (declarations and contract:
// include/nqcd_gpu.h).  Host-side runtime: handle and device-memory
// ownership, host<->device staging with layout gathers, kernel dispatch,
// deterministic reductions and CUDA-event timing on the engine stream.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <chrono>
#include <new>
#include <string>
#include <algorithm>
#include <vector>

#include "../../include/nqcd_gpu.h"
#include "engine_params.h"
#include "nqcd_math.h"
#include "nqcd_models.h"
#include "mlp.h"
#include "ring_polymer.h"
#include "rpsh_kernels.cuh"
#include "iesh_kernels.cuh"

using namespace nqcd;

namespace nqcd {
int rpsh_grid_fp64();
cudaError_t launch_rpsh_fp64(const RpshParams& p, int blocks, cudaStream_t s);
cudaError_t launch_mdef_fp64(const MdefParams& p, cudaStream_t s);
cudaError_t launch_mdef_fp32(const MdefParams& p, cudaStream_t s);
cudaError_t launch_iesh_fp64(const IeshParams& p, cudaStream_t s);
cudaError_t launch_iesh_fp32(const IeshParams& p, cudaStream_t s);
}  // namespace nqcd

namespace {

// bead counts with an instantiated ring-polymer kernel
constexpr int kRpCounts[] = {1, 2, 4, 5, 8, 10, 16, 32};
constexpr int kNumRpCounts = 8;
// nqcd_run_host: host initial conditions in this many chunks (fewer for small ensembles)
constexpr int kPipeChunks = 8;
constexpr int kMaxRpGrid = 8192;

thread_local std::string g_create_error;

// ---------------------------------------------------------------------------
// Small device kernels: layout gathers and reductions
// ---------------------------------------------------------------------------

// AoS [n][m] -> SoA [m][n] (doubles), through a shared-memory tile so that
// both the read and the write are coalesced.
__global__ void transpose_kernel(const double* __restrict__ in, double* __restrict__ out, int64_t n, int64_t m) {
    __shared__ double tile[32][33];
    int64_t bx = (int64_t)blockIdx.x * 32, by = (int64_t)blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        int64_t row = by + j, col = bx + threadIdx.x;
        if (row < n && col < m) tile[j][threadIdx.x] = in[row * m + col];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        int64_t row = bx + j, col = by + threadIdx.x;  // out[row][col], row < m, col < n
        if (row < m && col < n) out[row * n + col] = tile[threadIdx.x][j];
    }
}

cudaError_t transpose(const double* in, double* out, int64_t n, int64_t m, cudaStream_t s) {
    if (n == 0 || m == 0) return cudaSuccess;
    dim3 block(32, 8);
    dim3 grid((unsigned)((m + 31) / 32), (unsigned)((n + 31) / 32));
    transpose_kernel<<<grid, block, 0, s>>>(in, out, n, m);
    return cudaGetLastError();
}

// Rows [0, n) of the row-major n x m block `in` into columns of two column-major arrays with
// leading dimension ld: out1[c * ld + r] = out2[c * ld + r] = in[r * m + c] (a chunk of
// trajectories from the host layout into the initial and the working state at once).
__global__ void transpose2_kernel(const double* __restrict__ in, double* __restrict__ out1, double* __restrict__ out2,
                                  int64_t n, int64_t m, int64_t ld) {
    __shared__ double tile[32][33];
    int64_t bx = (int64_t)blockIdx.x * 32, by = (int64_t)blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        int64_t row = by + j, col = bx + threadIdx.x;
        if (row < n && col < m) tile[j][threadIdx.x] = in[row * m + col];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        int64_t row = bx + j, col = by + threadIdx.x;  // out[row][col], row < m, col < n
        if (row < m && col < n) {
            const double x = tile[threadIdx.x][j];
            out1[row * ld + col] = x;
            out2[row * ld + col] = x;
        }
    }
}

cudaError_t transpose2(const double* in, double* out1, double* out2, int64_t n, int64_t m, int64_t ld, cudaStream_t s) {
    if (n == 0 || m == 0) return cudaSuccess;
    dim3 block(32, 8);
    dim3 grid((unsigned)((m + 31) / 32), (unsigned)((n + 31) / 32));
    transpose2_kernel<<<grid, block, 0, s>>>(in, out1, out2, n, m, ld);
    return cudaGetLastError();
}

__global__ void fill_i32_kernel(int32_t* p, int64_t n, int32_t v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// tmp[c][k] = sum of partial[p][k] over the rows p of chunk c, ascending p.
template <typename T>
__global__ void reduce_chunks_kernel(const T* __restrict__ partial, int64_t nparts, int64_t width,
                                     int64_t rows_per_chunk, double* __restrict__ tmp) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= width) return;
    const int64_t p0 = (int64_t)blockIdx.y * rows_per_chunk;
    const int64_t p1 = p0 + rows_per_chunk < nparts ? p0 + rows_per_chunk : nparts;
    double acc = 0.0;
    for (int64_t q = p0; q < p1; ++q) acc += (double)partial[q * width + k];
    tmp[(int64_t)blockIdx.y * width + k] = acc;
}

// out[k] = sum_p partial[p][k] in ascending p (deterministic).
__global__ void reduce_partials_kernel(const double* __restrict__ partial, int64_t nparts, int64_t width,
                                       double* __restrict__ out) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= width) return;
    double acc = 0.0;
    for (int64_t p = 0; p < nparts; ++p) acc += partial[p * width + k];
    out[k] = acc;
}

// Ehrenfest state-resolved scattering (OutputStateResolvedScattering1D with
// the adiabatic populations diag(Re sigma), ehrenfest.jl:74-77): per
// trajectory (reflected p, reflected q, transmitted p, transmitted q), summed
// afterwards by the fixed-order partial reduction.
__global__ void ehrenfest_scatter_kernel(const double* __restrict__ r, const double* __restrict__ sigma, int64_t n,
                                         double* __restrict__ part) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const bool tr = r[i] > 0.0;
        const double p0 = sigma[i], p1 = sigma[6 * n + i];
        part[4 * i + 0] = tr ? 0.0 : p0;
        part[4 * i + 1] = tr ? 0.0 : p1;
        part[4 * i + 2] = tr ? p0 : 0.0;
        part[4 * i + 3] = tr ? p1 : 0.0;
    }
}

// Device-side initial conditions (nqcd_sample_initial): entry q of the
// [2][ndof][n] grid is (position|velocity, degree of freedom d, trajectory t),
// drawn from its own Philox block; written to the SoA initial-condition arrays.
// Uniform draws use explicitly rounded operations so that they equal the
// documented formula bit for bit.
__global__ void sample_initial_kernel(const nqcd_sampler* __restrict__ tab, int ndof, int64_t n, int64_t offset,
                                      uint64_t seed, double* __restrict__ r0, double* __restrict__ v0) {
    const int64_t total = 2 * (int64_t)ndof * n;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = q % n, rest = q / n;
        const int d = (int)(rest % ndof), which = (int)(rest / ndof);
        const nqcd_sampler sp = tab[which * ndof + d];
        double x = sp.a;
        if (sp.kind != NQCD_SAMPLE_FIXED) {
            const u32x4 w = rng_block(seed, (uint64_t)(offset + t), (uint32_t)d, which ? RNG_INIT_VELOCITY : RNG_INIT_POSITION);
            const double u = u01_from_words(w.x, w.y);
            if (sp.kind == NQCD_SAMPLE_UNIFORM) {
                x = __dadd_rn(sp.a, __dmul_rn(__dsub_rn(sp.b, sp.a), u));
            } else {
                const double g = sqrt(-2.0 * log(1.0 - u)) * cos(6.283185307179586 * u01_from_words(w.z, w.w));
                x = __dadd_rn(sp.a, __dmul_rn(sp.b, g));
            }
        }
        (which ? v0 : r0)[(int64_t)d * n + t] = x;
    }
}

// Run statistics: steps, hops, frustrated hops, non-finite trajectories.
__global__ void stats_kernel(const int32_t* nsteps, const int32_t* nhops, const int32_t* nfrust,
                             const double* r, const double* v, int64_t ndof, int64_t ntraj,
                             unsigned long long* out, const int32_t* fp64_steps, unsigned long long* out_fp64) {
    unsigned long long a = 0, b = 0, c = 0, d = 0, e = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ntraj; i += (int64_t)gridDim.x * blockDim.x) {
        if (fp64_steps) e += (unsigned long long)fp64_steps[i];
        a += (unsigned long long)nsteps[i];
        b += (unsigned long long)nhops[i];
        c += (unsigned long long)nfrust[i];
        bool bad = false;
        for (int64_t I = 0; I < ndof; ++I) bad |= !isfinite(r[I * ntraj + i]) || !isfinite(v[I * ntraj + i]);
        d += bad ? 1ull : 0ull;
    }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
        c += __shfl_xor_sync(0xffffffffu, c, off);
        d += __shfl_xor_sync(0xffffffffu, d, off);
        e += __shfl_xor_sync(0xffffffffu, e, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out + 0, a);
        atomicAdd(out + 1, b);
        atomicAdd(out + 2, c);
        atomicAdd(out + 3, d);
        if (fp64_steps) atomicAdd(out_fp64, e);
    }
}

// Per-trajectory status: 1 where a final position or velocity is not finite.
__global__ void nonfinite_kernel(const double* r, const double* v, int64_t ndof, int64_t ntraj, int32_t* flag) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ntraj; i += (int64_t)gridDim.x * blockDim.x) {
        bool bad = false;
        for (int64_t I = 0; I < ndof; ++I) bad |= !isfinite(r[I * ntraj + i]) || !isfinite(v[I * ntraj + i]);
        flag[i] = bad ? 1 : 0;
    }
}

// FMA throughput probe: 8 independent chains per thread, register resident.
template <typename T>
__global__ void fma_peak_kernel(T* sink, int iters, T seed) {
    T a0 = seed + (T)threadIdx.x, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
    T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
    const T b = (T)0.999999, c = (T)1e-7;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fma(a0, b, c);
            a1 = fma(a1, b, c);
            a2 = fma(a2, b, c);
            a3 = fma(a3, b, c);
            a4 = fma(a4, b, c);
            a5 = fma(a5, b, c);
            a6 = fma(a6, b, c);
            a7 = fma(a7, b, c);
        }
    }
    T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == (T)-12345.0) sink[threadIdx.x] = s;  // never true; keeps the chains live
}

}  // namespace

// ---------------------------------------------------------------------------
// Handle
// ---------------------------------------------------------------------------
struct nqcd_handle {
    nqcd_config cfg;
    nqcd_mapping map = {};  // launch shapes (nqcd_set_mapping); zeros: defaults
    std::string err;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
    // fast ring polymers: one stream per bead-count kernel, forked from and joined to `stream`
    cudaStream_t rp_streams[kNumRpCounts] = {nullptr};
    cudaEvent_t rp_fork = nullptr, rp_join[kNumRpCounts] = {nullptr};
    // nqcd_run_host: a copy stream, two compute streams and their events (created on first use)
    cudaStream_t pipe_copy = nullptr, pipe_run[2] = {nullptr, nullptr};
    cudaEvent_t pipe_start = nullptr, pipe_ready[kPipeChunks] = {nullptr}, pipe_done[2] = {nullptr, nullptr};
    int64_t cap = 0;
    int64_t ntraj = 0;
    int64_t ndof = 0;  // per trajectory (ndofs * natoms)
    int nstates = 2;
    std::vector<double> params;
    double mass0 = 0.0;  // mass of the first atom (ring polymers: the one atom)
    double sum_c2_over_m = 0.0;
    bool initial_set = false;
    bool has_run = false;
    int32_t nsave_last = 0;
    // device buffers
    double *d_mass = nullptr, *d_bath_c = nullptr, *d_bath_w2 = nullptr;
    double *d_r0 = nullptr, *d_v0 = nullptr, *d_r = nullptr, *d_v = nullptr;
    double *d_sig0 = nullptr, *d_sig = nullptr;
    int32_t *d_state0 = nullptr, *d_state = nullptr;
    double* d_scratch = nullptr;
    int32_t *d_nhops = nullptr, *d_nfrust = nullptr, *d_nsteps = nullptr, *d_hoplog = nullptr;
    double* d_energy = nullptr;
    double* d_partial = nullptr;
    int64_t partial_cap = 0;
    double* d_redtmp = nullptr;  // chunk sums of the partial reduction
    int64_t redtmp_cap = 0;
    double* d_popcorr = nullptr;
    unsigned long long* d_counts = nullptr;  // [0..3] scatter, [4..7] stats, [8..11] method counters,
                                             // [12] FP64-electronics steps, [13] IESH overlap LUs,
                                             // [16..19] surrogate judge
    double* d_stage = nullptr;               // staging for layout gathers
    int64_t stage_cap = 0;
    // ring polymers: normal-mode tables per instantiated bead count, bead-count classes
    int64_t rp_U_off[kNumRpCounts] = {0};
    double *d_rpU = nullptr, *d_rpcay = nullptr;
    float* d_rpcirc = nullptr;  // fast path: circulant free-step coefficients, [count][32][4]
    int32_t *d_nbeads = nullptr, *d_class_traj = nullptr, *d_block_class = nullptr;
    unsigned long long* d_queue = nullptr;
    int32_t* d_fp64steps = nullptr;  // two-state methods: per trajectory, steps with FP64 electronics
    double* d_rptab = nullptr;       // ring-polymer MDEF / IESH: normal-mode matrix [n*n] and Cayley steps [n][4]
    int rp_beads = 1;                // ring-polymer MDEF / IESH: beads of every trajectory (1 otherwise)
    double* d_rpscratch = nullptr;  // plain path bead arrays, grown on demand
    int64_t rpscratch_cap = 0;
    int nclass = 0;
    int class_beads[kRpshMaxClasses] = {0};
    int class_slot[kRpshMaxClasses] = {0};  // index into kRpCounts
    int class_model[kRpshMaxClasses] = {0};
    int64_t class_begin[kRpshMaxClasses + 1] = {0};
    std::vector<int32_t> traj_beads, traj_models;  // host copies (ring polymers)
    std::vector<float> traj_speed;                 // |initial centroid velocity| (host initial conditions only)
    // MDEF: bath levels and squared couplings; friction surrogate
    double *d_eps = nullptr, *d_V2 = nullptr;
    MlpState mlp;
    // IESH: occupations [nelec][traj] (given initial, final) and final orbitals [traj][nelec][nstates]
    int32_t *d_occ0 = nullptr, *d_occ = nullptr;
    double *d_psi_re = nullptr, *d_psi_im = nullptr;
    int nelec = 0;
    double sumV2 = 0.0;
};

namespace {

int fail(nqcd_handle* h, int code, const std::string& msg) {
    if (h)
        h->err = msg;
    else
        g_create_error = msg;
    return code;
}

int cuda_fail(nqcd_handle* h, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return fail(h, e == cudaErrorMemoryAllocation ? NQCD_ERR_OOM : NQCD_ERR_CUDA, m);
}

#define NQCD_CUDA(h, call)                                 \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
    } while (0)

template <typename T>
cudaError_t dalloc(T** p, int64_t n) {
    if (n <= 0) n = 1;
    return cudaMalloc((void**)p, (size_t)n * sizeof(T));
}

void free_all(nqcd_handle* h) {
    void* ptrs[] = {h->d_mass, h->d_bath_c, h->d_bath_w2, h->d_r0, h->d_v0, h->d_r, h->d_v, h->d_sig0,
                    h->d_sig, h->d_state0, h->d_state, h->d_scratch, h->d_nhops, h->d_nfrust, h->d_nsteps,
                    h->d_hoplog, h->d_energy, h->d_partial, h->d_popcorr, h->d_counts, h->d_stage,
                    h->d_rpU, h->d_rpcay, h->d_rpcirc, h->d_nbeads, h->d_class_traj,
                    h->d_block_class, h->d_queue, h->d_rpscratch, h->d_eps, h->d_V2, h->d_rptab,
                    h->d_occ0, h->d_occ, h->d_psi_re, h->d_psi_im, h->d_redtmp, h->d_fp64steps};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    mlp_free(h->mlp);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->evk0) cudaEventDestroy(h->evk0);
    if (h->evk1) cudaEventDestroy(h->evk1);
    for (int c = 0; c < kNumRpCounts; ++c) {
        if (h->rp_streams[c]) cudaStreamDestroy(h->rp_streams[c]);
        if (h->rp_join[c]) cudaEventDestroy(h->rp_join[c]);
    }
    if (h->rp_fork) cudaEventDestroy(h->rp_fork);
    if (h->pipe_start) cudaEventDestroy(h->pipe_start);
    for (int c = 0; c < kPipeChunks; ++c)
        if (h->pipe_ready[c]) cudaEventDestroy(h->pipe_ready[c]);
    for (int k = 0; k < 2; ++k) {
        if (h->pipe_done[k]) cudaEventDestroy(h->pipe_done[k]);
        if (h->pipe_run[k]) cudaStreamDestroy(h->pipe_run[k]);
    }
    if (h->pipe_copy) cudaStreamDestroy(h->pipe_copy);
    if (h->stream) cudaStreamDestroy(h->stream);
}

int ensure_stage(nqcd_handle* h, int64_t n) {
    if (n <= h->stage_cap) return NQCD_OK;
    if (h->d_stage) cudaFree(h->d_stage);
    h->d_stage = nullptr;
    h->stage_cap = 0;
    NQCD_CUDA(h, dalloc(&h->d_stage, n));
    h->stage_cap = n;
    return NQCD_OK;
}

// Steps of the reference's clock from t0 to t1 (whole steps of dt, a
// shortened last step, a time within 100 ulp of t1 snapped to t1).  The count
// stops at (t1 - t0) / dt + 2, which only a clock that no longer advances (dt
// below the spacing of doubles near t) reaches; the caller rejects it.
int64_t count_steps(double t0, double t1, double dt) {
    int64_t n = 0;
    double t = t0;
    const int64_t cap = (int64_t)((t1 - t0) / dt) + 2;
    while (t < t1 && n <= cap) {
        double hh = (t1 - t) < dt ? (t1 - t) : dt;
        t = snap_time(t + hh, t1);
        ++n;
    }
    return n;
}

// Lanes per trajectory of the fast ring-polymer kernel of a bead count under
// the handle's mapping (0: the default shape).
int rp_lanes_of(const nqcd_handle* h, int beads) {
    switch (beads) {
        case 4: return h->map.rp_lanes[0];
        case 8: return h->map.rp_lanes[1];
        case 16: return h->map.rp_lanes[2];
        case 32: return h->map.rp_lanes[3];
        default: return 0;
    }
}

// MDEF launch parameters of a handle (device pointers of the handle).
MdefParams mdef_params(nqcd_handle* h, int64_t N, double dt, int32_t nsteps, uint64_t seed, int stride, int nsave) {
    MdefParams m;
    memset(&m, 0, sizeof(m));
    m.nbath = h->cfg.nbath;
    m.eps = h->d_eps;
    m.V2 = h->d_V2;
    if (h->cfg.model == NQCD_MODEL_NEWNS_ANDERSON_3D) {
        m.model3d = 1;
        m.kxy = h->params[0];
        m.A = h->params[1];
        m.a = h->params[2];
        m.delta = h->params[3];
        m.B = h->params[4];
        m.b = h->params[5];
        m.mu = h->params[6];
        m.sigma = h->params[7];
    } else {
        m.k = h->params[0];
        m.g = h->params[1];
        m.delta = h->params[2];
        m.mu = h->params[3];
        m.sigma = h->params[4];
    }
    m.beta = h->cfg.beta;
    m.mass = h->mass0;
    m.ntraj = N;
    m.traj_offset = h->cfg.traj_offset;
    m.dt = dt;
    m.h_last = dt;
    m.nsteps = nsteps;
    m.seed = seed;
    m.save_stride = stride;
    m.nsave = nsave;
    m.use_mlp = (h->cfg.use_friction_surrogate && h->cfg.precision != NQCD_PREC_FP64) ? 1 : 0;
    m.exact_friction_every = h->cfg.exact_friction_every;
    m.judge_tol = h->cfg.surrogate_tolerance > 0.0 ? h->cfg.surrogate_tolerance : 0.1;
    m.mlp = mlp_view(h->mlp);
    m.x = h->d_r;
    m.v = h->d_v;
    m.energy = h->d_energy;
    m.obs_partial = h->d_partial;
    m.counters = h->d_counts + 8;
    return m;
}

}  // namespace

extern "C" {

int nqcd_version(void) { return NQCD_ABI_VERSION; }

int nqcd_create(const nqcd_config* cfg, nqcd_handle** out) {
    if (!cfg || !out) return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: null argument");
    *out = nullptr;
    if (cfg->method != NQCD_METHOD_FSSH && cfg->method != NQCD_METHOD_RPSH && cfg->method != NQCD_METHOD_MDEF &&
        cfg->method != NQCD_METHOD_IESH && cfg->method != NQCD_METHOD_EHRENFEST &&
        cfg->method != NQCD_METHOD_EHRENFEST_NA)
        return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: method not supported by this build");
    const bool rp = cfg->method == NQCD_METHOD_RPSH;
    const bool mdef = cfg->method == NQCD_METHOD_MDEF;
    // EhrenfestNA runs in the IESH kernel (same model, integrator and initial orbitals)
    const bool iesh = cfg->method == NQCD_METHOD_IESH || cfg->method == NQCD_METHOD_EHRENFEST_NA;
    const int model = cfg->model;
    if (iesh) {
        if (model != NQCD_MODEL_NEWNS_ANDERSON_3D)
            return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: IESH runs on the three-dimensional Newns-Anderson model");
        if (cfg->natoms != 1 || cfg->ndofs != 3)
            return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: IESH runs one atom with three degrees of freedom");
        if (cfg->nbath < 2 || !cfg->bath_a || !cfg->bath_b)
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: IESH needs bath levels and couplings");
        if (cfg->nstates != cfg->nbath + 1 || cfg->nstates > kIeshMaxStates)
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: IESH needs nstates == nbath + 1 <= 128");
        for (int k = 1; k < cfg->nbath; ++k)
            if (!(cfg->bath_a[k] > cfg->bath_a[k - 1]))
                return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: bath levels must be strictly ascending");
        for (int k = 0; k < cfg->nbath; ++k)
            if (cfg->bath_b[k] == 0.0) return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: bath couplings must be nonzero");
        if (cfg->nelectrons < 1 || cfg->nelectrons >= cfg->nstates)
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: IESH needs 1 <= nelectrons < nstates");
        if (iesh_tiles(cfg->nstates, cfg->nelectrons) > kIeshBlock)
            return fail(nullptr, NQCD_ERR_UNSUPPORTED,
                        "nqcd_create: IESH needs ceil(nstates/4) * ceil(nelectrons/4) <= 256");
        const size_t smem = cfg->precision == NQCD_PREC_FP64 ? iesh_layout<double>(cfg->nstates, cfg->nelectrons).bytes
                                                             : iesh_layout<float>(cfg->nstates, cfg->nelectrons).bytes;
        if (smem > 227 * 1024) return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: IESH system too large for one CTA");
        if (cfg->nparams < 6 || !cfg->params)
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: IESH model needs kxy, A, a, delta, B, b");
        if (cfg->init_kind != NQCD_INIT_GIVEN && cfg->init_kind != NQCD_INIT_FERMI_DIRAC)
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: IESH starts from given or Fermi-Dirac occupations");
        if (cfg->init_kind == NQCD_INIT_FERMI_DIRAC && !(cfg->beta > 0.0))
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: Fermi-Dirac occupations need beta > 0");
        if (cfg->precision == NQCD_PREC_FP32_KAHAN)
            return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: IESH runs NQCD_PREC_FP64 or NQCD_PREC_FP32");
        if (cfg->nbeads_max > 1) {  // RingPolymerSimulation{AdiabaticIESH}
            if (cfg->method != NQCD_METHOD_IESH)
                return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: ring polymers run IESH, not EhrenfestNA");
            if (cfg->nbeads_max > kRpIeshMaxBeads || cfg->nelectrons > kRpIeshMaxElectrons)
                return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: ring-polymer IESH takes 2..32 beads and <= 64 electrons");
            if (!(cfg->beta > 0.0)) return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: ring polymers need beta > 0");
            if (cfg->decoherence_C != 0.0)
                return fail(nullptr, NQCD_ERR_UNSUPPORTED,
                            "nqcd_create: ring-polymer IESH runs without decoherence correction (a ring polymer's "
                            "eigenvalues are per bead)");
            const size_t smem_rp = cfg->precision == NQCD_PREC_FP64
                                       ? iesh_layout<double>(cfg->nstates, cfg->nelectrons, cfg->nbeads_max).bytes
                                       : iesh_layout<float>(cfg->nstates, cfg->nelectrons, cfg->nbeads_max).bytes;
            if (smem_rp > 227 * 1024)
                return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: ring-polymer IESH system too large for one CTA");
        }
    } else if (mdef) {
        const bool m3 = model == NQCD_MODEL_NEWNS_ANDERSON_3D;
        if (model != NQCD_MODEL_NEWNS_ANDERSON && !m3)
            return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: MDEF runs on the Newns-Anderson models");
        if (m3 ? (cfg->natoms != 1 || cfg->ndofs != 3) : cfg->ndofs * cfg->natoms != 1)
            return fail(nullptr, NQCD_ERR_UNSUPPORTED,
                        "nqcd_create: MDEF runs one degree of freedom (displaced harmonic) or one atom in three "
                        "dimensions (adsorbate)");
        if (m3 && (cfg->nparams < 8 || !cfg->params || !(cfg->params[7] > 0.0)))
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: the 3-D adsorbate needs kxy, A, a, delta, B, b, mu, sigma > 0");
        if (m3 && (cfg->nbeads_max > 1 || cfg->use_friction_surrogate))
            return fail(nullptr, NQCD_ERR_UNSUPPORTED,
                        "nqcd_create: MDEF on the 3-D adsorbate runs classical nuclei with the exact friction");
        if (cfg->nbath < 1 || cfg->nbath > kMdefMaxBath || !cfg->bath_a || !cfg->bath_b)
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: MDEF needs 1..512 bath levels and couplings");
        for (int k = 1; k < cfg->nbath; ++k)
            if (!(cfg->bath_a[k] > cfg->bath_a[k - 1]))
                return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: bath levels must be strictly ascending");
        for (int k = 0; k < cfg->nbath; ++k)
            if (cfg->bath_b[k] == 0.0) return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: bath couplings must be nonzero");
        if (!m3 && (cfg->nparams < 5 || !cfg->params || !(cfg->params[4] > 0.0)))
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: Newns-Anderson needs k, g, delta, mu, sigma > 0");
        if (!(cfg->beta > 0.0)) return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: MDEF needs beta > 0");
        if (cfg->nbeads_max > 1) {  // RingPolymerSimulation{DiabaticMDEF}
            if (cfg->nbeads_max > kRpMdefMaxBeads)
                return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: ring-polymer MDEF takes 2..32 beads");
            if (cfg->save_stride != 0 || cfg->use_friction_surrogate)
                return fail(nullptr, NQCD_ERR_UNSUPPORTED,
                            "nqcd_create: ring-polymer MDEF reports final states only and uses the exact friction");
        }
        if (!cfg->masses || !(cfg->masses[0] > 0.0) || cfg->ntraj_max <= 0 || cfg->save_stride < 0)
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: mass, ntraj_max and save_stride are required");
    }
    if (!mdef && !iesh) {
        if (model != NQCD_MODEL_TULLY1 && model != NQCD_MODEL_TULLY2 && model != NQCD_MODEL_TULLY3 &&
            model != NQCD_MODEL_SPINBOSON)
            return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: unknown model");
        if (cfg->nstates != 2) return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: only two-state models");
    }
    if (!(cfg->surrogate_tolerance < 1e300) || cfg->surrogate_tolerance != cfg->surrogate_tolerance)
        return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: surrogate_tolerance must be finite");
    if (!(cfg->decoherence_C >= 0.0 && cfg->decoherence_C < 1e300))
        return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: decoherence_C must be finite and >= 0");
    if (cfg->decoherence_C != 0.0 && cfg->method != NQCD_METHOD_IESH)
        return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: the decoherence correction applies to IESH");
    if (cfg->precision != NQCD_PREC_FP64 && cfg->precision != NQCD_PREC_FP32 && cfg->precision != NQCD_PREC_FP32_KAHAN)
        return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: unknown precision");
    if (cfg->rescaling < 0 || cfg->rescaling > 2) return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: unknown rescaling");
    if (cfg->ndofs <= 0 || cfg->natoms <= 0 || cfg->ntraj_max <= 0 || !cfg->masses)
        return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: ndofs, natoms, ntraj_max and masses are required");
    if (!iesh && (cfg->init_kind < 0 || cfg->init_kind > 2 || cfg->init_state < 0 || cfg->init_state >= cfg->nstates))
        return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: bad initial electronic specification");
    if (cfg->save_stride < 0 || cfg->max_hops < 0 || cfg->traj_offset < 0)
        return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: negative count");
    if (rp) {
        if (model == NQCD_MODEL_SPINBOSON || cfg->ndofs * cfg->natoms != 1)
            return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: ring-polymer surface hopping runs on one-dimensional Tully models");
        if (cfg->nbeads_max < 1 || cfg->nbeads_max > 32)
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: nbeads_max must be 1..32");
        if (!(cfg->beta > 0.0)) return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: ring polymers need beta > 0");
        if (cfg->init_kind == NQCD_INIT_DIABATIC_PURE)
            return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: ring-polymer runs start from an adiabatic state");
        if (cfg->save_stride != 0)
            return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: ring-polymer runs report final-state outputs only");
        if (!(cfg->terminate_x >= 0.0)) return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: terminate_x must be >= 0");
    }
    const bool rp_mdef = mdef && cfg->nbeads_max > 1;
    const bool rp_iesh = iesh && cfg->nbeads_max > 1;
    const int64_t ndof = (rp || rp_mdef) ? (int64_t)cfg->nbeads_max
                                         : (int64_t)cfg->ndofs * cfg->natoms * (rp_iesh ? cfg->nbeads_max : 1);
    int need_params = model == NQCD_MODEL_TULLY2 ? 5 : (model == NQCD_MODEL_TULLY3 ? 3 : (model == NQCD_MODEL_SPINBOSON ? 2 : (mdef ? (model == NQCD_MODEL_NEWNS_ANDERSON_3D ? 8 : 5) : (iesh ? 6 : 4))));
    if (cfg->nparams < need_params || !cfg->params)
        return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: too few model parameters");
    if (mdef || iesh) {
        // validated above
    } else if (model == NQCD_MODEL_SPINBOSON) {
        if (cfg->nbath != ndof || !cfg->bath_a || !cfg->bath_b)
            return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: spin-boson needs nbath == ndofs*natoms couplings and frequencies");
    } else if (!rp && ndof != 1) {
        return fail(nullptr, NQCD_ERR_UNSUPPORTED, "nqcd_create: Tully models have one degree of freedom");
    }
    for (int a = 0; a < cfg->natoms; ++a)
        if (!(cfg->masses[a] > 0.0)) return fail(nullptr, NQCD_ERR_ARG, "nqcd_create: masses must be positive");

    int dev_count = 0;
    cudaError_t e = cudaGetDeviceCount(&dev_count);
    if (e != cudaSuccess || dev_count == 0) {
        cudaGetLastError();
        return fail(nullptr, NQCD_ERR_CUDA, std::string("nqcd_create: no CUDA device (") + cudaGetErrorString(e) + ")");
    }

    nqcd_handle* h = new (std::nothrow) nqcd_handle();
    if (!h) return fail(nullptr, NQCD_ERR_OOM, "nqcd_create: out of host memory");
    h->cfg = *cfg;
    h->cfg.params = nullptr;
    h->cfg.bath_a = h->cfg.bath_b = h->cfg.masses = nullptr;
    h->cap = cfg->ntraj_max;
    h->ndof = ndof;
    h->params.assign(cfg->params, cfg->params + cfg->nparams);
    h->params.resize(8, 0.0);
    h->mass0 = cfg->masses[0];
    if (iesh) {
        h->nstates = cfg->nstates;
        h->nelec = cfg->nelectrons;
    }

    auto bail = [&](cudaError_t ee, const char* what) {
        std::string m = std::string("nqcd_create: ") + what + ": " + cudaGetErrorString(ee);
        cudaGetLastError();
        free_all(h);
        delete h;
        return fail(nullptr, ee == cudaErrorMemoryAllocation ? NQCD_ERR_OOM : NQCD_ERR_CUDA, m);
    };
#define NQCD_CREATE(call)                       \
    do {                                        \
        cudaError_t ee_ = (call);               \
        if (ee_ != cudaSuccess) return bail(ee_, #call); \
    } while (0)

    NQCD_CREATE(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    NQCD_CREATE(cudaEventCreate(&h->ev0));
    NQCD_CREATE(cudaEventCreate(&h->ev1));
    NQCD_CREATE(cudaEventCreate(&h->evk0));
    NQCD_CREATE(cudaEventCreate(&h->evk1));
    if (rp) {
        NQCD_CREATE(cudaEventCreateWithFlags(&h->rp_fork, cudaEventDisableTiming));
        for (int c = 0; c < kNumRpCounts; ++c) {
            NQCD_CREATE(cudaStreamCreateWithFlags(&h->rp_streams[c], cudaStreamNonBlocking));
            NQCD_CREATE(cudaEventCreateWithFlags(&h->rp_join[c], cudaEventDisableTiming));
        }
    }

    std::vector<double> mass(ndof), bc(ndof, 0.0), bw2(ndof, 0.0);
    for (int64_t I = 0; I < ndof; ++I) mass[I] = rp ? cfg->masses[0] : cfg->masses[I / cfg->ndofs];
    if (model == NQCD_MODEL_SPINBOSON) {
        for (int64_t I = 0; I < ndof; ++I) {
            bc[I] = cfg->bath_a[I];
            bw2[I] = cfg->bath_b[I] * cfg->bath_b[I];
            h->sum_c2_over_m += bc[I] * bc[I] / mass[I];
        }
    }
    const int64_t cap = h->cap;
    NQCD_CREATE(dalloc(&h->d_mass, ndof));
    NQCD_CREATE(dalloc(&h->d_bath_c, ndof));
    NQCD_CREATE(dalloc(&h->d_bath_w2, ndof));
    NQCD_CREATE(cudaMemcpy(h->d_mass, mass.data(), ndof * sizeof(double), cudaMemcpyHostToDevice));
    NQCD_CREATE(cudaMemcpy(h->d_bath_c, bc.data(), ndof * sizeof(double), cudaMemcpyHostToDevice));
    NQCD_CREATE(cudaMemcpy(h->d_bath_w2, bw2.data(), ndof * sizeof(double), cudaMemcpyHostToDevice));
    NQCD_CREATE(dalloc(&h->d_r0, ndof * cap));
    NQCD_CREATE(dalloc(&h->d_v0, ndof * cap));
    NQCD_CREATE(dalloc(&h->d_r, ndof * cap));
    NQCD_CREATE(dalloc(&h->d_v, ndof * cap));
    NQCD_CREATE(dalloc(&h->d_sig0, 8 * cap));
    NQCD_CREATE(dalloc(&h->d_sig, 8 * cap));
    NQCD_CREATE(dalloc(&h->d_state0, cap));
    NQCD_CREATE(dalloc(&h->d_state, cap));
    if (model == NQCD_MODEL_SPINBOSON && cfg->precision == NQCD_PREC_FP64) NQCD_CREATE(dalloc(&h->d_scratch, ndof * cap));
    NQCD_CREATE(dalloc(&h->d_nhops, cap));
    NQCD_CREATE(dalloc(&h->d_nfrust, cap));
    NQCD_CREATE(dalloc(&h->d_nsteps, cap));
    if (rp_mdef || rp_iesh) {
        h->rp_beads = cfg->nbeads_max;
        NQCD_CREATE(dalloc(&h->d_rptab, cfg->nbeads_max * cfg->nbeads_max + 4 * cfg->nbeads_max));
    }
    if (!mdef) {  // FSSH, Ehrenfest, RPSH, IESH: per-trajectory counts of steps with FP64 electronics
        NQCD_CREATE(dalloc(&h->d_fp64steps, cap));
        NQCD_CREATE(cudaMemset(h->d_fp64steps, 0, cap * sizeof(int32_t)));
    }
    if (cfg->max_hops > 0) NQCD_CREATE(dalloc(&h->d_hoplog, (int64_t)cfg->max_hops * 3 * cap));
    NQCD_CREATE(dalloc(&h->d_energy, 2 * cap));
    NQCD_CREATE(dalloc(&h->d_counts, 24));
    if (mdef || iesh) {
        std::vector<double> eps(cfg->bath_a, cfg->bath_a + cfg->nbath), V2(cfg->nbath);
        for (int k = 0; k < cfg->nbath; ++k) V2[k] = cfg->bath_b[k] * cfg->bath_b[k];
        for (int k = 0; k < cfg->nbath; ++k) h->sumV2 += V2[k];
        NQCD_CREATE(dalloc(&h->d_eps, cfg->nbath));
        NQCD_CREATE(dalloc(&h->d_V2, cfg->nbath));
        NQCD_CREATE(cudaMemcpy(h->d_eps, eps.data(), eps.size() * sizeof(double), cudaMemcpyHostToDevice));
        NQCD_CREATE(cudaMemcpy(h->d_V2, V2.data(), V2.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    if (iesh) {
        const int64_t ne = cfg->nelectrons, ns = cfg->nstates;
        NQCD_CREATE(dalloc(&h->d_occ0, ne * cap));
        NQCD_CREATE(dalloc(&h->d_occ, ne * cap));
        NQCD_CREATE(dalloc(&h->d_psi_re, ne * ns * cap));
        NQCD_CREATE(dalloc(&h->d_psi_im, ne * ns * cap));
        NQCD_CREATE(cudaMemset(h->d_occ0, 0, ne * cap * sizeof(int32_t)));
    }
    NQCD_CREATE(cudaMemset(h->d_sig0, 0, 8 * cap * sizeof(double)));
    NQCD_CREATE(cudaMemset(h->d_state0, 0, cap * sizeof(int32_t)));
    if (rp) {
        // normal-mode matrices of every instantiated bead count (dt-independent)
        int64_t off = 0;
        for (int c = 0; c < kNumRpCounts; ++c) {
            h->rp_U_off[c] = off;
            off += (int64_t)kRpCounts[c] * kRpCounts[c];
        }
        std::vector<double> U(off);
        for (int c = 0; c < kNumRpCounts; ++c) nm_transform_matrix(kRpCounts[c], U.data() + h->rp_U_off[c]);
        NQCD_CREATE(dalloc(&h->d_rpU, off));
        NQCD_CREATE(cudaMemcpy(h->d_rpU, U.data(), off * sizeof(double), cudaMemcpyHostToDevice));
        NQCD_CREATE(dalloc(&h->d_rpcay, 4 * 32 * kNumRpCounts));
        NQCD_CREATE(dalloc(&h->d_rpcirc, 4 * 32 * kNumRpCounts));
        NQCD_CREATE(dalloc(&h->d_nbeads, cap));
        NQCD_CREATE(dalloc(&h->d_class_traj, cap));
        NQCD_CREATE(dalloc(&h->d_queue, kRpshMaxClasses));
        NQCD_CREATE(dalloc(&h->d_block_class, kMaxRpGrid));
    }
#undef NQCD_CREATE
    *out = h;
    return NQCD_OK;
}

// Ring polymers: group trajectories by (Tully model, bead count) into the
// classes served by the persistent kernel, from the host copies of the
// per-trajectory bead counts and models.
static int build_rp_classes(nqcd_handle* h, int64_t* h2d) {
    const int64_t ntraj = (int64_t)h->traj_beads.size();
    constexpr int nkey = 3 * kNumRpCounts;
    std::vector<int64_t> count(nkey, 0);
    std::vector<int> key_of(ntraj);
    for (int64_t t = 0; t < ntraj; ++t) {
        int b = h->traj_beads[t], slot = -1;
        for (int c = 0; c < kNumRpCounts; ++c)
            if (kRpCounts[c] == b) slot = c;
        key_of[t] = (h->traj_models[t] - NQCD_MODEL_TULLY1) * kNumRpCounts + slot;
        count[key_of[t]] += 1;
    }
    h->nclass = 0;
    h->class_begin[0] = 0;
    std::vector<int64_t> fillpos(nkey, 0);
    for (int key = 0; key < nkey; ++key) {
        if (!count[key]) continue;
        const int k = h->nclass;
        h->class_slot[k] = key % kNumRpCounts;
        h->class_beads[k] = kRpCounts[key % kNumRpCounts];
        h->class_model[k] = NQCD_MODEL_TULLY1 + key / kNumRpCounts;
        fillpos[key] = h->class_begin[k];
        h->class_begin[k + 1] = h->class_begin[k] + count[key];
        h->nclass += 1;
    }
    std::vector<int32_t> order(ntraj);
    for (int64_t t = 0; t < ntraj; ++t) order[fillpos[key_of[t]]++] = (int32_t)t;
    if ((int64_t)h->traj_speed.size() == ntraj) {
        // slowest first within each class: the slow trajectories run longest,
        // and starting them first keeps them off the end of the launch
        // (results do not depend on the order)
        const float* sp = h->traj_speed.data();
        for (int k = 0; k < h->nclass; ++k)
            std::stable_sort(order.begin() + h->class_begin[k], order.begin() + h->class_begin[k + 1],
                             [sp](int32_t a, int32_t b) { return sp[a] < sp[b]; });
    }
    NQCD_CUDA(h, cudaMemcpyAsync(h->d_class_traj, order.data(), ntraj * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    *h2d += ntraj * (int64_t)sizeof(int32_t);
    return NQCD_OK;
}

// Per-trajectory bead counts (host array nbeads, NULL = nbeads_max for all);
// every trajectory starts on the handle's model.
static int set_bead_classes(nqcd_handle* h, int64_t ntraj, const int32_t* nbeads, const double* v0_host,
                            int64_t* h2d) {
    if (h->cfg.method != NQCD_METHOD_RPSH) return NQCD_OK;
    h->traj_beads.assign(ntraj, h->cfg.nbeads_max);
    h->traj_models.assign(ntraj, h->cfg.model);
    h->traj_speed.clear();
    for (int64_t t = 0; t < ntraj; ++t) {
        int b = nbeads ? nbeads[t] : h->cfg.nbeads_max;
        bool known = false;
        for (int c = 0; c < kNumRpCounts; ++c) known |= kRpCounts[c] == b;
        if (!known || b > h->cfg.nbeads_max)
            return fail(h, NQCD_ERR_UNSUPPORTED,
                        "nqcd_set_initial: bead counts must be one of 1, 2, 4, 5, 8, 10, 16, 32 and <= nbeads_max");
        h->traj_beads[t] = b;
    }
    if (v0_host) {
        h->traj_speed.resize(ntraj);
        const int64_t nd = h->ndof;
        for (int64_t t = 0; t < ntraj; ++t) {
            double sv = 0.0;
            for (int j = 0; j < h->traj_beads[t]; ++j) sv += v0_host[t * nd + j];
            h->traj_speed[t] = (float)fabs(sv / h->traj_beads[t]);
        }
    }
    return build_rp_classes(h, h2d);
}

static int set_initial_common(nqcd_handle* h, int64_t ntraj, const double* sig_re, const double* sig_im,
                              const int32_t* state0, int64_t* h2d) {
    const int64_t N = ntraj;
    // MDEF carries no electronic state: only FSSH and RPSH read sigma and state0
    const bool two_state = h->cfg.method == NQCD_METHOD_FSSH || h->cfg.method == NQCD_METHOD_RPSH ||
                           h->cfg.method == NQCD_METHOD_EHRENFEST;
    if ((h->cfg.method == NQCD_METHOD_IESH || h->cfg.method == NQCD_METHOD_EHRENFEST_NA) &&
        h->cfg.init_kind == NQCD_INIT_GIVEN) {
        // occupations (nelectrons, ntraj) column-major -> device [electron][trajectory]
        if (!state0) return fail(h, NQCD_ERR_ARG, "nqcd_set_initial: IESH with NQCD_INIT_GIVEN needs the occupations in state0");
        const int ne = h->nelec, ns = h->nstates;
        std::vector<int32_t> soa((size_t)ne * N);
        for (int64_t t = 0; t < N; ++t) {
            unsigned long long m2[2] = {0ull, 0ull};
            for (int j = 0; j < ne; ++j) {
                const int32_t s = state0[t * ne + j];
                if (s < 0 || s >= ns || ((m2[s >> 6] >> (s & 63)) & 1ull))
                    return fail(h, NQCD_ERR_ARG, "nqcd_set_initial: occupations must be distinct states in 0..nstates-1");
                m2[s >> 6] |= 1ull << (s & 63);
                soa[(size_t)j * N + t] = s;
            }
        }
        NQCD_CUDA(h, cudaMemcpyAsync(h->d_occ0, soa.data(), soa.size() * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
        NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
        *h2d += (int64_t)(soa.size() * sizeof(int32_t));
    }
    if (two_state && h->cfg.init_kind == NQCD_INIT_GIVEN) {
        if (!sig_re || !state0) return fail(h, NQCD_ERR_ARG, "nqcd_set_initial: sig_re and state0 required for NQCD_INIT_GIVEN");
        // host (2,2,ntraj) column-major re/im -> device [8][ntraj]: component 2*(2*i+j)+{0,1}
        std::vector<double> soa(8 * N);
        for (int64_t t = 0; t < N; ++t)
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j) {
                    soa[(2 * (2 * i + j)) * N + t] = sig_re[t * 4 + i + 2 * j];
                    soa[(2 * (2 * i + j) + 1) * N + t] = sig_im ? sig_im[t * 4 + i + 2 * j] : 0.0;
                }
        for (int64_t t = 0; t < N; ++t)
            if (state0[t] < 0 || state0[t] >= h->nstates) return fail(h, NQCD_ERR_ARG, "nqcd_set_initial: state out of range");
        NQCD_CUDA(h, cudaMemcpyAsync(h->d_sig0, soa.data(), 8 * N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        NQCD_CUDA(h, cudaMemcpyAsync(h->d_state0, state0, N * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
        NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
        *h2d += 8 * N * (int64_t)sizeof(double) + N * (int64_t)sizeof(int32_t);
    }
    h->ntraj = ntraj;
    h->initial_set = true;
    h->has_run = false;
    return NQCD_OK;
}

int nqcd_set_initial(nqcd_handle* h, int64_t ntraj, const double* r0, const double* v0, const double* sig_re,
                     const double* sig_im, const int32_t* state0, const int32_t* nbeads) {
    if (!h) return NQCD_ERR_ARG;
    if (ntraj <= 0 || ntraj > h->cap) return fail(h, NQCD_ERR_ARG, "nqcd_set_initial: ntraj outside 1..ntraj_max");
    if (!r0 || !v0) return fail(h, NQCD_ERR_ARG, "nqcd_set_initial: r0 and v0 are required");
    const int64_t n = ntraj * h->ndof;
    int rc = ensure_stage(h, n);
    if (rc) return rc;
    int64_t h2d = 0;
    // (ndof, ntraj) column-major host == AoS [ntraj][ndof]; gather to SoA [ndof][ntraj]
    NQCD_CUDA(h, cudaMemcpyAsync(h->d_stage, r0, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    NQCD_CUDA(h, transpose(h->d_stage, h->d_r0, ntraj, h->ndof, h->stream));
    NQCD_CUDA(h, cudaMemcpyAsync(h->d_stage, v0, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    NQCD_CUDA(h, transpose(h->d_stage, h->d_v0, ntraj, h->ndof, h->stream));
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    h2d += 2 * n * (int64_t)sizeof(double);
    rc = set_bead_classes(h, ntraj, nbeads, v0, &h2d);
    if (rc) return rc;
    return set_initial_common(h, ntraj, sig_re, sig_im, state0, &h2d);
}

int nqcd_set_initial_device(nqcd_handle* h, int64_t ntraj, const double* d_r0, const double* d_v0,
                            const int32_t* nbeads) {
    if (!h) return NQCD_ERR_ARG;
    if (ntraj <= 0 || ntraj > h->cap) return fail(h, NQCD_ERR_ARG, "nqcd_set_initial_device: ntraj outside 1..ntraj_max");
    if (!d_r0 || !d_v0) return fail(h, NQCD_ERR_ARG, "nqcd_set_initial_device: r0 and v0 are required");
    if (h->cfg.method != NQCD_METHOD_MDEF && h->cfg.init_kind == NQCD_INIT_GIVEN)
        return fail(h, NQCD_ERR_ARG, "nqcd_set_initial_device: NQCD_INIT_GIVEN needs nqcd_set_initial");
    const int64_t n = ntraj * h->ndof;
    NQCD_CUDA(h, cudaMemcpyAsync(h->d_r0, d_r0, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    NQCD_CUDA(h, cudaMemcpyAsync(h->d_v0, d_v0, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    int64_t h2d = 0;
    int rc = set_bead_classes(h, ntraj, nbeads, nullptr, &h2d);
    if (rc) return rc;
    return set_initial_common(h, ntraj, nullptr, nullptr, nullptr, &h2d);
}

int nqcd_sample_initial(nqcd_handle* h, int64_t ntraj, const nqcd_sampler* position, const nqcd_sampler* velocity,
                        uint64_t seed) {
    if (!h) return NQCD_ERR_ARG;
    if (ntraj <= 0 || ntraj > h->cap) return fail(h, NQCD_ERR_ARG, "nqcd_sample_initial: ntraj outside 1..ntraj_max");
    if (!position || !velocity) return fail(h, NQCD_ERR_ARG, "nqcd_sample_initial: position and velocity samplers are required");
    if (h->cfg.method == NQCD_METHOD_RPSH || h->rp_beads > 1)
        return fail(h, NQCD_ERR_UNSUPPORTED, "nqcd_sample_initial: ring-polymer beads take nqcd_set_initial");
    if (h->cfg.method != NQCD_METHOD_MDEF && h->cfg.init_kind == NQCD_INIT_GIVEN)
        return fail(h, NQCD_ERR_ARG, "nqcd_sample_initial: NQCD_INIT_GIVEN needs nqcd_set_initial");
    const int nd = (int)h->ndof;
    std::vector<nqcd_sampler> tab(2 * (size_t)nd);
    for (int d = 0; d < 2 * nd; ++d) {
        const nqcd_sampler sp = d < nd ? position[d] : velocity[d - nd];
        const bool ok = (sp.kind == NQCD_SAMPLE_FIXED && isfinite(sp.a)) ||
                        (sp.kind == NQCD_SAMPLE_NORMAL && isfinite(sp.a) && isfinite(sp.b) && sp.b >= 0.0) ||
                        (sp.kind == NQCD_SAMPLE_UNIFORM && isfinite(sp.a) && isfinite(sp.b) && sp.b >= sp.a);
        if (!ok) return fail(h, NQCD_ERR_ARG, "nqcd_sample_initial: bad sampler (kind, finite parameters, width >= 0, b >= a)");
        tab[d] = sp;
    }
    const int64_t bytes = (int64_t)(tab.size() * sizeof(nqcd_sampler));
    int rc = ensure_stage(h, (bytes + 7) / 8);
    if (rc) return rc;
    NQCD_CUDA(h, cudaMemcpyAsync(h->d_stage, tab.data(), bytes, cudaMemcpyHostToDevice, h->stream));
    const int64_t total = 2 * (int64_t)nd * ntraj;
    const int64_t blocks = (total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096;
    sample_initial_kernel<<<(unsigned)blocks, 256, 0, h->stream>>>(reinterpret_cast<const nqcd_sampler*>(h->d_stage), nd,
                                                                     ntraj, h->cfg.traj_offset, seed, h->d_r0, h->d_v0);
    NQCD_CUDA(h, cudaGetLastError());
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    int64_t h2d = bytes;
    return set_initial_common(h, ntraj, nullptr, nullptr, nullptr, &h2d);
}

int nqcd_get_status(nqcd_handle* h, int32_t* nonfinite, int32_t* fp64_steps) {
    if (!h) return NQCD_ERR_ARG;
    if (!h->has_run) return fail(h, NQCD_ERR_STATE, "nqcd_get_status: call nqcd_run first");
    const int64_t N = h->ntraj;
    if (nonfinite) {
        int rc = ensure_stage(h, (N + 1) / 2);
        if (rc) return rc;
        int32_t* flag = reinterpret_cast<int32_t*>(h->d_stage);
        nonfinite_kernel<<<(unsigned)((N + 255) / 256 < 1024 ? (N + 255) / 256 : 1024), 256, 0, h->stream>>>(
            h->d_r, h->d_v, h->ndof, N, flag);
        NQCD_CUDA(h, cudaGetLastError());
        NQCD_CUDA(h, cudaMemcpyAsync(nonfinite, flag, N * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    }
    if (fp64_steps) {
        if (h->d_fp64steps)
            NQCD_CUDA(h, cudaMemcpyAsync(fp64_steps, h->d_fp64steps, N * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
        else
            memset(fp64_steps, 0, N * sizeof(int32_t));
    }
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    return NQCD_OK;
}

// nqcd_run_host's fast spin-boson path: the host initial conditions (AoS [ntraj][ndof]) are copied
// in chunks of whole blocks on a copy stream and transposed into the initial (d_r0, d_v0) and the
// working (d_r, d_v) state; chunk c runs on compute stream c % 2 once its copy has landed, so the
// transfer of later chunks overlaps the integration of earlier ones and a chunk's tail overlaps the
// next one's start.  Each block integrates the same trajectories and writes the same partial-sum
// rows as in one launch over all of them, so the results are the same.
static int run_pipelined(nqcd_handle* h, FsshParams p, int64_t lanes, int64_t blk, const double* r_host,
                         const double* v_host, int64_t* h2d, int* launches) {
    const int64_t N = h->ntraj, nd = h->ndof;
    cudaStream_t s = h->stream;
    if (!h->pipe_copy) {
        NQCD_CUDA(h, cudaStreamCreateWithFlags(&h->pipe_copy, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            NQCD_CUDA(h, cudaStreamCreateWithFlags(&h->pipe_run[k], cudaStreamNonBlocking));
            NQCD_CUDA(h, cudaEventCreateWithFlags(&h->pipe_done[k], cudaEventDisableTiming));
        }
        NQCD_CUDA(h, cudaEventCreateWithFlags(&h->pipe_start, cudaEventDisableTiming));
        for (int c = 0; c < kPipeChunks; ++c)
            NQCD_CUDA(h, cudaEventCreateWithFlags(&h->pipe_ready[c], cudaEventDisableTiming));
    }
    int rc = ensure_stage(h, 2 * nd * N);
    if (rc) return rc;
    double* stage_r = h->d_stage;
    double* stage_v = h->d_stage + nd * N;
    const int64_t per_block = blk / lanes;  // trajectories per block
    const int64_t nblocks = (N + per_block - 1) / per_block;
    const int K = (int)(nblocks < kPipeChunks ? nblocks : kPipeChunks);
    // everything queued on the main stream (resets of counters and outputs) comes first
    NQCD_CUDA(h, cudaEventRecord(h->pipe_start, s));
    NQCD_CUDA(h, cudaStreamWaitEvent(h->pipe_copy, h->pipe_start, 0));
    for (int k = 0; k < 2; ++k) NQCD_CUDA(h, cudaStreamWaitEvent(h->pipe_run[k], h->pipe_start, 0));
    NQCD_CUDA(h, cudaEventRecord(h->evk0, s));
    for (int c = 0; c < K; ++c) {
        const int64_t lo = nblocks * c / K * per_block;
        const int64_t hi = std::min<int64_t>(nblocks * (c + 1) / K * per_block, N);
        if (lo >= hi) continue;
        const size_t bytes = (size_t)((hi - lo) * nd) * sizeof(double);
        NQCD_CUDA(h, cudaMemcpyAsync(stage_r + lo * nd, r_host + lo * nd, bytes, cudaMemcpyHostToDevice, h->pipe_copy));
        NQCD_CUDA(h, cudaMemcpyAsync(stage_v + lo * nd, v_host + lo * nd, bytes, cudaMemcpyHostToDevice, h->pipe_copy));
        NQCD_CUDA(h, transpose2(stage_r + lo * nd, h->d_r0 + lo, h->d_r + lo, hi - lo, nd, N, h->pipe_copy));
        NQCD_CUDA(h, transpose2(stage_v + lo * nd, h->d_v0 + lo, h->d_v + lo, hi - lo, nd, N, h->pipe_copy));
        NQCD_CUDA(h, cudaEventRecord(h->pipe_ready[c], h->pipe_copy));
        *h2d += 2 * (int64_t)bytes;
        cudaStream_t rs = h->pipe_run[c & 1];
        NQCD_CUDA(h, cudaStreamWaitEvent(rs, h->pipe_ready[c], 0));
        p.traj_lo = lo;
        p.traj_hi = hi;
        const cudaError_t e = h->cfg.precision == NQCD_PREC_FP32 ? launch_fssh2_fp32(p, rs) : launch_fssh2_fp32_kahan(p, rs);
        if (e != cudaSuccess) return cuda_fail(h, e, "nqcd_run_host: ensemble kernel launch");
        *launches += 3;  // two transposes and the chunk's kernel
    }
    for (int k = 0; k < 2; ++k) {
        NQCD_CUDA(h, cudaEventRecord(h->pipe_done[k], h->pipe_run[k]));
        NQCD_CUDA(h, cudaStreamWaitEvent(s, h->pipe_done[k], 0));
    }
    return NQCD_OK;
}

// Whether nqcd_run_host pipelines this configuration (the fast spin-boson FSSH / Ehrenfest kernel
// with sampled electronic initial states); the others take nqcd_set_initial + nqcd_run.
static bool pipelined_config(const nqcd_handle* h) {
    return (h->cfg.method == NQCD_METHOD_FSSH || h->cfg.method == NQCD_METHOD_EHRENFEST) &&
           h->cfg.model == NQCD_MODEL_SPINBOSON && h->cfg.precision != NQCD_PREC_FP64 &&
           h->cfg.init_kind != NQCD_INIT_GIVEN;
}

static int run_impl(nqcd_handle* h, double t0, double t1, double dt, uint64_t seed, nqcd_outputs* out,
                    nqcd_stats* stats, const double* r_host, const double* v_host) {
    if (!h) return NQCD_ERR_ARG;
    if (!h->initial_set) return fail(h, NQCD_ERR_STATE, "nqcd_run: call nqcd_set_initial first");
    if (!(dt > 0.0) || !(t1 >= t0) || !isfinite(t0) || !isfinite(t1))
        return fail(h, NQCD_ERR_ARG, "nqcd_run: need dt > 0 and finite t0 <= t1");
    auto wall0 = std::chrono::steady_clock::now();
    const int64_t N = h->ntraj;
    const bool mdef = h->cfg.method == NQCD_METHOD_MDEF;
    const bool iesh = h->cfg.method == NQCD_METHOD_IESH || h->cfg.method == NQCD_METHOD_EHRENFEST_NA;
    // FSSH and RPSH step like the reference's integrator (its FP64 clock, a
    // last partial step up to t1).  MDEF and IESH take steps of dt and, when
    // t1 - t0 is not a whole number of steps, a shortened last step h_last
    // that reaches t1 (ring polymers need whole steps: their Cayley matrices
    // are built for dt).
    const double span = (t1 - t0) / dt;
    if (!(span < 2147483645.0)) return fail(h, NQCD_ERR_ARG, "nqcd_run: too many steps");
    int64_t nsteps = 0;
    double h_last = dt;
    if (mdef || iesh) {
        nsteps = (int64_t)llround(span);
        if (fabs((double)nsteps * dt - (t1 - t0)) > 1e-9 * (fabs(t1 - t0) + dt)) {
            if (h->cfg.nbeads_max > 1)
                return fail(h, NQCD_ERR_ARG, "nqcd_run: ring-polymer MDEF and IESH need t1 - t0 to be a whole "
                                              "number of steps");
            nsteps = (int64_t)floor(span) + 1;
            h_last = (t1 - t0) - (double)(nsteps - 1) * dt;
        }
    } else {
        nsteps = count_steps(t0, t1, dt);
    }
    if (nsteps > (int64_t)span + 2)
        return fail(h, NQCD_ERR_ARG, "nqcd_run: dt is below the spacing of doubles between t0 and t1");
    const int stride = h->cfg.save_stride;
    const int nsave = stride > 0 ? (int)(nsteps / stride + 1) : 0;
    const int64_t lanes =
        mdef ? 32 : (iesh ? 1 : fssh2_lanes_per_traj(h->cfg.model, h->cfg.precision, h->map.sb_lanes));
    // the fast spin-boson kernel's block size follows the mapping; the other kernels use 128 threads
    const bool sb_fast = !mdef && !iesh && h->cfg.method != NQCD_METHOD_RPSH &&
                         h->cfg.model == NQCD_MODEL_SPINBOSON && h->cfg.precision != NQCD_PREC_FP64;
    const int64_t blk = sb_fast && h->map.sb_block > 0 ? h->map.sb_block : 128;
    const int64_t blocks = (N * lanes + blk - 1) / blk;
    // rows of observable partial sums: one per warp (FSSH, MDEF) or per trajectory (IESH)
    const int64_t nwarps = iesh ? N : blocks * (blk / 32);
    if (nsave > 0 && nwarps * nsave * 4 > h->partial_cap) {
        if (h->d_partial) cudaFree(h->d_partial);
        if (h->d_popcorr) cudaFree(h->d_popcorr);
        h->d_partial = h->d_popcorr = nullptr;
        h->partial_cap = 0;
        NQCD_CUDA(h, dalloc(&h->d_partial, nwarps * nsave * 4));
        NQCD_CUDA(h, dalloc(&h->d_popcorr, (int64_t)nsave * 4));
        h->partial_cap = nwarps * nsave * 4;
    }
    cudaStream_t s = h->stream;
    int launches = 0;
    if (h->cfg.method == NQCD_METHOD_EHRENFEST && out && out->scattering) {
        // population-sum buffers of the Ehrenfest scattering output
        int rc = ensure_stage(h, 4 * N + 4);
        if (rc) return rc;
        const int64_t need = reduce_chunks(N, 4) * 4;
        if (need > h->redtmp_cap) {
            if (h->d_redtmp) cudaFree(h->d_redtmp);
            h->d_redtmp = nullptr;
            h->redtmp_cap = 0;
            NQCD_CUDA(h, dalloc(&h->d_redtmp, need));
            h->redtmp_cap = need;
        }
    }
    NQCD_CUDA(h, cudaEventRecord(h->ev0, s));
    const int64_t nd = h->ndof;
    if (!r_host) {  // (nqcd_run_host writes the working state from the host chunks)
        NQCD_CUDA(h, cudaMemcpyAsync(h->d_r, h->d_r0, nd * N * sizeof(double), cudaMemcpyDeviceToDevice, s));
        NQCD_CUDA(h, cudaMemcpyAsync(h->d_v, h->d_v0, nd * N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    NQCD_CUDA(h, cudaMemcpyAsync(h->d_sig, h->d_sig0, 8 * N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    NQCD_CUDA(h, cudaMemcpyAsync(h->d_state, h->d_state0, N * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    NQCD_CUDA(h, cudaMemsetAsync(h->d_counts, 0, 24 * sizeof(unsigned long long), s));
    if (h->d_fp64steps) NQCD_CUDA(h, cudaMemsetAsync(h->d_fp64steps, 0, N * sizeof(int32_t), s));
    if (h->d_hoplog) {
        int64_t nl = (int64_t)h->cfg.max_hops * 3 * N;
        fill_i32_kernel<<<(unsigned)((nl + 255) / 256 < 4096 ? (nl + 255) / 256 : 4096), 256, 0, s>>>(h->d_hoplog, nl, -1);
        NQCD_CUDA(h, cudaGetLastError());
        ++launches;
    }

    FsshParams p;
    memset(&p, 0, sizeof(p));
    p.model = h->cfg.model;
    for (int q = 0; q < 8; ++q) p.mp[q] = h->params[q];
    p.ndof = (int32_t)nd;
    p.mass = h->d_mass;
    p.bath_c = h->d_bath_c;
    p.bath_w2 = h->d_bath_w2;
    p.sum_c2_over_m = h->sum_c2_over_m;
    p.sum_c2_over_m_f = (float)h->sum_c2_over_m;
    p.sb_group = h->map.sb_lanes;
    p.sb_block = h->map.sb_block;
    p.rescaling = h->cfg.rescaling;
    p.ehrenfest = h->cfg.method == NQCD_METHOD_EHRENFEST ? 1 : 0;
    p.init_kind = h->cfg.init_kind;
    p.init_state = h->cfg.init_state;
    p.gap_fp64 = (float)h->cfg.gap_fp64;
    p.ntraj = N;
    p.traj_lo = 0;
    p.traj_hi = N;
    p.traj_offset = h->cfg.traj_offset;
    p.t0 = t0;
    p.t1 = t1;
    p.dt = dt;
    {
        // the reference integrator's step schedule, for the fast kernels (the
        // plain kernels run the same FP64 clock themselves)
        double tt = t0, hf = 0.0, hl = 0.0;
        int64_t n = 0;
        while (tt < t1 && n < nsteps + 1) {
            const double hh = (t1 - tt) < dt ? (t1 - tt) : dt;
            if (n == 0) hf = hh;
            hl = hh;
            tt = snap_time(tt + hh, t1);
            ++n;
        }
        p.nsteps_total = (int32_t)n;
        p.h_first = (float)hf;
        p.h_mid = (float)dt;
        p.h_last = (float)hl;
        const double den = t0 + hf;  // the interpolation buffer starts at t = 0
        p.sa1 = den != 0.0 ? (float)(t0 / den) : 0.f;
        p.sb1 = den != 0.0 ? (float)(hf / den) : 0.f;
        p.dtsub = (float)(dt / 5.0);
    }
    p.seed = seed;
    p.save_stride = stride;
    p.nsave = nsave;
    p.max_hops = h->cfg.max_hops;
    p.r = h->d_r;
    p.v = h->d_v;
    p.scratch = h->d_scratch;
    p.sigma = h->d_sig;
    p.state = h->d_state;
    p.nhops = h->d_nhops;
    p.nfrustrated = h->d_nfrust;
    p.nsteps = h->d_nsteps;
    p.hop_log = h->d_hoplog;
    p.energy = h->d_energy;
    p.popcorr_partial = h->d_partial;
    p.scatter = p.ehrenfest ? nullptr : h->d_counts;  // Ehrenfest: population sums after the run
    p.fp64_steps = h->d_fp64steps;
    cudaError_t e = cudaSuccess;
    int64_t h2d = 0;
    if (h->cfg.method == NQCD_METHOD_RPSH) {
        // Cayley propagators for this dt, one slot of 32 modes per instantiated bead count
        const bool plain = h->cfg.precision == NQCD_PREC_FP64;
        std::vector<double> cay(4 * 32 * kNumRpCounts, 0.0);
        std::vector<float> circ(cay.size(), 0.0f);
        RpshParams rq;
        memset(&rq, 0, sizeof(rq));
        for (int k = 0; k < h->nclass; ++k) {
            const int slot = h->class_slot[k], n = h->class_beads[k];
            cayley_matrices(n, h->cfg.beta, dt, cay.data() + 4 * 32 * slot);
            rq.class_beads[k] = n;
            rq.U[k] = h->d_rpU + h->rp_U_off[slot];
            rq.cay[k] = h->d_rpcay + 4 * 32 * slot;
            rq.circf[k] = reinterpret_cast<const float4*>(h->d_rpcirc + 4 * 32 * slot);
            if (!plain && !circulant_free_step(n, h->cfg.beta, dt, circ.data() + 4 * 32 * slot))
                return fail(h, NQCD_ERR_UNSUPPORTED, "nqcd_run: ring-polymer free step is not circulant");
        }
        // persistent grid; blocks start on classes in proportion to their estimated work
        const bool one = !plain && h->map.rp_one_launch;
        int grid = plain ? rpsh_grid_fp64() : (one ? rpsh_one_launch_grid() : 0);
        for (int k = 0; k < h->nclass && !plain && !one; ++k) {
            const int gk = rpsh_group_grid(h->class_beads[k], rp_lanes_of(h, h->class_beads[k]));
            grid = gk > grid ? gk : grid;
        }
        if (grid > kMaxRpGrid) grid = kMaxRpGrid;
        if (grid < 1) grid = 1;
        std::vector<double> cost(h->nclass);
        double total = 0.0;
        for (int k = 0; k < h->nclass; ++k) {
            double b = h->class_beads[k];
            cost[k] = (double)(h->class_begin[k + 1] - h->class_begin[k]) * (2000.0 + 60.0 * b + 4.0 * b * b);
            total += cost[k];
        }
        std::vector<int32_t> bc(grid, 0);
        if (!plain && !one) {
            // each bead-count kernel serves only its own classes: block b starts
            // at class b mod nclass and takes the next one of its bead count,
            // which spreads a kernel's blocks evenly over its classes
            for (int q = 0; q < grid; ++q) bc[q] = q % h->nclass;
        } else {
            int pos = 0;
            for (int k = 0; k < h->nclass; ++k) {
                int nb = (int)(grid * cost[k] / (total > 0 ? total : 1.0));
                if (nb < 1) nb = 1;
                for (int q = 0; q < nb && pos < grid; ++q) bc[pos++] = k;
            }
            for (; pos < grid; ++pos) bc[pos] = h->nclass - 1;
        }
        NQCD_CUDA(h, cudaMemcpyAsync(h->d_rpcay, cay.data(), cay.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        NQCD_CUDA(h, cudaMemcpyAsync(h->d_rpcirc, circ.data(), circ.size() * sizeof(float), cudaMemcpyHostToDevice, s));
        NQCD_CUDA(h, cudaMemcpyAsync(h->d_block_class, bc.data(), grid * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        NQCD_CUDA(h, cudaMemsetAsync(h->d_queue, 0, kRpshMaxClasses * sizeof(unsigned long long), s));
        h2d += (int64_t)(cay.size() * sizeof(double) + circ.size() * sizeof(float) + grid * sizeof(int32_t));
        for (int k = 0; k < h->nclass; ++k) {
            // the handle's model uses its parameters; the other Tully models their published defaults
            static const double kTullyDefaults[3][8] = {{0.01, 1.6, 0.005, 1.0, 0, 0, 0, 0},
                                                        {0.1, 0.28, 0.015, 0.06, 0.05, 0, 0, 0},
                                                        {6e-4, 0.1, 0.9, 0, 0, 0, 0, 0}};
            rq.class_model[k] = h->class_model[k];
            for (int q = 0; q < 8; ++q)
                rq.class_mp[k][q] = h->class_model[k] == h->cfg.model
                                        ? h->params[q]
                                        : kTullyDefaults[h->class_model[k] - NQCD_MODEL_TULLY1][q];
        }
        rq.mass = h->mass0;
        rq.beta = h->cfg.beta;
        rq.rescaling = h->cfg.rescaling;
        rq.init_kind = h->cfg.init_kind;
        rq.init_state = h->cfg.init_state;
        rq.gap_fp64 = (float)h->cfg.gap_fp64;
        rq.ntraj = N;
        rq.traj_offset = h->cfg.traj_offset;
        rq.t0 = t0;
        rq.t1 = t1;
        rq.dt = dt;
        rq.nsteps_total = p.nsteps_total;
        rq.h_first = p.h_first;
        rq.h_mid = p.h_mid;
        rq.h_last = p.h_last;
        rq.sa1 = p.sa1;
        rq.sb1 = p.sb1;
        rq.dtsub = p.dtsub;
        rq.seed = seed;
        rq.terminate_x = h->cfg.terminate_x;
        rq.max_hops = h->cfg.max_hops;
        rq.nclass = h->nclass;
        for (int k = 0; k <= h->nclass; ++k) rq.class_begin[k] = h->class_begin[k];
        rq.class_traj = h->d_class_traj;
        rq.queue = h->d_queue;
        rq.block_class = h->d_block_class;
        rq.r = h->d_r;
        rq.v = h->d_v;
        rq.sigma = h->d_sig;
        rq.state = h->d_state;
        rq.nhops = h->d_nhops;
        rq.nfrustrated = h->d_nfrust;
        rq.nsteps = h->d_nsteps;
        rq.hop_log = h->d_hoplog;
        rq.energy = h->d_energy;
        rq.scatter = h->d_counts;
        rq.fp64_steps = h->d_fp64steps;
        if (plain) {
            int maxb = 1;
            for (int k = 0; k < h->nclass; ++k) maxb = h->class_beads[k] > maxb ? h->class_beads[k] : maxb;
            const int64_t threads = (int64_t)grid * kRpshBlock, need = 6 * (int64_t)maxb * threads;
            if (need > h->rpscratch_cap) {
                NQCD_CUDA(h, cudaStreamSynchronize(s));
                if (h->d_rpscratch) cudaFree(h->d_rpscratch);
                h->d_rpscratch = nullptr;
                h->rpscratch_cap = 0;
                NQCD_CUDA(h, dalloc(&h->d_rpscratch, need));
                h->rpscratch_cap = need;
            }
            rq.scratch = h->d_rpscratch;
            rq.scratch_stride = threads;
        }
        NQCD_CUDA(h, cudaEventRecord(h->evk0, s));
        if (plain) {
            e = launch_rpsh_fp64(rq, grid, s);
        } else if (one) {
            e = launch_rpsh_one(rq, grid, s);
        } else {
            // one persistent kernel per bead count present, each with the grid
            // that fills the GPU, concurrently on forked streams and largest
            // bead count first: a kernel's blocks retire as its queues drain
            // and the next kernel's blocks take their place
            NQCD_CUDA(h, cudaEventRecord(h->rp_fork, s));
            int k = 0;
            for (int c = kNumRpCounts - 1; c >= 0 && e == cudaSuccess; --c) {
                bool present = false;
                for (int q = 0; q < h->nclass; ++q) present |= h->class_beads[q] == kRpCounts[c];
                if (!present) continue;
                NQCD_CUDA(h, cudaStreamWaitEvent(h->rp_streams[k], h->rp_fork, 0));
                const int ln = rp_lanes_of(h, kRpCounts[c]);
                e = launch_rpsh_group(kRpCounts[c], ln, rq, rpsh_group_grid(kRpCounts[c], ln), h->rp_streams[k]);
                if (e != cudaSuccess) break;
                NQCD_CUDA(h, cudaEventRecord(h->rp_join[k], h->rp_streams[k]));
                NQCD_CUDA(h, cudaStreamWaitEvent(s, h->rp_join[k], 0));
                ++k;
                if (k > 1) ++launches;  // the common path below counts one
            }
        }
    } else if (iesh) {
        IeshParams q;
        memset(&q, 0, sizeof(q));
        q.nbath = h->cfg.nbath;
        q.nstates = h->nstates;
        q.nelec = h->nelec;
        q.eps = h->d_eps;
        q.V2 = h->d_V2;
        q.sumV2 = h->sumV2;
        q.kxy = h->params[0];
        q.A = h->params[1];
        q.a = h->params[2];
        q.delta = h->params[3];
        q.B = h->params[4];
        q.b = h->params[5];
        q.beta = h->cfg.beta;
        q.mass = h->mass0;
        q.rescaling = h->cfg.rescaling;
        q.init_kind = h->cfg.init_kind;
        q.exact_probability = h->cfg.exact_hop_probability ? 1 : 0;
        q.ehrenfest_na = h->cfg.method == NQCD_METHOD_EHRENFEST_NA ? 1 : 0;
        q.edc_C = h->cfg.decoherence_C;
        q.save_stride = stride;
        q.nsave = nsave;
        q.max_hops = h->cfg.max_hops;
        q.ntraj = N;
        q.traj_offset = h->cfg.traj_offset;
        q.dt = dt;
        q.h_last = h_last;
        q.nsteps = (int32_t)nsteps;
        q.seed = seed;
        // series tail below the rounding of each path's arithmetic
        q.cheb_tol = h->cfg.precision == NQCD_PREC_FP64 ? 1e-17 : 1e-8;
        q.r = h->d_r;
        q.v = h->d_v;
        q.occ0 = h->d_occ0;
        q.occ = h->d_occ;
        q.psi_re = h->d_psi_re;
        q.psi_im = h->d_psi_im;
        q.nhops = h->d_nhops;
        q.nfrustrated = h->d_nfrust;
        q.nsteps_out = h->d_nsteps;
        q.hop_log = h->d_hoplog;
        q.energy = h->d_energy;
        q.obs_partial = nsave > 0 ? h->d_partial : nullptr;
        q.counters = h->d_counts + 8;
        q.gap_fp64 = h->cfg.precision == NQCD_PREC_FP64 ? 0.0 : h->cfg.gap_fp64;
        q.fp64_steps = h->d_fp64steps;
        q.tensor = (h->cfg.precision != NQCD_PREC_FP64 && h->map.iesh_cores == 0 &&
                    iesh_tc_shape(q.nstates, q.nelec)) ? 1 : 0;
        q.lu_always = h->map.iesh_lu_always;
        q.nbeads = h->rp_beads;
        if (h->rp_beads > 1) {
            // ring polymer: normal modes and full-step Cayley matrices of the free ring polymer
            // (cayley_propagator(half=false), ring_polymer.jl:71-82, omega_n = nbeads / beta)
            const int nb = h->rp_beads;
            std::vector<double> tab((size_t)nb * nb + 4 * (size_t)nb);
            nm_transform_matrix(nb, tab.data());
            cayley_matrices(nb, h->cfg.beta, dt, tab.data() + (size_t)nb * nb);
            NQCD_CUDA(h, cudaMemcpyAsync(h->d_rptab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, s));
            q.rp_U = h->d_rptab;
            q.rp_cay = h->d_rptab + (size_t)nb * nb;
            q.omega_n = nb / h->cfg.beta;
        }
        NQCD_CUDA(h, cudaEventRecord(h->evk0, s));
        e = h->cfg.precision == NQCD_PREC_FP64 ? launch_iesh_fp64(q, s) : launch_iesh_fp32(q, s);
    } else if (mdef) {
        MdefParams mp = mdef_params(h, N, dt, (int32_t)nsteps, seed, stride, nsave);
        mp.h_last = h_last;
        if (mp.use_mlp && !h->mlp.trained)
            return fail(h, NQCD_ERR_STATE, "nqcd_run: use_friction_surrogate needs nqcd_train_friction_mlp or nqcd_mlp_set");
        // steps and hop counters are not written by MDEF; observables need zeroed partials
        NQCD_CUDA(h, cudaMemsetAsync(h->d_nsteps, 0, N * sizeof(int32_t), s));
        NQCD_CUDA(h, cudaMemsetAsync(h->d_nhops, 0, N * sizeof(int32_t), s));
        NQCD_CUDA(h, cudaMemsetAsync(h->d_nfrust, 0, N * sizeof(int32_t), s));
        if (nsave > 0) NQCD_CUDA(h, cudaMemsetAsync(h->d_partial, 0, nwarps * nsave * 4 * sizeof(double), s));
        if (h->cfg.nbeads_max > 1) {
            // ring polymer: normal modes and half-step Cayley matrices (cayley_propagator(half=true),
            // ring_polymer.jl:71-82: the square root of the full step, (C + I) / sqrt(tr C + 2) as det C = 1)
            const int nb = h->cfg.nbeads_max;
            std::vector<double> tab((size_t)nb * nb + 4 * (size_t)nb);
            nm_transform_matrix(nb, tab.data());
            double* hc = tab.data() + (size_t)nb * nb;
            cayley_matrices(nb, h->cfg.beta, dt, hc);
            for (int k = 0; k < nb; ++k) {
                double* c = hc + 4 * k;
                const double sc = 1.0 / sqrt(c[0] + c[3] + 2.0);
                c[0] = (c[0] + 1.0) * sc;
                c[1] = c[1] * sc;
                c[2] = c[2] * sc;
                c[3] = (c[3] + 1.0) * sc;
            }
            NQCD_CUDA(h, cudaMemcpyAsync(h->d_rptab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, s));
            NQCD_CUDA(h, cudaMemsetAsync(h->d_energy, 0, 2 * N * sizeof(double), s));
            mp.nbeads = nb;
            mp.rp_U = h->d_rptab;
            mp.rp_half = h->d_rptab + (size_t)nb * nb;
            mp.energy = nullptr;
            mp.obs_partial = nullptr;
        }
        NQCD_CUDA(h, cudaEventRecord(h->evk0, s));
        e = h->cfg.precision == NQCD_PREC_FP64 ? launch_mdef_fp64(mp, s) : launch_mdef_fp32(mp, s);
    } else if (r_host) {
        const int rc = run_pipelined(h, p, lanes, blk, r_host, v_host, &h2d, &launches);
        if (rc) return rc;
        --launches;  // counted per chunk
    } else {
        NQCD_CUDA(h, cudaEventRecord(h->evk0, s));
        e = h->cfg.precision == NQCD_PREC_FP64   ? launch_fssh2_fp64(p, s)
            : h->cfg.precision == NQCD_PREC_FP32 ? launch_fssh2_fp32(p, s)
                                                 : launch_fssh2_fp32_kahan(p, s);
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "nqcd_run: ensemble kernel launch");
    NQCD_CUDA(h, cudaEventRecord(h->evk1, s));
    ++launches;
    if (nsave > 0) {
        const int64_t need = reduce_chunks(nwarps, (int64_t)nsave * 4) * nsave * 4;
        if (need > h->redtmp_cap) {
            NQCD_CUDA(h, cudaStreamSynchronize(s));
            if (h->d_redtmp) cudaFree(h->d_redtmp);
            h->d_redtmp = nullptr;
            h->redtmp_cap = 0;
            NQCD_CUDA(h, dalloc(&h->d_redtmp, need));
            h->redtmp_cap = need;
        }
        // the fast FSSH / Ehrenfest kernels write FP32 partial sums
        const bool partial_f32 = !mdef && !iesh && h->cfg.precision != NQCD_PREC_FP64;
        if (partial_f32)
            NQCD_CUDA(h, launch_reduce_partials(reinterpret_cast<const float*>(h->d_partial), nwarps, (int64_t)nsave * 4,
                                                h->d_redtmp, h->d_popcorr, s));
        else
            NQCD_CUDA(h, launch_reduce_partials(h->d_partial, nwarps, (int64_t)nsave * 4, h->d_redtmp, h->d_popcorr, s));
        ++launches;
        ++launches;
    }
    stats_kernel<<<(unsigned)((N + 255) / 256 < 1024 ? (N + 255) / 256 : 1024), 256, 0, s>>>(
        h->d_nsteps, h->d_nhops, h->d_nfrust, h->d_r, h->d_v, nd, N, h->d_counts + 4, h->d_fp64steps,
        h->d_counts + 12);
    NQCD_CUDA(h, cudaGetLastError());
    ++launches;
    // Ehrenfest scattering: population sums in a fixed order (buffers sized before the run)
    const bool ehr_scatter = h->cfg.method == NQCD_METHOD_EHRENFEST && out && out->scattering;
    double esc[4] = {0.0, 0.0, 0.0, 0.0};
    if (ehr_scatter) {
        ehrenfest_scatter_kernel<<<(unsigned)((N + 255) / 256 < 1024 ? (N + 255) / 256 : 1024), 256, 0, s>>>(
            h->d_r, h->d_sig, N, h->d_stage);
        NQCD_CUDA(h, cudaGetLastError());
        NQCD_CUDA(h, launch_reduce_partials(h->d_stage, N, 4, h->d_redtmp, h->d_stage + 4 * N, s));
        NQCD_CUDA(h, cudaMemcpyAsync(esc, h->d_stage + 4 * N, sizeof(esc), cudaMemcpyDeviceToHost, s));
        launches += 3;
    }
    NQCD_CUDA(h, cudaEventRecord(h->ev1, s));

    unsigned long long counts[24];
    int64_t d2h = 0;
    NQCD_CUDA(h, cudaMemcpyAsync(counts, h->d_counts, sizeof(counts), cudaMemcpyDeviceToHost, s));
    d2h += sizeof(counts);
    std::vector<double> pc;
    if (out && ((mdef || iesh) ? out->observables : out->population_correlation) && nsave > 0) {
        pc.resize((size_t)nsave * 4);
        NQCD_CUDA(h, cudaMemcpyAsync(pc.data(), h->d_popcorr, pc.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        d2h += (int64_t)pc.size() * sizeof(double);
    }
    NQCD_CUDA(h, cudaStreamSynchronize(s));
    float ms = 0.0f, kms = 0.0f;
    NQCD_CUDA(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    NQCD_CUDA(h, cudaEventElapsedTime(&kms, h->evk0, h->evk1));
    if (out) {
        out->nsave = nsave;
        if (out->scattering)
            for (int q = 0; q < 4; ++q)
                out->scattering[q] = (ehr_scatter ? esc[q] : (double)counts[q]) / (double)N;
        double* dst = (mdef || iesh) ? out->observables : out->population_correlation;
        if (dst && nsave > 0)
            for (int k = 0; k < nsave * 4; ++k) dst[k] = pc[k] / (double)N;
    }
    h->nsave_last = nsave;
    h->has_run = true;
    if (stats) {
        stats->traj_steps = mdef ? N * nsteps : (int64_t)counts[4];
        stats->exact_friction_evals = mdef ? (int64_t)counts[8] : 0;
        stats->surrogate_friction_evals = mdef ? (int64_t)counts[9] : 0;
        stats->unconverged_roots = (int64_t)counts[10];
        stats->hop_evaluations = iesh ? (int64_t)counts[8] : 0;
        stats->propagator_terms = iesh ? (int64_t)counts[9] : 0;
        stats->overlap_factorizations = iesh ? (int64_t)counts[13] : 0;
        stats->hops = (int64_t)counts[5];
        stats->frustrated = (int64_t)counts[6];
        stats->flagged = (int64_t)counts[7];
        stats->electronics_fp64_steps = h->d_fp64steps ? (int64_t)counts[12] : 0;
        stats->surrogate_judged = mdef ? (int64_t)counts[16] : 0;
        stats->surrogate_rejected = mdef ? (int64_t)counts[17] : 0;
        double emax = 0.0, esum = 0.0;
        memcpy(&emax, &counts[18], sizeof(double));
        memcpy(&esum, &counts[19], sizeof(double));
        stats->surrogate_max_rel_error = mdef ? emax : 0.0;
        stats->surrogate_mean_rel_error = (mdef && counts[16] > 0) ? esum / (double)counts[16] : 0.0;
        stats->device_ms = ms;
        stats->kernel_ms = kms;
        stats->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
        stats->h2d_bytes = h2d;
        stats->d2h_bytes = d2h;
        stats->kernel_launches = launches;
    }
    if (iesh && counts[11] > 0)
        return fail(h, NQCD_ERR_TIMEOUT, "nqcd_run: a wait for the tensor-core propagator gave up");
    if (counts[7] > 0) return fail(h, NQCD_ERR_NAN, "nqcd_run: non-finite final positions or velocities");
    return NQCD_OK;
}

int nqcd_run(nqcd_handle* h, double t0, double t1, double dt, uint64_t seed, nqcd_outputs* out, nqcd_stats* stats) {
    return run_impl(h, t0, t1, dt, seed, out, stats, nullptr, nullptr);
}

int nqcd_run_host(nqcd_handle* h, int64_t ntraj, const double* r0, const double* v0, double t0, double t1, double dt,
                  uint64_t seed, nqcd_outputs* out, nqcd_stats* stats) {
    if (!h) return NQCD_ERR_ARG;
    if (!pipelined_config(h)) {
        const int rc = nqcd_set_initial(h, ntraj, r0, v0, nullptr, nullptr, nullptr, nullptr);
        return rc ? rc : nqcd_run(h, t0, t1, dt, seed, out, stats);
    }
    if (ntraj <= 0 || ntraj > h->cap) return fail(h, NQCD_ERR_ARG, "nqcd_run_host: ntraj outside 1..ntraj_max");
    if (!r0 || !v0) return fail(h, NQCD_ERR_ARG, "nqcd_run_host: r0 and v0 are required");
    if (!(dt > 0.0) || !(t1 >= t0) || !isfinite(t0) || !isfinite(t1))
        return fail(h, NQCD_ERR_ARG, "nqcd_run: need dt > 0 and finite t0 <= t1");
    // the handle's state as nqcd_set_initial leaves it; the positions and velocities arrive in the run
    int64_t h2d = 0;
    const int rc = set_initial_common(h, ntraj, nullptr, nullptr, nullptr, &h2d);
    if (rc) return rc;
    const int rr = run_impl(h, t0, t1, dt, seed, out, stats, r0, v0);
    // a run that failed on the device may not have copied the initial conditions: a later
    // nqcd_run must not start from the previous ones (a non-finite final state, NQCD_ERR_NAN,
    // leaves them in place)
    if (rr == NQCD_ERR_CUDA || rr == NQCD_ERR_OOM || rr == NQCD_ERR_TIMEOUT) h->initial_set = false;
    return rr;
}

int nqcd_get_final(nqcd_handle* h, double* r, double* v, double* sig_re, double* sig_im, int32_t* state,
                   int32_t* nhops, int32_t* nfrustrated, int32_t* nsteps, double* energy) {
    if (!h) return NQCD_ERR_ARG;
    if (!h->has_run) return fail(h, NQCD_ERR_STATE, "nqcd_get_final: no completed run");
    const int64_t N = h->ntraj, nd = h->ndof;
    cudaStream_t s = h->stream;
    int rc = ensure_stage(h, std::max<int64_t>(nd * N, 8 * N));
    if (rc) return rc;
    double* pairs[2] = {r, v};
    double* srcs[2] = {h->d_r, h->d_v};
    for (int q = 0; q < 2; ++q) {
        if (!pairs[q]) continue;
        NQCD_CUDA(h, transpose(srcs[q], h->d_stage, nd, N, s));
        NQCD_CUDA(h, cudaMemcpyAsync(pairs[q], h->d_stage, nd * N * sizeof(double), cudaMemcpyDeviceToHost, s));
        NQCD_CUDA(h, cudaStreamSynchronize(s));
    }
    if (h->cfg.method == NQCD_METHOD_IESH || h->cfg.method == NQCD_METHOD_EHRENFEST_NA) {
        const int64_t ne = h->nelec, ns = h->nstates;
        if (sig_re) NQCD_CUDA(h, cudaMemcpyAsync(sig_re, h->d_psi_re, ne * ns * N * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (sig_im) NQCD_CUDA(h, cudaMemcpyAsync(sig_im, h->d_psi_im, ne * ns * N * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (state) {
            std::vector<int32_t> soa((size_t)(ne * N));
            NQCD_CUDA(h, cudaMemcpyAsync(soa.data(), h->d_occ, soa.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            NQCD_CUDA(h, cudaStreamSynchronize(s));
            for (int64_t t = 0; t < N; ++t)
                for (int64_t j = 0; j < ne; ++j) state[t * ne + j] = soa[(size_t)(j * N + t)];
            state = nullptr;  // written
        }
        sig_re = sig_im = nullptr;
    }
    if (sig_re || sig_im) {
        std::vector<double> soa(8 * N);
        NQCD_CUDA(h, cudaMemcpyAsync(soa.data(), h->d_sig, 8 * N * sizeof(double), cudaMemcpyDeviceToHost, s));
        NQCD_CUDA(h, cudaStreamSynchronize(s));
        for (int64_t t = 0; t < N; ++t)
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j) {
                    if (sig_re) sig_re[t * 4 + i + 2 * j] = soa[(2 * (2 * i + j)) * N + t];
                    if (sig_im) sig_im[t * 4 + i + 2 * j] = soa[(2 * (2 * i + j) + 1) * N + t];
                }
    }
    struct {
        int32_t* dst;
        int32_t* src;
    } ints[4] = {{state, h->d_state}, {nhops, h->d_nhops}, {nfrustrated, h->d_nfrust}, {nsteps, h->d_nsteps}};
    for (auto& q : ints)
        if (q.dst) NQCD_CUDA(h, cudaMemcpyAsync(q.dst, q.src, N * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (energy) {
        NQCD_CUDA(h, transpose(h->d_energy, h->d_stage, 2, N, s));
        NQCD_CUDA(h, cudaMemcpyAsync(energy, h->d_stage, 2 * N * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    NQCD_CUDA(h, cudaStreamSynchronize(s));
    return NQCD_OK;
}

// Exact force and friction at n host positions, in chunks of the handle's capacity.
static int mdef_eval_device(nqcd_handle* h, const double* d_x, int64_t n, double* d_force, double* d_fric) {
    MdefParams m = mdef_params(h, n, 1.0, 0, 0, 0, 0);
    m.x = const_cast<double*>(d_x);
    m.v = d_fric;  // unused in evaluation mode
    m.energy = nullptr;
    m.obs_partial = nullptr;
    m.use_mlp = 0;
    m.force_out = d_force;
    m.friction_out = d_fric;
    cudaError_t e = h->cfg.precision == NQCD_PREC_FP64 ? launch_mdef_fp64(m, h->stream) : launch_mdef_fp32(m, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "MDEF evaluation kernel");
    return NQCD_OK;
}

int nqcd_mdef_evaluate(nqcd_handle* h, int64_t n, const double* x, double* force, double* friction) {
    if (!h || !x || n <= 0) return NQCD_ERR_ARG;
    if (h->cfg.method != NQCD_METHOD_MDEF) return fail(h, NQCD_ERR_UNSUPPORTED, "nqcd_mdef_evaluate: MDEF handles only");
    int rc = ensure_stage(h, 3 * n);
    if (rc) return rc;
    double *dx = h->d_stage, *dF = h->d_stage + n, *dG = h->d_stage + 2 * n;
    NQCD_CUDA(h, cudaMemcpyAsync(dx, x, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    rc = mdef_eval_device(h, dx, n, dF, dG);
    if (rc) return rc;
    if (force) NQCD_CUDA(h, cudaMemcpyAsync(force, dF, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (friction) NQCD_CUDA(h, cudaMemcpyAsync(friction, dG, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    return NQCD_OK;
}

// Friction floor of the surrogate's judge: 0.1 x the largest exact friction
// on 257 evenly spaced points of the network's domain (relative errors of
// judged values are taken against max(|exact|, floor), so that a region of
// vanishing friction does not turn rounding into a rejection).
static int mlp_set_friction_floor(nqcd_handle* h) {
    const int64_t n = 257;
    int rc = ensure_stage(h, 3 * n);
    if (rc) return rc;
    std::vector<double> xs(n), G(n);
    for (int64_t i = 0; i < n; ++i) xs[i] = h->mlp.lo + (h->mlp.hi - h->mlp.lo) * (double)i / (double)(n - 1);
    double *dx = h->d_stage, *dF = h->d_stage + n, *dG = h->d_stage + 2 * n;
    NQCD_CUDA(h, cudaMemcpyAsync(dx, xs.data(), n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    rc = mdef_eval_device(h, dx, n, dF, dG);
    if (rc) return rc;
    NQCD_CUDA(h, cudaMemcpyAsync(G.data(), dG, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    double gmax = 0.0;
    for (double g : G) gmax = fabs(g) > gmax ? fabs(g) : gmax;
    h->mlp.friction_floor = gmax > 0.0 ? 0.1 * gmax : 1e-300;
    return NQCD_OK;
}

__global__ void uniform_positions_kernel(double* x, int64_t n, double lo, double hi, uint64_t seed) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = lo + (hi - lo) * rng_uniform(seed, (uint64_t)i, 0u, 9u);
}

__global__ void cholesky_target_kernel(const double* fric, double* L, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) L[i] = sqrt(fric[i] > 0.0 ? fric[i] : 0.0);
}

int nqcd_train_friction_mlp(nqcd_handle* h, double x_lo, double x_hi, int64_t npoints, int32_t epochs, int32_t batch,
                            double learning_rate, uint64_t seed, double* final_loss) {
    if (!h) return NQCD_ERR_ARG;
    if (h->cfg.method != NQCD_METHOD_MDEF || h->cfg.model != NQCD_MODEL_NEWNS_ANDERSON)
        return fail(h, NQCD_ERR_UNSUPPORTED, "nqcd_train_friction_mlp: MDEF handles of the one-dimensional model only");
    if (!(x_hi > x_lo) || npoints < 16 || epochs < 1 || batch < 16 || batch > 65536 || !(learning_rate > 0))
        return fail(h, NQCD_ERR_ARG, "nqcd_train_friction_mlp: bad domain, sizes or learning rate");
    cudaStream_t s = h->stream;
    if (!h->mlp.master) {
        cudaError_t e = mlp_alloc(h->mlp, 65536);
        if (e != cudaSuccess) return cuda_fail(h, e, "nqcd_train_friction_mlp: allocation");
    }
    double *dx = nullptr, *dF = nullptr, *dG = nullptr, *dL = nullptr;
    auto release = [&]() {  // cudaFree(nullptr) is a no-op
        cudaFree(dx);
        cudaFree(dF);
        cudaFree(dG);
        cudaFree(dL);
    };
    {
        cudaError_t ea = dalloc(&dx, npoints);
        if (ea == cudaSuccess) ea = dalloc(&dF, npoints);
        if (ea == cudaSuccess) ea = dalloc(&dG, npoints);
        if (ea == cudaSuccess) ea = dalloc(&dL, npoints);
        if (ea != cudaSuccess) {
            release();
            return cuda_fail(h, ea, "nqcd_train_friction_mlp: allocation");
        }
    }
    uniform_positions_kernel<<<(unsigned)((npoints + 255) / 256), 256, 0, s>>>(dx, npoints, x_lo, x_hi, seed);
    int rc = mdef_eval_device(h, dx, npoints, dF, dG);  // training data from the method itself
    if (rc) {
        release();
        return rc;
    }
    cholesky_target_kernel<<<(unsigned)((npoints + 255) / 256), 256, 0, s>>>(dG, dL, npoints);
    // output bias starts at the mean target so that training starts near the data
    std::vector<double> Lh(npoints);
    cudaError_t e = cudaMemcpyAsync(Lh.data(), dL, npoints * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        release();
        return cuda_fail(h, e, "nqcd_train_friction_mlp: targets");
    }
    double mean = 0.0;
    for (double v : Lh) mean += v;
    mean /= (double)npoints;
    float bias = (float)(mean > 20.0 ? mean : log(expm1(mean > 1e-6 ? mean : 1e-6)));  // inverse softplus
    h->mlp.shift = 0.5 * (x_lo + x_hi);
    h->mlp.scale = 2.0 / (x_hi - x_lo);
    h->mlp.lo = x_lo;
    h->mlp.hi = x_hi;
    e = mlp_init_weights(h->mlp, seed, bias, s);
    if (e == cudaSuccess) {
        int64_t nsteps = (int64_t)epochs * ((npoints + batch - 1) / batch);
        e = mlp_train_device(h->mlp, dx, dL, npoints, nsteps, batch, (float)learning_rate, seed, s, final_loss);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    release();
    if (e != cudaSuccess) return cuda_fail(h, e, "nqcd_train_friction_mlp: training");
    rc = mlp_set_friction_floor(h);
    if (rc) return rc;
    h->mlp.trained = true;
    return NQCD_OK;
}

int nqcd_mlp_get(nqcd_handle* h, float* params, double* meta) {
    if (!h || !params) return NQCD_ERR_ARG;
    if (!h->mlp.master) return fail(h, NQCD_ERR_STATE, "nqcd_mlp_get: no network");
    NQCD_CUDA(h, cudaMemcpyAsync(params, h->mlp.master, kMlpN * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    if (meta) {
        meta[0] = h->mlp.shift;
        meta[1] = h->mlp.scale;
        meta[2] = h->mlp.lo;
        meta[3] = h->mlp.hi;
    }
    return NQCD_OK;
}

int nqcd_mlp_set(nqcd_handle* h, const float* params, const double* meta) {
    if (!h || !params || !meta) return NQCD_ERR_ARG;
    if (h->cfg.method != NQCD_METHOD_MDEF || h->cfg.model != NQCD_MODEL_NEWNS_ANDERSON)
        return fail(h, NQCD_ERR_UNSUPPORTED, "nqcd_mlp_set: MDEF handles of the one-dimensional model only");
    if (!isfinite(meta[0]) || !(meta[1] > 0.0 && meta[1] < 1e300) || !isfinite(meta[2]) || !isfinite(meta[3]) ||
        !(meta[3] > meta[2]))
        return fail(h, NQCD_ERR_ARG, "nqcd_mlp_set: need finite shift, scale > 0 and a domain lo < hi");
    if (!h->mlp.master) {
        cudaError_t e = mlp_alloc(h->mlp, 65536);
        if (e != cudaSuccess) return cuda_fail(h, e, "nqcd_mlp_set: allocation");
    }
    NQCD_CUDA(h, cudaMemcpyAsync(h->mlp.master, params, kMlpN * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    NQCD_CUDA(h, mlp_sync_bf16(h->mlp, h->stream));
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    h->mlp.shift = meta[0];
    h->mlp.scale = meta[1];
    h->mlp.lo = meta[2];
    h->mlp.hi = meta[3];
    int rc = mlp_set_friction_floor(h);
    if (rc) return rc;
    h->mlp.trained = true;
    return NQCD_OK;
}

int nqcd_mlp_loss_grad(nqcd_handle* h, int64_t n, const double* x, const double* target_L, double* loss, float* grad) {
    if (!h || !x || !target_L || n <= 0 || n > 65536) return NQCD_ERR_ARG;
    if (!h->mlp.master) return fail(h, NQCD_ERR_STATE, "nqcd_mlp_loss_grad: no network");
    int rc = ensure_stage(h, 2 * n);
    if (rc) return rc;
    NQCD_CUDA(h, cudaMemcpyAsync(h->d_stage, x, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    NQCD_CUDA(h, cudaMemcpyAsync(h->d_stage + n, target_L, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    NQCD_CUDA(h, mlp_loss_grad_device(h->mlp, h->d_stage, h->d_stage + n, (int)n, h->stream));
    std::vector<float> g(kMlpN + 1);
    NQCD_CUDA(h, cudaMemcpyAsync(g.data(), h->mlp.grad, g.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    if (grad) memcpy(grad, g.data(), kMlpN * sizeof(float));
    if (loss) *loss = g[kMlpN];
    return NQCD_OK;
}

int nqcd_set_mapping(nqcd_handle* h, const nqcd_mapping* m) {
    if (!h || !m) return NQCD_ERR_ARG;
    if (m->sb_lanes != 0 && m->sb_lanes != 4 && m->sb_lanes != 8)
        return fail(h, NQCD_ERR_ARG, "nqcd_set_mapping: sb_lanes must be 0, 4 or 8");
    if (m->sb_block != 0 && m->sb_block != 64 && m->sb_block != 128 && m->sb_block != 256)
        return fail(h, NQCD_ERR_ARG, "nqcd_set_mapping: sb_block must be 0, 64, 128 or 256");
    static const int kAllowed[4][4] = {{1, 2, 4, 0}, {2, 4, 8, 0}, {4, 8, 16, 0}, {4, 8, 16, 32}};
    for (int q = 0; q < 4; ++q) {
        bool ok = m->rp_lanes[q] == 0;
        for (int a = 0; a < 4; ++a) ok |= kAllowed[q][a] != 0 && m->rp_lanes[q] == kAllowed[q][a];
        if (!ok) return fail(h, NQCD_ERR_ARG, "nqcd_set_mapping: rp_lanes outside the shapes of its bead count");
    }
    if (m->rp_one_launch != 0 && m->rp_one_launch != 1)
        return fail(h, NQCD_ERR_ARG, "nqcd_set_mapping: rp_one_launch must be 0 or 1");
    if (m->iesh_cores != 0 && m->iesh_cores != 1)
        return fail(h, NQCD_ERR_ARG, "nqcd_set_mapping: iesh_cores must be 0 (tensor cores) or 1 (CUDA cores)");
    if (m->iesh_lu_always != 0 && m->iesh_lu_always != 1)
        return fail(h, NQCD_ERR_ARG, "nqcd_set_mapping: iesh_lu_always must be 0 or 1");
    if (m->sb_lanes == 8) {
        const bool sb = h->cfg.model == NQCD_MODEL_SPINBOSON && h->cfg.method != NQCD_METHOD_RPSH;
        if (sb && (h->cfg.precision != NQCD_PREC_FP32_KAHAN || h->cfg.nbath > 128))
            return fail(h, NQCD_ERR_UNSUPPORTED,
                        "nqcd_set_mapping: 8 lanes per trajectory need NQCD_PREC_FP32_KAHAN and at most 128 modes");
    }
    h->map = *m;
    return NQCD_OK;
}

int nqcd_set_trajectory_models(nqcd_handle* h, const int32_t* models) {
    if (!h || !models) return NQCD_ERR_ARG;
    if (h->cfg.method != NQCD_METHOD_RPSH)
        return fail(h, NQCD_ERR_UNSUPPORTED, "nqcd_set_trajectory_models: ring-polymer handles only");
    if (!h->initial_set) return fail(h, NQCD_ERR_STATE, "nqcd_set_trajectory_models: call nqcd_set_initial first");
    for (int64_t t = 0; t < h->ntraj; ++t)
        if (models[t] < NQCD_MODEL_TULLY1 || models[t] > NQCD_MODEL_TULLY3)
            return fail(h, NQCD_ERR_UNSUPPORTED, "nqcd_set_trajectory_models: Tully models 1-3 only");
    h->traj_models.assign(models, models + h->ntraj);
    int64_t h2d = 0;
    h->has_run = false;
    return build_rp_classes(h, &h2d);
}

int nqcd_get_hop_log(nqcd_handle* h, int32_t* log) {
    if (!h || !log) return NQCD_ERR_ARG;
    if (!h->has_run) return fail(h, NQCD_ERR_STATE, "nqcd_get_hop_log: no completed run");
    if (!h->d_hoplog) return fail(h, NQCD_ERR_STATE, "nqcd_get_hop_log: created with max_hops = 0");
    const int64_t N = h->ntraj, w = (int64_t)h->cfg.max_hops * 3;
    std::vector<int32_t> soa(w * N);
    NQCD_CUDA(h, cudaMemcpyAsync(soa.data(), h->d_hoplog, soa.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    NQCD_CUDA(h, cudaStreamSynchronize(h->stream));
    for (int64_t t = 0; t < N; ++t)
        for (int64_t c = 0; c < w; ++c) log[t * w + c] = soa[c * N + t];
    return NQCD_OK;
}

const char* nqcd_last_error(const nqcd_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

void nqcd_destroy(nqcd_handle* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
}

int nqcd_pin_host(void* ptr, int64_t bytes) {
    if (!ptr || bytes <= 0) return NQCD_ERR_ARG;
    cudaError_t e = cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "nqcd_pin_host");
    return NQCD_OK;
}

int nqcd_unpin_host(void* ptr) {
    if (!ptr) return NQCD_ERR_ARG;
    cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "nqcd_unpin_host");
    return NQCD_OK;
}

int nqcd_measure_fma_peaks(double* fp64_tflops, double* fp32_tflops) {
    if (!fp64_tflops || !fp32_tflops) return NQCD_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return cuda_fail(nullptr, cudaGetLastError(), "nqcd_measure_fma_peaks");
    double* sink64 = nullptr;
    float* sink32 = nullptr;
    cudaEvent_t a, b;
    if (cudaMalloc(&sink64, 1024 * sizeof(double)) != cudaSuccess || cudaMalloc(&sink32, 1024 * sizeof(float)) != cudaSuccess) {
        const cudaError_t ea = cudaGetLastError();
        cudaFree(sink64);  // no-op when null
        return cuda_fail(nullptr, ea, "nqcd_measure_fma_peaks: alloc");
    }
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int threads = 256;
    const int blocks = sms * 8;
    auto run = [&](bool f64, int iters) -> double {
        // warm-up then timed launch
        for (int rep = 0; rep < 2; ++rep) {
            cudaEventRecord(a);
            if (f64)
                fma_peak_kernel<double><<<blocks, threads>>>(sink64, iters, 1.0);
            else
                fma_peak_kernel<float><<<blocks, threads>>>(sink32, iters, 1.0f);
            cudaEventRecord(b);
            cudaEventSynchronize(b);
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        double flops = 2.0 * 8.0 * 16.0 * (double)iters * (double)threads * (double)blocks;
        return flops / (ms * 1e-3) / 1e12;
    };
    *fp64_tflops = run(true, 256);
    *fp32_tflops = run(false, 4096);
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink64);
    cudaFree(sink32);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "nqcd_measure_fma_peaks: kernel");
    return NQCD_OK;
}

}  // extern "C"

namespace nqcd {
int64_t reduce_chunks(int64_t nparts, int64_t width) {
    const int64_t colblocks = (width + 127) / 128;
    int64_t chunks = 2048 / (colblocks > 0 ? colblocks : 1);  // about 2048 blocks in the first pass
    if (chunks < 1) chunks = 1;
    if (chunks > 65535) chunks = 65535;
    return chunks < nparts ? chunks : (nparts > 0 ? nparts : 1);
}

template <typename T>
static cudaError_t reduce_partials_t(const T* partial, int64_t nparts, int64_t width, double* tmp, double* out,
                                     cudaStream_t s) {
    const int64_t chunks = reduce_chunks(nparts, width);
    const int64_t rows = (nparts + chunks - 1) / chunks;
    dim3 grid((unsigned)((width + 127) / 128), (unsigned)chunks);
    reduce_chunks_kernel<<<grid, 128, 0, s>>>(partial, nparts, width, rows, tmp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    reduce_partials_kernel<<<(unsigned)((width + 127) / 128), 128, 0, s>>>(tmp, chunks, width, out);
    return cudaGetLastError();
}

cudaError_t launch_reduce_partials(const double* partial, int64_t nparts, int64_t width, double* tmp, double* out,
                                   cudaStream_t s) {
    return reduce_partials_t(partial, nparts, width, tmp, out, s);
}

cudaError_t launch_reduce_partials(const float* partial, int64_t nparts, int64_t width, double* tmp, double* out,
                                   cudaStream_t s) {
    return reduce_partials_t(partial, nparts, width, tmp, out, s);
}
}  // namespace nqcd
