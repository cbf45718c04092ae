// Allocation-free entry point: the plain FP64 spin-boson FSSH ensemble
// kernel with its per-mode coupling scratch in a fixed device array.
//
// Why: some hosts of this library cannot call cudaMalloc once they are
// running -- a Julia host whose CUDA.jl memory pool owns all device memory,
// a service that reserves its device memory at start-up and forbids later
// allocation, or code that must not allocate while another library captures
// the stream.  The handle API allocates state and scratch in nqcd_create, so
// it is not usable there; this entry point works on the caller's device
// buffers for inputs and outputs and allocates nothing, on the device or on
// the host.
//
// The scratch (one double per bath mode and trajectory, written and then read
// within each nuclear step) is g_noalloc_scratch below: a file-scope
// __device__ array of NQCD_NOALLOC_SCRATCH_DOUBLES doubles (8 MiB) that every
// GPU which loads this library holds until the process exits.  All calls
// share it and it keeps the last call's contents; nothing in it needs to
// start at zero.  Two calls whose kernels overlap on the GPU (different
// streams, or different host threads on one device) race on it.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include "../../include/nqcd_gpu.h"
#include "engine_params.h"
#include "nqcd_math.h"
#include "nqcd_models.h"

namespace {

__device__ __align__(256) double g_noalloc_scratch[NQCD_NOALLOC_SCRATCH_DOUBLES];

int noalloc_fail(char* errbuf, int32_t len, int code, const char* msg, const char* detail = "") {
    if (errbuf && len > 0) snprintf(errbuf, (size_t)len, "nqcd_fssh_spinboson_fp64_noalloc: %s%s", msg, detail);
    return code;
}

// Device address of g_noalloc_scratch in the current context.  In host code
// the symbol's name is only a host-side stand-in, so the device address is
// looked up with cudaGetSymbolAddress, with the caller's device current.  It
// is looked up on every call (the lookup allocates nothing): after a device
// reset, or in another context on the same device, the module loads at a new
// address, so a cached address could go stale.
int scratch_address(double** out, char* errbuf, int32_t len) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return noalloc_fail(errbuf, len, NQCD_ERR_CUDA, "cudaGetSymbolAddress: ", cudaGetErrorString(e));
    }
    *out = static_cast<double*>(p);
    return NQCD_OK;
}

// Number of nuclear steps the kernel takes from t0 to t1 (its clock: whole
// steps of dt, a shortened last step, a time within 100 ulp of t1 snapped to
// t1), or -1 once it exceeds max_steps.  A dt below the spacing of doubles
// near t never advances the clock; the cap turns that into a rejection
// instead of a kernel that never ends.
int64_t bounded_step_count(double t0, double t1, double dt, int64_t max_steps) {
    int64_t n = 0;
    double t = t0;
    while (t < t1) {
        if (++n > max_steps) return -1;
        double h = (t1 - t) < dt ? (t1 - t) : dt;
        t = nqcd::snap_time(t + h, t1);
    }
    return n;
}

}  // namespace

extern "C" int nqcd_fssh_spinboson_fp64_noalloc(int64_t ntraj, int32_t nmodes, const double* d_bath_c,
                                                const double* d_bath_omega2, const double* d_mass, double eps,
                                                double delta, int32_t rescaling, int32_t diabatic_state,
                                                double* d_r, double* d_v, double* d_sigma, int32_t* d_state,
                                                int32_t* d_nhops, int32_t* d_nfrustrated, int32_t* d_nsteps,
                                                double t0, double t1, double dt, uint64_t seed, void* stream,
                                                char* errbuf, int32_t errbuf_len) {
    if (errbuf && errbuf_len > 0) errbuf[0] = '\0';
    if (ntraj <= 0 || nmodes <= 0)
        return noalloc_fail(errbuf, errbuf_len, NQCD_ERR_ARG, "ntraj and nmodes must be positive");
    if (ntraj > (int64_t)NQCD_NOALLOC_SCRATCH_DOUBLES / nmodes)
        return noalloc_fail(errbuf, errbuf_len, NQCD_ERR_ARG,
                            "nmodes * ntraj exceeds the fixed scratch of NQCD_NOALLOC_SCRATCH_DOUBLES "
                            "(1048576) doubles; split the ensemble or use the handle API");
    if (!d_bath_c || !d_bath_omega2 || !d_mass || !d_r || !d_v || !d_sigma || !d_state)
        return noalloc_fail(errbuf, errbuf_len, NQCD_ERR_ARG, "null device buffer");
    if (rescaling < 0 || rescaling > 2 || diabatic_state < 0 || diabatic_state > 1)
        return noalloc_fail(errbuf, errbuf_len, NQCD_ERR_ARG, "rescaling must be 0..2 and diabatic_state 0..1");
    if (!(dt > 0.0) || !(t1 >= t0) || !isfinite(t0) || !isfinite(t1))
        return noalloc_fail(errbuf, errbuf_len, NQCD_ERR_ARG, "need dt > 0 and finite t0 <= t1");
    // the kernel counts steps in 32-bit integers; the span bounds the count
    // before the clock is stepped through on the host
    if (!((t1 - t0) / dt < 2147483646.0))
        return noalloc_fail(errbuf, errbuf_len, NQCD_ERR_ARG, "more than 2^31 - 2 steps");
    if (bounded_step_count(t0, t1, dt, (int64_t)((t1 - t0) / dt) + 2) < 0)
        return noalloc_fail(errbuf, errbuf_len, NQCD_ERR_ARG,
                            "dt is below the spacing of doubles between t0 and t1, so the clock would not advance");

    double* scratch = nullptr;
    int rc = scratch_address(&scratch, errbuf, errbuf_len);
    if (rc != NQCD_OK) return rc;

    nqcd::FsshParams p;
    memset(&p, 0, sizeof(p));
    p.model = nqcd::MODEL_SPINBOSON;
    p.mp[0] = eps;
    p.mp[1] = delta;
    p.ndof = nmodes;
    p.mass = d_mass;
    p.bath_c = d_bath_c;
    p.bath_w2 = d_bath_omega2;
    p.rescaling = rescaling;
    p.init_kind = NQCD_INIT_DIABATIC_PURE;
    p.init_state = diabatic_state;
    p.ntraj = ntraj;
    p.traj_hi = ntraj;
    p.t0 = t0;
    p.t1 = t1;
    p.dt = dt;
    p.seed = seed;
    p.r = d_r;
    p.v = d_v;
    p.scratch = scratch;
    p.sigma = d_sigma;
    p.state = d_state;
    p.nhops = d_nhops;
    p.nfrustrated = d_nfrustrated;
    p.nsteps = d_nsteps;
    cudaError_t e = nqcd::launch_fssh2_fp64(p, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return noalloc_fail(errbuf, errbuf_len, NQCD_ERR_CUDA, "launch: ", cudaGetErrorString(e));
    return NQCD_OK;
}
