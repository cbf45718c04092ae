// Plain FP64 path.  Built with -fmad=false: no multiply-add contraction, so
// every operation rounds exactly as in the CPU oracle (bit-identical hop
// sequences and phase-space paths).
#include "fssh2_kernels.cuh"
#include "mdef_kernels.cuh"
#include "rpsh_kernels.cuh"

namespace nqcd {

cudaError_t launch_fssh2_fp64(const FsshParams& p, cudaStream_t s) { return launch_fssh2<double>(p, s); }

// The persistent ring-polymer kernel calls non-inlined per-bead-count
// trajectory functions; make sure this context's stack limit covers the
// kernel's local-memory requirement (the default is 1 KiB).
static cudaError_t ensure_rpsh_stack_fp64() {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, rpsh_persistent_kernel<double>);
    if (e != cudaSuccess) return e;
    size_t cur = 0;
    e = cudaDeviceGetLimit(&cur, cudaLimitStackSize);
    if (e != cudaSuccess) return e;
    size_t need = a.localSizeBytes;
    if (cur < need) e = cudaDeviceSetLimit(cudaLimitStackSize, need);
    return e;
}

int rpsh_grid_fp64() {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, rpsh_persistent_kernel<double>, kRpshBlock, 0);
    return sms * (per > 0 ? per : 1);
}

cudaError_t launch_rpsh_fp64(const RpshParams& p, int blocks, cudaStream_t s) {
    cudaError_t e = ensure_rpsh_stack_fp64();
    if (e != cudaSuccess) return e;
    return launch_rpsh_plain<double>(p, blocks, s);
}

cudaError_t launch_mdef_fp64(const MdefParams& p, cudaStream_t s) { return launch_mdef<double>(p, s); }

}  // namespace nqcd
