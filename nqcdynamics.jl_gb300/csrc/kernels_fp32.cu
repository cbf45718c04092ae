// Fast paths: FP32 Hamiltonian, eigen-decomposition, couplings and density
// matrix propagation; positions and velocities accumulated in FP64
// (NQCD_PREC_FP32) or in Kahan-compensated FP32 (NQCD_PREC_FP32_KAHAN);
// observables accumulated in FP64.  Built with multiply-add contraction
// enabled (the compensated sums use explicitly rounded intrinsics).
#include "fssh2_sb_fast.cuh"
#include "mdef_kernels.cuh"
#include "rpsh_kernels.cuh"

namespace nqcd {

cudaError_t launch_fssh2_fp32(const FsshParams& p, cudaStream_t s) {
    if (p.model == MODEL_SPINBOSON) return launch_sb_fast<AccF64>(p, s);
    return launch_fssh2<float>(p, s);
}

cudaError_t launch_fssh2_fp32_kahan(const FsshParams& p, cudaStream_t s) {
    if (p.model == MODEL_SPINBOSON) return launch_sb_fast<AccKahan>(p, s);
    return launch_fssh2<float>(p, s);
}

// The per-thread stack limit must cover the kernel's spilled bead arrays.
static cudaError_t ensure_rpsh_stack_fp32() {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, rpsh_persistent_kernel<float>);
    if (e != cudaSuccess) return e;
    size_t cur = 0;
    e = cudaDeviceGetLimit(&cur, cudaLimitStackSize);
    if (e != cudaSuccess) return e;
    size_t need = a.localSizeBytes;
    if (cur < need) e = cudaDeviceSetLimit(cudaLimitStackSize, need);
    return e;
}

int rpsh_grid_fp32() {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, rpsh_persistent_kernel<float>, kRpshBlock, 0);
    return sms * (per > 0 ? per : 1);
}

cudaError_t launch_rpsh_fp32(const RpshParams& p, int blocks, cudaStream_t s) {
    cudaError_t e = ensure_rpsh_stack_fp32();
    if (e != cudaSuccess) return e;
    return launch_rpsh<float>(p, blocks, s);
}

cudaError_t launch_mdef_fp32(const MdefParams& p, cudaStream_t s) { return launch_mdef<float>(p, s); }

}  // namespace nqcd
