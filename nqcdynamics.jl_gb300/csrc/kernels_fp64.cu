// Plain FP64 path.  Built with -fmad=false: no multiply-add contraction, so
// every operation rounds exactly as in the CPU oracle (bit-identical hop
// sequences and phase-space paths).
#include "fssh2_kernels.cuh"

namespace nqcd {

cudaError_t launch_fssh2_fp64(const FsshParams& p, cudaStream_t s) { return launch_fssh2<double>(p, s); }

}  // namespace nqcd
