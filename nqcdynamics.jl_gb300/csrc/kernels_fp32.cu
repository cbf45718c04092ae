// Fast path: FP32 Hamiltonian, eigen-decomposition, couplings and density
// matrix propagation; FP64 position/velocity accumulation and observables.
// Built with multiply-add contraction enabled.
#include "fssh2_kernels.cuh"

namespace nqcd {

cudaError_t launch_fssh2_fp32(const FsshParams& p, cudaStream_t s) { return launch_fssh2<float>(p, s); }

}  // namespace nqcd
