// IESH ensemble kernels, both precisions.  This translation unit keeps the
// compiler's default FMA contraction: the plain IESH path matches the oracle
// to rounding (its propagator is not the reference's eigendecomposition), so
// it gains nothing from -fmad=false and would run at half the FP64 rate.
#include "iesh_kernels.cuh"

namespace nqcd {

cudaError_t launch_iesh_fp64(const IeshParams& p, cudaStream_t s) { return launch_iesh<double>(p, s); }
cudaError_t launch_iesh_fp32(const IeshParams& p, cudaStream_t s) { return launch_iesh<float>(p, s); }

}  // namespace nqcd
