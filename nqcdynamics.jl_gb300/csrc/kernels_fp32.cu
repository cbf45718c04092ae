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
    return launch_tully_fast(p, s);
}

cudaError_t launch_fssh2_fp32_kahan(const FsshParams& p, cudaStream_t s) {
    if (p.model == MODEL_SPINBOSON) return launch_sb_fast<AccKahan>(p, s);
    return launch_tully_fast(p, s);
}

// Fast ring-polymer kernels, one per bead count (see rpsh_group_kernel): the
// default lane-group shapes here, the other shapes a mapping may select in
// kernels_tune.cu.
#define NQCD_RP_SHAPES(X) X(1, 1) X(1, 2) X(1, 4) X(5, 1) X(2, 4) X(5, 2) X(4, 4) X(8, 4)

int rpsh_group_grid(int beads, int lanes) {
#define X(Q, GL) \
    if (beads == Q * GL && (lanes == 0 || lanes == GL)) return rpsh_group_grid_t<Q, GL>();
    NQCD_RP_SHAPES(X)
#undef X
    return rpsh_group_grid_tuned(beads, lanes);
}

cudaError_t launch_rpsh_group(int beads, int lanes, const RpshParams& p, int blocks, cudaStream_t s) {
#define X(Q, GL)                                                    \
    if (beads == Q * GL && (lanes == 0 || lanes == GL)) {           \
        rpsh_group_kernel<Q, GL><<<blocks, kRpshBlock, 0, s>>>(p); \
        return cudaGetLastError();                                  \
    }
    NQCD_RP_SHAPES(X)
#undef X
    return launch_rpsh_group_tuned(beads, lanes, p, blocks, s);
}
#undef NQCD_RP_SHAPES

cudaError_t launch_mdef_fp32(const MdefParams& p, cudaStream_t s) { return launch_mdef<float>(p, s); }

}  // namespace nqcd
