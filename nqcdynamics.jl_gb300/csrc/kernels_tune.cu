// Kernel shapes that a mapping (nqcd_set_mapping) may select besides the
// defaults: the fast spin-boson kernel with eight lanes per trajectory, and
// the fast ring-polymer kernels with other lane groups per bead count.  The
// autotuner (nqcd_gb300/autotune.py) times them against the defaults.  In a
// translation unit of their own so that they compile in parallel with the
// default kernels.
#include "fssh2_sb_fast.cuh"
#include "rpsh_kernels.cuh"

namespace nqcd {

cudaError_t launch_sb_fast_g8_kahan(const FsshParams& p, cudaStream_t s) {
    const int need = (p.ndof + 7) / 8;
    if (need <= 2) return launch_sb_fast_npl<AccKahan, 8, 2>(p, s);
    if (need <= 4) return launch_sb_fast_npl<AccKahan, 8, 4>(p, s);
    if (need <= 8) return launch_sb_fast_npl<AccKahan, 8, 8>(p, s);
    if (need <= 13) return launch_sb_fast_npl<AccKahan, 8, 13>(p, s);
    if (need <= 16) return launch_sb_fast_npl<AccKahan, 8, 16>(p, s);
    return cudaErrorInvalidValue;
}

#define NQCD_RP_TUNED_SHAPES(X) X(4, 1) X(2, 2) X(4, 2) X(1, 8) X(2, 8) X(1, 16) X(4, 8) X(2, 16) X(1, 32)

int rpsh_group_grid_tuned(int beads, int lanes) {
#define X(Q, GL) \
    if (beads == Q * GL && lanes == GL) return rpsh_group_grid_t<Q, GL>();
    NQCD_RP_TUNED_SHAPES(X)
#undef X
    return 0;
}

cudaError_t launch_rpsh_group_tuned(int beads, int lanes, const RpshParams& p, int blocks, cudaStream_t s) {
#define X(Q, GL)                                                    \
    if (beads == Q * GL && lanes == GL) {                           \
        rpsh_group_kernel<Q, GL><<<blocks, kRpshBlock, 0, s>>>(p); \
        return cudaGetLastError();                                  \
    }
    NQCD_RP_TUNED_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}
#undef NQCD_RP_TUNED_SHAPES

}  // namespace nqcd
