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

// One persistent launch for every bead count (the mapping's rp_one_launch):
// each block starts on the class the host gave it and then helps the other
// classes as their queues drain (a refill of the whole grid), calling the
// class loop of its bead count's default lane-group shape.  The loops are
// not inlined, so each keeps its own register allocation, but the launch
// reserves the registers of the largest for every warp; the autotuner times
// this against the concurrent per-bead-count kernels.
template <int Q, int GL>
static __device__ __noinline__ void rp_serve_class_call(const RpshParams& p, int cls) {
    rp_serve_class<Q, GL>(p, cls);
}

__global__ void __launch_bounds__(kRpshBlock) rpsh_one_launch_kernel(const RpshParams p) {
    int cls = p.block_class[blockIdx.x];
    for (int visited = 0; visited < p.nclass; ++visited, cls = (cls + 1) % p.nclass) {
        switch (p.class_beads[cls]) {
            case 1: rp_serve_class_call<1, 1>(p, cls); break;
            case 2: rp_serve_class_call<1, 2>(p, cls); break;
            case 4: rp_serve_class_call<1, 4>(p, cls); break;
            case 5: rp_serve_class_call<5, 1>(p, cls); break;
            case 8: rp_serve_class_call<2, 4>(p, cls); break;
            case 10: rp_serve_class_call<5, 2>(p, cls); break;
            case 16: rp_serve_class_call<4, 4>(p, cls); break;
            case 32: rp_serve_class_call<8, 4>(p, cls); break;
            default: break;  // the host admits only these bead counts
        }
    }
}

int rpsh_one_launch_grid() {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, rpsh_one_launch_kernel, kRpshBlock, 0);
    return sms * (per > 0 ? per : 1);
}

cudaError_t launch_rpsh_one(const RpshParams& p, int blocks, cudaStream_t s) {
    rpsh_one_launch_kernel<<<blocks, kRpshBlock, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace nqcd
