// Tensor-core self-test: one 128 x 80 x 80 product D = A B on the fifth-
// generation tensor cores (tcgen05.mma kind::tf32, accumulator in TMEM), in
// one pass (A and B rounded to tf32) or split in three (3xTF32: A = Ah + Al,
// B = Bh + Bl, D = Ah Bh + Ah Bl + Al Bh, close to fp32 accuracy).  The shape
// is the one of the IESH propagator terms (an 80 x 80 coupling matrix padded
// to the MMA's 128 rows, times an 80 x 80 real block).  It checks the
// descriptor and layout encoding of tc_mma.cuh on the device.
#include <cuda_runtime.h>
#include <stdio.h>

#include "../../include/nqcd_gpu.h"
#include "tc_mma.cuh"

namespace nqcd {
namespace {

constexpr int kTM = 128, kTN = 80, kTK = 80;
constexpr uint32_t kABytes = kTM * kTK * 4, kBBytes = kTN * kTK * 4;
constexpr uint32_t kMaxPolls = 1u << 22;  // the product takes microseconds; a wait this long has failed

__global__ void __launch_bounds__(128) tc_selftest_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                          float* __restrict__ D, int passes, int* status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* a_hi = smem;
    unsigned char* a_lo = smem + kABytes;
    unsigned char* b_hi = smem + 2 * kABytes;
    unsigned char* b_lo = smem + 2 * kABytes + kBBytes;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // operands into the K-major core-matrix layout, split into tf32 high and low parts
    for (int q = tid; q < kTM * kTK; q += blockDim.x) {
        const int row = q / kTK, k = q - row * kTK;
        const float x = A[q];
        const float h = tc::to_tf32(x);
        const uint32_t off = tc::smem_kmajor_offset(row, k, kTK);
        *(float*)(a_hi + off) = h;
        *(float*)(a_lo + off) = tc::to_tf32(x - h);
    }
    for (int q = tid; q < kTN * kTK; q += blockDim.x) {
        const int k = q / kTN, n = q - k * kTN;  // B[k][n]: column n of the product is row n of the operand
        const float x = B[q];
        const float h = tc::to_tf32(x);
        const uint32_t off = tc::smem_kmajor_offset(n, k, kTK);
        *(float*)(b_hi + off) = h;
        *(float*)(b_lo + off) = tc::to_tf32(x - h);
    }
    tc::fence_proxy_async();
    if (tid == 0) {
        tc::mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::tmem_alloc(&tslot, 128);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;

    if (tid == 0) {
        constexpr uint32_t idesc = tc::idesc_f32acc(tc::kTypeTF32, kTM, kTN);
        const uint32_t sbo = kTK * 32, lbo = 128;
        const uint32_t ah = tc::smem_u32(a_hi), al = tc::smem_u32(a_lo), bh = tc::smem_u32(b_hi),
                       bl = tc::smem_u32(b_lo);
        const uint32_t as[3] = {ah, ah, al}, bs[3] = {bh, bl, bh};
        bool acc = false;
        for (int p = 0; p < (passes == 3 ? 3 : 1); ++p)
            for (int s = 0; s < kTK / 8; ++s) {
                tc::mma<tc::kTypeTF32>(tmem, tc::smem_desc(as[p] + 256u * s, lbo, sbo),
                                       tc::smem_desc(bs[p] + 256u * s, lbo, sbo), idesc, acc);
                acc = true;
            }
        tc::commit(&bar);
    }
    const bool ok = tc::mbar_wait(&bar, 0, kMaxPolls);
    tc::fence_after_sync();
    if (ok) {
        const int row = 32 * warp + lane;
        const uint32_t t = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll
        for (int c = 0; c < kTN / 16; ++c) {
            float v[16];
            tc::ld16(t + 16 * c, v);
            tc::wait_ld();
#pragma unroll
            for (int q = 0; q < 16; ++q) D[row * kTN + 16 * c + q] = v[q];
        }
    } else if (lane == 0) {
        atomicExch(status, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

}  // namespace
}  // namespace nqcd

extern "C" int nqcd_tensor_selftest(int32_t passes, const float* A, const float* B, float* D) {
    using namespace nqcd;
    if (!A || !B || !D || (passes != 1 && passes != 3)) return NQCD_ERR_ARG;
    float *dA = nullptr, *dB = nullptr, *dD = nullptr;
    int* dst = nullptr;
    int rc = NQCD_OK;
    const size_t smem = 2 * kABytes + 2 * kBBytes;
    cudaError_t e = cudaMalloc(&dA, sizeof(float) * kTM * kTK);
    if (e == cudaSuccess) e = cudaMalloc(&dB, sizeof(float) * kTK * kTN);
    if (e == cudaSuccess) e = cudaMalloc(&dD, sizeof(float) * kTM * kTN);
    if (e == cudaSuccess) e = cudaMalloc(&dst, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(dA, A, sizeof(float) * kTM * kTK, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dB, B, sizeof(float) * kTK * kTN, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dst, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) {
        tc_selftest_kernel<<<1, 128, smem>>>(dA, dB, dD, passes, dst);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int status = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&status, dst, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(D, dD, sizeof(float) * kTM * kTN, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        cudaGetLastError();
        rc = NQCD_ERR_CUDA;
    } else if (status) {
        rc = NQCD_ERR_TIMEOUT;
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dst);
    return rc;
}
