// Friction surrogate network: BF16 tensor-core training kernels.
//
// One block trains on a tile of 128 samples (4 warps):
//   forward   h1 = silu(W1 u + b1)                         (CUDA cores, FP32)
//             z2 = h1 W2^T + b2                            (mma.sync m16n8k16 BF16 -> FP32)
//             o = W3 . silu(z2) + b3,  L = softplus(o)     (CUDA cores)
//   loss      mean over the batch of (L - L*)^2
//   backward  dz2 = (dL/do) W3 * silu'(z2)
//             dh1 = dz2 W2                                 (mma.sync BF16)
//             dW2 = dz2^T h1                               (mma.sync BF16, K = batch)
//             dz1 = dh1 * silu'(z1), dW1 = sum dz1 u, biases by warp-shuffle sums
// Each block writes its own gradient partial; a second kernel sums the
// partials in block order (deterministic), and an Adam kernel updates the
// FP32 master weights and refreshes the BF16 copy.  The GEMM operands that
// go through the tensor cores (h1, dz2, W2) are BF16; everything else FP32.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <random>
#include <vector>

#include "mlp.h"

namespace nqcd {

namespace {

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ float bfr(float x) { return __bfloat162float(__float2bfloat16(x)); }

// D = A (16x16, row) * B (16x8, col) + C, BF16 inputs, FP32 accumulate.
__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// One 16x8 output tile accumulated over K (multiple of 16) with element
// accessors A(m, k) and B(k, n) returning float (already BF16-representable).
// Fragment layout of m16n8k16 (g = lane / 4, t = lane % 4):
//   A regs: (g, 2t..2t+1), (g+8, 2t..2t+1), (g, 2t+8..), (g+8, 2t+8..)
//   B regs: (k = 2t..2t+1, n = g), (k = 2t+8..2t+9, n = g)
//   C:      (g, 2t), (g, 2t+1), (g+8, 2t), (g+8, 2t+1)
template <typename FA, typename FB>
__device__ __forceinline__ void tile_mma(float c[4], int m0, int n0, int K, FA A, FB B) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int k0 = 0; k0 < K; k0 += 16) {
        uint32_t a[4], b[2];
        a[0] = pack_bf16(A(m0 + g, k0 + 2 * t), A(m0 + g, k0 + 2 * t + 1));
        a[1] = pack_bf16(A(m0 + g + 8, k0 + 2 * t), A(m0 + g + 8, k0 + 2 * t + 1));
        a[2] = pack_bf16(A(m0 + g, k0 + 2 * t + 8), A(m0 + g, k0 + 2 * t + 9));
        a[3] = pack_bf16(A(m0 + g + 8, k0 + 2 * t + 8), A(m0 + g + 8, k0 + 2 * t + 9));
        b[0] = pack_bf16(B(k0 + 2 * t, n0 + g), B(k0 + 2 * t + 1, n0 + g));
        b[1] = pack_bf16(B(k0 + 2 * t + 8, n0 + g), B(k0 + 2 * t + 9, n0 + g));
        mma16816(c, a, b);
    }
}

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_f(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z) {
    float s = sigm(z);
    return s * (1.0f + z * (1.0f - s));
}

struct TrainSmem {
    __nv_bfloat16 W2[64][64];  // [out][in]
    float h1[kMlpTile][65];    // BF16-rounded values (rows padded against bank conflicts)
    float z2[kMlpTile][65];    // pre-activation of layer 2, later dh1
    float dz2[kMlpTile][65];   // BF16-rounded values
    float u[kMlpTile];
    float small[5][64];        // W1, b1, b2, W3 (BF16 values), b3 in small[4][0]
    float red[4][64 * 4 + 2];  // per-warp partial sums of dW1, db1, db2, dW3, db3, loss
};

// Gradient partial of one tile.  Samples idx[s] (or s when idx == null) of
// (x, t); n_total scales the mean.
__global__ void __launch_bounds__(128) mlp_fwd_bwd_kernel(const __nv_bfloat16* __restrict__ bfw,
                                                          const double* __restrict__ x,
                                                          const double* __restrict__ tgt, const int* idx,
                                                          int n, float n_total, float shift, float scale,
                                                          float* __restrict__ partial) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int q = tid; q < 64 * 64; q += 128) S.W2[q / 64][q % 64] = bfw[kMlpOffW2 + q];
    if (tid < 64) {
        S.small[0][tid] = __bfloat162float(bfw[kMlpOffW1 + tid]);
        S.small[1][tid] = __bfloat162float(bfw[kMlpOffB1 + tid]);
        S.small[2][tid] = __bfloat162float(bfw[kMlpOffB2 + tid]);
        S.small[3][tid] = __bfloat162float(bfw[kMlpOffW3 + tid]);
    }
    if (tid == 0) S.small[4][0] = __bfloat162float(bfw[kMlpOffB3]);
    const int s = tid;
    const int64_t gs = (int64_t)blockIdx.x * kMlpTile + s;
    const bool valid = gs < n;
    double xs = 0.0, ts = 0.0;
    if (valid) {
        int64_t j = idx ? idx[gs] : gs;
        xs = x[j];
        ts = tgt[j];
    }
    __syncthreads();
    const float u = valid ? ((float)xs - shift) * scale : 0.0f;
    S.u[s] = u;
    for (int j = 0; j < 64; ++j) S.h1[s][j] = valid ? bfr(silu_f(S.small[0][j] * u + S.small[1][j])) : 0.0f;
    __syncthreads();
    // z2 = h1 W2^T: warp w owns rows 32w..32w+31
    for (int mt = 0; mt < 2; ++mt)
        for (int nt = 0; nt < 8; ++nt) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            const int m0 = 32 * warp + 16 * mt, n0 = 8 * nt;
            tile_mma(c, m0, n0, 64, [&](int m, int k) { return S.h1[m][k]; },
                     [&](int k, int nn) { return __bfloat162float(S.W2[nn][k]); });
            const int g = lane >> 2, t = lane & 3;
            S.z2[m0 + g][n0 + 2 * t] = c[0] + S.small[2][n0 + 2 * t];
            S.z2[m0 + g][n0 + 2 * t + 1] = c[1] + S.small[2][n0 + 2 * t + 1];
            S.z2[m0 + g + 8][n0 + 2 * t] = c[2] + S.small[2][n0 + 2 * t];
            S.z2[m0 + g + 8][n0 + 2 * t + 1] = c[3] + S.small[2][n0 + 2 * t + 1];
        }
    __syncthreads();
    // output, loss, dz2
    float o = S.small[4][0];
    for (int j = 0; j < 64; ++j) o += S.small[3][j] * silu_f(S.z2[s][j]);
    const float L = o > 20.f ? o : log1pf(__expf(o));
    const float err = valid ? L - (float)ts : 0.0f;
    const float dL = 2.0f * err / n_total;
    const float dO = dL * sigm(o);
    float* myred = S.red[warp];
    for (int j = 0; j < 64; ++j) {
        float z = S.z2[s][j];
        float dz = dO * S.small[3][j] * dsilu(z);
        S.dz2[s][j] = bfr(dz);
        float a = dz, b = dO * silu_f(z);  // db2, dW3 contributions
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, off);
            b += __shfl_xor_sync(0xffffffffu, b, off);
        }
        if (lane == 0) {
            myred[128 + j] = a;
            myred[192 + j] = b;
        }
    }
    {
        float a = dO, b = err * err / n_total;
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, off);
            b += __shfl_xor_sync(0xffffffffu, b, off);
        }
        if (lane == 0) {
            myred[256] = a;
            myred[257] = b;
        }
    }
    __syncthreads();
    float* P = partial + (int64_t)blockIdx.x * (kMlpN + 1);
    // dW2 = dz2^T h1 (64 x 64, K = 128): warp w owns output rows 16w..16w+15
    for (int nt = 0; nt < 8; ++nt) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        const int m0 = 16 * warp, n0 = 8 * nt;
        tile_mma(c, m0, n0, kMlpTile, [&](int m, int k) { return S.dz2[k][m]; },
                 [&](int k, int nn) { return S.h1[k][nn]; });
        const int g = lane >> 2, t = lane & 3;
        P[kMlpOffW2 + (m0 + g) * 64 + n0 + 2 * t] = c[0];
        P[kMlpOffW2 + (m0 + g) * 64 + n0 + 2 * t + 1] = c[1];
        P[kMlpOffW2 + (m0 + g + 8) * 64 + n0 + 2 * t] = c[2];
        P[kMlpOffW2 + (m0 + g + 8) * 64 + n0 + 2 * t + 1] = c[3];
    }
    // dh1 = dz2 W2 (rows 32w..), stored over z2 (no longer needed)
    __syncthreads();
    for (int mt = 0; mt < 2; ++mt)
        for (int nt = 0; nt < 8; ++nt) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            const int m0 = 32 * warp + 16 * mt, n0 = 8 * nt;
            tile_mma(c, m0, n0, 64, [&](int m, int k) { return S.dz2[m][k]; },
                     [&](int k, int nn) { return __bfloat162float(S.W2[k][nn]); });
            const int g = lane >> 2, t = lane & 3;
            S.z2[m0 + g][n0 + 2 * t] = c[0];
            S.z2[m0 + g][n0 + 2 * t + 1] = c[1];
            S.z2[m0 + g + 8][n0 + 2 * t] = c[2];
            S.z2[m0 + g + 8][n0 + 2 * t + 1] = c[3];
        }
    __syncthreads();
    // layer 1
    for (int j = 0; j < 64; ++j) {
        float z1 = S.small[0][j] * u + S.small[1][j];
        float dz1 = valid ? S.z2[s][j] * dsilu(z1) : 0.0f;
        float a = dz1 * u, b = dz1;
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, off);
            b += __shfl_xor_sync(0xffffffffu, b, off);
        }
        if (lane == 0) {
            myred[j] = a;
            myred[64 + j] = b;
        }
    }
    __syncthreads();
    // per-block partial of the small parameters: sum of the 4 warps in order
    for (int q = tid; q < 258; q += 128) {
        float v = S.red[0][q] + S.red[1][q] + S.red[2][q] + S.red[3][q];
        int dst;
        if (q < 64)
            dst = kMlpOffW1 + q;
        else if (q < 128)
            dst = kMlpOffB1 + q - 64;
        else if (q < 192)
            dst = kMlpOffB2 + q - 128;
        else if (q < 256)
            dst = kMlpOffW3 + q - 192;
        else if (q == 256)
            dst = kMlpOffB3;
        else
            dst = kMlpN;  // loss
        P[dst] = v;
    }
}

__global__ void mlp_reduce_kernel(const float* __restrict__ partial, int nblocks, float* __restrict__ grad) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > kMlpN) return;
    float acc = 0.f;
    for (int b = 0; b < nblocks; ++b) acc += partial[(int64_t)b * (kMlpN + 1) + i];
    grad[i] = acc;
}

__global__ void mlp_tick_kernel(unsigned long long* counter) { *counter += 1ull; }

__global__ void mlp_adam_kernel(float* __restrict__ w, float* __restrict__ m1, float* __restrict__ m2,
                                const float* __restrict__ g, __nv_bfloat16* __restrict__ bf,
                                const unsigned long long* counter, float lr0, float total_steps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpN) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float t = (float)*counter;
    // cosine decay from lr0 to lr0 / 100 over the run
    float frac = total_steps > 1.f ? fminf((t - 1.f) / total_steps, 1.f) : 0.f;
    float lr = lr0 * (0.01f + 0.495f * (1.f + cospif(frac)));
    float gi = g[i];
    float a = b1 * m1[i] + (1.f - b1) * gi;
    float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    float ah = a / (1.f - powf(b1, t)), bh = b / (1.f - powf(b2, t));
    float wi = w[i] - lr * ah / (sqrtf(bh) + eps);
    w[i] = wi;
    bf[i] = __float2bfloat16(wi);
}

__global__ void mlp_to_bf16_kernel(const float* __restrict__ w, __nv_bfloat16* __restrict__ bf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kMlpN) bf[i] = __float2bfloat16(w[i]);
}

// Minibatch indices of the current step (Philox keyed by seed, counter step).
__global__ void mlp_sample_kernel(int* idx, int batch, int64_t npts, uint64_t seed,
                                  const unsigned long long* counter) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= batch) return;
    u32x4 b = rng_block(seed, (uint64_t)i, (uint32_t)*counter, 7u);
    uint64_t r = ((uint64_t)b.x << 32) | b.y;
    idx[i] = (int)(r % (uint64_t)npts);
}

size_t train_smem() { return sizeof(TrainSmem); }

}  // namespace

cudaError_t mlp_alloc(MlpState& s, int max_batch) {
    if (s.master) return cudaSuccess;
    s.max_blocks = (max_batch + kMlpTile - 1) / kMlpTile;
    cudaError_t e;
    if ((e = cudaMalloc(&s.master, kMlpN * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.m1, kMlpN * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.m2, kMlpN * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.bf, kMlpN * sizeof(__nv_bfloat16))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.grad, (kMlpN + 1) * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.partial, (size_t)s.max_blocks * (kMlpN + 1) * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.step_counter, sizeof(unsigned long long))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.batch_index, (size_t)max_batch * sizeof(int))) != cudaSuccess) return e;
    return cudaFuncSetAttribute(mlp_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem());
}

void mlp_free(MlpState& s) {
    void* p[] = {s.master, s.m1, s.m2, s.bf, s.grad, s.partial, s.step_counter, s.batch_index};
    for (void* q : p)
        if (q) cudaFree(q);
    s = MlpState();
}

cudaError_t mlp_sync_bf16(MlpState& s, cudaStream_t st) {
    mlp_to_bf16_kernel<<<(kMlpN + 255) / 256, 256, 0, st>>>(s.master, s.bf);
    return cudaGetLastError();
}

cudaError_t mlp_init_weights(MlpState& s, uint64_t seed, float out_bias, cudaStream_t st) {
    std::vector<float> w(kMlpN, 0.0f);
    std::mt19937_64 gen(seed);
    std::uniform_real_distribution<float> U(-1.0f, 1.0f);
    for (int j = 0; j < 64; ++j) {
        w[kMlpOffW1 + j] = 3.0f * U(gen);
        w[kMlpOffB1 + j] = 3.0f * U(gen);
        w[kMlpOffB2 + j] = 0.0f;
        w[kMlpOffW3 + j] = 0.125f * U(gen);
    }
    for (int q = 0; q < 64 * 64; ++q) w[kMlpOffW2 + q] = 0.2165f * U(gen);  // uniform with variance 1/64
    w[kMlpOffB3] = out_bias;
    cudaError_t e = cudaMemcpyAsync(s.master, w.data(), kMlpN * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(s.m1, 0, kMlpN * sizeof(float), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(s.m2, 0, kMlpN * sizeof(float), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(s.step_counter, 0, sizeof(unsigned long long), st)) != cudaSuccess) return e;
    return mlp_sync_bf16(s, st);
}

cudaError_t mlp_loss_grad_device(MlpState& s, const double* d_x, const double* d_t, int n, cudaStream_t st) {
    int nb = (n + kMlpTile - 1) / kMlpTile;
    if (nb > s.max_blocks) return cudaErrorInvalidValue;
    mlp_fwd_bwd_kernel<<<nb, 128, train_smem(), st>>>(s.bf, d_x, d_t, nullptr, n, (float)n, (float)s.shift,
                                                      (float)s.scale, s.partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    mlp_reduce_kernel<<<(kMlpN + 1 + 255) / 256, 256, 0, st>>>(s.partial, nb, s.grad);
    return cudaGetLastError();
}

cudaError_t mlp_train_device(MlpState& s, const double* d_x, const double* d_t, int64_t npts, int64_t nsteps,
                             int batch, float lr, uint64_t seed, cudaStream_t st, double* final_loss) {
    const int nb = (batch + kMlpTile - 1) / kMlpTile;
    if (nb > s.max_blocks || batch <= 0) return cudaErrorInvalidValue;
    // one training step = tick, sample, forward/backward, reduce, Adam; captured once, replayed nsteps times
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    mlp_tick_kernel<<<1, 1, 0, st>>>(s.step_counter);
    mlp_sample_kernel<<<(batch + 255) / 256, 256, 0, st>>>(s.batch_index, batch, npts, seed, s.step_counter);
    mlp_fwd_bwd_kernel<<<nb, 128, train_smem(), st>>>(s.bf, d_x, d_t, s.batch_index, batch, (float)batch,
                                                      (float)s.shift, (float)s.scale, s.partial);
    mlp_reduce_kernel<<<(kMlpN + 1 + 255) / 256, 256, 0, st>>>(s.partial, nb, s.grad);
    mlp_adam_kernel<<<(kMlpN + 255) / 256, 256, 0, st>>>(s.master, s.m1, s.m2, s.grad, s.bf, s.step_counter, lr,
                                                         (float)nsteps);
    e = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return e;
    }
    for (int64_t k = 0; k < nsteps && e == cudaSuccess; ++k) e = cudaGraphLaunch(exec, st);
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return e;
    // final loss over all samples (mean squared error of L)
    if (final_loss) {
        double total = 0.0;
        int64_t done = 0;
        const int64_t chunk = (int64_t)s.max_blocks * kMlpTile;
        while (done < npts) {
            int n = (int)((npts - done) < chunk ? (npts - done) : chunk);
            if ((e = mlp_loss_grad_device(s, d_x + done, d_t + done, n, st)) != cudaSuccess) return e;
            float l = 0.f;
            if ((e = cudaMemcpyAsync(&l, s.grad + kMlpN, sizeof(float), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
                return e;
            if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
            total += (double)l * n;
            done += n;
        }
        *final_loss = total / (double)npts;
    }
    return cudaSuccess;
}

MlpWeights mlp_view(const MlpState& s) {
    MlpWeights w;
    w.W1 = s.bf + kMlpOffW1;
    w.b1 = s.bf + kMlpOffB1;
    w.W2 = s.bf + kMlpOffW2;
    w.b2 = s.bf + kMlpOffB2;
    w.W3 = s.bf + kMlpOffW3;
    w.b3 = s.bf + kMlpOffB3;
    w.x_shift = (float)s.shift;
    w.x_scale = (float)s.scale;
    w.lo = (float)s.lo;
    w.hi = (float)s.hi;
    w.floor = (float)s.friction_floor;
    return w;
}

}  // namespace nqcd
