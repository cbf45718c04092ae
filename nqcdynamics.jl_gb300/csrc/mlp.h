// Friction surrogate network: host-side state and interface.
//
// 1-64-64-1 network, SiLU hidden activations, softplus output giving the
// Cholesky factor L of the (1 x 1) friction tensor, Lambda = L^2.  Parameters
// are packed W1[64] b1[64] W2[64][64] (row = output unit) b2[64] W3[64] b3[1].
// FP32 master weights and Adam moments; a BF16 copy serves the forward pass
// of training and inference.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mdef_kernels.cuh"

namespace nqcd {

constexpr int kMlpH = 64;
constexpr int kMlpOffW1 = 0, kMlpOffB1 = 64, kMlpOffW2 = 128, kMlpOffB2 = 128 + 4096, kMlpOffW3 = 4288,
              kMlpOffB3 = 4352, kMlpN = 4353;
constexpr int kMlpTile = 128;  // samples per block of the training kernel

struct MlpState {
    float* master = nullptr;  // [kMlpN]
    float* m1 = nullptr;      // Adam first moment
    float* m2 = nullptr;      // Adam second moment
    __nv_bfloat16* bf = nullptr;  // [kMlpN] BF16 copy
    float* grad = nullptr;    // [kMlpN + 1] (last entry: loss)
    float* partial = nullptr; // [max_blocks][kMlpN + 1]
    int max_blocks = 0;
    unsigned long long* step_counter = nullptr;  // device: Adam step (graph replays advance it)
    int* batch_index = nullptr;  // device scratch: minibatch sample indices
    double shift = 0.0, scale = 1.0, lo = 0.0, hi = 0.0;
    double friction_floor = 0.0;  // judge: 0.1 x the largest exact friction on a grid of the domain
    bool trained = false;
};

cudaError_t mlp_alloc(MlpState& s, int max_batch);
void mlp_free(MlpState& s);
cudaError_t mlp_init_weights(MlpState& s, uint64_t seed, float out_bias, cudaStream_t st);
// Loss (mean squared error of L) and gradient on n samples already on the device.
cudaError_t mlp_loss_grad_device(MlpState& s, const double* d_x, const double* d_t, int n, cudaStream_t st);
// Train on npts device samples: nsteps Adam steps with random minibatches of `batch`.
cudaError_t mlp_train_device(MlpState& s, const double* d_x, const double* d_t, int64_t npts, int64_t nsteps,
                             int batch, float lr, uint64_t seed, cudaStream_t st, double* final_loss);
// BF16 weights view for the MDEF kernel.
MlpWeights mlp_view(const MlpState& s);
cudaError_t mlp_sync_bf16(MlpState& s, cudaStream_t st);

}  // namespace nqcd
