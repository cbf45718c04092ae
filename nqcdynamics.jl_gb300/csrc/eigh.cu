// Batched eigendecomposition of dense real symmetric matrices: cyclic Jacobi
// in shared memory, one CTA per matrix.
//
// The trajectory kernels of this engine do not call it: the metal models of
// the benchmark (AndersonHolstein, an impurity level coupled to a bath) have
// arrowhead Hamiltonians whose eigenvalues are the roots of a secular
// equation (secular.h), O(N) per root instead of O(N^3) per matrix.  This is
// the general path the reference takes through LAPACK for any Hamiltonian
// (NQCCalculators' update_cache!/get_eigen, called from
// src/DynamicsMethods/SurfaceHoppingMethods/SurfaceHoppingMethods.jl:58 and
// src/DynamicsMethods/ClassicalMethods/mdef.jl:103-115), for models without
// that structure (bath-bath couplings, several impurities) and as an
// independent check of the secular solver.
//
// Algorithm: parallel cyclic Jacobi with the round-robin (tournament)
// ordering.  A sweep has n - 1 rounds (n even; an odd matrix is bordered by
// one decoupled row and column); a round rotates n/2 disjoint index pairs at
// once: each pair's rotation (c, s) zeroes A_pq (the classical formula
// t = sign(tau) / (|tau| + sqrt(1 + tau^2)), tau = (A_qq - A_pp) / (2 A_pq)),
// then all rows p, q, all columns p, q and the eigenvector columns p, q are
// rotated in parallel.  Sweeps stop when the off-diagonal Frobenius norm is
// below n units in the last place (2^-52 in FP64, 2^-23 in FP32) times the
// matrix's, or after 30 sweeps.
// Eigenvalues are returned ascending with their eigenvectors; each
// eigenvector's largest component (the first on ties) is made positive.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "../../include/nqcd_gpu.h"

namespace nqcd {

constexpr int kEighBlock = 256;
constexpr int kEighMaxSweeps = 30;

template <typename R>
__device__ inline R eigh_block_sum(R x, R* red) {
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) red[w] = x;
    __syncthreads();
    R s = R(0);
    for (int q = 0; q < nw; ++q) s += red[q];
    __syncthreads();
    return s;
}

// Pair k (0 <= k < n/2) of round r: (p, q) with p < q.  Positions 0..n-2 sit
// on a circle rotated by r; position n - 1 is fixed.  Pair 0 joins the fixed
// index with the circle's position r; pair k > 0 joins circle positions
// r + k and r - k.
__device__ inline void eigh_pair(int k, int r, int n, int& p, int& q) {
    const int m = n - 1;
    int a, b;
    if (k == 0) {
        a = m;
        b = r % m;
    } else {
        a = (r + k) % m;
        b = (r - k + m) % m;
    }
    p = a < b ? a : b;
    q = a < b ? b : a;
}

template <typename R>
__global__ void __launch_bounds__(kEighBlock) eigh_jacobi_kernel(const double* __restrict__ Ain, int n, int64_t batch,
                                                                 double* __restrict__ wout, double* __restrict__ Zout,
                                                                 int* __restrict__ sweeps_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int64_t b = blockIdx.x;
    if (b >= batch) return;
    const int ne = n + (n & 1);  // bordered to an even order
    R* A = (R*)smem;             // [ne][ne], A[i * ne + j]
    R* V = A + ne * ne;          // [ne][ne], V[i * ne + j]: component i of vector j
    R* cs = V + ne * ne;         // [ne/2][2] rotation of each pair
    R* red = cs + ne;            // [32] block sums
    int* perm = (int*)(red + 32);
    const int tid = threadIdx.x, nthr = blockDim.x;
    const double* src = Ain + b * (int64_t)n * n;
    R fro = R(0);
    for (int q = tid; q < ne * ne; q += nthr) {
        const int i = q / ne, j = q - i * ne;
        const R a = (i < n && j < n) ? (R)(0.5 * (src[(int64_t)i * n + j] + src[(int64_t)j * n + i])) : R(0);
        A[q] = a;
        V[q] = i == j ? R(1) : R(0);
        fro += a * a;
    }
    fro = eigh_block_sum<R>(fro, red);
    // stop at an off-diagonal norm of n units in the last place of the matrix norm (squared here)
    const R ulp = std::is_same<R, double>::value ? R(0x1p-52) : R(0x1p-23);
    const R tol = (R)n * (R)n * ulp * ulp * fro;
    int sweep = 0;
    for (; sweep < kEighMaxSweeps; ++sweep) {
        R off = R(0);
        for (int q = tid; q < ne * ne; q += nthr) {
            const int i = q / ne, j = q - i * ne;
            if (i != j) off += A[q] * A[q];
        }
        off = eigh_block_sum<R>(off, red);
        if (!(off > tol)) break;
        for (int r = 0; r < ne - 1; ++r) {
            // rotations of this round's pairs
            for (int k = tid; k < ne / 2; k += nthr) {
                int p, q;
                eigh_pair(k, r, ne, p, q);
                const R apq = A[p * ne + q];
                R c = R(1), s = R(0);
                if (apq != R(0)) {
                    const R tau = (A[q * ne + q] - A[p * ne + p]) / (R(2) * apq);
                    const R t = (tau >= R(0) ? R(1) : R(-1)) / (fabs(tau) + sqrt(R(1) + tau * tau));
                    c = R(1) / sqrt(R(1) + t * t);
                    s = t * c;
                }
                cs[2 * k] = c;
                cs[2 * k + 1] = s;
            }
            __syncthreads();
            // rows p, q of every pair
            for (int w = tid; w < (ne / 2) * ne; w += nthr) {
                const int k = w / ne, j = w - k * ne;
                int p, q;
                eigh_pair(k, r, ne, p, q);
                const R c = cs[2 * k], s = cs[2 * k + 1];
                const R ap = A[p * ne + j], aq = A[q * ne + j];
                A[p * ne + j] = c * ap - s * aq;
                A[q * ne + j] = s * ap + c * aq;
            }
            __syncthreads();
            // columns p, q of every pair, and the eigenvector columns
            for (int w = tid; w < (ne / 2) * ne; w += nthr) {
                const int k = w / ne, i = w - k * ne;
                int p, q;
                eigh_pair(k, r, ne, p, q);
                const R c = cs[2 * k], s = cs[2 * k + 1];
                const R ap = A[i * ne + p], aq = A[i * ne + q];
                A[i * ne + p] = c * ap - s * aq;
                A[i * ne + q] = s * ap + c * aq;
                const R vp = V[i * ne + p], vq = V[i * ne + q];
                V[i * ne + p] = c * vp - s * vq;
                V[i * ne + q] = s * vp + c * vq;
            }
            __syncthreads();
        }
    }
    // ascending order of the first n eigenvalues (the border's 0 eigenvalue, of the unit vector
    // e_n, is left out): rank by count, ties by index
    for (int j = tid; j < ne; j += nthr) {
        int rank = 0;
        const bool real_j = n == ne || V[n * ne + j] == R(0);  // not the border's eigenvector
        if (real_j) {
            const R lj = A[j * ne + j];
            for (int k = 0; k < ne; ++k) {
                if (k == j) continue;
                const bool real_k = n == ne || V[n * ne + k] == R(0);
                if (!real_k) continue;
                const R lk = A[k * ne + k];
                if (lk < lj || (lk == lj && k < j)) ++rank;
            }
            perm[rank] = j;
        }
    }
    __syncthreads();
    for (int o = tid; o < n; o += nthr) {
        const int j = perm[o];
        wout[b * n + o] = (double)A[j * ne + j];
        // sign: the largest component positive (the first on ties)
        int im = 0;
        R am = R(-1);
        for (int i = 0; i < n; ++i) {
            const R a = fabs(V[i * ne + j]);
            if (a > am) {
                am = a;
                im = i;
            }
        }
        const R sg = V[im * ne + j] < R(0) ? R(-1) : R(1);
        for (int i = 0; i < n; ++i) Zout[(b * n + o) * (int64_t)n + i] = (double)(sg * V[i * ne + j]);
    }
    if (tid == 0 && sweeps_out) sweeps_out[b] = sweep;
}

static size_t eigh_smem(int n, int prec) {
    const int ne = n + (n & 1);
    const size_t el = prec == NQCD_PREC_FP64 ? sizeof(double) : sizeof(float);
    return el * (2 * (size_t)ne * ne + ne + 32) + sizeof(int) * (size_t)ne;
}

}  // namespace nqcd

using namespace nqcd;

extern "C" int nqcd_eigh_batched(int32_t precision, int32_t n, int64_t batch, const double* A, double* w, double* Z,
                                 int32_t* sweeps) {
    if (!A || !w || !Z || n < 1 || batch < 1) return NQCD_ERR_ARG;
    if (precision != NQCD_PREC_FP64 && precision != NQCD_PREC_FP32) return NQCD_ERR_ARG;
    const size_t sm = eigh_smem(n, precision);
    if (sm > 227 * 1024) return NQCD_ERR_UNSUPPORTED;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
        cudaGetLastError();
        return NQCD_ERR_CUDA;
    }
    const size_t nA = (size_t)batch * n * n, nw = (size_t)batch * n;
    double *dA = nullptr, *dw = nullptr, *dZ = nullptr;
    int* ds = nullptr;
    cudaError_t e = cudaMalloc(&dA, nA * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dw, nw * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dZ, nA * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&ds, (size_t)batch * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(dA, A, nA * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        if (precision == NQCD_PREC_FP64) {
            e = cudaFuncSetAttribute(eigh_jacobi_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (e == cudaSuccess) eigh_jacobi_kernel<double><<<(unsigned)batch, kEighBlock, sm>>>(dA, n, batch, dw, dZ, ds);
        } else {
            e = cudaFuncSetAttribute(eigh_jacobi_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (e == cudaSuccess) eigh_jacobi_kernel<float><<<(unsigned)batch, kEighBlock, sm>>>(dA, n, batch, dw, dZ, ds);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(w, dw, nw * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(Z, dZ, nA * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && sweeps) {
        std::vector<int> hs(batch);
        e = cudaMemcpy(hs.data(), ds, (size_t)batch * sizeof(int), cudaMemcpyDeviceToHost);
        for (int64_t b = 0; b < batch; ++b) sweeps[b] = hs[b];
    }
    cudaFree(dA);
    cudaFree(dw);
    cudaFree(dZ);
    cudaFree(ds);
    return e == cudaSuccess ? NQCD_OK : NQCD_ERR_CUDA;
}
