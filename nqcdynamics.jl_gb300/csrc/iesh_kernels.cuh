// IESH (independent-electron surface hopping) ensemble kernel on a
// three-dimensional Newns-Anderson adsorbate; one CTA per trajectory.
//
// Reference algorithm (NQCDynamics.jl):
//   VerletwithElectronics.perform_step!  src/DynamicsMethods/IntegrationAlgorithms/verlet_with_electronics.jl:42-69
//   IESH acceleration!                   src/DynamicsMethods/SurfaceHoppingMethods/iesh.jl:190-207
//   get_quantum_propagator,
//   propagate_wavefunction!              src/DynamicsUtils/wavefunction_dynamics.jl:15-58
//   evaluate_hopping_probability!        iesh.jl:231-283 (estimate screen :251-254)
//   evaluate_v_dot_d!, calculate_Akj,
//   compute_overlap!                     iesh.jl:285-316
//   select_new_state                     iesh.jl:318-335
//   iesh_check_hop!, iesh_execute_hop!   iesh.jl:390-411
//   rescale_velocity!                    src/DynamicsMethods/SurfaceHoppingMethods/surface_hopping.jl:64-168
//   FermiDiracState{Adiabatic} start     iesh.jl:99-128 with sample_fermi_dirac_distribution
//                                        src/DynamicsUtils/DynamicsUtils.jl:194-208
//   iesh_diabatic_population             iesh.jl:351-369
//   classical_potential_energy           iesh.jl:380-388
//
// Model: one atom (x, y, z) above a metal band, AndersonHolstein form
//     U0 = kxy (x^2 + y^2) / 2 + A exp(-a z),   h = U1 - U0 = delta - B exp(-b z),
//     H  = [[h, V_k], [V_k, diag(e_k)]]          (N = M + 1 one-electron states).
// The reference diagonalises H (LAPACK) every step.  H is an arrowhead matrix
// whose derivative is dh e0 e0^T, so the eigenvalues l_i are the roots of the
// secular equation (secular.h), the adiabatic derivative is
// (Z^T dH Z)_ij = dh z0_i z0_j and the couplings are d_ij = dh A_ij with
// A_ij = z0_i z0_j / (l_j - l_i): O(N^2) per step instead of O(N^3).
//
// Propagator: the reference forms H_eff = diag(l) - i (v . grad h) A, takes its
// full Hermitian eigendecomposition and applies U exp(-i mu dt) U^H to the
// N x Ne orbital matrix psi.  Here exp(-i H_eff dt) psi is applied directly as
// a Chebyshev series (Tal-Ezer and Kosloff, J. Chem. Phys. 81, 3967 (1984)):
//     exp(-i H dt) = exp(-i c dt) sum_k (2 - delta_k0) (-i)^k J_k(alpha) T_k(Ht),
//     Ht = (H - c) / w,  alpha = w dt,
// with [c - w, c + w] a Gershgorin enclosure of the spectrum and the series cut
// where |J_k(alpha)| falls below the tolerance (1e-17 on the plain path, so
// the result equals the eigendecomposition to rounding).  Each term is one
// product of the real N x N matrix A with the complex N x Ne block, done with
// 4 x 4 register tiles per thread.
//
// Hop probabilities: S = psi[state, :] (Ne x Ne) is LU-factorised once per
// step for det S and the estimate screen.  Where the screen does not reject,
// the reference evaluates the determinant of every row-replaced S' (1600 LU
// factorisations for 40 electrons in 80 states); by the matrix determinant
// lemma det S' = det S (psi[m, :] S^-1)_n, so all of them follow from one
// solve S^T Y = psi[unocc, :]^T, and
//     p_mn = 2 dt Re(Y_nm) (v.d)_mn = prefactor Re(det S conj(det S')) (v.d)_mn.
//
// R = double: plain path.  R = float: fast path (FP32 electronic structure,
// propagation and hop linear algebra; positions, velocities and the hop
// decision's scalar logic in FP64; initial occupations from FP64 roots).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "fssh2_traj.h"
#include "nqcd_math.h"
#include "secular.h"
#include "tc_mma.cuh"

namespace nqcd {

constexpr int kIeshBlock = 256;
constexpr int kIeshMaxStates = 128;
constexpr int kRpIeshMaxBeads = 32;      // ring polymer: beads (one per lane of warp 0)
constexpr int kRpIeshMaxElectrons = 64;  // ring polymer: electrons (two per lane in the bead roots)
constexpr int kIeshMaxTerms = 128;  // Chebyshev terms
constexpr int kIeshInv = 192;       // table of 1/n for the Bessel power series
constexpr int kIeshFdChunk = 256;   // Metropolis iterations whose random numbers are drawn together

enum IeshInit : int32_t { IESH_INIT_GIVEN = 0, IESH_INIT_FERMI_DIRAC = 3 };

struct IeshParams {
    int32_t nbath, nstates, nelec;  // nstates = nbath + 1
    const double* eps;              // [nbath] ascending bath levels
    const double* V2;               // [nbath] V_k^2
    double sumV2;
    double kxy, A, a, delta, B, b;  // model, see above
    double beta;                    // electronic inverse temperature (Fermi-Dirac start)
    double mass;
    int32_t rescaling;
    int32_t init_kind;
    int32_t exact_probability;      // 1: every step evaluates all probabilities (estimate_probability = false)
    int32_t ehrenfest_na;           // 1: Simulation{EhrenfestNA} (mean-field force of the orbitals, no hops)
    double edc_C;                   // > 0: energy-based decoherence correction after every step
    int32_t nbeads;                 // > 1: RingPolymerSimulation{AdiabaticIESH} (rpiesh_kernel)
    const double* rp_U;             // [nbeads * nbeads] normal-mode matrix, column-major U[j + n k]
    const double* rp_cay;           // [nbeads][4] full-step Cayley matrices (c11, c12, c21, c22)
    double omega_n;                 // ring-polymer frequency nbeads / beta (spring energy)
    int32_t save_stride, nsave, max_hops;
    int64_t ntraj, traj_offset;
    double dt;
    double h_last;                  // length of the last step (dt unless the span is not a whole number of steps)
    int32_t nsteps;
    uint64_t seed;
    double cheb_tol;                // truncation of the Chebyshev series
    double* r;                      // [3 * nbeads][ntraj] in/out (dof d of bead j at row d + 3 j)
    double* v;                      // [3 * nbeads][ntraj] in/out
    const int32_t* occ0;            // [nelec][ntraj] given initial occupations (IESH_INIT_GIVEN)
    int32_t* occ;                   // [nelec][ntraj] final occupations (electron order)
    double* psi_re;                 // [ntraj][nelec][nstates] final orbitals, or null
    double* psi_im;
    int32_t* nhops;
    int32_t* nfrustrated;
    int32_t* nsteps_out;
    int32_t* hop_log;               // [max_hops][3][ntraj]: step, from, to
    double* energy;                 // [2][ntraj] total energy at start and end, or null
    double* obs_partial;            // [ntraj][nsave][4]: z, kinetic, impurity population, potential
    unsigned long long* counters;   // [0] full hop evaluations, [1] Chebyshev terms, [2] unconverged roots,
                                    // [3] tensor-core waits that gave up, [5] overlap LUs
    // FP32 path: adjacent roots closer than gap_fp64 are solved again in FP64 and the couplings
    // between them, z0_i z0_j / (l_j - l_i), formed from the FP64 roots; fp64_steps[ti] counts the
    // steps that needed it (null: not counted)
    double gap_fp64;
    int32_t* fp64_steps;
    // FP32 path: the propagator's products on the tensor cores (tcgen05, iesh_tc_shape); counters[3]
    // counts waits for them that gave up
    int32_t tensor;
    // FP32 path: 1 runs the LU of the overlap matrix every step; 0 skips it where the bound of the
    // estimate from the occupied Gram matrix is already below the random number
    int32_t lu_always;
};

template <typename R>
struct alignas(2 * sizeof(R)) Cx {
    R re, im;
};

// Dynamic shared memory layout of one CTA (identical on host and device).
struct IeshLayout {
    int N, Ne, Nu, Np, Nep, B;
    bool tc;  // tensor-core propagator: o_tc replaces At, phiB and out
    size_t o_eps, o_V2, o_lam, o_z2, o_z0, o_w64, o_At, o_phiA, o_phiB, o_out, o_J, o_Jr, o_inv, o_fdu, o_fdi, o_occ,
        o_unocc, o_piv, o_red, o_misc, o_rph, o_rpq, o_tc, tc_sa, o_dl, bytes;
};

// The tensor-core propagator handles N states and Ne electrons when N is a
// multiple of 16 (the MMA's N), at most 80 (three N-column TMEM regions fit
// the 256 columns of a CTA that shares its SM), and 2 Ne <= 128 (the MMA's M).
NQCD_HD bool iesh_tc_shape(int N, int Ne) { return N % 16 == 0 && N >= 16 && N <= 80 && Ne >= 1 && 2 * Ne <= 128; }

NQCD_HD size_t iesh_take(size_t& o, size_t bytes) {
    size_t at = o;
    o += (bytes + 15) & ~(size_t)15;
    return at;
}

// B > 1: ring polymer of B beads (per-bead levels and sums, normal-mode scratch).
template <typename R>
NQCD_HD IeshLayout iesh_layout(int N, int Ne, int B = 1, bool tc = false) {
    IeshLayout L;
    L.B = B;
    L.tc = tc;
    L.o_tc = 0;
    L.tc_sa = 0;
    L.o_dl = 0;
    L.N = N;
    L.Ne = Ne;
    L.Nu = N - Ne;
    L.Np = (N + 3) & ~3;
    L.Nep = (Ne + 3) & ~3;
    size_t o = 0;
    L.o_eps = iesh_take(o, sizeof(R) * L.Np);
    L.o_V2 = iesh_take(o, sizeof(R) * L.Np);
    L.o_lam = iesh_take(o, sizeof(R) * L.Np);
    L.o_z2 = iesh_take(o, sizeof(R) * L.Np);
    L.o_z0 = iesh_take(o, sizeof(R) * L.Np);
    L.o_w64 = iesh_take(o, sizeof(double) * L.Np);
    const size_t pb = 2 * sizeof(R) * (size_t)L.Np * L.Nep;
    const size_t lu = 2 * sizeof(R) * (size_t)L.Nep * (L.Nep + L.Nu);  // S^T and the right-hand sides
    if (tc) {
        // [A operand high | A operand low | B operand], tf32 in 4-byte words, K-major core
        // matrices: the orbital block transposed (2 Ne rows: re, im of each electron) and the
        // coupling matrix (N rows).  The MMA reads 128 A rows; rows past 2 Ne fall in the next
        // buffer (their products land in accumulator rows that are never read), so the region
        // reaches 128 rows past the low buffer's start.  The hop test's LU workspace shares it.
        L.o_At = 0;
        L.o_phiA = iesh_take(o, pb);
        const size_t sa = (size_t)((2 * Ne + 7) / 8 * 8) * N * 4, sb = (size_t)N * N * 4;
        size_t tr = sa + (sa + sb > (size_t)128 * N * 4 ? sa + sb : (size_t)128 * N * 4);
        if (lu > tr) tr = lu;
        L.tc_sa = sa;
        L.o_tc = iesh_take(o, tr);
        L.o_dl = iesh_take(o, sizeof(float) * L.Np);
        L.o_phiB = L.o_tc;
        L.o_out = L.o_tc;
    } else {
        L.o_At = iesh_take(o, sizeof(R) * L.Np * L.Np);
        L.o_phiA = iesh_take(o, pb);
        L.o_phiB = iesh_take(o, lu > pb ? lu : pb);
        L.o_out = iesh_take(o, pb);
    }
    L.o_J = iesh_take(o, sizeof(double) * kIeshMaxTerms);
    L.o_Jr = iesh_take(o, sizeof(R) * kIeshMaxTerms);
    L.o_inv = iesh_take(o, sizeof(double) * kIeshInv);
    L.o_fdu = iesh_take(o, sizeof(double) * kIeshFdChunk);
    L.o_fdi = iesh_take(o, 2 * kIeshFdChunk);
    L.o_occ = iesh_take(o, sizeof(int) * L.Nep);
    L.o_unocc = iesh_take(o, sizeof(int) * L.Np);
    L.o_piv = iesh_take(o, sizeof(int) * L.Nep);
    L.o_red = iesh_take(o, sizeof(double) * 72);
    L.o_misc = iesh_take(o, sizeof(double) * 32);
    // ring polymer: [4][B] bead h, dh/dz, occupied z0^2 sum, occupied eigenvalue sum; [6][B] normal modes
    L.o_rph = B > 1 ? iesh_take(o, sizeof(double) * 4 * B) : 0;
    L.o_rpq = B > 1 ? iesh_take(o, sizeof(double) * 6 * B) : 0;
    L.bytes = o;
    return L;
}

// Register tiles of the A * phi products: 4 rows x 4 orbitals per thread,
// interleaved (rows rt + RG rr, orbitals ct + CG cc with RG = Np/4, CG = Nep/4)
// so that the lanes of a warp address consecutive shared-memory banks.
NQCD_HD int iesh_tiles(int N, int Ne) { return (((N + 3) & ~3) / 4) * (((Ne + 3) & ~3) / 4); }

// Chebyshev coefficients J_k(alpha), k = 0 .. kIeshMaxTerms-1, computed by one
// warp.  For alpha <= 4 each lane sums the power series
//     J_k(x) = sum_m (-1)^m (x/2)^(2m+k) / (m! (m+k)!)
// for its orders (terms at most e^4 / 2 in size, so the sum keeps 1e-14
// relative accuracy); larger alpha use Miller's backward recurrence
// J_{k-1} = (2k/alpha) J_k - J_{k+1} on lane 0, normalised with
// J_0 + 2 sum J_2k = 1.  Returns the last order K with |J_K| >= tol (the
// series uses terms 0..K), or -1 if the tail does not fall below tol.
__device__ inline int iesh_bessel_warp(double alpha, double tol, double* J, const double* inv) {
    const int lane = threadIdx.x & 31;
    if (alpha <= 4.0) {
        // orders 0..31 (J_k(4) < 1e-25 beyond), 24 series terms ((x/2)^2m / (m! (m+k)!) < 1e-20 beyond)
        const double x = 0.5 * alpha, mx2 = -x * x;
        const int k = lane;
        double t = 1.0;
        for (int q = 1; q <= k; ++q) t *= x * inv[q];  // x^k / k!
        double s = t;
#pragma unroll 4
        for (int m = 1; m <= 24; ++m) {
            t *= mx2 * (inv[m] * inv[m + k]);
            s += t;
        }
        J[k] = s;
        for (int q = 32 + lane; q < kIeshMaxTerms; q += 32) J[q] = 0.0;
    } else if (lane == 0) {
        const double ia = 1.0 / alpha;
        const int top = kIeshMaxTerms + 20;
        double jp1 = 0.0, jk = 1e-280, sum = 0.0;
        for (int k = top; k > 0; --k) {
            const double jm1 = (2.0 * k * ia) * jk - jp1;
            jp1 = jk;
            jk = jm1;  // J_{k-1}
            if (k - 1 < kIeshMaxTerms) J[k - 1] = jk;
            if (k - 1 > 0 && ((k - 1) & 1) == 0) sum += 2.0 * jk;
            if (fabs(jk) > 1e250) {
                jk *= 1e-250;
                jp1 *= 1e-250;
                sum *= 1e-250;
                for (int q = k - 1; q < kIeshMaxTerms; ++q) J[q] *= 1e-250;
            }
        }
        const double norm = 1.0 / (sum + jk);
        for (int q = 0; q < kIeshMaxTerms; ++q) J[q] *= norm;
    }
    __syncwarp();
    int K = -1;
    for (int k = lane; k < kIeshMaxTerms; k += 32)
        if (fabs(J[k]) >= tol) K = k;
    for (int off = 16; off > 0; off >>= 1) K = max(K, __shfl_xor_sync(0xffffffffu, K, off));
    return K >= kIeshMaxTerms - 2 ? -1 : K;
}

// iesh_bessel_warp with fewer FP64 instructions (the FP32 path; the FP64 unit of the GPU issues a
// warp instruction every few dozen cycles): x^k / k! of lane k as a prefix product over the lanes
// (5 steps instead of k), and the power series stopped once every lane's term is below 2^-60 of its
// sum (an integer test of the exponents).  The Miller recurrence beyond alpha = 4 is iesh_bessel_warp's.
__device__ inline int iesh_bessel_warp_fast(double alpha, double tol, double* J, const double* inv) {
    if (alpha > 4.0) return iesh_bessel_warp(alpha, tol, J, inv);
    const int lane = threadIdx.x & 31;
    const double x = 0.5 * alpha, mx2 = -x * x;
    const int k = lane;
    double f = k == 0 ? 1.0 : x * inv[k];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const double g = __shfl_up_sync(0xffffffffu, f, off);
        if (lane >= off) f *= g;
    }
    double t = f, s = f;
    for (int m = 1; m <= 24; ++m) {
        t *= mx2 * (inv[m] * inv[m + k]);
        s += t;
        const int et = (__double2hiint(t) >> 20) & 0x7ff, es = (__double2hiint(s) >> 20) & 0x7ff;
        if (__all_sync(0xffffffffu, et + 60 < es || et == 0)) break;
    }
    J[k] = s;
    for (int q = 32 + lane; q < kIeshMaxTerms; q += 32) J[q] = 0.0;
    __syncwarp();
    int K = -1;
    for (int q = lane; q < kIeshMaxTerms; q += 32)
        if (fabs(J[q]) >= tol) K = q;
    for (int off = 16; off > 0; off >>= 1) K = max(K, __shfl_xor_sync(0xffffffffu, K, off));
    return K >= kIeshMaxTerms - 2 ? -1 : K;
}

// k-th (0-based) unset bit among bits [0, n) of a 128-bit mask.
__device__ inline int iesh_nth_unset(const unsigned long long* m, int n, int k) {
    for (int w = 0; w < 2; ++w) {
        const int lo = 64 * w;
        if (lo >= n) break;
        const int nb = n - lo < 64 ? n - lo : 64;
        const unsigned long long valid = nb == 64 ? ~0ull : ((1ull << nb) - 1ull);
        const unsigned long long z = ~m[w] & valid;
        const int c = __popcll(z);
        if (k < c) {
            const unsigned lo32 = (unsigned)z, hi32 = (unsigned)(z >> 32);
            const int c32 = __popc(lo32);
            if (k < c32) return lo + (int)__fns(lo32, 0, k + 1);
            return lo + 32 + (int)__fns(hi32, 0, k - c32 + 1);
        }
        k -= c;
    }
    return -1;
}

// Deterministic block reductions (fixed order), result broadcast to all threads.
__device__ inline double iesh_block_sum(double x, double* red) {
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) red[w] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        double s = l < nw ? red[l] : 0.0;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (l == 0) red[64] = s;
    }
    __syncthreads();
    return red[64];
}

// FP32 form of iesh_block_sum (the fast path keeps its per-step sums off the FP64 pipe).
__device__ inline float iesh_block_sum_f(float x, double* red_) {
    float* red = (float*)red_;
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) red[w] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = l < nw ? red[l] : 0.f;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (l == 0) red[64] = s;
    }
    __syncthreads();
    return red[64];
}

// FP32 form of iesh_block_minmax; every thread receives the block's extremes.
__device__ inline void iesh_block_minmax_f(float& lo, float& hi, double* red_) {
    float* red = (float*)red_;
    for (int off = 16; off > 0; off >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, off));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, off));
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) {
        red[w] = lo;
        red[32 + w] = hi;
    }
    __syncthreads();
    for (int q = 0; q < nw; ++q) {
        lo = fminf(lo, red[q]);
        hi = fmaxf(hi, red[32 + q]);
    }
    __syncthreads();  // red is reused by the next reduction
}

// Three FP32 block sums at once (one pair of barriers); every thread receives the totals.
__device__ inline void iesh_block_sum3_f(float& a, float& b, float& c, double* red_) {
    float* red = (float*)red_;
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
        c += __shfl_xor_sync(0xffffffffu, c, off);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) {
        red[w] = a;
        red[32 + w] = b;
        red[64 + w] = c;
    }
    __syncthreads();
    a = b = c = 0.f;
    for (int q = 0; q < nw; ++q) {  // the same order in every thread
        a += red[q];
        b += red[32 + q];
        c += red[64 + q];
    }
    __syncthreads();  // red is reused by the next reduction
}

__device__ inline void iesh_block_minmax(double& lo, double& hi, double* red) {
    for (int off = 16; off > 0; off >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, off));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, off));
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) {
        red[w] = lo;
        red[32 + w] = hi;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        double a = l < nw ? red[l] : 1e300, b = l < nw ? red[32 + l] : -1e300;
        for (int off = 16; off > 0; off >>= 1) {
            a = fmin(a, __shfl_xor_sync(0xffffffffu, a, off));
            b = fmax(b, __shfl_xor_sync(0xffffffffu, b, off));
        }
        if (l == 0) {
            red[64] = a;
            red[65] = b;
        }
    }
    __syncthreads();
    lo = red[64];
    hi = red[65];
}

template <typename R>
__device__ inline R warp_sum(R x) {
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    return x;
}

template <typename R>
__device__ inline Cx<R> cx_div(Cx<R> a, Cx<R> b) {
    const R d = b.re * b.re + b.im * b.im;
    return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}

// (re, im) * 2^e with |re| + |im| kept in [0.5, 1): products of many pivots
// without overflow or underflow, in the working precision.
template <typename T>
__device__ inline void scaled_mul(T& re, T& im, int& e, T br, T bi, int be) {
    const T nr = re * br - im * bi, ni = re * bi + im * br;
    int ex;
    frexp(fabs(nr) + fabs(ni), &ex);
    re = ldexp(nr, -ex);
    im = ldexp(ni, -ex);
    e += be + ex;
}

template <typename R>
constexpr int iesh_min_blocks() {
    return std::is_same<R, float>::value ? 2 : 1;
}

// Per-thread partial sums of tr X and |X|_F^2 for X = I - G, G = S^H S the Gram matrix of the
// occupied rows of the orbitals (FP32 path, see the hop-estimate bound in iesh_body): one 2 x 2
// tile of G per thread over the upper block triangle, summed over all occupied rows.  Out of
// line, so that its registers do not add to the step loop's.
static __device__ __noinline__ float2 iesh_gram_partials(const Cx<float>* phiA, const int32_t* occ, int Ne, int Nep) {
    float trx = 0.f, fx2 = 0.f;
    const int nbk = (Ne + 1) >> 1, ntile = nbk * (nbk + 1) / 2;
    for (int t = threadIdx.x; t < ntile; t += blockDim.x) {
        // tile t, row-major over the upper block triangle: block row bi starts at
        // bi nbk - bi (bi - 1) / 2; the float estimate of bi is corrected by the integer tests
        const float c = 2.f * (float)nbk + 1.f;
        int bi = (int)((c - sqrtf(c * c - 8.f * (float)t)) * 0.5f);
        bi = bi < 0 ? 0 : (bi >= nbk ? nbk - 1 : bi);
        while (bi > 0 && bi * nbk - bi * (bi - 1) / 2 > t) --bi;
        while (bi + 1 < nbk && (bi + 1) * nbk - (bi + 1) * bi / 2 <= t) ++bi;
        const int bj = bi + t - (bi * nbk - bi * (bi - 1) / 2);
        const int a0 = 2 * bi, b0 = 2 * bj;
        float gr[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, gi[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
        for (int j = 0; j < Ne; ++j) {  // columns a0, a0 + 1 < Nep of row occ[j]
            const float4* row = (const float4*)(phiA + occ[j] * Nep);
            const float4 x = row[a0 >> 1], y = row[b0 >> 1];
            const float xr[2] = {x.x, x.z}, xi[2] = {x.y, x.w};
            const float yr[2] = {y.x, y.z}, yi[2] = {y.y, y.w};
#pragma unroll
            for (int uu = 0; uu < 2; ++uu)
#pragma unroll
                for (int vv = 0; vv < 2; ++vv) {  // conj(x) y
                    gr[uu][vv] = fmaf(xr[uu], yr[vv], fmaf(xi[uu], yi[vv], gr[uu][vv]));
                    gi[uu][vv] = fmaf(xr[uu], yi[vv], fmaf(-xi[uu], yr[vv], gi[uu][vv]));
                }
        }
#pragma unroll
        for (int uu = 0; uu < 2; ++uu)
#pragma unroll
            for (int vv = 0; vv < 2; ++vv) {
                const int a = a0 + uu, b = b0 + vv;
                if (a >= Ne || b >= Ne || a > b) continue;
                if (a == b) {
                    const float d = 1.f - gr[uu][vv];
                    trx += d;
                    fx2 = fmaf(d, d, fx2);
                } else {
                    fx2 += 2.f * (gr[uu][vv] * gr[uu][vv] + gi[uu][vv] * gi[uu][vv]);
                }
            }
    }
    return make_float2(trx, fx2);
}

// Model functions at height z: h, dh/dz (FP32 on the fast path).
template <typename R>
__device__ inline void iesh_level(const IeshParams& p, double z, double& h, double& dh) {
    if constexpr (std::is_same<R, float>::value) {
        const float e = expf(-(float)p.b * (float)z);
        h = (double)((float)p.delta - (float)p.B * e);
        dh = (double)((float)p.B * (float)p.b * e);
    } else {
        const double e = nqcd_exp(-p.b * z);
        h = p.delta - p.B * e;
        dh = p.B * p.b * e;
    }
}

template <typename R>
__device__ inline double iesh_wall(const IeshParams& p, double z) {  // exp(-a z)
    if constexpr (std::is_same<R, float>::value)
        return (double)expf(-(float)p.a * (float)z);
    else
        return nqcd_exp(-p.a * z);
}

// One CTA integrates one trajectory.  Warp 0 owns the nuclear state (every
// lane holds the same copy) and the serial FP64 work; it publishes h, dh/dz
// and v . grad h through shared memory.  All threads share the root solve,
// the coupling matrix, the propagator and the hop linear algebra.
//
// RP = true: RingPolymerSimulation{AdiabaticIESH} (rpiesh.jl) with
// BCBWavefunction (bcb_wavefunction.jl:37-69).  Lane j of warp 0 holds bead j;
// the step is a half kick, the full Cayley step of the free ring polymer in
// normal modes (ring_polymer.jl:71-82), the bead forces from each bead's own
// eigenstates summed over the shared occupied set (rpiesh.jl:20-37) and a half
// kick.  The orbitals are propagated with the centroid velocity of the step's
// start and the centroid eigenvalues and couplings of its end (the calculator
// cache holds the end positions when propagate_wavefunction! reads it,
// bcb_wavefunction.jl:59-68 with SurfaceHoppingMethods.jl:81-103); hops use
// the final centroid velocity, and their velocity change is the same in every
// bead (rpsh.jl:30-50).  Fermi-Dirac occupations come from the centroid
// eigenvalues (iesh.jl:99-128).
// TC: the tensor-core propagator (R = float only); a separate instantiation so
// that the CUDA-core kernel keeps its own register allocation.
template <typename R, bool RP, bool TC>
__device__ __forceinline__ void iesh_body(const IeshParams& p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const IeshLayout L = iesh_layout<R>(p.nstates, p.nelec, RP ? p.nbeads : 1, TC);
    R* eps = (R*)(smem + L.o_eps);
    R* V2 = (R*)(smem + L.o_V2);
    R* lam = (R*)(smem + L.o_lam);
    R* z2 = (R*)(smem + L.o_z2);
    R* z0 = (R*)(smem + L.o_z0);
    double* w64 = (double*)(smem + L.o_w64);
    R* At = (R*)(smem + L.o_At);
    Cx<R>* phiA = (Cx<R>*)(smem + L.o_phiA);
    Cx<R>* phiB = (Cx<R>*)(smem + L.o_phiB);
    Cx<R>* outb = (Cx<R>*)(smem + L.o_out);
    double* Jc = (double*)(smem + L.o_J);
    R* Jr = (R*)(smem + L.o_Jr);  // 2 J_k in the working precision
    double* inv = (double*)(smem + L.o_inv);
    double* fdu = (double*)(smem + L.o_fdu);
    unsigned char* fdi = (unsigned char*)(smem + L.o_fdi);
    int* occ = (int*)(smem + L.o_occ);
    int* unocc = (int*)(smem + L.o_unocc);
    int* piv = (int*)(smem + L.o_piv);
    double* red = (double*)(smem + L.o_red);
    // misc: [0] K [1] sin(c dt) [2] cos(c dt), then the full-evaluation flag [3] v_z [4] h [5] dh/dz
    //       [6] v . grad h [8] c [9] 1/hw [10] w/hw [11] J_0
    double* misc = (double*)(smem + L.o_misc);
    // FP32 path: the same step values as floats and ints, written once by their producer so that
    // their readers convert nothing (conversions issue on this GPU's FP64 unit): mf[1] sin, [2] cos,
    // [4] h, [5] root bracket |h| + L, [6] v . grad h, [8] c, [9] 1/hw, [10] w/hw, [11] J_0,
    // [12] final centroid v . grad h, [13] cached alpha; mi[0] K
    float* mf = (float*)(misc + 20);
    int* mi = (int*)(misc + 28);
    // ring polymer: rph[b] h, rph[NB + b] dh/dz, rph[2 NB + b] sum of occupied z0^2, rph[3 NB + b] sum of
    // occupied eigenvalues of bead b; rpq [6][NB] normal-mode scratch.  misc[12] v . grad h of the final
    // centroid velocity (hops), [13] final centroid v_z, [14] centroid z
    double* rph = (double*)(smem + L.o_rph);
    double* rpq = (double*)(smem + L.o_rpq);
    const int NB = RP ? p.nbeads : 1;

    const int N = L.N, Ne = L.Ne, Nu = L.Nu, Np = L.Np, Nep = L.Nep, M = p.nbath;
    const int tid = threadIdx.x, nthr = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ti = blockIdx.x;
    const int64_t NT = p.ntraj;
    const uint64_t gid = (uint64_t)(p.traj_offset + ti);
    const double mass = p.mass, inv_mass = 1.0 / p.mass, dt = p.dt;
    unsigned long long* nonconv = p.counters ? p.counters + 2 : nullptr;

    for (int k = tid; k < Np; k += nthr) {
        eps[k] = k < M ? (R)p.eps[k] : R(0);
        V2[k] = k < M ? (R)p.V2[k] : R(0);
        lam[k] = R(0);
        z2[k] = R(0);
        z0[k] = R(0);
    }
    constexpr bool kF32 = std::is_same<R, float>::value;
    // tensor-core propagator (FP32 path): operands in shared memory, accumulator, phi_{k-2} and the
    // series sum in TMEM columns of this CTA
    constexpr bool tcp = kF32 && TC;
    unsigned char* aop_hi = smem + L.o_tc;  // A operand: the orbital block transposed, rows 2 e + (re, im)
    unsigned char* aop_lo = aop_hi + L.tc_sa;
    unsigned char* bop = aop_hi + 2 * L.tc_sa;  // B operand: the coupling matrix A (tf32), row i, k = j
    __shared__ __align__(8) uint64_t tc_bar;
    __shared__ uint32_t tc_slot;
    __shared__ int tc_fail;
    uint32_t tmem = 0, tc_phase = 0;
    // TMEM columns: a power of two >= 3 N (256 at N = 80: two CTAs share an SM's 512)
    uint32_t tc_cols = 32;
    while (tc_cols < 3u * (uint32_t)L.N) tc_cols <<= 1;
    if constexpr (tcp) {
        {
            if (tid == 0) {
                tc::mbar_init(&tc_bar, 1);
                asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
                tc_fail = 0;
            }
            if (warp == 0) tc::tmem_alloc(&tc_slot, tc_cols);
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            tmem = tc_slot;
        }
    }
    if (!tcp)
        for (int q = tid; q < Np * Np; q += nthr) At[q] = R(0);
    for (int q = tid; q < Np * Nep; q += nthr) {
        phiA[q] = {R(0), R(0)};
        phiB[q] = {R(0), R(0)};
        outb[q] = {R(0), R(0)};
    }
    for (int q = tid; q < kIeshInv; q += nthr) inv[q] = q ? 1.0 / q : 0.0;

    double r[3], v[3], k[3];  // meaningful in warp 0 (ring polymer: bead `lane`, lanes >= NB a copy of bead 0)
    const int bead = RP && lane < NB ? lane : 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        r[d] = p.r[(int64_t)(d + 3 * bead) * NT + ti];
        v[d] = p.v[(int64_t)(d + 3 * bead) * NT + ti];
        k[d] = 0.0;
    }
    const double Lpad = fabs(p.eps[0]) + fabs(p.eps[M - 1]) + 1.0 + p.sumV2;
    // thread i < N owns root i and warm-starts it from the previous step
    R lam_own = R(0);
    // FP32 path: during the step loop the w64 region holds every root as a float pair whi + wlo
    // (the FP64 root of a refined one, the FP32 root and 0 for the others), and fp64_now tells
    // whether this step refined any
    float* whi = (float*)w64;
    float* wlo = whi + Np;
    bool fp64_now = false;
    int nfp64 = 0;
    auto roots = [&]() {  // after a barrier that published misc[4] = h
        const double hz = misc[4];
        if (tid < N) {
            R zz;
            if constexpr (kF32)
                secular_root<R>(eps, V2, M, tid, mf[4], mf[5], lam_own, zz, nonconv);
            else
                secular_root<R>(eps, V2, M, tid, (R)hz, (R)(fabs(hz) + Lpad), lam_own, zz, nonconv);
            lam[tid] = lam_own;
            z2[tid] = zz;
            z0[tid] = sqrt(zz);
        }
        if constexpr (std::is_same<R, float>::value) {
            // near-degeneracy fallback: a root whose neighbour lies closer than gap_fp64 is solved
            // again in FP64 (warm start from the FP32 root), which fixes the small gap that divides
            // its couplings.  Two roots closer than the threshold are both flagged: each has the
            // other as a neighbour, and a root whose neighbours are both at least the threshold
            // away is at least that far from every root.
            __syncthreads();
            bool flag = false;
            if (tid < N && p.gap_fp64 > 0.0) {
                // neighbouring roots differ by less than a factor of 2 where it matters, so the
                // FP32 differences are exact there (Sterbenz)
                const float lo = tid > 0 ? (float)lam[tid] - (float)lam[tid - 1] : 3.0e38f;
                const float hi = tid + 1 < N ? (float)lam[tid + 1] - (float)lam[tid] : 3.0e38f;
                flag = fminf(lo, hi) < (float)p.gap_fp64;
                float h = (float)lam_own, l = 0.f;
                if (flag) {
                    double l64 = (double)lam_own, zz64;
                    secular_root<double>(p.eps, p.V2, M, tid, hz, fabs(hz) + Lpad, l64, zz64, nonconv);
                    z0[tid] = (R)sqrt(zz64);
                    z2[tid] = (R)zz64;
                    h = (float)l64;
                    l = (float)(l64 - (double)h);
                }
                whi[tid] = h;
                wlo[tid] = l;
            }
            fp64_now = __syncthreads_or(flag) != 0;
            nfp64 += fp64_now ? 1 : 0;
        } else {
            __syncthreads();
        }
    };
    // coupling denominator l_j - l_i: on a step with refined roots from the float pairs (the high
    // parts of close roots subtract exactly, the low parts add the FP64 remainder)
    auto gap = [&](int i, int j) -> R {
        if constexpr (std::is_same<R, float>::value) {
            if (fp64_now) return (whi[j] - whi[i]) + (wlo[j] - wlo[i]);
        }
        return lam[j] - lam[i];
    };
    // A_ij = z0_i z0_j / (l_j - l_i): from the step's matrix, or formed here where the tensor-core layout
    // keeps only its tf32 copy
    auto coup = [&](int i, int j) -> R { return tcp ? z0[i] * z0[j] / gap(i, j) : At[j * Np + i]; };
    // FP32 path, bound on the hop estimate without the LU.  S = psi[occ, :] (Ne x Ne) and
    // |det S|^2 = det G with G = S^H S, the Gram matrix of the occupied rows.  X = I - G is
    // Hermitian; for its eigenvalues |mu| <= rho < 1, log(1 - mu) >= -mu - mu^2 / (2 (1 - rho)), so
    //     -log |det S|^2 <= tr X + |X|_F^2 / (2 (1 - |X|_F))   when |X|_F < 1,
    // and with |Re d| + |Im d| <= sqrt(2) |d| the estimate 2 dt sum|v.d| (|Re d| + |Im d|) / |d|^2
    // of iesh.jl:253-256 is at most 2 sqrt(2) dt sum|v.d| / |det S|.
    auto gram_partials = [&](float& trx, float& fx2) {
        if constexpr (kF32) {
            const float2 g = iesh_gram_partials(phiA, occ, Ne, Nep);
            trx += g.x;
            fx2 += g.y;
        }
    };
    // The bound of gram_partials against u.  The margins cover the FP32 sums: each G entry sums
    // at most 2 Ne products of unit-bounded terms (error below 3e-6 for Ne <= 64), so tr X is off by
    // less than 2e-4 and |X|_F by less than 3e-4; sum|A| and exp by far less than 1 %.
    auto estimate_certainly_below = [&](float trx, float fx2, float sabs, float wh_, float u_) -> bool {
        const float tr = fmaxf(trx, 0.f) * 1.001f + 1e-3f;
        const float fr = sqrtf(fmaxf(fx2, 0.f)) * 1.001f + 1e-3f;
        if (!(fr < 0.95f)) return false;
        const float ld = tr + fr * fr / (2.f * (1.f - fr));  // >= -log |det S|^2
        const float bound = 2.8285f * (float)dt * fabsf(wh_) * sabs * expf(0.5f * ld);
        return bound * 1.02f < u_;
    };
    // ---- ring polymer ----
    // mean over the beads of warp 0 (the same value in every lane)
    auto bead_mean = [&](double x) {
        double sm = lane < NB ? x : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, off);
        return sm / (double)NB;
    };
    // warp 0: h and dh/dz of each bead into rph, the centroid's into hz, dhz and misc[4], misc[5]
    auto publish_levels = [&](double& hz_, double& dhz_) {
        if constexpr (RP) {
            double hb, dhb;
            iesh_level<R>(p, r[2], hb, dhb);
            if (lane < NB) {
                rph[lane] = hb;
                rph[NB + lane] = dhb;
            }
            const double zc = bead_mean(r[2]);
            iesh_level<R>(p, zc, hz_, dhz_);
            if (lane == 0) misc[14] = zc;
        } else {
            iesh_level<R>(p, r[2], hz_, dhz_);
        }
        if (lane == 0) {
            misc[4] = hz_;
            misc[5] = dhz_;
            if constexpr (kF32) {
                mf[4] = (float)hz_;
                mf[5] = (float)(fabs(hz_) + Lpad);
            }
        }
    };
    // roots of the occupied states of every bead (warp w: beads w, w + 8, ...; lane: electrons lane,
    // lane + 32), reduced per bead to the sums of z0^2 and of the eigenvalues; after a barrier that
    // published rph[0, 2 NB) and the occupations
    R wl[kRpIeshMaxBeads / (kIeshBlock / 32)][2];  // warm starts (any value is a valid start)
    if constexpr (RP) {
#pragma unroll
        for (int i = 0; i < kRpIeshMaxBeads / (kIeshBlock / 32); ++i) wl[i][0] = wl[i][1] = R(0);
    }
    auto bead_roots = [&]() {
        if constexpr (RP) {
#pragma unroll 1
            for (int i = 0; i < kRpIeshMaxBeads / (kIeshBlock / 32); ++i) {
                const int b = warp + (kIeshBlock / 32) * i;
                if (b >= NB) break;  // warp-uniform
                const double hb = rph[b];
                R sz = R(0), sl = R(0);
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const int e = lane + 32 * j;
                    if (e < Ne) {
                        R zz;
                        secular_root<R>(eps, V2, M, occ[e], (R)hb, (R)(fabs(hb) + Lpad), wl[i][j], zz, nonconv);
                        sz += zz;
                        sl += wl[i][j];
                    }
                }
                sz = warp_sum<R>(sz);
                sl = warp_sum<R>(sl);
                if (lane == 0) {
                    rph[2 * NB + b] = (double)sz;
                    rph[3 * NB + b] = (double)sl;
                }
            }
            if (tid == 0) misc[15] = 0.0;  // the sums hold the current occupations
            __syncthreads();
        }
    };
    // warp 0: full Cayley step of the free ring polymer (cayley_propagator(half=false),
    // bcb_wavefunction.jl:52-56): to normal modes, rotate each mode, back to beads; per Cartesian dof
    auto free_step = [&](double* x, double* y) {
        if (lane < NB)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                rpq[d * NB + lane] = x[d];
                rpq[(3 + d) * NB + lane] = y[d];
            }
        __syncwarp();
        double qx[3] = {0.0, 0.0, 0.0}, qy[3] = {0.0, 0.0, 0.0};
        if (lane < NB) {
            const double* c = p.rp_cay + 4 * lane;  // mode `lane`
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                double a = 0.0, b = 0.0;
                for (int j = 0; j < NB; ++j) {
                    const double u = p.rp_U[j + NB * lane];
                    a = a + u * rpq[d * NB + j];
                    b = b + u * rpq[(3 + d) * NB + j];
                }
                qx[d] = c[0] * a + c[1] * b;
                qy[d] = c[2] * a + c[3] * b;
            }
        }
        __syncwarp();
        if (lane < NB)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                rpq[d * NB + lane] = qx[d];
                rpq[(3 + d) * NB + lane] = qy[d];
            }
        __syncwarp();
        if (lane < NB)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                double a = 0.0, b = 0.0;
                for (int q = 0; q < NB; ++q) {
                    const double u = p.rp_U[lane + NB * q];
                    a = a + u * rpq[d * NB + q];
                    b = b + u * rpq[(3 + d) * NB + q];
                }
                x[d] = a;
                y[d] = b;
            }
        __syncwarp();
    };
    // warp 0: ring-polymer Hamiltonian (DynamicsUtils.jl:74-79): kinetic + sum over beads of U0 and the
    // occupied eigenvalues (rpiesh.jl:39-52) + spring energy (ring_polymer.jl:85-107); after bead_roots
    auto rp_energy = [&]() {
        const int nb = lane + 1 < NB ? lane + 1 : 0;
        double sp = 0.0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double dx = r[d] - __shfl_sync(0xffffffffu, r[d], nb);
            sp += dx * dx;
        }
        const double e = 0.5 * mass * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) + 0.5 * p.kxy * (r[0] * r[0] + r[1] * r[1]) +
                         p.A * iesh_wall<R>(p, r[2]) + rph[3 * NB + bead] + 0.5 * mass * p.omega_n * p.omega_n * sp;
        return bead_mean(e) * (double)NB;
    };
    // EhrenfestNA (ehrenfest_na.jl): the force and energy come from the orbitals
    // instead of the occupations.  With A = dh z0 z0^T the force weight
    // sum_e sum_nm A_nm Re(psi_ne conj(psi_me)) is dh times the impurity
    // population sum_e |sum_a z0_a psi_ae|^2 (ehrenfest_na.jl:74-90); the band
    // energy is sum_e sum_i l_i |psi_ie|^2 (ehrenfest_na.jl:106-117).  Block-wide.
    const bool ena = p.ehrenfest_na != 0;
    double ena_imp = 0.0, ena_band = 0.0;
    auto orbital_sums = [&]() {
        double ci = 0.0, cb = 0.0;
        for (int e = tid; e < Ne; e += nthr) {
            R ar = R(0), ai = R(0), b = R(0);
            for (int a = 0; a < N; ++a) {
                const Cx<R> c = phiA[a * Nep + e];
                ar += z0[a] * c.re;
                ai += z0[a] * c.im;
                b += lam[a] * (c.re * c.re + c.im * c.im);
            }
            ci += (double)ar * (double)ar + (double)ai * (double)ai;
            cb += (double)b;
        }
        ena_imp = iesh_block_sum(ci, red);
        ena_band = iesh_block_sum(cb, red);
    };
    auto accel = [&](double dh) {  // warp 0
        if constexpr (RP) {  // bead `lane`: its own level derivative and occupied z0^2 (after bead_roots)
            const double eaz = iesh_wall<R>(p, r[2]);
            k[0] = -(p.kxy * r[0]) * inv_mass;
            k[1] = -(p.kxy * r[1]) * inv_mass;
            k[2] = -(-p.A * p.a * eaz + rph[NB + bead] * rph[2 * NB + bead]) * inv_mass;
            return;
        }
        R acc = R(0);
        for (int jj = lane; jj < Ne; jj += 32) acc += z2[occ[jj]];
        const double occsum = ena ? ena_imp : (double)warp_sum<R>(acc);
        const double eaz = iesh_wall<R>(p, r[2]);
        k[0] = -(p.kxy * r[0]) * inv_mass;
        k[1] = -(p.kxy * r[1]) * inv_mass;
        k[2] = -(-p.A * p.a * eaz + dh * occsum) * inv_mass;
    };
    auto potential = [&]() {  // warp 0: U0 + sum of occupied eigenvalues (iesh.jl:380-388)
        R acc = R(0);
        for (int jj = lane; jj < Ne; jj += 32) acc += lam[occ[jj]];
        const double band = ena ? ena_band : (double)warp_sum<R>(acc);
        return 0.5 * p.kxy * (r[0] * r[0] + r[1] * r[1]) + p.A * iesh_wall<R>(p, r[2]) + band;
    };
    auto kinetic = [&]() { return 0.5 * mass * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
    auto rebuild_unocc = [&]() {  // ascending, as set_unoccupied_states! (DynamicsUtils.jl:162-171)
        unsigned long long m2[2] = {0ull, 0ull};
        for (int jj = 0; jj < Ne; ++jj) m2[occ[jj] >> 6] |= 1ull << (occ[jj] & 63);
        int u = 0;
        for (int s = 0; s < N; ++s)
            if (!((m2[s >> 6] >> (s & 63)) & 1ull)) unocc[u++] = s;
    };

    // ---- initial electronic structure and occupations ----
    lam_own = tid == 0 ? eps[0] - R(1e-3) : (tid <= M ? eps[tid - 1] + R(1e-9) : R(0));
    double hz = 0.0, dhz = 0.0;
    if (warp == 0) publish_levels(hz, dhz);
    __syncthreads();
    roots();
    nfp64 = 0;  // the count is of integration steps
    const double z_fd = RP ? misc[14] : r[2];  // where the Fermi-Dirac eigenvalues are taken
    if (p.init_kind == IESH_INIT_FERMI_DIRAC) {
        // Metropolis over occupations with the Boltzmann ratio (DynamicsUtils.jl:194-208).
        // Acceptance exp(-beta (e_j - e_i)) > u is tested as w_j > u w_i with
        // w_s = exp(-beta (e_s - e_ref)); FP64 eigenvalues on both paths.
        __shared__ int bad_weight;
        if (tid == 0) bad_weight = 0;
        __syncthreads();
        const double eref = 0.5 * (p.eps[0] + p.eps[M - 1]);
        if (tid < N) {
            double l64;
            if constexpr (std::is_same<R, double>::value) {
                l64 = lam[tid];
            } else {
                // FP64 roots warm-started from the FP32 roots just solved at the same height (a
                // step or two of Newton instead of a cold start's many)
                const double h64 = p.delta - p.B * nqcd_exp(-p.b * z_fd);
                double zz;
                l64 = (double)lam_own;
                secular_root<double>(p.eps, p.V2, M, tid, h64, fabs(h64) + Lpad, l64, zz, nonconv);
            }
            const double wt = nqcd_exp(-p.beta * (l64 - eref));
            w64[tid] = l64;
            if (!(wt > 0.0 && wt < 1e300)) bad_weight = 1;
            else w64[tid] = wt;
        }
        __syncthreads();
        const bool direct = bad_weight != 0;  // weights out of range: exponentiate each difference
        if (direct && tid < N) {               // w64 must hold the eigenvalues then
            if constexpr (std::is_same<R, double>::value) {
                w64[tid] = lam[tid];
            } else {
                const double h64 = p.delta - p.B * nqcd_exp(-p.b * z_fd);
                double zz, l64 = (double)lam_own;
                secular_root<double>(p.eps, p.V2, M, tid, h64, fabs(h64) + Lpad, l64, zz, nullptr);
                w64[tid] = l64;
            }
        }
        unsigned long long m2[2] = {0ull, 0ull};
        if (tid == 0)
            for (int jj = 0; jj < Ne; ++jj) {
                occ[jj] = jj;
                m2[jj >> 6] |= 1ull << (jj & 63);
            }
        const int total = N * Ne;
        for (int base = 0; base < total; base += kIeshFdChunk) {
            const int cnt = total - base < kIeshFdChunk ? total - base : kIeshFdChunk;
            __syncthreads();
            for (int q = tid; q < cnt; q += nthr) {
                const int it = base + q;
                const u32x4 wa = rng_block(p.seed, gid, (uint32_t)it, RNG_INIT_FD);
                const u32x4 wb = rng_block(p.seed, gid, (uint32_t)it, RNG_INIT_FD + 16);
                int ci = (int)(u01_from_words(wa.x, wa.y) * Ne);
                if (ci > Ne - 1) ci = Ne - 1;
                int pick = (int)(u01_from_words(wa.z, wa.w) * Nu);
                if (pick > Nu - 1) pick = Nu - 1;
                fdi[2 * q] = (unsigned char)ci;
                fdi[2 * q + 1] = (unsigned char)pick;
                fdu[q] = u01_from_words(wb.x, wb.y);
            }
            __syncthreads();
            if (tid == 0)
                for (int q = 0; q < cnt; ++q) {
                    const int ci = fdi[2 * q];
                    const int j = iesh_nth_unset(m2, N, fdi[2 * q + 1]);
                    const int i = occ[ci];
                    const bool acc = direct ? nqcd_exp(-p.beta * (w64[j] - w64[i])) > fdu[q] : w64[j] > fdu[q] * w64[i];
                    if (acc) {
                        m2[i >> 6] &= ~(1ull << (i & 63));
                        m2[j >> 6] |= 1ull << (j & 63);
                        occ[ci] = j;
                    }
                }
        }
        if (tid == 0) {
            for (int a = 1; a < Ne; ++a) {  // sort!(state)
                const int x = occ[a];
                int b = a - 1;
                while (b >= 0 && occ[b] > x) {
                    occ[b + 1] = occ[b];
                    --b;
                }
                occ[b + 1] = x;
            }
            rebuild_unocc();
        }
    } else if (tid == 0) {
        for (int jj = 0; jj < Ne; ++jj) occ[jj] = p.occ0[(int64_t)jj * NT + ti];
        rebuild_unocc();
    }
    __syncthreads();
    for (int jj = tid; jj < Ne; jj += nthr) phiA[occ[jj] * Nep + jj] = {R(1), R(0)};
    if (ena) {
        __syncthreads();
        orbital_sums();
    }
    bead_roots();
    double e0 = 0.0;
    if (warp == 0) {
        accel(dhz);
        if constexpr (RP) {
            e0 = rp_energy();
        } else {
            const double pe = potential();
            e0 = kinetic() + pe;
        }
    }
    __syncthreads();

    // matrix-product tiles
    const int CG = Nep >> 2, RG = Np >> 2;
    const int ntile = RG * CG;
    const bool tile_on = tid < ntile;
    const int i0 = tile_on ? tid / CG : 0;  // rows i0 + RG rr
    const int c0 = tile_on ? tid % CG : 0;  // orbitals c0 + CG cc

    auto save = [&](int isave) {
        // impurity population (iesh_diabatic_population, row 0 of Z rho Z^T)
        double contrib = 0.0;
        if (tid < Ne) {
            R ar = R(0), ai = R(0), sq = R(0);
            for (int a = 0; a < N; ++a) {
                const Cx<R> c = phiA[a * Nep + tid];
                ar += z0[a] * c.re;
                ai += z0[a] * c.im;
                sq += z2[a] * (c.re * c.re + c.im * c.im);
            }
            contrib = (double)ar * (double)ar + (double)ai * (double)ai - (double)sq + (double)z2[occ[tid]];
        }
        double nimp = iesh_block_sum(contrib, red);
        if (ena) {  // impurity population of the orbitals themselves
            orbital_sums();
            nimp = ena_imp;
        }
        if constexpr (RP) {
            // bead eigenvalue sums of the current occupations (a hop of this step changed them)
            // every thread reads the flag before bead_roots clears it
            const bool stale = misc[15] != 0.0;
            __syncthreads();
            if (stale) bead_roots();
        }
        if (warp == 0) {
            double pe, ke, zs;
            if constexpr (RP) {
                // centroid height, kinetic energy of all beads, sum over beads of U0 and the occupied
                // eigenvalues (classical_kinetic_energy, DynamicsUtils.jl:122-132; rpiesh.jl:40-52)
                pe = bead_mean(0.5 * p.kxy * (r[0] * r[0] + r[1] * r[1]) + p.A * iesh_wall<R>(p, r[2]) +
                               rph[3 * NB + bead]) * (double)NB;
                ke = bead_mean(kinetic()) * (double)NB;
                zs = bead_mean(r[2]);
            } else {
                pe = potential();
                ke = kinetic();
                zs = r[2];
            }
            if (lane == 0 && isave < p.nsave) {
                double* dst = p.obs_partial + (ti * p.nsave + isave) * 4;
                dst[0] = zs;
                dst[1] = ke;
                dst[2] = nimp;
                dst[3] = pe;
            }
        }
        __syncthreads();  // the next step rewrites the roots warp 0 just read
    };
    int isave = 0;
    if (tid == 0) {
        mf[13] = -1.f;    // no Bessel coefficients cached yet (FP32 path)
        misc[15] = 0.0;   // ring polymer: bead eigenvalue sums current
    }
    if (p.save_stride > 0 && p.obs_partial) save(isave++);

    int nh = 0, nf = 0;
    unsigned long long nterms = 0;
    unsigned nfull = 0, nlu = 0;  // per trajectory at most one per step
    for (int step = 1; step <= p.nsteps; ++step) {
        // ---- velocity Verlet (verlet_with_electronics.jl:55-63) ----
        // the integrator's dt (the shortened last step reaches t1); the hop probability and the
        // decoherence correction read get_proposed_dt, the full dt
        const double hs = step == p.nsteps ? p.h_last : dt, hh = hs / 2.0;
        double vzc0 = 0.0;  // ring polymer: centroid v_z at the step's start
        if (warp == 0) {
            if constexpr (RP) vzc0 = bead_mean(v[2]);
            // v holds the half-step velocity until the second kick
#pragma unroll
            for (int d = 0; d < 3; ++d) v[d] = v[d] + hh * k[d];
            if constexpr (RP) {
                free_step(r, v);
            } else {
#pragma unroll
                for (int d = 0; d < 3; ++d) r[d] = r[d] + hs * v[d];
            }
            publish_levels(hz, dhz);
        }
        __syncthreads();
        roots();
        bead_roots();
        if (ena) orbital_sums();  // orbitals before this step's propagation, roots at the new position
        if (warp == 0) {
            accel(dhz);
#pragma unroll
            for (int d = 0; d < 3; ++d) v[d] = v[d] + hh * k[d];
            // v . grad h: the couplings are d_alpha = dh/dalpha A
            if constexpr (RP) {
                const double vzc = bead_mean(v[2]);
                if (lane == 0) {
                    misc[6] = vzc0 * dhz;
                    misc[12] = vzc * dhz;
                    misc[13] = vzc;
                    if constexpr (kF32) {
                        mf[6] = (float)misc[6];
                        mf[12] = (float)misc[12];
                    }
                }
            } else {
                if (lane == 0) {
                    misc[6] = v[2] * dhz;
                    if constexpr (kF32) mf[6] = (float)misc[6];
                }
            }
        }
        // ---- propagator (wavefunction_dynamics.jl:15-58) ----
        if constexpr (tcp) {
            // the coupling matrix rounded to tf32 as the B operand (row i, k = j); rounding to
            // nearest keeps it antisymmetric, so H_eff stays Hermitian.  Thread i of part p
            // (tid = p N + i) writes row i of the k-blocks p, p + parts, ...: consecutive threads
            // fill one core matrix with 16-byte stores (no bank conflicts), and the four z0_j and
            // l_j of a block are one broadcast float4 load each.  The quotient takes the
            // approximate reciprocal (2 ulp, far below the tf32 rounding; it is odd in the
            // denominator, so the matrix stays antisymmetric).  The branch on refined roots is
            // taken once, outside the loop.
            const int parts = nthr / N, part = tid / N, i = tid - part * N;
            if (part < parts) {
                const float zi = z0[i];
                auto bval = [&](int j, float zj, float g) -> float {
                    return i == j ? 0.f : tc::to_tf32(__fdividef(zi * zj, g));
                };
                if (fp64_now) {  // gaps from the float pairs of the refined roots
                    for (int j4 = part; j4 < N / 4; j4 += parts) {
                        const int j0 = 4 * j4;
                        const float4 zj = *(const float4*)(z0 + j0);
                        const float4 a = make_float4(bval(j0, zj.x, gap(i, j0)), bval(j0 + 1, zj.y, gap(i, j0 + 1)),
                                                     bval(j0 + 2, zj.z, gap(i, j0 + 2)), bval(j0 + 3, zj.w, gap(i, j0 + 3)));
                        *(float4*)(bop + tc::smem_kmajor_offset(i, j0, N)) = a;
                    }
                } else {
                    const float li = lam[i];
                    for (int j4 = part; j4 < N / 4; j4 += parts) {
                        const int j0 = 4 * j4;
                        const float4 zj = *(const float4*)(z0 + j0);
                        const float4 lj = *(const float4*)(lam + j0);
                        const float4 a = make_float4(bval(j0, zj.x, lj.x - li), bval(j0 + 1, zj.y, lj.y - li),
                                                     bval(j0 + 2, zj.z, lj.z - li), bval(j0 + 3, zj.w, lj.w - li));
                        *(float4*)(bop + tc::smem_kmajor_offset(i, j0, N)) = a;
                    }
                }
            }
        } else {
            for (int q = tid; q < N * N; q += nthr) {
                const int j = q / N, i = q - j * N;
                At[j * Np + i] = i == j ? R(0) : z0[i] * z0[j] / gap(i, j);
            }
        }
        __syncthreads();
        const double w = misc[6];
        const double wh = RP ? misc[12] : w;  // hops: v . grad h with the final (centroid) velocity
        if constexpr (kF32) {
            // FP32 path: the enclosure in FP32 (its margin covers the rounding), the Bessel
            // coefficients for alpha = hw h rounded up to 1/32 (a wider enclosure is still one), kept
            // in shared memory while alpha does not change (misc[16] alpha, misc[17] K)
            float flo = 3.0e38f, fhi = -3.0e38f;
            if (tid < N) {
                float sacc = 0.f;
                if (tcp) {  // row sums of the matrix the tensor cores multiply with
                    for (int j4 = 0; j4 < N / 4; ++j4) {
                        const float4 a = *(const float4*)(bop + tc::smem_kmajor_offset(tid, 4 * j4, N));
                        sacc += fabsf(a.x) + fabsf(a.y) + fabsf(a.z) + fabsf(a.w);
                    }
                } else {
                    for (int j = 0; j < N; ++j) sacc += fabsf((float)At[j * Np + tid]);
                }
                const float rad = fabsf(mf[6]) * sacc;
                flo = (float)lam[tid] - rad;
                fhi = (float)lam[tid] + rad;
            }
            iesh_block_minmax_f(flo, fhi, red);
            if (warp == 0) {
                const float cen = 0.5f * (fhi + flo);
                const float hw = 0.5f * (fhi - flo) * (1.f + 1e-5f) + 1e-30f;
                const float aq = ceilf(hw * (float)hs * 32.f) * (1.f / 32.f);
                if (aq != mf[13]) {  // the same in every lane
                    const int Kq = iesh_bessel_warp_fast((double)aq, p.cheb_tol, Jc, inv);
                    for (int q = lane; q < kIeshMaxTerms; q += 32) Jr[q] = (R)(2.0 * Jc[q]);
                    __syncwarp();
                    if (lane == 0) {
                        mf[13] = aq;
                        mi[0] = Kq;
                        mf[11] = (float)Jc[0];
                    }
                }
                if (lane == 0) {
                    float sn, cs;
                    sincosf(cen * (float)hs, &sn, &cs);  // exp(-i c h) = cs - i sn
                    const float hwq = aq / (float)hs;
                    mf[1] = sn;
                    mf[2] = cs;
                    mf[8] = cen;
                    mf[9] = 1.f / hwq;
                    mf[10] = mf[6] / hwq;
                }
            }
        } else {
        double elo = 1e300, ehi = -1e300;
            if (tid < N) {
                R sacc = R(0);
                if (tcp) {  // row sums of the matrix the tensor cores multiply with
                    for (int j4 = 0; j4 < N / 4; ++j4) {
                        const float4 a = *(const float4*)(bop + tc::smem_kmajor_offset(tid, 4 * j4, N));
                        sacc += (R)(fabsf(a.x) + fabsf(a.y) + fabsf(a.z) + fabsf(a.w));
                    }
                } else {
                    for (int j = 0; j < N; ++j) sacc += fabs(At[j * Np + tid]);
                }
                const double rad = fabs(w) * (double)sacc;
                elo = (double)lam[tid] - rad;
                ehi = (double)lam[tid] + rad;
            }
            iesh_block_minmax(elo, ehi, red);
            if (warp == 0) {
                // enclosure [c - hw, c + hw] of the spectrum, widened by a margin that
                // covers the rounding of the bound in the working precision
                const double cen = 0.5 * (ehi + elo);
                const double hw = 0.5 * (ehi - elo) * (1.0 + (std::is_same<R, float>::value ? 1e-5 : 1e-12)) + 1e-300;
                const int K = iesh_bessel_warp(hw * hs, p.cheb_tol, Jc, inv);
                for (int q = lane; q < kIeshMaxTerms; q += 32) Jr[q] = (R)(2.0 * Jc[q]);
                if (lane == 0) {
                    double sn, cs;
                    sincos(cen * hs, &sn, &cs);  // exp(-i c h) = cs - i sn
                    misc[0] = (double)K;
                    misc[1] = sn;
                    misc[2] = cs;
                    misc[8] = cen;
                    misc[9] = 1.0 / hw;
                    misc[10] = w / hw;
                    misc[11] = Jc[0];
                }
            }
        }
        __syncthreads();
        const int K = kF32 ? mi[0] : (int)misc[0];
        if (K < 0) {  // step too long for the series: leave psi unchanged, count as unconverged
            if (tid == 0 && nonconv) atomicAdd(nonconv, 1ull);
        } else {
            nterms += (unsigned long long)K;
            if constexpr (tcp) {
                {
                    // Chebyshev terms on the tensor cores: D = Phi^T A^T (M = 2 Ne orbital components
                    // padded to 128, N = N states, K = N states) with Phi split into tf32 high and low
                    // parts (two products) and A in tf32.  Thread (warp w, lane l) owns accumulator row
                    // tn = 32 (w % 4) + l, i.e. component tcmp (0 re, 1 im) of electron te, and the
                    // states s0 .. s0 + N/2 - 1 of its half (w / 4); the partner component is lane
                    // l ^ 1.  TMEM columns: [0, N) D, [N, 2N) phi_{k-2}, [2N, 3N) the series sum.
                    // phi_{k-1} is read back as the high + low tf32 pair the tensor cores multiply
                    // (2^-22 relative), so the whole of Ht phi_{k-1} has that precision.
                    const float st = mf[10];
                    const float cenf = mf[8], ihwf = mf[9];
                    const int tq = warp & 3, NH = N >> 1, s0 = (warp >> 2) * NH;
                    const int tn = 32 * tq + lane, te = tn >> 1, tcmp = tn & 1;
                    const bool twarp = 32 * tq < 2 * Ne;  // warp-uniform: the warp holds orbital rows
                    const bool trow = tn < 2 * Ne;
                    const uint32_t tl = tmem + ((uint32_t)(32 * tq) << 16);
                    const uint32_t cD = 0, cP = (uint32_t)N, cO = 2u * (uint32_t)N;
                    const float sgn = tcmp ? -1.f : 1.f;
                    // The A operand keeps each component in its partner's row (re of electron e in row
                    // 2 e + 1, im in row 2 e), so that accumulator row tn holds A times the partner
                    // component, the one H_t phi needs for component tcmp, without a shuffle.
                    const int arow = tn ^ 1;
                    // phi_{k-1} of this thread's states i0 .. i0 + 7 from the A operand (zero off the rows)
                    auto get_a = [&](int i0, float (&v)[8]) {
                        if (!trow) {
#pragma unroll
                            for (int t = 0; t < 8; ++t) v[t] = 0.f;
                            return;
                        }
                        const uint32_t o0 = tc::smem_kmajor_offset(arow, i0, N), o1 = tc::smem_kmajor_offset(arow, i0 + 4, N);
                        const float4 h0 = *(const float4*)(aop_hi + o0), h1 = *(const float4*)(aop_hi + o1);
                        const float4 l0 = *(const float4*)(aop_lo + o0), l1 = *(const float4*)(aop_lo + o1);
                        v[0] = h0.x + l0.x; v[1] = h0.y + l0.y; v[2] = h0.z + l0.z; v[3] = h0.w + l0.w;
                        v[4] = h1.x + l1.x; v[5] = h1.y + l1.y; v[6] = h1.z + l1.z; v[7] = h1.w + l1.w;
                    };
                    // A operand (rows tn, k = states i0 .. i0 + 7) from 8 values, high and low tf32 parts
                    auto put_a = [&](int i0, const float (&v)[8]) {
                        if (!trow) return;
                        float4 h0, h1, l0, l1;
                        float* hv0 = &h0.x; float* hv1 = &h1.x; float* lv0 = &l0.x; float* lv1 = &l1.x;
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            hv0[t] = tc::to_tf32(v[t]);
                            lv0[t] = tc::to_tf32(v[t] - hv0[t]);
                            hv1[t] = tc::to_tf32(v[4 + t]);
                            lv1[t] = tc::to_tf32(v[4 + t] - hv1[t]);
                        }
                        const uint32_t o0 = tc::smem_kmajor_offset(arow, i0, N), o1 = tc::smem_kmajor_offset(arow, i0 + 4, N);
                        *(float4*)(aop_hi + o0) = h0;
                        *(float4*)(aop_hi + o1) = h1;
                        *(float4*)(aop_lo + o0) = l0;
                        *(float4*)(aop_lo + o1) = l1;
                    };
                    // (lam_i - c) / hw of every state, read by the terms as float4 pairs
                    float* dlt = (float*)(smem + L.o_dl);
                    for (int i = tid; i < N; i += nthr) dlt[i] = (lam[i] - cenf) * ihwf;
                    // phi_0 = psi; series sum J_0 phi_0
                    if (twarp) {
                        const float j0 = mf[11];
#pragma unroll
                        for (int q = 0; q < 5; ++q) {
                            if (8 * q >= NH) break;
                            float v[8], o[8];
#pragma unroll
                            for (int t = 0; t < 8; ++t) {
                                const Cx<R> x = phiA[(s0 + 8 * q + t) * Nep + (trow ? te : 0)];
                                v[t] = trow ? (tcmp ? x.im : x.re) : 0.f;
                                o[t] = j0 * v[t];
                            }
                            tc::st8(tl + cO + s0 + 8 * q, o);
                            put_a(s0 + 8 * q, v);
                        }
                        tc::wait_st();
                    }
                    tc::fence_proxy_async();
                    tc::fence_before_sync();
                    __syncthreads();
                    constexpr uint32_t kPolls = 1u << 20;  // a product takes about a microsecond
                    for (int kk = 1; kk <= K; ++kk) {
                        if (tid == 0) {
                            tc::fence_after_sync();
                            const uint32_t idesc = tc::idesc_f32acc(tc::kTypeTF32, 128, N);
                            const uint32_t sbo = (uint32_t)N * 32u, ah = tc::smem_u32(aop_hi),
                                           al = tc::smem_u32(aop_lo), bb = tc::smem_u32(bop);
                            for (int ks = 0; ks < N / 8; ++ks)
                                tc::mma<tc::kTypeTF32>(tmem + cD, tc::smem_desc(ah + 256u * ks, 128, sbo),
                                                       tc::smem_desc(bb + 256u * ks, 128, sbo), idesc, ks > 0);
                            // The low tf32 part of phi_{k-1} changes the product by at most
                            // 2^-11 |phi_{k-1}| <= 2^-11 (|T_k| <= 1 on the scaled spectrum, orbitals of
                            // unit norm), and phi_k's contribution to the sum by |2 J_k| 2^-10: below an
                            // FP32 unit once |2 J_k| <= 2^-15 (with room for its growth through the
                            // recurrence, whose later terms weigh less still).  The last terms of the
                            // series take the high part only.
                            if (fabsf((float)Jr[kk]) > 0x1p-15f)
                                for (int ks = 0; ks < N / 8; ++ks)
                                    tc::mma<tc::kTypeTF32>(tmem + cD, tc::smem_desc(al + 256u * ks, 128, sbo),
                                                           tc::smem_desc(bb + 256u * ks, 128, sbo), idesc, true);
                            tc::commit(&tc_bar);
                        }
                        const bool ok = tc::mbar_wait(&tc_bar, tc_phase, kPolls);
                        tc_phase ^= 1u;
                        if (__syncthreads_or(!ok)) {  // record and stop the series; psi keeps the partial sum
                            if (tid == 0) tc_fail = 1;
                            break;
                        }
                        tc::fence_after_sync();
                        if (twarp) {
                            // series sum += 2 J_k (-i)^k phi_k: even k add +-2 J_k phi_k to the same
                            // component, odd k +-2 J_k times the partner component (one shuffle)
                            const float jk = (float)Jr[kk];
                            const int ph = kk & 3;
                            const bool odd = (kk & 1) != 0;
                            const float cjk = (ph < 2 ? jk : -jk) * (odd ? sgn : 1.f);
                            const float sst = sgn * st;
#pragma unroll
                            for (int q = 0; q < 5; ++q) {
                                if (8 * q >= NH) break;
                                const int i0 = s0 + 8 * q;
                                float d[8], p2[8], o[8], nw[8], p1[8];
                                get_a(i0, p1);
                                tc::ld8(tl + cD + i0, d);
                                if (kk > 1) tc::ld8(tl + cP + i0, p2);
                                tc::ld8(tl + cO + i0, o);
                                const float4 dl0 = *(const float4*)(dlt + i0), dl1 = *(const float4*)(dlt + i0 + 4);
                                const float dl[8] = {dl0.x, dl0.y, dl0.z, dl0.w, dl1.x, dl1.y, dl1.z, dl1.w};
                                tc::wait_ld();
#pragma unroll
                                for (int t = 0; t < 8; ++t) {
                                    // Ht phi = dl phi - i s (A phi); d is A times the partner component
                                    const float hv = fmaf(dl[t], p1[t], sst * d[t]);
                                    nw[t] = kk == 1 ? hv : fmaf(2.f, hv, -p2[t]);
                                    p2[t] = p1[t];
                                }
                                if (odd) {
#pragma unroll
                                    for (int t = 0; t < 8; ++t)
                                        o[t] = fmaf(cjk, __shfl_xor_sync(0xffffffffu, nw[t], 1), o[t]);
                                } else {
#pragma unroll
                                    for (int t = 0; t < 8; ++t) o[t] = fmaf(cjk, nw[t], o[t]);
                                }
                                tc::st8(tl + cP + i0, p2);
                                tc::st8(tl + cO + i0, o);
                                put_a(i0, nw);
                            }
                            tc::wait_st();
                        }
                        tc::fence_proxy_async();
                        tc::fence_before_sync();
                        __syncthreads();
                    }
                    tc::fence_after_sync();
                    // psi = exp(-i c h) sum
                    const float snf = mf[1], csf = mf[2];
                    if (twarp) {
                        // the series-sum columns in two batches of loads, each with one wait: a
                        // wait for TMEM loads takes long while the tensor cores run the other
                        // CTA's products
#pragma unroll
                        for (int b = 0; b < 2; ++b) {
                            float o[3][8];
#pragma unroll
                            for (int g = 0; g < 3; ++g) {
                                const int q = 3 * b + g;
                                if (q < 5 && 8 * q < NH) tc::ld8(tl + cO + s0 + 8 * q, o[g]);
                            }
                            tc::wait_ld();
#pragma unroll
                            for (int g = 0; g < 3; ++g) {
                                const int q = 3 * b + g;
                                if (q >= 5 || 8 * q >= NH) break;
                                const int i0 = s0 + 8 * q;
                                // states t, t + 1 of electron te: the re lane writes state t and the im
                                // lane state t + 1, each as one 8-byte element (one shuffle per pair;
                                // single-component 4-byte stores from lane pairs were far slower)
#pragma unroll
                                for (int t = 0; t < 8; t += 2) {
                                    const float y = __shfl_xor_sync(0xffffffffu, tcmp ? o[g][t] : o[g][t + 1], 1);
                                    const float re = tcmp ? y : o[g][t], im = tcmp ? o[g][t + 1] : y;
                                    if (trow)
                                        phiA[(i0 + t + tcmp) * Nep + te] = {re * csf + im * snf, im * csf - re * snf};
                                }
                            }
                        }
                    }
                    tc::fence_before_sync();
                    __syncthreads();
                }
            } else {
                const R s = kF32 ? (R)mf[10] : (R)misc[10];
                const R cenr = kF32 ? (R)mf[8] : (R)misc[8], ihwr = kF32 ? (R)mf[9] : (R)misc[9];
                R dl[4];
    #pragma unroll
                for (int rr = 0; rr < 4; ++rr) dl[rr] = (lam[i0 + RG * rr] - cenr) * ihwr;
                if (tile_on) {
                    const R j0 = kF32 ? (R)mf[11] : (R)misc[11];
    #pragma unroll
                    for (int rr = 0; rr < 4; ++rr)
    #pragma unroll
                        for (int cc = 0; cc < 4; ++cc) {
                            const int ix = (i0 + RG * rr) * Nep + c0 + CG * cc;
                            const Cx<R> x = phiA[ix];
                            outb[ix] = {j0 * x.re, j0 * x.im};
                        }
                }
                for (int kk = 1; kk <= K; ++kk) {
                    // phi_k = 2 Ht phi_{k-1} - phi_{k-2}: dst holds phi_{k-2} on entry and
                    // each thread reads back only its own tile before overwriting it
                    const Cx<R>* src = (kk & 1) ? phiA : phiB;
                    Cx<R>* dst = (kk & 1) ? phiB : phiA;
                    __syncthreads();
                    if (tile_on) {
                        R ar[4][4], ai[4][4];
    #pragma unroll
                        for (int rr = 0; rr < 4; ++rr)
    #pragma unroll
                            for (int cc = 0; cc < 4; ++cc) ar[rr][cc] = ai[rr][cc] = R(0);
                        for (int j = 0; j < N; ++j) {
                            const R* aj = At + j * Np + i0;
                            const Cx<R>* pj = src + j * Nep + c0;
                            R av[4];
                            Cx<R> pv[4];
    #pragma unroll
                            for (int rr = 0; rr < 4; ++rr) av[rr] = aj[RG * rr];
    #pragma unroll
                            for (int cc = 0; cc < 4; ++cc) pv[cc] = pj[CG * cc];
    #pragma unroll
                            for (int rr = 0; rr < 4; ++rr)
    #pragma unroll
                                for (int cc = 0; cc < 4; ++cc) {
                                    ar[rr][cc] += av[rr] * pv[cc].re;
                                    ai[rr][cc] += av[rr] * pv[cc].im;
                                }
                        }
                        const R jk = Jr[kk];
                        const int ph = kk & 3;
    #pragma unroll
                        for (int rr = 0; rr < 4; ++rr)
    #pragma unroll
                            for (int cc = 0; cc < 4; ++cc) {
                                const int ix = (i0 + RG * rr) * Nep + c0 + CG * cc;
                                const Cx<R> cur = src[ix];
                                // Ht phi = dl phi - i s (A phi)
                                const R hre = dl[rr] * cur.re + s * ai[rr][cc];
                                const R him = dl[rr] * cur.im - s * ar[rr][cc];
                                Cx<R> nw;
                                if (kk == 1) {
                                    nw = {hre, him};
                                } else {
                                    const Cx<R> pr = dst[ix];
                                    nw = {R(2) * hre - pr.re, R(2) * him - pr.im};
                                }
                                dst[ix] = nw;
                                Cx<R> o = outb[ix];
                                if (ph == 0) {
                                    o.re += jk * nw.re;
                                    o.im += jk * nw.im;
                                } else if (ph == 1) {  // (-i) nw
                                    o.re += jk * nw.im;
                                    o.im -= jk * nw.re;
                                } else if (ph == 2) {
                                    o.re -= jk * nw.re;
                                    o.im -= jk * nw.im;
                                } else {  // (+i) nw
                                    o.re -= jk * nw.im;
                                    o.im += jk * nw.re;
                                }
                                outb[ix] = o;
                            }
                    }
                }
                __syncthreads();
                const R snr = kF32 ? (R)mf[1] : (R)misc[1], csr = kF32 ? (R)mf[2] : (R)misc[2];
                if (tile_on) {
    #pragma unroll
                    for (int rr = 0; rr < 4; ++rr)
    #pragma unroll
                        for (int cc = 0; cc < 4; ++cc) {
                            const int ix = (i0 + RG * rr) * Nep + c0 + CG * cc;
                            const Cx<R> o = outb[ix];
                            phiA[ix] = {o.re * csr + o.im * snr, o.im * csr - o.re * snr};
                        }
                }
                __syncthreads();
            }
        }

        if (!ena) {  // EhrenfestNA: no hopping
        // ---- hop test (iesh.jl:231-335, 390-411) ----
        // FP32 path: where the bound on the estimate from the occupied Gram matrix already lies
        // below the random number, the estimate does too and the LU is not needed (the decision
        // and every result are those of the LU path); sabs_pre is then the step's sum |A_mn|
        bool lu = true;
        float sabs_pre = 0.f;
        if constexpr (kF32) {
            if (!p.exact_probability && !p.lu_always) {
                float trx = 0.f, fx2 = 0.f;
                gram_partials(trx, fx2);
                for (int q = tid; q < 4 * Nu; q += nthr) {  // unoccupied state q / 4, a quarter of the electrons
                    const int m = unocc[q >> 2];
                    // (the approximate quotient: 2 ulp, inside the bound's 2 % margin)
                    for (int n = q & 3; n < Ne; n += 4) {
                        const int j = occ[n];
                        sabs_pre += tcp ? fabsf(__fdividef(z0[m] * z0[j], gap(m, j))) : fabsf(coup(m, j));
                    }
                }
                iesh_block_sum3_f(trx, fx2, sabs_pre, red);
                lu = !estimate_certainly_below(trx, fx2, sabs_pre, RP ? mf[12] : mf[6],
                                               rng_uniform_f(p.seed, gid, (uint32_t)step, RNG_HOP));
            }
        }
        if (lu) {
        ++nlu;
        // S^T stored by columns: column c of S^T is row occ[c] of psi, Qc[c * Nep + r] = S^T[r][c]
        Cx<R>* Qc = phiB;
        Cx<R>* Rh = phiB + Nep * Nep;  // right-hand sides psi[unocc, :]^T, [Nep][Nu]
        for (int q = tid; q < Ne * Ne; q += nthr) {
            const int c = q / Ne, r = q - c * Ne;
            Qc[c * Nep + r] = phiA[occ[c] * Nep + r];
        }
        __syncthreads();
        double det_r = 0.0, det_i = 0.0;
        int det_e = 0;
        // LU with partial pivoting of S^T, column c owned by warp c % nwarp.  The
        // owner of a column picks its pivot, swaps and scales it right after its
        // own updates; after one barrier each warp applies the row swap to all
        // its columns (the factored L columns too, as getrf) and the rank-1
        // update to its columns right of the pivot.  piv[col] = -1 marks a zero
        // pivot (each entry is written once, so a late warp reads its own).
        bool singular = false;
        const int nwarp = nthr >> 5;
        for (int col = 0; col < Ne; ++col) {
            if (warp == col % nwarp) {
                Cx<R>* qc = Qc + col * Nep;
                // pivot: largest |re| + |im| (first on ties) via a max-reduction of
                // the magnitude's bit pattern (non-negative floats order as integers)
                unsigned key = 0u;
                int bi = Ne;
                for (int rr = col + lane; rr < Ne; rr += 32) {
                    const Cx<R> x = qc[rr];
                    const unsigned kk = __float_as_uint((float)(fabs(x.re) + fabs(x.im)));
                    if (kk > key || bi == Ne) {
                        key = kk;
                        bi = rr;
                    }
                }
                const unsigned kmax = __reduce_max_sync(0xffffffffu, key);
                const int cand = (key == kmax && bi < Ne) ? bi : Ne;
                bi = __reduce_min_sync(0xffffffffu, (unsigned)cand);
                const bool ok = kmax > 0u;
                if (ok) {
                    if (lane == 0 && bi != col) {
                        const Cx<R> t = qc[col];
                        qc[col] = qc[bi];
                        qc[bi] = t;
                    }
                    __syncwarp();
                    const Cx<R> pv = qc[col];
                    const R inv = R(1) / (pv.re * pv.re + pv.im * pv.im);  // x / pv = x conj(pv) / |pv|^2
                    for (int rr = col + 1 + lane; rr < Ne; rr += 32) {
                        const Cx<R> x = qc[rr];
                        qc[rr] = {(x.re * pv.re + x.im * pv.im) * inv, (x.im * pv.re - x.re * pv.im) * inv};
                    }
                }
                if (lane == 0) piv[col] = ok ? bi : -1;
            }
            __syncthreads();
            const int pr = piv[col];
            if (pr < 0) {
                singular = true;
                break;
            }
            // this warp's columns: w, w + nwarp, ...; swap rows col and pr in all of them
            if (pr != col)
                for (int cc = warp + nwarp * lane; cc < Ne; cc += 32 * nwarp) {
                    if (cc == col) continue;
                    Cx<R>* qcc = Qc + cc * Nep;
                    const Cx<R> t = qcc[col];
                    qcc[col] = qcc[pr];
                    qcc[pr] = t;
                }
            __syncwarp();
            const Cx<R>* lcol = Qc + col * Nep;
            const int r0 = col + 1 + lane, r1 = r0 + 32;
            const Cx<R> l0 = r0 < Ne ? lcol[r0] : Cx<R>{R(0), R(0)};
            const Cx<R> l1 = r1 < Ne ? lcol[r1] : Cx<R>{R(0), R(0)};
            const int cc0 = col + 1 + ((warp - (col + 1)) % nwarp + nwarp) % nwarp;
#pragma unroll 2
            for (int cc = cc0; cc < Ne; cc += nwarp) {
                Cx<R>* qcc = Qc + cc * Nep;
                const Cx<R> u = qcc[col];
                if (r0 < Ne) {
                    Cx<R> t = qcc[r0];
                    t.re -= l0.re * u.re - l0.im * u.im;
                    t.im -= l0.re * u.im + l0.im * u.re;
                    qcc[r0] = t;
                }
                if (r1 < Ne) {
                    Cx<R> t = qcc[r1];
                    t.re -= l1.re * u.re - l1.im * u.im;
                    t.im -= l1.re * u.im + l1.im * u.re;
                    qcc[r1] = t;
                }
            }
            for (int rr = col + 65 + lane; rr < Ne; rr += 32)  // systems beyond 64 + 1 electrons
                for (int cc = cc0; cc < Ne; cc += nwarp) {
                    Cx<R>* qcc = Qc + cc * Nep;
                    const Cx<R> l = lcol[rr], u = qcc[col];
                    Cx<R> t = qcc[rr];
                    t.re -= l.re * u.re - l.im * u.im;
                    t.im -= l.re * u.im + l.im * u.re;
                    qcc[rr] = t;
                }
        }
        __syncthreads();
        R sabs = R(0);
        if (warp == 0) {
            if (!singular) {  // det S on lane 0, as a scaled product in the working precision
                R dr = R(1), di = R(0);
                int de = 0, swaps = 0;
                for (int q = lane; q < Ne; q += 32) {
                    const Cx<R> d = Qc[q * Nep + q];
                    scaled_mul<R>(dr, di, de, d.re, d.im, 0);
                    if (piv[q] != q) ++swaps;
                }
                for (int off = 16; off > 0; off >>= 1) {
                    const R orr = __shfl_xor_sync(0xffffffffu, dr, off);
                    const R oii = __shfl_xor_sync(0xffffffffu, di, off);
                    const int oe = __shfl_xor_sync(0xffffffffu, de, off);
                    scaled_mul<R>(dr, di, de, orr, oii, oe);
                    swaps += __shfl_xor_sync(0xffffffffu, swaps, off);
                }
                if (swaps & 1) {
                    dr = -dr;
                    di = -di;
                }
                det_r = (double)dr;
                det_i = (double)di;
                det_e = de;
            }
        } else if (!(kF32 && !p.exact_probability && !p.lu_always)) {  // else the sum is sabs_pre
            // sum |v.d| over unoccupied rows and electrons (the estimate's sum(abs, v_dot_d))
            for (int q = tid - 32; q < Nu * Ne; q += nthr - 32) {
                const int mm = q / Ne, n = q - mm * Ne;
                sabs += fabs(coup(unocc[mm], occ[n]));
            }
        }
        double sumabs;
        if constexpr (std::is_same<R, float>::value)
            sumabs = fabs(wh) * (double)(!p.exact_probability && !p.lu_always ? sabs_pre
                                                                              : iesh_block_sum_f(sabs, red));
        else
            sumabs = fabs(wh) * iesh_block_sum((double)sabs, red);
        const double u = std::is_same<R, double>::value
                             ? rng_uniform(p.seed, gid, (uint32_t)step, RNG_HOP)
                             : (double)rng_uniform_f(p.seed, gid, (uint32_t)step, RNG_HOP);
        if (tid == 0) {
            int full = 0;
            if (!singular) {
                // estimate = 2 dt / |det|^2 * sum|v.d| * (|Re det| + |Im det|)
                const double est =
                    2.0 * dt * sumabs * ldexp((fabs(det_r) + fabs(det_i)) / (det_r * det_r + det_i * det_i), -det_e);
                full = (p.exact_probability || !(est < u)) ? 1 : 0;
            }
            misc[2] = full;
        }
        __syncthreads();
        if (misc[2] != 0.0) {
            ++nfull;
            for (int q = tid; q < Ne * Nu; q += nthr) {
                const int c = q / Nu, mm = q - c * Nu;
                Rh[c * Nu + mm] = phiA[unocc[mm] * Nep + c];
            }
            __syncthreads();
            if (tid < Nu) {  // one right-hand side per thread: P, L, U solves
                const int mm = tid;
                for (int q = 0; q < Ne; ++q) {
                    const int pq = piv[q];
                    if (pq != q) {
                        const Cx<R> t = Rh[q * Nu + mm];
                        Rh[q * Nu + mm] = Rh[pq * Nu + mm];
                        Rh[pq * Nu + mm] = t;
                    }
                }
                for (int rr = 1; rr < Ne; ++rr) {
                    Cx<R> y = Rh[rr * Nu + mm];
                    for (int q = 0; q < rr; ++q) {
                        const Cx<R> l = Qc[q * Nep + rr], x = Rh[q * Nu + mm];
                        y.re -= l.re * x.re - l.im * x.im;
                        y.im -= l.re * x.im + l.im * x.re;
                    }
                    Rh[rr * Nu + mm] = y;
                }
                for (int rr = Ne - 1; rr >= 0; --rr) {
                    Cx<R> y = Rh[rr * Nu + mm];
                    for (int q = rr + 1; q < Ne; ++q) {
                        const Cx<R> a = Qc[q * Nep + rr], x = Rh[q * Nu + mm];
                        y.re -= a.re * x.re - a.im * x.im;
                        y.im -= a.re * x.im + a.im * x.re;
                    }
                    Rh[rr * Nu + mm] = cx_div<R>(y, Qc[rr * Nep + rr]);
                }
                // p_mn = 2 dt Re(Y_nm) (v.d)_mn, (v.d)_mn = -w A[m][state n]
                const int m = unocc[mm];
                for (int n = 0; n < Ne; ++n) {
                    const double vdd = -wh * (double)coup(m, occ[n]);
                    const double pr = clamp01<double>(2.0 * dt * (double)Rh[n * Nu + mm].re * vdd);
                    Rh[n * Nu + mm].re = (R)pr;
                }
            }
            __syncthreads();
            if (tid == 0) {
                double shift = 0.0;  // ring polymer: velocity change of every bead's z component
                int sel_n = -1, sel_m = -1;
                double cum = 0.0;
                for (int n = 0; n < Ne && sel_n < 0; ++n)
                    for (int mm = 0; mm < Nu; ++mm) {
                        cum += (double)Rh[n * Nu + mm].re;
                        if (u < cum) {
                            sel_n = n;
                            sel_m = unocc[mm];
                            break;
                        }
                    }
                if (sel_n >= 0) {
                    const int old = occ[sel_n], nw = sel_m;
                    bool accept = true;
                    if (p.rescaling != RESCALE_OFF) {
                        // d[new, old] = dh A[new][old]; only its z component is nonzero
                        const double dz = dhz * (double)z0[nw] * (double)z0[old] / (double)gap(nw, old);
                        const double aa = (dz * dz / mass) / 2.0;
                        const double vz = RP ? misc[13] : v[2];  // hopping velocity: the centroid's
                        const double bb = dz * vz;
                        const double cc = (double)lam[nw] - (double)lam[old];
                        const double disc = bb * bb - 4.0 * aa * cc;
                        if (disc < 0.0) {
                            accept = false;
                            // invert the (centroid) velocity along d = dz e_z
                            if (p.rescaling == RESCALE_VINVERSION) {
                                if constexpr (RP) shift = -2.0 * vz;
                                else v[2] = -v[2];
                            }
                        } else {
                            const double root = sqrt(disc);
                            const double gam = bb < 0.0 ? (bb + root) / (2.0 * aa) : (bb - root) / (2.0 * aa);
                            if constexpr (RP) shift = -(gam * dz / mass);
                            else v[2] = v[2] - gam * dz / mass;
                        }
                    }
                    if (accept) {
                        if (p.hop_log && nh < p.max_hops) {
                            p.hop_log[((int64_t)nh * 3 + 0) * NT + ti] = step;
                            p.hop_log[((int64_t)nh * 3 + 1) * NT + ti] = old;
                            p.hop_log[((int64_t)nh * 3 + 2) * NT + ti] = nw;
                        }
                        ++nh;
                        occ[sel_n] = nw;
                        if constexpr (RP) misc[15] = 1.0;  // the bead eigenvalue sums are stale
                        rebuild_unocc();
                    } else {
                        ++nf;
                    }
                }
                misc[3] = RP ? shift : v[2];
            }
            __syncthreads();
            if (warp == 0) {  // hop counts live in thread 0, which writes them out
                if constexpr (RP) v[2] = v[2] + misc[3];
                else v[2] = misc[3];
            }
        }
        }  // lu
        }  // !ena
        if (p.edc_C > 0.0) {
            // DecoherenceCorrectionEDC (decoherence_corrections.jl:21-39, callback
            // iesh.jl:424-441), after the hop: in the column of electron e with
            // occupied state s, psi_j *= exp(-dt / tau_j), tau_j = (1 + C / Ekin) /
            // |E_j - E_s| for j != s, then psi_s rescaled to restore the norm
            if (tid == 0) misc[7] = kinetic();
            __syncthreads();
            const double ekin = misc[7];
            for (int e = tid; e < Ne; e += nthr) {
                const int s = occ[e];
                R unocc_norm = R(0);
                for (int j = 0; j < N; ++j) {
                    if (j == s) continue;
                    const R tau = (R)((1.0 + p.edc_C / ekin) / fabs((double)lam[j] - (double)lam[s]));
                    R f;
                    if constexpr (std::is_same<R, float>::value)
                        f = __expf(-(R)dt / tau);
                    else
                        f = nqcd_exp(-dt / tau);
                    Cx<R> c = phiA[j * Nep + e];
                    c.re *= f;
                    c.im *= f;
                    phiA[j * Nep + e] = c;
                    unocc_norm += c.re * c.re + c.im * c.im;
                }
                const Cx<R> cm = phiA[s * Nep + e];
                const R g = sqrt((R(1) - unocc_norm) / (cm.re * cm.re + cm.im * cm.im));
                phiA[s * Nep + e] = {cm.re * g, cm.im * g};
            }
            __syncthreads();
        }
        // save points are the multiples of save_stride: a product, not an integer division per step
        if (p.save_stride > 0 && step == isave * p.save_stride) {
            if (p.obs_partial) save(isave++);
        }
    }

    double e1 = 0.0;
    if (ena && p.energy) orbital_sums();
    if constexpr (RP) {
        const bool stale = misc[15] != 0.0;  // a hop in the last step; read by all before it is cleared
        __syncthreads();
        if (p.energy && stale) bead_roots();
    }
    if (warp == 0 && p.energy) {
        if constexpr (RP) {
            e1 = rp_energy();  // bead sums of the last step's roots
        } else {
            const double pe = potential();
            e1 = kinetic() + pe;
        }
    }
    // final orbitals: (nstates, nelectrons) column-major per trajectory
    if (p.psi_re)
        for (int q = tid; q < N * Ne; q += nthr) {
            const int c = q / N, i = q - c * N;
            const Cx<R> x = phiA[i * Nep + c];
            p.psi_re[(ti * Ne + c) * N + i] = (double)x.re;
            p.psi_im[(ti * Ne + c) * N + i] = (double)x.im;
        }
    for (int jj = tid; jj < Ne; jj += nthr) p.occ[(int64_t)jj * NT + ti] = occ[jj];
    if (warp == 0 && lane < NB)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            p.r[(int64_t)(d + 3 * lane) * NT + ti] = r[d];
            p.v[(int64_t)(d + 3 * lane) * NT + ti] = v[d];
        }
    if (tid == 0) {
        if (p.nhops) p.nhops[ti] = nh;
        if (p.nfrustrated) p.nfrustrated[ti] = nf;
        if (p.nsteps_out) p.nsteps_out[ti] = p.nsteps;
        if (p.fp64_steps) p.fp64_steps[ti] = nfp64;
        if (p.energy) {
            p.energy[ti] = e0;
            p.energy[NT + ti] = e1;
        }
        if (p.counters) {
            atomicAdd(p.counters + 0, (unsigned long long)nfull);
            atomicAdd(p.counters + 1, nterms);
            atomicAdd(p.counters + 5, (unsigned long long)nlu);
        }
    }
    if constexpr (tcp) {
        {
            if (tid == 0 && tc_fail && p.counters) atomicAdd(p.counters + 3, 1ull);
            tc::fence_before_sync();
            __syncthreads();
            if (warp == 0) tc::tmem_dealloc(tmem, tc_cols);
        }
    }
}

template <typename R, bool TC>
__global__ void __launch_bounds__(kIeshBlock, iesh_min_blocks<R>()) iesh_kernel(const IeshParams p) {
    iesh_body<R, false, TC>(p);
}

// RingPolymerSimulation{AdiabaticIESH}: p.nbeads in 2..kRpIeshMaxBeads, p.nelec <= kRpIeshMaxElectrons
template <typename R, bool TC>
__global__ void __launch_bounds__(kIeshBlock, iesh_min_blocks<R>()) rpiesh_kernel(const IeshParams p) {
    iesh_body<R, true, TC>(p);
}

template <typename R, bool TC>
cudaError_t launch_iesh_tc(const IeshParams& p, cudaStream_t s) {
    const bool rp = p.nbeads > 1;
    const IeshLayout L = iesh_layout<R>(p.nstates, p.nelec, rp ? p.nbeads : 1, TC);
    cudaError_t e = cudaFuncSetAttribute(rp ? rpiesh_kernel<R, TC> : iesh_kernel<R, TC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.bytes);
    if (e != cudaSuccess) return e;
    if (rp)
        rpiesh_kernel<R, TC><<<(unsigned)p.ntraj, kIeshBlock, L.bytes, s>>>(p);
    else
        iesh_kernel<R, TC><<<(unsigned)p.ntraj, kIeshBlock, L.bytes, s>>>(p);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_iesh(const IeshParams& p, cudaStream_t s) {
    if (p.ntraj <= 0) return cudaSuccess;
    const bool rp = p.nbeads > 1;
    if (rp && (p.nbeads > kRpIeshMaxBeads || p.nelec > kRpIeshMaxElectrons)) return cudaErrorInvalidValue;
    if constexpr (std::is_same<R, float>::value) {
        if (p.tensor) {
            if (!iesh_tc_shape(p.nstates, p.nelec)) return cudaErrorInvalidValue;
            return launch_iesh_tc<float, true>(p, s);
        }
    }
    return launch_iesh_tc<R, false>(p, s);
}

}  // namespace nqcd
