// Host build of the engine's secular-equation solver (csrc/secular.h), for the CPU tests: the
// same source as the kernels' (host arithmetic: the IEEE quotient where the device takes the
// approximate reciprocal), called through plain C entry points.  Test infrastructure only.
#include <stdint.h>

#include "../../nqcdynamics.jl_gb300/csrc/secular.h"

namespace {

// All roots i = 0..M of the arrowhead Hamiltonian [[h, V], [V, diag(eps)]] (eps ascending, V2 = V^2)
// from the warm starts lam (updated), with secular_root (resumable = 0) or the resumable form a
// lane of the MDEF kernel runs (resumable = 1).  z2 = z0^2; evals = evaluations of f per root.
template <typename R>
int64_t roots(const R* eps, const R* V2, int M, R h, R Lbound, R* lam, R* z2, int32_t* evals, int resumable) {
    unsigned long long nonconv = 0;
    for (int i = 0; i <= M; ++i) {
        if (!resumable) {
            R l = lam[i], z = R(0);
            nqcd::secular_root<R>(eps, V2, M, i, h, Lbound, l, z, &nonconv);
            lam[i] = l;
            z2[i] = z;
            evals[i] = -1;
        } else {
            nqcd::SecularSolve<R> s;
            nqcd::secular_begin<R>(eps, M, i, Lbound, lam[i], s);
            int n = 1;
            while (!nqcd::secular_eval<R>(eps, V2, M, h, lam[i], s, &nonconv)) ++n;
            lam[i] = s.o + s.d;
            z2[i] = R(1) / s.fp;
            evals[i] = n;
        }
    }
    return (int64_t)nonconv;
}

}  // namespace

extern "C" int64_t secular_roots_f32(const float* eps, const float* V2, int32_t M, float h, float Lbound, float* lam,
                                     float* z2, int32_t* evals, int32_t resumable) {
    return roots<float>(eps, V2, M, h, Lbound, lam, z2, evals, resumable);
}

extern "C" int64_t secular_roots_f64(const double* eps, const double* V2, int32_t M, double h, double Lbound,
                                     double* lam, double* z2, int32_t* evals, int32_t resumable) {
    return roots<double>(eps, V2, M, h, Lbound, lam, z2, evals, resumable);
}
