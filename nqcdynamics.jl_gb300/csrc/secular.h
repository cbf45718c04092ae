// Roots of the secular equation of an arrowhead Hamiltonian
//     H = [[h, V_k], [V_k, diag(e_k)]],   f(l) = l - h - sum_k V_k^2 / (l - e_k),
// the one-electron Hamiltonian of the Newns-Anderson (AndersonHolstein) model
// that the reference diagonalises with LAPACK (NQCModels AndersonHolstein,
// docs/src/dynamicssimulations/dynamicsmethods/iesh.md:73).  There is one root
// below e_0, one in each interval (e_{k-1}, e_k) and one above e_{M-1}; the
// impurity weight of eigenvector i is z0_i^2 = 1 / f'(l_i), and the other
// components are V_k z0_i / (l_i - e_k).  With V_k > 0 all these columns have
// a positive component on their own basis state, so the reference's sign
// convention (continuity with the previous eigenvectors, identity first)
// selects z0_i > 0 at every step.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

namespace nqcd {

// Reciprocal of a secular-sum denominator.  FP32 (fast paths): the hardware
// approximate reciprocal (about 1 ulp); its error is of the order of the
// rounding already allowed for by the stopping test below.
template <typename R>
__device__ __forceinline__ R secular_rcp(R d) {
    if constexpr (std::is_same<R, float>::value)
        return __fdividef(1.0f, d);
    else
        return 1.0 / d;
}

// Solve root i of the secular equation.  o = origin pole, d = offset from it,
// (dlo, dhi) = bracket of d.  Returns l = o + d and z0^2 = 1/f'.
template <typename R>
__device__ __forceinline__ void secular_root(const R* __restrict__ eps, const R* __restrict__ V2, int M, int i, R h,
                                             R Lbound, R& lam_io, R& z2_out, unsigned long long* nonconv) {
    // interval of root i
    const bool first = i == 0, last = i == M;
    R a = first ? eps[0] : eps[i - 1];
    R b = last ? eps[M - 1] : eps[i];
    int jo;  // origin pole index
    R o, dlo, dhi;
    if (first) {
        jo = 0;
        o = a;
        dlo = -Lbound;
        dhi = R(0);
    } else if (last) {
        jo = M - 1;
        o = b;
        dlo = R(0);
        dhi = Lbound;
    } else if (std::is_same<R, float>::value && lam_io > a && lam_io < b) {
        // fast path with a warm start inside the interval: measure from the
        // pole nearer to it over the whole interval (the root moves little
        // between evaluations), which saves the midpoint evaluation
        if (lam_io - a < b - lam_io) {
            jo = i - 1;
            o = a;
            dlo = R(0);
            dhi = b - a;
        } else {
            jo = i;
            o = b;
            dlo = a - b;
            dhi = R(0);
        }
    } else {
        // which half: sign of f at the midpoint decides the nearer pole
        R mid = a + R(0.5) * (b - a);
        R s = R(0);
#pragma unroll 4
        for (int k = 0; k < M; ++k) s += V2[k] * secular_rcp<R>(mid - eps[k]);
        R fm = mid - h - s;
        if (fm > R(0)) {  // root in (a, mid): measure from a
            jo = i - 1;
            o = a;
            dlo = R(0);
            dhi = mid - a;
        } else {
            jo = i;
            o = b;
            dlo = mid - b;
            dhi = R(0);
        }
    }
    // warm start from the previous root if it lies in the bracket
    R d = lam_io - o;
    if (!(d > dlo && d < dhi)) d = R(0.5) * (dlo + dhi);
    // the pole at the other end of the interval (the origin itself for the outer roots)
    const R other = o == a ? b : a;
    R fp = R(1);
    bool conv = false;
    for (int it = 0; it < 80; ++it) {
        R s1 = R(0), s2 = R(0), s3 = R(0), sa = R(0);
#pragma unroll 4
        for (int k = 0; k < M; ++k) {
            R den = (k == jo) ? d : (o - eps[k]) + d;
            R t = secular_rcp<R>(den);
            R vt = V2[k] * t;
            s1 += vt;
            const R vt2 = vt * t;
            s2 += vt2;
            s3 += vt2 * t;
            sa += fabs(vt);
        }
        R f = (o + d) - h - s1;
        fp = R(1) + s2;
        if (f == R(0)) {  // exact root: keep d (a bisection here would leave it)
            conv = true;
            break;
        }
        if (f > R(0))
            dhi = d;
        else
            dlo = d;
        R dn = d - f / fp;
        // the Newton point may equal the bracket end just set (a step below
        // one ulp): that is convergence, not a reason to bisect
        if (!(dn >= dlo && dn <= dhi)) dn = R(0.5) * (dlo + dhi);
        R step = dn - d;
        d = dn;
        const R ulp = std::is_same<R, float>::value ? R(1.2e-7) : R(2.3e-16);
        R tol = R(2) * ulp * (fabs(d) + fabs(o) * R(1e-3));
        // f has reached the rounding error of its own evaluation: no further
        // Newton step can be trusted (the secular-equation stopping test).
        // The summed error of the M terms can exceed ulp * sum|terms| by about
        // sqrt(M); after the first iterations accept the bound used by LAPACK's
        // secular solver, 8 ulp * sum|terms|.
        R ferr = ulp * (fabs(o + d) + fabs(h) + sa);
        if (it >= 16) ferr *= R(8);
        if (fabs(step) <= tol || dhi - dlo <= tol || fabs(f) <= ferr) {
            conv = true;
            break;
        }
        // The Newton step just taken leaves an error of about |f''/(2 f')| step^2, f'' = -2 s3 at
        // the previous point.  While the step is at most a tenth of the distance to the nearest
        // pole, f'' changes along it by less than a factor (1/0.9)^3 < 1.4, so below the tolerance
        // that bound ends the iteration one evaluation early (a warm start is usually that close).
        // f' is then carried to the new point to first order, f' + f'' step (the impurity weight
        // 1/f' is returned; the remainder is of the order of the tolerance).
        const R pole = fmin(fabs(d), fabs((o + d) - other));
        if (fabs(step) <= R(0.1) * pole && R(1.4) * fabs(s3) * step * step <= tol * fp) {
            fp -= R(2) * s3 * step;
            conv = true;
            break;
        }
    }
    if (!conv && nonconv) atomicAdd(nonconv, 1ull);
    lam_io = o + d;
    z2_out = R(1) / fp;
}

}  // namespace nqcd
