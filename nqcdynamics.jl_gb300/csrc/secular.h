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

// Host and device: the kernels call these; a host build (the CPU test harness of the solver)
// takes the IEEE quotient and a plain counter where the device has the approximate reciprocal
// and an atomic.
#define NQCD_SECULAR_HD __host__ __device__ __forceinline__

// Reciprocal of a secular-sum denominator.  FP32 (fast paths): the hardware
// approximate reciprocal (about 1 ulp); its error is of the order of the
// rounding already allowed for by the stopping test below.
template <typename R>
NQCD_SECULAR_HD R secular_rcp(R d) {
#ifdef __CUDA_ARCH__
    if constexpr (std::is_same<R, float>::value)
        return __fdividef(1.0f, d);
    else
        return 1.0 / d;
#else
    return R(1) / d;
#endif
}

// One Newton step of root i's solve: f and f' at o + d (the sums over the poles), the bracket
// (dlo, dhi) updated, d moved.  Returns true when the root is done (converged, or 80 steps: then
// counted in nonconv); fp is then f' at the returned point.  other = the pole at the far end of
// the interval (the origin itself for the outer roots), it = steps taken so far.
template <typename R>
NQCD_SECULAR_HD bool secular_newton(const R* __restrict__ eps, const R* __restrict__ V2, int M, R h, int jo,
                                               R o, R other, R& d, R& dlo, R& dhi, R& fp, int& it,
                                               unsigned long long* nonconv) {
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
    if (f == R(0)) return true;  // exact root: keep d (a bisection here would leave it)
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
    if (fabs(step) <= tol || dhi - dlo <= tol || fabs(f) <= ferr) return true;
    // The Newton step just taken leaves an error of about |f''/(2 f')| step^2, f'' = -2 s3 at
    // the previous point.  While the step is at most a tenth of the distance to the nearest
    // pole, f'' changes along it by less than a factor (1/0.9)^3 < 1.4, so below the tolerance
    // that bound ends the iteration one evaluation early (a warm start is usually that close).
    // f' is then carried to the new point to first order, f' + f'' step (the impurity weight
    // 1/f' is returned; the remainder is of the order of the tolerance).
    const R pole = fmin(fabs(d), fabs((o + d) - other));
    if (fabs(step) <= R(0.1) * pole && R(1.4) * fabs(s3) * step * step <= tol * fp) {
        fp -= R(2) * s3 * step;
        return true;
    }
    if (++it >= 80) {
        if (nonconv) {
#ifdef __CUDA_ARCH__
            atomicAdd(nonconv, 1ull);
#else
            ++*nonconv;
#endif
        }
        return true;
    }
    return false;
}

// Solve root i of the secular equation.  o = origin pole, d = offset from it,
// (dlo, dhi) = bracket of d.  Returns l = o + d and z0^2 = 1/f'.
template <typename R>
NQCD_SECULAR_HD void secular_root(const R* __restrict__ eps, const R* __restrict__ V2, int M, int i, R h,
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
    int it = 0;
    while (!secular_newton(eps, V2, M, h, jo, o, other, d, dlo, dhi, fp, it, nonconv)) {
    }
    lam_io = o + d;
    z2_out = R(1) / fp;
}

// The same solve as resumable state, one evaluation of f at a time, so that a lane can start its
// next root while the other lanes of its warp still iterate theirs (MDEF: seven roots per lane).
// need_mid: the origin pole is still to be chosen by the sign of f at the interval's midpoint.
// secular_begin repeats secular_root's choice of interval, origin and bracket (secular_root keeps
// its own scalar form: the kernels that call it are at their register limit), and
// tests/test_secular_host.py checks that both forms give the same roots bit for bit.
template <typename R>
struct SecularSolve {
    R a, b, o, d, dlo, dhi, other, fp, mid;
    int i, jo, it;
    bool need_mid;
};

template <typename R>
NQCD_SECULAR_HD void secular_warm(SecularSolve<R>& s, R lam) {
    s.d = lam - s.o;
    if (!(s.d > s.dlo && s.d < s.dhi)) s.d = R(0.5) * (s.dlo + s.dhi);
    s.other = s.o == s.a ? s.b : s.a;
}

// Interval of root i, origin pole and bracket from the warm start lam (as secular_root).
template <typename R>
NQCD_SECULAR_HD void secular_begin(const R* __restrict__ eps, int M, int i, R Lbound, R lam,
                                              SecularSolve<R>& s) {
    const bool first = i == 0, last = i == M;
    s.i = i;
    s.a = first ? eps[0] : eps[i - 1];
    s.b = last ? eps[M - 1] : eps[i];
    s.fp = R(1);
    s.it = 0;
    s.need_mid = false;
    if (first) {
        s.jo = 0;
        s.o = s.a;
        s.dlo = -Lbound;
        s.dhi = R(0);
    } else if (last) {
        s.jo = M - 1;
        s.o = s.b;
        s.dlo = R(0);
        s.dhi = Lbound;
    } else if (std::is_same<R, float>::value && lam > s.a && lam < s.b) {
        if (lam - s.a < s.b - lam) {
            s.jo = i - 1;
            s.o = s.a;
            s.dlo = R(0);
            s.dhi = s.b - s.a;
        } else {
            s.jo = i;
            s.o = s.b;
            s.dlo = s.a - s.b;
            s.dhi = R(0);
        }
    } else {
        s.mid = s.a + R(0.5) * (s.b - s.a);
        s.need_mid = true;
        return;
    }
    secular_warm(s, lam);
}

// One evaluation of f: the midpoint test that picks the origin pole, or one Newton step (as
// secular_root).  Returns true when the root is done; then l = s.o + s.d, z0^2 = 1 / s.fp.
template <typename R>
NQCD_SECULAR_HD bool secular_eval(const R* __restrict__ eps, const R* __restrict__ V2, int M, R h, R lam,
                                             SecularSolve<R>& s, unsigned long long* nonconv) {
    if (s.need_mid) {
        R sm = R(0);
#pragma unroll 4
        for (int k = 0; k < M; ++k) sm += V2[k] * secular_rcp<R>(s.mid - eps[k]);
        const R fm = s.mid - h - sm;
        if (fm > R(0)) {  // root in (a, mid): measure from a
            s.jo = s.i - 1;
            s.o = s.a;
            s.dlo = R(0);
            s.dhi = s.mid - s.a;
        } else {
            s.jo = s.i;
            s.o = s.b;
            s.dlo = s.mid - s.b;
            s.dhi = R(0);
        }
        s.need_mid = false;
        secular_warm(s, lam);
        return false;
    }
    return secular_newton(eps, V2, M, h, s.jo, s.o, s.other, s.d, s.dlo, s.dhi, s.fp, s.it, nonconv);
}

}  // namespace nqcd
