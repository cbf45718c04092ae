// Host build of the FSSH electronic sub-integration (csrc/fssh2_traj.h), for the CPU tests: the
// fast path's FP32 Tsit5 macro step (stages sharing the p/q derivative, reading G = E0 - E1 and D)
// and the plain path's FP64 four-component Tsit5 macro step, through plain C entry points.  Test
// infrastructure only.
#include "../../nqcdynamics.jl_gb300/csrc/fssh2_traj.h"

// buf = (E0c, E1c, Dc, E0n, E1n, Dn) over the macro step [0, h] (the DoubleBuffer interval), sub-steps
// of dtsub; sg = (p, q, x, y) in and out.
extern "C" void electronics_fast_f32(const float* buf, float h, float dtsub, float* sg) {
    nqcd::EBuf<float> b = {buf[0], buf[1], buf[2], 0.0, buf[3], buf[4], buf[5], (double)h};
    nqcd::Sig2<float> u = {sg[0], sg[1], sg[2], sg[3]};
    nqcd::electronic_macro_step2_fast(b, 0.f, 1.f, h, dtsub, u);
    sg[0] = u.p;
    sg[1] = u.q;
    sg[2] = u.x;
    sg[3] = u.y;
}

extern "C" void electronics_plain_f64(const double* buf, double h, double dtsub, double* sg) {
    nqcd::EBuf<double> b = {buf[0], buf[1], buf[2], 0.0, buf[3], buf[4], buf[5], h};
    nqcd::Interp64 fn(b);
    nqcd::Sig2<double> u = {sg[0], sg[1], sg[2], sg[3]};
    nqcd::electronic_macro_step2<double>(fn, 0.0, h, dtsub, u);
    sg[0] = u.p;
    sg[1] = u.q;
    sg[2] = u.x;
    sg[3] = u.y;
}
