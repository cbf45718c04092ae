// CPU oracle of the ensemble trajectory hot path -- TEST INFRASTRUCTURE ONLY.
//
// An FP64 restatement of NQCDynamics.jl's CPU integration, written to follow
// the reference's operation order (every function cites the reference lines
// it restates).  Parity status: the reference is pure Julia and no Julia
// toolchain exists in the build environment, so this restatement is pinned
// by the reference's own known-answer tests and invariants (see tests/), not
// by running the reference.
//
// Deliberate conventions, shared with the CUDA engine and documented there:
//  * eigenvectors: ascending eigenvalues, sign fixed by continuity with the
//    previous step (identity before the first step of a trajectory);
//  * Z^T dH Z is evaluated as Z^T (dH Z) with ascending inner sums and the
//    upper triangle mirrored, so the nonadiabatic coupling is exactly
//    antisymmetric;
//  * random numbers come from Philox4x32-10 keyed by the run seed with
//    counter (trajectory, step, stream) instead of Julia's task-local
//    Xoshiro stream, which cannot be reproduced outside Julia;
//  * real(sigma_ms / sigma_ss) is evaluated as re(sigma_ms) * (1 / sigma_ss),
//    which is what Julia's complex division reduces to for a real divisor.
#include "nqcd_oracle.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "../nqcdynamics.jl_gb300/csrc/nqcd_math.h"
#include "../nqcdynamics.jl_gb300/csrc/nqcd_models.h"
#include "../nqcdynamics.jl_gb300/csrc/ring_polymer.h"

namespace {

struct cx {
    double re, im;
};
inline cx cmul(cx a, cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline cx cadd(cx a, cx b) { return {a.re + b.re, a.im + b.im}; }
inline cx csub(cx a, cx b) { return {a.re - b.re, a.im - b.im}; }
inline cx cscale(double s, cx a) { return {s * a.re, s * a.im}; }

constexpr int NS = 2;  // two-state models (Tully 1-3, spin-boson)

// ---------------------------------------------------------------------------
// Model evaluation (NQCModels restated; see nqcd_models.h)
// ---------------------------------------------------------------------------
struct Model {
    int kind;
    double p[8];
    int nbath;
    const double* c;
    const double* w2;
};

// Diabatic potential, stored (V00, V01, V11).
void potential(const Model& m, const double* r, int ndof, double V[3]) {
    if (m.kind == nqcd::MODEL_SPINBOSON) {
        // V = [[eps + c.R, Delta], [Delta, -eps - c.R]] + 1/2 sum_j w_j^2 R_j^2
        double s0 = 0.0, cr = 0.0;
        for (int j = 0; j < ndof; ++j) {
            s0 = s0 + m.w2[j] * (r[j] * r[j]);
            cr = cr + m.c[j] * r[j];
        }
        double V0 = 0.5 * s0;
        V[0] = (V0 + cr) + m.p[0];
        V[1] = m.p[1];
        V[2] = (V0 - cr) - m.p[0];
    } else {
        nqcd::tully_potential<double>(m.kind, m.p, r[0], V);
    }
}

// Derivative of the diabatic potential with respect to degree of freedom I.
void derivative(const Model& m, const double* r, int I, double D[3]) {
    if (m.kind == nqcd::MODEL_SPINBOSON) {
        double d0 = m.w2[I] * r[I];
        D[0] = d0 + m.c[I];
        D[1] = 0.0;
        D[2] = d0 - m.c[I];
    } else {
        nqcd::tully_derivative<double>(m.kind, m.p, r[0], D);
    }
}

// ---------------------------------------------------------------------------
// Electronic-structure cache (NQCCalculators.update_cache! restated):
// eigen (w, Z), adiabatic derivative Z^T dH Z, nonadiabatic coupling.
// ---------------------------------------------------------------------------
struct Cache {
    double w[NS];
    double Z[4];      // column-major
    double Zprev[4];  // eigenvectors of the previous evaluation (phase reference)
    std::vector<double> adi;  // [ndof][3] (A00, A01, A11)
    std::vector<double> nac;  // [ndof] d_01 (d_10 = -d_01, d_ii = 0)
};

void update_cache(const Model& m, const double* r, int ndof, Cache& c) {
    double V[3];
    potential(m, r, ndof, V);
    nqcd::eigen2_phase<double>(V, c.Zprev, c.w, c.Z);
    memcpy(c.Zprev, c.Z, sizeof(c.Z));
    for (int I = 0; I < ndof; ++I) {
        double dH[2][2];
        double D[3];
        derivative(m, r, I, D);
        dH[0][0] = D[0];
        dH[0][1] = D[1];
        dH[1][0] = D[1];
        dH[1][1] = D[2];
        double Zm[2][2] = {{c.Z[0], c.Z[2]}, {c.Z[1], c.Z[3]}};
        // T = dH * Z
        double T[2][2];
        for (int k = 0; k < NS; ++k)
            for (int j = 0; j < NS; ++j) {
                double acc = dH[k][0] * Zm[0][j];
                for (int l = 1; l < NS; ++l) acc = acc + dH[k][l] * Zm[l][j];
                T[k][j] = acc;
            }
        // A = Z^T T, upper triangle
        double A[2][2];
        for (int i = 0; i < NS; ++i)
            for (int j = i; j < NS; ++j) {
                double acc = Zm[0][i] * T[0][j];
                for (int k = 1; k < NS; ++k) acc = acc + Zm[k][i] * T[k][j];
                A[i][j] = acc;
            }
        c.adi[3 * I + 0] = A[0][0];
        c.adi[3 * I + 1] = A[0][1];
        c.adi[3 * I + 2] = A[1][1];
        c.nac[I] = A[0][1] / (c.w[1] - c.w[0]);
    }
}

inline double nac_elem(const Cache& c, int I, int i, int j) {
    if (i == j) return 0.0;
    return i < j ? c.nac[I] : -c.nac[I];
}
inline double adi_elem(const Cache& c, int I, int i, int j) {
    if (i == 0 && j == 0) return c.adi[3 * I + 0];
    if (i == 1 && j == 1) return c.adi[3 * I + 2];
    return c.adi[3 * I + 1];
}

// FSSH acceleration: a_I = -(Z^T dH_I Z)_ss / m_I   (fssh.jl:67-74)
void acceleration(const Cache& c, int ndof, const double* mass, int s, double* k) {
    for (int I = 0; I < ndof; ++I) k[I] = -adi_elem(c, I, s, s) / mass[I];
}

// Ehrenfest acceleration (ehrenfest.jl:50-68): a_I = -sum_m sum_n
// (Z^T dH_I Z)_nm Re sigma_nm / m_I, the sum in the reference's loop order
// (m outer, n inner); the models here have no separate state-independent
// derivative (the spin-boson bath term is on the diagonal of dH_I).
void acceleration_ehrenfest(const Cache& c, int ndof, const double* mass, const cx sig[NS][NS], double* k) {
    for (int I = 0; I < ndof; ++I) {
        double acc = adi_elem(c, I, 0, 0) * sig[0][0].re;
        for (int q = 1; q < NS * NS; ++q) {
            const int mm = q / NS, n = q % NS;
            acc = acc + adi_elem(c, I, n, mm) * sig[n][mm].re;
        }
        k[I] = -acc / mass[I];
    }
}

// Ehrenfest potential energy (ehrenfest.jl:85-95): sum_i Re sigma_ii E_i.
double ehrenfest_potential(const Cache& c, const cx sig[NS][NS]) {
    double pe = sig[0][0].re * c.w[0];
    for (int i = 1; i < NS; ++i) pe = pe + sig[i][i].re * c.w[i];
    return pe;
}

// ---------------------------------------------------------------------------
// Electronic density-matrix ODE (electronic_dynamics.jl:15-140)
// ---------------------------------------------------------------------------
struct ElecParams {
    double E[NS];
    double Dc[NS][NS];  // dynamical coupling sum_I d_I v_I
    double t;
};
struct DoubleBuffer {
    ElecParams cur, next;
};

// update_parameters! (electronic_dynamics.jl:38-53, 132-140)
void update_parameters(DoubleBuffer& b, const Cache& c, int ndof, const double* v, double t) {
    std::swap(b.cur, b.next);
    for (int i = 0; i < NS; ++i) b.next.E[i] = c.w[i];
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j) b.next.Dc[i][j] = 0.0;
    for (int I = 0; I < ndof; ++I)
        for (int j = 0; j < NS; ++j)      // column-major element order J
            for (int i = 0; i < NS; ++i) b.next.Dc[i][j] = b.next.Dc[i][j] + nac_elem(c, I, i, j) * v[I];
    b.next.t = t;
}

// f!(du, u, p, t) = -i [A(t), u] with A = diag(E(t)) - i D(t)   (electronic_dynamics.jl:106-116)
void density_rhs(const DoubleBuffer& b, double t, const cx u[NS][NS], cx du[NS][NS]) {
    double s = (t - b.cur.t) / (b.next.t - b.cur.t);
    if (s != s) s = 0.0;
    cx A[NS][NS];
    const cx minus_i = {0.0, -1.0};
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j) {
            double d = b.cur.Dc[i][j] + (b.next.Dc[i][j] - b.cur.Dc[i][j]) * s;
            A[i][j] = cmul({d, 0.0}, minus_i);
        }
    for (int i = 0; i < NS; ++i) A[i][i] = {b.cur.E[i] + (b.next.E[i] - b.cur.E[i]) * s, 0.0};
    // commutator!(C, A, B): C = B*A; C = A*B - C  (density_matrix_dynamics.jl:29-33)
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j) {
            cx ab = cmul(A[i][0], u[0][j]);
            cx ba = cmul(u[i][0], A[0][j]);
            for (int k = 1; k < NS; ++k) {
                ab = cadd(ab, cmul(A[i][k], u[k][j]));
                ba = cadd(ba, cmul(u[i][k], A[k][j]));
            }
            cx C = csub(ab, ba);
            du[i][j] = cmul(C, minus_i);
        }
}

// One Tsit5 step of size h from t (k1 supplied: first-same-as-last).
void tsit5_step(const DoubleBuffer& b, double t, double h, cx u[NS][NS], cx k1[NS][NS]) {
    using nqcd::Tsit5;
    cx k2[NS][NS], k3[NS][NS], k4[NS][NS], k5[NS][NS], k6[NS][NS], k7[NS][NS], tmp[NS][NS];
#define NQCD_COMB(expr)                                                  \
    for (int i = 0; i < NS; ++i)                                         \
        for (int j = 0; j < NS; ++j) {                                   \
            double re, im;                                               \
            {                                                            \
                auto R = [&](const cx (*k)[NS]) { return k[i][j].re; };    \
                re = u[i][j].re + h * (expr);                            \
            }                                                            \
            {                                                            \
                auto R = [&](const cx (*k)[NS]) { return k[i][j].im; };    \
                im = u[i][j].im + h * (expr);                            \
            }                                                            \
            tmp[i][j] = {re, im};                                        \
        }
    NQCD_COMB(Tsit5::a21 * R(k1));
    density_rhs(b, t + Tsit5::c2 * h, tmp, k2);
    NQCD_COMB(Tsit5::a31 * R(k1) + Tsit5::a32 * R(k2));
    density_rhs(b, t + Tsit5::c3 * h, tmp, k3);
    NQCD_COMB(Tsit5::a41 * R(k1) + Tsit5::a42 * R(k2) + Tsit5::a43 * R(k3));
    density_rhs(b, t + Tsit5::c4 * h, tmp, k4);
    NQCD_COMB(Tsit5::a51 * R(k1) + Tsit5::a52 * R(k2) + Tsit5::a53 * R(k3) + Tsit5::a54 * R(k4));
    density_rhs(b, t + Tsit5::c5 * h, tmp, k5);
    NQCD_COMB(Tsit5::a61 * R(k1) + Tsit5::a62 * R(k2) + Tsit5::a63 * R(k3) + Tsit5::a64 * R(k4) +
              Tsit5::a65 * R(k5));
    density_rhs(b, t + h, tmp, k6);
    NQCD_COMB(Tsit5::a71 * R(k1) + Tsit5::a72 * R(k2) + Tsit5::a73 * R(k3) + Tsit5::a74 * R(k4) +
              Tsit5::a75 * R(k5) + Tsit5::a76 * R(k6));
    density_rhs(b, t + h, tmp, k7);
#undef NQCD_COMB
    memcpy(u, tmp, sizeof(tmp));
    memcpy(k1, k7, sizeof(k7));
}

// SciMLBase.step!(integrator, dt, true) with fixed sub-step dtsub
// (bab_electronics.jl:87-90): sub-steps of dtsub, the last one shortened to
// land on t + h, times within 100 eps of the stop snapped to it.
void electronic_macro_step(const DoubleBuffer& b, double t, double h, double dtsub, cx u[NS][NS]) {
    double tend = t + h;
    cx k1[NS][NS];
    density_rhs(b, t, u, k1);  // u was reset by set_ut!: first-same-as-last re-evaluated
    double tc = t;
    for (int guard = 0; tc < tend && guard < 64; ++guard) {
        double hs = std::min(dtsub, tend - tc);
        tsit5_step(b, tc, hs, u, k1);
        tc = nqcd::snap_time(tc + hs, tend);
    }
}

// ---------------------------------------------------------------------------
// Surface hopping (surface_hopping.jl, fssh.jl)
// ---------------------------------------------------------------------------
int select_new_state(const double* cum, int n, int s, double u) {  // fssh.jl:110-121
    for (int i = 0; i < n; ++i)
        if (i != s && cum[i] > u) return i;
    return s;
}

struct Traj {
    std::vector<double> r, v, k, vtmp;
    cx sig[NS][NS];
    int state;
    Cache cache;
    DoubleBuffer buf;
};

// rescale_velocity! (surface_hopping.jl:64-99); returns true if the hop is accepted
bool rescale_velocity(const oracle_fssh_args& a, Traj& tr, const double* mass, int ndof, int newst,
                      int oldst) {
    if (a.rescaling == 2) return true;
    std::vector<double> d(ndof);
    for (int I = 0; I < ndof; ++I) d[I] = nac_elem(tr.cache, I, newst, oldst);
    double aa = 0.0;
    for (int I = 0; I < ndof; ++I) aa = aa + d[I] * d[I] / mass[I];
    aa = aa / 2.0;
    double bb = 0.0;
    for (int I = 0; I < ndof; ++I) bb = bb + d[I] * tr.v[I];
    double cc = tr.cache.w[newst] - tr.cache.w[oldst];
    double disc = bb * bb - 4.0 * aa * cc;
    if (disc < 0.0) {
        if (a.rescaling == 1) {  // frustrated_hop_invert_velocity! (:155-164)
            double nrm = 0.0;
            for (int I = 0; I < ndof; ++I) nrm = nrm + d[I] * d[I];
            nrm = sqrt(nrm);
            double g = 0.0;
            for (int I = 0; I < ndof; ++I) g = g + tr.v[I] * (d[I] / nrm);
            for (int I = 0; I < ndof; ++I) tr.v[I] = tr.v[I] - 2.0 * g * (d[I] / nrm);
        }
        return false;
    }
    double root = sqrt(disc);
    double gamma = bb < 0.0 ? (bb + root) / (2.0 * aa) : (bb - root) / (2.0 * aa);
    for (int I = 0; I < ndof; ++I) tr.v[I] = tr.v[I] - gamma * d[I] / mass[I];
    return true;
}

// diabatic population of FSSH (fssh.jl:132-142): diag(U sigma' U^T) with the
// occupied state on the diagonal of sigma'; Ehrenfest (ehrenfest.jl:75-83):
// sigma' = Re sigma.
void diabatic_population(const Traj& tr, double pop[NS], bool ehrenfest = false) {
    double sp[NS][NS];
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j) sp[i][j] = tr.sig[i][j].re;
    if (!ehrenfest) {
        for (int i = 0; i < NS; ++i) sp[i][i] = 0.0;
        sp[tr.state][tr.state] = 1.0;
    }
    double U[NS][NS] = {{tr.cache.Z[0], tr.cache.Z[2]}, {tr.cache.Z[1], tr.cache.Z[3]}};
    double M[NS][NS];
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j) {
            double acc = U[i][0] * sp[0][j];
            for (int k = 1; k < NS; ++k) acc = acc + U[i][k] * sp[k][j];
            M[i][j] = acc;
        }
    for (int i = 0; i < NS; ++i) {
        double acc = M[i][0] * U[i][0];
        for (int k = 1; k < NS; ++k) acc = acc + M[i][k] * U[i][k];
        pop[i] = acc;
    }
}

double kinetic_energy(const std::vector<double>& v, const double* mass) {
    double ke = 0.0;
    for (size_t I = 0; I < v.size(); ++I) ke = ke + mass[I] * (v[I] * v[I]);
    return ke / 2.0;
}

// Initial electronic variables (fssh.jl:47-65, density_matrix_dynamics.jl:37-75)
void init_electronics(const oracle_fssh_args& a, int64_t gid, Traj& tr) {
    if (a.init_kind == 0) return;
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j) tr.sig[i][j] = {0.0, 0.0};
    if (a.init_kind == 1) {
        tr.sig[a.init_state][a.init_state] = {1.0, 0.0};
        tr.state = a.init_state;
        return;
    }
    // diabatic pure state -> adiabatic: sigma = U' rho U
    double U[NS][NS] = {{tr.cache.Z[0], tr.cache.Z[2]}, {tr.cache.Z[1], tr.cache.Z[3]}};
    double rho[NS][NS] = {{0.0, 0.0}, {0.0, 0.0}};
    rho[a.init_state][a.init_state] = 1.0;
    double T[NS][NS], S[NS][NS];
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j) {
            double acc = U[0][i] * rho[0][j];
            for (int l = 1; l < NS; ++l) acc = acc + U[l][i] * rho[l][j];
            T[i][j] = acc;
        }
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j) {
            double acc = T[i][0] * U[0][j];
            for (int l = 1; l < NS; ++l) acc = acc + T[i][l] * U[l][j];
            S[i][j] = acc;
            tr.sig[i][j] = {acc, 0.0};
        }
    // state = sample(Weights(diag(real(sigma))))  (StatsBase weighted sampling)
    double wsum = S[0][0] + S[1][1];
    double tt = nqcd::rng_uniform(a.seed, (uint64_t)gid, 0u, nqcd::RNG_INIT_STATE) * wsum;
    int i = 0;
    double cw = S[0][0];
    while (cw < tt && i < NS - 1) {
        i += 1;
        cw = cw + S[i][i];
    }
    tr.state = i;
}

struct Partial {
    std::vector<double> popcorr;
    double scatter[4] = {0, 0, 0, 0};
};

void run_one_fssh(const oracle_fssh_args& a, const Model& m, int64_t it, oracle_fssh_out* o, Partial& part) {
    const int ndof = a.ndof;
    const int64_t gid = a.traj_offset + it;
    Traj tr;
    tr.r.assign(o->r + it * ndof, o->r + (it + 1) * ndof);
    tr.v.assign(o->v + it * ndof, o->v + (it + 1) * ndof);
    tr.k.assign(ndof, 0.0);
    tr.vtmp.assign(ndof, 0.0);
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j)
            tr.sig[i][j] = {o->sigma[it * 8 + 2 * (2 * i + j)], o->sigma[it * 8 + 2 * (2 * i + j) + 1]};
    tr.state = o->state[it];
    tr.cache.adi.assign(3 * ndof, 0.0);
    tr.cache.nac.assign(ndof, 0.0);
    tr.cache.Zprev[0] = 1.0;
    tr.cache.Zprev[1] = 0.0;
    tr.cache.Zprev[2] = 0.0;
    tr.cache.Zprev[3] = 1.0;
    // DensityMatrixODEProblem parameters start zeroed at t = 0 (electronic_dynamics.jl:118-127)
    memset(&tr.buf, 0, sizeof(tr.buf));

    // initialize!: update_cache!(r); k = a(r, state) or a(r, sigma)   (bab_electronics.jl:48-59)
    const bool ehr = a.method == 1;
    update_cache(m, tr.r.data(), ndof, tr.cache);
    init_electronics(a, gid, tr);
    if (ehr)
        acceleration_ehrenfest(tr.cache, ndof, a.mass, tr.sig, tr.k.data());
    else
        acceleration(tr.cache, ndof, a.mass, tr.state, tr.k.data());

    double e0 = kinetic_energy(tr.v, a.mass) + (ehr ? ehrenfest_potential(tr.cache, tr.sig) : tr.cache.w[tr.state]);
    int nsave = 0;
    double pop0[NS];
    if (a.save_stride > 0) {
        diabatic_population(tr, pop0, ehr);
        for (int i = 0; i < NS; ++i)
            for (int j = 0; j < NS; ++j) part.popcorr[0 * 4 + 2 * i + j] += pop0[i] * pop0[j];
        nsave = 1;
    }

    int nh = 0, nf = 0;
    double t = a.t0;
    int step = 0;
    const double dtsub = a.dt / 5.0;
    while (t < a.t1) {
        double h = std::min(a.dt, a.t1 - t);
        // perform_step! (bab_electronics.jl:61-91)
        double half = h / 2.0;
        for (int I = 0; I < ndof; ++I) tr.vtmp[I] = tr.v[I] + half * tr.k[I];
        for (int I = 0; I < ndof; ++I) tr.r[I] = tr.r[I] + h * tr.vtmp[I];
        update_cache(m, tr.r.data(), ndof, tr.cache);
        // Ehrenfest: the force of the density matrix the step starts with (sigma_prev)
        if (ehr)
            acceleration_ehrenfest(tr.cache, ndof, a.mass, tr.sig, tr.k.data());
        else
            acceleration(tr.cache, ndof, a.mass, tr.state, tr.k.data());
        for (int I = 0; I < ndof; ++I) tr.v[I] = tr.vtmp[I] + half * tr.k[I];
        update_parameters(tr.buf, tr.cache, ndof, tr.v.data(), t + h);
        electronic_macro_step(tr.buf, t, h, dtsub, tr.sig);
        t = nqcd::snap_time(t + h, a.t1);
        step += 1;

        if (ehr) {  // no hopping callback
            if (a.save_stride > 0 && step % a.save_stride == 0) {
                double pop[NS];
                diabatic_population(tr, pop, true);
                for (int i = 0; i < NS; ++i)
                    for (int j = 0; j < NS; ++j) part.popcorr[nsave * 4 + 2 * i + j] += pop0[i] * pop[j];
                nsave += 1;
            }
            continue;
        }
        // HoppingCallback (surface_hopping.jl:2-16, fssh.jl:86-121)
        double prob[NS] = {0.0, 0.0};
        const int s = tr.state;
        for (int mm = 0; mm < NS; ++mm) {
            if (mm == s) continue;
            // real(sigma[m, s] / sigma[s, s]): Julia's Complex{Float64} division (fssh.jl:101)
            double re = nqcd::cdiv_real(tr.sig[mm][s].re, tr.sig[mm][s].im, tr.sig[s][s].re, tr.sig[s][s].im);
            for (int I = 0; I < ndof; ++I)
                prob[mm] = prob[mm] + 2.0 * tr.v[I] * re * nac_elem(tr.cache, I, s, mm) * a.dt;
        }
        for (int i = 0; i < NS; ++i) prob[i] = std::min(std::max(prob[i], 0.0), 1.0);
        for (int i = 1; i < NS; ++i) prob[i] = prob[i - 1] + prob[i];
        double u = nqcd::rng_uniform(a.seed, (uint64_t)gid, (uint32_t)step, nqcd::RNG_HOP);
        int ns = select_new_state(prob, NS, s, u);
        if (ns != s) {
            if (rescale_velocity(a, tr, a.mass, ndof, ns, s)) {
                if (o->hop_log && nh < a.max_hops) {
                    int32_t* e = o->hop_log + (it * a.max_hops + nh) * 3;
                    e[0] = step;
                    e[1] = s;
                    e[2] = ns;
                }
                nh += 1;
                tr.state = ns;
            } else {
                nf += 1;
            }
        }
        if (a.save_stride > 0 && step % a.save_stride == 0) {
            double pop[NS];
            diabatic_population(tr, pop);
            for (int i = 0; i < NS; ++i)
                for (int j = 0; j < NS; ++j) part.popcorr[nsave * 4 + 2 * i + j] += pop0[i] * pop[j];
            nsave += 1;
        }
    }

    // write back
    std::copy(tr.r.begin(), tr.r.end(), o->r + it * ndof);
    std::copy(tr.v.begin(), tr.v.end(), o->v + it * ndof);
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j) {
            o->sigma[it * 8 + 2 * (2 * i + j)] = tr.sig[i][j].re;
            o->sigma[it * 8 + 2 * (2 * i + j) + 1] = tr.sig[i][j].im;
        }
    o->state[it] = tr.state;
    if (o->nhops) o->nhops[it] = nh;
    if (o->nfrustrated) o->nfrustrated[it] = nf;
    if (o->nsteps) o->nsteps[it] = step;
    if (o->energy) {
        o->energy[2 * it] = e0;
        o->energy[2 * it + 1] =
            kinetic_energy(tr.v, a.mass) + (ehr ? ehrenfest_potential(tr.cache, tr.sig) : tr.cache.w[tr.state]);
    }
    // OutputStateResolvedScattering1D, adiabatic populations (DynamicsOutputs.jl:313-338):
    // the occupied state (FSSH) or diag(Re sigma) (Ehrenfest, ehrenfest.jl:74-77)
    const int side = tr.r[0] > 0.0 ? 2 : 0;
    if (ehr) {
        for (int i = 0; i < NS; ++i) part.scatter[side + i] += tr.sig[i][i].re;
    } else {
        part.scatter[side + tr.state] += 1.0;
    }
}


// ---------------------------------------------------------------------------
// Ring-polymer surface hopping (BCBwithTsit5 + rpsh.jl), Tully models.
// ---------------------------------------------------------------------------
struct RPTables {
    std::vector<double> U;    // n*n column-major
    std::vector<double> cay;  // [n][4]
};

// Per-bead FSSH force on the active state: -(Z^T dH Z)_ss / m for each bead
// (fssh.jl:67-74 applied bead-wise).  The eigenvector sign cancels in the
// diagonal element, so each bead is diagonalised without phase tracking.
double bead_accel(const Model& m, double x, int s, double mass, double* w_s) {
    double V[3], D[3], w[2], Z[4];
    const double I2[4] = {1.0, 0.0, 0.0, 1.0};
    nqcd::tully_potential<double>(m.kind, m.p, x, V);
    nqcd::eigen2_phase<double>(V, I2, w, Z);
    nqcd::tully_derivative<double>(m.kind, m.p, x, D);
    double dH[2][2] = {{D[0], D[1]}, {D[1], D[2]}};
    double Zm[2][2] = {{Z[0], Z[2]}, {Z[1], Z[3]}};
    double T0 = dH[0][0] * Zm[0][s] + dH[0][1] * Zm[1][s];
    double T1 = dH[1][0] * Zm[0][s] + dH[1][1] * Zm[1][s];
    double a = Zm[0][s] * T0 + Zm[1][s] * T1;
    if (w_s) *w_s = w[s];
    return -a / mass;
}

double centroid(const double* x, int n) {
    double acc = 0.0;
    for (int j = 0; j < n; ++j) acc = acc + x[j];
    return acc / n;
}

// to normal modes: q_k = sum_j U[j,k] x_j ; from: x_j = sum_k U[j,k] q_k
void to_modes(const RPTables& tb, int n, const double* x, double* q) {
    for (int k = 0; k < n; ++k) {
        double acc = tb.U[0 + n * k] * x[0];
        for (int j = 1; j < n; ++j) acc = acc + tb.U[j + n * k] * x[j];
        q[k] = acc;
    }
}
void from_modes(const RPTables& tb, int n, const double* q, double* x) {
    for (int j = 0; j < n; ++j) {
        double acc = tb.U[j] * q[0];
        for (int k = 1; k < n; ++k) acc = acc + tb.U[j + n * k] * q[k];
        x[j] = acc;
    }
}

void run_one_rpsh(const oracle_fssh_args& a, const Model& m, const RPTables& tb, int nb, int stride, int64_t it,
                  oracle_fssh_out* o, Partial& part) {
    const int64_t gid = a.traj_offset + it;
    const double mass = a.mass[0];
    std::vector<double> r(o->r + it * stride, o->r + it * stride + nb), v(o->v + it * stride, o->v + it * stride + nb);
    std::vector<double> k(nb), vt(nb), q(nb), p(nb);
    Traj tr;  // electronic part and centroid cache
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j)
            tr.sig[i][j] = {o->sigma[it * 8 + 2 * (2 * i + j)], o->sigma[it * 8 + 2 * (2 * i + j) + 1]};
    tr.state = o->state[it];
    tr.cache.adi.assign(3, 0.0);
    tr.cache.nac.assign(1, 0.0);
    tr.cache.Zprev[0] = 1.0;
    tr.cache.Zprev[1] = 0.0;
    tr.cache.Zprev[2] = 0.0;
    tr.cache.Zprev[3] = 1.0;
    memset(&tr.buf, 0, sizeof(tr.buf));

    // initialize!: update_cache!(r) (beads + centroid); k per bead
    double xc = centroid(r.data(), nb);
    update_cache(m, &xc, 1, tr.cache);
    init_electronics(a, gid, tr);
    for (int j = 0; j < nb; ++j) k[j] = bead_accel(m, r[j], tr.state, mass, nullptr);
    auto rp_energy = [&]() {
        double wn = nb / a.beta;
        double spring = 0.0;
        if (nb > 1) {
            spring = spring + mass * ((r[nb - 1] - r[0]) * (r[nb - 1] - r[0]));
            for (int j = 0; j < nb - 1; ++j) spring = spring + mass * ((r[j] - r[j + 1]) * (r[j] - r[j + 1]));
        }
        spring = spring * (wn * wn) / 2.0;
        double ke = 0.0, pe = 0.0;
        for (int j = 0; j < nb; ++j) ke = ke + mass * (v[j] * v[j]);
        for (int j = 0; j < nb; ++j) {
            double ws;
            bead_accel(m, r[j], tr.state, mass, &ws);
            pe = pe + ws;
        }
        return spring + ke / 2.0 + pe;
    };
    double e0 = rp_energy();

    int nh = 0, nf = 0, step = 0;
    double t = a.t0;
    const double dtsub = a.dt / 5.0;
    while (t < a.t1) {
        double h = std::min(a.dt, a.t1 - t);
        double half = h / 2.0;
        // perform_step! (bcb_electronics.jl:53-97)
        for (int j = 0; j < nb; ++j) vt[j] = v[j] + half * k[j];
        to_modes(tb, nb, r.data(), q.data());
        to_modes(tb, nb, vt.data(), p.data());
        for (int j = 0; j < nb; ++j) {  // step_C! (steps.jl:10-17)
            const double* c = &tb.cay[4 * j];
            double rn = c[0] * q[j] + c[1] * p[j];
            double vn = c[2] * q[j] + c[3] * p[j];
            q[j] = rn;
            p[j] = vn;
        }
        from_modes(tb, nb, q.data(), r.data());
        from_modes(tb, nb, p.data(), vt.data());
        for (int j = 0; j < nb; ++j) k[j] = bead_accel(m, r[j], tr.state, mass, nullptr);
        for (int j = 0; j < nb; ++j) v[j] = vt[j] + half * k[j];
        xc = centroid(r.data(), nb);
        update_cache(m, &xc, 1, tr.cache);  // centroid eigen and coupling
        double vc = centroid(v.data(), nb);
        update_parameters(tr.buf, tr.cache, 1, &vc, t + h);
        electronic_macro_step(tr.buf, t, h, dtsub, tr.sig);
        t = nqcd::snap_time(t + h, a.t1);
        step += 1;

        // HoppingCallback with centroid quantities (rpsh.jl, fssh.jl:86-121)
        const int s = tr.state;
        double prob[NS] = {0.0, 0.0};
        for (int mm = 0; mm < NS; ++mm) {
            if (mm == s) continue;
            // real(sigma[m, s] / sigma[s, s]): Julia's Complex{Float64} division (fssh.jl:101)
            double re = nqcd::cdiv_real(tr.sig[mm][s].re, tr.sig[mm][s].im, tr.sig[s][s].re, tr.sig[s][s].im);
            prob[mm] = prob[mm] + 2.0 * vc * re * nac_elem(tr.cache, 0, s, mm) * a.dt;
        }
        for (int i = 0; i < NS; ++i) prob[i] = std::min(std::max(prob[i], 0.0), 1.0);
        for (int i = 1; i < NS; ++i) prob[i] = prob[i - 1] + prob[i];
        double u = nqcd::rng_uniform(a.seed, (uint64_t)gid, (uint32_t)step, nqcd::RNG_HOP);
        int ns = select_new_state(prob, NS, s, u);
        if (ns != s) {
            bool accept = true;
            if (a.rescaling != 2) {
                double d = nac_elem(tr.cache, 0, ns, s);
                double aa = (0.0 + d * d / mass) / 2.0;
                double bb = 0.0 + d * vc;
                double cc = tr.cache.w[ns] - tr.cache.w[s];
                double disc = bb * bb - 4.0 * aa * cc;
                if (disc < 0.0) {
                    accept = false;
                    if (a.rescaling == 1) {  // rpsh.jl:39-50
                        double nrm = sqrt(0.0 + d * d);
                        double dn = d / nrm;
                        double vcom = 0.0;
                        for (int j = 0; j < nb; ++j) vcom = vcom + v[j];
                        vcom = vcom / nb;
                        double g = 0.0 + vcom * dn;
                        for (int j = 0; j < nb; ++j) v[j] = v[j] - 2.0 * g * dn;
                    }
                } else {
                    double root = sqrt(disc);
                    double gamma = bb < 0.0 ? (bb + root) / (2.0 * aa) : (bb - root) / (2.0 * aa);
                    double dv = gamma * d / mass;  // rpsh.jl:30-37
                    for (int j = 0; j < nb; ++j) v[j] = v[j] - dv;
                }
            }
            if (accept) {
                if (o->hop_log && nh < a.max_hops) {
                    int32_t* e = o->hop_log + (it * a.max_hops + nh) * 3;
                    e[0] = step;
                    e[1] = s;
                    e[2] = ns;
                }
                nh += 1;
                tr.state = ns;
            } else {
                nf += 1;
            }
        }
        // TerminatingCallback(|x_centroid| > L)  (callbacks.jl:29)
        if (a.terminate_x > 0.0 && fabs(centroid(r.data(), nb)) > a.terminate_x) break;
    }
    std::copy(r.begin(), r.end(), o->r + it * stride);
    std::copy(v.begin(), v.end(), o->v + it * stride);
    for (int i = 0; i < NS; ++i)
        for (int j = 0; j < NS; ++j) {
            o->sigma[it * 8 + 2 * (2 * i + j)] = tr.sig[i][j].re;
            o->sigma[it * 8 + 2 * (2 * i + j) + 1] = tr.sig[i][j].im;
        }
    o->state[it] = tr.state;
    if (o->nhops) o->nhops[it] = nh;
    if (o->nfrustrated) o->nfrustrated[it] = nf;
    if (o->nsteps) o->nsteps[it] = step;
    if (o->energy) {
        o->energy[2 * it] = e0;
        o->energy[2 * it + 1] = rp_energy();
    }
    // OutputStateResolvedScattering1D reads the first bead's position
    if (r[0] > 0.0)
        part.scatter[2 + tr.state] += 1.0;
    else
        part.scatter[tr.state] += 1.0;
}

int64_t count_saves(const oracle_fssh_args& a) {
    if (a.save_stride <= 0) return 0;
    int64_t n = 0;
    double t = a.t0;
    while (t < a.t1) {
        double h = std::min(a.dt, a.t1 - t);
        t = nqcd::snap_time(t + h, a.t1);
        n += 1;
    }
    return n / a.save_stride + 1;
}

template <typename F>
void parallel_over_traj(const oracle_fssh_args& a, int64_t nsave, oracle_fssh_out* o, F&& body) {
    int nth = a.nthreads > 0 ? a.nthreads : 1;
    if ((int64_t)nth > a.ntraj) nth = (int)std::max<int64_t>(1, a.ntraj);
    std::vector<Partial> parts(nth);
    for (auto& p : parts) p.popcorr.assign((size_t)std::max<int64_t>(nsave, 1) * 4, 0.0);
    std::vector<std::thread> pool;
    for (int th = 0; th < nth; ++th) {
        pool.emplace_back([&, th]() {
            int64_t lo = a.ntraj * th / nth, hi = a.ntraj * (th + 1) / nth;
            for (int64_t it = lo; it < hi; ++it) body(it, parts[th]);
        });
    }
    for (auto& t : pool) t.join();
    if (o->popcorr)
        for (int64_t s = 0; s < nsave * 4; ++s) {
            double acc = 0.0;
            for (int th = 0; th < nth; ++th) acc += parts[th].popcorr[s];
            o->popcorr[s] = acc;
        }
    if (o->scatter)
        for (int q = 0; q < 4; ++q) {
            double acc = 0.0;
            for (int th = 0; th < nth; ++th) acc += parts[th].scatter[q];
            o->scatter[q] = acc;
        }
}

}  // namespace

extern "C" int oracle_fssh_run(const oracle_fssh_args* a, oracle_fssh_out* o) {
    if (!a || !o || !o->r || !o->v || !o->sigma || !o->state || a->ndof <= 0 || a->dt <= 0) return -1;
    Model m;
    m.kind = a->model;
    memcpy(m.p, a->params, sizeof(m.p));
    m.nbath = a->nbath;
    m.c = a->bath_c;
    m.w2 = a->bath_w2;
    int64_t nsave = count_saves(*a);
    parallel_over_traj(*a, nsave, o, [&](int64_t it, Partial& part) { run_one_fssh(*a, m, it, o, part); });
    return 0;
}

extern "C" void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    nqcd::u32x4 c = {ctr[0], ctr[1], ctr[2], ctr[3]};
    nqcd::u32x4 r = nqcd::philox4x32_10(c, key[0], key[1]);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.w;
}

extern "C" double oracle_exp(double x) { return nqcd::nqcd_exp(x); }

extern "C" double oracle_cdiv_real(double a, double b, double c, double d) { return nqcd::cdiv_real(a, b, c, d); }

extern "C" double oracle_uniform(uint64_t seed, uint64_t traj, uint32_t step, uint32_t stream) {
    return nqcd::rng_uniform(seed, traj, step, stream);
}

extern "C" void oracle_tully(int32_t kind, const double* params, double x, double V[3], double D[3]) {
    nqcd::tully_potential<double>(kind, params, x, V);
    nqcd::tully_derivative<double>(kind, params, x, D);
}

extern "C" int32_t oracle_select_new_state(const double* cumulative, int32_t nstates, int32_t state, double u) {
    return select_new_state(cumulative, nstates, state, u);
}

extern "C" int oracle_rpsh_run(const oracle_fssh_args* a, const int32_t* nbeads_per_traj, int32_t stride,
                               oracle_fssh_out* o) {
    if (!a || !o || !o->r || !o->v || !o->sigma || !o->state || a->dt <= 0 || stride <= 0 || !(a->beta > 0))
        return -1;
    if (a->model < 1 || a->model > 3) return -6;
    Model m;
    m.kind = a->model;
    memcpy(m.p, a->params, sizeof(m.p));
    m.nbath = 0;
    m.c = m.w2 = nullptr;
    std::vector<RPTables> tables(stride + 1);
    for (int n = 1; n <= stride; ++n) {
        tables[n].U.resize((size_t)n * n);
        tables[n].cay.resize((size_t)4 * n);
        nqcd::nm_transform_matrix(n, tables[n].U.data());
        nqcd::cayley_matrices(n, a->beta, a->dt, tables[n].cay.data());
    }
    for (int64_t i = 0; i < a->ntraj; ++i) {
        int nb = nbeads_per_traj ? nbeads_per_traj[i] : a->nbeads;
        if (nb < 1 || nb > stride) return -1;
    }
    parallel_over_traj(*a, 0, o, [&](int64_t it, Partial& part) {
        int nb = nbeads_per_traj ? nbeads_per_traj[it] : a->nbeads;
        run_one_rpsh(*a, m, tables[nb], nb, stride, it, o, part);
    });
    return 0;
}

extern "C" void oracle_nm_transform(int32_t n, double* U) { nqcd::nm_transform_matrix(n, U); }

extern "C" void oracle_cayley(int32_t n, double beta, double dt, double* prop) {
    nqcd::cayley_matrices(n, beta, dt, prop);
}
