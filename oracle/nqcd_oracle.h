// CPU oracle of the ensemble trajectory hot path -- TEST INFRASTRUCTURE.
//
// This library is the correctness checker and the timed CPU baseline.  It is
// an FP64 restatement of NQCDynamics.jl's CPU integration (the reference is
// pure Julia and cannot run in this build environment, so nothing here calls
// it).  Only tests, the smoke check and the benchmark's CPU-baseline leg may
// load it; the engine never does.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t model;          // nqcd::ModelKind
    double params[8];       // model parameters (Tully: A,B,C,D[,E0]; spin-boson: eps, Delta)
    int32_t nbath;          // spin-boson: number of bath modes (== ndof)
    const double* bath_c;   // spin-boson coupling c_j
    const double* bath_w2;  // spin-boson omega_j^2
    int32_t ndof;           // degrees of freedom per trajectory (ndofs * natoms)
    const double* mass;     // mass of each degree of freedom [ndof]
    int32_t rescaling;      // 0 standard, 1 velocity inversion, 2 off
    int32_t init_kind;      // 0 sigma/state given, 1 adiabatic pure state, 2 diabatic pure state
    int32_t init_state;     // 0-based state for init_kind 1/2
    double t0, t1, dt;
    uint64_t seed;
    int64_t ntraj;
    int64_t traj_offset;    // global id of trajectory 0 (RNG counter)
    int32_t save_stride;    // population-correlation save every k steps (0 = off)
    int32_t nthreads;
    int32_t max_hops;       // hop-log capacity per trajectory
    int32_t nbeads;         // ring polymer: beads per trajectory (RPSH entry only)
    double beta;            // ring polymer: inverse temperature
    double terminate_x;     // ring polymer: stop when |x_centroid| > terminate_x (0 = off)
    int32_t method;         // 0 FSSH, 1 Ehrenfest (oracle_fssh_run only)
} oracle_fssh_args;

typedef struct {
    double* r;           // [ntraj][ndof] in/out (RPSH: [ntraj][nbeads])
    double* v;           // [ntraj][ndof] in/out
    double* sigma;       // [ntraj][8] in/out: re00 im00 re01 im01 re10 im10 re11 im11
    int32_t* state;      // [ntraj] in/out (0-based)
    int32_t* hop_log;    // [ntraj][max_hops][3]: step, from, to (accepted hops) or NULL
    int32_t* nhops;      // [ntraj] accepted hops or NULL
    int32_t* nfrustrated;// [ntraj] frustrated hops or NULL
    double* popcorr;     // [nsave][4] summed diabatic population correlation or NULL
    double* scatter;     // [4]: reflection(state0,state1), transmission(state0,state1) sums or NULL
    int32_t* nsteps;     // [ntraj] steps taken or NULL
    double* energy;      // [ntraj][2] total energy at start and end or NULL
} oracle_fssh_out;

int oracle_fssh_run(const oracle_fssh_args* a, oracle_fssh_out* o);
int oracle_rpsh_run(const oracle_fssh_args* a, const int32_t* nbeads_per_traj, int32_t beads_stride,
                    oracle_fssh_out* o);

// Primitive checks (KATs and unit tests).
void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double oracle_exp(double x);
double oracle_uniform(uint64_t seed, uint64_t traj, uint32_t step, uint32_t stream);
void oracle_tully(int32_t kind, const double* params, double x, double V[3], double D[3]);
int32_t oracle_select_new_state(const double* cumulative, int32_t nstates, int32_t state, double u);
void oracle_nm_transform(int32_t n, double* U /* n*n column-major: U[j + n*k] */);
void oracle_cayley(int32_t n, double beta, double dt, double* prop /* [n][4] */);

#ifdef __cplusplus
}
#endif
