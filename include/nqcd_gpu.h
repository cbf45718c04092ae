/*
 * nqcd_gpu.h -- C ABI of the GB300 ensemble trajectory engine.
 *
 * The engine runs NQCDynamics.jl's ensemble trajectory loop (FSSH surface
 * hopping on two-state models, ring-polymer surface hopping) on one GPU.
 * It is the body of a GPU `ensemble_algorithm` that `run_dynamics` forwards to
 * `SciMLBase.solve` (reference: src/Ensembles/run_dynamics.jl:42-136, the
 * solve call at :91-97), so that a Julia host calls it through `ccall` in
 * place of the per-trajectory CPU loop of `EnsembleSerial`/`EnsembleThreads`.
 *
 * Conventions
 *  - Every entry point returns 0 (NQCD_OK) or a negative NQCD_ERR_* code;
 *    no C++ exception crosses the boundary.  nqcd_last_error() gives text.
 *  - Host arrays use the reference's (Julia, column-major) layout with the
 *    trajectory index slowest: positions/velocities as (ndofs, natoms, ntraj)
 *    or (ndofs, natoms, nbeads, ntraj), density matrices as
 *    (nstates, nstates, ntraj).  States are 0-based.
 *  - The caller owns host buffers; the handle owns device memory and its
 *    CUDA stream until nqcd_destroy().  A handle is used by one host thread
 *    at a time; separate handles may run concurrently.
 *  - There is no CPU fallback: without a usable GPU, nqcd_create() fails
 *    with NQCD_ERR_CUDA.
 */
#ifndef NQCD_GPU_H
#define NQCD_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NQCD_ABI_VERSION 111

enum nqcd_status {
    NQCD_OK = 0,
    NQCD_ERR_ARG = -1,         /* invalid argument or configuration */
    NQCD_ERR_CUDA = -2,        /* CUDA runtime error (message in nqcd_last_error) */
    NQCD_ERR_OOM = -3,         /* device or host allocation failed */
    NQCD_ERR_TIMEOUT = -4,     /* a bounded device wait gave up */
    NQCD_ERR_NAN = -5,         /* non-finite values detected in the final state */
    NQCD_ERR_UNSUPPORTED = -6, /* method/model/output combination not supported */
    NQCD_ERR_STATE = -7        /* call out of order (e.g. run before set_initial) */
};

enum nqcd_method {
    NQCD_METHOD_FSSH = 1,
    NQCD_METHOD_RPSH = 2,
    NQCD_METHOD_IESH = 3,
    NQCD_METHOD_MDEF = 4,
    NQCD_METHOD_EHRENFEST = 5, /* Simulation{Ehrenfest} (EhrenfestMethods/ehrenfest.jl): the FSSH integrator
                                (BABwithTsit5) with the mean-field force -sum_nm (Z^T dH Z)_nm Re sigma_nm of
                                the step's initial density matrix and no hopping; two-state models.
                                Scattering outputs are the populations diag(Re sigma) summed by side. */
    NQCD_METHOD_EHRENFEST_NA = 6 /* Simulation{EhrenfestNA} (EhrenfestMethods/ehrenfest_na.jl) on
                                NQCD_MODEL_NEWNS_ANDERSON_3D: the IESH integrator and Fermi-Dirac initial
                                orbitals with the mean-field force of the orbitals before each propagation,
                                -dh/dq sum_e |sum_n z0_n psi_ne|^2, and no hopping (configured like IESH;
                                observables[2] is sum_e |sum_n z0_n psi_ne|^2, [3] U0 + sum l_i |psi_ie|^2). */
};

enum nqcd_model {
    NQCD_MODEL_TULLY1 = 1,    /* params: A, B, C, D */
    NQCD_MODEL_TULLY2 = 2,    /* params: A, B, C, D, E0 */
    NQCD_MODEL_TULLY3 = 3,    /* params: A, B, C */
    NQCD_MODEL_SPINBOSON = 10, /* params: eps, Delta; bath_a = c_j, bath_b = omega_j */
    NQCD_MODEL_NEWNS_ANDERSON = 20, /* AndersonHolstein with a displaced-harmonic impurity:
                                      U0 = k x^2/2, U1 = k (x-g)^2/2 + delta; params: k, g, delta, mu, sigma
                                      (Fermi level, Gaussian broadening width of the friction);
                                      bath_a = bath levels e_k (ascending), bath_b = couplings V_k */
    NQCD_MODEL_NEWNS_ANDERSON_3D = 21 /* AndersonHolstein, one atom (x, y, z) above the metal:
                                      U0 = kxy (x^2+y^2)/2 + A exp(-a z), h = U1 - U0 = delta - B exp(-b z);
                                      params: kxy, A, a, delta, B, b (IESH, EhrenfestNA), then mu, sigma
                                      (MDEF: ndofs = 3, the friction tensor along z); bath_a = e_k
                                      (ascending), bath_b = V_k; nstates = nbath + 1 */
};

enum nqcd_precision {
    NQCD_PREC_FP64 = 0,      /* plain path: bit-identical to the FP64 reference integration */
    NQCD_PREC_FP32 = 1,      /* fast path: FP32 electronic structure, FP64 position/velocity accumulation */
    NQCD_PREC_FP32_KAHAN = 2 /* fast path with Kahan-compensated FP32 accumulation (no FP64 pipe work per mode) */
};

enum nqcd_rescaling { NQCD_RESCALE_STANDARD = 0, NQCD_RESCALE_VINVERSION = 1, NQCD_RESCALE_OFF = 2 };

enum nqcd_init {
    NQCD_INIT_GIVEN = 0,          /* density matrix and state from nqcd_set_initial */
    NQCD_INIT_ADIABATIC_PURE = 1, /* PureState(init_state, Adiabatic()) */
    NQCD_INIT_DIABATIC_PURE = 2,  /* PureState(init_state, Diabatic()): rotated, state sampled */
    NQCD_INIT_FERMI_DIRAC = 3     /* IESH: FermiDiracState(mu, 1/beta, Adiabatic()), occupations sampled
                                     (src/DynamicsUtils/DynamicsUtils.jl:194-208); NQCD_INIT_GIVEN reads them */
};

typedef struct nqcd_config {
    int32_t method;       /* nqcd_method */
    int32_t model;        /* nqcd_model */
    int32_t precision;    /* nqcd_precision */
    int32_t rescaling;    /* nqcd_rescaling (FSSH `rescaling` keyword) */
    int32_t ndofs;        /* degrees of freedom per atom */
    int32_t natoms;       /* atoms */
    int32_t nstates;      /* electronic states (2 for the supported models) */
    int32_t nbeads_max;   /* ring polymer: largest bead count (0 or 1 for classical nuclei); with
                             NQCD_METHOD_MDEF, 2..32 selects ring-polymer MDEF (BCOCB, rpmdef.jl) with
                             this many beads for every trajectory (final states only); with
                             NQCD_METHOD_IESH, 2..32 selects ring-polymer IESH (BCBWavefunction,
                             rpiesh.jl; <= 64 electrons, final states and energies only, no decoherence
                             correction, beta also the Fermi-Dirac inverse temperature): bead forces from
                             each bead's eigenstates, orbitals and hops from the centroid's */
    int32_t nparams;      /* entries of params */
    const double* params; /* model parameters, see nqcd_model */
    int32_t nbath;        /* spin-boson bath modes (== natoms * ndofs) */
    const double* bath_a; /* spin-boson: couplings c_j */
    const double* bath_b; /* spin-boson: frequencies omega_j */
    const double* masses; /* [natoms] */
    double beta;          /* ring polymer: inverse temperature 1/kT (atomic units) */
    int64_t ntraj_max;    /* capacity: trajectories per run */
    int32_t init_kind;    /* nqcd_init */
    int32_t init_state;   /* 0-based state for NQCD_INIT_*_PURE */
    int32_t save_stride;  /* population correlation every save_stride steps (0 = off) */
    int32_t max_hops;     /* hop-log capacity per trajectory (0 = no log) */
    double terminate_x;   /* ring polymer: stop a trajectory once |centroid x| > terminate_x (0 = off) */
    double gap_fp64;      /* fast path: propagate electronics in FP64 when the adiabatic gap is below this;
                             IESH: solve adjacent roots closer than this again in FP64 and form the
                             couplings between them from the FP64 roots (0 = off) */
    int64_t traj_offset;  /* global index of trajectory 0 (Philox counter), for sharded ensembles */
    int32_t use_friction_surrogate; /* MDEF fast path: friction from the trained network inside its domain */
    int32_t exact_friction_every; /* MDEF with surrogate: exact friction every k steps (0 = never) */
    int32_t nelectrons;   /* IESH: electrons (occupied one-electron states) */
    int32_t exact_hop_probability; /* IESH: 1 = no estimate screen (estimate_probability = false) */
    int32_t reserved[2];
    double decoherence_C; /* IESH: energy-based decoherence correction (DecoherenceCorrectionEDC(C),
                             decoherence_corrections.jl:21-39, applied after every step as the callback
                             of iesh.jl:424-441); 0 = none (the reference's default), 0.1 = EDC() */
    double surrogate_tolerance; /* MDEF with surrogate: on each exact_friction_every-th step the network is
                             judged against the exact friction (mdef.jl:131-140); a relative error
                             |net - exact| / max(|exact|, 0.1 max friction of the domain) above this
                             switches the trajectory to exact friction for the rest of the run
                             (<= 0: 0.1) */
} nqcd_config;

typedef struct nqcd_outputs {
    /* Ensemble means (MeanReduction, src/Ensembles/reductions.jl:36-52).  Host pointers; NULL to skip. */
    double* scattering;             /* [2][nstates]: reflection, transmission (OutputStateResolvedScattering1D) */
    double* population_correlation; /* [nsave][nstates][nstates] (PopulationCorrelationFunction, Diabatic) */
    double* observables;            /* MDEF: [nsave][4] means of x, x^2, kinetic energy, friction;
                                       IESH: [nsave][4] means of z, kinetic energy, impurity (diabatic)
                                       population (iesh.jl:351-369), potential energy (iesh.jl:380-388) */
    int32_t nsave;                  /* out: save points written */
    int32_t reserved;
} nqcd_outputs;

typedef struct nqcd_stats {
    int64_t traj_steps;     /* nuclear steps summed over trajectories */
    int64_t hops;           /* accepted hops */
    int64_t frustrated;     /* frustrated hops */
    int64_t flagged;        /* trajectories with non-finite final state */
    double device_ms;       /* CUDA-event time of the whole call's device work on the engine stream */
    double kernel_ms;       /* CUDA-event time of the ensemble kernel alone */
    double wall_ms;         /* host wall time of the call */
    int64_t h2d_bytes;      /* bytes copied host->device inside the call */
    int64_t d2h_bytes;      /* bytes copied device->host inside the call */
    int32_t kernel_launches;/* engine kernels launched by the call */
    int32_t reserved;
    int64_t exact_friction_evals;     /* MDEF: electronic friction evaluations */
    int64_t surrogate_friction_evals; /* MDEF: friction values taken from the surrogate network */
    int64_t unconverged_roots;        /* MDEF, IESH: secular roots that hit the iteration cap */
    int64_t hop_evaluations;          /* IESH: steps whose hop probabilities were evaluated in full */
    int64_t propagator_terms;         /* IESH: Chebyshev terms summed over trajectory steps */
    int64_t electronics_fp64_steps;   /* FSSH, Ehrenfest, RPSH fast paths: steps whose electronics ran in
                                         FP64 because the adiabatic gap was below gap_fp64; IESH fast
                                         path: steps with adjacent roots refined in FP64 */
    int64_t surrogate_judged;         /* MDEF with surrogate: steps where network and exact friction were compared */
    int64_t surrogate_rejected;       /* MDEF with surrogate: trajectories switched to exact friction by the judge */
    double surrogate_max_rel_error;   /* MDEF with surrogate: largest judged relative error */
    double surrogate_mean_rel_error;  /* MDEF with surrogate: mean judged relative error */
    int64_t overlap_factorizations;   /* IESH: hop tests that LU-factorized the overlap matrix (all of them
                                         on the FP64 path; on the FP32 path those that the Gram-matrix
                                         bound of the estimate did not settle) */
} nqcd_stats;

typedef struct nqcd_handle nqcd_handle;

/* ABI version (NQCD_ABI_VERSION). */
int nqcd_version(void);

/* Create an engine for one Simulation (reference: Simulation/RingPolymerSimulation
 * constructors, src/simulations.jl:12-73, with the method of
 * src/DynamicsMethods/SurfaceHoppingMethods/fssh.jl:38-45).  Allocates device
 * memory for cfg->ntraj_max trajectories. */
int nqcd_create(const nqcd_config* cfg, nqcd_handle** out);

/* Initial conditions for `ntraj` trajectories (reference: Selection /
 * sample_distribution, src/Ensembles/selections.jl:70-99, and
 * DynamicsVariables, fssh.jl:47-65).  r0, v0: (ndofs, natoms[, nbeads], ntraj).
 * sig_re/sig_im/state0 are read only for NQCD_INIT_GIVEN (else may be NULL).
 * IESH: state0 holds the occupied states (nelectrons, ntraj), 0-based and
 * distinct, the orbitals start as unit vectors on them (iesh.jl:89-97);
 * sig_re/sig_im are not read.
 * nbeads: per-trajectory bead counts for ring polymers (NULL = nbeads_max). */
int nqcd_set_initial(nqcd_handle* h, int64_t ntraj, const double* r0, const double* v0, const double* sig_re,
                     const double* sig_im, const int32_t* state0, const int32_t* nbeads);

/* Per-degree-of-freedom distribution of a DynamicalDistribution component
 * (NQCDistributions; src/Ensembles/selections.jl:24-101): a fixed value, a
 * normal distribution (PositionHarmonicWigner / VelocityHarmonicWigner are
 * normal with the harmonic Wigner widths) or a uniform distribution. */
enum nqcd_sampler_kind { NQCD_SAMPLE_FIXED = 0, NQCD_SAMPLE_NORMAL = 1, NQCD_SAMPLE_UNIFORM = 2 };

typedef struct nqcd_sampler {
    int32_t kind;     /* nqcd_sampler_kind */
    int32_t reserved;
    double a, b;      /* FIXED: value a; NORMAL: mean a, standard deviation b >= 0; UNIFORM: [a, b) */
} nqcd_sampler;

/* Initial positions and velocities sampled on the device for `ntraj`
 * trajectories (no host sampling or host-to-device copy of the ensemble):
 * position[d], velocity[d] for d < ndofs*natoms in the (ndofs, natoms)
 * column-major order of nqcd_set_initial.  Trajectory t (global index
 * traj_offset + t) draws from the Philox4x32-10 block with counter
 * (index low, index high, d, 5) for its position and (..., d, 6) for its
 * velocity and key = seed: with U(h, l) = ((h << 32 | l) >> 11) * 2^-53,
 *   NORMAL:  a + b * sqrt(-2 ln(1 - U(w0, w1))) * cos(2 pi U(w2, w3)),
 *   UNIFORM: a + (b - a) * U(w0, w1),
 * so a sharded ensemble equals the single-process one.  The electronic
 * initial state follows cfg->init_kind as in nqcd_set_initial
 * (NQCD_INIT_GIVEN is rejected: it needs host data).  Not for ring polymers
 * (NQCD_ERR_UNSUPPORTED: their beads take nqcd_set_initial).
 * NQCD_ERR_ARG on a bad sampler (unknown kind, negative width, b < a). */
int nqcd_sample_initial(nqcd_handle* h, int64_t ntraj, const nqcd_sampler* position, const nqcd_sampler* velocity,
                        uint64_t seed);

/* Same as nqcd_set_initial with r0/v0 already on the device in the engine's
 * structure-of-arrays layout [dof][trajectory] (dof = ndofs*natoms[*nbeads]). */
int nqcd_set_initial_device(nqcd_handle* h, int64_t ntraj, const double* d_r0_soa, const double* d_v0_soa,
                            const int32_t* nbeads);

/* Run the ensemble from t0 to t1 with step dt (reference: the ensemble solve,
 * src/Ensembles/run_dynamics.jl:91-97, with the method's integrator,
 * src/DynamicsMethods/IntegrationAlgorithms/bab_electronics.jl:61-91,
 * bcb_electronics.jl:53-97, verlet_with_electronics.jl:42-69 (IESH) or
 * mdef_baoab.jl:163-180 (MDEF), and hopping callbacks surface_hopping.jl:2-16,
 * iesh.jl:390-411).
 * Every run starts from the initial conditions last set.  Random numbers are
 * Philox4x32-10 keyed by `seed` with counter (trajectory, step, stream). */
int nqcd_run(nqcd_handle* h, double t0, double t1, double dt, uint64_t seed, nqcd_outputs* out,
             nqcd_stats* stats);

/* nqcd_set_initial(h, ntraj, r0, v0, NULL, NULL, NULL, NULL) followed by
 * nqcd_run(...) in one call, with the same results: the ensemble solve from
 * the initial conditions the distribution produced on the host (reference:
 * src/Ensembles/run_dynamics.jl:91-97).  For the fast spin-boson FSSH and
 * Ehrenfest kernels (NQCD_PREC_FP32 / NQCD_PREC_FP32_KAHAN, electronic
 * initial state not NQCD_INIT_GIVEN) the positions and velocities are copied
 * in chunks of trajectories while earlier chunks already integrate, so the
 * host-to-device transfer overlaps the dynamics (pinned host buffers make the
 * copies asynchronous; see nqcd_pin_host); every other configuration runs the
 * two calls in turn.  r0 and v0 may be reused when the call returns; a later
 * nqcd_run repeats the run from the same initial conditions, except after a
 * device error (NQCD_ERR_CUDA, NQCD_ERR_OOM, NQCD_ERR_TIMEOUT), which leaves
 * the handle needing nqcd_set_initial (NQCD_ERR_STATE from nqcd_run). */
int nqcd_run_host(nqcd_handle* h, int64_t ntraj, const double* r0, const double* v0, double t0, double t1, double dt,
                  uint64_t seed, nqcd_outputs* out, nqcd_stats* stats);

/* Final per-trajectory state of the last run (any pointer may be NULL):
 * r, v as in nqcd_set_initial; sig_re/sig_im (nstates, nstates, ntraj);
 * state, nhops, nfrustrated, nsteps [ntraj]; energy [ntraj][2] (initial, final
 * total energy, DynamicsOutputs.OutputTotalEnergy).
 * IESH: sig_re/sig_im receive the orbitals psi (nstates, nelectrons, ntraj)
 * and state the occupations (nelectrons, ntraj) in electron order. */
int nqcd_get_final(nqcd_handle* h, double* r, double* v, double* sig_re, double* sig_im, int32_t* state,
                   int32_t* nhops, int32_t* nfrustrated, int32_t* nsteps, double* energy);

/* Ring polymers: per-trajectory Tully model (NQCD_MODEL_TULLY1..3, host array
 * [ntraj]) for one batched launch that mixes the three models; the handle's
 * own model keeps its parameters, the others use Tully's published values.
 * Call after nqcd_set_initial.  No counterpart call in the reference, where one
 * run_dynamics call has one Simulation and so one model: it lets the ensembles
 * of several Simulations share a launch. */
int nqcd_set_trajectory_models(nqcd_handle* h, const int32_t* models);

/* MDEF: exact Fermi-weighted force and broadened friction of the model at n
 * positions (host arrays), the quantities of DiabaticMDEF's acceleration! and
 * friction! (src/DynamicsMethods/ClassicalMethods/mdef.jl:102-140), evaluated on
 * the GPU with the handle's precision.  For the 3-D adsorbate x holds heights z,
 * force the z component of the gradient and friction the tensor's zz entry
 * (its only nonzero one). */
int nqcd_mdef_evaluate(nqcd_handle* h, int64_t n, const double* x, double* force, double* friction);

/* MDEF friction surrogate on the one-dimensional model (1-64-64-1 network, BF16 weights): generate npoints
 * exact friction values at positions uniform in [x_lo, x_hi] with the engine,
 * then train the network on the GPU (BF16 tensor-core kernels, FP32 master
 * weights, Adam with the step size decaying from learning_rate to
 * learning_rate / 100 on a cosine) for `epochs` passes of minibatches of
 * `batch`.  The trained
 * network serves runs with use_friction_surrogate inside [x_lo, x_hi].  No
 * counterpart in the reference.  final_loss: mean squared error of the
 * predicted Cholesky factor sqrt(Lambda) (may be NULL). */
int nqcd_train_friction_mlp(nqcd_handle* h, double x_lo, double x_hi, int64_t npoints, int32_t epochs,
                            int32_t batch, double learning_rate, uint64_t seed, double* final_loss);

/* Surrogate network parameters as FP32, packed W1[64] b1[64] W2[64*64] b2[64]
 * W3[64] b3[1] (4353 values): get from / set into the handle (set also fixes
 * the input normalisation x -> (x - shift) * scale and the domain [lo, hi]
 * from shift_scale_lo_hi; NQCD_ERR_ARG unless shift is finite, scale > 0 and
 * lo < hi). */
#define NQCD_MLP_NPARAMS 4353
int nqcd_mlp_get(nqcd_handle* h, float* params, double* shift_scale_lo_hi);
int nqcd_mlp_set(nqcd_handle* h, const float* params, const double* shift_scale_lo_hi);

/* Loss and gradient of the surrogate on a host batch (x, target Cholesky
 * factors), with the device training kernels: for checking them against a
 * reference implementation.  grad: NQCD_MLP_NPARAMS values. */
int nqcd_mlp_loss_grad(nqcd_handle* h, int64_t n, const double* x, const double* target_L, double* loss,
                       float* grad);

/* Accepted hops of the last run, [ntraj][max_hops][3] = (step, from, to), -1 padded
 * (DynamicsOutputs.OutputSurfaceHops, src/DynamicsOutputs.jl:235-243). */
int nqcd_get_hop_log(nqcd_handle* h, int32_t* log);

/* Launch shapes of the fast kernels (no counterpart in the reference: the
 * thread/warp-per-trajectory mapping that the project's autotuner,
 * nqcd_gb300/autotune.py, picks by timing the candidates on the GPU).  Zero
 * fields keep the defaults.  Results do not depend on the mapping except
 * through the order of floating-point sums inside a trajectory. */
typedef struct nqcd_mapping {
    int32_t sb_lanes;    /* fast spin-boson kernel: lanes per trajectory, 4 or 8 (0 = 4; 8 needs
                            NQCD_PREC_FP32_KAHAN and at most 128 modes) */
    int32_t sb_block;    /* fast spin-boson kernel: threads per block, 64, 128 or 256 (0 = 128) */
    int32_t rp_lanes[4]; /* fast ring-polymer kernels: lanes per trajectory for 4, 8, 16 and 32 beads
                            (0 = 4; 4 beads: 1, 2, 4; 8: 2, 4, 8; 16: 4, 8, 16; 32: 4, 8, 16, 32) */
    int32_t iesh_cores;  /* IESH FP32 path, products of the propagator's Chebyshev terms: 0 = fifth-generation
                            tensor cores (tcgen05, the orbitals split into tf32 high and low parts) where
                            nstates is a multiple of 16 up to 80 and 2 nelectrons <= 128, else CUDA cores;
                            1 = CUDA cores (FP32 register tiles) */
    int32_t rp_one_launch; /* fast ring-polymer path: 0 = one persistent kernel per bead count, concurrent
                              on forked streams; 1 = one persistent launch serving every bead count
                              (default lane groups) with a refill over all classes */
    int32_t iesh_lu_always; /* IESH FP32 path: 0 = the LU of the overlap matrix runs only in steps where a
                               bound of the hop estimate from the Gram matrix of the occupied rows does not
                               already lie below the step's random number (the decision and the results are
                               those of the LU path); 1 = the LU every step, as iesh.jl:241 */
} nqcd_mapping;

/* Eigenvalues and eigenvectors of `batch` dense real symmetric n x n matrices
 * (host arrays; A [batch][n][n], symmetrised as (A + A^T)/2), cyclic Jacobi
 * in shared memory on the GPU, one CTA per matrix, in NQCD_PREC_FP64 or
 * NQCD_PREC_FP32: w [batch][n] ascending, Z [batch][n][n] with eigenvector o
 * of matrix b at Z[(b n + o) n + i] and its largest component positive; sweeps
 * [batch] (may be NULL) the Jacobi sweeps taken.  The general eigensolver of the
 * reference's calculators (NQCCalculators get_eigen, LAPACK) for Hamiltonians
 * without the arrowhead structure the trajectory kernels solve through the
 * secular equation.  n up to 120 (FP64) or 168 (FP32); NQCD_ERR_UNSUPPORTED
 * beyond.  Stateless: allocates and frees its device buffers. */
int nqcd_eigh_batched(int32_t precision, int32_t n, int64_t batch, const double* A, double* w, double* Z,
                      int32_t* sweeps);

/* Set the handle's launch shapes for the following runs; NQCD_ERR_ARG for a
 * shape outside the lists above, NQCD_ERR_UNSUPPORTED for 8 spin-boson lanes
 * without Kahan accumulation or with more than 128 modes. */
int nqcd_set_mapping(nqcd_handle* h, const nqcd_mapping* m);

/* Per-trajectory status of the last nqcd_run (host arrays of ntraj, NULL to
 * skip): nonfinite[t] = 1 where a final position or velocity is not finite
 * (the trajectories counted in nqcd_stats.flagged), fp64_steps[t] = steps of
 * a fast path whose electronics ran in FP64 because the adiabatic gap was
 * below gap_fp64, or (IESH) whose near-degenerate roots were refined in FP64
 * (0 on the plain path and for MDEF).  Frustrated-hop counts come from
 * nqcd_get_final. */
int nqcd_get_status(nqcd_handle* h, int32_t* nonfinite, int32_t* fp64_steps);

/* Message of the last failed call on this handle (or of the last failed
 * nqcd_create in this thread when h is NULL). */
const char* nqcd_last_error(const nqcd_handle* h);

/* Free the handle, its device memory and stream. */
void nqcd_destroy(nqcd_handle* h);

/* Page-lock caller memory for asynchronous copies (cudaHostRegister). */
int nqcd_pin_host(void* ptr, int64_t bytes);
int nqcd_unpin_host(void* ptr);

/* Measure this GPU's FP64 and FP32 CUDA-core fused multiply-add throughput
 * (TFLOP/s, 2 flops per FMA) with a register-resident FMA chain kernel. */
int nqcd_measure_fma_peaks(double* fp64_tflops, double* fp32_tflops);

/* Tensor-core self-test (no counterpart in the reference): D = A B for
 * A 128 x 80, B 80 x 80 (row-major host arrays, D 128 x 80) on the fifth-
 * generation tensor cores, kind::tf32 with the accumulator in tensor memory;
 * passes = 1 rounds A and B to tf32, passes = 3 splits each into tf32 high
 * and low parts (3xTF32, near fp32 accuracy).  The shape is the one of the
 * IESH propagator terms.  NQCD_ERR_TIMEOUT if the device wait for the
 * product gave up. */
int nqcd_tensor_selftest(int32_t passes, const float* A, const float* B, float* D);

/* Allocation-free plain FP64 spin-boson FSSH ensemble.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory while
 * they run (a Julia host whose CUDA.jl pool owns the device memory, a service
 * that reserves all its memory at start-up, code that must not allocate while
 * a stream is being captured).  It allocates nothing, on the device or the
 * host: inputs and outputs are the caller's device buffers, and the per-mode
 * coupling scratch is a fixed array of NQCD_NOALLOC_SCRATCH_DOUBLES doubles
 * (8 MiB) built into the library, held by every GPU that loads it until exit.
 *
 * Same kernel and results as nqcd_run with NQCD_METHOD_FSSH,
 * NQCD_MODEL_SPINBOSON, NQCD_PREC_FP64, NQCD_INIT_DIABATIC_PURE(diabatic_state).
 *  d_bath_c, d_bath_omega2 (omega_j^2), d_mass: device [nmodes]
 *  d_r, d_v: device [nmodes][ntraj] (trajectory fastest); initial conditions
 *            in, final positions and velocities out
 *  d_sigma: device [8][ntraj] out (re00 im00 re01 im01 re10 im10 re11 im11)
 *  d_state: device [ntraj] out; d_nhops, d_nfrustrated, d_nsteps: device
 *            [ntraj] out or NULL
 *  stream: cudaStream_t (NULL = default stream); the call only enqueues.
 * Returns NQCD_ERR_ARG (message in errbuf, if given) when nmodes * ntraj >
 * NQCD_NOALLOC_SCRATCH_DOUBLES, when t0, t1 or dt is not finite, t1 < t0,
 * dt <= 0, the run needs 2^31 - 2 steps or more, or dt is too small to advance
 * the clock.  Every call looks up the scratch array's device address in the
 * current context (cudaGetSymbolAddress, which allocates nothing); the first
 * call in a context may also load the library's device code, so make that
 * first call before any stream capture.  All calls share the scratch array,
 * so calls whose kernels overlap on the GPU race. */
#define NQCD_NOALLOC_SCRATCH_DOUBLES 1048576
int nqcd_fssh_spinboson_fp64_noalloc(int64_t ntraj, int32_t nmodes, const double* d_bath_c,
                                     const double* d_bath_omega2, const double* d_mass, double eps, double delta,
                                     int32_t rescaling, int32_t diabatic_state, double* d_r, double* d_v,
                                     double* d_sigma, int32_t* d_state, int32_t* d_nhops, int32_t* d_nfrustrated,
                                     int32_t* d_nsteps, double t0, double t1, double dt, uint64_t seed, void* stream,
                                     char* errbuf, int32_t errbuf_len);

#ifdef __cplusplus
}
#endif

#endif /* NQCD_GPU_H */
