/*
 * ngrav_gpu.h -- C-ABI of the GB300 Barnes-Hut force evaluation and KDK step.
 *
 * A drop-in replacement for the force/step path of HasanHelal429/OpenGL-Physics
 * projects/nbody_core.  Every entry point is extern "C", takes plain pointers
 * and sizes, never throws, and returns an int status (NGRAV_OK == 0);
 * ngrav_gpu_last_error() gives the text of the last failure on a context.
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   System<3>::SetParticles          include/ngrav/System.hpp:29-35   -> ngrav_gpu_set_particles
 *   System<3>::ComputeAccel (BH)     include/ngrav/System.hpp:43-66   -> ngrav_gpu_compute_accel
 *   ComputeAccelBarnesHut(v, sp, out) include/ngrav/Solvers.hpp:56-57 -> ngrav_gpu_compute_accel
 *   AccelFn<3> adapter               include/ngrav/Integrator.hpp:13-14 -> ngrav_gpu_compute_accel
 *   System<3>::Prime                 include/ngrav/System.hpp:82-85   -> ngrav_gpu_prime
 *   System<3>::Step / LeapfrogStep   include/ngrav/System.hpp:89-108, src/Integrator.cpp:9-39
 *                                                                      -> ngrav_gpu_step
 *   System<3>::State                 include/ngrav/System.hpp:194     -> ngrav_gpu_get_state
 *   System<3>::TotalEnergy / CenterOfMass / AngularMomentum, the momentum
 *     sum of DeckSim::Snapshot       include/ngrav/System.hpp:119-193, src/DeckSim.cpp:132-153
 *                                                                      -> ngrav_gpu_diagnostics
 *   GpuBarnesHutStats                include/ngrav/gpu/GpuBarnesHut.hpp:23-31 -> ngrav_gpu_get_stats
 *   AdaptiveTree<3> node arrays      include/ngrav/Tree.hpp:44-63      -> ngrav_gpu_debug_tree
 *   the force-error measure of --bench  projects/02_nbody_gravity/src/main.cpp:313-331
 *                                                                      -> ngrav_gpu_force_error
 *
 * Threading: one context per host thread.  Calls are synchronous: every
 * entry point has finished its GPU work when it returns.
 */
#ifndef NGRAV_GPU_H
#define NGRAV_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NGRAV_GPU_ABI_VERSION 1

/* Status codes. */
enum {
    NGRAV_OK = 0,
    NGRAV_ERR_INVALID_ARG = 1,   /* bad pointer, size or option */
    NGRAV_ERR_CUDA = 2,          /* a CUDA runtime call failed */
    NGRAV_ERR_NO_PARTICLES = 3,  /* no particle set on the context */
    NGRAV_ERR_CAPACITY = 4,      /* node pool or walk stack overflow that could not be grown */
    NGRAV_ERR_NONFINITE = 5,     /* NaN/Inf in positions or masses */
    NGRAV_ERR_OOM = 6,           /* device allocation failed */
    NGRAV_ERR_TIMEOUT = 7,       /* a bounded device wait ran out */
    NGRAV_ERR_DEPTH = 8          /* strict_depth set and a leaf needs more than 21 levels */
};

/* Softening kernel (include/ngrav/Softening.hpp:30-33): Plummer with length
 * eps, or the Hernquist & Katz cubic spline with smoothing length h = eps
 * (exactly Newtonian beyond 2 eps). */
enum { NGRAV_SOFTENING_PLUMMER = 0, NGRAV_SOFTENING_SPLINE = 1 };

/* Multipole acceptance criterion (include/ngrav/Mac.hpp:8-11).  GEOMETRIC:
 * the grouped walk with the group opening test; RELATIVE: the per-particle
 * walk with the GADGET-2 test M s^2 < alpha |a_old| d^4 / G (geometric for a
 * particle without a previous |a|), alpha from ngrav_gpu_set_mac_alpha;
 * LEARNED: the grouped walk with the learned test (below). */
enum { NGRAV_MAC_GEOMETRIC = 0, NGRAV_MAC_LEARNED = 1, NGRAV_MAC_RELATIVE = 2 };

/* Precision of the particle state and of the force sums.
 * PLAIN: FP32 absolute positions, plain FP32 accumulation.
 * SPLIT: positions kept as double-float (hi + lo) pairs, force evaluation on
 *        FP32 offsets from each leaf cell's centre, Kahan-compensated
 *        per-target accumulators. */
enum { NGRAV_PRECISION_PLAIN = 0, NGRAV_PRECISION_SPLIT = 1 };

typedef struct ngrav_gpu_opts {
    int abi_version;       /* NGRAV_GPU_ABI_VERSION */
    int device;            /* CUDA device ordinal */
    int leaf_capacity;     /* ncrit: a leaf splits when it would hold more (Tree.hpp:38; default 8) */
    int max_depth;         /* maxDepth of AdaptiveTree (default 40); keys resolve 21 levels */
    int quadrupole;        /* 1: monopole + quadrupole far field (the System path), 0: monopole */
    int mac;               /* NGRAV_MAC_* */
    int precision;         /* NGRAV_PRECISION_* */
    int fp64_mac_retest;   /* 1: re-decide borderline FP32 opening tests in FP64 */
    int strict_depth;      /* 1: a leaf deeper than 21 levels is an error, 0: counted in stats */
    int timing;            /* 1: record per-phase CUDA-event times in ngrav_gpu_stats */
    double G;              /* gravitational constant (StepParams::G) */
    double eps;            /* Plummer softening length (Softening::eps) */
    double theta;          /* opening angle (MacParams::theta) */
} ngrav_gpu_opts;

typedef struct ngrav_gpu_diag {
    double kinetic;        /* sum 1/2 m v^2 */
    double potential;      /* pair potential sum (exact O(N^2) FP64, or tree estimate) */
    double energy;         /* kinetic + potential (System::TotalEnergy) */
    double com[3];         /* centre of mass */
    double L[3];           /* angular momentum about the COM */
    double P[3];           /* linear momentum */
    int potential_exact;   /* 1: exact pairwise sum in FP64; 2: exact pair set, FP32 pair terms; 0: none (NaN) */
} ngrav_gpu_diag;

typedef struct ngrav_gpu_ferr {
    double rms;            /* rms of |a - a_ref| / |a_ref| over the sampled targets */
    double max;
    double median;
    double mean;           /* the --bench error column (main.cpp:323-331) */
    int nsample;
} ngrav_gpu_ferr;

typedef struct ngrav_gpu_stats {
    /* last force evaluation (milliseconds; 0 unless opts.timing) */
    double ms_bbox_keys, ms_sort, ms_build, ms_moments, ms_walk, ms_force, ms_total;
    /* interaction counts of the last force evaluation (device counters) */
    long long p2p_pairs;   /* softened particle-particle terms (self excluded) */
    long long p2c_terms;   /* far-node terms */
    long long mac_tests;   /* opening tests on internal nodes */
    long long mac_retests; /* borderline tests re-decided in FP64 */
    long long groups;      /* target groups (leaves) walked */
    int nodes, leaves, levels, max_leaf_count;
    int depth_limited_leaves; /* leaves at the 21-level key limit holding > leaf_capacity */
    int walk_stack_max;
    unsigned status_bits;  /* raw device status word of the last evaluation */
    long long force_evals; /* force evaluations since the context was created */
    long long n;
    /* cumulative since ngrav_gpu_reset_cumulative (CUDA-event times on the
     * context's stream; the per-phase ones need opts.timing) */
    long long cum_evals;
    long long cum_p2p_pairs, cum_p2c_terms;
    double cum_ms_walk;    /* tree walk kernel (opening tests, interaction lists) */
    double cum_ms_force;   /* evaluation kernel (P2P + P2C + closing kick) */
    double cum_ms_eval;    /* whole force evaluations */
    double cum_ms_step;    /* ngrav_gpu_step calls, first to last kernel */
    long long cum_launches; /* kernels this context launched */
    /* interaction lists of the last evaluation */
    long long far_entries, near_entries;
    int list_max;          /* longest per-group list */
    /* learned opening test, last evaluation: pairs handed to the network,
     * accepted by it, decided by the geometric fallback (low confidence);
     * tensor-core flushes; band pairs the error bound accepted unasked; whether it ran, whether the run reverted to the
     * geometric test, checks made and the last checked rms error */
    long long lmac_queries, lmac_accepts, lmac_fallbacks, lmac_flushes, lmac_screened;
    int lmac_active, lmac_reverted, lmac_checks;
    double lmac_last_check_rms;
    /* KDK steps launched as a captured CUDA graph: captures made, replays */
    long long graph_captures, graph_replays;
    /* System::ParticleEvals (include/ngrav/System.hpp:115): accelerations
     * computed, all particles per evaluation, the closing set per block-step
     * substep; cumulative */
    long long cum_particle_evals;
    /* radix-sort passes of the last evaluation: the keys are sorted one
     * level below the last tree's depth, in whole 9-bit passes (7 = the full
     * 63-bit key) */
    int sort_passes;
} ngrav_gpu_stats;

typedef struct ngrav_gpu_ctx ngrav_gpu_ctx;

/* Fill opts with the reference defaults: leaf_capacity 8, max_depth 40,
 * quadrupole on, geometric MAC, theta 0.5, G 1, eps 0.05 (StepParams,
 * include/ngrav/Solvers.hpp:22-27), split precision, FP64 retest on. */
int ngrav_gpu_default_opts(ngrav_gpu_opts* opts);

int ngrav_gpu_create(ngrav_gpu_ctx** ctx, const ngrav_gpu_opts* opts);
void ngrav_gpu_destroy(ngrav_gpu_ctx* ctx);
const char* ngrav_gpu_last_error(const ngrav_gpu_ctx* ctx);

/* Change G, eps, theta, leaf capacity, MAC or precision between calls. */
int ngrav_gpu_set_opts(ngrav_gpu_ctx* ctx, const ngrav_gpu_opts* opts);

/* Copy a particle set in (the caller keeps its arrays).  FP64 in, so the
 * SoA<3> layout maps 1:1; positions are held as double-float pairs in SPLIT
 * precision and rounded to FP32 in PLAIN.  Velocities and masses are FP32 on
 * the device.  vx/vy/vz may be NULL (zero velocity).  Resets acceleration
 * and the primed flag, as System::SetParticles does. */
int ngrav_gpu_set_particles(ngrav_gpu_ctx* ctx, int64_t n, const double* x, const double* y, const double* z,
                            const double* vx, const double* vy, const double* vz, const double* m);
/* FP32 variant: no conversion, for large N. */
int ngrav_gpu_set_particles_f32(ngrav_gpu_ctx* ctx, int64_t n, const float* x, const float* y, const float* z,
                                const float* vx, const float* vy, const float* vz, const float* m);

/* ChooseAdaptiveDt (src/Integrator.cpp:41-59): dt = eta min_i sqrt(eps / |a_i|)
 * from the current accelerations, clamped to [dt_max / 4096, dt_max]; dt_max
 * when no particle accelerates or eps = 0.  Primes first if needed.  Take the
 * step with ngrav_gpu_step(ctx, 1, *dt). */
int ngrav_gpu_adaptive_dt(ngrav_gpu_ctx* ctx, double eta, double dt_max, double* dt);

/* One coarse step of length dt with power-of-two rung timesteps
 * (System::BlockStep, include/ngrav/System.hpp:239-294): each particle's rung
 * k = min(max_rung, ceil(log2(dt / tau))), tau = eta sqrt(eps / |a|), from its
 * current acceleration; KDK per rung over 2^rung_max finest substeps, the
 * force refreshed after every substep for the particles whose step ends there
 * (geometric per-particle walk, ComputeAccelBarnesHutTargets) on a tree
 * rebuilt from the drifted positions.  Every particle ends the step with a
 * fresh acceleration.  rung_max: the largest rung used. */
int ngrav_gpu_block_step(ngrav_gpu_ctx* ctx, double dt, double eta, int max_rung, int* rung_max);

/* The frame fields of DeckSim::Snapshot (src/DeckSim.cpp:112-127): pos and
 * vel as N x 3 FP32 rows in input order, each component the FP64 state value
 * rounded once to FP32 (24 bytes per particle cross the bus instead of the 48
 * of ngrav_gpu_get_state).  Either pointer may be NULL. */
int ngrav_gpu_get_frame_f32(ngrav_gpu_ctx* ctx, float* pos, float* vel);

/* System::Rungs (include/ngrav/System.hpp:203-205): each particle's rung
 * from the last block step, in input order (all zero before any). */
int ngrav_gpu_get_rungs(ngrav_gpu_ctx* ctx, int* rung);

/* MacParams::alpha of the relative test (include/ngrav/Mac.hpp:18-22;
 * default 0.001). */
int ngrav_gpu_set_mac_alpha(ngrav_gpu_ctx* ctx, double alpha);

/* Softening of every pair force, far-field monopole and potential
 * (Softening::Plummer / Softening::Spline, include/ngrav/Softening.hpp:120-140);
 * the quadrupole term stays unsoftened, as in AddQuadrupole. */
int ngrav_gpu_set_softening(ngrav_gpu_ctx* ctx, int kind);

/* New positions (and velocities, unless NULL) for the particles already set,
 * in the caller's order; masses stay, and so do the accelerations of the last
 * evaluation (the next KDK step's opening kick and the learned test's
 * per-group scale use them).  Writes through System<3>::MutableState
 * (include/ngrav/System.hpp:197) on an unchanged particle set. */
int ngrav_gpu_set_state(ngrav_gpu_ctx* ctx, const double* x, const double* y, const double* z, const double* vx,
                        const double* vy, const double* vz);
int ngrav_gpu_set_state_f32(ngrav_gpu_ctx* ctx, const float* x, const float* y, const float* z, const float* vx,
                            const float* vy, const float* vz);

/* One force evaluation on the current positions, written in the caller's
 * original particle order, G included -- the contract of
 * ComputeAccelBarnesHut(pts, sp, out).  Does not advance or prime the state. */
int ngrav_gpu_compute_accel(ngrav_gpu_ctx* ctx, double* ax, double* ay, double* az);

/* a(t) for the first half-kick (System::Prime). */
int ngrav_gpu_prime(ngrav_gpu_ctx* ctx);

/* nsteps kick-drift-kick steps of length dt, device resident (primes first
 * if needed).  Equivalent to nsteps calls of System::Step with the fixed
 * global scheme. */
int ngrav_gpu_step(ngrav_gpu_ctx* ctx, int nsteps, double dt);

/* Read the state back in original particle order.  Any pointer may be NULL. */
int ngrav_gpu_get_state(ngrav_gpu_ctx* ctx, double* x, double* y, double* z, double* vx, double* vy, double* vz);
int ngrav_gpu_get_accel(ngrav_gpu_ctx* ctx, double* ax, double* ay, double* az);

/* FP64 conservation diagnostics of the current state.  exact_potential:
 * 1 = exact O(N^2) pairwise potential on the GPU, every pair term in FP64;
 * 2 = the same pair set with FP32 pair terms and FP64 sums (the offset of a
 *     pair formed from the double-float positions, so its error is of order
 *     2^-24 of the separation; Plummer softening, a spline run takes mode 1),
 *     about 2.5 s at n = 4,194,304 where mode 1 takes minutes;
 * 0 = mode 1 up to 262,144 particles, else no potential (NaN).
 * out->potential_exact reports the mode used (0, 1 or 2). */
int ngrav_gpu_diagnostics(ngrav_gpu_ctx* ctx, int exact_potential, ngrav_gpu_diag* out);

/* rms / max / median relative error of the current accelerations against a
 * direct sum with FP64 accumulation over nsample uniformly drawn targets
 * (seeded; nsample <= n).  fp64_pairs = 1 evaluates every pair term in FP64,
 * 0 evaluates pair terms in FP32 and accumulates in FP64. */
int ngrav_gpu_force_error(ngrav_gpu_ctx* ctx, int nsample, uint64_t seed, int fp64_pairs, ngrav_gpu_ferr* out);

int ngrav_gpu_get_stats(ngrav_gpu_ctx* ctx, ngrav_gpu_stats* out);
/* Zero the cum_* fields of ngrav_gpu_stats.  (No reference counterpart:
 * measurement support.) */
int ngrav_gpu_reset_cumulative(ngrav_gpu_ctx* ctx);

/* Measured FP32 FMA throughput of the device in TFLOP/s (2 flops per FMA),
 * from a register-resident FMA-chain kernel timed with CUDA events.  The
 * denominator of the P2P roofline.  (No reference counterpart: measurement
 * support.) */
int ngrav_gpu_probe_fp32_peak(int device, double* tflops);

/* Largest n ngrav_gpu_diagnostics_noalloc accepts: its block partials live in
 * a fixed 256 KiB device array (4,096 blocks of 4,096 particles). */
#define NGRAV_NOALLOC_MAX_N 16777216

/* The conservation diagnostics of ngrav_gpu_diagnostics for callers that
 * cannot allocate device memory -- e.g. a loop running under a framework's
 * caching allocator that owns the device's memory, or one that must keep
 * cudaMalloc/cudaFree (and cudaFree's device-wide synchronisation) out of
 * its frame loop.  No reference counterpart.
 *   x..m        caller-owned DEVICE arrays of n FP32 values on `device`
 *   with_potential  1: also the exact O(N^2) FP64 Plummer pair potential
 *               (G, eps; Plummer softening only, whatever softening a context
 *               uses).  It costs n^2/2 FP64 pair terms: about 1 s at
 *               n = 262,144 on one GB300, above an hour at the maximum n.
 *               0: potential and energy are NaN, as in ngrav_gpu_diagnostics.
 *   out         HOST struct, filled like ngrav_gpu_diagnostics fills it
 * Allocates nothing: its scratch is a static 256 KiB device array that every
 * GPU loading this library holds until exit.  The first call on a device
 * looks that array's address up (so make it before any stream capture).
 * Calls share the array, so calls overlapping on the GPU race; serialise
 * them.  Runs on the legacy default stream of `device` and returns when
 * done, with the caller's current device restored.
 * Returns NGRAV_ERR_INVALID_ARG for n > NGRAV_NOALLOC_MAX_N. */
int ngrav_gpu_diagnostics_noalloc(int device, int64_t n, const float* x, const float* y, const float* z,
                                  const float* vx, const float* vy, const float* vz, const float* m, double G,
                                  double eps, int with_potential, ngrav_gpu_diag* out);

/* Testing support for the capacity-recovery paths (no reference
 * counterpart; the reference's GPU path fails silently when its pools run
 * out, src/gpu/GpuBarnesHut.cpp:259-260, :428).  Replaces each pool whose
 * size is > 0 by one of exactly that size: node records, far and near
 * interaction-list chunks (128 entries each), and the learned walk's
 * deferred-pair chunks (the size its pools start at from then on).  The
 * next evaluation then overflows, detects it on the device, grows the pool
 * and re-runs; results equal those of a context that never shrank. */
int ngrav_gpu_debug_shrink_pools(ngrav_gpu_ctx* ctx, int node_cap, int far_chunks, int near_chunks,
                                 int pend_chunks);

/* Export the last tree for bit-exact checks.  Call with node arrays NULL to
 * get *nnodes; then call again with arrays of that size.
 *   keys[n]        63-bit octant-path key of each particle (original order)
 *   order[n]       leaf-ordered original indices, ascending within a leaf
 *                  (AdaptiveTree::order)
 *   level, prefix  depth and octant path (3 bits per level) of each node
 *   count          particles under each node; is_leaf
 *   center[3*nn], half, com[3*nn], mass, max_radius, quad[5*nn] (Qxx Qyy Qxy Qxz Qyz)
 * Node numbering is the GPU's own; compare in (level, prefix) order. */
/* ---- autotuner ------------------------------------------------------------
 * No reference counterpart.  Times force evaluations of the current state
 * over candidate leaf capacities (= target-group sizes: every leaf is one
 * group), P2P batch tiles (sources staged per near batch) and walk stack
 * depths (per-warp shared-memory entries), keeps the fastest candidate whose
 * rms force error (FP64-summed direct sum on check_targets samples) stays
 * within rms_tolerance x that of the starting configuration, and installs
 * it.  The state is not advanced. */
typedef struct ngrav_gpu_tune_opts {
    int reps;                  /* timed evaluations per candidate */
    int check_targets;         /* targets of each error check */
    double rms_tolerance;      /* admissible rms error / starting rms error */
    int leaf_capacities[8];    /* candidates, 0-terminated; all 0: 8, 12, 16, 24, 32, 48 */
} ngrav_gpu_tune_opts;

typedef struct ngrav_gpu_tune_report {
    int leaf_capacity, p2p_tile, walk_stack;   /* chosen */
    double ms_before, ms_after;                /* force evaluation, device time */
    double rms_before, rms_after;
    int ntried;
    double tried[32][5];                       /* leaf capacity, tile, stack, ms, rms (-1: not checked) */
} ngrav_gpu_tune_report;

int ngrav_gpu_default_tune_opts(ngrav_gpu_tune_opts* o);
int ngrav_gpu_autotune(ngrav_gpu_ctx* ctx, const ngrav_gpu_tune_opts* o, ngrav_gpu_tune_report* out);
/* Set the tuned kernel shapes directly: p2p_tile in {64, 128, 256} (0: 256),
 * walk_stack in {1024, 2048, 4096}. */
int ngrav_gpu_set_tuning(ngrav_gpu_ctx* ctx, int p2p_tile, int walk_stack);

/* ---- ensembles of independent systems ------------------------------------
 * No reference counterpart (the reference runs one System<3> per process).
 * After ngrav_gpu_set_particles with the particles of nsys systems stored one
 * system after another, system s occupying [offsets[s], offsets[s+1]), every
 * system gets its own root cube and tree (System<3> semantics per system:
 * no force between systems) and all systems advance together, one launch
 * per phase.  nsys = 1 (or a new set_particles) returns to one system.
 * Systems share G, eps, theta, leaf capacity and dt. */
int ngrav_gpu_set_ensemble(ngrav_gpu_ctx* ctx, int nsys, const int64_t* offsets);
/* rms[s] / max[s]: relative force error of system s against the direct sum
 * over its own particles (FP32 pairs, FP64 sums) on targets_per_system
 * sampled members. */
int ngrav_gpu_ensemble_force_error(ngrav_gpu_ctx* ctx, int targets_per_system, uint64_t seed, double* rms,
                                   double* max);
/* FP64 diagnostics per system (out[nsys]); the potential is the exact pair
 * sum when exact_potential, NaN otherwise. */
int ngrav_gpu_ensemble_diagnostics(ngrav_gpu_ctx* ctx, int exact_potential, ngrav_gpu_diag* out);

/* ---- learned opening test (NGRAV_MAC_LEARNED) --------------------------
 * No reference counterpart: it replaces the geometric test of
 * include/ngrav/Mac.hpp:25-29 / src/Solvers.cpp:261-271 inside the grouped
 * walk.  A network of 8 features -> 32 -> 32 -> 1 predicts whether a node's
 * multipole keeps every member of the target group within the per-target
 * error budget; it is trained on the GPU (ngrav_gpu_lmac_train) on pairs
 * the method labels itself, evaluated in BF16 on the tensor cores inside the
 * walk, backed by the geometric test where it is not confident, and checked
 * every check_every evaluations against the FP64 direct sum on
 * check_targets samples: above revert_rms the run reverts to the geometric
 * test for good. */
#define NGRAV_LMAC_PARAMS 1377  /* W1[32][8], b1[32], W2[32][32], b2[32], w3[32], b3 */
#define NGRAV_LMAC_FEATURES 8

typedef struct ngrav_gpu_lmac_opts {
    double budget;         /* per-target error budget of one accepted node */
    double gate;           /* |logit| below which the geometric test decides */
    double rho_lo, rho_hi; /* 2h/worst at or below rho_lo: accept; at or above rho_hi: open */
    int check_every;       /* evaluations between FP64 checks (0: never) */
    int check_targets;     /* sampled targets of one check */
    double revert_rms;     /* rms relative force error that triggers the revert */
    int rounds;            /* walk rounds, 2..8: pairs for the network are decided between
                            * rounds; the last round accepts the screened ones and decides
                            * the rest geometrically */
    double screen;         /* accept a band pair without the network when the quadrupole
                            * truncation bound on its error is at most screen x budget x
                            * the group's smallest |a| (0: every band pair goes to the
                            * network); the bound is loose by orders of magnitude, hence
                            * the default 1000 */
} ngrav_gpu_lmac_opts;

typedef struct ngrav_gpu_lmac_train_opts {
    int snapshots;         /* states the training pairs are drawn from */
    int steps_between;     /* KDK steps (geometric test) between snapshots */
    double dt;             /* their step; 0 keeps the state fixed */
    long long pairs;       /* labelled (group, node) pairs in total */
    double theta_record;   /* geometric test of the recording walk */
    double u_range;        /* budgets drawn at r * 2^U(-u_range, u_range) */
    int epochs;            /* passes over the training pairs */
    int batch;             /* mini-batch size (multiple of 128) */
    double lr;             /* Adam step size */
    uint64_t seed;
} ngrav_gpu_lmac_train_opts;

typedef struct ngrav_gpu_lmac_report {
    long long pairs;       /* labelled pairs kept (training + held out) */
    long long band_pairs;  /* band pairs the recording walks met */
    double loss_first, loss_last, acc_last;  /* training BCE and accuracy */
    double val_loss, val_acc;                /* held-out pairs */
    double ms_data, ms_train;
} ngrav_gpu_lmac_report;

int ngrav_gpu_lmac_default_opts(ngrav_gpu_lmac_opts* o);
int ngrav_gpu_lmac_set_opts(ngrav_gpu_ctx* ctx, const ngrav_gpu_lmac_opts* o);
int ngrav_gpu_lmac_default_train_opts(ngrav_gpu_lmac_train_opts* o);
/* Generate pairs on the current system (advancing it between snapshots with
 * the geometric test), train from a fresh initialisation and install the
 * model.  The system's state afterwards is the last snapshot's. */
int ngrav_gpu_lmac_train(ngrav_gpu_ctx* ctx, const ngrav_gpu_lmac_train_opts* o, ngrav_gpu_lmac_report* out);
/* FP32 parameters (NGRAV_LMAC_PARAMS) and the feature standardisation
 * (mu[8], 1/sd[8]). */
int ngrav_gpu_lmac_get_model(ngrav_gpu_ctx* ctx, float* params, float* norm);
int ngrav_gpu_lmac_set_model(ngrav_gpu_ctx* ctx, const float* params, const float* norm);
/* Clear the revert flag (the next learned evaluation uses the network again). */
int ngrav_gpu_lmac_reset(ngrav_gpu_ctx* ctx);
/* Inspection: pairs of the current tree met in the band by a recording walk
 * at theta_record, each kept with probability keep; their group leaf and node
 * ids (numbering of ngrav_gpu_debug_tree), unit-budget features and measured
 * worst relative multipole error r (-1: group too large to label). */
int ngrav_gpu_lmac_collect(ngrav_gpu_ctx* ctx, double theta_record, double rho_lo, double rho_hi, double keep,
                           uint64_t seed, int cap, int* npairs, long long* nband, int* group_leaf, int* node,
                           float* features, float* r);
/* Network outputs: FP32 on standardised features (the training forward
 * pass), or BF16 on the tensor cores from raw features (the walk's path). */
int ngrav_gpu_lmac_forward(ngrav_gpu_ctx* ctx, const float* x_std, int n, float* z);
int ngrav_gpu_lmac_forward_tc(ngrav_gpu_ctx* ctx, const float* x_raw, int n, float* z);
/* Gradient of scale * sum_k w_k BCE(z_k, y_k) at `params` (NULL: the
 * installed model) on standardised features; loss = sum_k w_k BCE. */
int ngrav_gpu_lmac_grad(ngrav_gpu_ctx* ctx, const float* x_std, const float* y, const float* w, int n,
                        const float* params, double scale, float* grad, double* loss);

int ngrav_gpu_debug_tree(ngrav_gpu_ctx* ctx, int* nnodes, uint64_t* keys, int* order, int* level, uint64_t* prefix,
                         int* count, int* is_leaf, double* center, double* half, double* com, double* mass,
                         double* max_radius, double* quad);

#ifdef __cplusplus
}
#endif

#endif /* NGRAV_GPU_H */
