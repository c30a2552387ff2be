/*
 * ngrav_oracle.h -- CPU restatement of the reference's Barnes-Hut path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: a plain-C (C99 + OpenMP)
 * restatement of the algorithm in HasanHelal429/OpenGL-Physics
 * projects/nbody_core, used by tests/ (parity), __graft_entry__.smoke() and
 * bench.py's cpu_baseline / --impl reference leg (the reference's CPU path
 * timed on the host cores).  The product library (libngrav_gpu.so) never
 * links it and never falls back to it.  Its results are pinned against the
 * reference itself, compiled from its own sources by oracle/build_ref.sh,
 * through the golden fixtures in tests/golden/.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project root).
 */
#ifndef NGRAV_ORACLE_H
#define NGRAV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Node arrays of the bucket-PR octree, numbered in creation order like
 * AdaptiveTree<3> (include/ngrav/Tree.hpp:44-63).  prefix/level give the
 * octant path of each node (3 bits per level, root = level 0, prefix 0). */
typedef struct or_tree {
    int n;           /* particles */
    int nnodes;
    int cap;         /* allocated node capacity */
    int ncrit;
    int max_depth;
    double *cx, *cy, *cz, *half;           /* geometric centre, half edge */
    double *comx, *comy, *comz, *mass;     /* running centre of mass / mass */
    double *max_radius;
    double *q;                             /* 5 per node: Qxx Qyy Qxy Qxz Qyz */
    int *child;                            /* 8 per node, -1 = empty */
    int *nchild, *parent, *first, *count;  /* first/count: leaves only */
    int *level;
    unsigned long long *prefix;
    int *subtree_count;                    /* particles under each node */
    int *order;                            /* n: leaf-ordered original indices */
    /* build-only bucket lists (linked through next[]) */
    int *head, *tail, *bucket, *next;
    int has_quad;
} or_tree;

typedef struct or_counters {
    long long p2p_pairs;   /* softened particle-particle terms */
    long long p2c_terms;   /* far-node (monopole+quadrupole) terms */
    long long mac_tests;   /* group opening tests on internal nodes */
    long long groups;      /* leaf groups walked */
} or_counters;

/* Softening of every pair force and potential after this call: 0 Plummer,
 * 1 the cubic spline with h = eps (Softening.hpp:30-33).  Process-wide. */
void or_set_softening(int kind);

/* Tree build: Tree.cpp:33-52 (ctor), :54-88 (BuildRoot), :90-145
 * (NewChild/Insert/InsertIntoChild), :147-203 (Finalize).  Returns 0 on
 * success, -1 on allocation failure. */
int or_tree_build(or_tree* t, int n, const double* x, const double* y, const double* z, const double* m,
                  int ncrit, int max_depth);
/* Tree.cpp:205-254 */
void or_tree_quadrupoles(or_tree* t, const double* x, const double* y, const double* z, const double* m);
void or_tree_free(or_tree* t);

/* Grouped Barnes-Hut walk, geometric MAC, Plummer softening:
 * Solvers.cpp:248-277 (CollectGroupInteractions), :279-355
 * (ComputeAccelBarnesHutGroup), :19-38 (AccumPairPlummer), :147-179
 * (AddQuadrupole).  Quadrupole terms are applied iff the tree has them.
 * cnt may be NULL. */
void or_bh_group(const or_tree* t, const double* x, const double* y, const double* z, const double* m,
                 double G, double eps2, double theta, double* ax, double* ay, double* az, or_counters* cnt);

/* Convenience: tree (ncrit) + quadrupoles (if quad) + grouped walk, the
 * body of the Barnes-Hut branch of System::ComputeAccel
 * (include/ngrav/System.hpp:57-66).  Returns 0 on success. */
/* Solvers.cpp:181-227, :359-405: per-particle walk, geometric or relative
 * MAC (aold: previous |a| per particle, NULL = none), optional target subset. */
int or_bh_pp_accel(int n, const double* x, const double* y, const double* z, const double* m, double G, double eps,
                   double theta, int ncrit, int quad, int relative, double alpha, const double* aold,
                   const unsigned char* targets, double* ax, double* ay, double* az, or_counters* cnt);
/* System::BlockStep (include/ngrav/System.hpp:239-294), one coarse step. */
int or_block_step(int n, double* x, double* y, double* z, double* vx, double* vy, double* vz, const double* m,
                  double* ax, double* ay, double* az, double G, double eps, double theta, int ncrit, double dt,
                  double eta, int max_rung, int* rung);
int or_bh_accel(int n, const double* x, const double* y, const double* z, const double* m, double G, double eps,
                double theta, int ncrit, int quad, double* ax, double* ay, double* az, or_counters* cnt);

/* Direct O(N^2) sum, FP64, i != j: Solvers.cpp:77-106.  Targets form:
 * Solvers.cpp:108-134 (writes ax[t], ay[t], az[t] for t = 0..nt-1). */
void or_direct(int n, const double* x, const double* y, const double* z, const double* m, double G, double eps2,
               double* ax, double* ay, double* az);
void or_direct_targets(int n, const double* x, const double* y, const double* z, const double* m, double G,
                       double eps2, int nt, const int* targets, double* ax, double* ay, double* az);

/* KDK leapfrog with the Barnes-Hut force: Integrator.cpp:9-39 with the
 * acceleration of System::ComputeAccel's BH branch at leaf capacity ncrit.
 * If primed == 0, a(t) is computed first (System::Prime, System.hpp:82-85).
 * Updates the state in place.  Returns 0 on success. */
int or_leapfrog(int n, double* x, double* y, double* z, double* vx, double* vy, double* vz, const double* m,
                double* ax, double* ay, double* az, double G, double eps, double theta, int ncrit, double dt,
                int nsteps, int primed);

/* Diagnostics: out[0] total energy with the O(N^2) Plummer potential
 * (System.hpp:119-164), out[1..3] COM (:166-175), out[4..6] angular momentum
 * about the COM (:177-193), out[7..9] linear momentum (DeckSim.cpp:147-153). */
void or_diagnostics(int n, const double* x, const double* y, const double* z, const double* vx, const double* vy,
                    const double* vz, const double* m, double G, double eps, double* out);

/* Relative force error of a candidate field against the FP64 direct sum on
 * nt target indices: out[0] rms, out[1] max, out[2] median of
 * |a - a_ref| / |a_ref| (the error measure of main.cpp:323-331). */
void or_force_error(int n, const double* x, const double* y, const double* z, const double* m, double G, double eps2,
                    int nt, const int* targets, const double* ax, const double* ay, const double* az, double* out);

/* Handle-based tree access for language bindings: build (+ quadrupoles if
 * quad), then export the node arrays in creation order in the same layout as
 * oracle/ref_driver.cpp's ref_tree_export.  Returns NULL on failure. */
void* or_tree_create(int n, const double* x, const double* y, const double* z, const double* m, int ncrit,
                     int max_depth, int quad, int* nnodes);
void or_tree_export(void* h, int* level, unsigned long long* prefix, int* count, int* is_leaf, double* center,
                    double* half, double* com, double* mass, double* max_radius, double* quad, int* order,
                    int* parent, int* first);
void or_tree_destroy(void* h);

/* Bounded-time CPU baseline: full tree build (+ quadrupoles) and the grouped
 * walk over every group_stride-th leaf group only.  out[0] build ms, out[1]
 * walk ms, out[2] fraction of particles walked, out[3] P2P pairs walked.
 * A full step's time extrapolates as out[0] + out[1] / out[2].  acc_out
 * (3 x n, or NULL): ax, ay, az of the walked targets, NaN for the others. */
int or_bh_time_sampled(int n, const double* x, const double* y, const double* z, const double* m, double G,
                       double eps, double theta, int ncrit, int quad, int group_stride, double* out,
                       double* acc_out);

/* Number of OpenMP threads the oracle will use. */
int or_num_threads(void);

#ifdef __cplusplus
}
#endif

#endif
