/*
 * ngrav_oracle.c -- CPU restatement of the reference's Barnes-Hut path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  See ngrav_oracle.h for the role of
 * this file and for which reference function each entry point restates.
 * Written in plain C99 + OpenMP so it builds with gcc on both the x86 build
 * container and the aarch64 GPU host.  Arithmetic is FP64 throughout, like
 * the reference.
 */
#include "ngrav_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Tree build                                                               */
/* ------------------------------------------------------------------------ */

static int grow(void** p, size_t elem, int cap) {
    void* q = realloc(*p, elem * (size_t)cap);
    if (!q) return -1;
    *p = q;
    return 0;
}

static int ensure_capacity(or_tree* t, int need) {
    if (need <= t->cap) return 0;
    int cap = t->cap > 0 ? t->cap : 64;
    while (cap < need) cap *= 2;
    if (grow((void**)&t->cx, sizeof(double), cap) || grow((void**)&t->cy, sizeof(double), cap) ||
        grow((void**)&t->cz, sizeof(double), cap) || grow((void**)&t->half, sizeof(double), cap) ||
        grow((void**)&t->comx, sizeof(double), cap) || grow((void**)&t->comy, sizeof(double), cap) ||
        grow((void**)&t->comz, sizeof(double), cap) || grow((void**)&t->mass, sizeof(double), cap) ||
        grow((void**)&t->child, 8 * sizeof(int), cap) || grow((void**)&t->nchild, sizeof(int), cap) ||
        grow((void**)&t->parent, sizeof(int), cap) || grow((void**)&t->first, sizeof(int), cap) ||
        grow((void**)&t->count, sizeof(int), cap) || grow((void**)&t->level, sizeof(int), cap) ||
        grow((void**)&t->prefix, sizeof(unsigned long long), cap) || grow((void**)&t->head, sizeof(int), cap) ||
        grow((void**)&t->tail, sizeof(int), cap) || grow((void**)&t->bucket, sizeof(int), cap))
        return -1;
    t->cap = cap;
    return 0;
}

static void init_node(or_tree* t, int idx, int parent, double cx, double cy, double cz, double half, int level,
                      unsigned long long prefix) {
    t->cx[idx] = cx;
    t->cy[idx] = cy;
    t->cz[idx] = cz;
    t->half[idx] = half;
    t->comx[idx] = t->comy[idx] = t->comz[idx] = 0.0;
    t->mass[idx] = 0.0;
    for (int c = 0; c < 8; ++c) t->child[8 * idx + c] = -1;
    t->nchild[idx] = 0;
    t->parent[idx] = parent;
    t->first[idx] = -1;
    t->count[idx] = 0;
    t->level[idx] = level;
    t->prefix[idx] = prefix;
    t->head[idx] = t->tail[idx] = -1;
    t->bucket[idx] = 0;
}

/* OctantOf: bit 1 = x >= cx, 2 = y >= cy, 4 = z >= cz (Tree.cpp:11-20). */
static int octant_of(const or_tree* t, int nd, double px, double py, double pz) {
    int oct = 0;
    if (px >= t->cx[nd]) oct |= 1;
    if (py >= t->cy[nd]) oct |= 2;
    if (pz >= t->cz[nd]) oct |= 4;
    return oct;
}

/* NewChild: child centre = parent centre +/- half of the parent half size,
 * per axis, in FP64 (Tree.cpp:90-112). */
static int child_for(or_tree* t, int nd, int oct) {
    int ch = t->child[8 * nd + oct];
    if (ch != -1) return ch;
    if (ensure_capacity(t, t->nnodes + 1)) return -1;
    ch = t->nnodes++;
    const double h = 0.5 * t->half[nd];
    const double cx = t->cx[nd] + ((oct & 1) ? h : -h);
    const double cy = t->cy[nd] + ((oct & 2) ? h : -h);
    const double cz = t->cz[nd] + ((oct & 4) ? h : -h);
    init_node(t, ch, nd, cx, cy, cz, h, t->level[nd] + 1, (t->prefix[nd] << 3) | (unsigned long long)oct);
    t->child[8 * nd + oct] = ch;
    t->nchild[nd] += 1;
    return ch;
}

/* Running mass / centre of mass update of Insert (Tree.cpp:119-122). */
static void accumulate(or_tree* t, int nd, double px, double py, double pz, double mp) {
    const double M = t->mass[nd];
    const double newMass = M + mp;
    t->comx[nd] = (t->comx[nd] * M + px * mp) / newMass;
    t->comy[nd] = (t->comy[nd] * M + py * mp) / newMass;
    t->comz[nd] = (t->comz[nd] * M + pz * mp) / newMass;
    t->mass[nd] = newMass;
}

static void append(or_tree* t, int nd, int p) {
    t->next[p] = -1;
    if (t->tail[nd] == -1)
        t->head[nd] = p;
    else
        t->next[t->tail[nd]] = p;
    t->tail[nd] = p;
    t->bucket[nd] += 1;
}

/* Insert / InsertIntoChild (Tree.cpp:114-145), iterative.  A leaf keeps up to
 * ncrit particles (or any number at max_depth); the arrival of one more
 * splits it: its bucket is re-inserted, in stored order, into the children
 * (none of which can overflow during that redistribution), then the new
 * particle continues downwards. */
static int insert(or_tree* t, int p, const double* x, const double* y, const double* z, const double* m) {
    int nd = 0, depth = 0;
    for (;;) {
        accumulate(t, nd, x[p], y[p], z[p], m[p]);
        if (t->nchild[nd] == 0) {
            if (t->bucket[nd] < t->ncrit || depth >= t->max_depth) {
                append(t, nd, p);
                return 0;
            }
            int q = t->head[nd];
            t->head[nd] = t->tail[nd] = -1;
            t->bucket[nd] = 0;
            while (q != -1) {
                const int nq = t->next[q];
                const int ch = child_for(t, nd, octant_of(t, nd, x[q], y[q], z[q]));
                if (ch < 0) return -1;
                accumulate(t, ch, x[q], y[q], z[q], m[q]);
                append(t, ch, q);
                q = nq;
            }
        }
        const int ch = child_for(t, nd, octant_of(t, nd, x[p], y[p], z[p]));
        if (ch < 0) return -1;
        nd = ch;
        ++depth;
    }
}

int or_tree_build(or_tree* t, int n, const double* x, const double* y, const double* z, const double* m, int ncrit,
                  int max_depth) {
    memset(t, 0, sizeof(*t));
    t->n = n;
    t->ncrit = ncrit;
    t->max_depth = max_depth;
    const int reserve = (int)((long long)n * 2 / (ncrit > 1 ? ncrit : 1) + 64);
    if (ensure_capacity(t, reserve)) return -1;
    t->next = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    t->order = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!t->next || !t->order) return -1;

    /* BuildRoot (Tree.cpp:54-88): FP64 bounding box, cube centred on it,
     * half edge = the largest half extent (1.0 if degenerate) padded x1.001. */
    double lo[3], hi[3];
    if (n == 0) {
        lo[0] = lo[1] = lo[2] = 0.0;
        hi[0] = hi[1] = hi[2] = 0.0;
    } else {
        lo[0] = lo[1] = lo[2] = 1.7976931348623157e308;
        hi[0] = hi[1] = hi[2] = -1.7976931348623157e308;
        for (int i = 0; i < n; ++i) {
            const double p[3] = {x[i], y[i], z[i]};
            for (int a = 0; a < 3; ++a) {
                if (p[a] < lo[a]) lo[a] = p[a];
                if (hi[a] < p[a]) hi[a] = p[a];
            }
        }
    }
    double half = 0.5 * (hi[0] - lo[0]);
    const double hy = 0.5 * (hi[1] - lo[1]);
    const double hz = 0.5 * (hi[2] - lo[2]);
    if (half < hy) half = hy;
    if (half < hz) half = hz;
    if (!(half > 1e-12)) half = 1.0;
    t->nnodes = 1;
    init_node(t, 0, -1, 0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2]), half * 1.001, 0, 0ull);

    for (int i = 0; i < n; ++i)
        if (insert(t, i, x, y, z, m)) return -1;

    /* Finalize (Tree.cpp:147-203): DFS in ascending octant order emits each
     * leaf's bucket contiguously into `order`. */
    const int nn = t->nnodes;
    int* stack = (int*)malloc(sizeof(int) * (size_t)(8 * 64 + nn + 1));
    if (!stack) return -1;
    int sp = 0, k = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int nd = stack[--sp];
        if (t->nchild[nd] == 0) {
            t->first[nd] = k;
            for (int q = t->head[nd]; q != -1; q = t->next[q]) t->order[k++] = q;
            t->count[nd] = t->bucket[nd];
            continue;
        }
        for (int c = 7; c >= 0; --c) {
            const int ch = t->child[8 * nd + c];
            if (ch != -1) stack[sp++] = ch;
        }
    }
    free(stack);

    t->max_radius = (double*)calloc((size_t)nn, sizeof(double));
    t->subtree_count = (int*)calloc((size_t)nn, sizeof(int));
    if (!t->max_radius || !t->subtree_count) return -1;
    for (int idx = nn - 1; idx >= 0; --idx) {
        if (t->nchild[idx] == 0) t->subtree_count[idx] += t->count[idx];
        if (idx > 0) t->subtree_count[t->parent[idx]] += t->subtree_count[idx];
        if (t->mass[idx] <= 0.0) continue;
        double r = 0.0;
        if (t->nchild[idx] == 0) {
            for (int j = t->first[idx]; j < t->first[idx] + t->count[idx]; ++j) {
                const int p = t->order[j];
                const double dx = x[p] - t->comx[idx], dy = y[p] - t->comy[idx], dz = z[p] - t->comz[idx];
                const double d = sqrt(dx * dx + dy * dy + dz * dz);
                if (r < d) r = d;
            }
        } else {
            for (int c = 0; c < 8; ++c) {
                const int ch = t->child[8 * idx + c];
                if (ch == -1) continue;
                const double dx = t->comx[ch] - t->comx[idx], dy = t->comy[ch] - t->comy[idx],
                             dz = t->comz[ch] - t->comz[idx];
                const double d = t->max_radius[ch] + sqrt(dx * dx + dy * dy + dz * dz);
                if (r < d) r = d;
            }
        }
        t->max_radius[idx] = r;
    }
    return 0;
}

/* ComputeQuadrupoles (Tree.cpp:205-254): traceless Q = sum m (3 d d - d^2 I)
 * about each node's COM; leaves sum their members, internal nodes shift
 * their children's Q by the parallel-axis term.  Qzz = -(Qxx + Qyy). */
void or_tree_quadrupoles(or_tree* t, const double* x, const double* y, const double* z, const double* m) {
    const int nn = t->nnodes;
    free(t->q);
    t->q = (double*)calloc((size_t)nn * 5, sizeof(double));
    if (!t->q) return;
    for (int idx = nn - 1; idx >= 0; --idx) {
        double* Q = t->q + 5 * idx;
        if (t->mass[idx] <= 0.0) continue;
        if (t->nchild[idx] == 0) {
            const int lo = t->first[idx], hi = lo + t->count[idx];
            if (hi - lo <= 1) continue;
            for (int j = lo; j < hi; ++j) {
                const int p = t->order[j];
                const double dx = x[p] - t->comx[idx], dy = y[p] - t->comy[idx], dz = z[p] - t->comz[idx];
                const double d2 = dx * dx + dy * dy + dz * dz;
                const double mp = m[p];
                Q[0] += mp * (3.0 * dx * dx - d2);
                Q[1] += mp * (3.0 * dy * dy - d2);
                Q[2] += mp * 3.0 * dx * dy;
                Q[3] += mp * 3.0 * dx * dz;
                Q[4] += mp * 3.0 * dy * dz;
            }
            continue;
        }
        for (int c = 0; c < 8; ++c) {
            const int ch = t->child[8 * idx + c];
            if (ch == -1 || t->mass[ch] <= 0.0) continue;
            const double* C = t->q + 5 * ch;
            const double dx = t->comx[ch] - t->comx[idx], dy = t->comy[ch] - t->comy[idx],
                         dz = t->comz[ch] - t->comz[idx];
            const double d2 = dx * dx + dy * dy + dz * dz;
            const double mc = t->mass[ch];
            Q[0] += C[0] + mc * (3.0 * dx * dx - d2);
            Q[1] += C[1] + mc * (3.0 * dy * dy - d2);
            Q[2] += C[2] + mc * 3.0 * dx * dy;
            Q[3] += C[3] + mc * 3.0 * dx * dz;
            Q[4] += C[4] + mc * 3.0 * dy * dz;
        }
    }
    t->has_quad = 1;
}

void or_tree_free(or_tree* t) {
    free(t->cx); free(t->cy); free(t->cz); free(t->half);
    free(t->comx); free(t->comy); free(t->comz); free(t->mass);
    free(t->max_radius); free(t->q); free(t->child); free(t->nchild);
    free(t->parent); free(t->first); free(t->count); free(t->level);
    free(t->prefix); free(t->subtree_count); free(t->order);
    free(t->head); free(t->tail); free(t->bucket); free(t->next);
    memset(t, 0, sizeof(*t));
}

/* ------------------------------------------------------------------------ */
/* Force kernels                                                            */
/* ------------------------------------------------------------------------ */

/* Softening kind of every pair force and potential: 0 Plummer, 1 spline
 * (Softening.hpp:30-33); the spline's smoothing length is h = sqrt(eps2). */
static int g_soft = 0;
void or_set_softening(int kind) { g_soft = kind; }

/* SplineChi3D / SplinePotential3D (Softening.hpp:36-56): enclosed-mass
 * fraction and pair potential (times h / (G m)) of the cubic-spline kernel. */
static inline double spline_chi(double q) {
    if (q >= 2.0) return 1.0;
    if (q < 1.0) return q * q * q * (4.0 / 3.0 - 1.2 * q * q + 0.5 * q * q * q);
    const double t = 2.0 - q, t2 = t * t, t4 = t2 * t2;
    return 1.0 - 4.0 * (t4 / 4.0 - t4 * t / 5.0 + t4 * t2 / 24.0);
}

static inline double spline_phi(double q) {
    if (q >= 2.0) return -1.0 / q;
    if (q < 1.0) return -(1.4 - (2.0 / 3.0) * q * q + 0.3 * q * q * q * q - 0.1 * q * q * q * q * q);
    const double t = 2.0 - q, t2 = t * t, t4 = t2 * t2;
    const double F = t4 / 4.0 - t4 * t / 5.0 + t4 * t2 / 24.0;
    return -((1.0 - 4.0 * F) / q + t4 / 2.0 - t4 * t / 5.0);
}

/* AccumPairSpline (Solvers.cpp:43-63): a += G m chi(r/h) d / r^3, nothing
 * for coincident points. */
static inline void accum_pair_spline(double dx, double dy, double dz, double gm, double h, double* ax, double* ay,
                                     double* az) {
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double r = sqrt(r2);
    if (r <= 1e-300) return;
    const double s = gm * spline_chi(r / h) / (r2 * r);
    *ax += s * dx;
    *ay += s * dy;
    *az += s * dz;
}

/* AccumPairPlummer (Solvers.cpp:19-38): a += G m d / (|d|^2 + eps^2)^(3/2);
 * the spline pair when g_soft selects it (AccumPair, :65-73). */
static inline void accum_pair(double dx, double dy, double dz, double gm, double eps2, double* ax, double* ay,
                              double* az) {
    if (g_soft == 1) {
        accum_pair_spline(dx, dy, dz, gm, sqrt(eps2), ax, ay, az);
        return;
    }
    const double dist2 = dx * dx + dy * dy + dz * dz + eps2;
    const double inv = 1.0 / sqrt(dist2);
    const double inv3 = inv * inv * inv;
    const double s = gm * inv3;
    *ax += s * dx;
    *ay += s * dy;
    *az += s * dz;
}

/* AddQuadrupole (Solvers.cpp:147-179), unsoftened:
 * a += -G Q.d / r^5 + 2.5 G (d.Q.d) d / r^7, d = com - target. */
static inline void add_quadrupole(const double* Q, double dx, double dy, double dz, double dist2, double G,
                                  double* ax, double* ay, double* az) {
    const double Qxx = Q[0], Qyy = Q[1], Qzz = -(Qxx + Qyy), Qxy = Q[2], Qxz = Q[3], Qyz = Q[4];
    const double Qdx = Qxx * dx + Qxy * dy + Qxz * dz;
    const double Qdy = Qxy * dx + Qyy * dy + Qyz * dz;
    const double Qdz = Qxz * dx + Qyz * dy + Qzz * dz;
    const double Qd2 = dx * Qdx + dy * Qdy + dz * Qdz;
    const double invR2 = 1.0 / dist2;
    const double invR = sqrt(invR2);
    const double invR5 = invR2 * invR2 * invR;
    const double invR7 = invR5 * invR2;
    const double c1 = -G * invR5;
    const double c2 = 2.5 * G * Qd2 * invR7;
    *ax += c1 * Qdx + c2 * dx;
    *ay += c1 * Qdy + c2 * dy;
    *az += c1 * Qdz + c2 * dz;
}

typedef struct {
    int* far;
    int nfar, capfar;
    int* near;
    int nnear, capnear;
    int* stack;
    int capstack;
} walk_lists;

static void push_int(int** a, int* n, int* cap, int v) {
    if (*n == *cap) {
        *cap = *cap ? 2 * *cap : 256;
        *a = (int*)realloc(*a, sizeof(int) * (size_t)*cap);
    }
    (*a)[(*n)++] = v;
}

/* CollectGroupInteractions (Solvers.cpp:248-277) with an explicit stack that
 * visits children in ascending octant order, like the recursion.  Group MAC:
 * accept iff worst = |com_node - com_group| - maxRadius_group > 0 and
 * (2 half)^2 < theta^2 worst^2; leaves are always near (exact). */
static long long collect(const or_tree* t, int group, double theta2, walk_lists* L) {
    const double gx = t->comx[group], gy = t->comy[group], gz = t->comz[group];
    const double gr = t->max_radius[group];
    long long tests = 0;
    L->nfar = L->nnear = 0;
    int sp = 0;
    int* stk = L->stack;
    stk[sp++] = 0;
    while (sp > 0) {
        const int nd = stk[--sp];
        if (nd == group) continue;
        if (t->mass[nd] <= 0.0) continue;
        if (t->nchild[nd] == 0) {
            push_int(&L->near, &L->nnear, &L->capnear, nd);
            continue;
        }
        ++tests;
        const double dx = t->comx[nd] - gx, dy = t->comy[nd] - gy, dz = t->comz[nd] - gz;
        const double dist2 = dx * dx + dy * dy + dz * dz;
        const double size = 2.0 * t->half[nd];
        const double worst = sqrt(dist2) - gr;
        if (worst > 0.0 && size * size < theta2 * worst * worst) {
            push_int(&L->far, &L->nfar, &L->capfar, nd);
            continue;
        }
        for (int c = 7; c >= 0; --c) {
            const int ch = t->child[8 * nd + c];
            if (ch != -1) stk[sp++] = ch;
        }
    }
    return tests;
}

void or_bh_group(const or_tree* t, const double* x, const double* y, const double* z, const double* m, double G,
                 double eps2, double theta, double* ax, double* ay, double* az, or_counters* cnt) {
    const int nn = t->nnodes;
    const double theta2 = theta * theta;
    int* leaves = (int*)malloc(sizeof(int) * (size_t)(nn > 0 ? nn : 1));
    int nleaves = 0;
    for (int i = 0; i < nn; ++i)
        if (t->nchild[i] == 0 && t->count[i] > 0) leaves[nleaves++] = i;
    int maxlevel = 0;
    for (int i = 0; i < nn; ++i)
        if (t->level[i] > maxlevel) maxlevel = t->level[i];
    long long pairs = 0, p2c = 0, tests = 0;

#pragma omp parallel reduction(+ : pairs, p2c, tests) if (t->n > 256)
    {
        walk_lists L;
        memset(&L, 0, sizeof(L));
        L.capstack = 8 * (maxlevel + 2) + 8;
        L.stack = (int*)malloc(sizeof(int) * (size_t)L.capstack);
#pragma omp for schedule(dynamic, 32)
        for (int li = 0; li < nleaves; ++li) {
            const int g = leaves[li];
            tests += collect(t, g, theta2, &L);
            const int lo = t->first[g], hi = lo + t->count[g];
            for (int k = lo; k < hi; ++k) {
                const int i = t->order[k];
                const double xi = x[i], yi = y[i], zi = z[i];
                double axi = 0.0, ayi = 0.0, azi = 0.0;
                for (int f = 0; f < L.nfar; ++f) {
                    const int nd = L.far[f];
                    const double dx = t->comx[nd] - xi, dy = t->comy[nd] - yi, dz = t->comz[nd] - zi;
                    const double dist2 = dx * dx + dy * dy + dz * dz;
                    accum_pair(dx, dy, dz, G * t->mass[nd], eps2, &axi, &ayi, &azi);
                    if (t->has_quad) add_quadrupole(t->q + 5 * nd, dx, dy, dz, dist2, G, &axi, &ayi, &azi);
                }
                p2c += L.nfar;
                for (int l = 0; l < L.nnear; ++l) {
                    const int lf = L.near[l];
                    const int lo2 = t->first[lf], hi2 = lo2 + t->count[lf];
                    for (int k2 = lo2; k2 < hi2; ++k2) {
                        const int p = t->order[k2];
                        accum_pair(x[p] - xi, y[p] - yi, z[p] - zi, G * m[p], eps2, &axi, &ayi, &azi);
                    }
                    pairs += hi2 - lo2;
                }
                for (int k2 = lo; k2 < hi; ++k2) {
                    if (k2 == k) continue;
                    const int p = t->order[k2];
                    accum_pair(x[p] - xi, y[p] - yi, z[p] - zi, G * m[p], eps2, &axi, &ayi, &azi);
                }
                pairs += hi - lo - 1;
                ax[i] = axi;
                ay[i] = ayi;
                az[i] = azi;
            }
        }
        free(L.far);
        free(L.near);
        free(L.stack);
    }
    free(leaves);
    if (cnt) {
        cnt->p2p_pairs = pairs;
        cnt->p2c_terms = p2c;
        cnt->mac_tests = tests;
        cnt->groups = nleaves;
    }
}

int or_bh_accel(int n, const double* x, const double* y, const double* z, const double* m, double G, double eps,
                double theta, int ncrit, int quad, double* ax, double* ay, double* az, or_counters* cnt) {
    or_tree t;
    if (or_tree_build(&t, n, x, y, z, m, ncrit, 40)) {
        or_tree_free(&t);
        return -1;
    }
    if (quad) or_tree_quadrupoles(&t, x, y, z, m);
    for (int i = 0; i < n; ++i) ax[i] = ay[i] = az[i] = 0.0;
    or_bh_group(&t, x, y, z, m, G, eps * eps, theta, ax, ay, az, cnt);
    or_tree_free(&t);
    return 0;
}

/* WalkBH (Solvers.cpp:181-227): the per-particle walk.  Leaves: every member
 * but the target itself, exactly; internal nodes: accepted by the geometric
 * test (2h)^2 < theta^2 d^2, or, with the relative MAC and a previous
 * |a| > 0, by M s^2 < alpha |a_old| d^4 / G (Mac.hpp:31-42); accepted nodes
 * add the softened monopole and the unsoftened quadrupole. */
static void walk_pp(const or_tree* t, const double* x, const double* y, const double* z, const double* m, int nd,
                    int i, double G, double eps2, double theta2, int relative, double alpha, double aold,
                    double* ax, double* ay, double* az, long long* pairs, long long* p2c, long long* tests) {
    if (t->mass[nd] <= 0.0) return;
    if (t->nchild[nd] == 0) {
        const int lo = t->first[nd], hi = lo + t->count[nd];
        for (int k = lo; k < hi; ++k) {
            const int p = t->order[k];
            if (p == i) continue;
            accum_pair(x[p] - x[i], y[p] - y[i], z[p] - z[i], G * m[p], eps2, ax, ay, az);
            ++*pairs;
        }
        return;
    }
    const double dx = t->comx[nd] - x[i], dy = t->comy[nd] - y[i], dz = t->comz[nd] - z[i];
    const double dist2 = dx * dx + dy * dy + dz * dz;
    const double size = 2.0 * t->half[nd];
    ++*tests;
    int accept;
    if (relative && aold > 0.0)
        accept = (t->mass[nd] * size * size) < (alpha * aold * dist2 * dist2 / G);
    else
        accept = (size * size) < (theta2 * dist2);
    if (accept) {
        accum_pair(dx, dy, dz, G * t->mass[nd], eps2, ax, ay, az);
        if (t->has_quad) add_quadrupole(t->q + 5 * nd, dx, dy, dz, dist2, G, ax, ay, az);
        ++*p2c;
        return;
    }
    for (int c = 0; c < 8; ++c) {
        const int ch = t->child[8 * nd + c];
        if (ch != -1)
            walk_pp(t, x, y, z, m, ch, i, G, eps2, theta2, relative, alpha, aold, ax, ay, az, pairs, p2c, tests);
    }
}

/* ComputeAccelBarnesHutPerParticle (Solvers.cpp:359-382); aold may be NULL
 * (no history: every target takes the geometric test).  targets: NULL for
 * all particles, else only those i with targets[i] != 0 are computed
 * (ComputeAccelBarnesHutTargets, :384-405, geometric). */
int or_bh_pp_accel(int n, const double* x, const double* y, const double* z, const double* m, double G, double eps,
                   double theta, int ncrit, int quad, int relative, double alpha, const double* aold,
                   const unsigned char* targets, double* ax, double* ay, double* az, or_counters* cnt) {
    or_tree t;
    if (or_tree_build(&t, n, x, y, z, m, ncrit, 40)) {
        or_tree_free(&t);
        return -1;
    }
    if (quad) or_tree_quadrupoles(&t, x, y, z, m);
    long long pairs = 0, p2c = 0, tests = 0;
    const double eps2 = eps * eps, theta2 = theta * theta;
#pragma omp parallel for reduction(+ : pairs, p2c, tests) schedule(dynamic, 64) if (n > 256)
    for (int i = 0; i < n; ++i) {
        if (targets && !targets[i]) continue;
        double axi = 0.0, ayi = 0.0, azi = 0.0;
        walk_pp(&t, x, y, z, m, 0, i, G, eps2, theta2, relative, alpha, aold ? aold[i] : 0.0, &axi, &ayi, &azi, &pairs,
                &p2c, &tests);
        ax[i] = axi;
        ay[i] = ayi;
        az[i] = azi;
    }
    if (cnt) {
        cnt->p2p_pairs = pairs;
        cnt->p2c_terms = p2c;
        cnt->mac_tests = tests;
        cnt->groups = 0;
    }
    or_tree_free(&t);
    return 0;
}

#include <time.h>

static double now_ms(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

int or_bh_time_sampled(int n, const double* x, const double* y, const double* z, const double* m, double G,
                       double eps, double theta, int ncrit, int quad, int group_stride, double* out,
                       double* acc_out) {
    or_tree t;
    const double t0 = now_ms();
    if (or_tree_build(&t, n, x, y, z, m, ncrit, 40)) {
        or_tree_free(&t);
        return -1;
    }
    if (quad) or_tree_quadrupoles(&t, x, y, z, m);
    const double t1 = now_ms();
    /* Walk every group_stride-th leaf group: a leaf subset with a full tree. */
    const int nn = t.nnodes;
    int nleaves = 0;
    for (int i = 0; i < nn; ++i)
        if (t.nchild[i] == 0 && t.count[i] > 0) ++nleaves;
    double* ax = (double*)calloc((size_t)n, sizeof(double));
    double* ay = (double*)calloc((size_t)n, sizeof(double));
    double* az = (double*)calloc((size_t)n, sizeof(double));
    long long sampled = 0;
    int* groups = (int*)malloc(sizeof(int) * (size_t)(nleaves + 1));
    int ng = 0, li = 0;
    for (int i = 0; i < nn; ++i) {
        if (t.nchild[i] == 0 && t.count[i] > 0) {
            if (li % group_stride == 0) {
                groups[ng++] = i;
                sampled += t.count[i];
            }
            ++li;
        }
    }
    or_counters cnt;
    const double t2 = now_ms();
    {
        const double theta2 = theta * theta;
        const double eps2 = eps * eps;
        int maxlevel = 0;
        for (int i = 0; i < nn; ++i)
            if (t.level[i] > maxlevel) maxlevel = t.level[i];
        long long pairs = 0;
#pragma omp parallel reduction(+ : pairs)
        {
            walk_lists L;
            memset(&L, 0, sizeof(L));
            L.capstack = 8 * (maxlevel + 2) + 8;
            L.stack = (int*)malloc(sizeof(int) * (size_t)L.capstack);
#pragma omp for schedule(dynamic, 32)
            for (int gi = 0; gi < ng; ++gi) {
                const int g = groups[gi];
                collect(&t, g, theta2, &L);
                const int lo = t.first[g], hi = lo + t.count[g];
                for (int k = lo; k < hi; ++k) {
                    const int i = t.order[k];
                    const double xi = x[i], yi = y[i], zi = z[i];
                    double axi = 0.0, ayi = 0.0, azi = 0.0;
                    for (int f = 0; f < L.nfar; ++f) {
                        const int nd = L.far[f];
                        const double dx = t.comx[nd] - xi, dy = t.comy[nd] - yi, dz = t.comz[nd] - zi;
                        const double dist2 = dx * dx + dy * dy + dz * dz;
                        accum_pair(dx, dy, dz, G * t.mass[nd], eps2, &axi, &ayi, &azi);
                        if (t.has_quad) add_quadrupole(t.q + 5 * nd, dx, dy, dz, dist2, G, &axi, &ayi, &azi);
                    }
                    for (int l = 0; l < L.nnear; ++l) {
                        const int lf = L.near[l];
                        for (int k2 = t.first[lf]; k2 < t.first[lf] + t.count[lf]; ++k2) {
                            const int p = t.order[k2];
                            accum_pair(x[p] - xi, y[p] - yi, z[p] - zi, G * m[p], eps2, &axi, &ayi, &azi);
                        }
                        pairs += t.count[lf];
                    }
                    for (int k2 = lo; k2 < hi; ++k2) {
                        if (k2 == k) continue;
                        const int p = t.order[k2];
                        accum_pair(x[p] - xi, y[p] - yi, z[p] - zi, G * m[p], eps2, &axi, &ayi, &azi);
                    }
                    ax[i] = axi;
                    ay[i] = ayi;
                    az[i] = azi;
                }
            }
            free(L.far);
            free(L.near);
            free(L.stack);
        }
        cnt.p2p_pairs = pairs;
    }
    const double t3 = now_ms();
    if (acc_out) {  /* 3 x n: the sampled targets' accelerations, NaN elsewhere */
        for (int i = 0; i < n; ++i) acc_out[i] = acc_out[n + i] = acc_out[2 * (size_t)n + i] = NAN;
        for (int gi = 0; gi < ng; ++gi) {
            const int g = groups[gi];
            for (int k = t.first[g]; k < t.first[g] + t.count[g]; ++k) {
                const int i = t.order[k];
                acc_out[i] = ax[i];
                acc_out[n + i] = ay[i];
                acc_out[2 * (size_t)n + i] = az[i];
            }
        }
    }
    free(groups);
    free(ax);
    free(ay);
    free(az);
    or_tree_free(&t);
    out[0] = t1 - t0;                              /* tree build + quadrupoles, full */
    out[1] = t3 - t2;                              /* walk over the sampled groups */
    out[2] = (double)sampled / (n > 0 ? n : 1);    /* fraction of targets walked */
    out[3] = (double)cnt.p2p_pairs;
    return 0;
}

void or_direct(int n, const double* x, const double* y, const double* z, const double* m, double G, double eps2,
               double* ax, double* ay, double* az) {
#pragma omp parallel for schedule(static) if (n > 256)
    for (int i = 0; i < n; ++i) {
        const double xi = x[i], yi = y[i], zi = z[i];
        double axi = 0.0, ayi = 0.0, azi = 0.0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            accum_pair(x[j] - xi, y[j] - yi, z[j] - zi, G * m[j], eps2, &axi, &ayi, &azi);
        }
        ax[i] = axi;
        ay[i] = ayi;
        az[i] = azi;
    }
}

void or_direct_targets(int n, const double* x, const double* y, const double* z, const double* m, double G,
                       double eps2, int nt, const int* targets, double* ax, double* ay, double* az) {
#pragma omp parallel for schedule(static) if (nt > 64)
    for (int t = 0; t < nt; ++t) {
        const int i = targets[t];
        const double xi = x[i], yi = y[i], zi = z[i];
        double axi = 0.0, ayi = 0.0, azi = 0.0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            accum_pair(x[j] - xi, y[j] - yi, z[j] - zi, G * m[j], eps2, &axi, &ayi, &azi);
        }
        ax[t] = axi;
        ay[t] = ayi;
        az[t] = azi;
    }
}

/* LeapfrogStep (Integrator.cpp:9-39): half kick, drift, a(t+dt), half kick. */
int or_leapfrog(int n, double* x, double* y, double* z, double* vx, double* vy, double* vz, const double* m,
                double* ax, double* ay, double* az, double G, double eps, double theta, int ncrit, double dt,
                int nsteps, int primed) {
    if (!primed && or_bh_accel(n, x, y, z, m, G, eps, theta, ncrit, 1, ax, ay, az, NULL)) return -1;
    const double hdt = 0.5 * dt;
    for (int s = 0; s < nsteps; ++s) {
        for (int i = 0; i < n; ++i) {
            vx[i] += hdt * ax[i];
            vy[i] += hdt * ay[i];
            vz[i] += hdt * az[i];
        }
        for (int i = 0; i < n; ++i) {
            x[i] += dt * vx[i];
            y[i] += dt * vy[i];
            z[i] += dt * vz[i];
        }
        if (or_bh_accel(n, x, y, z, m, G, eps, theta, ncrit, 1, ax, ay, az, NULL)) return -1;
        for (int i = 0; i < n; ++i) {
            vx[i] += hdt * ax[i];
            vy[i] += hdt * ay[i];
            vz[i] += hdt * az[i];
        }
    }
    return 0;
}

/* One block (power-of-two rung) step: System::BlockStep
 * (include/ngrav/System.hpp:239-294).  a{x,y,z} hold a(t) on entry (primed)
 * and a(t + dt) on return; rung[i] receives each particle's rung.  The
 * refreshes use the geometric per-particle walk on the closing set
 * (ComputeAccelBarnesHutTargets, Solvers.cpp:384-405) on a tree rebuilt from
 * the drifted positions.  Returns the largest rung, or -1 on failure. */
int or_block_step(int n, double* x, double* y, double* z, double* vx, double* vy, double* vz, const double* m,
                  double* ax, double* ay, double* az, double G, double eps, double theta, int ncrit, double dt,
                  double eta, int max_rung, int* rung) {
    if (max_rung < 0) max_rung = 0;
    int rmax = 0;
    for (int i = 0; i < n; ++i) { /* System.hpp:250-262 */
        const double amag = sqrt(ax[i] * ax[i] + ay[i] * ay[i] + az[i] * az[i]);
        int k = 0;
        if (amag > 0.0 && eps > 0.0) {
            const double tau = eta * sqrt(eps / amag);
            if (tau < dt) {
                k = (int)ceil(log2(dt / tau));
                if (k > max_rung) k = max_rung;
            }
        }
        rung[i] = k;
        if (k > rmax) rmax = k;
    }
    const int nsub = 1 << rmax;
    const double dtmin = dt / nsub;
    unsigned char* act = (unsigned char*)malloc((size_t)(n > 0 ? n : 1));
    double* bx = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * 3);
    if (!act || !bx) {
        free(act);
        free(bx);
        return -1;
    }
    double* by = bx + n;
    double* bz = by + n;
    for (int sub = 0; sub < nsub; ++sub) {
        for (int i = 0; i < n; ++i) { /* opening half-kick of the rungs starting here */
            const int units = 1 << (rmax - rung[i]);
            if (sub % units == 0) {
                const double h = 0.5 * (dt / (1 << rung[i]));
                vx[i] += h * ax[i];
                vy[i] += h * ay[i];
                vz[i] += h * az[i];
            }
        }
        for (int i = 0; i < n; ++i) { /* drift everyone by the finest substep */
            x[i] += dtmin * vx[i];
            y[i] += dtmin * vy[i];
            z[i] += dtmin * vz[i];
        }
        int nact = 0;
        for (int i = 0; i < n; ++i) {
            const int units = 1 << (rmax - rung[i]);
            act[i] = (unsigned char)((sub + 1) % units == 0);
            nact += act[i];
        }
        if (nact) {
            if (or_bh_pp_accel(n, x, y, z, m, G, eps, theta, ncrit, 1, 0, 0.0, NULL, act, bx, by, bz, NULL)) {
                free(act);
                free(bx);
                return -1;
            }
            for (int i = 0; i < n; ++i) {
                if (!act[i]) continue;
                ax[i] = bx[i];
                ay[i] = by[i];
                az[i] = bz[i];
                const double h = 0.5 * (dt / (1 << rung[i]));
                vx[i] += h * ax[i];
                vy[i] += h * ay[i];
                vz[i] += h * az[i];
            }
        }
    }
    free(act);
    free(bx);
    return rmax;
}

void or_diagnostics(int n, const double* x, const double* y, const double* z, const double* vx, const double* vy,
                    const double* vz, const double* m, double G, double eps, double* out) {
    const double eps2 = eps * eps;
    double kinetic = 0.0;
    for (int i = 0; i < n; ++i) {
        const double v2 = vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i];
        kinetic += 0.5 * m[i] * v2;
    }
    double potential = 0.0;
#pragma omp parallel for reduction(+ : potential) schedule(dynamic, 32) if (n > 256)
    for (int i = 0; i < n; ++i) {
        double local = 0.0;
        for (int j = i + 1; j < n; ++j) {
            const double dx = x[j] - x[i], dy = y[j] - y[i], dz = z[j] - z[i];
            if (g_soft == 1) { /* System.hpp:140-147 */
                const double r = sqrt(dx * dx + dy * dy + dz * dz);
                const double q = r <= 1e-300 ? 0.0 : r / eps;
                local += G * m[i] * m[j] * spline_phi(q) / eps;
            } else {
                const double r2 = dx * dx + dy * dy + dz * dz + eps2;
                local -= G * m[i] * m[j] / sqrt(r2);
            }
        }
        potential += local;
    }
    out[0] = kinetic + potential;
    double tm = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
    for (int i = 0; i < n; ++i) {
        cx += m[i] * x[i];
        cy += m[i] * y[i];
        cz += m[i] * z[i];
        tm += m[i];
    }
    if (tm > 0.0) {
        cx /= tm;
        cy /= tm;
        cz /= tm;
    }
    out[1] = cx;
    out[2] = cy;
    out[3] = cz;
    double Lx = 0.0, Ly = 0.0, Lz = 0.0, px = 0.0, py = 0.0, pz = 0.0;
    for (int i = 0; i < n; ++i) {
        const double rx = x[i] - cx, ry = y[i] - cy, rz = z[i] - cz;
        Lx += m[i] * (ry * vz[i] - vy[i] * rz);
        Ly += m[i] * (rz * vx[i] - vz[i] * rx);
        Lz += m[i] * (rx * vy[i] - vx[i] * ry);
        px += m[i] * vx[i];
        py += m[i] * vy[i];
        pz += m[i] * vz[i];
    }
    out[4] = Lx;
    out[5] = Ly;
    out[6] = Lz;
    out[7] = px;
    out[8] = py;
    out[9] = pz;
}

static int cmp_double(const void* a, const void* b) {
    const double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

void or_force_error(int n, const double* x, const double* y, const double* z, const double* m, double G, double eps2,
                    int nt, const int* targets, const double* ax, const double* ay, const double* az, double* out) {
    double* rx = (double*)malloc(sizeof(double) * (size_t)(3 * nt + 1));
    double* rel = (double*)malloc(sizeof(double) * (size_t)(nt + 1));
    or_direct_targets(n, x, y, z, m, G, eps2, nt, targets, rx, rx + nt, rx + 2 * nt);
    double s2 = 0.0, mx = 0.0;
    for (int t = 0; t < nt; ++t) {
        const int i = targets[t];
        const double a0 = rx[t], a1 = rx[nt + t], a2 = rx[2 * nt + t];
        const double e0 = ax[i] - a0, e1 = ay[i] - a1, e2 = az[i] - a2;
        double ref = sqrt(a0 * a0 + a1 * a1 + a2 * a2);
        if (ref < 1e-30) ref = 1e-30;
        const double r = sqrt(e0 * e0 + e1 * e1 + e2 * e2) / ref;
        rel[t] = r;
        s2 += r * r;
        if (r > mx) mx = r;
    }
    qsort(rel, (size_t)nt, sizeof(double), cmp_double);
    out[0] = nt > 0 ? sqrt(s2 / nt) : 0.0;
    out[1] = mx;
    out[2] = nt > 0 ? ((nt & 1) ? rel[nt / 2] : 0.5 * (rel[nt / 2 - 1] + rel[nt / 2])) : 0.0;
    free(rx);
    free(rel);
}

void* or_tree_create(int n, const double* x, const double* y, const double* z, const double* m, int ncrit,
                     int max_depth, int quad, int* nnodes) {
    or_tree* t = (or_tree*)malloc(sizeof(or_tree));
    if (!t) return NULL;
    if (or_tree_build(t, n, x, y, z, m, ncrit, max_depth)) {
        or_tree_free(t);
        free(t);
        return NULL;
    }
    if (quad) or_tree_quadrupoles(t, x, y, z, m);
    *nnodes = t->nnodes;
    return t;
}

void or_tree_export(void* h, int* level, unsigned long long* prefix, int* count, int* is_leaf, double* center,
                    double* half, double* com, double* mass, double* max_radius, double* quad, int* order,
                    int* parent, int* first) {
    const or_tree* t = (const or_tree*)h;
    for (int i = 0; i < t->nnodes; ++i) {
        level[i] = t->level[i];
        prefix[i] = t->prefix[i];
        count[i] = t->subtree_count[i];
        is_leaf[i] = t->nchild[i] == 0;
        center[3 * i] = t->cx[i];
        center[3 * i + 1] = t->cy[i];
        center[3 * i + 2] = t->cz[i];
        half[i] = t->half[i];
        com[3 * i] = t->comx[i];
        com[3 * i + 1] = t->comy[i];
        com[3 * i + 2] = t->comz[i];
        mass[i] = t->mass[i];
        max_radius[i] = t->max_radius[i];
        for (int c = 0; c < 5; ++c) quad[5 * i + c] = t->q ? t->q[5 * i + c] : 0.0;
        parent[i] = t->parent[i];
        first[i] = t->first[i];
    }
    for (int k = 0; k < t->n; ++k) order[k] = t->order[k];
}

void or_tree_destroy(void* h) {
    if (!h) return;
    or_tree_free((or_tree*)h);
    free(h);
}
