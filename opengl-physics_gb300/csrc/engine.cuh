// engine.cuh -- device data layout and kernel launchers of the GB300
// Barnes-Hut engine (internal; the public surface is include/ngrav_gpu.h).
//
// Layout in HBM (all particle arrays in the current tree order, i.e. sorted
// by 63-bit octant-path key; `id` maps a slot back to the caller's index):
//   pos   float4 (x_hi, y_hi, z_hi, m)     the state (FP32, or the high half)
//   plo   float4 (x_lo, y_lo, z_lo, 0)     low half of double-float positions (SPLIT)
//   vel   float4 (vx, vy, vz, 0)
//   acc   float4 (ax, ay, az, 0)           G included
//   src   float4 (ox, oy, oz, m)           walk input: offset from the own leaf's
//                                           centre (SPLIT) or absolute (PLAIN)
//   id    int
// Nodes (one record per node, breadth-first by level; children of a node are
// contiguous and in ascending octant order):
//   start/count/first_child/parent/level/nchild, centre (FP64), FP64 moments,
//   and four float4 walk records (see NodeWalk below).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ngrav {

constexpr int kKeyLevels = 21;          // 63-bit keys: 3 bits per level
constexpr int kRsDigitBits = 9;         // radix sort digit: 7 passes over the 63-bit keys
constexpr int kRsBins = 1 << kRsDigitBits;
constexpr int kRsPasses = (3 * kKeyLevels + kRsDigitBits - 1) / kRsDigitBits;
constexpr int kMaxLevels = kKeyLevels + 1;

// Device status word bits (sticky within one force evaluation).
enum : unsigned {
    kStNodeOverflow = 1u,
    kStStackOverflow = 2u,
    kStDepthLimit = 4u,     // warning: a depth-21 leaf holds more than leaf_capacity
    kStNonFinite = 8u,
    kStTimeout = 16u,
    kStListOverflow = 32u,  // per-warp list staging or the final list pool
    kStCorrupt = 64u,       // walk visit limit breached
    kStPendOverflow = 128u, // learned walk: deferred-pair pool exhausted
    kStSortDepth = 256u,    // a node at the deepest sorted key level still needs splitting
    kStFatal = kStNodeOverflow | kStStackOverflow | kStNonFinite | kStTimeout | kStListOverflow | kStCorrupt |
               kStPendOverflow | kStSortDepth,
};

// Per-evaluation device counters (zeroed before each force evaluation).
struct Counters {
    unsigned long long p2p_pairs;
    unsigned long long p2c_terms;
    unsigned long long mac_tests;
    unsigned long long mac_retests;
    unsigned long long groups;
    unsigned long long bbox_min[3];   // order-preserving encoded FP64
    unsigned long long bbox_max[3];
    unsigned status;
    int next_free;                    // node allocator
    int level_begin[kMaxLevels + 2];
    int done_blocks;
    int nleaves;
    int max_leaf_count;
    int depth_limited;
    int work_next;                    // dynamic group scheduler (walk)
    int stack_max;
    int levels_used;
    int eval_next;                    // dynamic group scheduler (evaluation)
    double root_center[3];
    double root_half;
    unsigned long long far_total;     // list entries written (far, near)
    unsigned long long near_total;
    int list_max;                     // longest per-group list seen
    int far_chunks;                   // chunk allocators (may exceed the pool: then
    int near_chunks;                  //   they count what a retry needs)
    int pad2;
    // learned opening test: pairs handed to the network, accepted by it, and
    // decided by the geometric fallback (low confidence); tensor-core flushes
    unsigned long long lm_queries;
    unsigned long long lm_accepts;
    unsigned long long lm_fallbacks;
    unsigned long long lm_flushes;
    unsigned long long lm_screened;   // band pairs the error bound accepted without the network
    unsigned long long targets;       // particles whose acceleration a block-step evaluation refreshed
};

// Per-group interaction lists written by the walk, read by the evaluation.
// Each list is a chain of kListChunk-entry chunks taken from a pool with one
// atomic per chunk; next[c] links chunk c to the following one.
constexpr int kListChunk = 128;
struct ListBuffers {
    int far_chunk_cap = 0, near_chunk_cap = 0;
    int* far = nullptr;               // far node ids, far_chunk_cap * kListChunk
    int* near = nullptr;              // near leaf ids
    int* far_next = nullptr;          // chunk links
    int* near_next = nullptr;
    int4* ginfo = nullptr;            // per group: far first chunk, near first chunk, far count, near count
    int* stack = nullptr;             // per walking warp traversal stack
    int stack_cap = 0;
    int nwarps = 0;                   // resident walking warps
};

struct NodeArrays {
    int cap = 0;
    int* start = nullptr;
    int* count = nullptr;
    int* first_child = nullptr;       // -1 for leaves
    int* parent = nullptr;
    int* visit = nullptr;             // upward-pass arrival counters
    unsigned char* nchild = nullptr;
    unsigned char* level = nullptr;
    double* cx = nullptr;             // geometric centre (FP64 recurrence of the reference)
    double* cy = nullptr;
    double* cz = nullptr;
    double* half = nullptr;           // half size (0 on the system-id levels of an ensemble)
    int* sysroot = nullptr;           // root node of the node's system (0 for a single system)
    // FP64 moments
    double* mass = nullptr;
    double* comx = nullptr;
    double* comy = nullptr;
    double* comz = nullptr;
    double* maxr = nullptr;
    double* quad = nullptr;           // 5 per node
    float* amin = nullptr;            // leaves: min |a| over the members (learned opening test)
    // FP32 walk records
    float4* wA = nullptr;             // com_hi.xyz, mass
    float4* wB = nullptr;             // Qxx, Qyy, Qxy, Qxz
    float4* wC = nullptr;             // maxR (rounded up), 2h, link (int bits), meta (int bits)
    float4* wD = nullptr;             // com_lo.xyz, Qyz
    float4* chi = nullptr;            // centre hi (leaves; SPLIT)
    float4* clo = nullptr;            // centre lo (leaves; SPLIT)
};

// wC.w meta: bit 31 leaf flag; bits 0..23 count (leaf) or nchild (internal);
// bits 24..28 level.
__host__ __device__ inline int meta_pack(bool leaf, int count_or_nchild, int level) {
    return (leaf ? (int)0x80000000u : 0) | ((level & 31) << 24) | (count_or_nchild & 0xFFFFFF);
}

struct Particles {
    long long cap = 0;
    float4* pos = nullptr;
    float4* plo = nullptr;
    float4* vel = nullptr;
    float4* vlo = nullptr;            // velocity low halves (SPLIT): kicks accumulate ~48 bits
    float4* acc = nullptr;
    float4* src = nullptr;
    int* id = nullptr;
    // ping-pong partners for the permutation
    float4* pos2 = nullptr;
    float4* plo2 = nullptr;
    float4* vel2 = nullptr;
    float4* vlo2 = nullptr;
    float4* acc2 = nullptr;
    int* id2 = nullptr;
};

struct SortBuffers {
    long long cap = 0;
    unsigned long long* keys = nullptr;
    unsigned long long* keys_alt = nullptr;
    unsigned* vals = nullptr;
    unsigned* vals_alt = nullptr;
    unsigned* hist = nullptr;         // kRsBins x blocks
    unsigned* scan_tmp = nullptr;
    long long hist_cap = 0;
    long long scan_tmp_cap = 0;
    long long* ktab = nullptr;        // centres of the top key levels, ordered images (key_table_entries())
};

struct WalkParams {
    float eps2;
    float theta;
    float theta2;
    float G;
    double theta2_d;
    double eps2_d;
    int quadrupole;
    int split;
    int retest;
    int kick;                         // apply closing half-kick v += hdt * a
    float hdt;
    int stack_cap;
    int node_limit;                   // visits per group beyond this mean a corrupt tree
    int global_stack;                 // walk stack in global memory (fallback for deep frontiers)
    int smem_stack;                   // per-warp shared-memory walk stack: 1024, 2048 or 4096 entries
    int soft;                         // kSoftPlummer or kSoftSpline (softening.cuh)
    float ih;                         // spline: 1 / h (h = eps)
    int p2p_tile;                     // sources per near batch of the evaluation (64..256; 0: 256)
    // learned opening test (walk_lmac_kernel)
    int learned;
    float lm_log2b;                   // log2 of the per-target error budget
    float lm_gate;                    // |logit| below which the geometric test decides
    float lm_rho_lo, lm_rho_hi;       // band of 2h/worst handed to the network
    float lm_mu[8], lm_isd[8];        // feature standardisation of the network
    float lm_screen;                  // accept unasked when the error bound <= lm_screen * budget (0: off)
    float lm_budget;                  // the budget itself
};

// A forest of independent systems in one particle set (ensemble).  System s
// holds slots [off[s], off[s+1]) in every tree order; its id occupies the top
// sys_levels key digits, the remaining 21 - sys_levels digits are the octant
// path from its own root cube (the reference's BuildRoot on its particles).
// The system-id levels are virtual: they always split and carry no geometry.
// A single system is sys_levels = 0, nsys = 1, off = nullptr.
struct Forest {
    int nsys = 1;
    int sys_levels = 0;
    const long long* off = nullptr;   // nsys + 1 slot offsets
    double* root = nullptr;           // per system: centre x, y, z, half (4 doubles)
    unsigned long long* bbox = nullptr;  // per system: encoded min x, y, z, max x, y, z
};

// System of a slot (binary search over the offsets).
// (h, l) += d for a double-float pair: error-free two-sum, renormalised.
__device__ __forceinline__ void df_add(float& h, float& l, float d) {
    const float s = h + d;
    const float bb = s - h;
    const float e = (h - (s - bb)) + (d - bb);
    const float l2 = l + e;
    const float h2 = s + l2;
    l = l2 - (h2 - s);
    h = h2;
}

// Closing or opening half-kick of one particle: v += h a, as a double-float
// pair when vl is given (split precision), else in FP32.
__device__ __forceinline__ void kick_v(float4& v, float4* vl, float h, const float4& a) {
    if (vl) {
        df_add(v.x, vl->x, h * a.x);
        df_add(v.y, vl->y, h * a.y);
        df_add(v.z, vl->z, h * a.z);
    } else {
        v.x = fmaf(h, a.x, v.x);
        v.y = fmaf(h, a.y, v.y);
        v.z = fmaf(h, a.z, v.z);
    }
}

__device__ __forceinline__ int forest_system(const Forest& F, long long k) {
    int lo = 0, hi = F.nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (F.off[mid] <= k)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// ---- launchers (each enqueues on `s`; no host synchronisation) ----
void launch_bbox(const float4* pos, const float4* plo, long long n, Counters* C, cudaStream_t s);
void launch_root(Counters* C, long long n, cudaStream_t s);
// Ensemble: per-system bounding boxes and root cubes (F.nsys > 1).
void launch_forest_bbox(const float4* pos, const float4* plo, long long n, const Forest& F, Counters* C,
                        cudaStream_t s);
void launch_forest_root(const Forest& F, cudaStream_t s);
void launch_collapse_split(float4* pos, float4* plo, long long n, cudaStream_t s);
// Keys of the current order (vals = 0 .. n-1); a single system also fills
// the centre table ktab (key_table_entries() doubles).  Returns the launches made.
int launch_keys(const float4* pos, const float4* plo, long long n, Counters* C, const Forest& F, long long* ktab,
                unsigned long long* keys, unsigned* vals, cudaStream_t s);
// Stable LSD radix sort of (keys, vals) over bits [shift0, shift0 + kRsDigitBits*passes);
// result ends in (keys, vals) (the alternates are scratch).
void radix_sort_pairs(SortBuffers& sb, long long n, int passes, int shift0, cudaStream_t s);
// Entries of SortBuffers::hist for n keys: the tile histograms, then the
// digit totals.
long long radix_hist_size(long long n);
// Doubles of SortBuffers::ktab: the tabulated key centres of the three axes.
long long key_table_entries();
void launch_permute(const Particles& P, const unsigned* perm, long long n, bool split, cudaStream_t s);
void launch_tree_init(NodeArrays& T, Counters* C, long long n, int leaf_cap, int max_depth, cudaStream_t s);
// Builds levels 1 .. levels (keys sorted on their top `levels` digits); a node
// at level `levels` that would still split sets kStSortDepth.
void launch_tree_levels(NodeArrays& T, Counters* C, const unsigned long long* keys, long long n, int leaf_cap,
                        int max_depth, const Forest& F, int levels, cudaStream_t s);
void launch_leaf_list(NodeArrays& T, Counters* C, long long n, int* leaf_at, unsigned* flags, unsigned* scan_out,
                      int* leaf_list, SortBuffers& sb, cudaStream_t s);
void launch_moments(NodeArrays& T, Counters* C, const Particles& P, const int* leaf_list, long long n,
                    int max_leaves, bool split, bool quadrupole, int levels, cudaStream_t s);
void launch_walk(const NodeArrays& T, Counters* C, const int* leaf_list, const WalkParams& wp,
                 const ListBuffers& LB, cudaStream_t s);
void launch_eval(const NodeArrays& T, Counters* C, const Particles& P, const int* leaf_list, const WalkParams& wp,
                 const ListBuffers& LB, int nwarps, cudaStream_t s);
void launch_kick_drift(const Particles& P, long long n, float hdt, float dt, bool split, Counters* C,
                       cudaStream_t s);
void launch_scatter_accel(const Particles& P, long long n, double* ax, double* ay, double* az, cudaStream_t s);
void device_exclusive_scan(const unsigned* in, unsigned* out, long long n, unsigned* tmp, cudaStream_t s);
long long scan_tmp_size(long long n);

}  // namespace ngrav
