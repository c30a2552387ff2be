// tree.cu -- linear octree from sorted keys, leaf list, upward moment pass.
//
// Topology rule (restating projects/nbody_core/src/Tree.cpp:114-145): a node
// at level l whose particle count exceeds the leaf capacity (ncrit) and whose
// level is below maxDepth is internal; its children are its non-empty
// octants.  The node set of the reference's insertion build is exactly this
// set, independent of insertion order, so it is built here top-down, one
// level per launch, by splitting each internal node's contiguous key range at
// its level-l digit boundaries (binary search).  Children of a node are
// allocated contiguously in ascending octant order.
//
// Moments (restating Tree.cpp:119-122 running COM, :179-202 maxRadius,
// :205-254 quadrupoles): leaves sum their members (mass and COM in FP64,
// quadrupole in FP32 on offsets from the COM); internal nodes combine their
// children in FP64 (the top-level moment accumulation), bottom-up with
// per-node arrival counters so each parent is finished by the last child to
// arrive.
#include "engine.cuh"

namespace ngrav {

__global__ void reset_counters_kernel(Counters* C) {
    if (threadIdx.x == 0) {
        Counters z{};
        for (int a = 0; a < 3; ++a) {
            z.bbox_min[a] = ~0ull;
            z.bbox_max[a] = 0ull;
        }
        *C = z;
    }
}

__global__ void tree_init_kernel(NodeArrays T, Counters* C, long long n, int leaf_cap, int max_depth) {
    T.start[0] = 0;
    T.count[0] = (int)n;
    T.first_child[0] = -1;
    T.parent[0] = -1;
    T.visit[0] = 0;
    T.nchild[0] = 0;
    T.level[0] = 0;
    T.cx[0] = C->root_center[0];
    T.cy[0] = C->root_center[1];
    T.cz[0] = C->root_center[2];
    T.half[0] = C->root_half;
    T.sysroot[0] = 0;
    C->next_free = 1;
    C->level_begin[0] = 0;
    C->level_begin[1] = 1;
    C->levels_used = 0;
    C->max_leaf_count = 0;
}

void launch_tree_init(NodeArrays& T, Counters* C, long long n, int leaf_cap, int max_depth, cudaStream_t s) {
    tree_init_kernel<<<1, 1, 0, s>>>(T, C, n, leaf_cap, max_depth);
}

// First index k in [lo, hi) whose level digit (at `shift`) is >= d.
__device__ __forceinline__ int digit_lower_bound(const unsigned long long* __restrict__ keys, int lo, int hi,
                                                 int shift, unsigned d) {
    while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);
        const unsigned v = (unsigned)(__ldg(keys + mid) >> shift) & 7u;
        if (v < d)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

constexpr int kLevelThreads = 256;

// One level of the split, eight lanes per node: lane d finds where octant d
// begins in the node's key range (d = 1..7 by independent binary searches,
// so the top levels' long ranges cost one search's latency, not seven) and
// creates child d.  Ensemble (F.sys_levels > 0): levels above sys_levels
// group systems by id digits, always split and carry no geometry; a child at
// level sys_levels is a system root and takes that system's cube; below it
// the reference's recurrence runs from that root.
__global__ void __launch_bounds__(kLevelThreads) tree_level_kernel(NodeArrays T, Counters* C,
                                                                   const unsigned long long* __restrict__ keys,
                                                                   int l, int leaf_cap, int max_depth, Forest F,
                                                                   int levels) {
    const int begin = C->level_begin[l];
    const int end = C->level_begin[l + 1];
    const int shift = 3 * (kKeyLevels - 1 - l);
    const bool virt = l < F.sys_levels;                 // this level groups systems
    const bool sys_child = l + 1 == F.sys_levels;      // children are system roots
    const int depth_cap = max_depth + F.sys_levels;    // max_depth counts from each system root
    const int lane = threadIdx.x & 31;
    const int d = lane & 7;
    const unsigned gmask = 0xFFu << (lane & 24);       // the node's eight lanes
    const long long gid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 3;
    const long long ngroups = (gridDim.x * (long long)blockDim.x) >> 3;
    // every lane of a warp runs the same number of iterations (shuffles below)
    const int span = end - begin;
    const long long warp0 = gid & ~3ll;
    for (long long g0 = warp0; g0 < span; g0 += ngroups) {
        const int node = begin + (int)(g0 + (gid & 3));
        bool split = false;
        int s = 0, cnt = 0;
        if (node < end) {
            cnt = T.count[node];
            split = virt || (cnt > leaf_cap && l < depth_cap);  // else it stays a leaf
            s = T.start[node];
        }
        const int e = s + cnt;
        const int bd = split ? (d == 0 ? s : digit_lower_bound(keys, s, e, shift, (unsigned)d)) : 0;
        int bn = __shfl_down_sync(0xffffffffu, bd, 1, 8);  // where octant d + 1 begins
        if (d == 7) bn = e;
        const bool has = split && bn > bd;
        const unsigned hm = (__ballot_sync(0xffffffffu, has) & gmask) >> (lane & 24);
        const int nch = __popc(hm);
        int base = 0;
        if (split && d == 0) base = atomicAdd(&C->next_free, nch);
        base = __shfl_sync(0xffffffffu, base, lane & 24, 32);
        if (!split) continue;
        if (base + nch > T.cap) {
            if (d == 0) atomicOr(&C->status, kStNodeOverflow);
            // The slots of this allocation that still fall inside the pool
            // become inert records (no particles, no children), so the passes
            // that scan every node up to the pool's end never read an
            // unwritten record; the parent stays a leaf.  The walk and the
            // evaluation do not run on the truncated tree, and the host grows
            // the pool and builds again.
            if (has) {
                const int c = base + __popc(hm & ((1u << d) - 1u));
                if (c < T.cap) {
                    T.start[c] = 0;
                    T.count[c] = 0;
                    T.first_child[c] = -1;
                    T.parent[c] = node;
                    T.visit[c] = 0;
                    T.nchild[c] = 0;
                    T.level[c] = (unsigned char)(l + 1);
                    T.cx[c] = T.cx[node];
                    T.cy[c] = T.cy[node];
                    T.cz[c] = T.cz[node];
                    T.half[c] = 0.0;
                    T.sysroot[c] = T.sysroot[node];
                }
            }
            continue;
        }
        if (has) {
            const int c = base + __popc(hm & ((1u << d) - 1u));
            const int cs = bd, ce = bn;
            T.start[c] = cs;
            T.count[c] = ce - cs;
            T.first_child[c] = -1;
            T.parent[c] = node;
            T.visit[c] = 0;
            T.nchild[c] = 0;
            T.level[c] = (unsigned char)(l + 1);
            if (virt) {
                if (sys_child) {
                    const int sys = (int)(keys[cs] >> (3 * (kKeyLevels - F.sys_levels)));
                    T.cx[c] = F.root[4 * sys];
                    T.cy[c] = F.root[4 * sys + 1];
                    T.cz[c] = F.root[4 * sys + 2];
                    T.half[c] = F.root[4 * sys + 3];
                } else {
                    T.cx[c] = T.cy[c] = T.cz[c] = 0.0;
                    T.half[c] = 0.0;
                }
                T.sysroot[c] = c;
            } else {
                const double pcx = T.cx[node], pcy = T.cy[node], pcz = T.cz[node];
                const double child_half = 0.5 * T.half[node];
                T.cx[c] = (d & 1) ? __dadd_rn(pcx, child_half) : __dsub_rn(pcx, child_half);
                T.cy[c] = (d & 2) ? __dadd_rn(pcy, child_half) : __dsub_rn(pcy, child_half);
                T.cz[c] = (d & 4) ? __dadd_rn(pcz, child_half) : __dsub_rn(pcz, child_half);
                T.half[c] = child_half;
                T.sysroot[c] = T.sysroot[node];
            }
            if (l + 1 >= kKeyLevels && ce - cs > leaf_cap && l + 1 < depth_cap) {
                atomicOr(&C->status, kStDepthLimit);
                atomicAdd(&C->depth_limited, 1);
            } else if (l + 1 == levels && ce - cs > leaf_cap && l + 1 < depth_cap) {
                // the keys were sorted on `levels` digits only: this child
                // would split on an unsorted digit, so the build is redone on
                // the full key
                atomicOr(&C->status, kStSortDepth);
            }
        }
        if (d == 0) {
            T.first_child[node] = base;
            T.nchild[node] = (unsigned char)nch;
            atomicMax(&C->levels_used, l + 1);
        }
    }
    // The last block to finish publishes where level l+2 begins.
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const int prev = atomicAdd(&C->done_blocks, 1);
        if (prev == (int)gridDim.x - 1) {
            int nf = atomicAdd(&C->next_free, 0);
            if (nf > T.cap) nf = T.cap;
            C->level_begin[l + 2] = nf;
            C->done_blocks = 0;
        }
    }
}

void launch_tree_levels(NodeArrays& T, Counters* C, const unsigned long long* keys, long long n, int leaf_cap,
                        int max_depth, const Forest& F, int levels, cudaStream_t s) {
    // Enough threads for the widest level (nodes <= cap); levels above it
    // exit after a bounds check.
    long long blocks = ((long long)T.cap / 4 * 8 + kLevelThreads - 1) / kLevelThreads;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks < 1) blocks = 1;
    for (int l = 0; l < levels; ++l)
        tree_level_kernel<<<(unsigned)blocks, kLevelThreads, 0, s>>>(T, C, keys, l, leaf_cap, max_depth, F, levels);
}

// ---------------------------------------------------------------------------
// Leaf list in key order
// ---------------------------------------------------------------------------

__global__ void leaf_mark_kernel(NodeArrays T, Counters* C, long long n, int* __restrict__ leaf_at,
                                 unsigned* __restrict__ flags) {
    const int nn = min(C->next_free, T.cap);
    for (int node = blockIdx.x * blockDim.x + threadIdx.x; node < nn; node += gridDim.x * blockDim.x) {
        if (T.first_child[node] != -1) continue;
        const int s = T.start[node];
        // inert records of an overflowed allocation own no particles
        if (T.count[node] <= 0 || s < 0 || s >= n) continue;
        leaf_at[s] = node;
        flags[s] = 1u;
        atomicMax(&C->max_leaf_count, T.count[node]);
    }
}

__global__ void leaf_compact_kernel(const int* __restrict__ leaf_at, const unsigned* __restrict__ flags,
                                    const unsigned* __restrict__ pos, long long n, int* __restrict__ leaf_list,
                                    Counters* C) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        if (flags[k]) leaf_list[pos[k]] = leaf_at[k];
        if (k == n - 1) C->nleaves = (int)(pos[k] + flags[k]);
    }
}

void launch_leaf_list(NodeArrays& T, Counters* C, long long n, int* leaf_at, unsigned* flags, unsigned* scan_out,
                      int* leaf_list, SortBuffers& sb, cudaStream_t s) {
    cudaMemsetAsync(flags, 0, sizeof(unsigned) * n, s);
    long long b1 = ((long long)T.cap + 255) / 256;
    if (b1 > 152 * 8) b1 = 152 * 8;
    leaf_mark_kernel<<<(unsigned)b1, 256, 0, s>>>(T, C, n, leaf_at, flags);
    device_exclusive_scan(flags, scan_out, n, sb.scan_tmp, s);
    long long b2 = (n + 255) / 256;
    if (b2 > 152 * 8) b2 = 152 * 8;
    leaf_compact_kernel<<<(unsigned)b2, 256, 0, s>>>(leaf_at, flags, scan_out, n, leaf_list, C);
}

// ---------------------------------------------------------------------------
// Upward pass
// ---------------------------------------------------------------------------

__device__ __forceinline__ float round_up_f(double v) {
    float f = (float)v;
    if ((double)f < v) f = nextafterf(f, 3.0e38f);
    return f;
}

__device__ __forceinline__ void write_walk_record(NodeArrays& T, int node, double M, double cx, double cy,
                                                  double cz, const double* Q, double maxr, bool leaf, int link,
                                                  int cnt_or_nch, int level) {
    const float hx = (float)cx, hy = (float)cy, hz = (float)cz;
    T.wA[node] = make_float4(hx, hy, hz, (float)M);
    T.wB[node] = make_float4((float)Q[0], (float)Q[1], (float)Q[2], (float)Q[3]);
    const double size = 2.0 * T.half[node];
    T.wC[node] = make_float4(round_up_f(maxr), (float)size, __int_as_float(link),
                             __int_as_float(meta_pack(leaf, cnt_or_nch, level)));
    T.wD[node] = make_float4((float)(cx - (double)hx), (float)(cy - (double)hy), (float)(cz - (double)hz),
                             (float)Q[4]);
}

// Leaf moments, plus the group acceleration scale amin[leaf] = min over the
// members of |a| from `acc` (the accelerations carried into this tree order;
// zero before the first evaluation) that the learned opening test reads.
//
// GB300's FP64 pipe runs at 1/32 of the FP32 rate, so the per-particle work
// is FP32: each member's offset from the leaf centre is a double-float pair
// (error-free differences of the double-float position and centre), mass
// and first moment are summed as double-float pairs with exact products,
// and only the per-leaf results are FP64.  maxRadius keeps the reference's
// FP64 value: the members within FP32 rounding of the FP32 maximum distance
// are re-measured in FP64 (Tree.cpp:188-201).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    e = b - (s - a);
}

// Offset of a double-float coordinate (h + l) from a double-float centre
// (ch + cl), as a normalised double-float pair.
__device__ __forceinline__ void df_offset(float h, float l, float ch, float cl, float& oh, float& ol) {
    float s, e;
    two_sum(h, -ch, s, e);
    fast_two_sum(s, e + (l - cl), oh, ol);
}

// (Sh, Sl) += m * (oh + ol), the product of the high parts exact.
__device__ __forceinline__ void df_add_prod(float& Sh, float& Sl, float m, float oh, float ol) {
    const float p = m * oh;
    const float pe = fmaf(m, oh, -p) + m * ol;
    float t, e;
    two_sum(Sh, p, t, e);
    fast_two_sum(t, Sl + (e + pe), Sh, Sl);
}

__global__ void __launch_bounds__(128) moments_kernel(NodeArrays T, Counters* C, const float4* __restrict__ pos,
                                                      const float4* __restrict__ plo, float4* __restrict__ src,
                                                      const float4* __restrict__ acc,
                                                      const int* __restrict__ leaf_list, int split, int quadrupole) {
    const int nleaves = C->nleaves;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int li = blockIdx.x * blockDim.x + threadIdx.x; li < nleaves; li += gridDim.x * blockDim.x) {
        const int leaf = leaf_list[li];
        const int s = T.start[leaf], cnt = T.count[leaf];
        const double ccx = T.cx[leaf], ccy = T.cy[leaf], ccz = T.cz[leaf];
        const float chx = (float)ccx, chy = (float)ccy, chz = (float)ccz;
        const float clx = (float)(ccx - (double)chx), cly = (float)(ccy - (double)chy),
                    clz = (float)(ccz - (double)chz);
        // pass 1: mass and first moment about the leaf centre
        float Mh = 0.f, Ml = 0.f, Xh = 0.f, Xl = 0.f, Yh = 0.f, Yl = 0.f, Zh = 0.f, Zl = 0.f;
        for (int j = s; j < s + cnt; ++j) {
            const float4 p = pos[j];
            const float4 q = plo ? plo[j] : zero4;
            float ox, oxl, oy, oyl, oz, ozl;
            df_offset(p.x, q.x, chx, clx, ox, oxl);
            df_offset(p.y, q.y, chy, cly, oy, oyl);
            df_offset(p.z, q.z, chz, clz, oz, ozl);
            float t, e;
            two_sum(Mh, p.w, t, e);
            fast_two_sum(t, Ml + e, Mh, Ml);
            df_add_prod(Xh, Xl, p.w, ox, oxl);
            df_add_prod(Yh, Yl, p.w, oy, oyl);
            df_add_prod(Zh, Zl, p.w, oz, ozl);
        }
        const double M = (double)Mh + (double)Ml;
        double ocx = 0.0, ocy = 0.0, ocz = 0.0;  // COM - centre
        if (M > 0.0) {
            const double inv = 1.0 / M;
            ocx = ((double)Xh + (double)Xl) * inv;
            ocy = ((double)Yh + (double)Yl) * inv;
            ocz = ((double)Zh + (double)Zl) * inv;
        }
        const double cx = ccx + ocx, cy = ccy + ocy, cz = ccz + ocz;
        const float ohx = (float)ocx, ohy = (float)ocy, ohz = (float)ocz;
        const float olx = (float)(ocx - (double)ohx), oly = (float)(ocy - (double)ohy),
                    olz = (float)(ocz - (double)ohz);
        // pass 2: FP32 distances from the COM, quadrupole, amin, walk sources
        float maxf = 0.f;
        float q0 = 0.f, q1 = 0.f, q2 = 0.f, q3 = 0.f, q4 = 0.f;
        float amin2 = 3.0e38f;
        for (int j = s; j < s + cnt; ++j) {
            const float4 p = pos[j];
            const float4 a = acc[j];
            amin2 = fminf(amin2, a.x * a.x + a.y * a.y + a.z * a.z);
            const float4 l = plo ? plo[j] : zero4;
            float ox, oxl, oy, oyl, oz, ozl;
            df_offset(p.x, l.x, chx, clx, ox, oxl);
            df_offset(p.y, l.y, chy, cly, oy, oyl);
            df_offset(p.z, l.z, chz, clz, oz, ozl);
            const float fx = (ox - ohx) + (oxl - olx), fy = (oy - ohy) + (oyl - oly), fz = (oz - ohz) + (ozl - olz);
            const float d2 = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
            maxf = fmaxf(maxf, d2);
            if (quadrupole && cnt > 1) {
                const float m = p.w;
                q0 += m * (3.f * fx * fx - d2);
                q1 += m * (3.f * fy * fy - d2);
                q2 += m * 3.f * fx * fy;
                q3 += m * 3.f * fx * fz;
                q4 += m * 3.f * fy * fz;
            }
            src[j] = split ? make_float4(ox + oxl, oy + oyl, oz + ozl, p.w) : p;
        }
        // pass 3: the FP64 maximum over the members that can hold it.  An FP32
        // distance is within a few ulps of the leaf's half size of the FP64
        // one, so no member farther than the cut can be missed.
        double maxr2 = 0.0;
        const float rcut = sqrtf(maxf) * (1.f - 4e-6f) - 2e-6f * (float)T.half[leaf];
        const float cut = rcut > 0.f ? rcut * rcut : -1.f;
        for (int j = s; j < s + cnt; ++j) {
            const float4 p = pos[j];
            const float4 l = plo ? plo[j] : zero4;
            float ox, oxl, oy, oyl, oz, ozl;
            df_offset(p.x, l.x, chx, clx, ox, oxl);
            df_offset(p.y, l.y, chy, cly, oy, oyl);
            df_offset(p.z, l.z, chz, clz, oz, ozl);
            const float fx = (ox - ohx) + (oxl - olx), fy = (oy - ohy) + (oyl - oly), fz = (oz - ohz) + (ozl - olz);
            if (fmaf(fx, fx, fmaf(fy, fy, fz * fz)) >= cut) {
                const double x = (double)p.x + (double)l.x, y = (double)p.y + (double)l.y,
                             z = (double)p.z + (double)l.z;
                const double dx = x - cx, dy = y - cy, dz = z - cz;
                maxr2 = fmax(maxr2, dx * dx + dy * dy + dz * dz);
            }
        }
        const double maxr = sqrt(maxr2);
        const double Q[5] = {q0, q1, q2, q3, q4};
        T.mass[leaf] = M;
        T.comx[leaf] = cx;
        T.comy[leaf] = cy;
        T.comz[leaf] = cz;
        T.maxr[leaf] = maxr;
        T.amin[leaf] = cnt > 0 ? sqrtf(amin2) : 0.f;
        for (int k = 0; k < 5; ++k) T.quad[5 * leaf + k] = Q[k];
        const int level = T.level[leaf];
        write_walk_record(T, leaf, M, cx, cy, cz, Q, maxr, true, s, cnt, level);
        T.chi[leaf] = make_float4(chx, chy, chz, 0.f);
        T.clo[leaf] = make_float4(clx, cly, clz, 0.f);
    }
}

// Internal nodes of one level, from their (finished) children: mass and COM
// (sum m x / M) in FP64 in child order, as the reference's sequential sums;
// the traceless quadrupole by the parallel-axis shift (Tree.cpp:235-251) and
// maxRadius = max over children of maxR_c + |com_c - com| (Tree.cpp:194-201;
// massless nodes keep 0).  GB300's FP64 pipe is narrow, so the per-child
// work runs on the FP32 pipe from the children's walk records: offsets from
// the double-float parent COM, the quadrupole shift summed in FP32 (the walk
// evaluates quadrupoles in FP32), and maxRadius screened in FP32 with only
// the children within rounding of the FP32 maximum re-measured in FP64.  The
// geometric opening test reads maxRadius of leaves only; the learned one
// reads it for every node.
__global__ void __launch_bounds__(256) internal_moments_kernel(NodeArrays T, const Counters* __restrict__ C, int l,
                                                              int quadrupole) {
    const int begin = C->level_begin[l];
    const int end = C->level_begin[l + 1];
    for (int node = begin + blockIdx.x * blockDim.x + threadIdx.x; node < end; node += gridDim.x * blockDim.x) {
        const int fc = T.first_child[node];
        if (fc < 0) continue;
        const int nch = T.nchild[node];
        // the (at most eight) children unrolled: their loads and the FP64
        // chains of the combination overlap instead of running one child
        // after another
        double mc[8], cxs[8], cys[8], czs[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const bool in = k < nch;
            mc[k] = in ? T.mass[fc + k] : 0.0;
            cxs[k] = in ? T.comx[fc + k] : 0.0;
            cys[k] = in ? T.comy[fc + k] : 0.0;
            czs[k] = in ? T.comz[fc + k] : 0.0;
        }
        double PM = 0.0, px = 0.0, py = 0.0, pz = 0.0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {  // in child order, as the sequential sum
            PM += mc[k];
            px = fma(mc[k], cxs[k], px);
            py = fma(mc[k], cys[k], py);
            pz = fma(mc[k], czs[k], pz);
        }
        double pcx = T.cx[node], pcy = T.cy[node], pcz = T.cz[node];
        if (PM > 0.0) {
            const double inv = 1.0 / PM;
            pcx = px * inv;
            pcy = py * inv;
            pcz = pz * inv;
        }
        const float phx = (float)pcx, phy = (float)pcy, phz = (float)pcz;
        const float plx = (float)(pcx - (double)phx), ply = (float)(pcy - (double)phy),
                    plz = (float)(pcz - (double)phz);
        float q0 = 0.f, q1 = 0.f, q2 = 0.f, q3 = 0.f, q4 = 0.f;
        float cand[8];
        float best = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            cand[k] = -1.f;
            if (k >= nch) continue;
            const int c = fc + k;
            const float4 A = T.wA[c], D = T.wD[c];
            const float dx = (A.x - phx) + (D.x - plx), dy = (A.y - phy) + (D.y - ply),
                        dz = (A.z - phz) + (D.z - plz);
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (quadrupole && mc[k] > 0.0) {
                const float4 B = T.wB[c];
                const float m = A.w;
                q0 += B.x + m * (3.f * dx * dx - d2);
                q1 += B.y + m * (3.f * dy * dy - d2);
                q2 += B.z + m * 3.f * dx * dy;
                q3 += B.w + m * 3.f * dx * dz;
                q4 += D.w + m * 3.f * dy * dz;
            }
            cand[k] = T.wC[c].x + sqrtf(d2);  // >= maxR_c (rounded up) + |d| within FP32 rounding
            best = fmaxf(best, cand[k]);
        }
        double mr = 0.0;
        if (PM > 0.0) {
            const float cut = best * (1.f - 1e-5f) - 1e-30f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (k >= nch || cand[k] < cut) continue;
                const double dx = cxs[k] - pcx, dy = cys[k] - pcy, dz = czs[k] - pcz;
                mr = fmax(mr, T.maxr[fc + k] + sqrt(dx * dx + dy * dy + dz * dz));
            }
        }
        const double PQ[5] = {q0, q1, q2, q3, q4};
        T.mass[node] = PM;
        T.comx[node] = pcx;
        T.comy[node] = pcy;
        T.comz[node] = pcz;
        T.maxr[node] = mr;
        for (int k = 0; k < 5; ++k) T.quad[5 * node + k] = PQ[k];
        write_walk_record(T, node, PM, pcx, pcy, pcz, PQ, mr, false, fc, nch, l);
    }
}

void launch_moments(NodeArrays& T, Counters* C, const Particles& P, const int* leaf_list, long long n,
                    int max_leaves, bool split, bool quadrupole, int levels, cudaStream_t s) {
    long long blocks = ((long long)max_leaves + 127) / 128;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    moments_kernel<<<(unsigned)blocks, 128, 0, s>>>(T, C, P.pos, split ? P.plo : nullptr, P.src, P.acc, leaf_list,
                                                    split ? 1 : 0, quadrupole ? 1 : 0);
    long long b2 = ((long long)T.cap / 4 + 255) / 256;
    if (b2 > 152 * 4) b2 = 152 * 4;
    if (b2 < 1) b2 = 1;
    for (int l = levels - 1; l >= 0; --l)
        internal_moments_kernel<<<(unsigned)b2, 256, 0, s>>>(T, C, l, quadrupole ? 1 : 0);
}

void launch_reset_counters(Counters* C, cudaStream_t s) { reset_counters_kernel<<<1, 32, 0, s>>>(C); }

}  // namespace ngrav
