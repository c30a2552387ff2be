// lmac_data.cu -- training data for the learned opening test, generated by the
// method itself on its own trees.
//
//  1. lmac_record_kernel walks every leaf group with the geometric test at a
//     small theta (every node whose opening ratio rho = 2h/worst lies in the
//     network's band is reached) and keeps a hashed random sample of the
//     (group, node) pairs it meets in the band;
//  2. lmac_label_kernel measures, for each kept pair, the exact acceleration
//     of the node's particles on every member of the group against the
//     node's multipole (the P2C of the evaluation: softened monopole +
//     unsoftened traceless quadrupole), relative to the member's total |a|:
//        r = max_t |a_exact,N(t) - a_multipole,N(t)| / |a(t)|;
//  3. lmac_feature_kernel computes the pair's features (lmac.cuh) with a unit
//     budget (log2 b = 0), so that training can place the budget anywhere.
#include "engine.cuh"
#include "lmac.cuh"
#include "lmac_internal.cuh"

namespace ngrav {

__device__ __forceinline__ uint32_t lmac_hash(uint32_t a, uint32_t b, uint32_t seed) {
    uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ seed * 0xC2B2AE3Du;
    h ^= h >> 16;
    h *= 0x7FEB352Du;
    h ^= h >> 15;
    h *= 0x846CA68Bu;
    h ^= h >> 16;
    return h;
}

constexpr int kRecWarps = 4;
constexpr int kRecStack = 4096;

__global__ void __launch_bounds__(kRecWarps * 32) lmac_record_kernel(NodeArrays T, const Counters* __restrict__ C,
                                                                    const int* __restrict__ leaf_list,
                                                                    LmacRecordParams rp) {
    extern __shared__ int rec_stack[];
    const int lane = threadIdx.x & 31;
    int* stack = rec_stack + (threadIdx.x >> 5) * kRecStack;
    const int nleaves = C->nleaves;
    unsigned long long band = 0, kept = 0, dropped_groups = 0;
    for (;;) {
        int gi = 0;
        if (lane == 0) gi = atomicAdd(rp.work, 1);
        gi = __shfl_sync(0xffffffffu, gi, 0);
        if (gi >= nleaves) break;
        const int leaf = leaf_list[gi];
        const float4 gA = T.wA[leaf];
        const float4 gD = T.wD[leaf];
        const float gR = T.wC[leaf].x;
        int size = 0;
        const int root = T.sysroot[leaf];
        if (leaf != root) {
            if (lane == 0) stack[0] = root;
            size = 1;
        }
        __syncwarp();
        int visits = 0;
        while (size > 0) {
            const int take = min(size, 32);
            size -= take;
            visits += take;
            const int node = lane < take ? stack[size + lane] : -1;
            __syncwarp();
            int nch = 0, link = 0;
            bool in_band = false;
            if (node >= 0 && node != leaf) {
                const float4 A = T.wA[node];
                const float4 Cw = T.wC[node];
                const int meta = __float_as_int(Cw.w);
                if (A.w > 0.f && meta >= 0) {  // internal node with mass: a MAC decision
                    const float4 D = T.wD[node];
                    const float dx = (A.x - gA.x) + (D.x - gD.x);
                    const float dy = (A.y - gA.y) + (D.y - gD.y);
                    const float dz = (A.z - gA.z) + (D.z - gD.z);
                    const float worst = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - gR;
                    const float sz = Cw.y;
                    if (worst > 0.f && sz >= rp.rho_lo * worst && sz <= rp.rho_hi * worst) in_band = true;
                    if (!(worst > 0.f && sz < rp.theta * worst)) {
                        nch = meta & 0xFFFFFF;
                        link = __float_as_int(Cw.z);
                    }
                }
            }
            if (in_band) {
                ++band;
                if (lmac_hash((uint32_t)leaf, (uint32_t)node, rp.seed) < rp.threshold) {
                    const unsigned long long k = atomicAdd(rp.nkept, 1ull);
                    if (k < (unsigned long long)rp.cap) rp.pairs[k] = make_int2(leaf, node);
                    ++kept;
                }
            }
            // push opened children (exclusive scan of child counts)
            int off = nch;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, off, o);
                if (lane >= o) off += y;
            }
            const int tot = __shfl_sync(0xffffffffu, off, 31);
            off -= nch;
            if (size + tot > kRecStack || visits > rp.node_limit) {
                ++dropped_groups;  // best effort: the sample skips the rest of this group
                break;
            }
            for (int k = 0; k < nch; ++k) stack[size + off + k] = link + k;
            size += tot;
            __syncwarp();
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) {
        band += __shfl_xor_sync(0xffffffffu, band, o);
        dropped_groups = max(dropped_groups, __shfl_xor_sync(0xffffffffu, dropped_groups, o));
    }
    if (lane == 0) {
        atomicAdd(rp.nband, band);
        if (dropped_groups) atomicAdd(rp.ndropped, dropped_groups);
    }
    (void)kept;
}

// Per-leaf acceleration scale from the current accelerations (tree order).
__global__ void lmac_amin_kernel(NodeArrays T, const Counters* __restrict__ C, const int* __restrict__ leaf_list,
                                 const float4* __restrict__ acc) {
    const int nleaves = C->nleaves;
    for (int li = blockIdx.x * blockDim.x + threadIdx.x; li < nleaves; li += gridDim.x * blockDim.x) {
        const int leaf = leaf_list[li];
        const int s = T.start[leaf], cnt = T.count[leaf];
        float a2 = 3.0e38f;
        for (int j = s; j < s + cnt; ++j) {
            const float4 a = acc[j];
            a2 = fminf(a2, a.x * a.x + a.y * a.y + a.z * a.z);
        }
        T.amin[leaf] = cnt > 0 ? sqrtf(a2) : 0.f;
    }
}

// One warp per pair.  Positions are absolute double-float values (pos + plo
// when split); differences are formed hi-hi + lo-lo in FP32 as in the walk.
// Per lane the exact sum is Kahan-compensated in FP32, the warp total is
// formed in FP64.  Groups with more than kLabelMaxTargets members get r = -1.
constexpr int kLabelMaxTargets = 64;

__global__ void __launch_bounds__(256) lmac_label_kernel(NodeArrays T, const float4* __restrict__ pos,
                                                         const float4* __restrict__ plo,
                                                         const float4* __restrict__ acc,
                                                         const int2* __restrict__ pairs, int npairs, float G,
                                                         float eps2, float* __restrict__ r_out) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int p = wid; p < npairs; p += nw) {
        const int2 pr = pairs[p];
        const int gs = T.start[pr.x], gc = T.count[pr.x];
        const int ns = T.start[pr.y], nc = T.count[pr.y];
        if (gc > kLabelMaxTargets) {
            if (lane == 0) r_out[p] = -1.f;
            continue;
        }
        const float4 A = T.wA[pr.y];
        const float4 B = T.wB[pr.y];
        const float4 D = T.wD[pr.y];
        float rmax = 0.f;
        for (int t = gs; t < gs + gc; ++t) {
            const float4 ph = pos[t];
            const float4 pl = plo ? plo[t] : make_float4(0.f, 0.f, 0.f, 0.f);
            float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
            for (int j = ns + lane; j < ns + nc; j += 32) {
                const float4 qh = pos[j];
                const float4 ql = plo ? plo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float dx = (qh.x - ph.x) + (ql.x - pl.x);
                const float dy = (qh.y - ph.y) + (ql.y - pl.y);
                const float dz = (qh.z - ph.z) + (ql.z - pl.z);
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) + eps2;
                const float rs = rsqrtf(r2);
                const float w = qh.w * rs * rs * rs;
                // Kahan: s += w d
                float y = fmaf(w, dx, -cx), u = sx + y;
                cx = (u - sx) - y;
                sx = u;
                y = fmaf(w, dy, -cy);
                u = sy + y;
                cy = (u - sy) - y;
                sy = u;
                y = fmaf(w, dz, -cz);
                u = sz + y;
                cz = (u - sz) - y;
                sz = u;
            }
            double ex = (double)sx - (double)cx, ey = (double)sy - (double)cy, ez = (double)sz - (double)cz;
            for (int o = 16; o > 0; o >>= 1) {
                ex += __shfl_xor_sync(0xffffffffu, ex, o);
                ey += __shfl_xor_sync(0xffffffffu, ey, o);
                ez += __shfl_xor_sync(0xffffffffu, ez, o);
            }
            // the node's multipole on this member (the evaluation's P2C, G = 1)
            const float dx = (A.x - ph.x) + (D.x - pl.x);
            const float dy = (A.y - ph.y) + (D.y - pl.y);
            const float dz = (A.z - ph.z) + (D.z - pl.z);
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const float rs = rsqrtf(r2 + eps2);
            const float fm = A.w * (rs * rs * rs);
            float mx = fm * dx, my = fm * dy, mz = fm * dz;
            const float qyz = D.w, qzz = -(B.x + B.y);
            const float qdx = fmaf(B.x, dx, fmaf(B.z, dy, B.w * dz));
            const float qdy = fmaf(B.z, dx, fmaf(B.y, dy, qyz * dz));
            const float qdz = fmaf(B.w, dx, fmaf(qyz, dy, qzz * dz));
            const float qd2 = fmaf(dx, qdx, fmaf(dy, qdy, dz * qdz));
            const float ir = rsqrtf(r2);
            const float ir2 = ir * ir;
            const float ir5 = ir2 * ir2 * ir;
            const float c2 = 2.5f * qd2 * (ir5 * ir2);
            mx = fmaf(-ir5, qdx, fmaf(c2, dx, mx));
            my = fmaf(-ir5, qdy, fmaf(c2, dy, my));
            mz = fmaf(-ir5, qdz, fmaf(c2, dz, mz));
            const double ddx = ex - mx, ddy = ey - my, ddz = ez - mz;
            const float err = G * (float)sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
            const float4 at = acc[t];  // G included
            const float amag = sqrtf(at.x * at.x + at.y * at.y + at.z * at.z);
            rmax = fmaxf(rmax, err / fmaxf(amag, 1e-30f));
        }
        if (lane == 0) r_out[p] = rmax;
    }
}

// Features with a unit budget, one thread per pair.
__global__ void lmac_feature_kernel(NodeArrays T, const int2* __restrict__ pairs, int npairs, float G, float eps,
                                    float* __restrict__ X) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += gridDim.x * blockDim.x) {
        const int2 pr = pairs[p];
        const float4 gA = T.wA[pr.x], gD = T.wD[pr.x];
        const float gR = T.wC[pr.x].x;
        float f[kLmacIn];
        lmac_features(gA, gD, gR, T.amin[pr.x], T.wA[pr.y], T.wB[pr.y], T.wC[pr.y], T.wD[pr.y], T.count[pr.y], G,
                      eps, 0.f, f);
#pragma unroll
        for (int i = 0; i < kLmacIn; ++i) X[(long long)p * kLmacIn + i] = f[i];
    }
}

void launch_lmac_record(const NodeArrays& T, const Counters* C, const int* leaf_list, const LmacRecordParams& rp,
                        int blocks, cudaStream_t s) {
    const size_t smem = sizeof(int) * kRecWarps * kRecStack;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(lmac_record_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    lmac_record_kernel<<<blocks, kRecWarps * 32, smem, s>>>(T, C, leaf_list, rp);
}

void launch_lmac_amin(const NodeArrays& T, const Counters* C, const int* leaf_list, const float4* acc,
                      long long max_leaves, cudaStream_t s) {
    long long b = (max_leaves + 255) / 256;
    if (b > 152 * 8) b = 152 * 8;
    if (b < 1) b = 1;
    lmac_amin_kernel<<<(unsigned)b, 256, 0, s>>>(T, C, leaf_list, acc);
}

void launch_lmac_label(const NodeArrays& T, const float4* pos, const float4* plo, const float4* acc,
                       const int2* pairs, int npairs, float G, float eps2, float* r_out, cudaStream_t s) {
    if (npairs <= 0) return;
    long long b = ((long long)npairs * 32 + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    lmac_label_kernel<<<(unsigned)b, 256, 0, s>>>(T, pos, plo, acc, pairs, npairs, G, eps2, r_out);
}

void launch_lmac_features(const NodeArrays& T, const int2* pairs, int npairs, float G, float eps, float* X,
                          cudaStream_t s) {
    if (npairs <= 0) return;
    long long b = ((long long)npairs + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    lmac_feature_kernel<<<(unsigned)b, 256, 0, s>>>(T, pairs, npairs, G, eps, X);
}

}  // namespace ngrav
