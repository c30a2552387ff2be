// walk_common.cuh -- warp-level pieces shared by the traversal kernels:
// warp prefix sums and appends to chunked interaction lists.
#pragma once

#include "engine.cuh"

namespace ngrav {

__device__ __forceinline__ int warp_excl_scan(int v, int lane, int& total) {
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

// Warp-uniform state of one chunked list being appended to, with a private
// reservoir of chunk ids so the pool counter sees one atomic per kReserve
// chunks instead of one per chunk.
constexpr int kReserve = 16;
struct ChunkList {
    int first, cur, pos, count;
    int res_next, res_end;
};

__device__ __forceinline__ int alloc_chunk(ChunkList& L, int* counter, int lane) {
    if (L.res_next == L.res_end) {
        int c = 0;
        if (lane == 0) c = atomicAdd(counter, kReserve);
        L.res_next = __shfl_sync(0xffffffffu, c, 0);
        L.res_end = L.res_next + kReserve;
    }
    return L.res_next++;
}

// Lanes with `has` append `val`, in lane order.  Chunks beyond the pool are
// still counted (so the host learns what a retry needs) but not written.
__device__ __forceinline__ void list_append(ChunkList& L, bool has, int val, int* __restrict__ pool,
                                            int* __restrict__ next, int* counter, int cap, int lane,
                                            unsigned lt_mask, unsigned& bad) {
    const unsigned m = __ballot_sync(0xffffffffu, has);
    const int k = __popc(m);
    if (k == 0) return;
    if (L.cur < 0) {
        L.cur = L.first = alloc_chunk(L, counter, lane);
        L.pos = 0;
    }
    int newc = -1;
    if (L.pos + k > kListChunk) {
        newc = alloc_chunk(L, counter, lane);
        if (lane == 0 && L.cur < cap) next[L.cur] = newc;
    }
    if (has) {
        const int i = L.pos + __popc(m & lt_mask);
        const int c = i < kListChunk ? L.cur : newc;
        const int p = i < kListChunk ? i : i - kListChunk;
        if (c < cap)
            pool[(long long)c * kListChunk + p] = val;
        else
            bad |= kStListOverflow;
    }
    if (newc >= 0) {
        L.cur = newc;
        L.pos = L.pos + k - kListChunk;
    } else {
        L.pos += k;
    }
    L.count += k;
}

// Two candidates per lane (v0 then v1), appended as one batch of up to 64:
// all v0 in lane order, then all v1.  One chunk-boundary check for both.
__device__ __forceinline__ void list_append2(ChunkList& L, bool has0, int v0, bool has1, int v1,
                                             int* __restrict__ pool, int* __restrict__ next, int* counter, int cap,
                                             int lane, unsigned lt_mask, unsigned& bad) {
    const unsigned m0 = __ballot_sync(0xffffffffu, has0);
    const unsigned m1 = __ballot_sync(0xffffffffu, has1);
    const int k0 = __popc(m0);
    const int k = k0 + __popc(m1);
    if (k == 0) return;
    if (L.cur < 0) {
        L.cur = L.first = alloc_chunk(L, counter, lane);
        L.pos = 0;
    }
    int newc = -1;
    if (L.pos + k > kListChunk) {  // k <= 64 < kListChunk: at most one new chunk
        newc = alloc_chunk(L, counter, lane);
        if (lane == 0 && L.cur < cap) next[L.cur] = newc;
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        if (q == 0 ? has0 : has1) {
            const int i = L.pos + (q == 0 ? __popc(m0 & lt_mask) : k0 + __popc(m1 & lt_mask));
            const int c = i < kListChunk ? L.cur : newc;
            const int p = i < kListChunk ? i : i - kListChunk;
            if (c < cap)
                pool[(long long)c * kListChunk + p] = q == 0 ? v0 : v1;
            else
                bad |= kStListOverflow;
        }
    }
    if (newc >= 0) {
        L.cur = newc;
        L.pos = L.pos + k - kListChunk;
    } else {
        L.pos += k;
    }
    L.count += k;
}

}  // namespace ngrav
