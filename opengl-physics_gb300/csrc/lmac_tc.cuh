// lmac_tc.cuh -- evaluation of the learned opening test's network on the
// tensor cores by one CTA of four warps.
//
// Each warp owns 32 rows of a 128-row operand tile; a row carries two
// (group, node) pairs (pair slot p of warp w: row 32w + (p & 31), half p >> 5),
// so one flush evaluates up to 256 pairs:
//   layer 1: D[128 x 64] = A1[128 x 16] * W1t^T      (one MMA, K = 16)
//   ReLU(D + b1) -> BF16 -> A2[128 x 64]               (each warp its rows)
//   layer 2: D[128 x 64] = A2[128 x 64] * W2t^T      (four MMAs, K = 16 each)
//   z = b3 + w3 . ReLU(D + b2)                          (FP32, per row and pair)
// W1t / W2t are block-diagonal (lmac.cuh), so the pair halves never mix.  The
// accumulator lives in 64 tensor-memory columns; warp w reads lanes 32w..32w+31.
// A1 occupies the first 4 KiB of A2 (layer 1 is finished before A2 is written).
#pragma once

#include <cuda_bf16.h>

#include "lmac.cuh"
#include "tc.cuh"

namespace ngrav {

constexpr uint32_t kA1Lbo = 128, kA1Sbo = 256, kA2Lbo = 128, kA2Sbo = 1024;
constexpr uint32_t kLmTmemCols = 64;
constexpr uint32_t kLmWaitPolls = 1u << 26;

struct __align__(1024) LmacTiles {
    uint16_t a2[128 * 64];
    uint16_t w1[64 * 16];
    uint16_t w2[64 * 64];
    float mu[kLmacIn], isd[kLmacIn];
    float b1[kLmacHidden], b2[kLmacHidden], w3[kLmacHidden];
    float b3;
    uint64_t mbar;
    uint32_t tmem;
};

__device__ __forceinline__ LmacTiles* lmac_tiles_at(unsigned char* dyn) {
    const uintptr_t a = (reinterpret_cast<uintptr_t>(dyn) + 1023) & ~uintptr_t(1023);
    return reinterpret_cast<LmacTiles*>(a);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const uint32_t a = __bfloat16_as_ushort(__float2bfloat16_rn(lo));
    const uint32_t b = __bfloat16_as_ushort(__float2bfloat16_rn(hi));
    return a | (b << 16);
}

// Whole CTA: copy the model, clear the operand tile, allocate tensor memory,
// set up the mbarrier.
__device__ __forceinline__ void lmac_tc_init(LmacTiles& S, const LmacDev* __restrict__ M) {
    const int t = threadIdx.x;
    const uint4* w1s = reinterpret_cast<const uint4*>(M->w1t);
    const uint4* w2s = reinterpret_cast<const uint4*>(M->w2t);
    uint4* w1d = reinterpret_cast<uint4*>(S.w1);
    uint4* w2d = reinterpret_cast<uint4*>(S.w2);
    for (int i = t; i < (int)(sizeof(S.w1) / 16); i += blockDim.x) w1d[i] = w1s[i];
    for (int i = t; i < (int)(sizeof(S.w2) / 16); i += blockDim.x) w2d[i] = w2s[i];
    uint4* a2 = reinterpret_cast<uint4*>(S.a2);
    for (int i = t; i < (int)(sizeof(S.a2) / 16); i += blockDim.x) a2[i] = make_uint4(0, 0, 0, 0);
    for (int i = t; i < kLmacIn; i += blockDim.x) {
        S.mu[i] = M->mu[i];
        S.isd[i] = M->isd[i];
    }
    for (int i = t; i < kLmacHidden; i += blockDim.x) {
        S.b1[i] = M->b1[i];
        S.b2[i] = M->b2[i];
        S.w3[i] = M->w3[i];
    }
    if (t == 0) {
        S.b3 = M->b3;
        tc::mbar_init(&S.mbar, 1);
    }
    if ((t >> 5) == 0) tc::tmem_alloc(&S.tmem, kLmTmemCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

// Whole CTA, after the last flush.
__device__ __forceinline__ void lmac_tc_release(LmacTiles& S) {
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if ((threadIdx.x >> 5) == 0) tc::tmem_free(S.tmem, kLmTmemCols);
}

// Standardise and store the raw features of pair slot `slot` of warp `warp`.
__device__ __forceinline__ void lmac_put_features(LmacTiles& S, int warp, int slot, const float f[kLmacIn]) {
    const int row = 32 * warp + (slot & 31);
    const int k0 = 8 * (slot >> 5);
    uint4 v;
    v.x = pack_bf16x2((f[0] - S.mu[0]) * S.isd[0], (f[1] - S.mu[1]) * S.isd[1]);
    v.y = pack_bf16x2((f[2] - S.mu[2]) * S.isd[2], (f[3] - S.mu[3]) * S.isd[3]);
    v.z = pack_bf16x2((f[4] - S.mu[4]) * S.isd[4], (f[5] - S.mu[5]) * S.isd[5]);
    v.w = pack_bf16x2((f[6] - S.mu[6]) * S.isd[6], (f[7] - S.mu[7]) * S.isd[7]);
    *reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(S.a2) + tc::kmajor_offset(row, k0, kA1Lbo, kA1Sbo)) = v;
}

// Whole CTA: evaluate the network on every row of the tile.  Thread (warp w,
// lane l) returns the logits of pair slots l (z0) and l + 32 (z1) of warp w.
// `phase` is the mbarrier parity, advanced twice.  False if a wait ran out.
__device__ __forceinline__ bool lmac_tc_flush(LmacTiles& S, int warp, int lane, uint32_t& phase, float& z0,
                                              float& z1) {
    constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 64);
    const uint32_t a_addr = tc::smem_u32(S.a2), w1_addr = tc::smem_u32(S.w1), w2_addr = tc::smem_u32(S.w2);
    const uint32_t trow = S.tmem + ((uint32_t)(32 * warp) << 16);
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0) {
        tc::mma_bf16(S.tmem, tc::smem_desc(a_addr, kA1Lbo, kA1Sbo), tc::smem_desc(w1_addr, kW1Lbo, kW1Sbo), idesc,
                     false);
        tc::commit(&S.mbar);
    }
    bool ok = tc::mbar_wait(&S.mbar, phase, kLmWaitPolls);
    phase ^= 1u;
    tc::fence_after_sync();
    const int row = 32 * warp + lane;
    unsigned char* a2b = reinterpret_cast<unsigned char*>(S.a2);
    float v[32];
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        tc::tmem_ld32(trow + 32u * half, v);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            uint4 q;
            const int j = 8 * c;
            q.x = pack_bf16x2(fmaxf(v[j + 0] + S.b1[j + 0], 0.f), fmaxf(v[j + 1] + S.b1[j + 1], 0.f));
            q.y = pack_bf16x2(fmaxf(v[j + 2] + S.b1[j + 2], 0.f), fmaxf(v[j + 3] + S.b1[j + 3], 0.f));
            q.z = pack_bf16x2(fmaxf(v[j + 4] + S.b1[j + 4], 0.f), fmaxf(v[j + 5] + S.b1[j + 5], 0.f));
            q.w = pack_bf16x2(fmaxf(v[j + 6] + S.b1[j + 6], 0.f), fmaxf(v[j + 7] + S.b1[j + 7], 0.f));
            *reinterpret_cast<uint4*>(a2b + tc::kmajor_offset(row, 32 * half + j, kA2Lbo, kA2Sbo)) = q;
        }
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int kb = 0; kb < 4; ++kb)
            tc::mma_bf16(S.tmem, tc::smem_desc(a_addr + 2u * kA2Lbo * kb, kA2Lbo, kA2Sbo),
                         tc::smem_desc(w2_addr + 2u * kW2Lbo * kb, kW2Lbo, kW2Sbo), idesc, kb > 0);
        tc::commit(&S.mbar);
    }
    ok = tc::mbar_wait(&S.mbar, phase, kLmWaitPolls) && ok;
    phase ^= 1u;
    tc::fence_after_sync();
    float z[2];
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        tc::tmem_ld32(trow + 32u * half, v);
        float a = S.b3;
#pragma unroll
        for (int j = 0; j < 32; ++j) a = fmaf(S.w3[j], fmaxf(v[j] + S.b2[j], 0.f), a);
        z[half] = a;
    }
    z0 = z[0];
    z1 = z[1];
    return ok;
}

}  // namespace ngrav
