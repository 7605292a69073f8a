// Device code of the preconditioner MLP shared by the trainer (learned.cu) and
// the flexible CG (flexcg.cu): weights staged in shared memory, MMA issue and
// completion, and the forward pass of one 128-node tile on the tensor cores.
#pragma once
#include <cuda_bf16.h>

#include "learned.h"
#include "tc.cuh"

namespace prgpu {

constexpr long long MBAR_LIMIT = 1ll << 22;   // polls of an MMA-completion barrier before giving up

// ---------------------------------------------------------------------------
// shared-memory staging of the weights (bf16, [out][in] row-major in global)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void load_weight_tile(const __nv_bfloat16* __restrict__ w, uint8_t* s, bool transpose) {
    // 64 x 64 bf16; thread t copies rows/columns in 8-element chunks
    for (int e = threadIdx.x; e < 64 * 8; e += blockDim.x) {
        const int row = e >> 3, k0 = (e & 7) * 8;
        if (!transpose) {
            const uint4 v = *reinterpret_cast<const uint4*>(w + row * 64 + k0);
            *reinterpret_cast<uint4*>(s + op_offset(64, row, k0)) = v;
        } else {
            // element (row, k) of W^T is W[k][row]
            __align__(16) __nv_bfloat16 t[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) t[u] = w[(k0 + u) * 64 + row];
            *reinterpret_cast<uint4*>(s + op_offset(64, row, k0)) = *reinterpret_cast<const uint4*>(t);
        }
    }
}

// four MMAs over K = 64: D[tmem] = A (R_A x 64) * B (N x 64)^T
__device__ __forceinline__ void mma_k64(uint32_t d, const uint8_t* a, int ra, const uint8_t* b, int rb, uint32_t idesc,
                                        uint32_t acc0) {
#pragma unroll
    for (int kb = 0; kb < 4; ++kb) {
        const uint64_t ad = smem_desc(smem_u32(a) + kb * ra * 32, 128, 256);
        const uint64_t bd = smem_desc(smem_u32(b) + kb * rb * 32, 128, 256);
        mma_bf16(d, ad, bd, idesc, (kb > 0 || acc0) ? 1u : 0u);
    }
}

// Issue (thread 0), commit, and wait in every thread; false when the wait gave up.
struct MmaSync {
    uint64_t* bar;
    uint32_t phase;
    __device__ bool wait() {
        const bool ok = mbar_wait(bar, phase, MBAR_LIMIT);
        phase ^= 1u;
        return __syncthreads_and(ok ? 1 : 0) != 0;
    }
};

// ---------------------------------------------------------------------------
// forward of one 128-row tile whose features are in sx (operand layout, R = 128).
// 256 threads: warp w reads TMEM lanes 32*(w&3).. and columns 32*(w>>2)..; the
// row's output y is returned to the threads of warps 0-3 (row = threadIdx.x).
// D1 at TMEM column tbase, D2 at tbase + 64.  sx is overwritten with h1.
// ---------------------------------------------------------------------------
struct MlpSmem {
    const uint8_t* w1;   // operand layout, R = 64
    const uint8_t* w2;
    const float* b1;     // 64
    const float* b2;
    const float* w3;
    float b3;
};

__device__ __forceinline__ bool mlp_forward_tile(uint8_t* sx, const MlpSmem& m, uint32_t tbase, MmaSync& ms,
                                                 float* red, float& y) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, q = w & 3, hc = w >> 2;
    const int row = 32 * q + lane, k0 = 32 * hc;
    const uint32_t tl = tbase + ((uint32_t)(32 * q) << 16);
    constexpr uint32_t ID = idesc_bf16_f32(128, 64);
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc_fence_after();
        mma_k64(tbase, sx, 128, m.w1, 64, ID, 0);
        mma_commit(ms.bar);
    }
    if (!ms.wait()) return false;
    tc_fence_after();
    float v[32];
    tmem_ld32(tl + k0, v);
#pragma unroll
    for (int c = 0; c < 32; c += 8) {
        __align__(16) __nv_bfloat16 hb[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) hb[u] = __float2bfloat16_rn(fmaxf(v[c + u] + m.b1[k0 + c + u], 0.f));
        *reinterpret_cast<uint4*>(sx + op_offset(128, row, k0 + c)) = *reinterpret_cast<const uint4*>(hb);
    }
    tc_fence_before();
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc_fence_after();
        mma_k64(tbase + 64, sx, 128, m.w2, 64, ID, 0);
        mma_commit(ms.bar);
    }
    if (!ms.wait()) return false;
    tc_fence_after();
    tmem_ld32(tl + 64 + k0, v);
    float part = 0.f;
#pragma unroll
    for (int c = 0; c < 32; ++c) part = fmaf(fmaxf(v[c] + m.b2[k0 + c], 0.f), m.w3[k0 + c], part);
    red[threadIdx.x] = part;
    tc_fence_before();
    __syncthreads();
    y = (threadIdx.x < 128) ? red[threadIdx.x] + red[threadIdx.x + 128] + m.b3 : 0.f;
    return true;
}

// ---------------------------------------------------------------------------
// standalone forward over feature rows (bf16 [n][64]) -> y[n]
// ---------------------------------------------------------------------------
// The same forward pass for one of several 256-thread groups of a larger block
// (the flexible CG runs three): lt is the thread's index in its group, bar_id
// the group's named barrier (1..15), flag a shared word the group sets when an
// MMA wait gives up.  The group's warps keep the TMEM lane mapping of
// mlp_forward_tile (warp lt/32 reads lanes 32*((lt/32)&3)..), since groups start
// at multiples of 8 warps.
__device__ __forceinline__ void group_sync(int bar_id) {
    asm volatile("bar.sync %0, 256;" ::"r"(bar_id) : "memory");
}
__device__ __forceinline__ bool group_wait(uint64_t* bar, uint32_t& phase, int bar_id, volatile int* flag) {
    if (!mbar_wait(bar, phase, MBAR_LIMIT)) *flag = 1;
    phase ^= 1u;
    group_sync(bar_id);
    return *flag == 0;
}
__device__ __forceinline__ bool mlp_forward_tile_group(uint8_t* sx, const MlpSmem& m, uint32_t tbase, uint64_t* bar,
                                                       uint32_t& phase, float* red, float& y, int lt, int bar_id,
                                                       volatile int* flag) {
    const int w = lt >> 5, lane = lt & 31, q = w & 3, hc = w >> 2;
    const int row = 32 * q + lane, k0 = 32 * hc;
    const uint32_t tl = tbase + ((uint32_t)(32 * q) << 16);
    constexpr uint32_t ID = idesc_bf16_f32(128, 64);
    fence_async_smem();
    group_sync(bar_id);
    if (lt == 0) {
        tc_fence_after();
        mma_k64(tbase, sx, 128, m.w1, 64, ID, 0);
        mma_commit(bar);
    }
    if (!group_wait(bar, phase, bar_id, flag)) return false;
    tc_fence_after();
    float v[32];
    tmem_ld32(tl + k0, v);
    // bias in fp32, then two columns per conversion and per ReLU: rounding to bf16 keeps
    // the sign, so ReLU after rounding gives the values of ReLU before it
    const __nv_bfloat162 zero2 = __floats2bfloat162_rn(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 32; c += 8) {
        __align__(16) __nv_bfloat162 hb[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            hb[u] = __hmax2(__floats2bfloat162_rn(v[c + 2 * u] + m.b1[k0 + c + 2 * u],
                                                  v[c + 2 * u + 1] + m.b1[k0 + c + 2 * u + 1]),
                            zero2);
        *reinterpret_cast<uint4*>(sx + op_offset(128, row, k0 + c)) = *reinterpret_cast<const uint4*>(hb);
    }
    tc_fence_before();
    fence_async_smem();
    group_sync(bar_id);
    if (lt == 0) {
        tc_fence_after();
        mma_k64(tbase + 64, sx, 128, m.w2, 64, ID, 0);
        mma_commit(bar);
    }
    if (!group_wait(bar, phase, bar_id, flag)) return false;
    tc_fence_after();
    tmem_ld32(tl + 64 + k0, v);
    float part = 0.f;
#pragma unroll
    for (int c = 0; c < 32; ++c) part = fmaf(fmaxf(v[c] + m.b2[k0 + c], 0.f), m.w3[k0 + c], part);
    red[lt] = part;
    tc_fence_before();
    group_sync(bar_id);
    y = (lt < 128) ? red[lt] + red[lt + 128] + m.b3 : 0.f;
    return true;
}

__device__ __forceinline__ void stage_mlp_smem(const MlpWeights& wt, uint8_t* sw1, uint8_t* sw2, float* sb, MlpSmem& m) {
    load_weight_tile(wt.w1, sw1, false);
    load_weight_tile(wt.w2, sw2, false);
    for (int k = threadIdx.x; k < 192; k += blockDim.x)
        sb[k] = (k < 64) ? wt.p[P_B1 + k] : (k < 128 ? wt.p[P_B2 + k - 64] : wt.p[P_W3 + k - 128]);
    m.w1 = sw1;
    m.w2 = sw2;
    m.b1 = sb;
    m.b2 = sb + 64;
    m.w3 = sb + 128;
    m.b3 = wt.p[P_B3];
}

}  // namespace prgpu
