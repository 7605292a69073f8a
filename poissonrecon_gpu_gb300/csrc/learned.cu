// Learned preconditioner: a per-node MLP (64 -> 64 -> 64 -> 1, ReLU, BF16
// weights, FP32 accumulation) on the Blackwell tensor cores, its training, and
// the residual/error pairs it is trained on.  The reference has no counterpart:
// it runs plain CG per depth (CG_CUDA.cuh:256-324, driven by main.cu:1237-1329);
// the network only changes how flexible CG (flexcg.cu) picks its directions.
//
// Input of node i at depth d (64 features, 55 used):
//   f[0..26]  r_j / s for its 27 neighbours j (0 where there is none), with
//             s = max_j |r_j| over the neighbours present (i included);
//   f[27..53] c_j = L_d[j] / L_d[centre] where neighbour j is present, else 0
//             (the row's stencil coefficients, normalised);
//   f[54]     d / 16;  f[55..63] = 0.
// Output y; the correction is z_i = s * y / L_d[centre].  Training target: the
// error of a plain-CG iterate, t_i = e_i * L_d[centre] / s with e = x* - x_k.
//
// Tensor-core tiles: 128 nodes per tcgen05.mma (M = 128), N = 64, K = 64 in four
// K-blocks of 16; operands in shared memory in the K-major no-swizzle layout of
// tc.cuh, accumulators in TMEM.  Forward: D1 = X W1^T, D2 = relu(D1 + b1) W2^T.
// Backward (training): dz2 = dy w3 * relu'(z2), dh1 = dz2 W2 (MMA), dz1 = dh1 *
// relu'(z1), and both weight gradients in one M = 128, N = 128 MMA whose A
// stacks dz2^T over dz1^T and whose B stacks h1^T over x^T: the diagonal blocks
// are dW2 = dz2^T h1 and dW1 = dz1^T x, accumulated in TMEM over all tiles of a CTA.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "context.h"
#include "learned.h"
#include "mlp.cuh"
#include "prims.cuh"
#include "tc.cuh"

namespace prgpu {

constexpr int FWD_SMEM = 16384 + 8192 + 8192 + 1024;

__global__ void __launch_bounds__(256, 1) k_mlp_forward(MlpWeights wt, const __nv_bfloat16* __restrict__ feat, i64 n,
                                                        float* __restrict__ y, int* err) {
    extern __shared__ __align__(1024) uint8_t dsm[];
    uint8_t* sx = dsm;
    uint8_t* sw1 = dsm + 16384;
    uint8_t* sw2 = sw1 + 8192;
    __shared__ float sb[192];
    __shared__ float red[256];
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    if (threadIdx.x < 32) {
        tmem_alloc(&tslot, 128);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    MlpSmem m;
    stage_mlp_smem(wt, sw1, sw2, sb, m);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tslot;
    MmaSync ms{&bar, 0};
    bool ok = true;
    const i64 ntiles = (n + 127) / 128;
    for (i64 t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        // features: 128 rows x 128 bytes; thread -> (row, half)
        const int row = threadIdx.x >> 1, h = threadIdx.x & 1;
        const i64 g = t * 128 + row;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int k = 32 * h + 8 * c;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (g < n) v = *reinterpret_cast<const uint4*>(feat + g * 64 + k);
            *reinterpret_cast<uint4*>(sx + op_offset(128, row, k)) = v;
        }
        float yv;
        ok = mlp_forward_tile(sx, m, tbase, ms, red, yv);
        if (ok && threadIdx.x < 128 && t * 128 + threadIdx.x < n) y[t * 128 + threadIdx.x] = yv;
        __syncthreads();
    }
    if (!ok && threadIdx.x == 0) atomicExch(err, PRGPU_ERR_TIMEOUT);
    // every MMA this CTA issued has been waited for (or the CTA gave up above after
    // a bounded wait; wait once more for the last commit before releasing TMEM)
    if (!ok) mbar_wait(&bar, ms.phase ^ 1u, MBAR_LIMIT);   // the commit whose wait gave up
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(tbase, 128);
}

// ---------------------------------------------------------------------------
// training: forward + backward of 128-row tiles, weight gradients accumulated
// in TMEM per CTA, biases and w3 through warp reductions, loss = mean (y - t)^2
// (d loss / d b3 is the sum of dy over the rows)
// ---------------------------------------------------------------------------
// lane l receives sum over the warp's lanes of v[l] (31 shuffles)
__device__ __forceinline__ float warp_transpose_sum(float (&v)[32]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const bool up = (lane & s) != 0;
#pragma unroll
        for (int i = 0; i < s; ++i) {
            const float send = up ? v[i] : v[i + s];
            const float keep = up ? v[i + s] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, s);
        }
    }
    return v[0];
}

constexpr int TR_SX = 0;                   // x tile, R = 128, K = 64           16 KB
constexpr int TR_SH1 = 16384;              // h1 tile                           16 KB
constexpr int TR_SDZ2 = 32768;             // dz2 tile                          16 KB
constexpr int TR_SW1 = 49152;              // W1 (R = 64)                        8 KB
constexpr int TR_SW2 = 57344;              // W2                                 8 KB
constexpr int TR_SW2T = 65536;             // W2^T                               8 KB
constexpr int TR_AWG = 73728;              // [dz2^T; dz1^T], R = 128, K = 128  32 KB
constexpr int TR_BWG = 106496;             // [h1^T; x^T]                       32 KB
constexpr int TRAIN_SMEM = 139264 + 1024;

struct TrainArgs {
    MlpWeights wt;
    const __nv_bfloat16* feat;   // [n][64]
    const float* target;         // [n]
    const int* order;            // sample permutation (nullptr: identity)
    i64 first, n;                // samples order[first .. first+n)
    float scale;                 // d loss / d y = 2 (y - t) * scale
    float* grad;                 // P_COUNT, accumulated with atomics
    double* loss;                // sum of (y - t)^2
    int* err;
};

__global__ void __launch_bounds__(256, 1) k_mlp_train(TrainArgs a) {
    extern __shared__ __align__(1024) uint8_t dsm[];
    uint8_t* sx = dsm + TR_SX;
    uint8_t* sh1 = dsm + TR_SH1;
    uint8_t* sdz2 = dsm + TR_SDZ2;
    uint8_t* awg = dsm + TR_AWG;
    uint8_t* bwg = dsm + TR_BWG;
    __shared__ float sb[192];
    __shared__ float red[256];
    __shared__ float gacc[256];   // db1 | db2 | dw3 | (unused)
    __shared__ float ssum[2];
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    if (threadIdx.x < 32) {
        tmem_alloc(&tslot, 512);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
        ssum[0] = 0.f;
        ssum[1] = 0.f;
    }
    gacc[threadIdx.x] = 0.f;
    MlpSmem m;
    stage_mlp_smem(a.wt, dsm + TR_SW1, dsm + TR_SW2, sb, m);
    load_weight_tile(a.wt.w2, dsm + TR_SW2T, true);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tb = tslot;
    MmaSync ms{&bar, 0};
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, q = w & 3, hc = w >> 2;
    const int row = 32 * q + lane, k0 = 32 * hc;
    const uint32_t tl = tb + ((uint32_t)(32 * q) << 16);
    constexpr uint32_t ID64 = idesc_bf16_f32(128, 64), ID128 = idesc_bf16_f32(128, 128);
    bool ok = true;
    int tiles_done = 0;
    float lsum = 0.f, dysum = 0.f;
    const i64 ntiles = (a.n + 127) / 128;
    for (i64 t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        // ---- x tile and x^T (rows 64..127 of B_wg)
        {
            const int r = threadIdx.x >> 1, h = threadIdx.x & 1;
            const i64 s = t * 128 + r;
            const i64 g = (s < a.n) ? (a.order ? a.order[a.first + s] : a.first + s) : -1;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int k = 32 * h + 8 * c;
                uint4 v = make_uint4(0, 0, 0, 0);
                if (g >= 0) v = *reinterpret_cast<const uint4*>(a.feat + g * 64 + k);
                *reinterpret_cast<uint4*>(sx + op_offset(128, r, k)) = v;
                const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    *reinterpret_cast<__nv_bfloat16*>(bwg + op_offset(128, 64 + k + u, r)) = e[u];
            }
        }
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
            mma_k64(tb, sx, 128, m.w1, 64, ID64, 0);
            mma_commit(ms.bar);
        }
        if (!(ok = ms.wait())) break;
        tc_fence_after();
        // ---- epilogue 1: h1 = relu(z1 + b1) into sh1 and h1^T (rows 0..63 of B_wg)
        float v[32];
        tmem_ld32(tl + k0, v);
        uint32_t mask1 = 0;
#pragma unroll
        for (int c = 0; c < 32; c += 8) {
            __align__(16) __nv_bfloat16 hb[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const float z = v[c + u] + m.b1[k0 + c + u];
                if (z > 0.f) mask1 |= 1u << (c + u);
                hb[u] = __float2bfloat16_rn(fmaxf(z, 0.f));
                *reinterpret_cast<__nv_bfloat16*>(bwg + op_offset(128, k0 + c + u, row)) = hb[u];
            }
            *reinterpret_cast<uint4*>(sh1 + op_offset(128, row, k0 + c)) = *reinterpret_cast<const uint4*>(hb);
        }
        tc_fence_before();
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
            mma_k64(tb + 64, sh1, 128, m.w2, 64, ID64, 0);
            mma_commit(ms.bar);
        }
        if (!(ok = ms.wait())) break;
        tc_fence_after();
        // ---- epilogue 2: y, dy, dz2, dw3, db2
        tmem_ld32(tl + 64 + k0, v);
        float part = 0.f;
#pragma unroll
        for (int c = 0; c < 32; ++c) part = fmaf(fmaxf(v[c] + m.b2[k0 + c], 0.f), m.w3[k0 + c], part);
        red[threadIdx.x] = part;
        __syncthreads();
        const i64 s = t * 128 + row;
        const bool valid = s < a.n;
        float dy = 0.f;
        if (valid) {
            const i64 g = a.order ? a.order[a.first + s] : a.first + s;
            const float y = red[row] + red[row + 128] + m.b3;
            const float d = y - a.target[g];
            dy = 2.f * d * a.scale;
            if (hc == 0) {
                lsum += d * d;
                dysum += dy;
            }
        }
        float gw3[32], gb2[32];
#pragma unroll
        for (int c = 0; c < 32; c += 8) {
            __align__(16) __nv_bfloat16 db[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const float z = v[c + u] + m.b2[k0 + c + u];
                const float h2 = fmaxf(z, 0.f);
                const float dz = (z > 0.f) ? dy * m.w3[k0 + c + u] : 0.f;
                gw3[c + u] = dy * h2;
                gb2[c + u] = dz;
                db[u] = __float2bfloat16_rn(dz);
                *reinterpret_cast<__nv_bfloat16*>(awg + op_offset(128, k0 + c + u, row)) = db[u];
            }
            *reinterpret_cast<uint4*>(sdz2 + op_offset(128, row, k0 + c)) = *reinterpret_cast<const uint4*>(db);
        }
        atomicAdd(&gacc[128 + k0 + lane], warp_transpose_sum(gw3));
        atomicAdd(&gacc[64 + k0 + lane], warp_transpose_sum(gb2));
        tc_fence_before();
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
            mma_k64(tb + 128, sdz2, 128, dsm + TR_SW2T, 64, ID64, 0);   // dh1 = dz2 W2
            mma_commit(ms.bar);
        }
        if (!(ok = ms.wait())) break;
        tc_fence_after();
        // ---- epilogue 3: dz1 = dh1 * relu'(z1) into dz1^T (rows 64..127 of A_wg), db1
        tmem_ld32(tl + 128 + k0, v);
        float gb1[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) {
            const float dz = (mask1 >> c & 1u) ? v[c] : 0.f;
            const __nv_bfloat16 b = __float2bfloat16_rn(dz);
            gb1[c] = dz;
            *reinterpret_cast<__nv_bfloat16*>(awg + op_offset(128, 64 + k0 + c, row)) = b;
        }
        atomicAdd(&gacc[k0 + lane], warp_transpose_sum(gb1));
        tc_fence_before();
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
            // [dW2 .; . dW1] += A_wg (128 x K=128) * B_wg (128 x K=128)^T
#pragma unroll
            for (int kb = 0; kb < 8; ++kb) {
                const uint64_t ad = smem_desc(smem_u32(awg) + kb * 128 * 32, 128, 256);
                const uint64_t bd = smem_desc(smem_u32(bwg) + kb * 128 * 32, 128, 256);
                mma_bf16(tb + 256, ad, bd, ID128, (kb > 0 || tiles_done > 0) ? 1u : 0u);
            }
            mma_commit(ms.bar);
        }
        if (!(ok = ms.wait())) break;
        tc_fence_after();
        ++tiles_done;
    }
    if (ok && tiles_done > 0) {
        // weight gradients: rows 0..63 x columns 0..63 (dW2), rows 64..127 x columns 64..127 (dW1)
        const bool upper = q < 2;            // TMEM lanes 0..63
        const int col = (upper ? 0 : 64) + k0;
        float v[32];
        tmem_ld32(tl + 256 + col, v);
        const int out = row & 63;
        float* g = a.grad + (upper ? P_W2 : P_W1) + out * 64 + k0;
#pragma unroll
        for (int c = 0; c < 32; ++c) atomicAdd(g + c, v[c]);
    }
    atomicAdd(&ssum[0], lsum);
    atomicAdd(&ssum[1], dysum);
    tc_fence_before();
    __syncthreads();
    if (ok && tiles_done > 0) {
        const int k = threadIdx.x;
        if (k < 64) atomicAdd(a.grad + P_B1 + k, gacc[k]);
        else if (k < 128) atomicAdd(a.grad + P_B2 + k - 64, gacc[k]);
        else if (k < 192) atomicAdd(a.grad + P_W3 + k - 128, gacc[k]);
        if (threadIdx.x == 0) {
            atomicAdd(a.loss, (double)ssum[0]);
            atomicAdd(a.grad + P_B3, ssum[1]);
        }
    }
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(a.err, PRGPU_ERR_TIMEOUT);
        mbar_wait(&bar, ms.phase ^ 1u, MBAR_LIMIT);   // the commit whose wait gave up
    }
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(tb, 512);
}

// Adam on the fp32 parameters; bf16 mirrors of W1 and W2 refreshed; gradients zeroed
__global__ void k_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ mo, float* __restrict__ ve,
                       __nv_bfloat16* __restrict__ w1b, __nv_bfloat16* __restrict__ w2b, float lr, float b1c,
                       float b2c) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P_COUNT; k += gridDim.x * blockDim.x) {
        const float gr = g[k];
        const float m = 0.9f * mo[k] + 0.1f * gr;
        const float v = 0.999f * ve[k] + 0.001f * gr * gr;
        mo[k] = m;
        ve[k] = v;
        const float upd = lr * (m / b1c) / (sqrtf(v / b2c) + 1e-8f);
        const float nv = p[k] - upd;
        p[k] = nv;
        g[k] = 0.f;
        if (k < P_B1) w1b[k - P_W1] = __float2bfloat16_rn(nv);
        else if (k >= P_W2 && k < P_B2) w2b[k - P_W2] = __float2bfloat16_rn(nv);
    }
}

__global__ void k_mirror_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ w1b,
                              __nv_bfloat16* __restrict__ w2b) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 4096; k += gridDim.x * blockDim.x) {
        w1b[k] = __float2bfloat16_rn(p[P_W1 + k]);
        w2b[k] = __float2bfloat16_rn(p[P_W2 + k]);
    }
}

// ---------------------------------------------------------------------------
// residual/error pairs from the plain solver
// ---------------------------------------------------------------------------
// r = b - A x over all rows, FP64 accumulation of the 27 stencil products
__global__ void k_residual(const int* __restrict__ neigh, i64 M, const float* __restrict__ st, const int8_t* __restrict__ depth,
                           const float* __restrict__ b, const float* __restrict__ x, float* __restrict__ r) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (i64)gridDim.x * blockDim.x) {
        const float* s = st + 27 * depth[i];
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < 27; ++j) {
            const int nb = neigh[(i64)j * M + i];
            if (nb != -1) acc += (double)s[j] * (double)x[nb];
        }
        r[i] = (float)((double)b[i] - acc);
    }
}

// the 64 features of node i from r at its neighbours (learned.h feature layout);
// returns the scale s (0: no residual around the node)
__device__ __forceinline__ float node_features(const int* __restrict__ neigh, i64 M, i64 i, const float* __restrict__ r,
                                               const float* __restrict__ cnorm, int d, float (&f)[64]) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 27; ++j) {
        const int nb = neigh[(i64)j * M + i];
        const float v = (nb != -1) ? r[nb] : 0.f;
        f[j] = v;
        f[27 + j] = (nb != -1) ? cnorm[j] : 0.f;
        s = fmaxf(s, fabsf(v));
    }
    const float inv = s > 0.f ? 1.f / s : 0.f;
#pragma unroll
    for (int j = 0; j < 27; ++j) f[j] *= inv;
    f[54] = (float)d * (1.f / 16.f);
#pragma unroll
    for (int j = 55; j < 64; ++j) f[j] = 0.f;
    return s;
}

struct RecordArgs {
    const int* neigh;
    i64 M;
    const float* r;          // residual of the iterate
    const float* xk;         // the iterate
    const float* xs;         // converged solution
    const float* cnorm;      // 27 per depth: L_d[j] / L_d[13]
    const float* centre;     // per depth: L_d[13]
    const i64* rows;         // sampled rows
    const int* rdepth;       // their depths
    i64 n;
    float clip;
    __nv_bfloat16* feat;     // out: [n][64] at the dataset's end
    float* target;
};

__global__ void k_record(RecordArgs a) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < a.n; k += (i64)gridDim.x * blockDim.x) {
        const i64 i = a.rows[k];
        const int d = a.rdepth[k];
        float f[64];
        const float s = node_features(a.neigh, a.M, i, a.r, a.cnorm + 27 * d, d, f);
        __align__(16) __nv_bfloat16 fb[64];
#pragma unroll
        for (int j = 0; j < 64; ++j) fb[j] = __float2bfloat16_rn(f[j]);
#pragma unroll
        for (int c = 0; c < 8; ++c) reinterpret_cast<uint4*>(a.feat + k * 64)[c] = reinterpret_cast<const uint4*>(fb)[c];
        const float e = a.xs[i] - a.xk[i];
        float t = s > 0.f ? e * a.centre[d] / s : 0.f;
        t = fminf(fmaxf(t, -a.clip), a.clip);
        a.target[k] = t;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
void init_params(std::vector<float>& p, uint64_t seed) {
    p.assign(P_COUNT, 0.f);
    uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
    auto uni = [&]() {   // uniform in [-1, 1)
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return (float)((double)(st >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
    };
    // He-uniform for the ReLU layers; the output layer starts small
    const float a1 = std::sqrt(6.f / 55.f), a2 = std::sqrt(6.f / 64.f);
    for (int o = 0; o < 64; ++o)
        for (int i = 0; i < 64; ++i) p[P_W1 + o * 64 + i] = (i < FEAT_USED) ? a1 * uni() : 0.f;
    for (int k = 0; k < 4096; ++k) p[P_W2 + k] = a2 * uni();
    for (int k = 0; k < 64; ++k) p[P_W3 + k] = 0.1f * a2 * uni();
}

Trainer::Trainer(int dev, uint64_t s) : device(dev), seed(s) {
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaMalloc(&p, P_COUNT * sizeof(float)));
    CK(cudaMalloc(&g, P_COUNT * sizeof(float)));
    CK(cudaMalloc(&mo, P_COUNT * sizeof(float)));
    CK(cudaMalloc(&ve, P_COUNT * sizeof(float)));
    CK(cudaMalloc(&w1b, 4096 * sizeof(__nv_bfloat16)));
    CK(cudaMalloc(&w2b, 4096 * sizeof(__nv_bfloat16)));
    CK(cudaMalloc(&loss, sizeof(double)));
    CK(cudaMalloc(&err, sizeof(int)));
    std::vector<float> h;
    init_params(h, seed);
    set_params(h.data(), nullptr, nullptr);
    CK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, TRAIN_SMEM));
    CK(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, FWD_SMEM));
}

Trainer::~Trainer() {
    cudaSetDevice(device);
    cudaStreamSynchronize(stream);
    for (void* q : {(void*)p, (void*)g, (void*)mo, (void*)ve, (void*)w1b, (void*)w2b, (void*)loss, (void*)err,
                    (void*)feat, (void*)target, (void*)order})
        if (q) cudaFree(q);
    cudaStreamDestroy(stream);
}

void Trainer::set_params(const float* hp, const float* hm, const float* hv) {
    CK(cudaMemcpyAsync(p, hp, P_COUNT * sizeof(float), cudaMemcpyHostToDevice, stream));
    if (hm) CK(cudaMemcpyAsync(mo, hm, P_COUNT * sizeof(float), cudaMemcpyHostToDevice, stream));
    else CK(cudaMemsetAsync(mo, 0, P_COUNT * sizeof(float), stream));
    if (hv) CK(cudaMemcpyAsync(ve, hv, P_COUNT * sizeof(float), cudaMemcpyHostToDevice, stream));
    else CK(cudaMemsetAsync(ve, 0, P_COUNT * sizeof(float), stream));
    CK(cudaMemsetAsync(g, 0, P_COUNT * sizeof(float), stream));
    k_mirror_bf16<<<16, 256, 0, stream>>>(p, w1b, w2b);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(stream));
}

void Trainer::reserve(i64 want) {
    if (want <= cap) return;
    const i64 nc = std::max<i64>(want, cap + cap / 2 + (1 << 16));
    __nv_bfloat16* nf = nullptr;
    float* nt = nullptr;
    CK(cudaMalloc(&nf, (size_t)nc * 64 * sizeof(__nv_bfloat16)));
    CK(cudaMalloc(&nt, (size_t)nc * sizeof(float)));
    if (nsamples) {
        CK(cudaMemcpyAsync(nf, feat, (size_t)nsamples * 128, cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemcpyAsync(nt, target, (size_t)nsamples * 4, cudaMemcpyDeviceToDevice, stream));
        CK(cudaStreamSynchronize(stream));
    }
    if (feat) cudaFree(feat);
    if (target) cudaFree(target);
    feat = nf;
    target = nt;
    cap = nc;
}

MlpWeights Trainer::weights() const {
    MlpWeights w;
    w.w1 = w1b;
    w.w2 = w2b;
    w.p = p;
    return w;
}

// one pass of the training kernel over samples order[first .. first+n) (or the
// given arrays); gradients accumulate into g, the loss sum into *loss
static void run_train_pass(Trainer& T, const __nv_bfloat16* feat, const float* target, const int* order, i64 first, i64 n,
                           float scale) {
    cudaStream_t s = T.stream;
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, T.device));
    const i64 ntiles = (n + 127) / 128;
    const int grid = (int)std::max<i64>(1, std::min<i64>(ntiles, sms));
    TrainArgs a;
    a.wt = T.weights();
    a.feat = feat;
    a.target = target;
    a.order = order;
    a.first = first;
    a.n = n;
    a.scale = scale;
    a.grad = T.g;
    a.loss = T.loss;
    a.err = T.err;
    k_mlp_train<<<grid, 256, TRAIN_SMEM, s>>>(a);
    CK_LAUNCH();
}

static void check_err(Trainer& T) {
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, T.err, sizeof(int), cudaMemcpyDeviceToHost, T.stream));
    CK(cudaStreamSynchronize(T.stream));
    if (herr) {
        CK(cudaMemsetAsync(T.err, 0, sizeof(int), T.stream));
        set_last_error("tensor-core MMA completion wait gave up");
        throw Error{PRGPU_ERR_TIMEOUT, {0}};
    }
}

double Trainer::train(int steps, int batch, float lr) {
    if (nsamples < 1) {
        set_last_error("the trainer holds no samples");
        throw Error{PRGPU_ERR_ARG, {0}};
    }
    cudaStream_t s = stream;
    CK(cudaMemsetAsync(err, 0, sizeof(int), s));
    const i64 B = std::min<i64>(batch, nsamples);
    double total = 0.0;
    std::vector<int> perm;
    for (int it = 0; it < steps; ++it) {
        if (!order || cursor + B > nsamples) {   // new epoch: host shuffle of the sample order
            perm.resize(nsamples);
            for (i64 k = 0; k < nsamples; ++k) perm[k] = (int)k;
            uint64_t st = seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(epoch + 1));
            for (i64 k = nsamples - 1; k > 0; --k) {
                st = st * 6364136223846793005ull + 1442695040888963407ull;
                const i64 j = (i64)((st >> 17) % (uint64_t)(k + 1));
                std::swap(perm[k], perm[j]);
            }
            if (order) cudaFree(order);
            CK(cudaMalloc(&order, nsamples * sizeof(int)));
            CK(cudaMemcpyAsync(order, perm.data(), nsamples * sizeof(int), cudaMemcpyHostToDevice, s));
            CK(cudaStreamSynchronize(s));
            cursor = 0;
            ++epoch;
        }
        CK(cudaMemsetAsync(loss, 0, sizeof(double), s));
        run_train_pass(*this, feat, target, order, cursor, B, 1.f / (float)B);
        cursor += B;
        ++step;
        const float b1c = 1.f - std::pow(0.9f, (float)step), b2c = 1.f - std::pow(0.999f, (float)step);
        k_adam<<<(P_COUNT + 255) / 256, 256, 0, s>>>(p, g, mo, ve, w1b, w2b, lr, b1c, b2c);
        CK_LAUNCH();
        if (it == steps - 1 || (it & 63) == 63) {
            double l = 0;
            CK(cudaMemcpyAsync(&l, loss, sizeof(double), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            total = l / (double)B;
        }
    }
    check_err(*this);
    return total;
}

double Trainer::gradients(const __nv_bfloat16* dfeat, const float* dtarget, i64 n, float* hgrad) {
    cudaStream_t s = stream;
    CK(cudaMemsetAsync(err, 0, sizeof(int), s));
    CK(cudaMemsetAsync(g, 0, P_COUNT * sizeof(float), s));
    CK(cudaMemsetAsync(loss, 0, sizeof(double), s));
    run_train_pass(*this, dfeat, dtarget, nullptr, 0, n, 1.f / (float)n);
    double l = 0;
    CK(cudaMemcpyAsync(hgrad, g, P_COUNT * sizeof(float), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&l, loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemsetAsync(g, 0, P_COUNT * sizeof(float), s));
    check_err(*this);
    return l / (double)n;
}

void Trainer::forward(const __nv_bfloat16* dfeat, i64 n, float* dy) {
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    CK(cudaMemsetAsync(err, 0, sizeof(int), stream));
    const int grid = (int)std::max<i64>(1, std::min<i64>((n + 127) / 128, sms));
    k_mlp_forward<<<grid, 256, FWD_SMEM, stream>>>(weights(), dfeat, n, dy, err);
    CK_LAUNCH();
    check_err(*this);
}

// normalised stencil rows and centre coefficients of a context, per depth
static void stencil_features(const Ctx& c, std::vector<float>& cn, std::vector<float>& centre) {
    cn.assign(27 * (c.D + 1), 0.f);
    centre.assign(c.D + 1, 0.f);
    for (int d = 0; d <= c.D; ++d) {
        const float ctr = c.stencil[27 * d + 13];
        centre[d] = ctr;
        for (int j = 0; j < 27; ++j) cn[27 * d + j] = ctr != 0.f ? c.stencil[27 * d + j] / ctr : 0.f;
    }
}

// Records residual/error pairs of plain CG on the context's system (its
// right-hand side must exist): x* from a solve to relative 1e-7, then the
// iterates after k = 1, 2, 3, 5, 8, 12, 20 iterations; per depth >= 1 and iterate,
// rows_per_depth rows drawn at random.  The context's x is left at x*.
i64 Trainer::record(Ctx& c, int rows_per_depth) {
    cudaStream_t s = c.stream;
    const i64 M = c.nodes.M;
    const prgpu_params saved = c.params;
    c.params.solve_mode = PRGPU_SOLVE_RELATIVE;
    c.params.cg_tol = 1e-7;
    c.params.cg_max_iter = 10000;
    c.params.cascadic = 0;
    stage_solve_depths(c, 0, c.D, PRGPU_SOLVE_RELATIVE);
    float* xs = dalloc<float>(M, s);
    CK(cudaMemcpyAsync(xs, c.x, M * sizeof(float), cudaMemcpyDeviceToDevice, s));
    std::vector<float> cn, centre;
    stencil_features(c, cn, centre);
    float* dcn = dalloc<float>((i64)cn.size(), s);
    float* dcentre = dalloc<float>((i64)centre.size(), s);
    float* dst = dalloc<float>((i64)c.stencil.size(), s);
    CK(cudaMemcpyAsync(dcn, cn.data(), cn.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dcentre, centre.data(), centre.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dst, c.stencil.data(), c.stencil.size() * 4, cudaMemcpyHostToDevice, s));
    float* r = dalloc<float>(M, s);
    const int snaps[] = {1, 2, 3, 5, 8, 12, 20};
    i64 added = 0;
    uint64_t st = seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(++record_calls));
    auto rnd = [&]() {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return st >> 17;
    };
    for (int k : snaps) {
        c.params.cg_max_iter = k;
        stage_solve_depths(c, 0, c.D, PRGPU_SOLVE_RELATIVE);
        k_residual<<<grid_for(M, 256), 256, 0, s>>>(c.nodes.neigh, M, dst, c.nodes.depth, c.divergence, c.x, r);
        CK_LAUNCH();
        std::vector<i64> rows;
        std::vector<int> rd;
        for (int d = 1; d <= c.D; ++d) {
            if (c.count[d] < 8) continue;
            const int want = (int)std::min<i64>(rows_per_depth, c.count[d]);
            for (int j = 0; j < want; ++j) {
                rows.push_back(c.base[d] + (i64)(rnd() % (uint64_t)c.count[d]));
                rd.push_back(d);
            }
        }
        const i64 n = (i64)rows.size();
        if (!n) continue;
        CK(cudaStreamSynchronize(s));   // the previous iterate's samples are written before a regrow copies them
        reserve(nsamples + n);
        i64* drows = dalloc<i64>(n, s);
        int* drd = dalloc<int>(n, s);
        CK(cudaMemcpyAsync(drows, rows.data(), n * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(drd, rd.data(), n * 4, cudaMemcpyHostToDevice, s));
        RecordArgs a;
        a.neigh = c.nodes.neigh;
        a.M = M;
        a.r = r;
        a.xk = c.x;
        a.xs = xs;
        a.cnorm = dcn;
        a.centre = dcentre;
        a.rows = drows;
        a.rdepth = drd;
        a.n = n;
        a.clip = TARGET_CLIP;
        a.feat = feat + nsamples * 64;
        a.target = target + nsamples;
        k_record<<<grid_for(n, 128), 128, 0, s>>>(a);
        CK_LAUNCH();
        // rows with no residual around them (s = 0) stay: zero features and target, as the
        // solver treats them (z = 0)
        nsamples += n;
        added += n;
        dfree(drows, s);
        dfree(drd, s);
    }
    CK(cudaMemcpyAsync(c.x, xs, M * sizeof(float), cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    dfree(r, s);
    dfree(dcn, s);
    dfree(dcentre, s);
    dfree(dst, s);
    dfree(xs, s);
    c.params = saved;
    return added;
}

// checkpoint: "PRGPULPC", u32 version, u32 features, u32 hidden, u32 parameter count,
// i64 step, u64 seed, i64 epoch, f32 parameters, f32 Adam first and second moments
void Trainer::save(const char* path) {
    std::vector<float> hp(P_COUNT), hm(P_COUNT), hv(P_COUNT);
    CK(cudaMemcpyAsync(hp.data(), p, P_COUNT * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hm.data(), mo, P_COUNT * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hv.data(), ve, P_COUNT * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    write_checkpoint(path, hp.data(), hm.data(), hv.data(), step, seed, epoch);
}

void Trainer::load(const char* path) {
    std::vector<float> hp, hm, hv;
    i64 st = 0, ep = 0;
    uint64_t sd = 0;
    read_checkpoint(path, hp, hm, hv, st, sd, ep);
    set_params(hp.data(), hm.data(), hv.data());
    step = st;
    seed = sd;
    epoch = ep;
    cursor = 0;
    if (order) {
        cudaFree(order);
        order = nullptr;
    }
}

static const char CKPT_MAGIC[8] = {'P', 'R', 'G', 'P', 'U', 'L', 'P', 'C'};

void write_checkpoint(const char* path, const float* hp, const float* hm, const float* hv, i64 step, uint64_t seed,
                      i64 epoch) {
    FILE* f = fopen(path, "wb");
    if (!f) {
        set_last_error("cannot write %s", path);
        throw Error{PRGPU_ERR_IO, {0}};
    }
    const uint32_t hdr[4] = {CKPT_VERSION, 64, 64, (uint32_t)P_COUNT};
    bool ok = fwrite(CKPT_MAGIC, 1, 8, f) == 8 && fwrite(hdr, 4, 4, f) == 4 && fwrite(&step, 8, 1, f) == 1 &&
              fwrite(&seed, 8, 1, f) == 1 && fwrite(&epoch, 8, 1, f) == 1 &&
              fwrite(hp, 4, P_COUNT, f) == (size_t)P_COUNT && fwrite(hm, 4, P_COUNT, f) == (size_t)P_COUNT &&
              fwrite(hv, 4, P_COUNT, f) == (size_t)P_COUNT;
    ok = (fclose(f) == 0) && ok;
    if (!ok) {
        set_last_error("short write to %s", path);
        throw Error{PRGPU_ERR_IO, {0}};
    }
}

void read_checkpoint(const char* path, std::vector<float>& hp, std::vector<float>& hm, std::vector<float>& hv, i64& step,
                     uint64_t& seed, i64& epoch) {
    FILE* f = fopen(path, "rb");
    if (!f) {
        set_last_error("cannot read %s", path);
        throw Error{PRGPU_ERR_IO, {0}};
    }
    char mg[8];
    uint32_t hdr[4];
    hp.resize(P_COUNT);
    hm.resize(P_COUNT);
    hv.resize(P_COUNT);
    bool ok = fread(mg, 1, 8, f) == 8 && memcmp(mg, CKPT_MAGIC, 8) == 0 && fread(hdr, 4, 4, f) == 4 &&
              hdr[0] == CKPT_VERSION && hdr[1] == 64 && hdr[2] == 64 && hdr[3] == (uint32_t)P_COUNT &&
              fread(&step, 8, 1, f) == 1 && fread(&seed, 8, 1, f) == 1 && fread(&epoch, 8, 1, f) == 1 &&
              fread(hp.data(), 4, P_COUNT, f) == (size_t)P_COUNT && fread(hm.data(), 4, P_COUNT, f) == (size_t)P_COUNT &&
              fread(hv.data(), 4, P_COUNT, f) == (size_t)P_COUNT;
    fclose(f);
    if (!ok) {
        set_last_error("%s is not a preconditioner checkpoint (version %u, 64x64)", path, CKPT_VERSION);
        throw Error{PRGPU_ERR_IO, {0}};
    }
    for (float v : hp)
        if (!std::isfinite(v)) {
            set_last_error("%s holds non-finite weights", path);
            throw Error{PRGPU_ERR_IO, {0}};
        }
}

}  // namespace prgpu
