// Device primitives: exclusive scan, stable LSD radix sort of (u64 key, u32
// value) pairs with a shared-memory digit-binned scatter, and compaction.
// All work on the caller's stream; temporary memory comes from the stream's
// memory pool (cudaMallocAsync).
#pragma once
#include <utility>
#include <vector>

#include "common.cuh"

namespace prgpu {

// ------------------------------- memory ------------------------------------
// The device allocations an API call has made on this host thread and not yet
// freed (null outside a call); when the call fails, it frees the ones its stages
// left behind.
struct LiveAllocs {
    std::vector<std::pair<void*, cudaStream_t>> v;
};
extern thread_local LiveAllocs* g_live;
// PRGPU_HOOK_FAIL_ALLOC: allocations left before the one that fails (0: off)
extern std::atomic<long long> g_fail_alloc_countdown;

template <class T>
inline T* dalloc(i64 n, cudaStream_t s) {
    void* p = nullptr;
    if (n <= 0) n = 1;
    if (g_fail_alloc_countdown.load(std::memory_order_relaxed) > 0 && --g_fail_alloc_countdown == 0) {
        set_last_error("cudaMallocAsync(%lld bytes): failure injected by PRGPU_HOOK_FAIL_ALLOC",
                       (long long)((size_t)n * sizeof(T)));
        throw Error{PRGPU_ERR_NOMEM, {0}};
    }
    cudaError_t e = cudaMallocAsync(&p, (size_t)n * sizeof(T), s);
    if (e != cudaSuccess) {
        set_last_error("cudaMallocAsync(%lld bytes): %s", (long long)((size_t)n * sizeof(T)),
                       cudaGetErrorString(e));
        throw Error{PRGPU_ERR_NOMEM, {0}};
    }
    if (g_live) g_live->v.emplace_back(p, s);
    return (T*)p;
}
template <class T>
inline void dfree(T*& p, cudaStream_t s) {
    if (p) {
        if (g_live)
            for (size_t k = g_live->v.size(); k-- > 0;)
                if (g_live->v[k].first == (void*)p) {
                    g_live->v.erase(g_live->v.begin() + (long)k);
                    break;
                }
        cudaFreeAsync((void*)p, s);
    }
    p = nullptr;
}

// ------------------------------- scan ---------------------------------------
constexpr int SCAN_BLOCK = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

template <class T>
__device__ __forceinline__ T block_exclusive_sum(T v, T* smem_warp, T* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        T w = lane < nw ? smem_warp[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) smem_warp[lane] = w;
    }
    __syncthreads();
    T warp_off = warp ? smem_warp[warp - 1] : T(0);
    *total = smem_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_off + x - v;
}

template <class TI, class TO>
__global__ void k_tile_reduce(const TI* __restrict__ in, i64 n, TO* __restrict__ partial) {
    __shared__ TO sw[32];
    i64 base = (i64)blockIdx.x * SCAN_TILE + (i64)threadIdx.x * SCAN_ITEMS;
    TO s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) s += (TO)in[base + k];
    TO tot;
    block_exclusive_sum<TO>(s, sw, &tot);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

template <class TI, class TO>
__global__ void k_tile_scan(const TI* __restrict__ in, i64 n, TO* __restrict__ out,
                            const TO* __restrict__ partial_scanned, TO* __restrict__ total_out) {
    __shared__ TO sw[32];
    i64 base = (i64)blockIdx.x * SCAN_TILE + (i64)threadIdx.x * SCAN_ITEMS;
    TO v[SCAN_ITEMS];
    TO s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = (base + k < n) ? (TO)in[base + k] : TO(0);
        s += v[k];
    }
    TO tot;
    TO pre = block_exclusive_sum<TO>(s, sw, &tot);
    TO off = partial_scanned ? partial_scanned[blockIdx.x] : TO(0);
    TO run = off + pre;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) *total_out = run;
}

// out[i] = sum_{k<i} in[k]; *total_dev (device pointer, optional) receives the sum.
// 'in' and 'out' may alias.
template <class TI, class TO>
void exclusive_scan(const TI* in, TO* out, i64 n, TO* total_dev, cudaStream_t s) {
    if (n <= 0) {
        if (total_dev) CK(cudaMemsetAsync(total_dev, 0, sizeof(TO), s));
        return;
    }
    i64 nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb == 1) {
        k_tile_scan<TI, TO><<<1, SCAN_BLOCK, 0, s>>>(in, n, out, nullptr, total_dev);
        CK_LAUNCH();
        return;
    }
    TO* part = dalloc<TO>(nb, s);
    k_tile_reduce<TI, TO><<<(unsigned)nb, SCAN_BLOCK, 0, s>>>(in, n, part);
    CK_LAUNCH();
    exclusive_scan<TO, TO>(part, part, nb, (TO*)nullptr, s);
    k_tile_scan<TI, TO><<<(unsigned)nb, SCAN_BLOCK, 0, s>>>(in, n, out, part, total_dev);
    CK_LAUNCH();
    dfree(part, s);
}

// ----------------------------- radix sort -----------------------------------
constexpr int RS_BLOCK = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_BLOCK * RS_ITEMS;
constexpr int RS_BINS = 256;

static __global__ void k_rs_hist(const u64* __restrict__ keys, i64 n, int shift, u64 mask, unsigned* __restrict__ hist,
                          int nblocks) {
    __shared__ unsigned h[RS_BINS];
    h[threadIdx.x] = 0;
    __syncthreads();
    i64 base = (i64)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int i = 0; i < RS_ITEMS; ++i) {
        i64 e = base + (i64)i * RS_BLOCK + threadIdx.x;
        if (e < n) atomicAdd(&h[(unsigned)((keys[e] >> shift) & mask)], 1u);
    }
    __syncthreads();
    hist[(i64)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: elements of a tile are ranked in index order, round by round.
static __global__ void k_rs_scatter(const u64* __restrict__ kin, const uint32_t* __restrict__ vin, i64 n, int shift, u64 mask,
                             const unsigned* __restrict__ offs, int nblocks, u64* __restrict__ kout,
                             uint32_t* __restrict__ vout) {
    __shared__ unsigned wcnt[RS_BLOCK / 32][RS_BINS];
    __shared__ unsigned run[RS_BINS];
    __shared__ unsigned goff[RS_BINS];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    run[t] = 0;
    goff[t] = offs[(i64)t * nblocks + blockIdx.x];
    const unsigned lt = (1u << lane) - 1u;
    i64 base = (i64)blockIdx.x * RS_TILE;
    for (int i = 0; i < RS_ITEMS; ++i) {
#pragma unroll
        for (int w = 0; w < RS_BLOCK / 32; ++w) wcnt[w][t] = 0;
        __syncthreads();
        i64 e = base + (i64)i * RS_BLOCK + t;
        bool valid = e < n;
        u64 k = valid ? kin[e] : 0;
        uint32_t v = valid ? vin[e] : 0;
        unsigned dig = valid ? (unsigned)((k >> shift) & mask) : 0xffffffffu;
        unsigned peers = __match_any_sync(0xffffffffu, dig);
        unsigned lrank = __popc(peers & lt);
        if (valid && lrank == 0) wcnt[warp][dig] = __popc(peers);
        __syncthreads();
        {
            unsigned r = run[t];
#pragma unroll
            for (int w = 0; w < RS_BLOCK / 32; ++w) {
                unsigned c = wcnt[w][t];
                wcnt[w][t] = r;
                r += c;
            }
            run[t] = r;
        }
        __syncthreads();
        if (valid) {
            unsigned pos = goff[dig] + wcnt[warp][dig] + lrank;
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
    }
}

// Sorts n (key,value) pairs by key bits [0, nbits); stable.  Result ends in
// (keys, vals); tmp buffers are supplied by the caller.
inline void radix_sort_pairs(u64* keys, uint32_t* vals, u64* ktmp, uint32_t* vtmp, i64 n, int nbits,
                             cudaStream_t s) {
    if (n <= 1 || nbits <= 0) return;
    const int nb = (int)((n + RS_TILE - 1) / RS_TILE);
    unsigned* hist = dalloc<unsigned>((i64)RS_BINS * nb, s);
    u64 *ka = keys, *kb = ktmp;
    uint32_t *va = vals, *vb = vtmp;
    int passes = 0;
    for (int shift = 0; shift < nbits; shift += 8) {
        int bits = nbits - shift < 8 ? nbits - shift : 8;
        u64 mask = (1ull << bits) - 1;
        k_rs_hist<<<nb, RS_BLOCK, 0, s>>>(ka, n, shift, mask, hist, nb);
        CK_LAUNCH();
        exclusive_scan<unsigned, unsigned>(hist, hist, (i64)RS_BINS * nb, (unsigned*)nullptr, s);
        k_rs_scatter<<<nb, RS_BLOCK, 0, s>>>(ka, va, n, shift, mask, hist, nb, kb, vb);
        CK_LAUNCH();
        u64* kt = ka; ka = kb; kb = kt;
        uint32_t* vt = va; va = vb; vb = vt;
        ++passes;
    }
    if (passes & 1) {
        CK(cudaMemcpyAsync(keys, ka, (size_t)n * sizeof(u64), cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(vals, va, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    }
    dfree(hist, s);
}

// ---------------------------- small helpers ---------------------------------
template <class T>
__global__ void k_fill(T* p, i64 n, T v) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) p[i] = v;
}
template <class T>
inline void fill(T* p, i64 n, T v, cudaStream_t s) {
    if (n <= 0) return;
    k_fill<T><<<grid_for(n, 256), 256, 0, s>>>(p, n, v);
    CK_LAUNCH();
}

template <class T>
inline T read_scalar(const T* dptr, cudaStream_t s) {
    T h;
    CK(cudaMemcpyAsync(&h, dptr, sizeof(T), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return h;
}

}  // namespace prgpu
