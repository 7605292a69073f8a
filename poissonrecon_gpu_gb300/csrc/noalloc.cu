// prgpu_cg_csr_noalloc: the CSR conjugate-gradient solver of prgpu_cg_csr
// without any device allocation.
//
// Who needs it: callers that cannot call cudaMalloc/cudaFree at solve time --
// code running under a framework whose caching allocator has already reserved
// the device memory (a fresh cudaMalloc would fail or fragment that pool),
// latency-bound loops that must not pay for cudaFree's implicit device
// synchronisation, and embedded or real-time hosts that forbid allocation after
// start-up.  Their scratch vectors (r, p, Ap) and the solver's reduction and
// barrier state live in one fixed static device array declared below; the
// caller only passes the CSR matrix, the right-hand side and the solution.
//
// Limits and sharing:
//   * at most PRGPU_NOALLOC_MAX_ROWS rows; larger systems are rejected;
//   * the array is part of the library image, so every GPU that loads the
//     library holds it (about 3 MiB) until the process exits;
//   * every call uses the same array and leaves its contents behind; the state
//     block is cleared at the start of each call, the vectors are overwritten;
//     calls that overlap on the GPU (other streams, other host threads) race
//     on it and must be serialised by the caller;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current;
//   * a call blocks until its solve ends (it reads the iteration count back),
//     so it cannot be captured into a CUDA graph: on a capturing stream it
//     returns PRGPU_ERR_ARG without touching the stream.
#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace prgpu {

#define PRGPU_NOALLOC_MAX_ROWS (1 << 18)

namespace {

constexpr int NB_BLOCK = 256;
constexpr long long NB_SPIN_LIMIT = 1ll << 24;

struct NaState {           // first 256 bytes of the scratch array
    double acc[3];
    unsigned count;
    unsigned gen;
    int iters;
    float rr;
    int err;
};
constexpr size_t NA_STATE_BYTES = 256;
constexpr size_t NA_BYTES = NA_STATE_BYTES + 3ull * PRGPU_NOALLOC_MAX_ROWS * sizeof(float);

// the scratch: state block, then r, p and Ap of up to PRGPU_NOALLOC_MAX_ROWS rows
static __device__ __align__(256) unsigned char g_cg_scratch[NA_BYTES];

// host-side device addresses of g_cg_scratch, one per device, filled on first use
constexpr int NA_MAX_DEVICES = 64;
static void* g_scratch_addr[NA_MAX_DEVICES] = {nullptr};
static std::mutex g_scratch_mu;

__device__ __forceinline__ double na_block_sum(double v, double* sh) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    __syncthreads();
    return s;
}

// grid barrier with a bounded spin; returns false after a timeout
__device__ bool na_barrier(NaState* st, int* sh_ok) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &st->gen;
        unsigned g = *vgen;
        __threadfence();
        unsigned arrived = atomicAdd(&st->count, 1u);
        int ok = 1;
        if (arrived == gridDim.x - 1) {
            atomicExch(&st->count, 0u);
            __threadfence();
            atomicAdd(&st->gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == g) {
                if (++spins > NB_SPIN_LIMIT || *(volatile int*)&st->err) { ok = 0; break; }
                __nanosleep(32);
            }
        }
        __threadfence();
        if (!ok) atomicExch(&st->err, PRGPU_ERR_TIMEOUT);
        *sh_ok = ok && !*(volatile int*)&st->err;
    }
    __syncthreads();
    return *sh_ok != 0;
}

__global__ void __launch_bounds__(NB_BLOCK)
k_cg_csr_static(int n, const int* __restrict__ rowptr, const int* __restrict__ col, const float* __restrict__ val,
                const float* __restrict__ b, float* __restrict__ x, float tol2, int max_iter,
                unsigned char* __restrict__ scratch) {
    __shared__ double sh[NB_BLOCK / 32];
    __shared__ int sh_ok;
    __shared__ double sh_val;
    NaState* st = (NaState*)scratch;
    float* r = (float*)(scratch + NA_STATE_BYTES);
    float* p = r + PRGPU_NOALLOC_MAX_ROWS;
    float* q = p + PRGPU_NOALLOC_MAX_ROWS;
    const int stride = gridDim.x * blockDim.x;
    const int start = blockIdx.x * blockDim.x + threadIdx.x;
    int red = 0;
    auto reduce = [&](double v, bool& ok) -> double {
        double s = na_block_sum(v, sh);
        if (threadIdx.x == 0) atomicAdd(&st->acc[red % 3], s);
        ok = na_barrier(st, &sh_ok);
        if (threadIdx.x == 0) sh_val = *(volatile double*)&st->acc[red % 3];
        __syncthreads();
        double res = sh_val;
        if (blockIdx.x == 0 && threadIdx.x == 0) st->acc[(red + 2) % 3] = 0.0;
        ++red;
        return res;
    };
    double loc = 0;
    for (int i = start; i < n; i += stride) {
        x[i] = 0.f;
        r[i] = b[i];
        loc += (double)(b[i] * b[i]);
    }
    bool ok = true;
    float r1 = (float)reduce(loc, ok), r0 = 0.f;
    int k = 1;
    while (ok && r1 > tol2 && k <= max_iter) {
        if (k > 1) {
            const float beta = r1 / r0;
            for (int i = start; i < n; i += stride) p[i] = fmaf(beta, p[i], r[i]);
        } else {
            for (int i = start; i < n; i += stride) p[i] = r[i];
        }
        if (!na_barrier(st, &sh_ok)) break;
        loc = 0;
        for (int i = start; i < n; i += stride) {
            float o = 0.f;
            for (int e = rowptr[i]; e < rowptr[i + 1]; ++e) o = fmaf(val[e], p[col[e]], o);
            q[i] = o;
            loc += (double)(p[i] * o);
        }
        const double pq = reduce(loc, ok);
        if (!ok) break;
        const float al = (float)((double)r1 / pq), nal = -al;
        loc = 0;
        for (int i = start; i < n; i += stride) {
            x[i] = fmaf(al, p[i], x[i]);
            const float ri = fmaf(nal, q[i], r[i]);
            r[i] = ri;
            loc += (double)(ri * ri);
        }
        r0 = r1;
        r1 = (float)reduce(loc, ok);
        ++k;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->iters = k - 1;
        st->rr = r1;
    }
}

// device address of the scratch array on the current device (looked up once)
int scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_last_error("prgpu_cg_csr_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
        return PRGPU_ERR_CUDA;
    }
    if (dev < 0 || dev >= NA_MAX_DEVICES) {
        set_last_error("prgpu_cg_csr_noalloc: device %d beyond the supported %d", dev, NA_MAX_DEVICES);
        return PRGPU_ERR_LIMIT;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress((void**)&ptr, g_cg_scratch);
        if (e != cudaSuccess || !ptr) {
            set_last_error("prgpu_cg_csr_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return PRGPU_ERR_CUDA;
        }
        g_scratch_addr[dev] = ptr;
    }
    *out = g_scratch_addr[dev];
    return PRGPU_OK;
}

}  // namespace
}  // namespace prgpu

using namespace prgpu;

extern "C" int prgpu_cg_csr_noalloc(int32_t n, int32_t nz, const int32_t* d_rowptr, const int32_t* d_col,
                                    const float* d_val, const float* d_rhs, float* d_x, float tol, int32_t max_iter,
                                    void* stream, int32_t* iters) {
    (void)nz;
    if (n <= 0 || !d_rowptr || !d_col || !d_val || !d_rhs || !d_x || max_iter < 0) {
        set_last_error("prgpu_cg_csr_noalloc: invalid argument");
        return PRGPU_ERR_ARG;
    }
    if (n > PRGPU_NOALLOC_MAX_ROWS) {
        set_last_error("prgpu_cg_csr_noalloc: %d rows exceed the static scratch limit of %d rows", n,
                       PRGPU_NOALLOC_MAX_ROWS);
        return PRGPU_ERR_LIMIT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone) {
        set_last_error("prgpu_cg_csr_noalloc: the stream is capturing; the call blocks until the solve ends and "
                       "cannot be part of a CUDA graph");
        return PRGPU_ERR_ARG;
    }
    void* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_csr_static, NB_BLOCK, 0);
    // the state block must start at zero; the vectors are written before they are read
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0, NA_STATE_BYTES, s);
    if (e != cudaSuccess) {
        set_last_error("prgpu_cg_csr_noalloc: %s", cudaGetErrorString(e));
        return PRGPU_ERR_CUDA;
    }
    const int want = (n + NB_BLOCK - 1) / NB_BLOCK;
    const int grid = std::max(1, std::min(sms * std::max(per_sm, 1), want));
    float tol2 = tol * tol;
    unsigned char* sp = (unsigned char*)scratch;
    int na = n, mi = max_iter;
    void* args[] = {(void*)&na, (void*)&d_rowptr, (void*)&d_col, (void*)&d_val, (void*)&d_rhs, (void*)&d_x,
                    (void*)&tol2, (void*)&mi, (void*)&sp};
    e = cudaLaunchCooperativeKernel((void*)k_cg_csr_static, dim3(grid), dim3(NB_BLOCK), args, 0, s);
    if (e != cudaSuccess) {
        set_last_error("prgpu_cg_csr_noalloc: launch: %s", cudaGetErrorString(e));
        return PRGPU_ERR_CUDA;
    }
    ++g_kernel_launches;
    NaState h;
    e = cudaMemcpyAsync(&h, scratch, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_last_error("prgpu_cg_csr_noalloc: %s", cudaGetErrorString(e));
        return PRGPU_ERR_CUDA;
    }
    if (iters) *iters = h.iters;
    if (h.err) {
        set_last_error("prgpu_cg_csr_noalloc: grid barrier timed out");
        return PRGPU_ERR_TIMEOUT;
    }
    return (h.iters >= max_iter && h.rr > tol2) ? PRGPU_ERR_NOT_CONVERGED : PRGPU_OK;
}
