// Shared definitions for the sm_103a Poisson-reconstruction kernels.
//
// The library is compiled with --fmad=false: a*b+c never fuses implicitly, and
// every fused multiply-add below is an explicit fmaf()/fma().  That makes the
// rounding of each stage a property of the source, so the stages that restate
// the reference arithmetic reproduce it bit for bit.
#pragma once
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "../../include/prgpu.h"

namespace prgpu {

typedef int64_t i64;
typedef uint64_t u64;

constexpr int PRGPU_MAX_DEPTH = 15;   // the largest maxDepth prgpu_create accepts

// ---------------------------------------------------------------------------
// error handling: every CUDA call inside the library goes through CK()
// ---------------------------------------------------------------------------
struct Error {
    int status;
    char msg[256];
};
void set_last_error(const char* fmt, ...);
const char* last_error();

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            ::prgpu::set_last_error("%s:%d %s: %s", __FILE__, __LINE__, #call,          \
                                    cudaGetErrorString(e_));                            \
            throw ::prgpu::Error{PRGPU_ERR_CUDA, {0}};                                  \
        }                                                                               \
    } while (0)
// every kernel launch is followed by CK_LAUNCH(), which also counts it
extern std::atomic<unsigned long long> g_kernel_launches;

// Bounded waits of the persistent solver kernels: a barrier polls at most
// spin_limit times (about 32-64 ns apart) and then records PRGPU_ERR_TIMEOUT.
// PRGPU_HOOK_BARRIER_WAIT sets extra = 1 (an arrival that never comes) and a
// small limit, so tests reach the timeout path without a real hang.
constexpr long long DEFAULT_SPIN_LIMIT = 1ll << 24;   // about half a second
struct WaitLimits {
    long long spin_limit = DEFAULT_SPIN_LIMIT;
    int extra = 0;
};
WaitLimits wait_limits();   // current settings (host)
#define CK_LAUNCH()                            \
    do {                                       \
        ++::prgpu::g_kernel_launches;          \
        CK(cudaGetLastError());                \
    } while (0)

inline unsigned grid_for(i64 n, int block, i64 cap = (i64)152 * 64) {
    i64 g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

// ---------------------------------------------------------------------------
// neighbour numbering (main.cu:80-99): neighbour j = 9(dx+1)+3(dy+1)+(dz+1);
// child code = x<<2 | y<<1 | z.  k_neighbours computes the reference's lookup
// tables' values from this definition.
// ---------------------------------------------------------------------------

// ---------------------------------------------------------------------------
// keys: 3 bits per level, level 1 most significant; x bit 2, y bit 1, z bit 0.
// A node at depth d keeps its key in the full-depth layout (levels below d = 0).
// ---------------------------------------------------------------------------
// every third bit of v (bits 0, 3, 6, ...), packed: the Morton compaction by masks
__host__ __device__ inline uint32_t morton_compact3(u64 v) {
    v &= 0x1249249249249249ull;
    v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ull;
    v = (v ^ (v >> 4)) & 0x100f00f00f00f00full;
    v = (v ^ (v >> 8)) & 0x001f0000ff0000ffull;
    v = (v ^ (v >> 16)) & 0x001f00000000ffffull;
    v = (v ^ (v >> 32)) & 0x00000000001fffffull;
    return (uint32_t)v;
}
// cell coordinates at depth d of a key (3D bits, level l's triple x y z at bit 3(D-l))
__host__ __device__ inline void key_coords(u64 key, int d, int D, int xyz[3]) {
    const u64 k = d > 0 ? key >> (3 * (D - d)) : 0ull;
    const uint32_t m = (1u << d) - 1u;
    xyz[0] = (int)(morton_compact3(k >> 2) & m);
    xyz[1] = (int)(morton_compact3(k >> 1) & m);
    xyz[2] = (int)(morton_compact3(k) & m);
}
// bit i of x to bit 3i (21 bits): the Morton spread by masks
__host__ __device__ inline u64 morton_spread3(uint32_t x) {
    u64 v = x & 0x1fffffu;
    v = (v | (v << 32)) & 0x001f00000000ffffull;
    v = (v | (v << 16)) & 0x001f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
// the key of the depth-d cell (x, y, z): the low d bits of each coordinate, interleaved
__host__ __device__ inline u64 coords_key(int x, int y, int z, int d, int D) {
    if (d <= 0) return 0ull;
    const uint32_t m = (1u << d) - 1u;
    const u64 k = (morton_spread3((uint32_t)x & m) << 2) | (morton_spread3((uint32_t)y & m) << 1) |
                  morton_spread3((uint32_t)z & m);
    return k << (3 * (D - d));
}

// ---------------------------------------------------------------------------
// piecewise polynomials in the reference's "starting polynomial" form:
// value(x) = sum over pieces i with x > start[i] of poly_i(x)
// ---------------------------------------------------------------------------
struct CPoly {
    float start[4];
    float c[4][4];
};

// value() of ConfirmedPPolynomial (ConfirmedPPolynomial.cuh:79-91); the
// reference's device compiler fused v += temp*c into one FMA.
template <int DEG>
__device__ __forceinline__ float cpoly_value(const CPoly& p, float x) {
    float res = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (!(x > p.start[i])) break;
        float temp = 1.f, v = 0.f;
#pragma unroll
        for (int j = 0; j <= DEG; ++j) {
            v = fmaf(temp, p.c[i][j], v);
            temp = temp * x;
        }
        res = res + v;
    }
    return res;
}

// Closed form of the normalised basis F/F(0), F the quadratic B-spline of
// support [-1.5, 1.5] with F(0) = 3/4 (what GaussianApproximation builds,
// PPolynomial.inl:384-423), for params.stable_basis.  Callers form the offset t
// with one fmaf (q * 2^d - (n + 1/2), or (x + 1/2) - p * 2^D): the product is
// exact, so t carries a single rounding, and the evaluation needs no shifted
// polynomial whose single-precision coefficients grow as 4^d.
__host__ __device__ __forceinline__ float bspline_unit(float t) {
    t = fabsf(t);
    if (t < 0.5f) return (0.75f - t * t) * (4.0f / 3.0f);
    if (t < 1.5f) {
        const float u = 1.5f - t;
        return u * u * (2.0f / 3.0f);
    }
    return 0.f;
}
// basis function n of depth d at coordinate q in [0, 1]
__device__ __forceinline__ float basis_stable(int d, int n, float q) {
    return bspline_unit(fmaf(q, (float)(1 << d), -((float)n + 0.5f)));
}

// ConfirmedPPolynomial::shift (ConfirmedPPolynomial.cuh:37-50)
template <int DEG>
__device__ __forceinline__ void cpoly_shift(const CPoly& p, float t, CPoly& r) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        r.start[i] = p.start[i] + t;
#pragma unroll
        for (int k = 0; k < 4; ++k) r.c[i][k] = 0.f;
#pragma unroll
        for (int k = 0; k <= DEG; ++k) {
            float temp = 1.f;
#pragma unroll
            for (int j = k; j >= 0; --j) {
                r.c[i][j] = fmaf(p.c[i][k], temp, r.c[i][j]);
                temp = temp * (-t * (float)j);
                temp = temp / (float)(k - j + 1);
            }
        }
    }
}

}  // namespace prgpu
