// Definitions shared by the plain (solve.cu) and the flexible (flexcg.cu)
// persistent CG kernels: per-depth partition state and reduction barriers, the
// per-depth stencil description, block sums and compensated partial sums.
#pragma once
#include "common.cuh"

namespace prgpu {

constexpr int CG_BLOCK = 256;

struct PartState {          // one per depth, in global memory, zero-initialised
    double acc[3];
    unsigned count;
    unsigned gen;
    int iters;
    float rr;
    int status;
    int refines;            // true-residual refinements taken
    double bb;              // b.b (FP64 reduction)
    double rr_true;         // |b - Ax|^2 with FP64 accumulation (-1: not computed)
};

// reduction barrier of one depth's partition in k_cg_all: arrival counter, release
// generation and result on separate cache lines (the blocks poll 'gen' while the
// last one sums)
struct alignas(128) PartSync {
    unsigned count;
    unsigned pad0[31];
    unsigned gen;
    unsigned pad1[31];
    double res[2];
    double pad2[14];
};

struct CgDepth {
    i64 lo, n;              // global row range
    int first_block, nblocks;
    float st[27];
    // The Laplacian stencil is symmetric under the reflections and permutations of the
    // axes (a product of symmetric 1-D tables), so entry j depends only on how many of
    // its offsets are nonzero: cls[0] centre, [1] faces, [2] edges, [3] corners.  sym = 1
    // when the float entries are exactly so; the matrix-vector product then keeps the
    // four values in registers (the same values in the same FMA order).
    float cls[4];
    int sym;
};

// Shared-memory layout of a tile of 4 sibling groups' 4x4x4 blocks in the matrix-vector
// product.  For each stencil entry the lanes of a warp read the 8 children of 4 groups,
// at cell offsets {0,1,4,5,16,17,20,21} plus a constant from the group's block start;
// group gl's block starts 0, 2, 8 or 10 words past a multiple of 32, so the 32 reads fall
// in 32 distinct banks (with blocks 64 words apart, 4 groups hit the same banks).
constexpr int CG_TILE_WORDS = 272;
// The sibling-group table row by row for the solvers: a group's 27 first-child indices (and a
// pad), so a warp's consecutive groups are one contiguous run of the table.
constexpr int GN_ROW = 28;
__host__ __device__ constexpr int cg_block_base(int gl) { return gl * 66 + (gl >> 1) * 4; }

__host__ __device__ constexpr int stencil_class(int j) {
    return (j / 9 != 1) + ((j / 3) % 3 != 1) + (j % 3 != 1);
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    __syncthreads();
    return s;   // valid in thread 0
}

// per-thread partial dot product: a compensated float pair (Neumaier), exact to
// about 2u|sum| + n u^2 sum|term| -- FP64 accuracy for a thread's few dozen rows
// without FP64 arithmetic per row
struct FSum {
    float h = 0.f, l = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float t = h + v;
        l += (fabsf(h) >= fabsf(v)) ? (h - t) + v : (v - t) + h;
        h = t;
    }
    __device__ __forceinline__ double value() const { return (double)h + (double)l; }
};

}  // namespace prgpu
