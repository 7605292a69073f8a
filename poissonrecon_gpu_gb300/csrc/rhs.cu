// Right-hand side: vector-field splat at the finest depth and divergence at
// every depth.  Replaces computeVectorField (main.cu:913-964),
// computeEncodedFinerNodesDivergence (main.cu:1007-1060) and the per-node host
// loop of the coarse divergence (main.cu:3399-3458).
#include "context.h"
#include "prims.cuh"

namespace prgpu {

// BinaryNode<float>::CenterAndWidth for a finest-depth function index
__device__ __forceinline__ float finest_center(int off, int D) {
    float w = (float)(1.0 / (double)(1 << D));
    return (float)((0.5 + (double)off) * (double)w);
}

// One thread per finest slot, neighbours and their points in the reference's
// order; the splat weight is (F/F(0)) scaled to the finest width, shifted to
// the sample and evaluated at the node centre (main.cu:913-964).
__global__ void k_splat(NodeArrays nd, i64 lo, i64 hi, int D, CPoly f, const float* __restrict__ pts,
                        const float* __restrict__ nrm, float* __restrict__ vfield) {
    const i64 M = nd.M;
    for (i64 i = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (i64)gridDim.x * blockDim.x) {
        int xyz[3];
        key_coords(nd.key[i], D, D, xyz);
        const float oc0 = finest_center(xyz[0], D), oc1 = finest_center(xyz[1], D), oc2 = finest_center(xyz[2], D);
        float v0 = 0.f, v1 = 0.f, v2 = 0.f;
        for (int j = 0; j < 27; ++j) {
            const int nb = nd.neigh[(i64)j * M + i];
            if (nb == -1) continue;
            const int p0 = nd.pidx[nb], pn = nd.pnum[nb];
            for (int k = 0; k < pn; ++k) {
                const i64 pt = (i64)p0 + k;
                const float px = pts[3 * pt], py = pts[3 * pt + 1], pz = pts[3 * pt + 2];
                CPoly sx, sy, sz;
                cpoly_shift<2>(f, px, sx);
                cpoly_shift<2>(f, py, sy);
                cpoly_shift<2>(f, pz, sz);
                const float wx = cpoly_value<2>(sx, oc0);
                const float wy = cpoly_value<2>(sy, oc1);
                const float wz = cpoly_value<2>(sz, oc2);
                const float w = wx * wy * wz;
                v0 = fmaf(w, nrm[3 * pt], v0);
                v1 = fmaf(w, nrm[3 * pt + 1], v1);
                v2 = fmaf(w, nrm[3 * pt + 2], v2);
            }
        }
        const i64 o = i - lo;
        vfield[3 * o] = v0;
        vfield[3 * o + 1] = v1;
        vfield[3 * o + 2] = v2;
    }
}

// finest-slot coordinates, packed for the divergence gathers
__global__ void k_finest_coords(const u64* __restrict__ key, i64 lo, i64 n, int D, short4* __restrict__ out) {
    for (i64 o = (i64)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (i64)gridDim.x * blockDim.x) {
        int xyz[3];
        key_coords(key[lo + o], D, D, xyz);
        out[o] = make_short4((short)xyz[0], (short)xyz[1], (short)xyz[2], 0);
    }
}

struct DivArgs {
    int D;
    i64 M;
    const float* vfield;
    const short4* fc;          // finest coordinates
    const float* rows;         // compact inner-product rows
    const i64* row_start;      // per depth (device)
};

// one divergence term: float dot product of V_o with the three table values,
// ordered as DotProduct with the reference's fused multiply-adds (main.cu:966-972)
__device__ __forceinline__ float div_term(const DivArgs& a, const float* r0, const float* r1, const float* r2,
                                          const int t0[3], i64 o) {
    const short4 c = a.fc[o];
    const float u0 = r0[c.x - t0[0]], u1 = r1[c.y - t0[1]], u2 = r2[c.z - t0[2]];
    const float vx = a.vfield[3 * o], vy = a.vfield[3 * o + 1], vz = a.vfield[3 * o + 2];
    float t = vx * u0;
    t = fmaf(vy, u1, t);
    t = fmaf(vz, u2, t);
    return t;
}

__device__ __forceinline__ void node_rows(const DivArgs& a, u64 key, int d, const float*& r0, const float*& r1,
                                          const float*& r2, int t0[3]) {
    int xyz[3];
    key_coords(key, d, a.D, xyz);
    const i64 W = 3ll << (a.D - d);
    const i64 rs = a.row_start[d];
    r0 = a.rows + rs + xyz[0] * W;
    r1 = a.rows + rs + xyz[1] * W;
    r2 = a.rows + rs + xyz[2] * W;
    for (int q = 0; q < 3; ++q) t0[q] = (xyz[q] - 1) * (1 << (a.D - d));
}

// nodes with few terms: one thread per node, terms in neighbour order
__global__ void k_div_thread(NodeArrays nd, DivArgs a, i64 lo, i64 hi, float* __restrict__ out) {
    for (i64 i = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (i64)gridDim.x * blockDim.x) {
        const float *r0, *r1, *r2;
        int t0[3];
        node_rows(a, nd.key[i], nd.depth[i], r0, r1, r2, t0);
        double val = 0.0;
        for (int j = 0; j < 27; ++j) {
            const int nb = nd.neigh[(i64)j * a.M + i];
            if (nb == -1) continue;
            const int s0 = nd.didx[nb], sn = nd.dnum[nb];
            for (int k = 0; k < sn; ++k) val += (double)div_term(a, r0, r1, r2, t0, (i64)s0 + k);
        }
        out[i] = (float)val;
    }
}

// nodes with many terms: one block per node, FP64 block reduction
constexpr int DIV_BLOCK = 256;
__global__ void k_div_block(NodeArrays nd, DivArgs a, i64 lo, float* __restrict__ out) {
    __shared__ int pre[28];
    __shared__ int sidx[27];
    __shared__ double red[DIV_BLOCK / 32];
    const i64 i = lo + blockIdx.x;
    if (threadIdx.x == 0) {
        int run = 0;
        for (int j = 0; j < 27; ++j) {
            const int nb = nd.neigh[(i64)j * a.M + i];
            pre[j] = run;
            sidx[j] = (nb == -1) ? 0 : nd.didx[nb];
            run += (nb == -1) ? 0 : nd.dnum[nb];
        }
        pre[27] = run;
    }
    __syncthreads();
    const float *r0, *r1, *r2;
    int t0[3];
    node_rows(a, nd.key[i], nd.depth[i], r0, r1, r2, t0);
    const int total = pre[27];
    double val = 0.0;
    int j = 0;
    for (int t = threadIdx.x; t < total; t += DIV_BLOCK) {
        while (pre[j + 1] <= t) ++j;
        val += (double)div_term(a, r0, r1, r2, t0, (i64)sidx[j] + (t - pre[j]));
    }
    for (int o = 16; o; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = val;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < DIV_BLOCK / 32; ++w) s += red[w];
        out[i] = (float)s;
    }
}

void stage_splat(Ctx& c) {
    cudaStream_t s = c.stream;
    const int D = c.D;
    const i64 lo = c.base[D], hi = c.base[D + 1];
    dfree(c.vfield, s);
    c.vfield = dalloc<float>(3 * (hi - lo), s);
    // compulsory: points+normals once, finest keys and neighbour tables, V written
    const int kt = c.kbegin("splat", (double)c.N * 24 + (double)(hi - lo) * (8 + 108 + 12));
    k_splat<<<grid_for(hi - lo, 128, 1ll << 30), 128, 0, s>>>(c.nodes, lo, hi, D, c.basis_maxdepth, c.pts, c.nrm,
                                                               c.vfield);
    CK_LAUNCH();
    c.kend(kt);
}

void stage_divergence(Ctx& c) {
    cudaStream_t s = c.stream;
    const int D = c.D;
    const i64 M = c.nodes.M, lo = c.base[D], nD = c.count[D];
    dfree(c.divergence, s);
    c.divergence = dalloc<float>(M, s);
    short4* fc = dalloc<short4>(nD, s);
    k_finest_coords<<<grid_for(nD, 256), 256, 0, s>>>(c.nodes.key, lo, nD, D, fc);
    CK_LAUNCH();
    i64* rs = dalloc<i64>(D + 2, s);
    CK(cudaMemcpyAsync(rs, c.ddot_row_start.data(), (D + 2) * sizeof(i64), cudaMemcpyHostToDevice, s));
    DivArgs a;
    a.D = D;
    a.M = M;
    a.vfield = c.vfield;
    a.fc = fc;
    a.rows = c.ddot_div;
    a.row_start = rs;
    // depths D and D-1: at most 27 and 216 terms per node
    const int split = D >= 1 ? D - 1 : 0;
    // compulsory: every node's key, depth, neighbours and b; V and coordinates of the finest slots
    const int kt = c.kbegin("divergence", (double)M * (8 + 1 + 108 + 4) + (double)nD * (12 + 8));
    k_div_thread<<<grid_for(M - c.base[split], 128, 1ll << 30), 128, 0, s>>>(c.nodes, a, c.base[split], M,
                                                                             c.divergence);
    CK_LAUNCH();
    if (c.base[split] > 0) {
        k_div_block<<<(unsigned)c.base[split], DIV_BLOCK, 0, s>>>(c.nodes, a, 0, c.divergence);
        CK_LAUNCH();
    }
    c.kend(kt);
    dfree(fc, s);
    dfree(rs, s);
}

}  // namespace prgpu
