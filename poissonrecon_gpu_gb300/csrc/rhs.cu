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

// One lane per finest slot, neighbours and their points in the reference's order;
// the splat weight is (F/F(0)) scaled to the finest width, shifted to the sample
// and evaluated at the node centre (main.cu:913-964).  A warp takes 4 sibling
// groups: the 27-neighbourhoods of a group's 8 nodes are the 4x4x4 block of the
// children of the parent's 27 neighbours (the group table), whose point ranges
// are staged once per group; each lane then runs its node's (neighbour, point)
// pairs in neighbour order in one flat loop, so that the lanes stay together.
constexpr int SPLAT_BLOCK = 128;
__global__ void __launch_bounds__(SPLAT_BLOCK, 8) k_splat(NodeArrays nd, const int* __restrict__ gn, i64 ngroups_all,
                                                       i64 gfirst, i64 ng, i64 lo, int D, CPoly f,
                                                       const float* __restrict__ pts, const float* __restrict__ nrm,
                                                       float* __restrict__ vfield, int stable) {
    __shared__ int2 rng[SPLAT_BLOCK / 32][4][64];   // (first point, count) of each block cell
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
    for (i64 tile = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile * 4 < ng; tile += nwarps) {
        __syncwarp();
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int e = lane + 32 * m;
            const i64 g = tile * 4 + (e >> 6);
            const int cell = e & 63, bx = cell >> 4, by = (cell >> 2) & 3, bz = cell & 3;
            int2 r = make_int2(0, 0);
            if (g < ng) {
                const int jp = 9 * ((bx + 1) >> 1) + 3 * ((by + 1) >> 1) + ((bz + 1) >> 1);
                const int cn = gn[(i64)jp * ngroups_all + gfirst + g];
                if (cn != -1) {
                    const int node = cn + ((((bx + 1) & 1) << 2) | (((by + 1) & 1) << 1) | ((bz + 1) & 1));
                    r = make_int2(nd.pidx[node], nd.pnum[node]);
                }
            }
            rng[w][e >> 6][cell] = r;
        }
        __syncwarp();
        const i64 g = tile * 4 + (lane >> 3);
        if (g >= ng) continue;
        const int s = lane & 7, sx = s >> 2, sy = (s >> 1) & 1, sz = s & 1;
        const i64 i = lo + 8 * g + s;
        int xyz[3];
        key_coords(nd.key[i], D, D, xyz);
        const float oc0 = finest_center(xyz[0], D), oc1 = finest_center(xyz[1], D), oc2 = finest_center(xyz[2], D);
        const int2* br = rng[w][lane >> 3];
        int T = 0;
#pragma unroll
        for (int j = 0; j < 27; ++j) T += br[(sx + j / 9) * 16 + (sy + (j / 3) % 3) * 4 + (sz + j % 3)].y;
        float v0 = 0.f, v1 = 0.f, v2 = 0.f;
        int j = 0, k = 0;
        int2 cur = br[sx * 16 + sy * 4 + sz];
        for (int t = 0; t < T; ++t) {
            while (k >= cur.y) {
                ++j;
                k = 0;
                cur = br[(sx + j / 9) * 16 + (sy + (j / 3) % 3) * 4 + (sz + j % 3)];
            }
            const i64 pt = (i64)cur.x + k;
            ++k;
            const float px = pts[3 * pt], py = pts[3 * pt + 1], pz = pts[3 * pt + 2];
            float wx, wy, wz;
            if (stable) {   // F/F(0) at (centre - p) 2^D = (xyz + 1/2) - p 2^D, one rounding
                const float sD = (float)(1 << D);
                wx = bspline_unit(fmaf(-px, sD, (float)xyz[0] + 0.5f));
                wy = bspline_unit(fmaf(-py, sD, (float)xyz[1] + 0.5f));
                wz = bspline_unit(fmaf(-pz, sD, (float)xyz[2] + 0.5f));
            } else {
                CPoly cx, cy, cz;
                cpoly_shift<2>(f, px, cx);
                cpoly_shift<2>(f, py, cy);
                cpoly_shift<2>(f, pz, cz);
                wx = cpoly_value<2>(cx, oc0);
                wy = cpoly_value<2>(cy, oc1);
                wz = cpoly_value<2>(cz, oc2);
            }
            const float wgt = wx * wy * wz;
            v0 = fmaf(wgt, nrm[3 * pt], v0);
            v1 = fmaf(wgt, nrm[3 * pt + 1], v1);
            v2 = fmaf(wgt, nrm[3 * pt + 2], v2);
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
        // neighbours in three batches of nine: indices, then descendant ranges, then terms,
        // so that each batch's loads are in flight together
#pragma unroll
        for (int jb = 0; jb < 27; jb += 9) {
            int nb[9], s0[9], sn[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) nb[q] = nd.neigh[(i64)(jb + q) * a.M + i];
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                s0[q] = nb[q] == -1 ? 0 : nd.didx[nb[q]];
                sn[q] = nb[q] == -1 ? 0 : nd.dnum[nb[q]];
            }
#pragma unroll
            for (int q = 0; q < 9; ++q)
                for (int k = 0; k < sn[q]; ++k) val += (double)div_term(a, r0, r1, r2, t0, (i64)s0[q] + k);
        }
        out[i] = (float)val;
    }
}

// finest depth by sibling groups: the 27 neighbours of the 8 children of a node
// are the 4x4x4 block of the children of the parent's 27 neighbours (the solve's
// group table).  One warp stages the V of the blocks of 4 groups in shared
// memory; each row then sums its 27 terms in neighbour order in FP64, as
// k_div_thread does.  Every finest node has exactly one finest descendant
// (itself), and the neighbour at offset j = (jx,jy,jz) reads the row entries
// jx, jy, jz of the node's 3-entry rows.
__global__ void __launch_bounds__(256) k_div_finest(NodeArrays nd, DivArgs a, const int* __restrict__ gn,
                                                    i64 ngroups_all, i64 gfirst, i64 ng, i64 lo,
                                                    float* __restrict__ out) {
    __shared__ float4 cells[8][4 * 64];   // per warp: V of the 4x4x4 block of 4 groups, w = 1 if the cell exists
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int ch = lane & 7, gl = lane >> 3;
    const int sx = ch >> 2, sy = (ch >> 1) & 1, sz = ch & 1;
    const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
    float4* blk = cells[wib];
    for (i64 tile = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile * 4 < ng; tile += nwarps) {
        __syncwarp();
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int e = lane + 32 * m;
            const i64 g = tile * 4 + (e >> 6);
            const int cell = e & 63, bx = cell >> 4, by = (cell >> 2) & 3, bz = cell & 3;
            float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
            if (g < ng) {
                const int jp = 9 * ((bx + 1) >> 1) + 3 * ((by + 1) >> 1) + ((bz + 1) >> 1);
                const int cn = gn[(i64)jp * ngroups_all + gfirst + g];
                if (cn != -1) {
                    const i64 o = cn + ((((bx + 1) & 1) << 2) | (((by + 1) & 1) << 1) | ((bz + 1) & 1)) - lo;
                    val = make_float4(a.vfield[3 * o], a.vfield[3 * o + 1], a.vfield[3 * o + 2], 1.f);
                }
            }
            blk[e] = val;
        }
        __syncwarp();
        const i64 g = tile * 4 + gl;
        if (g < ng) {
            const i64 i = lo + 8 * g + ch;
            int xyz[3];
            key_coords(nd.key[i], a.D, a.D, xyz);
            const float* rr = a.rows + a.row_start[a.D];
            float R[3][3];
#pragma unroll
            for (int ax = 0; ax < 3; ++ax)
#pragma unroll
                for (int t = 0; t < 3; ++t) R[ax][t] = rr[xyz[ax] * 3 + t];
            const float4* b = blk + gl * 64;
            double val = 0.0;
#pragma unroll
            for (int j = 0; j < 27; ++j) {
                const int jx = j / 9, jy = (j / 3) % 3, jz = j % 3;
                const float4 c = b[(sx + jx) * 16 + (sy + jy) * 4 + (sz + jz)];
                if (c.w == 0.f) continue;   // no neighbour
                float t = c.x * R[0][jx];
                t = fmaf(c.y, R[1][jy], t);
                t = fmaf(c.z, R[2][jz], t);
                val += (double)t;
            }
            out[i] = (float)val;
        }
    }
}

// the root (all finest nodes are its terms): the node's terms, in neighbour order,
// are cut into chunks of DIV_CHUNK; one warp sums a chunk and the chunk sums are
// added per node in FP64 in a fixed order (k_div_sum: deterministic).  Within a chunk each
// lane keeps a compensated float pair (hi + lo, Neumaier's summation), whose
// error is at most 2u|sum| + O(n u^2) sum|term| -- FP64 accuracy for these
// lengths without FP64 arithmetic per term.
constexpr int DIV_CHUNK = 2048;
constexpr int DIV_WARPS = 8;

__device__ __forceinline__ i64 node_terms(const NodeArrays& nd, i64 M, i64 i) {
    i64 T = 0;
    for (int j = 0; j < 27; ++j) {
        const int nb = nd.neigh[(i64)j * M + i];
        if (nb != -1) T += nd.dnum[nb];
    }
    return T;
}

__global__ void k_div_count(NodeArrays nd, i64 n, int* __restrict__ nchunks) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        nchunks[i] = (int)((node_terms(nd, nd.M, i) + DIV_CHUNK - 1) / DIV_CHUNK);
}

__global__ void k_div_items(const int* __restrict__ nchunks, const int* __restrict__ first, i64 n,
                            int* __restrict__ item_node) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        for (int c = 0; c < nchunks[i]; ++c) item_node[first[i] + c] = (int)i;
}

__global__ void __launch_bounds__(DIV_WARPS * 32) k_div_chunks(NodeArrays nd, DivArgs a, const int* __restrict__ item_node,
                                                               const int* __restrict__ first, i64 nitems,
                                                               double* __restrict__ partial) {
    __shared__ int pre[DIV_WARPS][28];
    __shared__ int sidx[DIV_WARPS][27];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
    for (i64 it = warp; it < nitems; it += nwarps) {
        const i64 i = item_node[it];
        const int chunk = (int)(it - first[i]);
        // prefix of the neighbours' finest-descendant counts, in neighbour order
        int cnt = 0, sx = 0;
        if (lane < 27) {
            const int nb = nd.neigh[(i64)lane * a.M + i];
            if (nb != -1) { cnt = nd.dnum[nb]; sx = nd.didx[nb]; }
        }
        int inc = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        __syncwarp();
        if (lane < 27) { pre[w][lane] = inc - cnt; sidx[w][lane] = sx; }
        if (lane == 26) pre[w][27] = inc;
        __syncwarp();
        const float *r0, *r1, *r2;
        int t0[3];
        node_rows(a, nd.key[i], nd.depth[i], r0, r1, r2, t0);
        const int total = pre[w][27];
        const int lo = chunk * DIV_CHUNK, hi = min(total, lo + DIV_CHUNK);
        float sh = 0.f, sl = 0.f;
        int j = 0;
        while (pre[w][j + 1] <= lo) ++j;
        // neighbour by neighbour: each is a contiguous range of finest slots
        for (; j < 27 && pre[w][j] < hi; ++j) {
            const int a0 = max(lo, pre[w][j]), a1 = min(hi, pre[w][j + 1]);
            const i64 base = (i64)sidx[w][j] - pre[w][j];
            int t = a0 + lane;
            // four terms per step: their loads are issued together
            for (; t + 96 < a1; t += 128) {
                float tv[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) tv[q] = div_term(a, r0, r1, r2, t0, base + t + 32 * q);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float s = sh + tv[q];
                    sl += (fabsf(sh) >= fabsf(tv[q])) ? (sh - s) + tv[q] : (tv[q] - s) + sh;
                    sh = s;
                }
            }
            for (; t + 32 < a1; t += 64) {
                const float t1 = div_term(a, r0, r1, r2, t0, base + t);
                const float t2 = div_term(a, r0, r1, r2, t0, base + t + 32);
                float s = sh + t1;
                sl += (fabsf(sh) >= fabsf(t1)) ? (sh - s) + t1 : (t1 - s) + sh;
                sh = s;
                s = sh + t2;
                sl += (fabsf(sh) >= fabsf(t2)) ? (sh - s) + t2 : (t2 - s) + sh;
                sh = s;
            }
            if (t < a1) {
                const float term = div_term(a, r0, r1, r2, t0, base + t);
                const float s = sh + term;
                sl += (fabsf(sh) >= fabsf(term)) ? (sh - s) + term : (term - s) + sh;
                sh = s;
            }
        }
        double val = (double)sh + (double)sl;
        for (int o = 16; o; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
        if (lane == 0) partial[it] = val;
        __syncwarp();
    }
}

// Depths 1..D-2 by sibling groups.  The 27-neighbourhoods of the 8 children of a
// node are the 4x4x4 block of the children of the parent's 27 neighbours (the
// group table), and in x-major block order every child meets its own neighbours
// in neighbour order.  A group's terms are the finest descendants of the block's
// cells, concatenated in block order and cut into chunks of DIV_CHUNK finest
// nodes; one warp reads each finest node of a chunk once and adds its term to
// every child whose neighbourhood holds the cell (1, 2, 4 or 8 children), each
// child in its own compensated pair.  The term is the one k_div_chunks forms:
// child b on an axis reads the row of coordinate 2P+b at offset c - (2P+b-1)S,
// which is the row of 2P at offset (c - (2P-1)S) + 2bS.
__device__ __forceinline__ void neu_add(float& sh, float& sl, float t) {
    const float s = sh + t;
    sl += (fabsf(sh) >= fabsf(t)) ? (sh - s) + t : (t - s) + sh;
    sh = s;
}

__device__ __forceinline__ int group_cell_node(const int* __restrict__ gn, i64 ngroups_all, i64 g, int cell) {
    const int bx = cell >> 4, by = (cell >> 2) & 3, bz = cell & 3;
    const int jp = 9 * ((bx + 1) >> 1) + 3 * ((by + 1) >> 1) + ((bz + 1) >> 1);
    const int cn = gn[(i64)jp * ngroups_all + g];
    return cn == -1 ? -1 : cn + ((((bx + 1) & 1) << 2) | (((by + 1) & 1) << 1) | ((bz + 1) & 1));
}

__global__ void k_div_group_count(NodeArrays nd, const int* __restrict__ gn, i64 ngroups_all, i64 ng,
                                  int* __restrict__ nchunks) {
    for (i64 g = (i64)blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += (i64)gridDim.x * blockDim.x) {
        i64 T = 0;
        for (int cell = 0; cell < 64; ++cell) {
            const int n = group_cell_node(gn, ngroups_all, g, cell);
            if (n != -1) T += nd.dnum[n];
        }
        nchunks[g] = (int)((T + DIV_CHUNK - 1) / DIV_CHUNK);
    }
}

__global__ void __launch_bounds__(DIV_WARPS * 32) k_div_groups(NodeArrays nd, DivArgs a, const int* __restrict__ gn,
                                                               i64 ngroups_all, const int* __restrict__ item_group,
                                                               const int* __restrict__ first, i64 nitems,
                                                               double* __restrict__ partial) {
    __shared__ int pre[DIV_WARPS][65];
    __shared__ int sidx[DIV_WARPS][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
    for (i64 it = warp; it < nitems; it += nwarps) {
        const i64 g = item_group[it];
        const int chunk = (int)(it - first[g]);
        // prefix of the block cells' finest-descendant counts, two cells per lane
        int cnt[2], sx[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int n = group_cell_node(gn, ngroups_all, g, 2 * lane + q);
            cnt[q] = n == -1 ? 0 : nd.dnum[n];
            sx[q] = n == -1 ? 0 : nd.didx[n];
        }
        const int pair = cnt[0] + cnt[1];
        int inc = pair;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        __syncwarp();
        pre[w][2 * lane] = inc - pair;
        pre[w][2 * lane + 1] = inc - pair + cnt[0];
        sidx[w][2 * lane] = sx[0];
        sidx[w][2 * lane + 1] = sx[1];
        if (lane == 31) pre[w][64] = inc;
        __syncwarp();
        // child 0 of the group has the even coordinates 2P
        const i64 i0 = 1 + 8 * g;
        const int d = nd.depth[i0];
        int xyz[3];
        key_coords(nd.key[i0], d, a.D, xyz);
        const int S = 1 << (a.D - d), W = 3 * S;
        const float* R[3];
        int t0[3];
        const i64 rs = a.row_start[d];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            R[ax] = a.rows + rs + (i64)xyz[ax] * W;
            t0[ax] = (xyz[ax] - 1) * S;
        }
        const int total = pre[w][64];
        const int lo = chunk * DIV_CHUNK, hi = min(total, lo + DIV_CHUNK);
        float sh[8], sl[8];
#pragma unroll
        for (int s = 0; s < 8; ++s) { sh[s] = 0.f; sl[s] = 0.f; }
        // lanes run over the chunk across cell boundaries; each lane tracks its
        // cell (empty cells are skipped by the prefix)
        int j = 0;
        while (j < 63 && pre[w][j + 1] <= lo + lane) ++j;
        for (int t = lo + lane; t < hi; t += 32) {
            while (pre[w][j + 1] <= t) ++j;
            const i64 o = (i64)sidx[w][j] - pre[w][j] + t;
            const int bx = j >> 4, by = (j >> 2) & 3, bz = j & 3;
            // which children hold this cell, per axis: b = 0 for block 0..2, b = 1 for 1..3
            const bool x0 = bx <= 2, x1 = bx >= 1, y0 = by <= 2, y1 = by >= 1, z0 = bz <= 2, z1 = bz >= 1;
            const short4 c = a.fc[o];
            const float vx = a.vfield[3 * o], vy = a.vfield[3 * o + 1], vz = a.vfield[3 * o + 2];
            const int ox = c.x - t0[0], oy = c.y - t0[1], oz = c.z - t0[2];
            const float ux0 = x0 ? R[0][ox] : 0.f, ux1 = x1 ? R[0][ox + 2 * S] : 0.f;
            const float uy0 = y0 ? R[1][oy] : 0.f, uy1 = y1 ? R[1][oy + 2 * S] : 0.f;
            const float uz0 = z0 ? R[2][oz] : 0.f, uz1 = z1 ? R[2][oz + 2 * S] : 0.f;
            const float px[2] = {vx * ux0, vx * ux1};
            const float uy[2] = {uy0, uy1}, uz[2] = {uz0, uz1};
            const bool hx[2] = {x0, x1}, hy[2] = {y0, y1}, hz[2] = {z0, z1};
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                const int bsx = s >> 2, bsy = (s >> 1) & 1, bsz = s & 1;
                if (hx[bsx] && hy[bsy] && hz[bsz]) {
                    float term = fmaf(vy, uy[bsy], px[bsx]);
                    term = fmaf(vz, uz[bsz], term);
                    neu_add(sh[s], sl[s], term);
                }
            }
        }
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            double val = (double)sh[s] + (double)sl[s];
            for (int o = 16; o; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
            if (lane == 0) partial[it * 8 + s] = val;
        }
        __syncwarp();
    }
}

// one warp per node: the node's chunk partials (per entity of `per` nodes, node
// s of the entity at offset s) summed lane-strided in FP64 and then by a fixed
// butterfly, so the result does not depend on the schedule
__global__ void k_div_sum(const int* __restrict__ nchunks, const int* __restrict__ first,
                          const double* __restrict__ partial, i64 lo, i64 hi, int per, float* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
    for (i64 i = lo + (((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < hi; i += nwarps) {
        const i64 g = (i - lo) / per;
        const int s = (int)((i - lo) % per), n = nchunks[g];
        const i64 f = first[g];
        double v = 0.0;
        for (int q = lane; q < n; q += 32) v += partial[(f + q) * per + s];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) out[i] = (float)v;
    }
}

// the same sum of sibling-group partials (node i is child (i-1) % per of group
// (i-1) / per) for nodes with few chunks: one thread per node, in chunk order
__global__ void k_div_sum_thread(const int* __restrict__ nchunks, const int* __restrict__ first,
                                 const double* __restrict__ partial, i64 lo, i64 hi, int per, float* __restrict__ out) {
    for (i64 i = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (i64)gridDim.x * blockDim.x) {
        const i64 g = (i - 1) / per;
        const int s = (int)((i - 1) % per), n = nchunks[g];
        const i64 f = first[g];
        double v = 0.0;
        for (int q = 0; q < n; ++q) v += partial[(f + q) * per + s];
        out[i] = (float)v;
    }
}

// ---- density weights (params.density_weights; not in the reference)
// Kazhdan's weighting of non-uniform samples: at the kernel depth k, node o
// collects w_o = sum over the points p around it of B_o(p) (B_o the depth-k basis
// function of o, a product of its three axis functions); a point's density is
// W(s) = sum over the 27 depth-k nodes around it of B_o(s) w_o, and its weight
// 1/W(s), scaled to mean 1, multiplies its normal and its share of the iso-value.
__device__ __forceinline__ float node_basis_at(const CPoly* basis, int d, const int c[3], const float p[3]) {
    const int off = (1 << d) - 1;
    return cpoly_value<3>(basis[off + c[0]], p[0]) * cpoly_value<3>(basis[off + c[1]], p[1]) *
           cpoly_value<3>(basis[off + c[2]], p[2]);
}

__global__ void k_density_nodes(NodeArrays nd, i64 lo, i64 hi, int k, int D, const CPoly* __restrict__ basis,
                                const float* __restrict__ pts, float* __restrict__ w) {
    const i64 M = nd.M;
    for (i64 o = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; o < hi; o += (i64)gridDim.x * blockDim.x) {
        int c[3];
        key_coords(nd.key[o], k, D, c);
        float sum = 0.f;
        for (int j = 0; j < 27; ++j) {
            const int nb = nd.neigh[(i64)j * M + o];
            if (nb == -1) continue;
            const int p0 = nd.pidx[nb], pn = nd.pnum[nb];
            for (int q = 0; q < pn; ++q) {
                const float p[3] = {pts[3 * ((i64)p0 + q)], pts[3 * ((i64)p0 + q) + 1], pts[3 * ((i64)p0 + q) + 2]};
                sum += node_basis_at(basis, k, c, p);
            }
        }
        w[o - lo] = sum;
    }
}

__global__ void k_density_points(NodeArrays nd, i64 n, const int* __restrict__ point_node, int k, int D, i64 lo_k,
                                 const CPoly* __restrict__ basis, const float* __restrict__ pts,
                                 const float* __restrict__ w, float* __restrict__ inv, double* __restrict__ sum) {
    const i64 M = nd.M;
    double loc = 0.0;
    for (i64 s = (i64)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (i64)gridDim.x * blockDim.x) {
        i64 node = point_node[s];
        for (int d = D; d > k; --d) node = nd.parent[node];
        const float p[3] = {pts[3 * s], pts[3 * s + 1], pts[3 * s + 2]};
        float W = 0.f;
        for (int j = 0; j < 27; ++j) {
            const int nb = nd.neigh[(i64)j * M + node];
            if (nb == -1) continue;
            int c[3];
            key_coords(nd.key[nb], k, D, c);
            W += node_basis_at(basis, k, c, p) * w[nb - lo_k];
        }
        const float iw = W > 0.f ? 1.0f / W : 0.f;
        inv[s] = iw;
        loc += (double)iw;
    }
    for (int o = 16; o; o >>= 1) loc += __shfl_xor_sync(0xffffffffu, loc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, loc);
}

__global__ void k_weight_normals(i64 n, const double* __restrict__ sum, const float* __restrict__ nrm,
                                 float* __restrict__ weight, float* __restrict__ wnrm) {
    const float scale = (float)((double)n / *sum);
    for (i64 s = (i64)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (i64)gridDim.x * blockDim.x) {
        const float a = weight[s] * scale;
        weight[s] = a;
        wnrm[3 * s] = a * nrm[3 * s];
        wnrm[3 * s + 1] = a * nrm[3 * s + 1];
        wnrm[3 * s + 2] = a * nrm[3 * s + 2];
    }
}

static void density_weights(Ctx& c) {
    cudaStream_t s = c.stream;
    const int D = c.D, k = std::max(D - 2, 1);
    const i64 lo_k = c.base[k], hi_k = c.base[k + 1];
    float* w = dalloc<float>(hi_k - lo_k, s);
    double* sum = dalloc<double>(1, s);
    CK(cudaMemsetAsync(sum, 0, sizeof(double), s));
    dfree(c.point_weight, s);
    dfree(c.wnrm, s);
    c.point_weight = dalloc<float>(c.N, s);
    c.wnrm = dalloc<float>(3 * c.N, s);
    const int kt = c.kbegin("density_weights", (double)c.N * (12 + 12 + 4 + 12) + (double)(hi_k - lo_k) * 120);
    k_density_nodes<<<grid_for(hi_k - lo_k, 128), 128, 0, s>>>(c.nodes, lo_k, hi_k, k, D, c.basis, c.pts, w);
    CK_LAUNCH();
    k_density_points<<<grid_for(c.N, 128, (i64)c.sms * 32), 128, 0, s>>>(c.nodes, c.N, c.point_node, k, D, lo_k,
                                                                         c.basis, c.pts, w, c.point_weight, sum);
    CK_LAUNCH();
    k_weight_normals<<<grid_for(c.N, 256), 256, 0, s>>>(c.N, sum, c.nrm, c.point_weight, c.wnrm);
    CK_LAUNCH();
    c.kend(kt);
    dfree(w, s);
    dfree(sum, s);
}

void stage_splat(Ctx& c) {
    cudaStream_t s = c.stream;
    const int D = c.D;
    const i64 lo = c.base[D], hi = c.base[D + 1];
    dfree(c.vfield, s);
    c.vfield = dalloc<float>(3 * (hi - lo), s);
    const float* nrm = c.nrm;
    if (c.params.density_weights) {
        density_weights(c);
        nrm = c.wnrm;
    } else {
        dfree(c.point_weight, s);
        dfree(c.wnrm, s);
    }
    // compulsory: points+normals once, finest keys and neighbour tables, V written
    const int kt = c.kbegin("splat", (double)c.N * 24 + (double)(hi - lo) * (8 + 108 + 12));
    ensure_group_table(c);
    {
        const i64 ngroups_all = (c.nodes.M - 1) / 8, gfirst = (lo - 1) / 8, ng = (hi - lo) / 8;
        k_splat<<<grid_for(ng * 8, SPLAT_BLOCK, 1ll << 30), SPLAT_BLOCK, 0, s>>>(
            c.nodes, c.gn, ngroups_all, gfirst, ng, lo, D, c.basis_maxdepth, c.pts, nrm, c.vfield,
            c.params.stable_basis);
    }
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
    // depth D - 1 one thread per node; depth D by sibling groups
    const int kt1 = c.kbegin("divergence_d1", 0.0);
    k_div_thread<<<grid_for(c.base[D] - c.base[split], 128, 1ll << 30), 128, 0, s>>>(c.nodes, a, c.base[split],
                                                                                      c.base[D], c.divergence);
    CK_LAUNCH();
    c.kend(kt1);
    const int ktg = c.kbegin("group_table", 0.0);
    ensure_group_table(c);
    c.kend(ktg);
    const int kt2 = c.kbegin("divergence_d", 0.0);
    {
        const i64 ngroups_all = (M - 1) / 8, gfirst = (lo - 1) / 8, ng = nD / 8;
        k_div_finest<<<grid_for(ng * 8, 256, (i64)c.sms * 8 * 8), 256, 0, s>>>(c.nodes, a, c.gn, ngroups_all, gfirst,
                                                                               ng, lo, c.divergence);
        CK_LAUNCH();
    }
    c.kend(kt2);
    const i64 nc = c.base[split];   // nodes at depths < D-1
    if (nc > 0) {
        // the root: its terms in chunks; depths 1..D-2: sibling groups in chunks
        const i64 ngroups_all = (M - 1) / 8, ngc = (nc - 1) / 8;
        int* nch = dalloc<int>(1 + ngc, s);
        int* first = dalloc<int>(1 + 1 + ngc + 1, s);
        int* gfirst = first + 2;
        k_div_count<<<1, 32, 0, s>>>(c.nodes, 1, nch);
        CK_LAUNCH();
        exclusive_scan<int, int>(nch, first, 1, first + 1, s);
        if (ngc > 0) {
            k_div_group_count<<<grid_for(ngc, 256), 256, 0, s>>>(c.nodes, c.gn, ngroups_all, ngc, nch + 1);
            CK_LAUNCH();
            exclusive_scan<int, int>(nch + 1, gfirst, ngc, gfirst + ngc, s);
        }
        const i64 nroot = read_scalar(first + 1, s);
        const i64 ngitems = ngc > 0 ? read_scalar(gfirst + ngc, s) : 0;
        int* item_node = dalloc<int>(std::max<i64>(nroot + ngitems, 1), s);
        double* partial = dalloc<double>(std::max<i64>(nroot + 8 * ngitems, 1), s);
        const int ktr = c.kbegin("divergence_root", 0.0);
        if (nroot > 0) {
            k_div_items<<<1, 32, 0, s>>>(nch, first, 1, item_node);
            CK_LAUNCH();
            k_div_chunks<<<grid_for(nroot * 32, DIV_WARPS * 32, (i64)c.sms * 8), DIV_WARPS * 32, 0, s>>>(
                c.nodes, a, item_node, first, nroot, partial);
            CK_LAUNCH();
        }
        k_div_sum<<<1, 32, 0, s>>>(nch, first, partial, 0, 1, 1, c.divergence);
        CK_LAUNCH();
        c.kend(ktr);
        if (ngc > 0) {
            int* item_group = item_node + nroot;
            double* gpartial = partial + nroot;
            k_div_items<<<grid_for(ngc, 256), 256, 0, s>>>(nch + 1, gfirst, ngc, item_group);
            CK_LAUNCH();
            if (ngitems > 0) {
                const int kt3 = c.kbegin("divergence_groups", 0.0);
                k_div_groups<<<grid_for(ngitems * 32, DIV_WARPS * 32, (i64)c.sms * 8), DIV_WARPS * 32, 0, s>>>(
                    c.nodes, a, c.gn, ngroups_all, item_group, gfirst, ngitems, gpartial);
                CK_LAUNCH();
                c.kend(kt3);
            }
            // depths 1..3 (up to 584 nodes, thousands of chunks each at depths 1-2): a warp per
            // node; deeper nodes have few chunks: a thread per node
            const i64 wide = std::min<i64>(nc, c.base[std::min(4, D)]);
            k_div_sum<<<grid_for((wide - 1) * 32, 256), 256, 0, s>>>(nch + 1, gfirst, gpartial, 1, wide, 8,
                                                                     c.divergence);
            CK_LAUNCH();
            if (nc > wide) {
                k_div_sum_thread<<<grid_for(nc - wide, 256), 256, 0, s>>>(nch + 1, gfirst, gpartial, wide, nc, 8,
                                                                           c.divergence);
            }
            CK_LAUNCH();
        }
        dfree(nch, s);
        dfree(first, s);
        dfree(item_node, s);
        dfree(partial, s);
    }
    c.kend(kt);
    dfree(fc, s);
    dfree(rs, s);
}

}  // namespace prgpu
