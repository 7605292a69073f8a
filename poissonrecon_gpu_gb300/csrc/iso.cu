// Iso-surface stage: implicit function at the points, iso-value, octree corner
// values, marching cubes on the finest nodes and on subdivided coarse leaves.
// Replaces main.cu:1334-1381 and 1438-4561.
//
// Differences in mechanism (not in result) from the reference:
//   * corners, edges and faces are not materialised as records; each cell finds
//     the owner of a corner/edge/face (the minimum key among the cells that
//     share it, as initVertexOwner/initEdgeArray/initFaceArray do) from its
//     neighbour table, and a corner value is evaluated once, by its owner;
//   * edge vertices are de-duplicated by sorting edge keys (batch, lattice
//     edge) instead of by owner back-links, one sort for the whole mesh;
//   * subdivided leaves are never expanded into node arrays: their finest cells
//     are enumerated implicitly, and the real nodes around them are reached by
//     descending from the leaf's neighbour table.
// Every vertex value, crossing position and triangle follows the reference's
// arithmetic and owner rules.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "context.h"
#include "mc_table.h"
#include "prims.cuh"

namespace prgpu {

__constant__ int c_tri_count[256];
__constant__ signed char c_tri_edges[256][16];
__constant__ signed char c_edge_v[12][2];
__constant__ signed char c_pfk[8][6];        // parentFaceKind, reference layout
__constant__ signed char c_vid[8];           // cube-vertex id of corner kind j
__constant__ signed char c_face_edges[6][4];

// the tables go to each device's constant memory once (contexts may run on several host threads)
static std::mutex g_mc_mu;
static bool g_mc_uploaded[64] = {false};
static void upload_mc_tables() {
    prgpu_mc::Tables T;
    prgpu_mc::build(T);
    signed char te[256][16], ev[12][2], pfk[8][6], vid[8], fe[6][4];
    for (int c = 0; c < 256; ++c)
        for (int k = 0; k < 16; ++k) te[c][k] = (signed char)T.tri_edges[c][k];
    for (int e = 0; e < 12; ++e) { ev[e][0] = (signed char)T.edge_v[e][0]; ev[e][1] = (signed char)T.edge_v[e][1]; }
    for (int s = 0; s < 8; ++s) {
        int xyz[3] = {s & 1, (s >> 1) & 1, (s >> 2) & 1};
        for (int j = 0; j < 6; ++j) pfk[s][j] = (signed char)((xyz[j >> 1] == (j & 1)) ? j : -1);
    }
    pfk[7][0] = 0;   // the reference table's last row also lists face 0 (MarchingCubes.cuh:716)
    for (int j = 0; j < 8; ++j) vid[j] = (signed char)prgpu_mc::vertex_id(j & 1, (j >> 1) & 1, (j >> 2) & 1);
    for (int f = 0; f < 6; ++f) {
        int a = f >> 1, sd = f & 1, n = 0;
        for (int e = 0; e < 12; ++e) {
            int o = e >> 2;
            if (o == a) continue;
            int a0 = (o == 0) ? 1 : 0;
            int off = (a == a0) ? (e & 1) : ((e >> 1) & 1);
            if (off == sd) fe[f][n++] = (signed char)e;
        }
    }
    CK(cudaMemcpyToSymbol(c_tri_count, T.tri_count, sizeof T.tri_count));
    CK(cudaMemcpyToSymbol(c_tri_edges, te, sizeof te));
    CK(cudaMemcpyToSymbol(c_edge_v, ev, sizeof ev));
    CK(cudaMemcpyToSymbol(c_pfk, pfk, sizeof pfk));
    CK(cudaMemcpyToSymbol(c_vid, vid, sizeof vid));
    CK(cudaMemcpyToSymbol(c_face_edges, fe, sizeof fe));
}
static void ensure_mc_tables() {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_mc_mu);
    if (dev < 0 || dev >= 64) throw Error{PRGPU_ERR_LIMIT, {0}};
    if (!g_mc_uploaded[dev]) {
        upload_mc_tables();
        g_mc_uploaded[dev] = true;
    }
}

// ----------------------------- evaluation ----------------------------------
struct EvalArgs {
    NodeArrays nd;
    int D;
    const CPoly* basis;
    const float* x;
    const float* x27;      // nodes [0, nx27): x of the 27 neighbours (0: none), 28 floats per node; or null
    i64 nx27;
    const float* lb;       // basis values at finest-lattice points (see lattice_basis), or null
    int stable;            // params.stable_basis: closed-form basis values (basis_stable)
};

// start of depth d in the lattice basis table: sum_{l<d} 2^l (3 2^(D-l) + 1) = 3 d 2^D + 2^d - 1
__device__ __host__ __forceinline__ i64 lattice_basis_offset(int D, int d) {
    return 3ll * d * (1ll << D) + (1ll << d) - 1;
}

// B_{d,n}(u / 2^D) for a finest-lattice coordinate u: the value cpoly_value
// computes, read from the table when u lies in the support [(n-1)w, (n+2)w]
// (w = 2^(D-d), 3w+1 points per function), evaluated otherwise
__device__ __forceinline__ float lattice_basis(const EvalArgs& a, int d, int n, int u) {
    const int w = 1 << (a.D - d);
    const int k = u - (n - 1) * w;
    if (a.lb && k >= 0 && k <= 3 * w) return a.lb[lattice_basis_offset(a.D, d) + (i64)n * (3 * w + 1) + k];
    if (a.stable) return basis_stable(d, n, (float)u * (1.0f / (float)(1 << a.D)));
    return cpoly_value<3>(a.basis[(1 << d) - 1 + n], (float)u * (1.0f / (float)(1 << a.D)));
}

__global__ void k_lattice_basis(const CPoly* __restrict__ basis, int D, i64 total, float* __restrict__ lb, int stable) {
    const float inv = 1.0f / (float)(1 << D);
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        // depth d holds 2^d functions of 3w+1 points: offset sum_{l<d} 2^l (3 2^(D-l) + 1)
        int d = 0;
        i64 off = 0;
        for (;;) {
            const i64 len = (1ll << d) * (3ll * (1ll << (D - d)) + 1);
            if (e < off + len) break;
            off += len;
            ++d;
        }
        const int w = 1 << (D - d);
        const i64 r = e - off;
        const int n = (int)(r / (3 * w + 1)), k = (int)(r % (3 * w + 1));
        const float q = (float)((n - 1) * w + k) * inv;
        lb[e] = stable ? basis_stable(d, n, q) : cpoly_value<3>(basis[(1 << d) - 1 + n], q);
    }
}

// x of the 27 neighbours of every node below the finest depth, contiguous per
// node (the evaluation walks read one 112-byte row per ancestor)
constexpr int X27_STRIDE = 28;
__global__ void k_build_x27(NodeArrays nd, const float* __restrict__ x, i64 n, float* __restrict__ x27) {
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < n * X27_STRIDE; e += (i64)gridDim.x * blockDim.x) {
        const i64 i = e / X27_STRIDE;
        const int j = (int)(e % X27_STRIDE);
        float v = 0.f;
        if (j < 27) {
            const int nb = nd.neigh[(i64)j * nd.M + i];
            if (nb != -1) v = x[nb];
        }
        x27[e] = v;
    }
}

// sum over the 27 neighbours of real node 'node' (at depth d, coordinates xyz)
// of x_n * B_n(q), in neighbour order with the reference's FMA
// (calculatePointsImplicitFunctionValue main.cu:1351-1377)
__device__ __forceinline__ float level_sum(const EvalArgs& a, i64 node, int d, const int xyz[3], const float q[3],
                                           float val) {
    const int fb = (1 << d) - 1, lim = 1 << d;
    float bv[3][3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            int c = xyz[ax] + t - 1;
            bv[ax][t] = (c >= 0 && c < lim)
                            ? (a.stable ? basis_stable(d, c, q[ax]) : cpoly_value<3>(a.basis[fb + c], q[ax]))
                            : 0.f;
        }
    if (node < a.nx27) {
        // absent neighbours read 0: adding a zero product leaves the sum unchanged
        const float4* row = reinterpret_cast<const float4*>(a.x27 + node * X27_STRIDE);
        float xs[28];
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            const float4 t = row[k];
            xs[4 * k] = t.x; xs[4 * k + 1] = t.y; xs[4 * k + 2] = t.z; xs[4 * k + 3] = t.w;
        }
#pragma unroll
        for (int j = 0; j < 27; ++j) val = fmaf(xs[j] * bv[0][j / 9] * bv[1][(j / 3) % 3], bv[2][j % 3], val);
        return val;
    }
    const i64 M = a.nd.M;
#pragma unroll
    for (int j = 0; j < 27; ++j) {
        const int nb = a.nd.neigh[(i64)j * M + node];
        if (nb == -1) continue;
        const float vx = bv[0][j / 9], vy = bv[1][(j / 3) % 3], vz = bv[2][j % 3];
        val = fmaf(a.x[nb] * vx * vy, vz, val);
    }
    return val;
}

// the x27 rows for nodes [0, n) on the stage's stream; null when n is 0
inline float* build_x27(const Ctx& c, i64 n) {
    if (n <= 0) return nullptr;
    float* x27 = dalloc<float>(n * X27_STRIDE, c.stream);
    k_build_x27<<<grid_for(n * X27_STRIDE, 256), 256, 0, c.stream>>>(c.nodes, c.x, n, x27);
    CK_LAUNCH();
    return x27;
}

// level_sum at a finest-lattice point u (q = u / 2^D), basis values from the table
__device__ __forceinline__ float level_sum_u(const EvalArgs& a, i64 node, int d, const int xyz[3], const int u[3],
                                             float val) {
    const int lim = 1 << d;
    float bv[3][3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            const int c = xyz[ax] + t - 1;
            bv[ax][t] = (c >= 0 && c < lim) ? lattice_basis(a, d, c, u[ax]) : 0.f;
        }
    if (node < a.nx27) {
        const float4* row = reinterpret_cast<const float4*>(a.x27 + node * X27_STRIDE);
        float xs[28];
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            const float4 t = row[k];
            xs[4 * k] = t.x; xs[4 * k + 1] = t.y; xs[4 * k + 2] = t.z; xs[4 * k + 3] = t.w;
        }
#pragma unroll
        for (int j = 0; j < 27; ++j) val = fmaf(xs[j] * bv[0][j / 9] * bv[1][(j / 3) % 3], bv[2][j % 3], val);
        return val;
    }
    const i64 M = a.nd.M;
#pragma unroll
    for (int j = 0; j < 27; ++j) {
        const int nb = a.nd.neigh[(i64)j * M + node];
        if (nb == -1) continue;
        val = fmaf(a.x[nb] * bv[0][j / 9] * bv[1][(j / 3) % 3], bv[2][j % 3], val);
    }
    return val;
}
// from a node to the root: a parent is one depth up and its cell coordinates are the
// child's halved, so the node's key is decoded once
__device__ __forceinline__ float walk_up_u(const EvalArgs& a, i64 node, const int u[3], float val) {
    if (node == -1) return val;
    int d = a.nd.depth[node];
    int xyz[3];
    key_coords(a.nd.key[node], d, a.D, xyz);
    while (node != -1) {
        val = level_sum_u(a, node, d, xyz, u, val);
        node = a.nd.parent[node];
        --d;
        xyz[0] >>= 1; xyz[1] >>= 1; xyz[2] >>= 1;
    }
    return val;
}

__device__ __forceinline__ float walk_up(const EvalArgs& a, i64 node, const float q[3], float val) {
    if (node == -1) return val;
    int d = a.nd.depth[node];
    int xyz[3];
    key_coords(a.nd.key[node], d, a.D, xyz);
    while (node != -1) {
        val = level_sum(a, node, d, xyz, q, val);
        node = a.nd.parent[node];
        --d;
        xyz[0] >>= 1; xyz[1] >>= 1; xyz[2] >>= 1;
    }
    return val;
}

// the iso-value sum: sum of f(p), or of w(p) f(p) with density weights (mean 1)
__global__ void k_point_values(EvalArgs a, const float* __restrict__ pts, const int* __restrict__ point_node, i64 n,
                               const float* __restrict__ weight, float* __restrict__ out, double* __restrict__ sum) {
    double loc = 0;
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
        const float q[3] = {pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]};
        const float v = walk_up(a, point_node[k], q, 0.f);
        out[k] = v;
        if (weight) loc += (double)v * (double)weight[k];
        else loc += (double)v;
    }
    for (int o = 16; o; o >>= 1) loc += __shfl_xor_sync(0xffffffffu, loc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, loc);
}

void stage_points(Ctx& c) {
    cudaStream_t s = c.stream;
    dfree(c.point_value, s);
    c.point_value = dalloc<float>(c.N, s);
    double* sum = dalloc<double>(1, s);
    CK(cudaMemsetAsync(sum, 0, sizeof(double), s));
    float* x27 = build_x27(c, c.base[c.D]);
    EvalArgs a{c.nodes, c.D, c.basis, c.x, x27, x27 ? c.base[c.D] : 0, nullptr, c.params.stable_basis};
    const int kt = c.kbegin("point_values", (double)c.N * (12 + 4 + 4) + (double)c.nodes.M * (4 + 4 + 8 + 108));
    k_point_values<<<grid_for(c.N, 128, 1ll << 30), 128, 0, s>>>(a, c.pts, c.point_node, c.N, c.point_weight,
                                                                 c.point_value, sum);
    CK_LAUNCH();
    c.kend(kt);
    double h = read_scalar(sum, s);
    dfree(sum, s);
    dfree(x27, s);
    c.iso = (float)h / (float)c.N;
}

// ------------------------------ corners -------------------------------------
// owner of the corner 'kind' of real node i (min key among same-depth nodes
// sharing the corner); returns the owner and the corner's kind in its frame
__device__ __forceinline__ int corner_owner(const NodeArrays& nd, i64 i, int kind, int& okind) {
    const int sx = kind & 1, sy = (kind >> 1) & 1, sz = (kind >> 2) & 1;
    const i64 M = nd.M;
    u64 best = ~0ull;
    int own = -1;
    okind = kind;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int ex = e & 1, ey = (e >> 1) & 1, ez = (e >> 2) & 1;
        const int dx = sx - ex, dy = sy - ey, dz = sz - ez;
        const int j = 9 * (dx + 1) + 3 * (dy + 1) + (dz + 1);
        const int nb = nd.neigh[(i64)j * M + i];
        if (nb == -1) continue;
        const u64 kk = nd.key[nb];
        if (kk < best) { best = kk; own = nb; okind = ex | (ey << 1) | (ez << 2); }
    }
    return own;
}

__device__ __forceinline__ void corner_pos(const int xyz[3], int d, int kind, float q[3]) {
    const float inv = 1.0f / (float)(1 << d);
    q[0] = (float)(xyz[0] + (kind & 1)) * inv;
    q[1] = (float)(xyz[1] + ((kind >> 1) & 1)) * inv;
    q[2] = (float)(xyz[2] + ((kind >> 2) & 1)) * inv;
}

// value of corner 'kind' of owner o, minus the iso-value
// (computeVertexImplicitFunctionValue main.cu:2259-2326, including its descent
// through children[childrenVertexKind[kind]])
__device__ float owner_corner_value(const EvalArgs& a, i64 o, int kind, float iso) {
    const int d = a.nd.depth[o];
    int xyz[3];
    key_coords(a.nd.key[o], d, a.D, xyz);
    // the corner as a finest-lattice point: (xyz + bit) / 2^d = u / 2^D exactly
    const int sh = a.D - d;
    const int u[3] = {(xyz[0] + (kind & 1)) << sh, (xyz[1] + ((kind >> 1) & 1)) << sh, (xyz[2] + ((kind >> 2) & 1)) << sh};
    float val = 0.f;
    if (o > 0) {
        val = walk_up_u(a, o, u, val);
        const int exceed = c_vid[kind];
        i64 node = o;
        int cx[3] = {xyz[0], xyz[1], xyz[2]};
        for (int dd = d + 1; dd <= a.D; ++dd) {
            const int c0 = a.nd.child0[node];
            if (c0 == -1) break;
            node = c0 + exceed;   // child 'exceed': its coordinates are the parent's doubled plus its bits
            cx[0] = (cx[0] << 1) | ((exceed >> 2) & 1);
            cx[1] = (cx[1] << 1) | ((exceed >> 1) & 1);
            cx[2] = (cx[2] << 1) | (exceed & 1);
            val = level_sum_u(a, node, dd, cx, u, val);
        }
    }
    return val - iso;
}

// for each corner k in 'mask' of node 'node' (depth d, coordinates xyz): the
// walk_up_u sum from the node to the root at the corner's lattice point
// (xyz + bit) << sh, all corners sharing the walk (the same levels and
// neighbour x, each corner with its own basis values and FMA chain)
__device__ __forceinline__ void walk_up_corners(const EvalArgs& a, i64 node, int d, const int xyz[3], int sh,
                                                unsigned mask, float val[8]) {
    const NodeArrays& nd = a.nd;
    const i64 M = nd.M;
#pragma unroll
    for (int k = 0; k < 8; ++k) val[k] = 0.f;
    int c[3] = {xyz[0], xyz[1], xyz[2]};
    while (node != -1) {
        float xs[27];
        if (node < a.nx27) {
            const float4* row = reinterpret_cast<const float4*>(a.x27 + node * X27_STRIDE);
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const float4 t = row[k];
                xs[4 * k] = t.x; xs[4 * k + 1] = t.y; xs[4 * k + 2] = t.z; xs[4 * k + 3] = t.w;
            }
            const float4 t = row[6];
            xs[24] = t.x; xs[25] = t.y; xs[26] = t.z;
        } else {
#pragma unroll
            for (int j = 0; j < 27; ++j) {
                const int nb = nd.neigh[(i64)j * M + node];
                xs[j] = nb == -1 ? 0.f : a.x[nb];   // absent: a zero product leaves the sum unchanged
            }
        }
        const int lim = 1 << d;
#pragma unroll 1
        for (int kind = 0; kind < 8; ++kind) {
            if (!((mask >> kind) & 1)) continue;
            const int u[3] = {(xyz[0] + (kind & 1)) << sh, (xyz[1] + ((kind >> 1) & 1)) << sh,
                              (xyz[2] + ((kind >> 2) & 1)) << sh};
            float bv[3][3];
#pragma unroll
            for (int ax = 0; ax < 3; ++ax)
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    const int n = c[ax] + t - 1;
                    bv[ax][t] = (n >= 0 && n < lim) ? lattice_basis(a, d, n, u[ax]) : 0.f;
                }
            float v = val[kind];
#pragma unroll
            for (int j = 0; j < 27; ++j) v = fmaf(xs[j] * bv[0][j / 9] * bv[1][(j / 3) % 3], bv[2][j % 3], v);
            val[kind] = v;
        }
        node = nd.parent[node];
        --d;
        c[0] >>= 1; c[1] >>= 1; c[2] >>= 1;
    }
}

// finest-depth corners: each corner evaluated by its owner.  A node owns a
// corner when no other existing node of the 8 around it has a smaller key.
// Pass 1 (one thread per node): the mask of owned corners and their count.
__global__ void k_finest_owned(NodeArrays nd, i64 lo, i64 hi, unsigned char* __restrict__ owned_mask,
                               int* __restrict__ owned_count) {
    const i64 M = nd.M;
    for (i64 i = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (i64)gridDim.x * blockDim.x) {
        const u64 ki = nd.key[i];
        unsigned smaller = 0;   // bit j: neighbour j exists and has a smaller key
#pragma unroll
        for (int j = 0; j < 27; ++j) {
            if (j == 13) continue;
            const int nb = nd.neigh[(i64)j * M + i];
            if (nb != -1 && nd.key[nb] < ki) smaller |= 1u << j;
        }
        unsigned owned = 0;
#pragma unroll
        for (int kind = 0; kind < 8; ++kind) {
            const int sx = kind & 1, sy = (kind >> 1) & 1, sz = kind >> 2;
            bool own = true;
#pragma unroll
            for (int e = 1; e < 8; ++e) {
                const int j = 9 * (sx - (e & 1) + 1) + 3 * (sy - ((e >> 1) & 1) + 1) + (sz - (e >> 2) + 1);
                if ((smaller >> j) & 1) own = false;
            }
            if (own) owned |= 1u << kind;
        }
        owned_mask[i - lo] = (unsigned char)owned;
        owned_count[i - lo] = __popc(owned);
    }
}

// the owned corners as a list: (finest slot << 3) | corner
__global__ void k_finest_list(const unsigned char* __restrict__ owned_mask, const int* __restrict__ first, i64 nD,
                              int* __restrict__ list) {
    for (i64 l = (i64)blockIdx.x * blockDim.x + threadIdx.x; l < nD; l += (i64)gridDim.x * blockDim.x) {
        unsigned m = owned_mask[l];
        int q = first[l];
        while (m) {
            const int kind = __ffs(m) - 1;
            list[q++] = (int)(l << 3) | kind;
            m &= m - 1;
        }
    }
}

// pass 2 (one thread per owned corner): walk_up_u from the owner at the corner,
// the value of owner_corner_value (no descent at the finest depth)
__global__ void __launch_bounds__(128, 12) k_finest_corner_values(EvalArgs a, i64 lo, const int* __restrict__ list,
                                                                 i64 ncorner, float iso, float* __restrict__ cval) {
    const int D = a.D;
    for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < ncorner; q += (i64)gridDim.x * blockDim.x) {
        const int lk = list[q];
        const i64 l = lk >> 3;
        const int kind = lk & 7;
        const i64 i = lo + l;
        int xyz[3];
        key_coords(a.nd.key[i], D, D, xyz);
        const int u[3] = {xyz[0] + (kind & 1), xyz[1] + ((kind >> 1) & 1), xyz[2] + (kind >> 2)};
        cval[8 * l + kind] = walk_up_u(a, i, u, 0.f) - iso;
    }
}

// corner values of each finest cell (from the owners), cube category, triangle count
__global__ void k_finest_cells(NodeArrays nd, i64 lo, i64 hi, const float* __restrict__ cval, float* __restrict__ cell_v,
                               unsigned char* __restrict__ cat, int* __restrict__ ntri) {
    for (i64 i = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (i64)gridDim.x * blockDim.x) {
        int cc = 0;
        for (int kind = 0; kind < 8; ++kind) {
            int ok;
            const int own = corner_owner(nd, i, kind, ok);
            const float v = cval[8 * ((i64)own - lo) + ok];
            cell_v[8 * (i - lo) + kind] = v;
            if (v < 0.f) cc |= 1 << c_vid[kind];
        }
        cat[i - lo] = (unsigned char)cc;
        ntri[i - lo] = c_tri_count[cc];
    }
}

// ------------------------------- faces ---------------------------------------
// owner record of face j of node n: (owner node, face kind in its frame)
__device__ __forceinline__ void face_owner(const NodeArrays& nd, i64 n, int j, int& o, int& k) {
    const int ax = j >> 1, sd = j & 1;
    int dxyz[3] = {0, 0, 0};
    dxyz[ax] = sd ? 1 : -1;
    const int jj = 9 * (dxyz[0] + 1) + 3 * (dxyz[1] + 1) + (dxyz[2] + 1);
    const int nb = nd.neigh[(i64)jj * nd.M + n];
    if (nb != -1 && nd.key[nb] < nd.key[n]) { o = nb; k = j ^ 1; }
    else { o = (int)n; k = j; }
}
__device__ __forceinline__ int face_has_parent(const NodeArrays& nd, int o, int k, int D) {
    if (nd.parent[o] == -1) return -1;
    const int d = nd.depth[o];
    const int son = (int)((nd.key[o] >> (3 * (D - d))) & 7);
    return c_pfk[son][k] != -1 ? 1 : -1;
}

// surface-intersection marks (generateTrianglePos main.cu:2736-2755)
__global__ void k_mark_faces(NodeArrays nd, int D, i64 lo, i64 hi, const unsigned char* __restrict__ cat,
                             int* __restrict__ fflag) {
    for (i64 i = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (i64)gridDim.x * blockDim.x) {
        const int cc = cat[i - lo];
        const int nt = c_tri_count[cc];
        if (!nt) continue;
        int used = 0;
        for (int t = 0; t < 3 * nt; ++t) used |= 1 << c_tri_edges[cc][t];
        for (int j = 0; j < 6; ++j) {
            int m = 0;
            for (int q = 0; q < 4; ++q) m |= (used >> c_face_edges[j][q]) & 1;
            if (!m) continue;
            int o, k;
            face_owner(nd, i, j, o, k);
            fflag[6 * (i64)o + k] = 1;
            int par = nd.parent[i];
            while (face_has_parent(nd, o, k, D) != -1) {
                face_owner(nd, par, j, o, k);
                par = nd.parent[par];
                fflag[6 * (i64)o + k] = 1;
            }
        }
    }
}

// corners of the leaves above the finest depth: mark each owner's corner once
__global__ void k_coarse_need(NodeArrays nd, i64 lo, i64 hi, unsigned char* __restrict__ need) {
    for (i64 i = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (i64)gridDim.x * blockDim.x) {
        if (nd.child0[i] != -1) continue;
        for (int kind = 0; kind < 8; ++kind) {
            int ok;
            const int own = corner_owner(nd, i, kind, ok);
            need[8 * (i64)own + ok] = 1;
        }
    }
}
// the needed corners of one node share the walk up (owner_corner_value: walk
// up, then for each corner its own descent through children[childrenVertexKind])
__global__ void __launch_bounds__(128, 6) k_coarse_corner_values(EvalArgs a, i64 n, float iso,
                                                                 const unsigned char* __restrict__ need,
                                                                 float* __restrict__ cval) {
    const NodeArrays& nd = a.nd;
    const int D = a.D;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        unsigned mask = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) mask |= need[8 * i + k] ? (1u << k) : 0u;
        if (!mask) continue;
        float val[8];
        if (i == 0) {
#pragma unroll
            for (int k = 0; k < 8; ++k) val[k] = 0.f;   // the root has no corner value of its own
        } else {
            const int d = nd.depth[i];
            int xyz[3];
            key_coords(nd.key[i], d, D, xyz);
            const int sh = D - d;
            walk_up_corners(a, i, d, xyz, sh, mask, val);
            if (nd.child0[i] != -1) {
#pragma unroll 1
                for (int kind = 0; kind < 8; ++kind) {
                    if (!((mask >> kind) & 1)) continue;
                    const int u[3] = {(xyz[0] + (kind & 1)) << sh, (xyz[1] + ((kind >> 1) & 1)) << sh,
                                      (xyz[2] + ((kind >> 2) & 1)) << sh};
                    const int exceed = c_vid[kind];
                    i64 node = i;
                    float v = val[kind];
                    int cx[3] = {xyz[0], xyz[1], xyz[2]};
                    for (int dd = d + 1; dd <= D; ++dd) {
                        const int c0 = nd.child0[node];
                        if (c0 == -1) break;
                        node = c0 + exceed;
                        cx[0] = (cx[0] << 1) | ((exceed >> 2) & 1);
                        cx[1] = (cx[1] << 1) | ((exceed >> 1) & 1);
                        cx[2] = (cx[2] << 1) | (exceed & 1);
                        v = level_sum_u(a, node, dd, cx, u, v);
                    }
                    val[kind] = v;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if ((mask >> k) & 1) cval[8 * i + k] = val[k] - iso;
    }
}

// needed corners of each coarse node as a mask and a count
__global__ void k_need_mask(const unsigned char* __restrict__ need, i64 n, unsigned char* __restrict__ mask,
                            int* __restrict__ count) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        unsigned m = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) m |= need[8 * i + k] ? (1u << k) : 0u;
        mask[i] = (unsigned char)m;
        count[i] = __popc(m);
    }
}
__global__ void __launch_bounds__(128, 8) k_coarse_corner_list(EvalArgs a, const int* __restrict__ list, i64 n,
                                                               float iso, float* __restrict__ cval) {
    for (i64 q = (i64)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (i64)gridDim.x * blockDim.x) {
        const int lk = list[q];
        cval[lk] = owner_corner_value(a, lk >> 3, lk & 7, iso);   // cval index = 8 node + corner
    }
}

// leaves above the finest depth: sign change at their corners or a marked face
// (ProcessLeafNodesAtOtherDepth main.cu:2957-2986, ifSubdivide :2988-2992)
// (at most 64 registers: unbounded, the 8 corner-owner and 6 face-owner searches take 167
// registers and leave one warp in eight resident; measured 0.84 -> 0.66 ms with the stage's lists)
__global__ void __launch_bounds__(128, 8) k_coarse_leaves(EvalArgs a, i64 lo, i64 hi, const float* __restrict__ cval,
                                const int* __restrict__ fflag, int* __restrict__ has_tri, int* __restrict__ has_int,
                                int* __restrict__ is_root) {
    const NodeArrays& nd = a.nd;
    for (i64 i = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (i64)gridDim.x * blockDim.x) {
        if (nd.child0[i] != -1) { is_root[i] = 0; continue; }
        float v[8];
        for (int kind = 0; kind < 8; ++kind) {
            int ok;
            const int own = corner_owner(nd, i, kind, ok);
            v[c_vid[kind]] = cval[8 * (i64)own + ok];
        }
        const int sign = v[0] < 0 ? -1 : 1;
        int ht = 0;
        for (int j = 1; j < 8; ++j)
            if ((float)sign * v[j] < 0) { ht = 1; break; }
        int hi2 = 0;
        for (int j = 0; j < 6; ++j) {
            int o, k;
            face_owner(nd, i, j, o, k);
            if (fflag[6 * (i64)o + k]) { hi2 = 1; break; }
        }
        has_tri[i] = ht;
        has_int[i] = hi2;
        is_root[i] = (ht || hi2) ? 1 : 0;
    }
}

// ------------------------ subdivided leaves (virtual) ------------------------
struct VRoot {
    int node;          // real empty leaf
    int depth;         // r
    int batch;         // vertex-sharing batch id (1-based)
    int pad;
};

struct VArgs {
    EvalArgs e;
    const VRoot* roots;
    int nroots;
    const int* batch_root_flag;   // per node: batch id if the node is a root of a depth batch (>= 3), else 0
    float iso;
};

// real node at depth d with coordinates c[] reached from the depth-r node a
// (its ancestor), or -1
__device__ __forceinline__ i64 descend(const NodeArrays& nd, i64 a, int r, int d, const int c[3]) {
    i64 node = a;
    for (int l = r + 1; l <= d; ++l) {
        const int c0 = nd.child0[node];
        if (c0 == -1) return -1;
        const int b = d - l;
        const int k = (((c[0] >> b) & 1) << 2) | (((c[1] >> b) & 1) << 1) | ((c[2] >> b) & 1);
        node = c0 + k;
    }
    return node;
}

// is the finest cell 'cell' (depth-D coordinates) a member of the batch of root R?
// If so returns the root node that contains it (R or another root of R's depth batch).
__device__ __forceinline__ int batch_member(const VArgs& v, const VRoot& R, const int Lc[3], const int cell[3]) {
    const int D = v.e.D, sh = D - R.depth;
    const int lim = 1 << D;
    if (cell[0] < 0 || cell[1] < 0 || cell[2] < 0 || cell[0] >= lim || cell[1] >= lim || cell[2] >= lim) return -1;
    const int A[3] = {cell[0] >> sh, cell[1] >> sh, cell[2] >> sh};
    const int dx = A[0] - Lc[0], dy = A[1] - Lc[1], dz = A[2] - Lc[2];
    if (!dx && !dy && !dz) return R.node;
    if (R.depth < 3) return -1;                 // single-root batch
    const int j = 9 * (dx + 1) + 3 * (dy + 1) + (dz + 1);
    const int nb = v.e.nd.neigh[(i64)j * v.e.nd.M + R.node];
    if (nb == -1) return -1;
    return (v.batch_root_flag[nb] == R.batch) ? nb : -1;
}

// value at finest corner q (lattice coordinates) for a walk starting at the
// finest cell 'oc' inside root node L (computeSubdivideVertexImplicitFunctionValue
// main.cu:2328-2442): virtual levels contribute only the real nodes around them
__device__ float virtual_corner_value(const VArgs& v, int L, int r, const int oc[3], const int qc[3]) {
    const EvalArgs& a = v.e;
    const NodeArrays& nd = a.nd;
    const int D = a.D;
    int Lc[3];
    key_coords(nd.key[L], r, D, Lc);
    float val = 0.f;
    for (int d = D; d > r; --d) {
        const int sh = D - d;
        const int V[3] = {oc[0] >> sh, oc[1] >> sh, oc[2] >> sh};
        const int lim = 1 << d;
        // a virtual cell whose 3x3x3 block lies inside the leaf has no real neighbour
        const int span = 1 << (d - r);
        bool inner = true;
        for (int ax = 0; ax < 3; ++ax) {
            const int lo = Lc[ax] * span;
            if (V[ax] - 1 < lo || V[ax] + 1 >= lo + span) inner = false;
        }
        if (inner) continue;
        float bv[3][3];
        for (int ax = 0; ax < 3; ++ax)
            for (int t = 0; t < 3; ++t) {
                int cc = V[ax] + t - 1;
                bv[ax][t] = (cc >= 0 && cc < lim) ? lattice_basis(a, d, cc, qc[ax]) : 0.f;
            }
        for (int j = 0; j < 27; ++j) {
            const int N[3] = {V[0] + j / 9 - 1, V[1] + (j / 3) % 3 - 1, V[2] + j % 3 - 1};
            if (N[0] < 0 || N[1] < 0 || N[2] < 0 || N[0] >= lim || N[1] >= lim || N[2] >= lim) continue;
            const int s2 = d - r;
            const int A[3] = {N[0] >> s2, N[1] >> s2, N[2] >> s2};
            const int ddx = A[0] - Lc[0], ddy = A[1] - Lc[1], ddz = A[2] - Lc[2];
            if (!ddx && !ddy && !ddz) continue;    // inside the subdivided leaf: no coefficient
            const int jj = 9 * (ddx + 1) + 3 * (ddy + 1) + (ddz + 1);
            const int an = nd.neigh[(i64)jj * nd.M + L];
            if (an == -1) continue;
            const i64 node = descend(nd, an, r, d, N);
            if (node < 0) continue;
            const float vx = bv[0][j / 9], vy = bv[1][(j / 3) % 3], vz = bv[2][j % 3];
            val = fmaf(a.x[node] * vx * vy, vz, val);
        }
    }
    // the leaf itself and its real ancestors
    val = walk_up_u(a, L, qc, val);
    return val;
}

__device__ __forceinline__ u64 cell_key_D(const int c[3], int D) { return coords_key(c[0], c[1], c[2], D, D); }

// ---- subdivided leaves in bricks: the leaf's lattice of finest cells is cut
// into bricks of B^3 cells, B = min(lattice edge, 8).
//
// Most corners of a subdivided leaf lie far from the surface.  Each brick is
// bounded before any of its corners is evaluated:
//   * every term of a corner value is x_n * B_x * B_y * B_z with the
//     single-precision basis values the evaluation uses, so the range of a term
//     over the corners that include it is an interval product; terms that only
//     some corners include get intervals widened to 0;
//   * the rounding of the FMA chain is at most (K + 4) u sum|term| for K terms
//     (u = 2^-24);
//   * a brick whose bound proves that every corner value has the same sign as
//     (value - iso) is culled: none of its cells carries a triangle and its
//     corners are never read.
// The surviving ("live") bricks are evaluated exactly, in the order of
// virtual_corner_value, so culling changes no value.  Corners on the leaf's
// lower faces may be owned by a cell of another leaf of the same depth batch
// ("foreign" corners): their virtual depths read the same window (a real node
// is the same node in either leaf's frame, and every cell inside either leaf
// reads 0), their real ancestors are the owner's.  Such a corner is a corner
// of the owner leaf's brick that contains its owner cell, where the owner's own
// bound covers it; so a brick with foreign corners is culled only when its own
// bound and those of the owner bricks prove the same sign.
//
// The basis values a brick's corners use along one axis depend only on the
// leaf, the axis and the brick's index along it (a "brick row"):
//   BT[d][t][k]   basis value at corner k of the function of cell V_k + t - 1
//                 (depth d > r, V_k = (corner - 1) >> (D - d), t = 0..3; t = 3
//                 serves owner cells V_k + 1) or of ancestor cell + t - 1
//                 (depth d <= r); built per live brick by k_brick_eval
//   RA[l][t]      range over k of BT[l][t][k], l <= r
//   RW[d][n]      range (with 0) of the depth-d function of window cell n over
//                 the corners whose owner cell is within one cell of it
// RA and RW are tabulated once per row by k_brick_rows for the bounds.
constexpr int BR = 8;              // largest brick edge (cells); corners per axis up to BR+1
constexpr int BR1 = BR + 1;
constexpr int BR_CORNERS = BR1 * BR1 * BR1;
constexpr int BR_BLOCK = 128;
constexpr int BR_LEVELS = 16;      // depths 0..15
constexpr int BR_WEXT = BR + 4;    // window edge at the finest depth, with the extra upper cell
// window cells over all virtual depths of a brick whose first corner is a
// multiple of its edge B <= 8, with the extra upper cell per axis (bricks
// with foreign corners): at most 12^3 + 8^3 + 6^3 + 12 * 5^3 = 3956
constexpr int BR_XW = 3968;
// super-brick row table: RA (6 per depth), RW (24 per depth)
constexpr int ROW_RA = 0, ROW_RW = 6, ROW_PER_DEPTH = 30;
// brick row table: 24 floats per depth d > r (the ancestors, d <= r, are one polynomial per leaf)
//   d <= D - lg E  PW[n]  window cell n < 4: Bernstein form over the brick's corners (b0, b1, b2, M,
//                         see bern_fit) of its function, masked as RW is; the function's knots are
//                         multiples of its cell width 2^(D-d) >= E, so it is one quadratic piece there
//   d >  D - lg E  RW[n]  as above (12 cells, range with 0)
constexpr int PROW = 24;
constexpr int PW = 4;              // window cells per axis at the depths of knot spacing >= E
constexpr int ANC_STRIDE = 32;     // per root: Bernstein coefficients C[27] of the ancestors, S3, count, FIT

__device__ __forceinline__ int brick_edge(int D, int r) { return min(1 << (D - r), BR); }

// Roots are in depth order and every root of depth d has the same number of bricks
// (8^lg[d]) and super-bricks (8^slg[d]), so the root of a brick follows from the
// per-depth counts without a search.
struct DepthLayout {
    int first[17];                 // first root of depth d
    int lg[17], slg[17];           // log2 of bricks (super-bricks) per leaf edge at depth d
    i64 boff[17], soff[17];        // bricks (super-bricks) of the roots above depth d
    i64 roff[17], sroff[17];       // brick rows (super-brick rows) of the roots above depth d
};
struct BrickIndex {                // bricks of all subdivided leaves, numbered root by root
    const i64* prefix;             // first brick of each root
    const i64* row_prefix;         // first brick row of each root (3 * bricks per edge rows each)
    int nroots;
    const float* rows;             // brick-row tables, PROW (D+1) floats each
    const float* xl;               // per root: x of the 27 neighbours of each ancestor, 16 x 27
    const float* anc;              // per root: the ancestor polynomial, ANC_STRIDE floats
    DepthLayout dl;
};
struct VBrick {
    int root;                      // index into roots
    int b[3];                      // brick coordinates in the leaf
};
__device__ __forceinline__ VBrick brick_of(const VArgs& v, const BrickIndex& bx, i64 g) {
    const DepthLayout& L = bx.dl;
    int d = 0;
    while (d < v.e.D - 1 && L.boff[d + 1] <= g) ++d;   // roots are coarse nodes: depth < D
    const i64 loc = g - L.boff[d];
    const int lg = L.lg[d];
    VBrick b;
    b.root = L.first[d] + (int)(loc >> (3 * lg));
    const i64 l = loc & ((1ll << (3 * lg)) - 1);
    const int m = (1 << lg) - 1;
    b.b[0] = (int)(l >> (2 * lg));
    b.b[1] = (int)(l >> lg) & m;
    b.b[2] = (int)l & m;
    return b;
}
__device__ __forceinline__ const float* brick_row(const BrickIndex& bx, int D, int root, int nb, int ax, int b) {
    return bx.rows + (bx.row_prefix[root] + (i64)ax * nb + b) * (i64)(PROW * (D + 1));
}

__device__ __forceinline__ float f4_at(const float4& f, int i) { return i == 0 ? f.x : (i == 1 ? f.y : f.z); }

// Bernstein form over the corners k = 0..K (K a power of two <= 2^15) of a function tabulated
// there, val(k), that is one quadratic piece over them in exact arithmetic: b0 = v(0), b2 = v(K),
// b1 = 2 v(K/2) - (b0 + b2) / 2 (the quadratic Q through the three), returned as (b0, b1, b2, delta)
// with delta >= max_k |Q(k) - v(k)|.  The tabulated values are the reference's float evaluations of
// shifted polynomials, whose error grows about 4x per depth (near 1e-3 at depth 8 of a depth-10
// tree), so delta is that noise rather than rounding.  Q(k) = b0 B0 + b1 B1 + b2 B2 with
// B0 = (K-k)^2 / K^2, B1 = 2k(K-k) / K^2, B2 = k^2 / K^2 (exact in float for K <= 2^12, else rounded
// once); its float evaluation is within 4u max|b| of Q (the 5u max|b| term), a float |a - b| is
// within u of exact (the factor 1 + 2^-20), and the factor 1 + 2^-16 covers the last roundings.
template <class F>
__device__ __forceinline__ float4 bern_fit(F val, int K) {
    const float v0 = val(0), vm = val(K >> 1), vK = val(K);
    const float b1 = 2.0f * vm - 0.5f * (v0 + vK);
    const float mb = fmaxf(fmaxf(fabsf(v0), fabsf(vK)), fabsf(b1));
    const float inv = 1.0f / ((float)K * (float)K);   // a power of two: exact
    float dmax = 0.f;
    for (int k = 0; k <= K; ++k) {
        const float vk = val(k);
        const float B0 = (float)((K - k) * (K - k)) * inv, B1 = (float)(2 * k * (K - k)) * inv,
                    B2 = (float)(k * k) * inv;
        const float q = fmaf(v0, B0, fmaf(b1, B1, vK * B2));
        dmax = fmaxf(dmax, fabsf(q - vk));
    }
    const float u = 5.9604644775390625e-08f;   // 2^-24
    const float delta = (dmax * (1.0f + 9.5367431640625e-07f) + 5.0f * u * mb) * (1.0f + 1.52587890625e-05f);
    return make_float4(v0, b1, vK, delta);
}

// M = max|b_i| + delta for an entry (b0, b1, b2, delta) of bern_fit: it bounds |Q| (a Bernstein
// form lies within its coefficients' range) and |v(k)| <= |Q(k)| + delta; rounded up
__device__ __forceinline__ float bern_m(const float4& f) {
    return (fmaxf(fmaxf(fabsf(f.x), fabsf(f.y)), fabsf(f.z)) + f.w) * (1.0f + 9.5367431640625e-07f);
}

__device__ __forceinline__ float x_or_zero(const EvalArgs& a, int node) { return node < 0 ? 0.f : a.x[node]; }

// real node at depth d with coordinates N near leaf L (depth r, coords Lc), or -1 (none, or inside L)
__device__ i64 shell_node(const VArgs& v, int L, int r, const int Lc[3], int d, const int N[3]) {
    const NodeArrays& nd = v.e.nd;
    const int lim = 1 << d;
    if (N[0] < 0 || N[1] < 0 || N[2] < 0 || N[0] >= lim || N[1] >= lim || N[2] >= lim) return -1;
    const int s2 = d - r;
    const int dx = (N[0] >> s2) - Lc[0], dy = (N[1] >> s2) - Lc[1], dz = (N[2] >> s2) - Lc[2];
    if (!dx && !dy && !dz) return -1;
    if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) return -1;   // not a neighbour's cell
    const int an = nd.neigh[(i64)(9 * (dx + 1) + 3 * (dy + 1) + (dz + 1)) * nd.M + L];
    if (an == -1) return -1;
    return descend(nd, an, r, d, N);
}

// the leaf's ancestor levels l <= r of a bound, factored by axis: for every
// (l, jx, jy) the three z terms x[j] * Z[jz] (scalar times interval) are summed,
// then multiplied by the intervals Y[jy] and X[jx].  Interval arithmetic is
// subdistributive, so this encloses every corner's exact ancestor sum as the
// term-by-term form does, with a third of its interval products.  Each end is
// within 5u of the exact factored end per row (3 terms, 2 products), against
// 3u per term in the term-by-term form; the margins allow 2 BR_WEXT u A more.
// amax gains sum |x| |Z| |Y| |X| >= sum |term| over the corners.
__device__ __forceinline__ void ancestor_bound(const float* xl, const float* const row[3], int r, int D, int lane,
                                               float& lo, float& hi, float& amax, int& cnt) {
    const int ra = ROW_RA * (D + 1);
    for (int t = lane; t < 9 * (r + 1); t += 32) {
        const int l = r - t / 9, jx = (t % 9) / 3, jy = t % 3;
        const float* xs = xl + 27 * l + 9 * jx + 3 * jy;
        float slo = 0.f, shi = 0.f, sabs = 0.f;
        for (int jz = 0; jz < 3; ++jz) {
            const float x = xs[jz];
            if (x == 0.f) continue;
            const float zl = row[2][ra + (l * 3 + jz) * 2], zh = row[2][ra + (l * 3 + jz) * 2 + 1];
            const float p0 = x * zl, p1 = x * zh;
            slo += fminf(p0, p1);
            shi += fmaxf(p0, p1);
            sabs += fabsf(x) * fmaxf(fabsf(zl), fabsf(zh));
            ++cnt;
        }
        if (sabs == 0.f) continue;
        const float yl = row[1][ra + (l * 3 + jy) * 2], yh = row[1][ra + (l * 3 + jy) * 2 + 1];
        const float xl0 = row[0][ra + (l * 3 + jx) * 2], xh0 = row[0][ra + (l * 3 + jx) * 2 + 1];
        float c0 = slo * yl, c1 = slo * yh, c2 = shi * yl, c3 = shi * yh;
        const float alo = fminf(fminf(c0, c1), fminf(c2, c3)), ahi = fmaxf(fmaxf(c0, c1), fmaxf(c2, c3));
        c0 = alo * xl0; c1 = alo * xh0; c2 = ahi * xl0; c3 = ahi * xh0;
        lo += fminf(fminf(c0, c1), fminf(c2, c3));
        hi += fmaxf(fmaxf(c0, c1), fmaxf(c2, c3));
        amax += sabs * fmaxf(fabsf(yl), fabsf(yh)) * fmaxf(fabsf(xl0), fabsf(xh0));
    }
}

// can a corner of brick b[] (nb bricks per edge) be owned by a cell of another
// leaf of the batch?  The candidate cells of a corner lie in the leaf or in a
// neighbour at offset (dx,dy,dz): -1 on an axis only for corners on the leaf's
// lower face there, +1 only for corners on its upper face.  A cell outside the
// leaf can have the least key only if one offset is -1 (Morton order is
// monotone per axis).  So: only if such a neighbour is a root of the same batch
// (batch_member's rule)
__device__ __forceinline__ bool brick_foreign_possible(const VArgs& v, const VRoot& R, const int b[3], int nb) {
    if (R.depth < 3 || (b[0] && b[1] && b[2])) return false;
    const NodeArrays& nd = v.e.nd;
    for (int j = 0; j < 27; ++j) {
        const int off[3] = {j / 9 - 1, (j / 3) % 3 - 1, j % 3 - 1};
        bool ok = false, allowed = true;
        for (int ax = 0; ax < 3; ++ax) {
            if (off[ax] == -1) { ok = true; if (b[ax] != 0) allowed = false; }
            if (off[ax] == 1 && b[ax] != nb - 1) allowed = false;
        }
        if (!ok || !allowed) continue;
        const int n = nd.neigh[(i64)j * nd.M + R.node];
        if (n != -1 && v.batch_root_flag[n] == R.batch) return true;
    }
    return false;
}

// window of depth d around a brick (edge B) along one axis: origin and extent
// of the cells the brick's owner cells can reach (one more upper cell when
// 'extra': owner cells of foreign corners on the leaf's upper faces); 'cross'
// when that reaches outside the leaf
__device__ __forceinline__ void window_axis(int g0, int B, int Lc_ax, int r, int d, int D, int extra, int& wlo,
                                            int& ext, bool& cross) {
    const int sh = D - d, span = 1 << (d - r);
    const int llo = Lc_ax * span;
    // the first corner's owner cell: the one below it, or its own on the leaf's lower face
    const int Vlo = (g0 == (llo << sh)) ? (g0 >> sh) : ((g0 - 1) >> sh), Vhi = (g0 + B - 1) >> sh;
    cross = (Vlo - 1 < llo || Vhi + 1 >= llo + span);
    wlo = Vlo - 1;
    ext = Vhi - Vlo + 3 + extra;
}

// BT[d][t][k] of the brick row starting at corner g0 (see above).  Every entry a
// corner reads lies in its function's support [(n-1)w, (n+2)w] (the corner is
// in the closure of the owner cell n - t + 1; for t = 3 at the support's left
// end), so entries outside it -- never read -- are left 0.
__device__ __forceinline__ float brick_bt(const EvalArgs& a, int r, int Lc_ax, int g0, int d, int t, int k) {
    const int n = (d <= r) ? (Lc_ax >> (r - d)) + t - 1 : ((g0 + k - 1) >> (a.D - d)) + t - 1;
    if (n < 0 || n >= (1 << d)) return 0.f;
    const int w = 1 << (a.D - d);
    const int kk = g0 + k - (n - 1) * w;
    if (kk < 0 || kk > 3 * w) return 0.f;
    return a.lb[lattice_basis_offset(a.D, d) + (i64)n * (3 * w + 1) + kk];
}

// a / n for 0 <= a < 2^14 and 1 <= n <= 2^10 through the reciprocal inv = 1/n:
// (a + 0.5)/n lies at least 0.5/n from an integer and the float product is
// within 2^-9 of it, so truncation gives the quotient
__device__ __forceinline__ int small_div(int a, float inv) { return __float2int_rz(((float)a + 0.5f) * inv); }

// the part of a window box [wlo, wlo+ext) outside the leaf's box [llo, llo+span)
// (per axis, at one depth) as at most 6 disjoint boxes
struct Box3 {
    int lo[3];
    int n[3];
};
__device__ __forceinline__ int outside_boxes(const int wlo[3], const int ext[3], const int llo[3], int span,
                                             Box3 out[6]) {
    int lo[3] = {wlo[0], wlo[1], wlo[2]}, hi[3] = {wlo[0] + ext[0], wlo[1] + ext[1], wlo[2] + ext[2]};
    int nb = 0;
    for (int ax = 0; ax < 3; ++ax) {
        const int a = max(lo[ax], llo[ax]), b = min(hi[ax], llo[ax] + span);
        if (a >= b) {   // no overlap along this axis: the rest is outside
            Box3 bx;
            for (int q = 0; q < 3; ++q) { bx.lo[q] = lo[q]; bx.n[q] = hi[q] - lo[q]; }
            out[nb++] = bx;
            return nb;
        }
        if (lo[ax] < a) {
            Box3 bx;
            for (int q = 0; q < 3; ++q) { bx.lo[q] = lo[q]; bx.n[q] = hi[q] - lo[q]; }
            bx.n[ax] = a - lo[ax];
            out[nb++] = bx;
        }
        if (b < hi[ax]) {
            Box3 bx;
            for (int q = 0; q < 3; ++q) { bx.lo[q] = lo[q]; bx.n[q] = hi[q] - lo[q]; }
            bx.lo[ax] = b;
            bx.n[ax] = hi[ax] - b;
            out[nb++] = bx;
        }
        lo[ax] = a;
        hi[ax] = b;
    }
    return nb;   // what is left lies inside the leaf
}

// one thread per (brick row, depth)
// root k's batch id on its node (depth >= 3; shallower roots are single-root batches)
__global__ void k_batch_flags(const VRoot* __restrict__ roots, int nroots, int* __restrict__ bflag) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nroots; k += gridDim.x * blockDim.x)
        if (roots[k].depth >= 3) bflag[roots[k].node] = roots[k].batch;
}

// edge of the bricks (super == 0) or of the super-bricks (super == 1: 4^3 bricks of 8^3
// cells, in leaves with lattice edge >= 64; 0 elsewhere)
__device__ __forceinline__ int row_edge(int D, int r, int super) {
    return super ? ((D - r >= 6) ? 4 * BR : 0) : brick_edge(D, r);
}

// one thread per (brick row, depth); rows numbered root by root (row_prefix), 3 x bricks-per-edge each
// (rows of a single-brick leaf whose real corners change sign are skipped: k_brick_bound leaves
// such a brick unproven without reading them)
__global__ void k_brick_rows(VArgs v, DepthLayout dl, i64 nrows, int super, const int* __restrict__ has_tri,
                             float* __restrict__ rows) {
    const EvalArgs& a = v.e;
    const int D = a.D;
    const i64* off = super ? dl.sroff : dl.roff;
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < nrows * (D + 1); e += (i64)gridDim.x * blockDim.x) {
        const i64 row = e / (D + 1);
        const int d = (int)(e % (D + 1));
        // the root from the per-depth layout: 3 * 2^lg rows per root of depth dd
        int dd = 0;
        while (dd < D - 1 && off[dd + 1] <= row) ++dd;
        const int nbk = 1 << (super ? dl.slg[dd] : dl.lg[dd]);
        const i64 loc = row - off[dd];
        const int root = dl.first[dd] + (int)(loc / (3 * nbk));
        const int rl = (int)(loc % (3 * nbk));
        const int4 rd = make_int4(root, rl / nbk, rl % nbk, 0);   // root, axis, brick index
        const VRoot R = v.roots[rd.x];
        if (!super && nbk == 1 && has_tri[R.node]) continue;
        const int ax = rd.y, r = R.depth, S = 1 << (D - r), B = row_edge(D, r, super);
        int Lc[3];
        key_coords(a.nd.key[R.node], r, D, Lc);
        const int g0 = Lc[ax] * S + rd.z * B;
        const int c0 = rd.z * B;
        float* out = rows + row * (i64)((super ? ROW_PER_DEPTH : PROW) * (D + 1));
        if (d <= r) {
            if (!super) continue;   // bricks: the leaf's ancestor polynomial (k_brick_xl)
            for (int t = 0; t < 3; ++t) {
                float mn = brick_bt(a, r, Lc[ax], g0, d, t, 0), mx = mn;
                for (int k = 1; k <= B; ++k) {
                    const float b = brick_bt(a, r, Lc[ax], g0, d, t, k);
                    mn = fminf(mn, b);
                    mx = fmaxf(mx, b);
                }
                out[ROW_RA * (D + 1) + (d * 3 + t) * 2] = mn;
                out[ROW_RA * (D + 1) + (d * 3 + t) * 2 + 1] = mx;
            }
        } else {
            int wlo, ext;
            bool cross;
            window_axis(g0, B, Lc[ax], r, d, D, 0, wlo, ext, cross);
            const int sh = D - d, lim = 1 << d;
            // the term of window cell N at corner k: its basis value where the corner's owner cell
            // (the lower-face corner owns its own cell) is within one cell of N, else 0
            auto term = [&](int N, int k) {
                const int Va = (k == 0 && c0 == 0) ? (g0 >> sh) : ((g0 + k - 1) >> sh);
                return (N < Va - 1 || N > Va + 1) ? 0.f : lattice_basis(a, d, N, g0 + k);
            };
            if (!super && (1 << sh) >= B) {
                float4* pw = reinterpret_cast<float4*>(out + d * PROW);
                for (int n = 0; n < PW; ++n) {
                    const int N = wlo + n;
                    float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (n < ext && N >= 0 && N < lim) f = bern_fit([&](int k) { return term(N, k); }, B);
                    pw[n] = f;
                }
                continue;
            }
            float* rw = super ? out + ROW_RW * (D + 1) + d * BR_WEXT * 2 : out + d * PROW;
            for (int n = 0; n < BR_WEXT; ++n) {
                const int N = wlo + n;
                float mn = 0.f, mx = 0.f;             // 0: corners without this term
                if (n < ext && N >= 0 && N < lim) {
                    for (int k = 0; k <= B; ++k) {
                        const float b = term(N, k);
                        mn = fminf(mn, b);
                        mx = fmaxf(mx, b);
                    }
                }
                rw[n * 2] = mn;
                rw[n * 2 + 1] = mx;
            }
        }
    }
}

// Per root: x of the 27 neighbours of each ancestor (0: no neighbour; xl, for the evaluation),
// and the leaf's ancestor polynomial (anc, for the bounds).  Every ancestor function is one
// quadratic piece per axis over the leaf (its knots are multiples of its cell width, and the leaf
// lies in one such cell), so the ancestors' sum is one tri-quadratic over the leaf, kept in
// Bernstein form over t = (corner - leaf origin) / S per axis:
//   C[9i + 3j + l] = sum over levels and neighbours of x * bx_i * by_j * bz_l   (bern_fit's b)
// (lane k computes coefficient k, per level as sum_jx bx_i (sum_jy by_j (sum_jz x bz_l))), then
// S3 = sum |x| Mx My Mz, the number of terms and FIT = sum |x| (dx My Mz + Mx dy Mz + Mx My dz)
// (d the fits' residuals, M = bern_m), which bounds |sum x (vx vy vz - Qx Qy Qz)| at every corner.
// Single-brick leaves whose corners change sign are never bounded: their polynomial is left 0.
constexpr int XL_WARPS = 4;
__global__ void __launch_bounds__(32 * XL_WARPS) k_brick_xl(VArgs v, int nroots, const int* __restrict__ has_tri,
                                                            float* __restrict__ xl, float* __restrict__ anc) {
    // one warp per root: lane 0 walks up the leaf's ancestors once; the warp writes the 27
    // neighbours' x of every level, fits the ancestor functions of all levels (lanes over
    // level, axis, offset), then forms the polynomial
    __shared__ int sanc[XL_WARPS][BR_LEVELS];
    __shared__ float sx[XL_WARPS][BR_LEVELS * 27];
    __shared__ float4 sfit[XL_WARPS][BR_LEVELS * 9];   // [level][axis][t]
    const NodeArrays& nd = v.e.nd;
    const int D = v.e.D;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
    for (i64 ri = warp; ri < nroots; ri += nwarps) {
        const VRoot R = v.roots[ri];
        const int r = R.depth, S = 1 << (D - r);
        __syncwarp();   // the previous root's readers are done
        if (lane == 0) {
            int node = R.node;
            for (int q = r; q >= 0; --q) {
                sanc[w][q] = node;
                if (q > 0) node = nd.parent[node];
            }
        }
        __syncwarp();
        for (int t = lane; t < BR_LEVELS * 27; t += 32) {
            const int l = t / 27, j = t % 27;
            const float x = (l <= r) ? x_or_zero(v.e, nd.neigh[(i64)j * nd.M + sanc[w][l]]) : 0.f;
            xl[ri * BR_LEVELS * 27 + t] = x;
            sx[w][t] = x;
        }
        const bool poly = !(S <= BR && has_tri[R.node]);
        int Lc[3];
        key_coords(nd.key[R.node], r, D, Lc);
        if (poly) {
            for (int f = lane; f < 9 * (r + 1); f += 32) {
                const int l = f / 9, ax = (f % 9) / 3, t = f % 3, g0 = Lc[ax] * S;
                sfit[w][f] = bern_fit([&](int k) { return brick_bt(v.e, r, Lc[ax], g0, l, t, k); }, S);
            }
        }
        __syncwarp();
        float c = 0.f, s3 = 0.f, fit = 0.f;
        int cnt = 0;
        if (poly && lane < 27) {
            const int i = lane / 9, j = (lane / 3) % 3, lz = lane % 3;
            for (int l = 0; l <= r; ++l) {
                const float* xs = sx[w] + 27 * l;
                const float4* F = sfit[w] + 9 * l;
                float acc = 0.f;
                for (int jx = 0; jx < 3; ++jx) {
                    float ys = 0.f;
                    for (int jy = 0; jy < 3; ++jy) {
                        float zs = 0.f;
                        for (int jz = 0; jz < 3; ++jz) zs = fmaf(xs[9 * jx + 3 * jy + jz], f4_at(F[6 + jz], lz), zs);
                        ys = fmaf(f4_at(F[3 + jy], j), zs, ys);
                    }
                    acc = fmaf(f4_at(F[jx], i), ys, acc);
                }
                c += acc;
                const float ax = fabsf(xs[lane]);   // the neighbour at offset (i, j, lz)
                if (ax != 0.f) {
                    const float Mx = bern_m(F[i]), My = bern_m(F[3 + j]), Mz = bern_m(F[6 + lz]);
                    s3 += ax * Mx * My * Mz;
                    fit += ax * (F[i].w * My * Mz + Mx * F[3 + j].w * Mz + Mx * My * F[6 + lz].w);
                    ++cnt;
                }
            }
        }
        for (int o = 16; o; o >>= 1) {
            s3 += __shfl_xor_sync(0xffffffffu, s3, o);
            fit += __shfl_xor_sync(0xffffffffu, fit, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        anc[ri * ANC_STRIDE + lane] =
            lane < 27 ? c : (lane == 27 ? s3 : (lane == 28 ? (float)cnt : (lane == 29 ? fit : 0.f)));
    }
}

// lower_face_owner with the batch membership of the leaf's 27 neighbours looked up once
// (member[j]: batch_member's answer for the leaf at offset j, 13 = the leaf itself)
__device__ __forceinline__ int lower_face_owner_cached(const VArgs& v, const VRoot& R, const int Lc[3], const int qc[3],
                                                       const int* member, int oc[3]) {
    const int D = v.e.D, sh = D - R.depth, lim = 1 << D;
    u64 best = ~0ull;
    int own = -1;
    for (int eo = 0; eo < 8; ++eo) {
        const int cell[3] = {qc[0] - (eo & 1), qc[1] - ((eo >> 1) & 1), qc[2] - ((eo >> 2) & 1)};
        if (cell[0] < 0 || cell[1] < 0 || cell[2] < 0 || cell[0] >= lim || cell[1] >= lim || cell[2] >= lim) continue;
        const int j = 9 * ((cell[0] >> sh) - Lc[0] + 1) + 3 * ((cell[1] >> sh) - Lc[1] + 1) + ((cell[2] >> sh) - Lc[2] + 1);
        const int m = member[j];
        if (m < 0) continue;
        const u64 kk = cell_key_D(cell, D);
        if (kk < best) { best = kk; own = m; oc[0] = cell[0]; oc[1] = cell[1]; oc[2] = cell[2]; }
    }
    return own;
}

// owner of a lower-face corner (min key among batch cells sharing it)
__device__ __forceinline__ int lower_face_owner(const VArgs& v, const VRoot& R, const int Lc[3], const int qc[3],
                                                int oc[3]) {
    u64 best = ~0ull;
    int own = -1;
    for (int eo = 0; eo < 8; ++eo) {
        const int cell[3] = {qc[0] - (eo & 1), qc[1] - ((eo >> 1) & 1), qc[2] - ((eo >> 2) & 1)};
        const int m = batch_member(v, R, Lc, cell);
        if (m < 0) continue;
        const u64 kk = cell_key_D(cell, v.e.D);
        if (kk < best) { best = kk; own = m; oc[0] = cell[0]; oc[1] = cell[1]; oc[2] = cell[2]; }
    }
    return own;
}

// sign of a bound [lo, hi] of a brick's corner values against iso: 1 (all above), -1 (all
// below), 0 (not proven).  The margin m = (2 cnt + 2 BR_WEXT + 8) u A + 4u (|lo| + |hi| + 2|iso|),
// A = 1.01 amax, covers the evaluation's FMA chain and this bound's own float arithmetic.  It is
// evaluated in float: every operation of it rounds by at most u relative and every term is
// non-negative, so scaling by 1 + 2^-16 bounds the exact value from above; the tests are made as
// lo - iso > m and iso - hi > m, whose float differences are within u of exact, which the extra
// 2u (|lo| + |hi| + 2|iso|) covers.  (A non-finite bound compares false: not proven.)
__device__ __forceinline__ signed char bound_sign(float lo, float hi, float amax, int cnt, float iso) {
    const float u = 5.9604644775390625e-08f;   // 2^-24
    const float A = amax * 1.01f;
    const float m = ((2.0f * (float)cnt + (2.0f * BR_WEXT + 8.0f)) * u * A +
                     6.0f * u * (fabsf(lo) + fabsf(hi) + 2.0f * fabsf(iso)) + 1e-30f) * (1.0f + 1.52587890625e-05f);
    if (lo - iso > m) return 1;
    if (iso - hi > m) return -1;
    return 0;
}

// Shell terms of a bound at virtual depth d: the window cells outside the leaf that hold a
// real node, each term x * X * Y * Z over the row tables' ranges RW.
//  * Nodes: a cell's node is found by descending from the leaf's neighbour at depth r, through
//    two levels of "anchors" the warp finds first: the cells of depth d - 4 covering the window
//    (at most 2 per axis, one lane each; when d - r > 4) and of depth d - 2 (at most 4 per axis,
//    two per lane, each descending 2 levels from its depth d - 4 anchor; when d - r > 2).  A
//    cell then descends 2 levels from its anchor; cells under an absent anchor are skipped,
//    and a window without any anchor is skipped whole.  The path through the anchors is the
//    same path, so the node is the same.
//  * The lanes run over the cells of all boxes in turn (a lane's next cell continues into the
//    next box), so boxes smaller than a warp leave fewer lanes idle.
//  * rw[ax]: the depth's RW ranges of the window cells along each axis.
//  * An RW range always contains 0 (lo <= 0 <= hi), and float rounding is monotone, so
//    [a, b] x [lo, hi] = [min(b lo, a hi), max(a lo, b hi)]: exactly the min and max of the four
//    rounded products, in 4 multiplies and 2 min/max instead of 4 and 6.
// The window's extent is at most 12 < 16 cells per axis: at most 2 anchors of depth d - 4 and
// 4 of depth d - 2 per axis.
constexpr int SHELL_ANCHORS = 8 + 64;   // ints of shared memory per warp
__device__ __forceinline__ void shell_terms(const VArgs& v, int L, int r, const int Lc[3], int d, int D,
                                            const int wlo[3], const int ext[3], const float2* const rw[3],
                                            int lane, int* __restrict__ anchor, float& lo, float& hi, float& amax,
                                            int& cnt) {
    const float* __restrict__ xv = v.e.x;
    const NodeArrays& nd = v.e.nd;
    const bool anch = d - r > 2;
    int blo[3] = {0, 0, 0};
    if (anch) {
        int* a4 = anchor;        // depth d - 4
        int* a2 = anchor + 8;    // depth d - 2, 4 x 4 x 4
        // only anchors that cover window cells are looked up: those lie in the leaf's
        // neighbours (the window reaches at most 2 cells beyond the leaf)
        int alo[3], ahi[3], bhi[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            alo[ax] = wlo[ax] >> 4;   // floor, also below 0
            blo[ax] = wlo[ax] >> 2;
            ahi[ax] = (wlo[ax] + ext[ax] - 1) >> 4;
            bhi[ax] = (wlo[ax] + ext[ax] - 1) >> 2;
        }
        __syncwarp();                 // the previous depth's readers are done
        if (d - r > 4) {
            int an = -1;
            if (lane < 8) {
                const int A[3] = {alo[0] + ((lane >> 2) & 1), alo[1] + ((lane >> 1) & 1), alo[2] + (lane & 1)};
                if (A[0] <= ahi[0] && A[1] <= ahi[1] && A[2] <= ahi[2]) an = (int)shell_node(v, L, r, Lc, d - 4, A);
            }
            if (__ballot_sync(0xffffffffu, an >= 0) == 0) return;   // no real node near this window
            if (lane < 8) a4[lane] = an;
            __syncwarp();
        }
        int any = 0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int q = lane + 32 * h;
            const int B[3] = {blo[0] + (q >> 4), blo[1] + ((q >> 2) & 3), blo[2] + (q & 3)};
            int bn = -1;
            if (B[0] > bhi[0] || B[1] > bhi[1] || B[2] > bhi[2]) {
                // covers no window cell
            } else if (d - r > 4) {
                const int an = a4[(((B[0] >> 2) - alo[0]) << 2) | (((B[1] >> 2) - alo[1]) << 1) | ((B[2] >> 2) - alo[2])];
                bn = an < 0 ? -1 : (int)descend(nd, an, d - 4, d - 2, B);
            } else {
                bn = (int)shell_node(v, L, r, Lc, d - 2, B);
            }
            a2[q] = bn;
            any |= bn >= 0;
        }
        if (__ballot_sync(0xffffffffu, any) == 0) return;
        __syncwarp();
    }
    const int span = 1 << (d - r);
    const int llo[3] = {Lc[0] * span, Lc[1] * span, Lc[2] * span};
    Box3 bxs[6];
    const int nbx = outside_boxes(wlo, ext, llo, span, bxs);
    const int* a2 = anchor + 8;
    int g = lane, first = 0;
    for (int q = 0; q < nbx; ++q) {
        const Box3 bx = bxs[q];
        const int n12 = bx.n[1] * bx.n[2], ncell = bx.n[0] * n12;
        const float inv12 = 1.0f / (float)n12, inv2 = 1.0f / (float)bx.n[2];
        for (; g < first + ncell; g += 32) {
            const int t = g - first;
            const int i0 = small_div(t, inv12), rem = t - i0 * n12, i1 = small_div(rem, inv2),
                      i2 = rem - i1 * bx.n[2];
            const int N[3] = {bx.lo[0] + i0, bx.lo[1] + i1, bx.lo[2] + i2};
            i64 node;
            if (anch) {
                const int bn = a2[(((N[0] >> 2) - blo[0]) << 4) | (((N[1] >> 2) - blo[1]) << 2) | ((N[2] >> 2) - blo[2])];
                if (bn < 0) continue;
                node = descend(nd, bn, d - 2, d, N);
            } else {
                node = shell_node(v, L, r, Lc, d, N);
            }
            if (node < 0) continue;
            const float x = xv[node];
            const float2 X = rw[0][N[0] - wlo[0]], Y = rw[1][N[1] - wlo[1]], Z = rw[2][N[2] - wlo[2]];
            const float p0 = x * X.x, p1 = x * X.y;
            float a = fminf(p0, p1), b = fmaxf(p0, p1);
            const float a1 = fminf(b * Y.x, a * Y.y), b1 = fmaxf(a * Y.x, b * Y.y);
            a = fminf(b1 * Z.x, a1 * Z.y);
            b = fmaxf(a1 * Z.x, b1 * Z.y);
            lo += a;
            hi += b;
            amax += fmaxf(fabsf(a), fabsf(b));
            ++cnt;
        }
        first += ncell;
    }
}

// one warp per super-brick (4^3 bricks of leaves with lattice edge >= 64): the
// same bound over all its corners; decided only when every window it needs fits
// the row tables (away from the leaf's boundary).  ssign = 1, -1 or 0.
__global__ void __launch_bounds__(256) k_super_bound(VArgs v, DepthLayout dl,
                                                     const i64* __restrict__ srow_prefix,
                                                     const float* __restrict__ srows, const float* __restrict__ xl_all,
                                                     i64 nsuper, signed char* __restrict__ ssign) {
    __shared__ int s_anchor[256 / 32][SHELL_ANCHORS];
    const EvalArgs& a = v.e;
    const int D = a.D;
    const int lane = threadIdx.x & 31;
    const i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
    for (i64 si = warp; si < nsuper; si += nwarps) {
        int dd = 0;
        while (dd < D - 1 && dl.soff[dd + 1] <= si) ++dd;
        const i64 loc = si - dl.soff[dd];
        const int slg = dl.slg[dd];
        const int lo = dl.first[dd] + (int)(loc >> (3 * slg));
        const VRoot R = v.roots[lo];
        const int r = R.depth, S = 1 << (D - r), E = 4 * BR, ns = S / E, L = R.node;
        const i64 l = loc & ((1ll << (3 * slg)) - 1);
        const int sb[3] = {(int)(l >> (2 * slg)), (int)(l >> slg) & (ns - 1), (int)l & (ns - 1)};
        int Lc[3];
        key_coords(a.nd.key[L], r, D, Lc);
        const int g0[3] = {Lc[0] * S + sb[0] * E, Lc[1] * S + sb[1] * E, Lc[2] * S + sb[2] * E};
        const float* row[3];
        for (int ax = 0; ax < 3; ++ax)
            row[ax] = srows + (srow_prefix[lo] + (i64)ax * ns + sb[ax]) * (i64)(ROW_PER_DEPTH * (D + 1));
        const float* xl = xl_all + (i64)lo * BR_LEVELS * 27;
        float flo = 0.f, fhi = 0.f, amax = 0.f;
        int cnt = 0;
        bool decided = true;
        ancestor_bound(xl, row, r, D, lane, flo, fhi, amax, cnt);
        for (int d = r + 1; d <= D && decided; ++d) {
            int wlo[3], ext[3];
            bool cross = false;
            for (int ax = 0; ax < 3; ++ax) {
                bool c;
                window_axis(g0[ax], E, Lc[ax], r, d, D, 0, wlo[ax], ext[ax], c);
                cross |= c;
            }
            // the windows of successive depths are nested (in finest cells), so once a window
            // lies inside the leaf so do all finer ones
            if (!cross) break;
            if (ext[0] > BR_WEXT || ext[1] > BR_WEXT || ext[2] > BR_WEXT) { decided = false; break; }
            const float2* rw[3];
            for (int ax = 0; ax < 3; ++ax) rw[ax] = reinterpret_cast<const float2*>(row[ax] + ROW_RW * (D + 1)) + d * BR_WEXT;
            shell_terms(v, L, r, Lc, d, D, wlo, ext, rw, lane, s_anchor[threadIdx.x >> 5], flo, fhi, amax, cnt);
        }
        for (int o = 16; o; o >>= 1) {
            flo += __shfl_xor_sync(0xffffffffu, flo, o);
            fhi += __shfl_xor_sync(0xffffffffu, fhi, o);
            amax += __shfl_xor_sync(0xffffffffu, amax, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0) ssign[si] = decided ? bound_sign(flo, fhi, amax, cnt, v.iso) : 0;
    }
}

// Shell terms at a depth d of knot spacing >= the brick edge (d <= D - lg E): each window cell
// outside the leaf with a real node contributes x Qx Qy Qz, Q the cell's PW entries (Bernstein
// form over the brick), to the brick's coarse polynomial.  The window spans at most PW = 4 cells
// per axis there (the brick lies in one cell of depth d, and its first corner's owner may lie in
// the cell below), so the terms form a 4^3 grid X of x (0: no node, or inside the leaf; two cells
// per lane), contracted one axis at a time through shared memory:
//   T1[n0 n1 l] = sum_n2 X Qz_l(n2),  T2[n0 j l] = sum_n1 T1 Qy_j(n1),  C_ijl += sum_n0 T2 Qx_i(n0)
// (lane k < 27 holds coefficient k = 9i + 3j + l).  s3 gains |x| Mx My Mz, fit
// |x| (dx My Mz + Mx dy Mz + Mx My dz) (as k_brick_xl's), cnt the number of terms.
constexpr int SHELL_POLY_BUF = 64 + 48 + 36;   // floats of shared memory per warp
__device__ __forceinline__ void shell_poly(const VArgs& v, int L, int r, const int Lc[3], int d, const int wlo[3],
                                           const int ext[3], const float4* const pw[3], int lane,
                                           float* __restrict__ buf, float& coef, float& s3, float& fit, int& cnt) {
    float* X = buf;
    float* T1 = buf + 64;
    float* T2 = buf + 112;
    bool any = false;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int g = lane + 32 * h, n0 = g >> 4, n1 = (g >> 2) & 3, n2 = g & 3;
        float x = 0.f;
        if (n0 < ext[0] && n1 < ext[1] && n2 < ext[2]) {
            const int N[3] = {wlo[0] + n0, wlo[1] + n1, wlo[2] + n2};
            const i64 node = shell_node(v, L, r, Lc, d, N);
            if (node >= 0) x = v.e.x[node];
        }
        X[g] = x;
        if (x != 0.f) {
            const float4 QX = pw[0][n0], QY = pw[1][n1], QZ = pw[2][n2];
            const float Mx = bern_m(QX), My = bern_m(QY), Mz = bern_m(QZ), ax = fabsf(x);
            s3 += ax * Mx * My * Mz;
            fit += ax * (QX.w * My * Mz + Mx * QY.w * Mz + Mx * My * QZ.w);
            ++cnt;
            any = true;
        }
    }
    if (!__any_sync(0xffffffffu, any)) return;   // no real node near the brick at this depth
    __syncwarp();
    for (int e = lane; e < 48; e += 32) {
        const int nn = e / 3, l = e - 3 * nn;   // nn = 4 n0 + n1
        float t = 0.f;
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) t = fmaf(X[4 * nn + n2], f4_at(pw[2][n2], l), t);
        T1[e] = t;
    }
    __syncwarp();
    for (int e = lane; e < 36; e += 32) {
        const int n0 = e / 9, j = (e / 3) % 3, l = e % 3;
        float t = 0.f;
#pragma unroll
        for (int n1 = 0; n1 < 4; ++n1) t = fmaf(T1[(4 * n0 + n1) * 3 + l], f4_at(pw[1][n1], j), t);
        T2[e] = t;
    }
    __syncwarp();
    if (lane < 27) {
        const int i = lane / 9, jl = lane % 9;
        float t = 0.f;
#pragma unroll
        for (int n0 = 0; n0 < 4; ++n0) t = fmaf(T2[9 * n0 + jl], f4_at(pw[0][n0], i), t);
        coef += t;
    }
    __syncwarp();   // the buffer is reused by the next depth
}

// sign of a bound lo = min C + flo, hi = max C + fhi against iso: C the Bernstein coefficients over
// the brick of its coarse polynomial P (the leaf's ancestors and the shell terms of knot spacing
// >= E; P lies within their range over the brick's box), [flo, fhi] the interval sum of the finer
// shell terms.  The margin is bound_sign's over A = amax + s3 (the evaluation's FMA chain over all
// the terms, and the interval part's own arithmetic), plus fit (the fits' residuals: the corner
// values' coarse terms lie within fit of P), plus (cnt + 96) u s3 for P's coefficients,
// s3 = sum |x| Mx My Mz over its terms: (cnt + 56)u for forming them (at most 9 roundings per
// level and 16 levels for the ancestors, 12 per shell depth and one per further depth), 40u for the
// restriction to the brick (3 rounded factors and 27 FMAs per coefficient; the blossom rows are
// non-negative and sum to 1) and adding the two parts.
__device__ __forceinline__ signed char bound_sign_poly(float lo, float hi, float amax, float s3, float fit, int cnt,
                                                       float iso) {
    const float u = 5.9604644775390625e-08f;   // 2^-24
    const float A = (amax + s3) * 1.01f;
    const float m = ((2.0f * (float)cnt + (2.0f * BR_WEXT + 8.0f)) * u * A + ((float)cnt + 96.0f) * u * s3 * 1.01f +
                     fit * 1.01f + 6.0f * u * (fabsf(lo) + fabsf(hi) + 2.0f * fabsf(iso)) + 1e-30f) *
                    (1.0f + 1.52587890625e-05f);
    if (lo - iso > m) return 1;
    if (iso - hi > m) return -1;
    return 0;
}

// row q of the blossom matrix that takes quadratic Bernstein coefficients over [0, S] to those over
// [A, B] (0 <= A < B <= S, S a power of two <= 2^15): the blossom of the basis at (A, A), (A, B),
// (B, B), divided by S^2 (exact in float for S <= 2^11, else rounded once); non-negative, sums to 1
__device__ __forceinline__ void blossom_row(int A, int B, int S, int q, float out[3]) {
    const i64 a = A, b = B, s = S;
    i64 n0, n1, n2;
    if (q == 0) { n0 = (s - a) * (s - a); n1 = 2 * a * (s - a); n2 = a * a; }
    else if (q == 1) { n0 = (s - a) * (s - b); n1 = a * (s - b) + b * (s - a); n2 = a * b; }
    else { n0 = (s - b) * (s - b); n1 = 2 * b * (s - b); n2 = b * b; }
    const float inv = 1.0f / ((float)S * (float)S);
    out[0] = (float)n0 * inv;
    out[1] = (float)n1 * inv;
    out[2] = (float)n2 * inv;
}

// one warp per brick: the bound over the corners the brick's leaf owns;
// sign[bi] = 1 (all above iso), -1 (all below) or 0 (not proven).
//  * The coarse part, exact up to rounding and the tabulated values' noise: the leaf's ancestor
//    polynomial (per root, k_brick_xl) and the shell terms of depths d <= D - lg E (shell_poly),
//    bounded over the brick by the range of its Bernstein coefficients there.
//  * The finer shell terms (depths d > D - lg E, one to three cells of the finest lattice wide
//    around the leaf's faces) by intervals, as shell_terms sums them.
constexpr int BB_BLOCK = 256;
// A single-brick leaf whose own real corners change sign ('has_tri') is left unproven at once:
// its brick's corners include the leaf's corners, so its bound straddles iso (and a brick left
// unproven is only evaluated exactly, which changes no value).
// (4 blocks per SM: 64 registers, no spills; unbounded it takes 104 and halves the resident warps)
__global__ void __launch_bounds__(BB_BLOCK, 4) k_brick_bound(VArgs v, BrickIndex bix, i64 first, i64 nbricks,
                                                          const i64* __restrict__ sprefix,
                                                          const signed char* __restrict__ ssign,
                                                          const int* __restrict__ has_tri,
                                                          signed char* __restrict__ sign) {
    __shared__ int s_anchor[BB_BLOCK / 32][SHELL_ANCHORS];
    __shared__ float s_stage[BB_BLOCK / 32][SHELL_POLY_BUF];
    __shared__ float s_coef[BB_BLOCK / 32][27];   // the leaf's ancestor polynomial
    const EvalArgs& a = v.e;
    const int D = a.D;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
    for (i64 bi = first + warp; bi < nbricks; bi += nwarps) {
        const VBrick B = brick_of(v, bix, bi);
        const VRoot R = v.roots[B.root];
        if (ssign && v.e.D - R.depth >= 6) {   // decided by its super-brick?
            const int ns = (1 << (v.e.D - R.depth)) / (4 * BR);
            const signed char sg = ssign[sprefix[B.root] + ((i64)(B.b[0] >> 2) * ns + (B.b[1] >> 2)) * ns + (B.b[2] >> 2)];
            if (sg != 0) {
                if (lane == 0) sign[bi] = sg;
                continue;
            }
        }
        const int r = R.depth, S = 1 << (D - r), L = R.node, E = brick_edge(D, r), nb = S / E;
        if (nb == 1 && has_tri[L]) {
            if (lane == 0) sign[bi] = 0;
            continue;
        }
        int Lc[3];
        key_coords(a.nd.key[L], r, D, Lc);
        const int g0[3] = {Lc[0] * S + B.b[0] * E, Lc[1] * S + B.b[1] * E, Lc[2] * S + B.b[2] * E};
        const float* row[3];
        for (int ax = 0; ax < 3; ++ax) row[ax] = brick_row(bix, D, B.root, nb, ax, B.b[ax]);
        const int dpoly = D - (31 - __clz(E));   // depths of knot spacing >= E
        float lo = 0.f, hi = 0.f, amax = 0.f, s3 = 0.f, fit = 0.f, coef = 0.f;
        int cnt = 0;
        bool ok = true, inside = false;
        int d = r + 1;
        // real nodes around the leaf, at the virtual depths: coarse ones into the polynomial
        for (; d <= dpoly; ++d) {
            int wlo[3], ext[3];
            bool cross = false;
            for (int ax = 0; ax < 3; ++ax) {
                bool c;
                window_axis(g0[ax], E, Lc[ax], r, d, D, 0, wlo[ax], ext[ax], c);
                cross |= c;
            }
            if (!cross) { inside = true; break; }   // nested windows: the finer ones lie inside the leaf too
            if (ext[0] > PW || ext[1] > PW || ext[2] > PW) { ok = false; break; }   // (cannot happen)
            const float4* pw[3];
            for (int ax = 0; ax < 3; ++ax) pw[ax] = reinterpret_cast<const float4*>(row[ax] + d * PROW);
            shell_poly(v, L, r, Lc, d, wlo, ext, pw, lane, s_stage[w], coef, s3, fit, cnt);
        }
        // the finer ones by intervals; only window cells outside the leaf can hold a real node
        if (ok && !inside) {
            for (; d <= D; ++d) {
                int wlo[3], ext[3];
                bool cross = false;
                for (int ax = 0; ax < 3; ++ax) {
                    bool c;
                    window_axis(g0[ax], E, Lc[ax], r, d, D, 0, wlo[ax], ext[ax], c);
                    cross |= c;
                }
                if (!cross) break;
                const float2* rw[3];
                for (int ax = 0; ax < 3; ++ax) rw[ax] = reinterpret_cast<const float2*>(row[ax] + d * PROW);
                shell_terms(v, L, r, Lc, d, D, wlo, ext, rw, lane, s_anchor[w], lo, hi, amax, cnt);
            }
        }
        // the coarse polynomial's Bernstein coefficients over the brick: the leaf's ancestor
        // polynomial restricted to it (lane k < 27: coefficient k = 9i + 3j + l, through the
        // blossom rows i, j, l of the three axes; the identity for a single-brick leaf) plus the
        // shell part
        const float* an = bix.anc + (i64)B.root * ANC_STRIDE;
        __syncwarp();   // the previous brick's readers are done
        if (lane < 27) s_coef[w][lane] = an[lane];
        __syncwarp();
        float cmin = INFINITY, cmax = -INFINITY;
        if (lane < 27) {
            float c = s_coef[w][lane];
            if (nb > 1) {
                float tx[3], ty[3], tz[3];
                blossom_row(B.b[0] * E, (B.b[0] + 1) * E, S, lane / 9, tx);
                blossom_row(B.b[1] * E, (B.b[1] + 1) * E, S, (lane / 3) % 3, ty);
                blossom_row(B.b[2] * E, (B.b[2] + 1) * E, S, lane % 3, tz);
                c = 0.f;
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        const float tij = tx[i] * ty[j];
#pragma unroll
                        for (int l = 0; l < 3; ++l) c = fmaf(s_coef[w][9 * i + 3 * j + l], tij * tz[l], c);
                    }
            }
            c += coef;
            cmin = cmax = c;
        }
        for (int o = 16; o; o >>= 1) {
            lo += __shfl_xor_sync(0xffffffffu, lo, o);
            hi += __shfl_xor_sync(0xffffffffu, hi, o);
            amax += __shfl_xor_sync(0xffffffffu, amax, o);
            s3 += __shfl_xor_sync(0xffffffffu, s3, o);
            fit += __shfl_xor_sync(0xffffffffu, fit, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
            cmin = fminf(cmin, __shfl_xor_sync(0xffffffffu, cmin, o));
            cmax = fmaxf(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
        }
        if (lane == 0)
            sign[bi] = ok ? bound_sign_poly(cmin + lo, cmax + hi, amax, s3 + an[27], fit + an[29], cnt + (int)an[28], v.iso)
                          : (signed char)0;
    }
}

// culled: the brick's own bound is proven and, where some of its corners may be
// owned by another leaf L' of the batch, every brick of L' that can hold such
// an owner cell is proven with the same sign
__global__ void k_brick_cull(VArgs v, BrickIndex bix, const int* __restrict__ root_of, const signed char* __restrict__ sign,
                             i64 nbricks, unsigned char* __restrict__ culled) {
    const int D = v.e.D;
    const NodeArrays& nd = v.e.nd;
    for (i64 bi = (i64)blockIdx.x * blockDim.x + threadIdx.x; bi < nbricks; bi += (i64)gridDim.x * blockDim.x) {
        const int sg = sign[bi];
        if (sg == 0) { culled[bi] = 0; continue; }
        const VBrick B = brick_of(v, bix, bi);
        const VRoot R = v.roots[B.root];
        const int E = brick_edge(D, R.depth), nb = (1 << (D - R.depth)) / E;
        bool ok = true;
        if (R.depth >= 3 && !(B.b[0] && B.b[1] && B.b[2])) {
            for (int j = 0; j < 27 && ok; ++j) {
                const int off[3] = {j / 9 - 1, (j / 3) % 3 - 1, j % 3 - 1};
                bool lower = false, allowed = true;
                for (int ax = 0; ax < 3; ++ax) {
                    if (off[ax] == -1) { lower = true; if (B.b[ax] != 0) allowed = false; }
                    if (off[ax] == 1 && B.b[ax] != nb - 1) allowed = false;
                }
                if (!lower || !allowed) continue;
                const int n = nd.neigh[(i64)j * nd.M + R.node];
                if (n == -1 || v.batch_root_flag[n] != R.batch) continue;
                const int k2 = root_of[n];
                // bricks of the neighbour holding owner cells within one cell of this brick
                int lo3[3], hi3[3];
                for (int ax = 0; ax < 3; ++ax) {
                    if (off[ax] == -1) { lo3[ax] = hi3[ax] = nb - 1; }
                    else if (off[ax] == 1) { lo3[ax] = hi3[ax] = 0; }
                    else { lo3[ax] = max(B.b[ax] - 1, 0); hi3[ax] = min(B.b[ax] + 1, nb - 1); }
                }
                for (int x = lo3[0]; x <= hi3[0] && ok; ++x)
                    for (int y = lo3[1]; y <= hi3[1] && ok; ++y)
                        for (int z = lo3[2]; z <= hi3[2] && ok; ++z)
                            if (sign[bix.prefix[k2] + ((i64)x * nb + y) * nb + z] != sg) ok = false;
            }
        }
        culled[bi] = ok ? 1 : 0;
    }
}

// root index of each subdivided leaf's node (-1 elsewhere)
__global__ void k_root_of(const VRoot* __restrict__ roots, int nroots, int* __restrict__ root_of) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nroots; k += gridDim.x * blockDim.x)
        root_of[roots[k].node] = k;
}

// shared memory of one brick of edge at most EB: bricks of edge 8 (leaves with
// lattice edge >= 8) and of edge 2 or 4 (the smallest leaves) are evaluated by
// two instances.  Window bound for EB = 4 with the extra upper cell: 8^3 + 6^3.
template <int EB>
struct BrickShared {
    static constexpr int K1 = EB + 1;         // corners per axis
    // edge 2 (leaves one depth above the finest): one virtual depth, at most 5^3 window cells
    static constexpr int XW = (EB == BR) ? BR_XW : (EB == 4 ? 728 : 128);
    float4 Bt[3 * BR_LEVELS * K1];            // [axis][depth][k], the four t of a corner in one vector
    float4 xL[BR_LEVELS * 7];                 // neighbours of the leaf and its ancestors (0: none), 27 + 1 per level
    float Xw[XW];                             // window coefficients, virtual depths (0: none or inside the leaf)
    int wlo[BR_LEVELS][3];                    // window origin (cell coordinates at that depth)
    int wext[BR_LEVELS][3];
    int woff[BR_LEVELS];                      // offset into Xw, -1 when no corner reaches outside the leaf
    int member[27];                           // batch_member of the leaf at each neighbour offset
};
template <int EB>
__device__ __forceinline__ float4 bt_at(const BrickShared<EB>& sm, int ax, int d, int k) {
    return sm.Bt[(ax * BR_LEVELS + d) * BrickShared<EB>::K1 + k];
}

// virtual-depth part of the value of corner qc (brick-local kk) whose owner
// cell is oc -- in the brick's leaf or, for a foreign corner, in the leaf of
// the batch that owns it -- from the shared window, in the order of
// virtual_corner_value.  At depth d the owner cell is oc >> sh, the tabulated
// one (qc - 1) >> sh, so the basis row is taken t + ((oc >> sh) - ((qc-1) >> sh))
// (0 or 1).  Terms that virtual_corner_value skips (levels whose 3x3x3 block
// lies inside the owner's leaf, cells inside either leaf, absent nodes) read 0
// here, and adding a zero product leaves the sum unchanged, so the value is the
// same.
template <int EB>
__device__ __forceinline__ float brick_virtual(const BrickShared<EB>& sm, int D, int r, const int Lc[3], const int oc[3],
                                               const int qc[3], const int kk[3]) {
    float val = 0.f;
    for (int d = D; d > r; --d) {
        const int off = sm.woff[d];
        if (off < 0) continue;
        const int sh = D - d;
        const int V[3] = {oc[0] >> sh, oc[1] >> sh, oc[2] >> sh};
        // a 3x3x3 block inside the leaf reads only zeros: its terms leave the sum unchanged
        const int span = 1 << (d - r);
        bool inside = true;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int lo = Lc[ax] << (d - r);
            inside &= (V[ax] - 1 >= lo) && (V[ax] + 1 < lo + span);
        }
        if (inside) continue;
        float bv[3][3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const bool toff = V[ax] != ((qc[ax] - 1) >> sh);   // the owner cell is the tabulated one or the next
            const float4 b = bt_at(sm, ax, d, kk[ax]);
            bv[ax][0] = toff ? b.y : b.x;
            bv[ax][1] = toff ? b.z : b.y;
            bv[ax][2] = toff ? b.w : b.z;
        }
        const int e1 = sm.wext[d][1], e2 = sm.wext[d][2];
        const float* xw = sm.Xw + off + ((V[0] - 1 - sm.wlo[d][0]) * e1 + (V[1] - 1 - sm.wlo[d][1])) * e2 +
                          (V[2] - 1 - sm.wlo[d][2]);
#pragma unroll
        for (int j = 0; j < 27; ++j) {
            const int jx = j / 9, jy = (j / 3) % 3, jz = j % 3;
            val = fmaf(xw[(jx * e1 + jy) * e2 + jz] * bv[0][jx] * bv[1][jy], bv[2][jz], val);
        }
    }
    return val;
}

// the brick's leaf itself and its real ancestors (walk_up with absent neighbours as 0)
template <int EB>
__device__ __forceinline__ float brick_leaf_levels(const BrickShared<EB>& sm, int r, const int kk[3], float val) {
    for (int l = r; l >= 0; --l) {
        float xs[28];
#pragma unroll
        for (int q = 0; q < 7; ++q) {
            const float4 v4 = sm.xL[7 * l + q];
            xs[4 * q] = v4.x; xs[4 * q + 1] = v4.y; xs[4 * q + 2] = v4.z; xs[4 * q + 3] = v4.w;
        }
        float bv[3][3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const float4 b = bt_at(sm, ax, l, kk[ax]);
            bv[ax][0] = b.x; bv[ax][1] = b.y; bv[ax][2] = b.z;
        }
#pragma unroll
        for (int j = 0; j < 27; ++j) val = fmaf(xs[j] * bv[0][j / 9] * bv[1][(j / 3) % 3], bv[2][j % 3], val);
    }
    return val;
}

// live brick: root, brick coordinates; first corner value and first cell
struct LiveBrick {
    int root;
    int b[3];
    i64 lat;
    i64 cell;
};

// one block per live brick: exact corner values into the brick's (B+1)^3 slot
template <int EB, int NT>
__global__ void __launch_bounds__(NT) k_brick_eval(VArgs v, BrickIndex bix, const int* __restrict__ root_of,
                                                   const LiveBrick* __restrict__ live, const int* __restrict__ list,
                                                   i64 nlist, float* __restrict__ blat,
                                                   unsigned long long* __restrict__ nforeign,
                                                   int2* __restrict__ foreign, i64 foreign_cap) {
    __shared__ BrickShared<EB> sm;
    constexpr int K1 = BrickShared<EB>::K1;
    const EvalArgs& a = v.e;
    const int D = a.D;
    for (i64 it = blockIdx.x; it < nlist; it += gridDim.x) {
        const i64 li = list[it];
        const LiveBrick lb = live[li];
        const VRoot R = v.roots[lb.root];
        const int r = R.depth, S = 1 << (D - r), L = R.node, E = brick_edge(D, r), nb = S / E, E1 = E + 1;
        int Lc[3];
        key_coords(a.nd.key[L], r, D, Lc);
        const int g0[3] = {Lc[0] * S + lb.b[0] * E, Lc[1] * S + lb.b[1] * E, Lc[2] * S + lb.b[2] * E};
        const bool fposs = brick_foreign_possible(v, R, lb.b, nb);
        __syncthreads();
        // window layout (every thread sizes it; thread 0 records it), leaf tables, zeroed window
        int total = 0;
        for (int d = r + 1; d <= D; ++d) {
            int wl[3], we[3];
            bool cross = false;
            for (int ax = 0; ax < 3; ++ax) {
                bool c;
                window_axis(g0[ax], E, Lc[ax], r, d, D, 0, wl[ax], we[ax], c);
                cross |= c;
            }
            if (threadIdx.x == 0) {
                for (int ax = 0; ax < 3; ++ax) { sm.wlo[d][ax] = wl[ax]; sm.wext[d][ax] = we[ax]; }
                sm.woff[d] = cross ? total : -1;
            }
            if (cross) total += we[0] * we[1] * we[2];
        }
        if (total > BrickShared<EB>::XW) {   // cannot happen for aligned bricks: reported, brick skipped
            if (threadIdx.x == 0) atomicAdd(nforeign + 1, 1ull);
            continue;
        }
        float* xl_s = reinterpret_cast<float*>(sm.xL);
        for (int e = threadIdx.x; e < 28 * (r + 1); e += blockDim.x) {
            const int l = e / 28, j = e % 28;
            xl_s[e] = (j < 27) ? bix.xl[(i64)lb.root * BR_LEVELS * 27 + 27 * l + j] : 0.f;
        }
        float* bt_s = reinterpret_cast<float*>(sm.Bt);
        for (int e = threadIdx.x; e < 3 * 4 * K1 * (D + 1); e += blockDim.x) {
            const int ax = e / (4 * K1 * (D + 1)), q = e % (4 * K1 * (D + 1));
            const int d = q / (4 * K1), k = (q % (4 * K1)) / 4, t = q % 4;
            bt_s[ax * BR_LEVELS * 4 * K1 + q] = (k <= E) ? brick_bt(a, r, Lc[ax], g0[ax], d, t, k) : 0.f;
        }
        for (int t = threadIdx.x; t < total; t += blockDim.x) sm.Xw[t] = 0.f;
        if (fposs && threadIdx.x < 27) {
            const int j = threadIdx.x;
            const int cell[3] = {(Lc[0] + j / 9 - 1) << (D - r), (Lc[1] + (j / 3) % 3 - 1) << (D - r),
                                 (Lc[2] + j % 3 - 1) << (D - r)};
            sm.member[j] = batch_member(v, R, Lc, cell);
        }
        __syncthreads();
        // only window cells outside the leaf can hold a real node
        for (int d = r + 1; d <= D; ++d) {
            const int off = sm.woff[d];
            if (off < 0) continue;
            const int span = 1 << (d - r);
            const int llo[3] = {Lc[0] * span, Lc[1] * span, Lc[2] * span};
            const int wlo[3] = {sm.wlo[d][0], sm.wlo[d][1], sm.wlo[d][2]};
            const int ext[3] = {sm.wext[d][0], sm.wext[d][1], sm.wext[d][2]};
            Box3 bxs[6];
            const int nbx = outside_boxes(wlo, ext, llo, span, bxs);
            for (int q = 0; q < nbx; ++q) {
                const Box3& bx = bxs[q];
                const int n12 = bx.n[1] * bx.n[2], ncell = bx.n[0] * n12;
                const float inv12 = 1.0f / (float)n12, inv2 = 1.0f / (float)bx.n[2];
                for (int t = threadIdx.x; t < ncell; t += blockDim.x) {
                    const int i0 = small_div(t, inv12), rem = t - i0 * n12, i1 = small_div(rem, inv2),
                              i2 = rem - i1 * bx.n[2];
                    const int N[3] = {bx.lo[0] + i0, bx.lo[1] + i1, bx.lo[2] + i2};
                    const i64 node = shell_node(v, L, r, Lc, d, N);
                    if (node >= 0)
                        sm.Xw[off + ((N[0] - wlo[0]) * ext[1] + (N[1] - wlo[1])) * ext[2] + (N[2] - wlo[2])] = a.x[node];
                }
            }
        }
        __syncthreads();
        float* out = blat + lb.lat;
        const int ncorner = E1 * E1 * E1;
        const int lane = threadIdx.x & 31;
        // the warp's lanes take the same iterations (e = e0 + lane), so the foreign slots are
        // claimed with one atomic per warp
        for (int e0 = threadIdx.x - lane; e0 < ncorner; e0 += blockDim.x) {
            const int e = e0 + lane;
            const bool valid = e < ncorner;
            const int kk[3] = {e / (E1 * E1), (e / E1) % E1, e % E1};
            const int uu = lb.b[0] * E + kk[0], ww = lb.b[1] * E + kk[1], zz = lb.b[2] * E + kk[2];
            const int qc[3] = {g0[0] + kk[0], g0[1] + kk[1], g0[2] + kk[2]};
            // owner cell: the cell below the corner on every axis, except on the leaf's lower faces
            int oc[3] = {qc[0] - 1 + (uu == 0), qc[1] - 1 + (ww == 0), qc[2] - 1 + (zz == 0)};
            int own = L;
            if (valid && fposs && (uu == 0 || ww == 0 || zz == 0))
                own = lower_face_owner_cached(v, R, Lc, qc, sm.member, oc);
            // owned by another leaf of the batch: filled by k_foreign_fill
            const bool isf = valid && own != L;
            const unsigned fm = __ballot_sync(0xffffffffu, isf);
            if (fm) {
                const int leader = __ffs(fm) - 1;
                unsigned long long base = 0;
                if (lane == leader) base = atomicAdd(nforeign, (unsigned long long)__popc(fm));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (isf) {
                    const unsigned long long f = base + (unsigned long long)__popc(fm & ((1u << lane) - 1u));
                    if ((i64)f < foreign_cap) foreign[f] = make_int2((int)li, e);
                }
            }
            if (valid && !isf) out[e] = brick_leaf_levels(sm, r, kk, brick_virtual(sm, D, r, Lc, oc, qc, kk)) - v.iso;
        }
    }
}

// corners on a leaf's lower faces owned by a cell of another leaf L' of the
// batch: the same value is a corner of L''s brick holding the owner cell, where
// L' owns it -- copied when that brick is live, evaluated otherwise
__global__ void k_foreign_fill(VArgs v, BrickIndex bix, const int* __restrict__ root_of,
                               const LiveBrick* __restrict__ live, const unsigned char* __restrict__ culled,
                               const int* __restrict__ live_pos, const int2* __restrict__ foreign, i64 n,
                               float* __restrict__ blat, unsigned long long* __restrict__ nslow) {
    const int D = v.e.D;
    for (i64 f = (i64)blockIdx.x * blockDim.x + threadIdx.x; f < n; f += (i64)gridDim.x * blockDim.x) {
        const int2 fe = foreign[f];
        const LiveBrick lb = live[fe.x];
        const VRoot R = v.roots[lb.root];
        const int r = R.depth, S = 1 << (D - r), E = brick_edge(D, r), E1 = E + 1, nb = S / E;
        int Lc[3];
        key_coords(v.e.nd.key[R.node], r, D, Lc);
        const int e = fe.y;
        const int qc[3] = {Lc[0] * S + lb.b[0] * E + e / (E1 * E1), Lc[1] * S + lb.b[1] * E + (e / E1) % E1,
                           Lc[2] * S + lb.b[2] * E + e % E1};
        int oc[3] = {0, 0, 0};
        const int own = lower_face_owner(v, R, Lc, qc, oc);
        const int k2 = root_of[own];
        int Lc2[3];
        key_coords(v.e.nd.key[own], r, D, Lc2);
        int b2[3], kk2[3];
        for (int ax = 0; ax < 3; ++ax) {
            b2[ax] = (oc[ax] - Lc2[ax] * S) / E;
            kk2[ax] = qc[ax] - (Lc2[ax] * S + b2[ax] * E);
        }
        const i64 bi2 = bix.prefix[k2] + ((i64)b2[0] * nb + b2[1]) * nb + b2[2];
        float val;
        if (!culled[bi2]) {
            val = blat[live[live_pos[bi2]].lat + (kk2[0] * E1 + kk2[1]) * E1 + kk2[2]];
        } else {
            atomicAdd(nslow, 1ull);
            val = virtual_corner_value(v, own, r, oc, qc) - v.iso;
        }
        blat[lb.lat + e] = val;
    }
}

// live bricks in brick order
__global__ void k_live_bricks(VArgs v, BrickIndex bix, const unsigned char* __restrict__ culled,
                              const int* __restrict__ pos, i64 nbricks, LiveBrick* __restrict__ live,
                              i64* __restrict__ lat_size, i64* __restrict__ cell_size) {
    for (i64 bi = (i64)blockIdx.x * blockDim.x + threadIdx.x; bi < nbricks; bi += (i64)gridDim.x * blockDim.x) {
        if (culled[bi]) continue;
        const VBrick B = brick_of(v, bix, bi);
        const int E = brick_edge(v.e.D, v.roots[B.root].depth);
        const int p = pos[bi];
        LiveBrick lb;
        lb.root = B.root;
        lb.b[0] = B.b[0]; lb.b[1] = B.b[1]; lb.b[2] = B.b[2];
        lb.lat = 0;
        lb.cell = 0;
        live[p] = lb;
        lat_size[p] = (i64)(E + 1) * (E + 1) * (E + 1);
        cell_size[p] = (i64)E * E * E;
    }
}
__global__ void k_live_offsets(LiveBrick* __restrict__ live, const i64* __restrict__ lat_pos,
                               const i64* __restrict__ cell_pos, i64 n) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
        live[k].lat = lat_pos[k];
        live[k].cell = cell_pos[k];
    }
}
// live bricks split by edge: 8 (first list) and 2 or 4 (second list)
// live bricks by edge: 8 (cnt[0]), 4 (cnt[1]) and 2 (cnt[5])
__global__ void k_live_split(VArgs v, const LiveBrick* __restrict__ live, i64 n, int* __restrict__ big,
                             int* __restrict__ mid, int* __restrict__ small, unsigned long long* __restrict__ cnt) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
        const int E = brick_edge(v.e.D, v.roots[live[k].root].depth);
        if (E == BR) big[atomicAdd(&cnt[0], 1ull)] = (int)k;
        else if (E == 4) mid[atomicAdd(&cnt[1], 1ull)] = (int)k;
        else small[atomicAdd(&cnt[5], 1ull)] = (int)k;
    }
}
__global__ void k_live_flags(const unsigned char* __restrict__ culled, i64 n, int* __restrict__ f) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        f[k] = culled[k] ? 0 : 1;
}

// ---- virtual cells: the cells of the live bricks
struct VirtCells {
    const LiveBrick* live;
    i64 nlive;
    const float* lat;              // corner values (minus iso) of the live bricks
};

// root, cell coordinates in the root's lattice and the 8 corner values of virtual cell e
__device__ __forceinline__ int virt_cell(const VirtCells& vc, const VArgs& v, i64 e, int cu[3], float cv[8]) {
    i64 lo = 0, hi = vc.nlive - 1;
    while (lo < hi) {
        const i64 mid = (lo + hi + 1) >> 1;
        if (vc.live[mid].cell <= e) lo = mid; else hi = mid - 1;
    }
    const LiveBrick lb = vc.live[lo];
    const int E = brick_edge(v.e.D, v.roots[lb.root].depth), E1 = E + 1;
    const int loc = (int)(e - lb.cell);
    const int l3[3] = {loc / (E * E), (loc / E) % E, loc % E};
    cu[0] = lb.b[0] * E + l3[0];
    cu[1] = lb.b[1] * E + l3[1];
    cu[2] = lb.b[2] * E + l3[2];
    const float* L = vc.lat + lb.lat;
    for (int kind = 0; kind < 8; ++kind)
        cv[kind] = L[((l3[0] + (kind & 1)) * E1 + (l3[1] + ((kind >> 1) & 1))) * E1 + (l3[2] + ((kind >> 2) & 1))];
    return lb.root;
}

__global__ void k_virtual_cells(VArgs v, VirtCells vc, i64 total, unsigned char* __restrict__ cat,
                                int* __restrict__ ntri) {
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        int cu[3];
        float cv[8];
        virt_cell(vc, v, e, cu, cv);
        int cc = 0;
        for (int kind = 0; kind < 8; ++kind)
            if (cv[kind] < 0.f) cc |= 1 << c_vid[kind];
        cat[e] = (unsigned char)cc;
        ntri[e] = c_tri_count[cc];
    }
}

// ---------------------------- triangle emission ------------------------------
struct EmitArgs {
    int D;
    int local_bits;
    int weld;           // 1: keys without the batch (vertices shared across batches)
    i64 tri_offset;     // first global triangle of this emission
    u64* keys;          // 3 per triangle
    uint32_t* slot;     // payload: 3*t+q
    float* pos;         // 3 floats per emission
};

__device__ __forceinline__ u64 edge_key(const int lp[3], int o, int D, int batch, int local_bits) {
    const u64 S1 = (u64)(1 << D) + 1;
    u64 k = (((u64)lp[0] * S1 + (u64)lp[1]) * S1 + (u64)lp[2]) * 3 + (u64)o;
    return ((u64)batch << local_bits) | k;
}

// interpolatePoint (main.cu:2584-2597) with p1/p2 in the edge owner's frame
__device__ __forceinline__ void crossing(const int lo_pt[3], int o, bool reversed, float v_lo, float v_hi, int D,
                                         float out[3]) {
    const float inv = 1.0f / (float)(1 << D);
    float p1[3] = {(float)lo_pt[0] * inv, (float)lo_pt[1] * inv, (float)lo_pt[2] * inv};
    float p2[3] = {p1[0], p1[1], p1[2]};
    p2[o] = (float)(lo_pt[o] + 1) * inv;
    float f1 = v_lo, f2 = v_hi;
    if (reversed) {
        float t = p1[o]; p1[o] = p2[o]; p2[o] = t;
        f1 = v_hi; f2 = v_lo;
    }
    for (int i = 0; i < 3; ++i) out[i] = p1[i];
    const float pivot = f1 / (f1 - f2);
    const float another = 1.f - pivot;
    out[o] = fmaf(p2[o], pivot, p1[o] * another);
}

// lattice lower end of edge e of a cell at c[], its orientation and off bits
__device__ __forceinline__ void edge_geom(int e, const int c[3], int lp[3], int& o, int& a0, int& a1, int& b0, int& b1) {
    o = e >> 2;
    a0 = (o == 0) ? 1 : 0;
    a1 = (o == 2) ? 1 : 2;
    b0 = e & 1;
    b1 = (e >> 1) & 1;
    lp[0] = c[0]; lp[1] = c[1]; lp[2] = c[2];
    lp[a0] += b0;
    lp[a1] += b1;
}

// real finest cells
__global__ void k_emit_real(NodeArrays nd, EmitArgs em, i64 lo, const int* __restrict__ active, i64 nactive,
                            const unsigned char* __restrict__ cat, const int* __restrict__ tri_base,
                            const float* __restrict__ cell_v) {
    const int D = em.D;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < nactive; t += (i64)gridDim.x * blockDim.x) {
        const i64 s = active[t];
        const i64 i = lo + s;
        const int cc = cat[s];
        const int nt = c_tri_count[cc];
        int c[3];
        key_coords(nd.key[i], D, D, c);
        const float* cv = cell_v + 8 * s;
        const i64 tb = tri_base[t];
        for (int k = 0; k < 3 * nt; ++k) {
            const int e = c_tri_edges[cc][k];
            int lp[3], o, a0, a1, b0, b1;
            edge_geom(e, c, lp, o, a0, a1, b0, b1);
            // edge owner among the real cells sharing it
            u64 best = ~0ull;
            int own_b0 = b0;
            for (int q = 0; q < 4; ++q) {
                const int d0 = b0 - (q & 1), d1 = b1 - ((q >> 1) & 1);
                int dxyz[3] = {0, 0, 0};
                dxyz[a0] = d0;
                dxyz[a1] = d1;
                const int j = 9 * (dxyz[0] + 1) + 3 * (dxyz[1] + 1) + (dxyz[2] + 1);
                const int nb = nd.neigh[(i64)j * nd.M + i];
                if (nb == -1) continue;
                const u64 kk = nd.key[nb];
                if (kk < best) { best = kk; own_b0 = b0 - d0; }
            }
            const bool rev = (o == 0 && own_b0 == 1);
            const int ev0 = (b0 << a0) | (b1 << a1);   // corner kind of the lower end
            const int ev1 = ev0 | (1 << o);
            float p[3];
            crossing(lp, o, rev, cv[ev0], cv[ev1], D, p);
            const i64 slot = 3 * (tb + k / 3) + (k % 3);
            em.keys[slot] = edge_key(lp, o, D, 0, em.local_bits);
            em.slot[slot] = (uint32_t)slot;
            em.pos[3 * slot] = p[0];
            em.pos[3 * slot + 1] = p[1];
            em.pos[3 * slot + 2] = p[2];
        }
    }
}

__global__ void k_emit_virtual(VArgs v, EmitArgs em, VirtCells vc, const i64* __restrict__ active, i64 nactive,
                               const unsigned char* __restrict__ cat, const i64* __restrict__ tri_base) {
    const int D = em.D;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < nactive; t += (i64)gridDim.x * blockDim.x) {
        const i64 e = active[t];
        int cu[3];
        float cv[8];
        const VRoot R = v.roots[virt_cell(vc, v, e, cu, cv)];
        const int S = 1 << (D - R.depth);
        int Lc[3];
        key_coords(v.e.nd.key[R.node], R.depth, D, Lc);
        const int c[3] = {Lc[0] * S + cu[0], Lc[1] * S + cu[1], Lc[2] * S + cu[2]};
        const int cc = cat[e];
        const int nt = c_tri_count[cc];
        const i64 tb = em.tri_offset + tri_base[t];
        for (int k = 0; k < 3 * nt; ++k) {
            const int ed = c_tri_edges[cc][k];
            int lp[3], o, a0, a1, b0, b1;
            edge_geom(ed, c, lp, o, a0, a1, b0, b1);
            u64 best = ~0ull;
            int own_b0 = b0;
            for (int q = 0; q < 4; ++q) {
                const int d0 = b0 - (q & 1), d1 = b1 - ((q >> 1) & 1);
                int cell[3] = {c[0], c[1], c[2]};
                cell[a0] += d0;
                cell[a1] += d1;
                if (batch_member(v, R, Lc, cell) < 0) continue;
                const u64 kk = cell_key_D(cell, D);
                if (kk < best) { best = kk; own_b0 = b0 - d0; }
            }
            const bool rev = (o == 0 && own_b0 == 1);
            const int ev0 = (b0 << a0) | (b1 << a1);   // corner kind of the lower end
            const int ev1 = ev0 | (1 << o);
            float p[3];
            crossing(lp, o, rev, cv[ev0], cv[ev1], D, p);
            const i64 slot = 3 * (tb + k / 3) + (k % 3);
            em.keys[slot] = edge_key(lp, o, D, em.weld ? 0 : R.batch, em.local_bits);
            em.slot[slot] = (uint32_t)slot;
            em.pos[3 * slot] = p[0];
            em.pos[3 * slot + 1] = p[1];
            em.pos[3 * slot + 2] = p[2];
        }
    }
}

// after sorting: vertex id per sorted element, positions of the first element
__global__ void k_vertex_ids(const u64* __restrict__ keys, const uint32_t* __restrict__ slot, i64 n,
                             const int* __restrict__ pos_scan, const float* __restrict__ epos, float scale,
                             float3 center, int32_t* __restrict__ tri_vid, float* __restrict__ vpos) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
        const bool head = (k == 0) || keys[k] != keys[k - 1];
        const int vid = pos_scan[k] + (head ? 1 : 0) - 1;
        tri_vid[slot[k]] = vid;
        if (head) {
            // input coordinates: p*scale + centre (PlyWriteTriangles plyfile.cu:2801-2812), unfused
            const uint32_t sl = slot[k];
            vpos[3 * (i64)vid] = __fadd_rn(__fmul_rn(epos[3 * (i64)sl], scale), center.x);
            vpos[3 * (i64)vid + 1] = __fadd_rn(__fmul_rn(epos[3 * (i64)sl + 1], scale), center.y);
            vpos[3 * (i64)vid + 2] = __fadd_rn(__fmul_rn(epos[3 * (i64)sl + 2], scale), center.z);
        }
    }
}
// subdivision roots: node index and depth, in node order
__global__ void k_root_list(NodeArrays nd, const int* __restrict__ is_root, const int* __restrict__ pos, i64 n,
                            int2* __restrict__ out) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        if (is_root[i]) out[pos[i]] = make_int2((int)i, (int)nd.depth[i]);
}
// subdivision roots are in node order, hence in depth order: the index of the
// first root at depth d is the root prefix at the first node of depth d, and
// every per-root count (bricks, rows, batch) is a closed form of the depth
struct DepthStarts {
    i64 base[17];
};
__global__ void k_depth_firsts(const int* __restrict__ rpos, DepthStarts b, int D, int* __restrict__ out) {
    const int d = threadIdx.x;
    if (d <= D) out[d] = rpos[b.base[d]];
}
struct RootLayout {
    int first[17];    // first root at depth d
    int batch[17];    // batch of the roots at depth d >= 3
    i64 off[4][17];   // bricks, brick rows, super-bricks, super rows of the roots above depth d
    i64 per[4][17];   // the same per root at depth d
};
__global__ void k_make_roots(const int2* __restrict__ dr, int nr, int D, RootLayout L, VRoot* __restrict__ roots,
                             i64* __restrict__ pre) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nr; k += gridDim.x * blockDim.x) {
        const int2 r = dr[k];
        const int d = r.y;
        VRoot R;
        R.node = r.x;
        R.depth = d;
        R.batch = d < 3 ? k + 1 : L.batch[d];   // one batch per root above depth 3, one per depth from 3
        R.pad = 0;
        roots[k] = R;
        const i64 local = k - L.first[d];
#pragma unroll
        for (int q = 0; q < 4; ++q) pre[(i64)q * (nr + 1) + k] = L.off[q][d] + local * L.per[q][d];
        if (k == 0)
#pragma unroll
            for (int q = 0; q < 4; ++q) pre[(i64)q * (nr + 1) + nr] = L.off[q][D];
    }
}

__global__ void k_key_heads(const u64* __restrict__ keys, i64 n, int* __restrict__ f) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        f[k] = (k == 0 || keys[k] != keys[k - 1]) ? 1 : 0;
}
__global__ void k_active_flags(const int* __restrict__ ntri, i64 n, int* __restrict__ f) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        f[k] = ntri[k] > 0 ? 1 : 0;
}
template <class TI>
__global__ void k_compact_idx(const int* __restrict__ f, const int* __restrict__ pos, i64 n, TI* __restrict__ out) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        if (f[k]) out[pos[k]] = (TI)k;
}
__global__ void k_gather_ntri(const int* __restrict__ ntri, const i64* __restrict__ active, i64 n,
                              i64* __restrict__ out) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        out[k] = ntri[active[k]];
}
__global__ void k_gather_ntri32(const int* __restrict__ ntri, const int* __restrict__ active, i64 n,
                                int* __restrict__ out) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        out[k] = ntri[active[k]];
}

void stage_mesh(Ctx& c) {
    ensure_mc_tables();
    cudaStream_t s = c.stream;
    const int D = c.D;
    const NodeArrays& nd = c.nodes;
    const i64 M = nd.M, lo = c.base[D], nD = c.count[D];
    const int kx = c.kbegin("mesh_tables", 0.0);
    float* x27 = build_x27(c, lo);
    EvalArgs ea{c.nodes, D, c.basis, c.x, x27, x27 ? lo : 0, nullptr, c.params.stable_basis};
    float* lb = nullptr;
    {
        const i64 total = lattice_basis_offset(D, D + 1);
        lb = dalloc<float>(total, s);
        k_lattice_basis<<<grid_for(total, 256), 256, 0, s>>>(c.basis, D, total, lb, c.params.stable_basis);
        CK_LAUNCH();
        ea.lb = lb;
    }
    c.kend(kx);
    // ---- finest corner values, categories
    float* cval = dalloc<float>(8 * nD, s);
    float* cell_v = dalloc<float>(8 * nD, s);
    unsigned char* cat = dalloc<unsigned char>(nD, s);
    int* ntri = dalloc<int>(nD, s);
    int kt = c.kbegin("corner_values", (double)M * (108 + 8 + 4 + 4) + (double)nD * 8 * 4);
    {
        if (nD >= (1ll << 28)) {
            set_last_error("%lld finest nodes exceed the corner list's 2^28", (long long)nD);
            throw Error{PRGPU_ERR_LIMIT, {0}};
        }
        unsigned char* omask = dalloc<unsigned char>(nD, s);
        int* ocnt = dalloc<int>(nD, s);
        int* ofirst = dalloc<int>(nD + 1, s);
        k_finest_owned<<<grid_for(nD, 256), 256, 0, s>>>(nd, lo, M, omask, ocnt);
        CK_LAUNCH();
        exclusive_scan<int, int>(ocnt, ofirst, nD, ofirst + nD, s);
        const i64 nown = read_scalar(ofirst + nD, s);
        if (nown > 0) {
            int* olist = dalloc<int>(nown, s);
            k_finest_list<<<grid_for(nD, 256), 256, 0, s>>>(omask, ofirst, nD, olist);
            CK_LAUNCH();
            k_finest_corner_values<<<grid_for(nown, 128, 1ll << 30), 128, 0, s>>>(ea, lo, olist, nown, c.iso, cval);
            CK_LAUNCH();
            dfree(olist, s);
        }
        dfree(omask, s);
        dfree(ocnt, s);
        dfree(ofirst, s);
    }
    c.kend(kt);
    kt = c.kbegin("cells", (double)nD * (8 * 4 + 108 + 8 * 4 + 1 + 4));
    k_finest_cells<<<grid_for(nD, 128, 1ll << 30), 128, 0, s>>>(nd, lo, M, cval, cell_v, cat, ntri);
    CK_LAUNCH();
    c.kend(kt);
    dfree(cval, s);
    // ---- face marks and subdivision roots
    int* fflag = dalloc<int>(6 * M, s);
    CK(cudaMemsetAsync(fflag, 0, (size_t)(6 * M) * sizeof(int), s));
    kt = c.kbegin("mark_faces", (double)nD * (1 + 108) + (double)M * 24);
    k_mark_faces<<<grid_for(nD, 128, 1ll << 30), 128, 0, s>>>(nd, D, lo, M, cat, fflag);
    CK_LAUNCH();
    c.kend(kt);
    const i64 nCoarse = lo;   // nodes at depth < D
    dfree(c.d_has_tri, s);
    dfree(c.d_has_int, s);
    c.n_coarse = nCoarse;
    int* has_tri = c.d_has_tri = dalloc<int>(nCoarse, s);
    int* has_int = c.d_has_int = dalloc<int>(nCoarse, s);
    int* is_root = dalloc<int>(nCoarse, s);
    CK(cudaMemsetAsync(has_tri, 0, nCoarse * sizeof(int), s));
    CK(cudaMemsetAsync(has_int, 0, nCoarse * sizeof(int), s));
    CK(cudaMemsetAsync(is_root, 0, nCoarse * sizeof(int), s));
    if (nCoarse > 1) {
        const int kc = c.kbegin("coarse_leaves", (double)nCoarse * (4 + 108 + 8 + 3 * 4 + 8 * 4) + (double)M * 4);
        unsigned char* need = dalloc<unsigned char>(8 * nCoarse, s);
        float* ccv = dalloc<float>(8 * nCoarse, s);
        CK(cudaMemsetAsync(need, 0, 8 * nCoarse, s));
        k_coarse_need<<<grid_for(nCoarse - 1, 256), 256, 0, s>>>(nd, 1, nCoarse, need);
        CK_LAUNCH();
        {
            // one thread per needed corner (list of (node << 3) | corner)
            unsigned char* nmask = dalloc<unsigned char>(nCoarse, s);
            int* ncnt = dalloc<int>(nCoarse, s);
            int* nfirst = dalloc<int>(nCoarse + 1, s);
            k_need_mask<<<grid_for(nCoarse, 256), 256, 0, s>>>(need, nCoarse, nmask, ncnt);
            CK_LAUNCH();
            exclusive_scan<int, int>(ncnt, nfirst, nCoarse, nfirst + nCoarse, s);
            const i64 nneed = read_scalar(nfirst + nCoarse, s);
            if (nneed > 0) {
                int* nlist = dalloc<int>(nneed, s);
                k_finest_list<<<grid_for(nCoarse, 256), 256, 0, s>>>(nmask, nfirst, nCoarse, nlist);
                CK_LAUNCH();
                k_coarse_corner_list<<<grid_for(nneed, 128, 1ll << 30), 128, 0, s>>>(ea, nlist, nneed, c.iso, ccv);
                CK_LAUNCH();
                dfree(nlist, s);
            }
            dfree(nmask, s);
            dfree(ncnt, s);
            dfree(nfirst, s);
        }
        k_coarse_leaves<<<grid_for(nCoarse - 1, 128, 1ll << 30), 128, 0, s>>>(ea, 1, nCoarse, ccv, fflag, has_tri,
                                                                             has_int, is_root);
        CK_LAUNCH();
        c.kend(kc);
        dfree(need, s);
        dfree(ccv, s);
    }
    dfree(fflag, s);
    int kg = c.kbegin("mesh_lists", 0.0);
    // subdivision roots in node order, compacted on the device; the host reads only
    // the index of the first root of every depth
    int2* droot_list = nullptr;
    int nr = 0;
    RootLayout layout{};
    i64 tot[4] = {0, 0, 0, 0}, nbig = 0;
    int nbatches = 1;
    {
        int* rpos = dalloc<int>(nCoarse + 1, s);
        exclusive_scan<int, int>(is_root, rpos, nCoarse, rpos + nCoarse, s);
        DepthStarts ds{};
        for (int d = 0; d <= D; ++d) ds.base[d] = c.base[d];
        int* dfirst = dalloc<int>(D + 1, s);
        k_depth_firsts<<<1, 32, 0, s>>>(rpos, ds, D, dfirst);
        CK_LAUNCH();
        int hfirst[17];
        CK(cudaMemcpyAsync(hfirst, dfirst, (D + 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        dfree(dfirst, s);
        nr = hfirst[D];   // roots are coarse nodes (depth < D)
        droot_list = dalloc<int2>(std::max(nr, 1), s);
        k_root_list<<<grid_for(nCoarse, 256), 256, 0, s>>>(nd, is_root, rpos, nCoarse, droot_list);
        CK_LAUNCH();
        dfree(rpos, s);
        c.roots_per_depth.assign(D + 1, 0);
        int nb = 0;
        for (int d = 0; d <= D; ++d) {
            const int cnt = d < D ? hfirst[d + 1] - hfirst[d] : 0;
            c.roots_per_depth[d] = cnt;
            const int S = 1 << (D - d), E = std::min(S, BR), nbk = S / E;
            const int ns = (D - d >= 6) ? S / (4 * BR) : 0;
            layout.first[d] = hfirst[d];
            layout.per[0][d] = (i64)nbk * nbk * nbk;
            layout.per[1][d] = 3 * nbk;
            layout.per[2][d] = (i64)ns * ns * ns;
            layout.per[3][d] = 3 * ns;
            for (int q = 0; q < 4; ++q) {
                layout.off[q][d] = tot[q];
                tot[q] += (i64)cnt * layout.per[q][d];
            }
            if (D - d >= 4) nbig = tot[0];   // bricks of leaves with lattice edge >= 16 come first
            if (d < 3) nb += cnt;
            else if (cnt > 0) layout.batch[d] = ++nb;
        }
        nbatches = nb + 1;
    }
    dfree(is_root, s);
    c.subdivide_roots = nr;
    // ---- real cells: active list, triangle bases
    int* flags = dalloc<int>(std::max<i64>(nD, 1), s);
    int* fpos = dalloc<int>(nD + 1, s);
    k_active_flags<<<grid_for(nD, 256), 256, 0, s>>>(ntri, nD, flags);
    CK_LAUNCH();
    exclusive_scan<int, int>(flags, fpos, nD, fpos + nD, s);
    const i64 nact_real = read_scalar(fpos + nD, s);
    int* act_real = dalloc<int>(std::max<i64>(nact_real, 1), s);
    k_compact_idx<int><<<grid_for(nD, 256), 256, 0, s>>>(flags, fpos, nD, act_real);
    CK_LAUNCH();
    int* tri_real = dalloc<int>(nact_real + 1, s);
    {
        int* tmp = dalloc<int>(std::max<i64>(nact_real, 1), s);
        k_gather_ntri32<<<grid_for(nact_real, 256), 256, 0, s>>>(ntri, act_real, nact_real, tmp);
        CK_LAUNCH();
        exclusive_scan<int, int>(tmp, tri_real, nact_real, tri_real + nact_real, s);
        dfree(tmp, s);
    }
    const i64 ntri_real = read_scalar(tri_real + nact_real, s);
    dfree(flags, s);
    dfree(fpos, s);
    c.kend(kg);
    // ---- virtual cells: every subdivided leaf cut into bricks, bounded and culled
    // before evaluation
    i64 ntri_virt = 0, nact_virt = 0, total_cells = 0;
    c.total_bricks = 0;
    c.live_bricks = 0;
    c.foreign_corners = 0;
    c.foreign_slow = 0;
    VRoot* droots = nullptr;
    i64 *act_virt = nullptr, *tri_virt = nullptr;
    unsigned char* vcat = nullptr;
    int* vntri = nullptr;
    int* bflag = nullptr;
    float* lat_brick = nullptr;
    LiveBrick* live = nullptr;
    VArgs va;
    va.e = ea;
    va.iso = c.iso;
    va.nroots = nr;
    VirtCells vc{};
    if (nr > 0) {
        kg = c.kbegin("mesh_lists", 0.0);
        droots = dalloc<VRoot>(nr, s);
        bflag = dalloc<int>(M, s);
        // prefix tables: bricks, brick rows, super-bricks, super rows (nr + 1 entries each)
        i64* dpre = dalloc<i64>(4 * ((i64)nr + 1), s);
        k_make_roots<<<grid_for(nr, 256), 256, 0, s>>>(droot_list, nr, D, layout, droots, dpre);
        CK_LAUNCH();
        CK(cudaMemsetAsync(bflag, 0, M * sizeof(int), s));
        k_batch_flags<<<grid_for(nr, 256), 256, 0, s>>>(droots, nr, bflag);
        CK_LAUNCH();
        va.roots = droots;
        va.batch_root_flag = bflag;
        const i64 nbricks = tot[0], nrows = tot[1], nsuper = tot[2], nsrows = tot[3];
        i64* dbpre = dpre;
        i64* drpre = dpre + nr + 1;
        i64* dspre = dpre + 2 * (nr + 1);
        i64* dsrpre = dpre + 3 * (nr + 1);
        float* rows = dalloc<float>(nrows * PROW * (D + 1), s);
        float* xl = dalloc<float>((i64)nr * BR_LEVELS * 27, s);
        float* anc = dalloc<float>((i64)nr * ANC_STRIDE, s);
        BrickIndex bix{dbpre, drpre, nr, rows, xl, anc, {}};
        for (int d = 0; d <= D; ++d) {
            bix.dl.first[d] = layout.first[d];
            bix.dl.lg[d] = std::max(D - d - 3, 0);          // bricks per edge 2^(D-d) / min(2^(D-d), 8)
            bix.dl.slg[d] = std::max(D - d - 5, 0);         // super-bricks per edge 2^(D-d) / 32 (D-d >= 6)
            bix.dl.boff[d] = layout.off[0][d];
            bix.dl.soff[d] = layout.off[2][d];
            bix.dl.roff[d] = layout.off[1][d];
            bix.dl.sroff[d] = layout.off[3][d];
        }
        c.kend(kg);
        const int kr = c.kbegin("brick_rows", (double)nrows * PROW * (D + 1) * 4);
        k_brick_rows<<<grid_for(nrows * (D + 1), 128), 128, 0, s>>>(va, bix.dl, nrows, 0, c.d_has_tri, rows);
        CK_LAUNCH();
        float* srows = nullptr;
        if (nsrows > 0) {
            srows = dalloc<float>(nsrows * ROW_PER_DEPTH * (D + 1), s);
            k_brick_rows<<<grid_for(nsrows * (D + 1), 128), 128, 0, s>>>(va, bix.dl, nsrows, 1, c.d_has_tri, srows);
            CK_LAUNCH();
        }
        k_brick_xl<<<grid_for((i64)nr * 32, 32 * XL_WARPS), 32 * XL_WARPS, 0, s>>>(va, nr, c.d_has_tri, xl, anc);
        CK_LAUNCH();
        c.kend(kr);
        unsigned char* culled = dalloc<unsigned char>(nbricks, s);
        signed char* bsign = dalloc<signed char>(nbricks, s);
        int* root_of = dalloc<int>(nCoarse, s);
        CK(cudaMemsetAsync(root_of, 0xff, nCoarse * sizeof(int), s));
        k_root_of<<<grid_for(nr, 256), 256, 0, s>>>(droots, nr, root_of);
        CK_LAUNCH();
        // compulsory: every brick row and the leaves' ancestor polynomial (super-bricks: their
        // rows and the neighbour x) once, the sign written and read, the culled flag written
        signed char* ssign = nullptr;
        if (nsuper > 0) {
            ssign = dalloc<signed char>(nsuper, s);
            const int ksb = c.kbegin("super_bound", (double)nsrows * (6 + 2 * BR_WEXT) * (D + 1) * 4 +
                                                        (double)nr * BR_LEVELS * 27 * 4 + (double)nsuper);
            k_super_bound<<<grid_for(nsuper * 32, 256, (i64)c.sms * 8), 256, 0, s>>>(va, bix.dl, dsrpre, srows, xl,
                                                                                    nsuper, ssign);
            CK_LAUNCH();
            c.kend(ksb);
            if (c.profile) {   // statistics only
                std::vector<signed char> hs(nsuper);
                CK(cudaMemcpyAsync(hs.data(), ssign, nsuper, cudaMemcpyDeviceToHost, s));
                CK(cudaStreamSynchronize(s));
                c.super_bricks = nsuper;
                c.super_decided = 0;
                for (signed char v : hs) c.super_decided += (v != 0);
            }
        }
        // bricks of leaves with lattice edge >= 16 come first (roots are in depth order)
        const int kb = c.kbegin("brick_bound", (double)nrows * PROW * (D + 1) * 4 +
                                                   (double)nr * ANC_STRIDE * 4 + (double)nbricks * 3);
        k_brick_bound<<<grid_for(nbig * 32, BB_BLOCK, (i64)c.sms * 8), BB_BLOCK, 0, s>>>(va, bix, 0, nbig, dspre,
                                                                                         ssign, c.d_has_tri, bsign);
        CK_LAUNCH();
        c.kend(kb);
        const int kb2 = c.kbegin("brick_bound_small", (double)(nbricks - nbig) * 3);
        if (nbricks > nbig) {
            k_brick_bound<<<grid_for((nbricks - nbig) * 32, BB_BLOCK, (i64)c.sms * 8), BB_BLOCK, 0, s>>>(
                va, bix, nbig, nbricks, dspre, ssign, c.d_has_tri, bsign);
            CK_LAUNCH();
        }
        k_brick_cull<<<grid_for(nbricks, 256), 256, 0, s>>>(va, bix, root_of, bsign, nbricks, culled);
        CK_LAUNCH();
        c.kend(kb2);
        dfree(bsign, s);
        dfree(ssign, s);
        dfree(srows, s);
        dfree(anc, s);
        kg = c.kbegin("mesh_lists", 0.0);
        int* bf = dalloc<int>(nbricks, s);
        int* bp = dalloc<int>(nbricks + 1, s);
        k_live_flags<<<grid_for(nbricks, 256), 256, 0, s>>>(culled, nbricks, bf);
        CK_LAUNCH();
        exclusive_scan<int, int>(bf, bp, nbricks, bp + nbricks, s);
        const i64 nlive = read_scalar(bp + nbricks, s);
        c.total_bricks = nbricks;
        c.live_bricks = nlive;
        c.kend(kg);
        if (nlive > 0) {
            kg = c.kbegin("mesh_lists", 0.0);
            live = dalloc<LiveBrick>(nlive, s);
            i64* lsz = dalloc<i64>(nlive, s);
            i64* csz = dalloc<i64>(nlive, s);
            i64* lpos = dalloc<i64>(nlive + 1, s);
            i64* cpos = dalloc<i64>(nlive + 1, s);
            k_live_bricks<<<grid_for(nbricks, 256), 256, 0, s>>>(va, bix, culled, bp, nbricks, live, lsz, csz);
            CK_LAUNCH();
            exclusive_scan<i64, i64>(lsz, lpos, nlive, lpos + nlive, s);
            exclusive_scan<i64, i64>(csz, cpos, nlive, cpos + nlive, s);
            k_live_offsets<<<grid_for(nlive, 256), 256, 0, s>>>(live, lpos, cpos, nlive);
            CK_LAUNCH();
            const i64 lat_total = read_scalar(lpos + nlive, s);
            total_cells = read_scalar(cpos + nlive, s);
            lat_brick = dalloc<float>(lat_total, s);
            // bricks of edge 8, 4 and 2 go to three instances of the evaluation
            // counters: edge 8, edge 4, foreign corners, window layout overflows, foreign corners
            // evaluated, edge 2
            unsigned long long* cnt3 = dalloc<unsigned long long>(6, s);
            int* lists = dalloc<int>(3 * nlive, s);
            CK(cudaMemsetAsync(cnt3, 0, 6 * sizeof(unsigned long long), s));
            // corners owned by another leaf: at most the lower-face corners of the live bricks
            const i64 fcap = std::min<i64>(lat_total, nlive * (BR_CORNERS - BR * BR * BR));
            int2* foreign = dalloc<int2>(std::max<i64>(fcap, 1), s);
            k_live_split<<<grid_for(nlive, 256), 256, 0, s>>>(va, live, nlive, lists, lists + nlive,
                                                              lists + 2 * nlive, cnt3);
            CK_LAUNCH();
            unsigned long long hc[6];
            CK(cudaMemcpyAsync(hc, cnt3, sizeof hc, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            c.kend(kg);
            // compulsory: the corner values written (bricks of edge 8: 729 each)
            const int ke = c.kbegin("brick_eval", (double)hc[0] * BR_CORNERS * 4);
            if (hc[0] > 0) {
                k_brick_eval<BR, BR_BLOCK><<<grid_for((i64)hc[0], 1, (i64)c.sms * 16), BR_BLOCK, 0, s>>>(
                    va, bix, root_of, live, lists, (i64)hc[0], lat_brick, cnt3 + 2, foreign, fcap);
                CK_LAUNCH();
            }
            c.kend(ke);
            const int ks = c.kbegin("brick_eval_small", (double)(lat_total - (i64)hc[0] * BR_CORNERS) * 4);
            if (hc[1] > 0) {
                k_brick_eval<4, 64><<<grid_for((i64)hc[1], 1, (i64)c.sms * 24), 64, 0, s>>>(
                    va, bix, root_of, live, lists + nlive, (i64)hc[1], lat_brick, cnt3 + 2, foreign, fcap);
                CK_LAUNCH();
            }
            if (hc[5] > 0) {   // 27 corners: one warp per brick
                k_brick_eval<2, 32><<<grid_for((i64)hc[5], 1, (i64)c.sms * 32), 32, 0, s>>>(
                    va, bix, root_of, live, lists + 2 * nlive, (i64)hc[5], lat_brick, cnt3 + 2, foreign, fcap);
                CK_LAUNCH();
            }
            c.kend(ks);
            unsigned long long hf[2];
            CK(cudaMemcpyAsync(hf, cnt3 + 2, sizeof hf, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            c.foreign_corners = (i64)hf[0];
            if (hf[1]) {
                set_last_error("brick window layout overflow in %llu bricks", hf[1]);
                throw Error{PRGPU_ERR_LIMIT, {0}};
            }
            if ((i64)hf[0] > fcap) {
                set_last_error("foreign corner list overflow (%llu > %lld)", hf[0], (long long)fcap);
                throw Error{PRGPU_ERR_LIMIT, {0}};
            }
            if (hf[0] > 0) {
                const int kf = c.kbegin("foreign_fill", (double)hf[0] * 8);
                k_foreign_fill<<<grid_for((i64)hf[0], 128, 1ll << 30), 128, 0, s>>>(
                    va, bix, root_of, live, culled, bp, foreign, (i64)hf[0], lat_brick, cnt3 + 4);
                CK_LAUNCH();
                c.kend(kf);
                c.foreign_slow = (i64)read_scalar(cnt3 + 4, s);
            }
            dfree(cnt3, s);
            dfree(lists, s);
            dfree(foreign, s);
            dfree(lsz, s);
            dfree(csz, s);
            dfree(lpos, s);
            dfree(cpos, s);
        }
        dfree(bf, s);
        dfree(bp, s);
        dfree(culled, s);
        dfree(root_of, s);
        dfree(dpre, s);
        dfree(rows, s);
        dfree(xl, s);
        vc.live = live;
        vc.nlive = nlive;
        vc.lat = lat_brick;
        if (total_cells > 0) {
            vcat = dalloc<unsigned char>(total_cells, s);
            vntri = dalloc<int>(total_cells, s);
            const int kc2 = c.kbegin("virtual_cells", (double)total_cells * (8 * 4 + 5));
            k_virtual_cells<<<grid_for(total_cells, 256, 1ll << 30), 256, 0, s>>>(va, vc, total_cells, vcat, vntri);
            CK_LAUNCH();
            c.kend(kc2);
            kg = c.kbegin("mesh_lists", 0.0);
            int* vf = dalloc<int>(total_cells, s);
            int* vp = dalloc<int>(total_cells + 1, s);
            k_active_flags<<<grid_for(total_cells, 256), 256, 0, s>>>(vntri, total_cells, vf);
            CK_LAUNCH();
            exclusive_scan<int, int>(vf, vp, total_cells, vp + total_cells, s);
            nact_virt = read_scalar(vp + total_cells, s);
            act_virt = dalloc<i64>(std::max<i64>(nact_virt, 1), s);
            k_compact_idx<i64><<<grid_for(total_cells, 256), 256, 0, s>>>(vf, vp, total_cells, act_virt);
            CK_LAUNCH();
            dfree(vf, s);
            dfree(vp, s);
            tri_virt = dalloc<i64>(nact_virt + 1, s);
            i64* tmp = dalloc<i64>(std::max<i64>(nact_virt, 1), s);
            k_gather_ntri<<<grid_for(nact_virt, 256), 256, 0, s>>>(vntri, act_virt, nact_virt, tmp);
            CK_LAUNCH();
            exclusive_scan<i64, i64>(tmp, tri_virt, nact_virt, tri_virt + nact_virt, s);
            dfree(tmp, s);
            ntri_virt = read_scalar(tri_virt + nact_virt, s);
            c.kend(kg);
        }
    }
    c.virtual_cells = total_cells;
    // ---- emission, sort, vertex ids
    const i64 ntri_all = ntri_real + ntri_virt;
    const i64 nem = 3 * ntri_all;
    if (nem > 0x7fffffffLL) {
        set_last_error("mesh of %lld triangles exceeds 32-bit indexing", (long long)ntri_all);
        throw Error{PRGPU_ERR_LIMIT, {0}};
    }
    int local_bits = 0;
    {
        const double lat_edges = 3.0 * std::pow((double)((1 << D) + 1), 3.0);
        while ((double)(1ull << local_bits) < lat_edges) ++local_bits;
    }
    int batch_bits = 0;
    while (!c.params.weld && (1 << batch_bits) < nbatches) ++batch_bits;
    c.mesh_v.clear();
    c.mesh_f.clear();
    c.batch_tri.assign(1, ntri_real);
    c.batch_tri.push_back(ntri_virt);
    if (nem > 0) {
        EmitArgs em;
        em.D = D;
        em.local_bits = local_bits;
        em.weld = c.params.weld ? 1 : 0;
        em.tri_offset = 0;
        em.keys = dalloc<u64>(nem, s);
        em.slot = dalloc<uint32_t>(nem, s);
        em.pos = dalloc<float>(3 * nem, s);
        const int kem = c.kbegin("emit", (double)nem * (8 + 4 + 12));
        if (nact_real > 0) {
            k_emit_real<<<grid_for(nact_real, 128, 1ll << 30), 128, 0, s>>>(nd, em, lo, act_real, nact_real, cat,
                                                                            tri_real, cell_v);
            CK_LAUNCH();
        }
        if (nact_virt > 0) {
            EmitArgs ev = em;
            ev.tri_offset = ntri_real;
            k_emit_virtual<<<grid_for(nact_virt, 128, 1ll << 30), 128, 0, s>>>(va, ev, vc, act_virt, nact_virt, vcat,
                                                                               tri_virt);
            CK_LAUNCH();
        }
        c.kend(kem);
        u64* ktmp = dalloc<u64>(nem, s);
        uint32_t* stmp = dalloc<uint32_t>(nem, s);
        const int ks = c.kbegin("edge_sort", (double)nem * 12 * 2);
        radix_sort_pairs(em.keys, em.slot, ktmp, stmp, nem, local_bits + batch_bits, s);
        c.kend(ks);
        dfree(ktmp, s);
        dfree(stmp, s);
        const int kvi = c.kbegin("vertex_ids", (double)nem * (8 * 2 + 4 + 4 + 12));
        int* hf = dalloc<int>(nem, s);
        int* hp = dalloc<int>(nem + 1, s);
        k_key_heads<<<grid_for(nem, 256), 256, 0, s>>>(em.keys, nem, hf);
        CK_LAUNCH();
        exclusive_scan<int, int>(hf, hp, nem, hp + nem, s);
        const i64 nvert = read_scalar(hp + nem, s);
        int32_t* tri_vid = dalloc<int32_t>(nem, s);
        float* vpos = dalloc<float>(3 * std::max<i64>(nvert, 1), s);
        k_vertex_ids<<<grid_for(nem, 256), 256, 0, s>>>(em.keys, em.slot, nem, hp, em.pos, c.scale,
                                                        make_float3(c.center[0], c.center[1], c.center[2]),
                                                        tri_vid, vpos);
        CK_LAUNCH();
        c.kend(kvi);
        const int kd = c.kbegin("mesh_d2h", (double)(3 * nvert + nem) * 4);
        c.mesh_v.resize(3 * nvert);
        c.mesh_f.resize(nem);
        CK(cudaMemcpyAsync(c.mesh_v.data(), vpos, 3 * nvert * sizeof(float), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(c.mesh_f.data(), tri_vid, nem * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        c.kend(kd);
        CK(cudaStreamSynchronize(s));
        dfree(hf, s); dfree(hp, s); dfree(tri_vid, s); dfree(vpos, s);
        dfree(em.keys, s); dfree(em.slot, s); dfree(em.pos, s);
    }
    dfree(act_real, s);
    dfree(tri_real, s);
    dfree(droots, s); dfree(droot_list, s); dfree(act_virt, s); dfree(tri_virt, s);
    dfree(vcat, s); dfree(vntri, s); dfree(bflag, s);
    dfree(lat_brick, s); dfree(live, s);
    dfree(cell_v, s);
    dfree(x27, s);
    dfree(lb, s);
    dfree(cat, s);
    dfree(ntri, s);
}

}  // namespace prgpu
