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

static bool g_mc_uploaded = false;
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
    g_mc_uploaded = true;
}

// ----------------------------- evaluation ----------------------------------
struct EvalArgs {
    NodeArrays nd;
    int D;
    const CPoly* basis;
    const float* x;
};

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
            bv[ax][t] = (c >= 0 && c < lim) ? cpoly_value<3>(a.basis[fb + c], q[ax]) : 0.f;
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

__device__ __forceinline__ float walk_up(const EvalArgs& a, i64 node, const float q[3], float val) {
    while (node != -1) {
        const int d = a.nd.depth[node];
        int xyz[3];
        key_coords(a.nd.key[node], d, a.D, xyz);
        val = level_sum(a, node, d, xyz, q, val);
        node = a.nd.parent[node];
    }
    return val;
}

__global__ void k_point_values(EvalArgs a, const float* __restrict__ pts, const int* __restrict__ point_node, i64 n,
                               float* __restrict__ out, double* __restrict__ sum) {
    double loc = 0;
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
        const float q[3] = {pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]};
        const float v = walk_up(a, point_node[k], q, 0.f);
        out[k] = v;
        loc += (double)v;
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
    EvalArgs a{c.nodes, c.D, c.basis, c.x};
    const int kt = c.kbegin("point_values", (double)c.N * (12 + 4 + 4) + (double)c.nodes.M * (4 + 4 + 8 + 108));
    k_point_values<<<grid_for(c.N, 128, 1ll << 30), 128, 0, s>>>(a, c.pts, c.point_node, c.N, c.point_value, sum);
    CK_LAUNCH();
    c.kend(kt);
    double h = read_scalar(sum, s);
    dfree(sum, s);
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
    float q[3];
    corner_pos(xyz, d, kind, q);
    float val = 0.f;
    if (o > 0) {
        val = walk_up(a, o, q, val);
        const int exceed = c_vid[kind];
        i64 node = o;
        for (int dd = d + 1; dd <= a.D; ++dd) {
            const int c0 = a.nd.child0[node];
            if (c0 == -1) break;
            node = c0 + exceed;
            int cx[3];
            key_coords(a.nd.key[node], dd, a.D, cx);
            val = level_sum(a, node, dd, cx, q, val);
        }
    }
    return val - iso;
}

// finest-depth corners: each corner evaluated by its owner
__global__ void k_finest_corner_values(EvalArgs a, i64 lo, i64 hi, float iso, float* __restrict__ cval) {
    for (i64 i = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (i64)gridDim.x * blockDim.x) {
        for (int kind = 0; kind < 8; ++kind) {
            int ok;
            const int own = corner_owner(a.nd, i, kind, ok);
            if (own == i) cval[8 * (i - lo) + kind] = owner_corner_value(a, i, kind, iso);
        }
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

// leaves above the finest depth: sign change at their corners or a marked face
// (ProcessLeafNodesAtOtherDepth main.cu:2957-2986, ifSubdivide :2988-2992)
__global__ void k_coarse_leaves(EvalArgs a, i64 lo, i64 hi, float iso, const int* __restrict__ fflag,
                                int* __restrict__ has_tri, int* __restrict__ has_int, int* __restrict__ is_root) {
    const NodeArrays& nd = a.nd;
    for (i64 i = lo + (i64)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += (i64)gridDim.x * blockDim.x) {
        if (nd.child0[i] != -1) { is_root[i] = 0; continue; }
        float v[8];
        for (int kind = 0; kind < 8; ++kind) {
            int ok;
            const int own = corner_owner(nd, i, kind, ok);
            v[c_vid[kind]] = owner_corner_value(a, own, ok, iso);
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
    i64 lattice_base;  // first corner value of this root
    i64 cell_base;     // first virtual cell of this root
    i64 brick_base;    // first brick of this root, -1 for small roots (lattice edge <= 8)
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
    const float inv = 1.0f / (float)(1 << D);
    const float q[3] = {(float)qc[0] * inv, (float)qc[1] * inv, (float)qc[2] * inv};
    int Lc[3];
    key_coords(nd.key[L], r, D, Lc);
    float val = 0.f;
    for (int d = D; d > r; --d) {
        const int sh = D - d;
        const int V[3] = {oc[0] >> sh, oc[1] >> sh, oc[2] >> sh};
        const int fb = (1 << d) - 1, lim = 1 << d;
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
                bv[ax][t] = (cc >= 0 && cc < lim) ? cpoly_value<3>(a.basis[fb + cc], q[ax]) : 0.f;
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
    val = walk_up(a, L, q, val);
    return val;
}

__device__ __forceinline__ u64 cell_key_D(const int c[3], int D) { return coords_key(c[0], c[1], c[2], D, D); }

// one thread per lattice corner of the listed roots (the small ones)
__global__ void k_virtual_corners(VArgs v, const int* __restrict__ list, const i64* __restrict__ list_prefix,
                                  int nlist, i64 total, const i64* __restrict__ lat_prefix, float* __restrict__ lat) {
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        int lo = 0, hi = nlist - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (list_prefix[mid] <= e) lo = mid; else hi = mid - 1;
        }
        const int ri = list[lo];
        const VRoot R = v.roots[ri];
        const int D = v.e.D, S = 1 << (D - R.depth), S1 = S + 1;
        const i64 loc = e - list_prefix[lo];
        const int u = (int)(loc / ((i64)S1 * S1)), w = (int)((loc / S1) % S1), z = (int)(loc % S1);
        int Lc[3];
        key_coords(v.e.nd.key[R.node], R.depth, D, Lc);
        const int qc[3] = {Lc[0] * S + u, Lc[1] * S + w, Lc[2] * S + z};
        // owner: min key among batch cells sharing the corner
        u64 best = ~0ull;
        int own_root = -1, oc[3] = {0, 0, 0};
        for (int eo = 0; eo < 8; ++eo) {
            const int cell[3] = {qc[0] - (eo & 1), qc[1] - ((eo >> 1) & 1), qc[2] - ((eo >> 2) & 1)};
            const int m = batch_member(v, R, Lc, cell);
            if (m < 0) continue;
            const u64 kk = cell_key_D(cell, D);
            if (kk < best) { best = kk; own_root = m; oc[0] = cell[0]; oc[1] = cell[1]; oc[2] = cell[2]; }
        }
        lat[lat_prefix[ri] + loc] = virtual_corner_value(v, own_root, R.depth, oc, qc) - v.iso;
    }
}

// ---- large subdivided leaves (lattice edge >= 16): bricks of 8^3 cells.
//
// Most corners of a large subdivided leaf lie far from the surface.  One block
// takes one brick (8^3 cells, 9^3 corners) at a time:
//   1. it gathers into shared memory every coefficient the brick's corners can
//      read: the 27 neighbours of the leaf and of each ancestor, and at every
//      virtual depth the window of cells around the brick's owner cells (real
//      nodes outside the leaf, 0 where there is none);
//   2. it bounds the brick's corner values: each term is x_n * B_x * B_y * B_z
//      with the single-precision basis values the evaluation uses, so the range
//      of a term over the corners that include it is an interval product, and
//      the rounding of the FMA chain is at most (K + 4) u sum|term| for K terms
//      (u = 2^-24); terms only some corners include get intervals widened to 0;
//   3. if the bound proves that every corner value has the same sign as
//      (value - iso), the brick is culled: none of its cells carries a triangle
//      and its corners are never read;
//   4. otherwise every corner is evaluated from the shared window in the order
//      of virtual_corner_value, so culling changes no value.
// Corners on the leaf's lower faces may be owned by a cell of another leaf of
// the same depth batch: those go through virtual_corner_value, and a brick with
// such a corner is never culled.
constexpr int BR = 8;              // brick edge (cells); corners per axis BR+1
constexpr int BR1 = BR + 1;
constexpr int BR_BLOCK = 128;
constexpr int BR_LEVELS = 16;      // depths 0..15
constexpr int BR_WEXT = BR + 3;    // window edge at the finest depth
// window cells over all virtual depths of a brick whose first corner is a
// multiple of 8: 11^3 + 7^3 + 5^3 + 12 * 4^3 = 2567
constexpr int BR_XW = 2600;

struct VBrick {
    int root;                      // index into roots
    int bu, bv, bw;
};
struct BrickIndex {                // bricks of the large roots, numbered root by root
    const int* big;                // root indices of the large roots
    const i64* prefix;             // first brick of each large root
    int nbig;
};
__device__ __forceinline__ VBrick brick_of(const VArgs& v, const BrickIndex& bx, i64 g) {
    int lo = 0, hi = bx.nbig - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (bx.prefix[mid] <= g) lo = mid; else hi = mid - 1;
    }
    VBrick b;
    b.root = bx.big[lo];
    const int nb = (1 << (v.e.D - v.roots[b.root].depth)) / BR;
    const i64 l = g - bx.prefix[lo];
    b.bu = (int)(l / ((i64)nb * nb));
    b.bv = (int)((l / nb) % nb);
    b.bw = (int)(l % nb);
    return b;
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
    const int an = nd.neigh[(i64)(9 * (dx + 1) + 3 * (dy + 1) + (dz + 1)) * nd.M + L];
    if (an == -1) return -1;
    return descend(nd, an, r, d, N);
}

// interval of x * X * Y * Z (X, Y, Z intervals), in double
__device__ __forceinline__ void term_interval(double x, const float* lo, const float* hi, double& tlo, double& thi) {
    double a = x, b = x;
    for (int ax = 0; ax < 3; ++ax) {
        const double c0 = a * lo[ax], c1 = a * hi[ax], c2 = b * lo[ax], c3 = b * hi[ax];
        a = fmin(fmin(c0, c1), fmin(c2, c3));
        b = fmax(fmax(c0, c1), fmax(c2, c3));
    }
    tlo = a;
    thi = b;
}

struct BrickShared {
    float xL[BR_LEVELS * 27];                 // neighbours of the leaf and its ancestors (0: none)
    float Bt[BR_LEVELS * 9 * BR1];            // [depth][axis][t][k]: basis value of owner cell + t - 1 at corner k
    float Xw[BR_XW];                          // window coefficients, virtual depths
    float Wlo[BR_LEVELS * 3 * BR_WEXT];       // per window coordinate: basis range over the corners using it
    float Whi[BR_LEVELS * 3 * BR_WEXT];
    int wlo[BR_LEVELS][3];                    // window origin (cell coordinates at that depth)
    int wext[BR_LEVELS][3];
    int woff[BR_LEVELS];                      // offset into Xw, -1 when no corner reaches outside the leaf
    double red[4][BR_BLOCK / 32];
    int foreign;                              // a lower-face corner is owned by another leaf
    int cull;
};

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

// value of corner k (brick-local kk[], global qc[]) owned by the brick's leaf
// through owner cell oc[], from the shared window; 'interior' means oc = qc - 1
// so the tabulated basis values apply
__device__ __forceinline__ float brick_corner(const BrickShared& sm, const EvalArgs& a, int r, const int Lc[3],
                                              const int oc[3], const int qc[3], const int kk[3], bool interior) {
    const int D = a.D;
    const float inv = 1.0f / (float)(1 << D);
    float val = 0.f;
    for (int d = D; d > r; --d) {
        const int off = sm.woff[d];
        if (off < 0) continue;
        const int sh = D - d, span = 1 << (d - r);
        const int V[3] = {oc[0] >> sh, oc[1] >> sh, oc[2] >> sh};
        bool inner = true;
        for (int ax = 0; ax < 3; ++ax) {
            const int lo = Lc[ax] * span;
            if (V[ax] - 1 < lo || V[ax] + 1 >= lo + span) inner = false;
        }
        if (inner) continue;
        float bv[3][3];
        if (interior) {
            for (int ax = 0; ax < 3; ++ax)
                for (int t = 0; t < 3; ++t) bv[ax][t] = sm.Bt[((d * 3 + ax) * 3 + t) * BR1 + kk[ax]];
        } else {
            const int fb = (1 << d) - 1, lim = 1 << d;
            for (int ax = 0; ax < 3; ++ax)
                for (int t = 0; t < 3; ++t) {
                    const int cc = V[ax] + t - 1;
                    bv[ax][t] = (cc >= 0 && cc < lim) ? cpoly_value<3>(a.basis[fb + cc], (float)qc[ax] * inv) : 0.f;
                }
        }
        const int e1 = sm.wext[d][1], e2 = sm.wext[d][2];
        const int b0 = V[0] - 1 - sm.wlo[d][0], b1 = V[1] - 1 - sm.wlo[d][1], b2 = V[2] - 1 - sm.wlo[d][2];
        const int s2 = d - r;
        for (int j = 0; j < 27; ++j) {
            const int jx = j / 9, jy = (j / 3) % 3, jz = j % 3;
            if (((V[0] + jx - 1) >> s2) == Lc[0] && ((V[1] + jy - 1) >> s2) == Lc[1] && ((V[2] + jz - 1) >> s2) == Lc[2])
                continue;                                     // inside the subdivided leaf: no coefficient
            const float xn = sm.Xw[off + ((b0 + jx) * e1 + (b1 + jy)) * e2 + (b2 + jz)];
            val = fmaf(xn * bv[0][jx] * bv[1][jy], bv[2][jz], val);
        }
    }
    // the leaf itself and its real ancestors (walk_up with absent neighbours as 0)
    for (int l = r; l >= 0; --l) {
        const float* xs = sm.xL + 27 * l;
        const float* bx = sm.Bt + ((l * 3 + 0) * 3) * BR1 + kk[0];
        const float* by = sm.Bt + ((l * 3 + 1) * 3) * BR1 + kk[1];
        const float* bz = sm.Bt + ((l * 3 + 2) * 3) * BR1 + kk[2];
#pragma unroll
        for (int j = 0; j < 27; ++j)
            val = fmaf(xs[j] * bx[(j / 9) * BR1] * by[((j / 3) % 3) * BR1], bz[(j % 3) * BR1], val);
    }
    return val;
}

// one brick at a time per block, taken from a work counter
__global__ void __launch_bounds__(BR_BLOCK) k_bricks(VArgs v, BrickIndex bix, i64 nbricks,
                                                     unsigned long long* __restrict__ work,
                                                     unsigned long long* __restrict__ live,
                                                     unsigned char* __restrict__ culled,
                                                     const i64* __restrict__ lat_prefix, float* __restrict__ lat,
                                                     int* __restrict__ err) {
    __shared__ BrickShared sm;
    __shared__ long long sh_bi;
    const EvalArgs& a = v.e;
    const NodeArrays& nd = a.nd;
    const int D = a.D;
    const float inv = 1.0f / (float)(1 << D);
    const double u = 5.9604644775390625e-08;   // 2^-24
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) sh_bi = (long long)atomicAdd(work, 1ull);
        __syncthreads();
        const i64 bi = sh_bi;
        if (bi >= nbricks) break;
        const VBrick B = brick_of(v, bix, bi);
        const VRoot R = v.roots[B.root];
        const int r = R.depth, S = 1 << (D - r), S1 = S + 1, L = R.node;
        int Lc[3];
        key_coords(nd.key[L], r, D, Lc);
        const int c0[3] = {B.bu * BR, B.bv * BR, B.bw * BR};
        const int g0[3] = {Lc[0] * S + c0[0], Lc[1] * S + c0[1], Lc[2] * S + c0[2]};   // first corner (global)
        const bool lower = (B.bu == 0 || B.bv == 0 || B.bw == 0);
        // ---- 1. window layout, leaf coefficients, basis table
        if (threadIdx.x == 0) {
            int off = 0;
            for (int d = r + 1; d <= D; ++d) {
                const int sh = D - d, span = 1 << (d - r);
                bool inner = true;
                for (int ax = 0; ax < 3; ++ax) {
                    const int Vlo = (g0[ax] - 1) >> sh, Vhi = (g0[ax] + BR - 1) >> sh;
                    const int llo = Lc[ax] * span;
                    if (Vlo - 1 < llo || Vhi + 1 >= llo + span) inner = false;
                    sm.wlo[d][ax] = Vlo - 1;
                    sm.wext[d][ax] = Vhi - Vlo + 3;
                }
                if (inner) {
                    sm.woff[d] = -1;
                } else {
                    sm.woff[d] = off;
                    off += sm.wext[d][0] * sm.wext[d][1] * sm.wext[d][2];
                }
            }
            sm.foreign = 0;
            sm.cull = 0;
            if (off > BR_XW) {                        // cannot happen for 8-aligned bricks
                atomicExch(err, 1);
                for (int d = r + 1; d <= D; ++d) sm.woff[d] = -2;
            }
        }
        if ((int)threadIdx.x <= r) {
            int node = L;
            for (int l = r; l > (int)threadIdx.x; --l) node = nd.parent[node];
            for (int j = 0; j < 27; ++j) sm.xL[27 * threadIdx.x + j] = x_or_zero(a, nd.neigh[(i64)j * nd.M + node]);
        }
        for (int e = threadIdx.x; e < (D + 1) * 9 * BR1; e += blockDim.x) {
            const int k = e % BR1, t = (e / BR1) % 3, ax = (e / (3 * BR1)) % 3, d = e / (9 * BR1);
            const int uu = c0[ax] + k;
            int cidx;
            if (d <= r) cidx = (Lc[ax] >> (r - d)) + t - 1;
            else cidx = ((Lc[ax] * S + uu - 1) >> (D - d)) + t - 1;
            float val = 0.f;
            if (cidx >= 0 && cidx < (1 << d))
                val = cpoly_value<3>(a.basis[(1 << d) - 1 + cidx], (float)(Lc[ax] * S + uu) * inv);
            sm.Bt[((d * 3 + ax) * 3 + t) * BR1 + k] = val;
        }
        __syncthreads();
        if (sm.woff[D] == -2) continue;              // layout overflow (reported through err)
        // ---- 2a. basis ranges per window coordinate: corners k whose owner cell is within 1 of it
        for (int e = threadIdx.x; e < (D - r) * 3 * BR_WEXT; e += blockDim.x) {
            const int n = e % BR_WEXT, ax = (e / BR_WEXT) % 3, d = r + 1 + e / (3 * BR_WEXT);
            if (sm.woff[d] < 0 || n >= sm.wext[d][ax]) continue;
            const int sh = D - d, lim = 1 << d;
            const int N = sm.wlo[d][ax] + n;
            float mn = 0.f, mx = 0.f;                 // 0: corners without this term
            if (N >= 0 && N < lim) {
                for (int k = 0; k <= BR; ++k) {
                    const int Va = (g0[ax] + k - 1) >> sh;
                    const int Vb = (k == 0 && c0[ax] == 0) ? (g0[ax] >> sh) : Va;   // lower-face owner cell
                    if (N < Va - 1 || N > Vb + 1) continue;
                    const float b = cpoly_value<3>(a.basis[lim - 1 + N], (float)(g0[ax] + k) * inv);
                    mn = fminf(mn, b);
                    mx = fmaxf(mx, b);
                }
            }
            sm.Wlo[(d * 3 + ax) * BR_WEXT + n] = mn;
            sm.Whi[(d * 3 + ax) * BR_WEXT + n] = mx;
        }
        __syncthreads();
        // ---- 2b. window coefficients and the bound
        double lo = 0, hi = 0, amax = 0, cnt = 0;
        for (int t = threadIdx.x; t < 27 * (r + 1); t += blockDim.x) {
            const int l = r - t / 27, j = t % 27;
            const float x = sm.xL[27 * l + j];
            if (x == 0.f) continue;
            const int tt[3] = {j / 9, (j / 3) % 3, j % 3};
            float blo[3], bhi[3];
            for (int ax = 0; ax < 3; ++ax) {
                const float* row = sm.Bt + ((l * 3 + ax) * 3 + tt[ax]) * BR1;
                float mn = row[0], mx = row[0];
                for (int k = 1; k <= BR; ++k) { mn = fminf(mn, row[k]); mx = fmaxf(mx, row[k]); }
                blo[ax] = mn;
                bhi[ax] = mx;
            }
            double tl, th;
            term_interval((double)x, blo, bhi, tl, th);
            lo += tl; hi += th;
            amax += fmax(fabs(tl), fabs(th));
            cnt += 1;
        }
        for (int d = r + 1; d <= D; ++d) {
            const int off = sm.woff[d];
            if (off < 0) continue;
            const int e0 = sm.wext[d][0], e1 = sm.wext[d][1], e2 = sm.wext[d][2];
            for (int t = threadIdx.x; t < e0 * e1 * e2; t += blockDim.x) {
                const int n[3] = {t / (e1 * e2), (t / e2) % e1, t % e2};
                const int N[3] = {sm.wlo[d][0] + n[0], sm.wlo[d][1] + n[1], sm.wlo[d][2] + n[2]};
                const i64 node = shell_node(v, L, r, Lc, d, N);
                const float x = node < 0 ? 0.f : a.x[node];
                sm.Xw[off + t] = x;
                if (node < 0) continue;
                float blo[3], bhi[3];
                for (int ax = 0; ax < 3; ++ax) {
                    blo[ax] = sm.Wlo[(d * 3 + ax) * BR_WEXT + n[ax]];
                    bhi[ax] = sm.Whi[(d * 3 + ax) * BR_WEXT + n[ax]];
                }
                double tl, th;
                term_interval((double)x, blo, bhi, tl, th);
                lo += tl; hi += th;
                amax += fmax(fabs(tl), fabs(th));
                cnt += 1;
            }
        }
        // lower-face corners owned by another leaf of the batch
        if (lower && r >= 3) {
            for (int e = threadIdx.x; e < BR1 * BR1 * BR1; e += blockDim.x) {
                const int kk[3] = {e / (BR1 * BR1), (e / BR1) % BR1, e % BR1};
                const int uu = c0[0] + kk[0], ww = c0[1] + kk[1], zz = c0[2] + kk[2];
                if (!(uu == 0 || ww == 0 || zz == 0)) continue;
                const int qc[3] = {Lc[0] * S + uu, Lc[1] * S + ww, Lc[2] * S + zz};
                int oc[3];
                if (lower_face_owner(v, R, Lc, qc, oc) != L) atomicOr(&sm.foreign, 1);
            }
        }
        {
            double vals[4] = {lo, hi, amax, cnt};
            for (int k = 0; k < 4; ++k) {
                double x = vals[k];
                for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                if ((threadIdx.x & 31) == 0) sm.red[k][threadIdx.x >> 5] = x;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double sum[4] = {0, 0, 0, 0};
            for (int k = 0; k < 4; ++k)
                for (int w = 0; w < BR_BLOCK / 32; ++w) sum[k] += sm.red[k][w];
            const double iso = (double)v.iso;
            const double margin = (sum[3] + 4.0) * u * sum[2] + 2.0 * u * (fabs(sum[0]) + fabs(sum[1]) + 2.0 * fabs(iso)) +
                                  1e-12 * (sum[2] + fabs(iso));
            const bool above = sum[0] - margin > iso, below = sum[1] + margin < iso;
            sm.cull = (!sm.foreign && (above || below)) ? 1 : 0;
            culled[bi] = (unsigned char)sm.cull;
            if (!sm.cull) atomicAdd(live, 1ull);
        }
        __syncthreads();
        if (sm.cull) continue;
        // ---- 4. exact corner values
        float* out = lat + lat_prefix[B.root];
        for (int e = threadIdx.x; e < BR1 * BR1 * BR1; e += blockDim.x) {
            const int kk[3] = {e / (BR1 * BR1), (e / BR1) % BR1, e % BR1};
            const int uu = c0[0] + kk[0], ww = c0[1] + kk[1], zz = c0[2] + kk[2];
            const int qc[3] = {Lc[0] * S + uu, Lc[1] * S + ww, Lc[2] * S + zz};
            float val;
            if (uu && ww && zz) {
                const int oc[3] = {qc[0] - 1, qc[1] - 1, qc[2] - 1};
                val = brick_corner(sm, a, r, Lc, oc, qc, kk, true);
            } else {
                int oc[3] = {0, 0, 0};
                const int own = lower_face_owner(v, R, Lc, qc, oc);
                val = (own == L) ? brick_corner(sm, a, r, Lc, oc, qc, kk, false)
                                 : virtual_corner_value(v, own, r, oc, qc);
            }
            out[((i64)uu * S1 + ww) * S1 + zz] = val - v.iso;
        }
    }
}

__global__ void k_virtual_cells(VArgs v, const i64* __restrict__ cell_prefix, const i64* __restrict__ lat_prefix,
                                i64 total, const float* __restrict__ lat, const unsigned char* __restrict__ culled,
                                unsigned char* __restrict__ cat, int* __restrict__ ntri) {
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        int lo = 0, hi = v.nroots - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (cell_prefix[mid] <= e) lo = mid; else hi = mid - 1;
        }
        const VRoot R = v.roots[lo];
        const int S = 1 << (v.e.D - R.depth), S1 = S + 1;
        const i64 loc = e - cell_prefix[lo];
        const int u = (int)(loc / ((i64)S * S)), w = (int)((loc / S) % S), z = (int)(loc % S);
        if (R.brick_base >= 0) {
            const int nb = S / BR;
            if (culled[R.brick_base + ((i64)(u / BR) * nb + (w / BR)) * nb + (z / BR)]) {
                cat[e] = 0;
                ntri[e] = 0;
                continue;
            }
        }
        const float* L = lat + lat_prefix[lo];
        int cc = 0;
        for (int kind = 0; kind < 8; ++kind) {
            const i64 idx = ((i64)(u + (kind & 1)) * S1 + (w + ((kind >> 1) & 1))) * S1 + (z + ((kind >> 2) & 1));
            if (L[idx] < 0.f) cc |= 1 << c_vid[kind];
        }
        cat[e] = (unsigned char)cc;
        ntri[e] = c_tri_count[cc];
    }
}

// ---------------------------- triangle emission ------------------------------
struct EmitArgs {
    int D;
    int local_bits;
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

__global__ void k_emit_virtual(VArgs v, EmitArgs em, const i64* __restrict__ cell_prefix,
                               const i64* __restrict__ lat_prefix, const i64* __restrict__ active, i64 nactive,
                               const unsigned char* __restrict__ cat, const i64* __restrict__ tri_base,
                               const float* __restrict__ lat) {
    const int D = em.D;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < nactive; t += (i64)gridDim.x * blockDim.x) {
        const i64 e = active[t];
        int lo = 0, hi = v.nroots - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (cell_prefix[mid] <= e) lo = mid; else hi = mid - 1;
        }
        const VRoot R = v.roots[lo];
        const int S = 1 << (D - R.depth), S1 = S + 1;
        const i64 loc = e - cell_prefix[lo];
        const int u = (int)(loc / ((i64)S * S)), w = (int)((loc / S) % S), z = (int)(loc % S);
        int Lc[3];
        key_coords(v.e.nd.key[R.node], R.depth, D, Lc);
        const int c[3] = {Lc[0] * S + u, Lc[1] * S + w, Lc[2] * S + z};
        const float* L = lat + lat_prefix[lo];
        float cv[8];
        for (int kind = 0; kind < 8; ++kind)
            cv[kind] = L[((i64)(u + (kind & 1)) * S1 + (w + ((kind >> 1) & 1))) * S1 + (z + ((kind >> 2) & 1))];
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
            em.keys[slot] = edge_key(lp, o, D, R.batch, em.local_bits);
            em.slot[slot] = (uint32_t)slot;
            em.pos[3 * slot] = p[0];
            em.pos[3 * slot + 1] = p[1];
            em.pos[3 * slot + 2] = p[2];
        }
    }
}

// after sorting: vertex id per sorted element, positions of the first element
__global__ void k_vertex_ids(const u64* __restrict__ keys, const uint32_t* __restrict__ slot, i64 n,
                             const int* __restrict__ pos_scan, const float* __restrict__ epos,
                             int32_t* __restrict__ tri_vid, float* __restrict__ vpos) {
    for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
        const bool head = (k == 0) || keys[k] != keys[k - 1];
        const int vid = pos_scan[k] + (head ? 1 : 0) - 1;
        tri_vid[slot[k]] = vid;
        if (head) {
            const uint32_t sl = slot[k];
            vpos[3 * (i64)vid] = epos[3 * (i64)sl];
            vpos[3 * (i64)vid + 1] = epos[3 * (i64)sl + 1];
            vpos[3 * (i64)vid + 2] = epos[3 * (i64)sl + 2];
        }
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
    if (!g_mc_uploaded) upload_mc_tables();
    cudaStream_t s = c.stream;
    const int D = c.D;
    const NodeArrays& nd = c.nodes;
    const i64 M = nd.M, lo = c.base[D], nD = c.count[D];
    EvalArgs ea{c.nodes, D, c.basis, c.x};
    // ---- finest corner values, categories
    float* cval = dalloc<float>(8 * nD, s);
    float* cell_v = dalloc<float>(8 * nD, s);
    unsigned char* cat = dalloc<unsigned char>(nD, s);
    int* ntri = dalloc<int>(nD, s);
    int kt = c.kbegin("corner_values", (double)M * (108 + 8 + 4 + 4) + (double)nD * 8 * 4);
    k_finest_corner_values<<<grid_for(nD, 128, 1ll << 30), 128, 0, s>>>(ea, lo, M, c.iso, cval);
    CK_LAUNCH();
    c.kend(kt);
    kt = c.kbegin("cells", (double)nD * (8 * 4 + 108 + 8 * 4 + 1 + 4));
    k_finest_cells<<<grid_for(nD, 128, 1ll << 30), 128, 0, s>>>(nd, lo, M, cval, cell_v, cat, ntri);
    CK_LAUNCH();
    c.kend(kt);
    dfree(cval, s);
    // ---- face marks and subdivision roots
    int* fflag = dalloc<int>(6 * M, s);
    CK(cudaMemsetAsync(fflag, 0, (size_t)(6 * M) * sizeof(int), s));
    k_mark_faces<<<grid_for(nD, 128, 1ll << 30), 128, 0, s>>>(nd, D, lo, M, cat, fflag);
    CK_LAUNCH();
    const i64 nCoarse = lo;   // nodes at depth < D
    int* has_tri = dalloc<int>(nCoarse, s);
    int* has_int = dalloc<int>(nCoarse, s);
    int* is_root = dalloc<int>(nCoarse, s);
    CK(cudaMemsetAsync(has_tri, 0, nCoarse * sizeof(int), s));
    CK(cudaMemsetAsync(has_int, 0, nCoarse * sizeof(int), s));
    CK(cudaMemsetAsync(is_root, 0, nCoarse * sizeof(int), s));
    if (nCoarse > 1) {
        const int kc = c.kbegin("coarse_leaves", (double)nCoarse * (4 + 108 + 8 + 3 * 4) + (double)M * 4);
        k_coarse_leaves<<<grid_for(nCoarse - 1, 128, 1ll << 30), 128, 0, s>>>(ea, 1, nCoarse, c.iso, fflag, has_tri,
                                                                             has_int, is_root);
        CK_LAUNCH();
        c.kend(kc);
    }
    dfree(fflag, s);
    c.has_tri.assign(nCoarse, 0);
    c.has_int.assign(nCoarse, 0);
    std::vector<int> hroot(nCoarse, 0);
    CK(cudaMemcpyAsync(c.has_tri.data(), has_tri, nCoarse * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(c.has_int.data(), has_int, nCoarse * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hroot.data(), is_root, nCoarse * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    dfree(has_tri, s); dfree(has_int, s); dfree(is_root, s);
    // roots in node order; batches: one per root above depth 3, one per depth from 3
    std::vector<VRoot> roots;
    std::vector<int> bflag_host;   // filled lazily below
    std::vector<int> depth_of(nCoarse, 0);
    {
        std::vector<int8_t> hd(nCoarse);
        CK(cudaMemcpyAsync(hd.data(), nd.depth, nCoarse * sizeof(int8_t), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        for (i64 i = 0; i < nCoarse; ++i) depth_of[i] = hd[i];
    }
    int nb = 0;
    std::vector<int> depth_batch(D + 1, 0);
    for (i64 i = 0; i < nCoarse; ++i) {
        if (!hroot[i]) continue;
        VRoot R;
        R.node = (int)i;
        R.depth = depth_of[i];
        R.pad = 0;
        if (R.depth < 3) R.batch = ++nb;
        else {
            if (!depth_batch[R.depth]) depth_batch[R.depth] = ++nb;
            R.batch = depth_batch[R.depth];
        }
        roots.push_back(R);
    }
    c.subdivide_roots = (i64)roots.size();
    c.roots_per_depth.assign(D + 1, 0);
    for (auto& R : roots) c.roots_per_depth[R.depth]++;
    const int nbatches = nb + 1;
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
    // ---- virtual cells
    i64 ntri_virt = 0, nact_virt = 0, total_cells = 0, total_lat = 0;
    c.total_bricks = 0;
    c.live_bricks = 0;
    VRoot* droots = nullptr;
    i64 *cell_prefix = nullptr, *lat_prefix = nullptr, *act_virt = nullptr, *tri_virt = nullptr;
    float* lat = nullptr;
    unsigned char* vcat = nullptr;
    unsigned char* culled = nullptr;
    int* vntri = nullptr;
    int* bflag = nullptr;
    VArgs va;
    va.e = ea;
    va.iso = c.iso;
    va.nroots = (int)roots.size();
    if (!roots.empty()) {
        std::vector<i64> hcp(roots.size()), hlp(roots.size());
        i64 brick_run = 0;
        for (size_t k = 0; k < roots.size(); ++k) {
            const i64 S = 1ll << (D - roots[k].depth);
            hcp[k] = total_cells;
            hlp[k] = total_lat;
            roots[k].cell_base = total_cells;
            roots[k].lattice_base = total_lat;
            roots[k].brick_base = (S > BR) ? brick_run : -1;
            if (S > BR) brick_run += (S / BR) * (S / BR) * (S / BR);
            total_cells += S * S * S;
            total_lat += (S + 1) * (S + 1) * (S + 1);
        }
        bflag_host.assign(M, 0);
        for (auto& R : roots) if (R.depth >= 3) bflag_host[R.node] = R.batch;
        droots = dalloc<VRoot>((i64)roots.size(), s);
        cell_prefix = dalloc<i64>((i64)roots.size(), s);
        lat_prefix = dalloc<i64>((i64)roots.size(), s);
        bflag = dalloc<int>(M, s);
        CK(cudaMemcpyAsync(droots, roots.data(), roots.size() * sizeof(VRoot), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(cell_prefix, hcp.data(), hcp.size() * sizeof(i64), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(lat_prefix, hlp.data(), hlp.size() * sizeof(i64), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(bflag, bflag_host.data(), M * sizeof(int), cudaMemcpyHostToDevice, s));
        va.roots = droots;
        va.batch_root_flag = bflag;
        lat = dalloc<float>(total_lat, s);
        // small leaves (lattice edge <= 8): one thread per corner; large ones: 8^3-cell bricks
        std::vector<int> small_list, big_list;
        std::vector<i64> small_prefix, brick_prefix;
        i64 small_total = 0, nbricks = 0;
        for (size_t k = 0; k < roots.size(); ++k) {
            const int S = 1 << (D - roots[k].depth);
            if (S <= BR) {
                small_list.push_back((int)k);
                small_prefix.push_back(small_total);
                small_total += (i64)(S + 1) * (S + 1) * (S + 1);
            } else {
                big_list.push_back((int)k);
                brick_prefix.push_back(nbricks);
                nbricks += (i64)(S / BR) * (S / BR) * (S / BR);
            }
        }
        if (small_total > 0) {
            const int kvs = c.kbegin("virtual_small", (double)small_total * 4);
            int* dlist = dalloc<int>((i64)small_list.size(), s);
            i64* dpre = dalloc<i64>((i64)small_prefix.size(), s);
            CK(cudaMemcpyAsync(dlist, small_list.data(), small_list.size() * sizeof(int), cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dpre, small_prefix.data(), small_prefix.size() * sizeof(i64), cudaMemcpyHostToDevice, s));
            k_virtual_corners<<<grid_for(small_total, 128, 1ll << 30), 128, 0, s>>>(
                va, dlist, dpre, (int)small_list.size(), small_total, lat_prefix, lat);
            CK_LAUNCH();
            c.kend(kvs);
            dfree(dlist, s);
            dfree(dpre, s);
        }
        culled = dalloc<unsigned char>(std::max<i64>(nbricks, 1), s);
        if (nbricks > 0) {
            int* dbig = dalloc<int>((i64)big_list.size(), s);
            i64* dbpre = dalloc<i64>((i64)brick_prefix.size(), s);
            CK(cudaMemcpyAsync(dbig, big_list.data(), big_list.size() * sizeof(int), cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dbpre, brick_prefix.data(), brick_prefix.size() * sizeof(i64), cudaMemcpyHostToDevice, s));
            BrickIndex bix{dbig, dbpre, (int)big_list.size()};
            // work counter, live-brick count, layout error flag
            unsigned long long* wk = dalloc<unsigned long long>(3, s);
            CK(cudaMemsetAsync(wk, 0, 3 * sizeof(unsigned long long), s));
            int per_sm = 0;
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bricks, BR_BLOCK, 0));
            const i64 grid = std::min<i64>(nbricks, (i64)c.sms * std::max(per_sm, 1));
            // compulsory: the brick's lattice corners written once
            const int kb = c.kbegin("bricks", (double)nbricks * BR1 * BR1 * BR1 * 4);
            k_bricks<<<(unsigned)grid, BR_BLOCK, 0, s>>>(va, bix, nbricks, wk, wk + 1, culled, lat_prefix, lat,
                                                          (int*)(wk + 2));
            CK_LAUNCH();
            c.kend(kb);
            unsigned long long hw[3];
            CK(cudaMemcpyAsync(hw, wk, sizeof hw, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            dfree(wk, s);
            c.live_bricks = (i64)hw[1];
            if (hw[2]) {
                set_last_error("brick window layout overflow");
                throw Error{PRGPU_ERR_LIMIT, {0}};
            }
            c.total_bricks = nbricks;
            dfree(dbig, s);
            dfree(dbpre, s);
        }
        vcat = dalloc<unsigned char>(total_cells, s);
        vntri = dalloc<int>(total_cells, s);
        const int kc2 = c.kbegin("virtual_cells", (double)total_lat * 4 + (double)total_cells * 5);
        k_virtual_cells<<<grid_for(total_cells, 256, 1ll << 30), 256, 0, s>>>(va, cell_prefix, lat_prefix, total_cells,
                                                                              lat, culled, vcat, vntri);
        CK_LAUNCH();
        c.kend(kc2);
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
    while ((1 << batch_bits) < nbatches) ++batch_bits;
    c.mesh_v.clear();
    c.mesh_f.clear();
    c.batch_tri.assign(1, ntri_real);
    c.batch_tri.push_back(ntri_virt);
    if (nem > 0) {
        EmitArgs em;
        em.D = D;
        em.local_bits = local_bits;
        em.tri_offset = 0;
        em.keys = dalloc<u64>(nem, s);
        em.slot = dalloc<uint32_t>(nem, s);
        em.pos = dalloc<float>(3 * nem, s);
        if (nact_real > 0) {
            k_emit_real<<<grid_for(nact_real, 128, 1ll << 30), 128, 0, s>>>(nd, em, lo, act_real, nact_real, cat,
                                                                            tri_real, cell_v);
            CK_LAUNCH();
        }
        if (nact_virt > 0) {
            EmitArgs ev = em;
            ev.tri_offset = ntri_real;
            k_emit_virtual<<<grid_for(nact_virt, 128, 1ll << 30), 128, 0, s>>>(va, ev, cell_prefix, lat_prefix, act_virt,
                                                                               nact_virt, vcat, tri_virt, lat);
            CK_LAUNCH();
        }
        u64* ktmp = dalloc<u64>(nem, s);
        uint32_t* stmp = dalloc<uint32_t>(nem, s);
        const int ks = c.kbegin("edge_sort", (double)nem * 12 * 2);
        radix_sort_pairs(em.keys, em.slot, ktmp, stmp, nem, local_bits + batch_bits, s);
        c.kend(ks);
        dfree(ktmp, s);
        dfree(stmp, s);
        int* hf = dalloc<int>(nem, s);
        int* hp = dalloc<int>(nem + 1, s);
        k_key_heads<<<grid_for(nem, 256), 256, 0, s>>>(em.keys, nem, hf);
        CK_LAUNCH();
        exclusive_scan<int, int>(hf, hp, nem, hp + nem, s);
        const i64 nvert = read_scalar(hp + nem, s);
        int32_t* tri_vid = dalloc<int32_t>(nem, s);
        float* vpos = dalloc<float>(3 * std::max<i64>(nvert, 1), s);
        k_vertex_ids<<<grid_for(nem, 256), 256, 0, s>>>(em.keys, em.slot, nem, hp, em.pos, tri_vid, vpos);
        CK_LAUNCH();
        c.mesh_v.resize(3 * nvert);
        c.mesh_f.resize(nem);
        CK(cudaMemcpyAsync(c.mesh_v.data(), vpos, 3 * nvert * sizeof(float), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(c.mesh_f.data(), tri_vid, nem * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        dfree(hf, s); dfree(hp, s); dfree(tri_vid, s); dfree(vpos, s);
        dfree(em.keys, s); dfree(em.slot, s); dfree(em.pos, s);
    }
    dfree(act_real, s);
    dfree(tri_real, s);
    dfree(droots, s); dfree(cell_prefix, s); dfree(lat_prefix, s); dfree(act_virt, s); dfree(tri_virt, s);
    dfree(lat, s); dfree(vcat, s); dfree(vntri, s); dfree(bflag, s); dfree(culled, s);
    dfree(cell_v, s);
    dfree(cat, s);
    dfree(ntri, s);
    // input coordinates: p*scale + centre (PlyWriteTriangles plyfile.cu:2801-2812), unfused
    const i64 nv = (i64)c.mesh_v.size() / 3;
    for (i64 k = 0; k < nv; ++k)
        for (int a = 0; a < 3; ++a) {
            volatile float prod = c.mesh_v[3 * k + a] * c.scale;
            c.mesh_v[3 * k + a] = prod + c.center[a];
        }
}

}  // namespace prgpu
