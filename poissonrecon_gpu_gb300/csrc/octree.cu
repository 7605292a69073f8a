// Octree stage: normalisation, Morton keys, radix sort, level-by-level node
// arrays and 27-neighbour tables.  Replaces pipelineBuildNodeArray
// (main.cu:511-841) and the kernels it launches (main.cu:126-509).
//
// The node arrays are derived directly from the sorted leaf keys: at every
// depth the non-empty nodes are the runs of equal key prefixes, and each
// non-empty node owns one full group of 8 child slots one depth below.
// Parents, children, point ranges and finest-slot ranges follow from the run
// structure, so no hash table or atomic is needed and every field is exact
// (the reference's racy parent assignment, main.cu:331,357, is not reproduced:
// every slot receives its true parent).
#include <algorithm>
#include <cmath>
#include <vector>

#include "context.h"
#include "prims.cuh"

namespace prgpu {

// --------------------------- bounding box -----------------------------------
__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float ord2f(unsigned u) {
    unsigned b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, 4);
    return f;
#endif
}

__global__ void k_bbox(const float* __restrict__ xyz, i64 n, unsigned* __restrict__ mm) {
    unsigned mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0, 0, 0};
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            unsigned o = f2ord(xyz[3 * i + a]);
            mn[a] = min(mn[a], o);
            mx[a] = max(mx[a], o);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o; o >>= 1) {
            mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(&mm[a], mn[a]);
            atomicMax(&mm[3 + a], mx[a]);
        }
    }
}

// ----------------- normalisation + Morton key (main.cu:132-173,555-569) ------
__global__ void k_normalise_encode(const float* __restrict__ in_xyz, const float* __restrict__ in_nrm, i64 n,
                                   float cx, float cy, float cz, float scale, float nscale, int D,
                                   float* __restrict__ p_out, float* __restrict__ n_out, u64* __restrict__ keys,
                                   uint32_t* __restrict__ idx) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        float p[3] = {(in_xyz[3 * i] - cx) / scale, (in_xyz[3 * i + 1] - cy) / scale, (in_xyz[3 * i + 2] - cz) / scale};
        float nx = in_nrm[3 * i], ny = in_nrm[3 * i + 1], nz = in_nrm[3 * i + 2];
        float sq = nx * nx + ny * ny + nz * nz;   // unfused (--fmad=false), as on the reference host
        float len = (float)sqrt((double)sq);
        if (len > 1e-6f) len = 1.0f / len;
        len = len * nscale;
        p_out[3 * i] = p[0];
        p_out[3 * i + 1] = p[1];
        p_out[3 * i + 2] = p[2];
        n_out[3 * i] = nx * len;
        n_out[3 * i + 1] = ny * len;
        n_out[3 * i + 2] = nz * len;
        u64 key = 0;
        float mx = 0.5f, my = 0.5f, mz = 0.5f, w = 0.25f;
        for (int l = D - 1; l >= 0; --l) {
            if (p[0] > mx) { key |= 1ull << (3 * l + 2); mx += w; } else mx -= w;
            if (p[1] > my) { key |= 1ull << (3 * l + 1); my += w; } else my -= w;
            if (p[2] > mz) { key |= 1ull << (3 * l); mz += w; } else mz -= w;
            w *= 0.5f;
        }
        keys[i] = key;
        idx[i] = (uint32_t)i;
    }
}

__global__ void k_gather_points(const uint32_t* __restrict__ idx, i64 n, const float* __restrict__ p_in,
                                const float* __restrict__ n_in, float* __restrict__ p_out, float* __restrict__ n_out) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        i64 s = idx[i];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            p_out[3 * i + a] = p_in[3 * s + a];
            n_out[3 * i + a] = n_in[3 * s + a];
        }
    }
}

// ------------------------------- runs ---------------------------------------
// head flag of a run of equal masked keys
__global__ void k_head_flags(const u64* __restrict__ k, i64 n, u64 mask, int* __restrict__ f) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        f[i] = (i == 0 || ((k[i] & mask) != (k[i - 1] & mask))) ? 1 : 0;
}
// compacts run heads: unique key, first source index; every element learns its run rank
__global__ void k_runs(const u64* __restrict__ k, i64 n, u64 mask, const int* __restrict__ f,
                       const int* __restrict__ pos, u64* __restrict__ ukey, int* __restrict__ ufirst,
                       int* __restrict__ rank_of) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        int r = pos[i] + f[i] - 1;
        if (rank_of) rank_of[i] = r;
        if (f[i]) {
            ukey[r] = k[i] & mask;
            ufirst[r] = (int)i;
        }
    }
}
__global__ void k_iota(int* __restrict__ out, i64 n) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) out[i] = (int)i;
}
// first point of a unique node = first point of its first child run
__global__ void k_compose(const int* __restrict__ a, const int* __restrict__ b, i64 n, int* __restrict__ out) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) out[i] = a[b[i]];
}
// slot of each unique node inside its parent's group of 8, and the slot -> unique map
__global__ void k_unique_slots(const u64* __restrict__ ukey, const int* __restrict__ uparent, i64 nu, int shift,
                               int* __restrict__ uslot, int* __restrict__ slot2u) {
    for (i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x; r < nu; r += (i64)gridDim.x * blockDim.x) {
        int s = 8 * uparent[r] + (int)((ukey[r] >> shift) & 7);
        uslot[r] = s;
        slot2u[s] = (int)r;
    }
}

struct LevelArgs {
    int d, D;
    i64 base_prev, base_d, base_next;
    i64 n_slots;          // count[d]
    i64 N;                // points
    i64 u_d, u_dm1;       // unique nodes at d and d-1
    i64 u_last;           // unique nodes at depth D-1
};

// fills one depth of the node arrays (one thread per slot); the empty-slot
// conventions follow updateEmptyNodeInfo (main.cu:433-490)
__global__ void k_fill_level(LevelArgs a, const u64* __restrict__ ukey_prev, const int* __restrict__ uslot_prev,
                             const int* __restrict__ upidx_prev, const int* __restrict__ ulo_prev,
                             const int* __restrict__ upidx_d, const int* __restrict__ ulo_d,
                             const int* __restrict__ slot2u, NodeArrays nd) {
    for (i64 s = (i64)blockIdx.x * blockDim.x + threadIdx.x; s < a.n_slots; s += (i64)gridDim.x * blockDim.x) {
        const i64 g = s >> 3;
        const int k = (int)(s & 7);
        const i64 i = a.base_d + s;
        const int shift = 3 * (a.D - a.d);
        nd.key[i] = ukey_prev[g] | ((u64)k << shift);
        nd.depth[i] = (int8_t)a.d;
        nd.parent[i] = (int)(a.base_prev + uslot_prev[g]);
        // per-sibling point and finest-slot counts
        int ppre = 0, dpre = 0;
        int my_pnum = 0, my_dnum = 0;
        int r_self = -1;
        for (int q = 0; q < 8; ++q) {
            int r = slot2u[8 * g + q];
            int pn = 0, dn = 0;
            if (r >= 0) {
                i64 next_p = (r + 1 < a.u_d) ? upidx_d[r + 1] : a.N;
                pn = (int)(next_p - upidx_d[r]);
                if (a.d < a.D) {
                    i64 hi = (r + 1 < a.u_d) ? ulo_d[r + 1] : a.u_last;
                    dn = (int)(8 * (hi - ulo_d[r]));
                }
            }
            if (q < k) { ppre += pn; dpre += dn; }
            if (q == k) { my_pnum = pn; my_dnum = dn; r_self = r; }
        }
        nd.pnum[i] = my_pnum;
        nd.pidx[i] = upidx_prev[g] + ppre;
        if (a.d == a.D) {
            nd.didx[i] = (int)s;
            nd.dnum[i] = 1;
        } else {
            nd.dnum[i] = my_dnum;
            // parent's first finest slot: 8 * (rank of its first depth-(D-1) descendant)
            int pdidx = (a.d - 1 == a.D - 1) ? (int)(8 * g) : 8 * ulo_prev[g];
            nd.didx[i] = pdidx + dpre;
        }
        nd.child0[i] = (r_self >= 0 && a.d < a.D) ? (int)(a.base_next + 8 * (i64)r_self) : -1;
    }
}

__global__ void k_root(NodeArrays nd, i64 N, i64 countD, i64 M) {
    nd.key[0] = 0;
    nd.depth[0] = 0;
    nd.parent[0] = -1;
    nd.pidx[0] = 0;
    nd.pnum[0] = (int)N;
    nd.didx[0] = 0;
    nd.dnum[0] = (int)countD;
    nd.child0[0] = 1;
    for (int j = 0; j < 27; ++j) nd.neigh[(i64)j * M] = (j == 13) ? 0 : -1;
}

// computeNeighbor (main.cu:492-509): neighbour j of a node is a child of one of
// its parent's neighbours
// Neighbours of depth d from those of depth d-1 (main.cu:492-509): neighbour j of
// child s of P is child (s + off_j) & 1 of P's neighbour (s + off_j) >> 1 per axis,
// the values the reference's LUTs tabulate (main.cu:80-99).  The 8 children of a
// node are contiguous, so a warp takes 4 sibling groups: the first children of
// each parent's 27 neighbours are loaded once per group into shared memory, then
// every lane writes its node's 27 neighbours (coalesced along the nodes).
__global__ void __launch_bounds__(256) k_neighbours(NodeArrays nd, i64 lo, i64 ng) {
    __shared__ int cn[8][4][27];
    const i64 M = nd.M;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
    for (i64 tile = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile * 4 < ng; tile += nwarps) {
        for (int e = lane; e < 4 * 27; e += 32) {
            const i64 g = tile * 4 + e / 27;
            int v = -1;
            if (g < ng) {
                const int p = nd.parent[lo + 8 * g];
                const int np = nd.neigh[(i64)(e % 27) * M + p];
                if (np != -1) v = nd.child0[np];
            }
            cn[w][e / 27][e % 27] = v;
        }
        __syncwarp();
        const i64 g = tile * 4 + (lane >> 3);
        if (g < ng) {
            const int s = lane & 7, sx = s >> 2, sy = (s >> 1) & 1, sz = s & 1;
            const i64 i = lo + 8 * g + s;
#pragma unroll
            for (int j = 0; j < 27; ++j) {
                const int ax = sx + j / 9 - 1, ay = sy + (j / 3) % 3 - 1, az = sz + j % 3 - 1;
                const int jp = 9 * ((ax >> 1) + 1) + 3 * ((ay >> 1) + 1) + ((az >> 1) + 1);
                const int c0 = cn[w][lane >> 3][jp];
                nd.neigh[(i64)j * M + i] = c0 == -1 ? -1 : c0 + (((ax & 1) << 2) | ((ay & 1) << 1) | (az & 1));
            }
        }
        __syncwarp();
    }
}

__global__ void k_point_node(const int* __restrict__ leaf_rank, i64 n, const int* __restrict__ uslotD, i64 baseD,
                             int* __restrict__ point_node) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        point_node[i] = (int)(baseD + uslotD[leaf_rank[i]]);
}

void stage_octree(Ctx& c) {
    cudaStream_t s = c.stream;
    const int D = c.D;
    const i64 N = c.N;
    // ---- bounding box, scale and centre exactly as the reference host code
    unsigned* mm = dalloc<unsigned>(6, s);
    {
        unsigned init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0, 0, 0};
        CK(cudaMemcpyAsync(mm, init, sizeof init, cudaMemcpyHostToDevice, s));
        k_bbox<<<grid_for(N, 256, 152 * 8), 256, 0, s>>>(c.in_xyz, N, mm);
        CK_LAUNCH();
        unsigned h[6];
        CK(cudaMemcpyAsync(h, mm, sizeof h, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        float mn[3], mx[3];
        for (int a = 0; a < 3; ++a) { mn[a] = ord2f(h[a]); mx[a] = ord2f(h[3 + a]); }
        float scale = 1;
        for (int a = 0; a < 3; ++a) {
            if (!a || scale < mx[a] - mn[a]) scale = float(mx[a] - mn[a]);
            c.center[a] = float(mx[a] + mn[a]) / 2;
        }
        scale *= 1.25f;
        for (int a = 0; a < 3; ++a) c.center[a] -= scale / 2;
        c.scale = scale;
        if (!(scale > 0.f) || !std::isfinite(scale) || !std::isfinite(c.center[0]) || !std::isfinite(c.center[1]) ||
            !std::isfinite(c.center[2])) {
            dfree(mm, s);
            set_last_error("degenerate bounding box (all points coincide or are not finite)");
            throw Error{PRGPU_ERR_ARG, {0}};
        }
    }
    dfree(mm, s);
    // ---- normalise + keys, sort, gather
    float* ptmp = dalloc<float>(3 * N, s);
    float* ntmp = dalloc<float>(3 * N, s);
    u64* keys = dalloc<u64>(N, s);
    u64* ktmp = dalloc<u64>(N, s);
    uint32_t* idx = dalloc<uint32_t>(N, s);
    uint32_t* itmp = dalloc<uint32_t>(N, s);
    k_normalise_encode<<<grid_for(N, 256), 256, 0, s>>>(c.in_xyz, c.in_nrm, N, c.center[0], c.center[1], c.center[2],
                                                         c.scale, (float)(2 << D), D, ptmp, ntmp, keys, idx);
    CK_LAUNCH();
    const int ks = c.kbegin("point_sort", (double)N * 12 * 2);
    radix_sort_pairs(keys, idx, ktmp, itmp, N, 3 * D, s);
    c.kend(ks);
    dfree(ktmp, s);
    dfree(itmp, s);
    dfree(c.pts, s); dfree(c.nrm, s); dfree(c.sort_idx, s);
    c.pts = dalloc<float>(3 * N, s);
    c.nrm = dalloc<float>(3 * N, s);
    c.sort_idx = idx;
    k_gather_points<<<grid_for(N, 256), 256, 0, s>>>(idx, N, ptmp, ntmp, c.pts, c.nrm);
    CK_LAUNCH();
    dfree(ptmp, s);
    dfree(ntmp, s);

    // ---- unique nodes per depth
    std::vector<u64*> ukey(D + 1, nullptr);
    std::vector<int*> upidx(D + 1, nullptr), uparent(D + 1, nullptr), ufirstchild(D + 1, nullptr), ulo(D + 1, nullptr),
        uslot(D + 1, nullptr), slot2u(D + 1, nullptr);
    std::vector<i64> U(D + 1, 0);
    int* flags = dalloc<int>(N, s);
    int* pos = dalloc<int>(N + 1, s);
    int* leaf_rank = dalloc<int>(N, s);
    {
        k_head_flags<<<grid_for(N, 256), 256, 0, s>>>(keys, N, ~0ull, flags);
        CK_LAUNCH();
        exclusive_scan<int, int>(flags, pos, N, pos + N, s);
        U[D] = read_scalar(pos + N, s);
        ukey[D] = dalloc<u64>(U[D], s);
        upidx[D] = dalloc<int>(U[D], s);
        k_runs<<<grid_for(N, 256), 256, 0, s>>>(keys, N, ~0ull, flags, pos, ukey[D], upidx[D], leaf_rank);
        CK_LAUNCH();
    }
    for (int d = D - 1; d >= 0; --d) {
        const i64 n = U[d + 1];
        u64 mask = ~((1ull << (3 * (D - d))) - 1);
        k_head_flags<<<grid_for(n, 256), 256, 0, s>>>(ukey[d + 1], n, mask, flags);
        CK_LAUNCH();
        exclusive_scan<int, int>(flags, pos, n, pos + n, s);
        U[d] = read_scalar(pos + n, s);
        ukey[d] = dalloc<u64>(U[d], s);
        ufirstchild[d] = dalloc<int>(U[d], s);
        uparent[d + 1] = dalloc<int>(n, s);
        k_runs<<<grid_for(n, 256), 256, 0, s>>>(ukey[d + 1], n, mask, flags, pos, ukey[d], ufirstchild[d],
                                                 uparent[d + 1]);
        CK_LAUNCH();
        upidx[d] = dalloc<int>(U[d], s);
        k_compose<<<grid_for(U[d], 256), 256, 0, s>>>(upidx[d + 1], ufirstchild[d], U[d], upidx[d]);
        CK_LAUNCH();
    }
    dfree(flags, s);
    dfree(pos, s);
    // rank range of depth-(D-1) descendants: lo per unique node
    if (D >= 1) {
        ulo[D - 1] = dalloc<int>(U[D - 1], s);
        k_iota<<<grid_for(U[D - 1], 256), 256, 0, s>>>(ulo[D - 1], U[D - 1]);
        CK_LAUNCH();
        for (int d = D - 2; d >= 0; --d) {
            ulo[d] = dalloc<int>(U[d], s);
            k_compose<<<grid_for(U[d], 256), 256, 0, s>>>(ulo[d + 1], ufirstchild[d], U[d], ulo[d]);
            CK_LAUNCH();
        }
    }
    // ---- sizes
    c.count.assign(D + 1, 0);
    c.base.assign(D + 2, 0);
    c.count[0] = 1;
    for (int d = 1; d <= D; ++d) c.count[d] = 8 * U[d - 1];
    for (int d = 1; d <= D + 1; ++d) c.base[d] = c.base[d - 1] + c.count[d - 1];
    const i64 M = c.base[D + 1];
    if (M > 0x7fffffffLL) {
        set_last_error("node array of %lld nodes exceeds 32-bit indexing", (long long)M);
        throw Error{PRGPU_ERR_LIMIT, {0}};
    }
    c.free_nodes();
    NodeArrays& nd = c.nodes;
    nd.M = M;
    nd.key = dalloc<u64>(M, s);
    nd.pidx = dalloc<int>(M, s);
    nd.pnum = dalloc<int>(M, s);
    nd.didx = dalloc<int>(M, s);
    nd.dnum = dalloc<int>(M, s);
    nd.parent = dalloc<int>(M, s);
    nd.child0 = dalloc<int>(M, s);
    nd.depth = dalloc<int8_t>(M, s);
    nd.neigh = dalloc<int>(27 * M, s);
    // ---- slots of unique nodes
    uslot[0] = dalloc<int>(1, s);
    CK(cudaMemsetAsync(uslot[0], 0, sizeof(int), s));
    for (int d = 1; d <= D; ++d) {
        uslot[d] = dalloc<int>(U[d], s);
        slot2u[d] = dalloc<int>(c.count[d], s);
        fill<int>(slot2u[d], c.count[d], -1, s);
        k_unique_slots<<<grid_for(U[d], 256), 256, 0, s>>>(ukey[d], uparent[d], U[d], 3 * (D - d), uslot[d], slot2u[d]);
        CK_LAUNCH();
    }
    // ---- fill
    k_root<<<1, 1, 0, s>>>(nd, N, c.count[D], M);
    CK_LAUNCH();
    for (int d = 1; d <= D; ++d) {
        LevelArgs a;
        a.d = d; a.D = D;
        a.base_prev = c.base[d - 1]; a.base_d = c.base[d]; a.base_next = c.base[d + 1];
        a.n_slots = c.count[d]; a.N = N; a.u_d = U[d]; a.u_dm1 = U[d - 1];
        a.u_last = (D >= 1) ? U[D - 1] : 1;
        k_fill_level<<<grid_for(c.count[d], 256), 256, 0, s>>>(a, ukey[d - 1], uslot[d - 1], upidx[d - 1],
                                                                (d - 1 <= D - 2) ? ulo[d - 1] : nullptr, upidx[d],
                                                                (d <= D - 1) ? ulo[d] : nullptr, slot2u[d], nd);
        CK_LAUNCH();
    }
    // ---- neighbours, top-down
    const int kn = c.kbegin("neighbours", (double)M * (108 + 8 + 4 + 4));
    for (int d = 1; d <= D; ++d) {
        k_neighbours<<<grid_for(c.count[d] / 8 * 8, 256), 256, 0, s>>>(nd, c.base[d], c.count[d] / 8);
        CK_LAUNCH();
    }
    c.kend(kn);
    // ---- point -> leaf
    dfree(c.point_node, s);
    c.point_node = dalloc<int>(N, s);
    k_point_node<<<grid_for(N, 256), 256, 0, s>>>(leaf_rank, N, uslot[D], c.base[D], c.point_node);
    CK_LAUNCH();
    dfree(leaf_rank, s);
    dfree(keys, s);
    for (int d = 0; d <= D; ++d) {
        dfree(ukey[d], s); dfree(upidx[d], s); dfree(uparent[d], s); dfree(ufirstchild[d], s);
        dfree(ulo[d], s); dfree(uslot[d], s); dfree(slot2u[d], s);
    }
}

}  // namespace prgpu
