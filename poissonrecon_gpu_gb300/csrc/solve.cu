// Per-depth Laplacian solve.  Replaces LaplacianIteration (main.cu:1223-1332)
// and solverCG_DeviceToDevice / gpuConjugateGradient (CG_CUDA.cuh:186-509).
//
// The reference assembles a CSR matrix per depth and runs one cooperative CG
// kernel per depth, one depth after the other.  Here the matrix is never
// stored: same-depth inner products are translation invariant, so row i of L_d
// is the depth's 27 stencil coefficients applied through the node's neighbour
// table (the reference's |L_ij| <= 1e-6 drop rule is applied to the stencil).
// The depths are independent systems (each starts from x0 = 0 and never sees
// the others), so ONE persistent cooperative launch solves all of them at
// once: the co-resident blocks are partitioned between the depths in
// proportion to their row counts, and each partition runs its own CG with its
// own grid barrier.  Barriers spin with an iteration limit; on expiry the
// kernel records PRGPU_ERR_TIMEOUT and returns.
//
// Matrix-vector product by sibling groups: the 8 children of a node are
// contiguous, and their 27-neighbourhoods together form the 4x4x4 block of
// cells around them -- the children of the parent's 27 neighbours.  So the
// product reads, per group, the 27 first-child indices of the parent's
// neighbours (a table built once per solve, 13.5 bytes per row instead of the
// 108-byte neighbour rows) and the 64 values of r in the block, staged in
// shared memory.  A missing neighbour reads 0, and adding a zero product
// leaves the sum unchanged, so the product is the same as with the neighbour
// table.  The product is s = A r; the direction's product follows as
// q = A p = s + beta q_prev (p = r + beta p_prev), so each cell is gathered once
// per iteration (one vector) rather than forming p at every group that reads it.
#include <algorithm>
#include <cmath>
#include <vector>

#include "cg_common.cuh"
#include "context.h"
#include "prims.cuh"

namespace prgpu {


struct CgArgs {
    int ndepth;
    int mode;               // prgpu_solve_mode
    float tol2;             // reference mode: float(tol)*float(tol)
    double rel2;            // relative mode: tol^2
    int max_iter;
    i64 M;
    const int* neigh;       // 27 x M
    const int* gn;          // 27 x ngroups: first child of each neighbour of a sibling group's parent, or -1
    const int* gnr;         // the same, GN_ROW per group
    i64 ngroups;            // sibling groups (nodes 1..M-1, 8 per group)
    const float* b;
    float* x;
    float* r;
    float* p;               // search direction
    float* q;               // A p
    PartState* state;
    PartSync* sync;         // one per depth
    double* partial;        // one per block
    int* err;
    long long spin_limit;   // bounded waits (WaitLimits)
    int extra;
    int refine;             // relative mode: FP64 true-residual check and refinement
};

// barrier over the blocks of one partition; returns false after a timeout
__device__ bool part_barrier(PartState* ps, int nblocks, int* err, int* sh_ok, long long spin_limit, int extra) {
    __syncthreads();
    if (nblocks + extra > 1) {
        if (threadIdx.x == 0) {
            volatile unsigned* vgen = &ps->gen;
            unsigned g = *vgen;
            __threadfence();
            unsigned arrived = atomicAdd(&ps->count, 1u);
            int ok = 1;
            if (arrived == (unsigned)(nblocks + extra) - 1) {
                atomicExch(&ps->count, 0u);
                __threadfence();
                atomicAdd(&ps->gen, 1u);
            } else {
                long long spins = 0;
                while (*vgen == g) {
                    if (++spins > spin_limit || *(volatile int*)err) { ok = 0; break; }
                    __nanosleep(32);
                }
            }
            __threadfence();
            if (!ok) atomicExch(err, PRGPU_ERR_TIMEOUT);
            *sh_ok = ok && !*(volatile int*)err;
        }
    } else if (threadIdx.x == 0) {
        __threadfence_block();
        *sh_ok = 1;
    }
    __syncthreads();
    return *sh_ok != 0;
}

// sum of v over the blocks of a partition, returned to every thread: each block
// stores its partial, the last to arrive sums them all in a fixed order (so the
// result does not depend on arrival order) and releases the others.  Waits spin
// with a limit; on expiry the error flag is set and false returned.
__device__ double part_reduce(PartSync* ps, double* partial, int first_block, int nblocks, int slot, double v,
                              int* err, double* sh, int* sh_flag, double* sh_val, bool& ok, long long spin_limit,
                              int extra) {
    const double s = block_sum(v, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = s;
        __threadfence();
        const unsigned g = *(volatile unsigned*)&ps->gen;
        const unsigned arrived = atomicAdd(&ps->count, 1u);
        sh_flag[0] = (arrived == (unsigned)(nblocks + extra) - 1) ? 1 : 0;
        sh_flag[1] = (int)g;
    }
    __syncthreads();
    if (sh_flag[0]) {
        __threadfence();
        double t = 0.0;
        for (int k = threadIdx.x; k < nblocks; k += blockDim.x) t += *(volatile double*)&partial[first_block + k];
        t = block_sum(t, sh);
        if (threadIdx.x == 0) {
            ps->res[slot] = t;
            atomicExch(&ps->count, 0u);
            __threadfence();
            atomicAdd(&ps->gen, 1u);
            *sh_val = t;
            sh_flag[2] = 1;
        }
    } else if (threadIdx.x == 0) {
        const unsigned g = (unsigned)sh_flag[1];
        volatile unsigned* vgen = &ps->gen;
        long long spins = 0;
        int good = 1;
        while (*vgen == g) {
            if (++spins > spin_limit || *(volatile int*)err) { good = 0; break; }
            __nanosleep(64);
        }
        __threadfence();
        if (!good) atomicExch(err, PRGPU_ERR_TIMEOUT);
        *sh_val = *(volatile double*)&ps->res[slot];
        sh_flag[2] = good && !*(volatile int*)err;
    }
    __syncthreads();
    ok = sh_flag[2] != 0;
    return *sh_val;
}

// per sibling group: first child of each of the parent's 27 neighbours (-1: none or a leaf)
__global__ void k_group_table(NodeArrays nd, i64 ngroups, int* __restrict__ gn) {
    const i64 M = nd.M;
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < ngroups * 27; e += (i64)gridDim.x * blockDim.x) {
        const i64 g = e % ngroups;
        const int jp = (int)(e / ngroups);
        const int P = nd.parent[1 + 8 * g];
        const int pn = nd.neigh[(i64)jp * M + P];
        gn[e] = (pn == -1) ? -1 : nd.child0[pn];
    }
}

// the group table row by row (GN_ROW per group; the pad entry -1)
__global__ void k_group_rows(const int* __restrict__ gn, i64 ngroups, int* __restrict__ rows) {
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < ngroups * GN_ROW; e += (i64)gridDim.x * blockDim.x) {
        const i64 g = e / GN_ROW;
        const int jp = (int)(e % GN_ROW);
        rows[e] = (jp < 27) ? gn[(i64)jp * ngroups + g] : -1;
    }
}

constexpr int CG_TILE_GROUPS = CG_BLOCK / 8;   // sibling groups per tile, one thread per row
constexpr int CG_WARP_TILES = 2;               // tiles of 4 groups a warp stages at once

// 5 blocks per SM (48 registers): the partitions' warps wait on gathers and grid reductions, and
// 40 warps per SM hide more of that latency than 32 (measured: 2.41 -> 1.90 ms on the 1M-point
// torus at maxDepth 10; 6 blocks spill more and are slower again)
__global__ void __launch_bounds__(CG_BLOCK, 5) k_cg_all(CgArgs a, const CgDepth* __restrict__ deps,
                                                     const int* __restrict__ block_depth) {
    __shared__ float sp[(CG_BLOCK / 32) * CG_WARP_TILES * CG_TILE_WORDS];
    __shared__ int sgn[(CG_BLOCK / 32) * CG_WARP_TILES * 4 * GN_ROW];
    __shared__ float sst[27];
    __shared__ double sh[CG_BLOCK / 32];
    __shared__ double sh_val;
    const int d = block_depth[blockIdx.x];
    const CgDepth& dp = deps[d];
    if (threadIdx.x < 27) sst[threadIdx.x] = dp.st[threadIdx.x];
    const float cls[4] = {dp.cls[0], dp.cls[1], dp.cls[2], dp.cls[3]};
    __syncthreads();
    PartState* ps = &a.state[d];
    const int rank = blockIdx.x - dp.first_block;
    const i64 stride = (i64)dp.nblocks * blockDim.x;
    const i64 start = (i64)rank * blockDim.x + threadIdx.x;
    int red = 0;   // reduction counter selects the accumulator slot

    // reduce a per-thread double over the partition; every thread gets the sum
    __shared__ int sh_flag[3];
    auto preduce = [&](double v, bool& ok) -> double {
        const double res = part_reduce(&a.sync[d], a.partial, dp.first_block, dp.nblocks, red & 1, v, a.err, sh,
                                       sh_flag, &sh_val, ok, a.spin_limit, a.extra);
        ++red;
        return res;
    };

    // x = 0, r = b  (the host-side initialisation of CG_CUDA.cuh:435-439)
    FSum loc;
    for (i64 t = start; t < dp.n; t += stride) {
        const i64 i = dp.lo + t;
        const float bi = a.b[i];
        a.x[i] = 0.f;
        a.r[i] = bi;
        loc.add(bi * bi);
    }
    bool ok = true;
    const double bb = preduce(loc.value(), ok);   // ||b||^2 in double (relative mode)
    float r1 = (float)bb;
    float r0 = 0.f;
    int k = 1;
    int refines = 0;
    double rr_true = -1.0;
    bool restart = true;
    // The product gathers r only: s = A r, then q = A p = s + beta q and p = r + beta p
    // are formed row by row by the row's own thread (in place: no other thread reads a
    // row's p or q during the pass)
    while (ok) {
        const bool go = (a.mode == PRGPU_SOLVE_REFERENCE) ? (r1 > a.tol2) : ((double)r1 > a.rel2 * bb);
        if (!go || k > a.max_iter) {
            if (!a.refine || a.mode != PRGPU_SOLVE_RELATIVE || k > a.max_iter) break;
            // the recurrence says converged: recompute r = b - A x with FP64 accumulation
            double tsum = 0.0;
            for (i64 t = start; t < dp.n; t += stride) {
                const i64 i = dp.lo + t;
                double acc = (double)a.b[i];
#pragma unroll
                for (int j = 0; j < 27; ++j) {
                    const int nb = a.neigh[(i64)j * a.M + i];
                    if (nb != -1) acc = fma(-(double)sst[j], (double)a.x[nb], acc);
                }
                a.r[i] = (float)acc;
                tsum = fma(acc, acc, tsum);
            }
            rr_true = preduce(tsum, ok);
            if (!ok || rr_true <= a.rel2 * bb || refines >= 2) break;
            // restart CG from the current x on the true residual
            ++refines;
            r1 = (float)rr_true;
            restart = true;
            continue;
        }
        const bool first = restart;
        restart = false;
        const float beta = first ? 0.f : r1 / r0;
        // own row i with s_i = (A r)_i: p_i = r_i + beta p_i, q_i = s_i + beta q_i; partial p.q
        auto own_row = [&](i64 i, float ri, float si) {
            float pi = ri, qi = si;
            if (!first) {
                pi = fmaf(beta, a.p[i], ri);
                qi = fmaf(beta, a.q[i], si);
            }
            a.p[i] = pi;
            a.q[i] = qi;
            loc.add(pi * qi);
        };
        loc = FSum();
        if (d == 0) {
            for (i64 t = start; t < dp.n; t += stride) {
                const i64 i = dp.lo + t;
                float o = 0.f;
#pragma unroll
                for (int j = 0; j < 27; ++j) {
                    const int nb = a.neigh[(i64)j * a.M + i];
                    if (nb != -1 && sst[j] != 0.f) o = fmaf(sst[j], a.r[nb], o);
                }
                own_row(i, a.r[i], o);
            }
        } else {
            // one warp per CG_WARP_TILES tiles of 4 groups (32 rows each); warps run independently.
            // The tiles' group-table rows are one contiguous run, read coalesced into shared
            // memory; then every lane has 2 * CG_WARP_TILES * 8 independent gathers in flight.
            const i64 gfirst = (dp.lo - 1) >> 3, ng = dp.n >> 3;
            const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
            const int ch = lane & 7, gl = lane >> 3;
            const int sx = (ch >> 2) & 1, sy = (ch >> 1) & 1, sz = ch & 1;
            float* wsp = sp + wib * (CG_WARP_TILES * CG_TILE_WORDS);
            int* wgn = sgn + wib * (CG_WARP_TILES * 4 * GN_ROW);
            const i64 wstride = (i64)dp.nblocks * (CG_BLOCK / 32) * CG_WARP_TILES;
            for (i64 tile = ((i64)rank * (CG_BLOCK / 32) + wib) * CG_WARP_TILES; tile * 4 < ng; tile += wstride) {
                __syncwarp();
                {
                    const i64 row0 = (gfirst + tile * 4) * GN_ROW;
                    const i64 nvalid = min((i64)CG_WARP_TILES * 4, ng - tile * 4) * GN_ROW;
#pragma unroll
                    for (int k = 0; k < (CG_WARP_TILES * 4 * GN_ROW + 31) / 32; ++k) {
                        const int idx = lane + 32 * k;
                        if (idx < CG_WARP_TILES * 4 * GN_ROW) wgn[idx] = (idx < nvalid) ? a.gnr[row0 + idx] : -1;
                    }
                }
                __syncwarp();
                // the 4x4x4 block of each group: cell (bx,by,bz) is child ((bx+1)&1, ...) of the
                // parent's neighbour ((bx+1)>>1, ...) in 0..2 per axis
                int cn[CG_WARP_TILES * 8];
#pragma unroll
                for (int m = 0; m < CG_WARP_TILES * 8; ++m) {
                    const int e = lane + 32 * m;
                    const int cell = e & 63, bx = cell >> 4, by = (cell >> 2) & 3, bz = cell & 3;
                    const int jp = 9 * ((bx + 1) >> 1) + 3 * ((by + 1) >> 1) + ((bz + 1) >> 1);
                    cn[m] = wgn[(e >> 6) * GN_ROW + jp];
                }
#pragma unroll
                for (int m = 0; m < CG_WARP_TILES * 8; ++m) {
                    const int e = lane + 32 * m;
                    const int cell = e & 63, bx = cell >> 4, by = (cell >> 2) & 3, bz = cell & 3;
                    wsp[(e >> 8) * CG_TILE_WORDS + cg_block_base((e >> 6) & 3) + cell] = (cn[m] != -1)
                                 ? a.r[cn[m] + ((((bx + 1) & 1) << 2) | (((by + 1) & 1) << 1) | ((bz + 1) & 1))]
                                 : 0.f;
                }
                __syncwarp();
#pragma unroll
                for (int tt = 0; tt < CG_WARP_TILES; ++tt) {
                    const i64 g = (tile + tt) * 4 + gl;
                    if (g < ng) {
                        const float* blk = wsp + tt * CG_TILE_WORDS + cg_block_base(gl);
                        float o = 0.f;
                        if (dp.sym) {
#pragma unroll
                            for (int j = 0; j < 27; ++j)
                                o = fmaf(cls[stencil_class(j)],
                                         blk[(sx + j / 9) * 16 + (sy + (j / 3) % 3) * 4 + (sz + j % 3)], o);
                        } else {
#pragma unroll
                            for (int j = 0; j < 27; ++j)
                                o = fmaf(sst[j], blk[(sx + j / 9) * 16 + (sy + (j / 3) % 3) * 4 + (sz + j % 3)], o);
                        }
                        own_row(dp.lo + 8 * g + ch, blk[(sx + 1) * 16 + (sy + 1) * 4 + (sz + 1)], o);
                    }
                }
            }
        }
        const double pq = preduce(loc.value(), ok);
        if (!ok) break;
        const float al = (float)((double)r1 / pq);
        const float nal = -al;
        loc = FSum();
        {
            // four rows per thread per step, loads first (independent requests in flight)
            i64 t = start;
            for (; t + 3 * stride < dp.n; t += 4 * stride) {
                float pv[4], qv[4], xv[4], rv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const i64 i = dp.lo + t + u * stride;
                    pv[u] = a.p[i]; qv[u] = a.q[i]; xv[u] = a.x[i]; rv[u] = a.r[i];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const i64 i = dp.lo + t + u * stride;
                    a.x[i] = fmaf(al, pv[u], xv[u]);
                    const float ri = fmaf(nal, qv[u], rv[u]);
                    a.r[i] = ri;
                    loc.add(ri * ri);
                }
            }
            for (; t < dp.n; t += stride) {
                const i64 i = dp.lo + t;
                a.x[i] = fmaf(al, a.p[i], a.x[i]);
                const float ri = fmaf(nal, a.q[i], a.r[i]);
                a.r[i] = ri;
                loc.add(ri * ri);
            }
        }
        r0 = r1;
        r1 = (float)preduce(loc.value(), ok);
        ++k;
    }
    if (rank == 0 && threadIdx.x == 0) {
        ps->iters = k - 1;
        ps->rr = r1;
        ps->bb = bb;
        ps->rr_true = rr_true;
        ps->refines = refines;
        ps->status = ok ? 0 : PRGPU_ERR_TIMEOUT;
    }
}

// the group table row by row, built once per octree
void ensure_group_rows(Ctx& c) {
    if (c.gn_rows) return;
    ensure_group_table(c);
    const i64 ngroups = (c.nodes.M - 1) / 8;
    c.gn_rows = dalloc<int>(std::max<i64>(ngroups * GN_ROW, 1), c.stream);
    if (ngroups > 0) {
        k_group_rows<<<grid_for(ngroups * GN_ROW, 256), 256, 0, c.stream>>>(c.gn, ngroups, c.gn_rows);
        CK_LAUNCH();
    }
}

// the sibling-group table of the current octree, built once
void ensure_group_table(Ctx& c) {
    if (c.gn) return;
    const i64 ngroups = (c.nodes.M - 1) / 8;
    c.gn = dalloc<int>(std::max<i64>(ngroups * 27, 1), c.stream);
    if (ngroups > 0) {
        k_group_table<<<grid_for(ngroups * 27, 256), 256, 0, c.stream>>>(c.nodes, ngroups, c.gn);
        CK_LAUNCH();
    }
}

// ---------------------------------------------------------------------------
// Cascadic solve (params.cascadic; not the reference's): the depths are solved
// coarse to fine and depth d's right-hand side first loses the coarser depths'
// solution,
//   b'_i = b_i - sum_{e < d} sum_{j in N27(ancestor_e(i))} <grad B_i, grad B_j> x_j,
// the coarser nodes being the 27 neighbours of i's ancestor at each depth e (the
// truncation the reference's divergence uses).  The 3-D inner product has the
// same-depth stencil's form, dd_x t_y t_z + t_x dd_y t_z + t_x t_y dd_z, over
// the cross-depth 1-D tables (k_cascade_tables), so the sum over the 3x3x3
// neighbours factors axis by axis (z, then y, then x): 90 FP64 operations per
// ancestor instead of 27 x 11.  In double, with explicit fma, in this order:
//   zt[ox][oy] = fma(t_z0, X[ox][oy][0], fma(t_z1, X[ox][oy][1], t_z2 * X[ox][oy][2])), zd likewise
//   ytt = sum_oy t_y zt, ydt = sum_oy dd_y zt, ytd = sum_oy t_y zd   (the same nesting)
//   acc = fma(dd_x[ox], ytt, fma(t_x[ox], ydt + ytd, acc))          for ox = 0, 1, 2
// for e = 0.., X = x of the neighbour (0 where it is missing), read from a double
// copy of x.  One thread per node of depth d.
// ---------------------------------------------------------------------------
constexpr int CASCADE_MAX_DEPTH = 16;
// prgpu_create accepts maxDepth 2..15, so the per-ancestor arrays below always fit
static_assert(PRGPU_MAX_DEPTH < CASCADE_MAX_DEPTH, "the cascadic arrays need a slot per depth below maxDepth");

struct CascadeArgs {
    int d, D;
    i64 lo, n, M;
    const u64* key;
    const int* parent;
    const int* neigh;       // 27 x M
    const double2* tab;
    i64 off[CASCADE_MAX_DEPTH];   // start of the (d, e) table, e < d
    const double* xd;       // x in double, rows of the depths < d
    const float* b;
    float* rhs;
};

__device__ __forceinline__ double dot3(double a0, double a1, double a2, double x0, double x1, double x2) {
    return fma(a0, x0, fma(a1, x1, a2 * x2));
}

__global__ void __launch_bounds__(128) k_cascade_rhs(CascadeArgs a) {
    const int d = a.d, sh0 = 3 * (a.D - d);
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < a.n; t += (i64)gridDim.x * blockDim.x) {
        const i64 i = a.lo + t;
        const u64 key = a.key[i] >> sh0;
        int p[3] = {0, 0, 0};
        for (int l = d - 1; l >= 0; --l) {
            p[0] = (p[0] << 1) | (int)((key >> (3 * l + 2)) & 1);
            p[1] = (p[1] << 1) | (int)((key >> (3 * l + 1)) & 1);
            p[2] = (p[2] << 1) | (int)((key >> (3 * l)) & 1);
        }
        int anc[CASCADE_MAX_DEPTH];
        int q = (int)i;
        for (int e = d - 1; e >= 0; --e) {
            q = a.parent[q];
            anc[e] = q;
        }
        double acc = 0.0;
        for (int e = 0; e < d; ++e) {
            const int k = d - e;
            const int mask = (1 << k) - 1;
            const double2* T = a.tab + a.off[e];
            double tv[3][3], dv[3][3];
#pragma unroll
            for (int ax = 0; ax < 3; ++ax)
#pragma unroll
                for (int o = 0; o < 3; ++o) {
                    const double2 v = T[((i64)o << k) + (p[ax] & mask)];
                    tv[ax][o] = v.x;
                    dv[ax][o] = v.y;
                }
            const int A = anc[e];
#pragma unroll
            for (int ox = 0; ox < 3; ++ox) {
                double zt[3], zd[3];
#pragma unroll
                for (int oy = 0; oy < 3; ++oy) {
                    double X[3];
#pragma unroll
                    for (int oz = 0; oz < 3; ++oz) {
                        const int nb = a.neigh[(i64)(9 * ox + 3 * oy + oz) * a.M + A];
                        X[oz] = nb >= 0 ? a.xd[nb] : 0.0;
                    }
                    zt[oy] = dot3(tv[2][0], tv[2][1], tv[2][2], X[0], X[1], X[2]);
                    zd[oy] = dot3(dv[2][0], dv[2][1], dv[2][2], X[0], X[1], X[2]);
                }
                const double ytt = dot3(tv[1][0], tv[1][1], tv[1][2], zt[0], zt[1], zt[2]);
                const double ydt = dot3(dv[1][0], dv[1][1], dv[1][2], zt[0], zt[1], zt[2]);
                const double ytd = dot3(tv[1][0], tv[1][1], tv[1][2], zd[0], zd[1], zd[2]);
                acc = fma(dv[0][ox], ytt, fma(tv[0][ox], ydt + ytd, acc));
            }
        }
        a.rhs[i] = (float)((double)a.b[i] - acc);
    }
}

__global__ void k_rows_to_double(const float* __restrict__ x, i64 n, double* __restrict__ xd) {
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (i64)gridDim.x * blockDim.x)
        xd[t] = (double)x[t];
}

// depth d's rows of rhs: the divergence less the coarser depths' current solution
void cascade_rhs(Ctx& c, int d, float* rhs) {
    cudaStream_t s = c.stream;
    const i64 lo = c.base[d], n = c.count[d];
    if (n == 0) return;
    if (d == 0) {
        CK(cudaMemcpyAsync(rhs + lo, c.divergence + lo, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        return;
    }
    if (c.D >= CASCADE_MAX_DEPTH) {
        set_last_error("cascadic solve supports maxDepth < %d", CASCADE_MAX_DEPTH);
        throw Error{PRGPU_ERR_LIMIT, {0}};
    }
    ensure_cascade_tables(c);
    // the coarser rows of x in double (rows base[0] .. base[d])
    const i64 nc = c.base[d];
    double* xd = dalloc<double>(nc, s);
    k_rows_to_double<<<grid_for(nc, 256), 256, 0, s>>>(c.x, nc, xd);
    CK_LAUNCH();
    CascadeArgs a;
    a.d = d;
    a.D = c.D;
    a.lo = lo;
    a.n = n;
    a.M = c.nodes.M;
    a.key = c.nodes.key;
    a.parent = c.nodes.parent;
    a.neigh = c.nodes.neigh;
    a.tab = c.cascade_tab;
    for (int e = 0; e < CASCADE_MAX_DEPTH; ++e) a.off[e] = e < d ? c.cascade_off[(size_t)d * (c.D + 1) + e] : 0;
    a.xd = xd;
    a.b = c.divergence;
    a.rhs = rhs;
    // compulsory: key, parent, b and rhs of each node; the coarser depths' neighbour rows and x
    // (double)
    double bytes = (double)n * 20;
    for (int e = 0; e < d; ++e) bytes += (double)c.count[e] * (27 * 4 + 8);
    const int kt = c.kbegin("cascade_rhs", bytes);
    k_cascade_rhs<<<grid_for(n, 128), 128, 0, s>>>(a);
    CK_LAUNCH();
    c.kend(kt);
    dfree(xd, s);
}

void stage_solve(Ctx& c) {
    if (c.params.learned) {
        stage_solve_learned(c);
        return;
    }
    if (!c.params.cascadic) {
        stage_solve_depths(c, 0, c.D, c.params.solve_mode);
        return;
    }
    cudaStream_t s = c.stream;
    const i64 M = c.nodes.M;
    if (!c.x || c.x_rows != M) {
        dfree(c.x, s);
        c.x = dalloc<float>(M, s);
        c.x_rows = M;
        CK(cudaMemsetAsync(c.x, 0, M * sizeof(float), s));
    }
    float* rhs = dalloc<float>(M, s);
    for (int d = 0; d <= c.D; ++d) {
        cascade_rhs(c, d, rhs);
        stage_solve_depths(c, d, d, c.params.solve_mode, rhs);
    }
    dfree(rhs, s);
}

// co-resident blocks split between the depths d0..d1: one block for a depth of at most
// 4*256 rows, the rest in proportion to the rows; the depths outside d0..d1 get none
void partition_depths(const Ctx& c, int d0, int d1, int G, std::vector<CgDepth>& deps, std::vector<int>& block_depth) {
    const int D = c.D;
    deps.assign(D + 1, CgDepth());
    std::vector<int> nb(D + 1, 0);
    i64 big_rows = 0;
    const i64 small_rows = 4 * CG_BLOCK;
    int fixed = 0;
    for (int d = d0; d <= d1; ++d) {
        nb[d] = 1;
        if (c.count[d] <= small_rows) ++fixed;
        else big_rows += c.count[d];
    }
    int avail = std::max(0, G - fixed);
    for (int d = d0; d <= d1; ++d) {
        if (c.count[d] > small_rows) {
            i64 want = (i64)((double)avail * (double)c.count[d] / (double)std::max<i64>(big_rows, 1));
            i64 cap = (c.count[d] + CG_BLOCK - 1) / CG_BLOCK;
            nb[d] = (int)std::max<i64>(1, std::min(want, cap));
        }
    }
    int total = 0;
    for (int d = 0; d <= D; ++d) total += nb[d];
    while (total > G) {   // trim the largest partitions
        int dm = (int)(std::max_element(nb.begin(), nb.end()) - nb.begin());
        if (nb[dm] <= 1) break;
        --nb[dm];
        --total;
    }
    if (total > G) {
        set_last_error("solver needs %d co-resident blocks, device offers %d", total, G);
        throw Error{PRGPU_ERR_LIMIT, {0}};
    }
    block_depth.clear();
    for (int d = 0; d <= D; ++d) {
        deps[d].lo = c.base[d];
        deps[d].n = c.count[d];
        deps[d].first_block = (int)block_depth.size();
        deps[d].nblocks = nb[d];
        for (int j = 0; j < 27; ++j) deps[d].st[j] = c.stencil[27 * d + j];
        deps[d].sym = 1;
        for (int j = 0; j < 27; ++j) {
            const int k = stencil_class(j);
            const float rep = c.stencil[27 * d + (k == 0 ? 13 : k == 1 ? 4 : k == 2 ? 1 : 0)];
            if (c.stencil[27 * d + j] != rep) deps[d].sym = 0;
            deps[d].cls[k] = rep;
        }
        for (int k = 0; k < nb[d]; ++k) block_depth.push_back(d);
    }
}

// depths d0..d1 with the given mode (right-hand side: rhs, or the divergence);
// the other depths' rows of x are left as they are
void stage_solve_depths(Ctx& c, int d0, int d1, int mode, const float* rhs) {
    cudaStream_t s = c.stream;
    const int D = c.D;
    const i64 M = c.nodes.M;
    if (d0 == 0 && d1 == D) {   // every row is written
        dfree(c.x, s);
        c.x = dalloc<float>(M, s);
        c.x_rows = M;
    } else if (!c.x || c.x_rows != M) {   // the other depths start at 0
        dfree(c.x, s);
        c.x = dalloc<float>(M, s);
        c.x_rows = M;
        CK(cudaMemsetAsync(c.x, 0, M * sizeof(float), s));
    }
    float* r = dalloc<float>(M, s);
    float* p = dalloc<float>(M, s);
    float* q = dalloc<float>(M, s);
    // sibling-group table for the matrix-vector products
    const i64 ngroups = (M - 1) / 8;
    ensure_group_rows(c);
    const int* gn = c.gn;
    // co-resident capacity
    int dev = c.device, sms = 0, per_sm = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_all, CG_BLOCK, 0));
    if (per_sm < 1) per_sm = 1;
    const int G = sms * per_sm;
    c.solver_blocks = G;
    std::vector<CgDepth> deps;
    std::vector<int> block_depth;
    partition_depths(c, d0, d1, G, deps, block_depth);
    CgDepth* ddeps = dalloc<CgDepth>(D + 1, s);
    int* dbd = dalloc<int>((i64)block_depth.size(), s);
    PartState* st = dalloc<PartState>(D + 1, s);
    PartSync* psync = dalloc<PartSync>(D + 1, s);
    double* partial = dalloc<double>((i64)block_depth.size(), s);
    CK(cudaMemsetAsync(psync, 0, (D + 1) * sizeof(PartSync), s));
    int* err = dalloc<int>(1, s);
    CK(cudaMemcpyAsync(ddeps, deps.data(), (D + 1) * sizeof(CgDepth), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dbd, block_depth.data(), block_depth.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(st, 0, (D + 1) * sizeof(PartState), s));
    CK(cudaMemsetAsync(err, 0, sizeof(int), s));
    CgArgs a;
    a.ndepth = D + 1;
    a.mode = mode;
    const float tolf = (float)c.params.cg_tol;
    a.tol2 = tolf * tolf;
    a.rel2 = c.params.cg_tol * c.params.cg_tol;
    a.max_iter = c.params.cg_max_iter;
    a.M = M;
    a.neigh = c.nodes.neigh;
    a.gn = gn;
    a.gnr = c.gn_rows;
    a.ngroups = ngroups;
    a.b = rhs ? rhs : c.divergence;
    a.x = c.x;
    a.r = r;
    a.p = p;
    a.q = q;
    a.state = st;
    a.sync = psync;
    a.partial = partial;
    a.err = err;
    const WaitLimits wl = wait_limits();
    a.spin_limit = wl.spin_limit;
    a.extra = wl.extra;
    a.refine = c.params.refine;
    void* kargs[] = {(void*)&a, (void*)&ddeps, (void*)&dbd};
    const int kt = c.kbegin("cg", 0.0);
    CK(cudaLaunchCooperativeKernel((void*)k_cg_all, dim3((unsigned)block_depth.size()), dim3(CG_BLOCK), kargs, 0, s));
    ++g_kernel_launches;
    c.kend(kt);
    std::vector<PartState> hs(D + 1);
    int herr = 0;
    CK(cudaMemcpyAsync(hs.data(), st, (D + 1) * sizeof(PartState), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if ((int)c.cg_iters.size() != D + 1 || (d0 == 0 && d1 == D)) {
        c.cg_iters.assign(D + 1, 0);
        c.cg_rr.assign(D + 1, 0.f);
    }
    c.cg_fallback.assign(D + 1, -1);
    c.cg_true_rel.resize(D + 1, 0.0);
    c.cg_fp64_rel.resize(D + 1, -1.0);
    c.cg_refines.resize(D + 1, 0);
    for (int d = d0; d <= d1; ++d) {
        c.cg_iters[d] = hs[d].iters;
        c.cg_rr[d] = hs[d].rr;
        c.cg_true_rel[d] = hs[d].bb > 0 ? std::sqrt((double)hs[d].rr / hs[d].bb) : 0.0;
        c.cg_fp64_rel[d] = (hs[d].rr_true >= 0 && hs[d].bb > 0) ? std::sqrt(hs[d].rr_true / hs[d].bb) : -1.0;
        c.cg_refines[d] = hs[d].refines;
    }
    if (kt >= 0) {
        // compulsory per row and iteration: the group table (27 indices per 8 rows); r read
        // once by the product, p and q read and written; then p/q/x/r read and x/r written
        // (11 words)
        double bytes = 0;
        for (int d = d0; d <= d1; ++d) bytes += (double)hs[d].iters * (double)c.count[d] * (13.5 + 11 * 4);
        c.kpending[kt].bytes = bytes;
    }
    dfree(r, s); dfree(p, s); dfree(q, s);
    dfree(ddeps, s); dfree(dbd, s); dfree(st, s); dfree(psync, s); dfree(partial, s); dfree(err, s);
    if (herr) {
        set_last_error("solver barrier timed out");
        throw Error{PRGPU_ERR_TIMEOUT, {0}};
    }
}

// ---------------------------------------------------------------------------
// CSR conjugate gradients with the reference's interface (CG_CUDA.cuh:344-509)
// ---------------------------------------------------------------------------
struct CsrArgs {
    int n;
    const int* rowptr;
    const int* col;
    const float* val;
    const float* b;
    float* x;
    float* r;
    float* p;
    float* q;
    float tol2;
    int max_iter;
    PartState* state;
    int* err;
    long long spin_limit;
    int extra;
};

__global__ void __launch_bounds__(CG_BLOCK) k_cg_csr(CsrArgs a) {
    __shared__ double sh[CG_BLOCK / 32];
    __shared__ int sh_ok;
    __shared__ double sh_val;
    PartState* ps = a.state;
    const int nblocks = gridDim.x;
    const i64 stride = (i64)gridDim.x * blockDim.x;
    const i64 start = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    int red = 0;
    auto preduce = [&](double v, bool& ok) -> double {
        double s = block_sum(v, sh);
        if (threadIdx.x == 0) atomicAdd(&ps->acc[red % 3], s);
        ok = part_barrier(ps, nblocks, a.err, &sh_ok, a.spin_limit, a.extra);
        if (threadIdx.x == 0) sh_val = *(volatile double*)&ps->acc[red % 3];
        __syncthreads();
        double res = sh_val;
        if (blockIdx.x == 0 && threadIdx.x == 0) ps->acc[(red + 2) % 3] = 0.0;
        ++red;
        return res;
    };
    double loc = 0;
    for (i64 i = start; i < a.n; i += stride) {
        a.x[i] = 0.f;
        a.r[i] = a.b[i];
        loc += (double)(a.b[i] * a.b[i]);
    }
    bool ok = true;
    float r1 = (float)preduce(loc, ok), r0 = 0.f;
    int k = 1;
    while (ok && r1 > a.tol2 && k <= a.max_iter) {
        if (k > 1) {
            const float beta = r1 / r0;
            for (i64 i = start; i < a.n; i += stride) a.p[i] = fmaf(beta, a.p[i], a.r[i]);
        } else {
            for (i64 i = start; i < a.n; i += stride) a.p[i] = a.r[i];
        }
        if (!part_barrier(ps, nblocks, a.err, &sh_ok, a.spin_limit, a.extra)) break;
        loc = 0;
        for (i64 i = start; i < a.n; i += stride) {
            float o = 0.f;
            for (int e = a.rowptr[i]; e < a.rowptr[i + 1]; ++e) o = fmaf(a.val[e], a.p[a.col[e]], o);
            a.q[i] = o;
            loc += (double)(a.p[i] * o);
        }
        const double pq = preduce(loc, ok);
        if (!ok) break;
        const float al = (float)((double)r1 / pq), nal = -al;
        loc = 0;
        for (i64 i = start; i < a.n; i += stride) {
            a.x[i] = fmaf(al, a.p[i], a.x[i]);
            const float ri = fmaf(nal, a.q[i], a.r[i]);
            a.r[i] = ri;
            loc += (double)(ri * ri);
        }
        r0 = r1;
        r1 = (float)preduce(loc, ok);
        ++k;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ps->iters = k - 1;
        ps->rr = r1;
    }
}

int cg_csr_impl(int n, const int* rowptr, const int* col, const float* val, const float* rhs, float* x, float tol,
                int max_iter, int* iters, float* ms) {
    cudaStream_t s = 0;
    int dev = 0, sms = 0, per_sm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_csr, CG_BLOCK, 0));
    i64 want = ((i64)n + CG_BLOCK - 1) / CG_BLOCK;
    int G = (int)std::max<i64>(1, std::min<i64>((i64)sms * std::max(per_sm, 1), want));
    float *r = nullptr, *p = nullptr, *q = nullptr;
    PartState* st = nullptr;
    int* err = nullptr;
    CK(cudaMalloc(&r, sizeof(float) * std::max(n, 1)));
    CK(cudaMalloc(&p, sizeof(float) * std::max(n, 1)));
    CK(cudaMalloc(&q, sizeof(float) * std::max(n, 1)));
    CK(cudaMalloc(&st, sizeof(PartState)));
    CK(cudaMalloc(&err, sizeof(int)));
    CK(cudaMemset(st, 0, sizeof(PartState)));
    CK(cudaMemset(err, 0, sizeof(int)));
    CsrArgs a;
    a.n = n; a.rowptr = rowptr; a.col = col; a.val = val; a.b = rhs; a.x = x; a.r = r; a.p = p; a.q = q;
    a.tol2 = tol * tol;
    a.max_iter = max_iter;
    a.state = st;
    a.err = err;
    const WaitLimits wl = wait_limits();
    a.spin_limit = wl.spin_limit;
    a.extra = wl.extra;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    void* kargs[] = {(void*)&a};
    CK(cudaEventRecord(e0, s));
    CK(cudaLaunchCooperativeKernel((void*)k_cg_csr, dim3(G), dim3(CG_BLOCK), kargs, 0, s));
    ++g_kernel_launches;
    CK(cudaEventRecord(e1, s));
    CK(cudaEventSynchronize(e1));
    float t = 0;
    CK(cudaEventElapsedTime(&t, e0, e1));
    PartState hs;
    int herr = 0;
    CK(cudaMemcpy(&hs, st, sizeof hs, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&herr, err, sizeof herr, cudaMemcpyDeviceToHost));
    cudaFree(r); cudaFree(p); cudaFree(q); cudaFree(st); cudaFree(err);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    if (iters) *iters = hs.iters;
    if (ms) *ms = t;
    if (herr) {
        set_last_error("CG barrier timed out");
        return PRGPU_ERR_TIMEOUT;
    }
    return hs.iters >= max_iter && hs.rr > a.tol2 ? PRGPU_ERR_NOT_CONVERGED : PRGPU_OK;
}

}  // namespace prgpu
