// Flexible CG with the learned preconditioner (params.learned = 1).  The
// reference solves every depth with plain CG (CG_CUDA.cuh:256-324, one depth
// after the other from main.cu:1237-1329); here, as in solve.cu, all depths run
// in one persistent cooperative launch whose blocks are partitioned between the
// depths, and each partition runs
//
//   r = b, z = M(r), p = z
//   repeat:  q = A p;  alpha = (r.z) / (p.q);  x += alpha p;  r' = r - alpha q
//            z' = M(r');  beta = z'.(r' - r) / (r.z)   (Polak-Ribiere: flexible CG,
//            correct for a preconditioner that changes from step to step)
//            p = z' + beta p
//
// until the same stopping rule as plain CG (||r|| <= tol ||b|| with FP64
// reductions, or float(r.r) <= tol^2).  M is the per-node network of learned.cu:
// z_i = s_i y(features_i) / L_d[centre].  Plain CG is the fallback: a depth
// switches to it for good (restarting from p = r) as soon as a learned step
// fails to reduce the residual norm, gives r.z <= 0, or produces a non-finite
// value.  Depth 0 (one row) always runs plain CG.
//
// One iteration has two grid-wide reductions, as plain CG: the preconditioner
// needs r' at the 27 neighbours of every row, and r'_j = r_j - alpha q_j can be
// formed from r and q, both complete after the p.q reduction, so z' is computed
// in the same pass as the x and r updates, and r'.r', z'.r' and z'.r are reduced
// together.  r is double-buffered (a row's old value is still read by its
// neighbours' preconditioner while it is updated).
//
// The preconditioner works on tiles of 128 rows = 16 sibling groups: the 4x4x4
// blocks of r' around each group are staged in shared memory through the group
// table (as the matrix-vector product does), each row's 64 features are written
// in the tensor-core operand layout, and one tile goes through the two MMAs
// (tcgen05, TMEM accumulators) of mlp_forward_tile.
#include <algorithm>
#include <cmath>
#include <vector>

#include "cg_common.cuh"
#include "context.h"
#include "learned.h"
#include "mlp.cuh"
#include "prims.cuh"

namespace prgpu {

struct FcgState {           // one per depth
    int iters;
    int fallback_at;        // iteration at which plain CG took over (-1: never)
    double rr;              // final r.r
    double bb;              // b.b
    int status;
    int refines;            // restarts on the FP64 true residual (params.refine)
    double rr_true;         // |b - Ax|^2 with FP64 accumulation (-1: not computed)
};

constexpr int FCG_NV = 3;

struct alignas(128) FcgSync {
    unsigned count;
    unsigned pad0[31];
    unsigned gen;
    unsigned pad1[31];
    double res[2][4];
    double pad2[8];
};

struct FcgArgs {
    int mode;
    float tol2;
    double rel2;
    int max_iter;
    i64 M;
    const int* neigh;       // 27 x M
    const int* gn;          // group table
    const int* gnr;         // the group table row by row (GN_ROW per group)
    i64 ngroups;
    const float* b;
    float* x;
    float* ra;              // residual, two buffers used alternately
    float* rb;
    float* z;
    float* p;               // search direction, two buffers used alternately
    float* q;
    FcgState* state;
    FcgSync* sync;          // one per depth
    double* partial;        // 4 per block
    int* err;
    long long spin_limit;
    int extra;
    MlpWeights wt;
    const float* cnorm;     // 27 per depth: L_d[j] / L_d[13]
    const float* centre;    // per depth: L_d[13]
    int refine;             // relative mode: FP64 true-residual check and refinement
};

// A kernel that allocates tensor memory runs one block per SM (the occupancy the
// driver grants such kernels), so the block is large: 768 threads, all of which
// share the gathers, the matrix-vector product and the reductions; for the
// preconditioner they form three groups of 256 threads, each with its own MLP
// tile stream, TMEM columns (128 of the block's 512), mbarrier and named barrier.
constexpr int FCG_GROUPS = 3;
constexpr int FCG_THREADS = 256 * FCG_GROUPS;
constexpr int FCG_WARPS = FCG_THREADS / 32;
constexpr int FCG_WARP_TILES = 2;
constexpr i64 FCG_MIN_ROWS = 256;
constexpr int FCG_DSMEM = 8192 + 8192 + FCG_GROUPS * 16384 + 1024;   // W1, W2, feature tiles (+ alignment)

// sum of FCG_NV doubles over the blocks of a partition, in a fixed order, returned
// to every thread; false when a wait gave up (error flag set)
__device__ bool fcg_reduce(FcgSync* ps, double* partial, int first_block, int nblocks, int slot,
                           double (&v)[FCG_NV], const FcgArgs& a, double* sh, int* sh_flag, double* sh_val) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int j = 0; j < FCG_NV; ++j) {
        double t = v[j];
        for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) sh[w * FCG_NV + j] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 0; j < FCG_NV; ++j) {
            double s = 0.0;
            for (int k = 0; k < nw; ++k) s += sh[k * FCG_NV + j];
            partial[(i64)blockIdx.x * 4 + j] = s;
        }
        __threadfence();
        const unsigned g = *(volatile unsigned*)&ps->gen;
        const unsigned arrived = atomicAdd(&ps->count, 1u);
        sh_flag[0] = (arrived == (unsigned)(nblocks + a.extra) - 1) ? 1 : 0;
        sh_flag[1] = (int)g;
    }
    __syncthreads();
    if (sh_flag[0]) {
        __threadfence();
        double t[FCG_NV] = {0.0, 0.0, 0.0};
        for (int k = threadIdx.x; k < nblocks; k += blockDim.x)
#pragma unroll
            for (int j = 0; j < FCG_NV; ++j) t[j] += *(volatile double*)&partial[(i64)(first_block + k) * 4 + j];
#pragma unroll
        for (int j = 0; j < FCG_NV; ++j) {
            for (int o = 16; o; o >>= 1) t[j] += __shfl_xor_sync(0xffffffffu, t[j], o);
            if (lane == 0) sh[w * FCG_NV + j] = t[j];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int j = 0; j < FCG_NV; ++j) {
                double s = 0.0;
                for (int k = 0; k < nw; ++k) s += sh[k * FCG_NV + j];
                ps->res[slot][j] = s;
                sh_val[j] = s;
            }
            atomicExch(&ps->count, 0u);
            __threadfence();
            atomicAdd(&ps->gen, 1u);
            sh_flag[2] = 1;
        }
    } else if (threadIdx.x == 0) {
        const unsigned g = (unsigned)sh_flag[1];
        volatile unsigned* vgen = &ps->gen;
        long long spins = 0;
        int good = 1;
        while (*vgen == g) {
            if (++spins > a.spin_limit || *(volatile int*)a.err) { good = 0; break; }
            __nanosleep(64);
        }
        __threadfence();
        if (!good) atomicExch(a.err, PRGPU_ERR_TIMEOUT);
        for (int j = 0; j < FCG_NV; ++j) sh_val[j] = *(volatile double*)&ps->res[slot][j];
        sh_flag[2] = good && !*(volatile int*)a.err;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < FCG_NV; ++j) v[j] = sh_val[j];
    return sh_flag[2] != 0;
}

__global__ void __launch_bounds__(FCG_THREADS, 1) k_fcg_all(FcgArgs a, const CgDepth* __restrict__ deps,
                                                          const int* __restrict__ block_depth) {
    extern __shared__ __align__(1024) uint8_t dsm[];
    uint8_t* sw1 = dsm;
    uint8_t* sw2 = dsm + 8192;
    __shared__ float sp[FCG_WARPS * FCG_WARP_TILES * CG_TILE_WORDS];   // product staging; r' blocks per group in phase B
    __shared__ float sst[27];
    __shared__ float scn[27];
    __shared__ float sb[192];
    __shared__ float red[FCG_GROUPS][256];
    __shared__ float ss[FCG_GROUPS][128];
    __shared__ double sh[FCG_WARPS * FCG_NV];
    __shared__ double sh_val[FCG_NV];
    __shared__ int sh_flag[3];
    __shared__ int gflag[FCG_GROUPS];
    __shared__ uint64_t bars[FCG_GROUPS];
    __shared__ uint32_t tslot;
    __shared__ int2 cellmap[64];   // per cell of a 4x4x4 block: (parent-neighbour j, child of it)
    __shared__ int sgn[FCG_WARPS * FCG_WARP_TILES * 4 * GN_ROW];   // group-table rows: per warp (product) or per group (features)
    const int d = block_depth[blockIdx.x];
    const CgDepth& dp = deps[d];
    const int grp = threadIdx.x >> 8, lt = threadIdx.x & 255, gbar = 1 + grp;
    if (threadIdx.x < 32) {
        tmem_alloc(&tslot, 512);
        tmem_relinquish();
    }
    if (threadIdx.x < FCG_GROUPS) {
        mbar_init(&bars[threadIdx.x], 1);
        gflag[threadIdx.x] = 0;
    }
    if (threadIdx.x == 0) mbar_fence_init();
    if (threadIdx.x < 27) {
        sst[threadIdx.x] = dp.st[threadIdx.x];
        scn[threadIdx.x] = a.cnorm[27 * d + threadIdx.x];
    }
    if (threadIdx.x < 64) {
        const int cell = threadIdx.x, bx = cell >> 4, by = (cell >> 2) & 3, bz = cell & 3;
        cellmap[cell] = make_int2(9 * ((bx + 1) >> 1) + 3 * ((by + 1) >> 1) + ((bz + 1) >> 1),
                                  (((bx + 1) & 1) << 2) | (((by + 1) & 1) << 1) | ((bz + 1) & 1));
    }
    MlpSmem m;
    stage_mlp_smem(a.wt, sw1, sw2, sb, m);
    uint8_t* sx = dsm + 16384 + grp * 16384;   // this group's feature / activation tile
    const float cls[4] = {dp.cls[0], dp.cls[1], dp.cls[2], dp.cls[3]};
    const float icen = 1.f / a.centre[d];
    const float dfeat = (float)d * (1.f / 16.f);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tslot + (uint32_t)(grp * 128);
    uint32_t phase = 0;
    FcgSync* psync = &a.sync[d];
    const int rank = blockIdx.x - dp.first_block;
    const i64 stride = (i64)dp.nblocks * blockDim.x;
    const i64 start = (i64)rank * blockDim.x + threadIdx.x;
    const i64 lo = dp.lo, n = dp.n;
    int red_n = 0;
    bool ok = true, mma_ok = true;
    auto reduce = [&](double (&v)[FCG_NV]) -> bool {
        const bool r = fcg_reduce(psync, a.partial, dp.first_block, dp.nblocks, red_n & 1, v, a, sh, sh_flag, sh_val);
        ++red_n;
        return r;
    };

    // x = 0, r = b
    double v[FCG_NV] = {0.0, 0.0, 0.0};
    {
        FSum loc;
        for (i64 t = start; t < n; t += stride) {
            const float bi = a.b[lo + t];
            a.x[lo + t] = 0.f;
            a.ra[lo + t] = bi;
            loc.add(bi * bi);
        }
        v[0] = loc.value();
    }
    ok = reduce(v);
    const double bb = v[0];
    float* rcur = a.ra;
    float* rnext = a.rb;
    // depths of fewer than FCG_MIN_ROWS rows (tiny systems plain CG solves in a few
    // iterations) and depth 0 run plain CG
    bool plain = (d == 0) || (n < FCG_MIN_ROWS);
    int fallback_at = -1;
    const i64 gfirst = (lo - 1) >> 3, ng = n >> 3;

    // phase B: x += alpha p, r' = r - alpha q, z' = M(r'), partial sums of r'.r', z'.r', z'.r
    auto phase_b = [&](bool init, float al, const float* pnew) -> bool {
        const float nal = -al;
        double acc[FCG_NV] = {0.0, 0.0, 0.0};
        bool gok = true;
        if (plain) {
            FSum s0;
            for (i64 t = start; t < n; t += stride) {
                const i64 i = lo + t;
                const float rc = rcur[i];
                float rn = rc;
                if (!init) {
                    a.x[i] = fmaf(al, pnew[i], a.x[i]);
                    rn = fmaf(nal, a.q[i], rc);
                    rnext[i] = rn;
                }
                s0.add(rn * rn);
            }
            acc[0] = s0.value();
            acc[1] = acc[0];
        } else {
            float* sv = sp + grp * 2048;                                     // 16 groups x 64 cells
            uint8_t* spr = reinterpret_cast<uint8_t*>(sv + 16 * 64);         // their presence, one byte each
            const i64 ntile = (n + 127) / 128;
            for (i64 tile = (i64)rank * FCG_GROUPS + grp; tile < ntile; tile += (i64)dp.nblocks * FCG_GROUPS) {
                // the row's own vectors, loaded before the staging gathers so that both are in flight
                const bool own = lt < 128 && tile * 128 + lt < n;
                const i64 iown = lo + tile * 128 + lt;
                float own_r = 0.f, own_q = 0.f, own_x = 0.f, own_p = 0.f;
                if (own) {
                    own_r = rcur[iown];
                    if (!init) {
                        own_q = a.q[iown];
                        own_x = a.x[iown];
                        own_p = pnew[iown];
                    }
                }
                // the tile's 16 group-table rows (one contiguous run) through shared memory, then
                // the four cells' values: 4 and 8 independent loads in flight per thread
                int* sg = sgn + grp * (16 * GN_ROW);
                {
                    const i64 row0 = (gfirst + tile * 16) * GN_ROW;
                    const i64 nvalid = min((i64)16, ng - tile * 16) * GN_ROW;
                    for (int k = lt; k < 16 * GN_ROW; k += 256) sg[k] = (k < nvalid) ? a.gnr[row0 + k] : -1;
                }
                group_sync(gbar);
                int cns[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int e = lt + 256 * u;
                    cns[u] = sg[(e >> 6) * GN_ROW + cellmap[e & 63].x];
                }
                float rv[4], qv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int e = lt + 256 * u;
                    rv[u] = qv[u] = 0.f;
                    if (cns[u] != -1) {
                        const i64 node = cns[u] + cellmap[e & 63].y;
                        rv[u] = rcur[node];
                        if (!init) qv[u] = a.q[node];
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int e = lt + 256 * u;
                    sv[e] = init ? rv[u] : fmaf(nal, qv[u], rv[u]);
                    spr[e] = (cns[u] != -1) ? 1 : 0;
                }
                group_sync(gbar);
                {
                    const int row = lt >> 1, h = lt & 1;
                    const int gl = row >> 3, ch = row & 7;
                    const int cx = (ch >> 2) & 1, cy = (ch >> 1) & 1, cz = ch & 1;
                    const bool valid = tile * 128 + row < n;
                    float f[32];
                    if (h == 0) {
                        float s = 0.f;
#pragma unroll
                        for (int j = 0; j < 27; ++j) {
                            const float val = sv[gl * 64 + (cx + j / 9) * 16 + (cy + (j / 3) % 3) * 4 + (cz + j % 3)];
                            f[j] = val;
                            s = fmaxf(s, fabsf(val));
                        }
                        const float inv = s > 0.f ? 1.f / s : 0.f;
#pragma unroll
                        for (int j = 0; j < 27; ++j) f[j] *= inv;
#pragma unroll
                        for (int j = 0; j < 5; ++j)   // features 27..31: coefficients of neighbours 0..4
                            f[27 + j] = spr[gl * 64 + (cx + j / 9) * 16 + (cy + (j / 3) % 3) * 4 + (cz + j % 3)] ? scn[j] : 0.f;
                        ss[grp][row] = valid ? s : 0.f;
                    } else {
#pragma unroll
                        for (int u = 0; u < 22; ++u) {   // features 32..53: coefficients of neighbours 5..26
                            const int j = 5 + u;
                            f[u] = spr[gl * 64 + (cx + j / 9) * 16 + (cy + (j / 3) % 3) * 4 + (cz + j % 3)] ? scn[j] : 0.f;
                        }
                        f[22] = dfeat;
#pragma unroll
                        for (int u = 23; u < 32; ++u) f[u] = 0.f;
                    }
#pragma unroll
                    for (int c = 0; c < 32; c += 8) {
                        __align__(16) __nv_bfloat16 fb[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) fb[u] = __float2bfloat16_rn(valid ? f[c + u] : 0.f);
                        *reinterpret_cast<uint4*>(sx + op_offset(128, row, 32 * h + c)) =
                            *reinterpret_cast<const uint4*>(fb);
                    }
                }
                float y = 0.f;
                if (!mlp_forward_tile_group(sx, m, tbase, &bars[grp], phase, red[grp], y, lt, gbar, &gflag[grp])) {
                    gok = false;
                    break;
                }
                if (own) {
                    const float rc = own_r;
                    float rn = rc;
                    if (!init) {
                        a.x[iown] = fmaf(al, own_p, own_x);
                        rn = fmaf(nal, own_q, rc);
                        rnext[iown] = rn;
                    }
                    const float s = ss[grp][lt];
                    const float zi = s > 0.f ? s * y * icen : 0.f;
                    a.z[iown] = zi;
                    acc[0] += (double)rn * (double)rn;
                    acc[1] += (double)zi * (double)rn;
                    acc[2] += (double)zi * (double)rc;
                }
                group_sync(gbar);
            }
        }
        if (!gok) {
            mma_ok = false;
            if (lt == 0) atomicExch(a.err, PRGPU_ERR_TIMEOUT);
        }
#pragma unroll
        for (int j = 0; j < FCG_NV; ++j) v[j] = acc[j];
        const bool r = reduce(v);
        return r && !*(volatile int*)a.err;
    };

    double rz_prev = bb, rr_prev = bb;
    if (ok && !plain) {
        ok = phase_b(true, 0.f, nullptr);
        const double rz0 = v[1];
        if (!(rz0 > 0.0) || !isfinite(rz0)) {
            plain = true;
            fallback_at = 0;
        } else {
            rz_prev = rz0;
        }
    }
    int k = 1;
    bool restart = true;
    float beta = 0.f;
    float* pnew = a.p;   // p and q are updated in place, each row by its own thread
    int refines = 0;
    double rr_true = -1.0;
    while (ok) {
        const bool go = (a.mode == PRGPU_SOLVE_REFERENCE) ? ((float)rr_prev > a.tol2) : (rr_prev > a.rel2 * bb);
        if (!go || k > a.max_iter) {
            if (!a.refine || a.mode != PRGPU_SOLVE_RELATIVE || k > a.max_iter) break;
            // the recurrence says converged: r = b - A x with FP64 accumulation
            double tsum = 0.0;
            for (i64 t = start; t < n; t += stride) {
                const i64 i = lo + t;
                double acc = (double)a.b[i];
#pragma unroll
                for (int j = 0; j < 27; ++j) {
                    const int nb = a.neigh[(i64)j * a.M + i];
                    if (nb != -1) acc = fma(-(double)sst[j], (double)a.x[nb], acc);
                }
                rcur[i] = (float)acc;
                tsum = fma(acc, acc, tsum);
            }
            v[0] = tsum;
            v[1] = v[2] = 0.0;
            if (!(ok = reduce(v))) break;
            rr_true = v[0];
            if (rr_true <= a.rel2 * bb || refines >= 2) break;
            // restart from the current x on the true residual, as plain CG
            ++refines;
            plain = true;
            restart = true;
            rz_prev = rr_prev = rr_true;
            continue;
        }
        const float* zsrc = plain ? rcur : a.z;
        // phase A: s = A z (z gathered once per cell), then row by row p = z + beta p and
        // q = A p = s + beta q, partial p.q
        FSum loc;
        auto own_row = [&](i64 i, float zi, float si) {
            float pi = zi, qi = si;
            if (!restart) {
                pi = fmaf(beta, pnew[i], zi);
                qi = fmaf(beta, a.q[i], si);
            }
            pnew[i] = pi;
            a.q[i] = qi;
            loc.add(pi * qi);
        };
        if (d == 0) {
            for (i64 t = start; t < n; t += stride) {
                const i64 i = lo + t;
                float o = 0.f;
#pragma unroll
                for (int j = 0; j < 27; ++j) {
                    const int nb = a.neigh[(i64)j * a.M + i];
                    if (nb != -1 && sst[j] != 0.f) o = fmaf(sst[j], zsrc[nb], o);
                }
                own_row(i, zsrc[i], o);
            }
        } else {
            const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
            const int ch = lane & 7, gl = lane >> 3;
            const int sx_ = (ch >> 2) & 1, sy = (ch >> 1) & 1, sz = ch & 1;
            float* wsp = sp + wib * (FCG_WARP_TILES * CG_TILE_WORDS);
            int* wgn = sgn + wib * (FCG_WARP_TILES * 4 * GN_ROW);
            const i64 wstride = (i64)dp.nblocks * FCG_WARPS * FCG_WARP_TILES;
            for (i64 tile = ((i64)rank * FCG_WARPS + wib) * FCG_WARP_TILES; tile * 4 < ng; tile += wstride) {
                __syncwarp();
                {
                    const i64 row0 = (gfirst + tile * 4) * GN_ROW;
                    const i64 nvalid = min((i64)FCG_WARP_TILES * 4, ng - tile * 4) * GN_ROW;
                    for (int k = lane; k < FCG_WARP_TILES * 4 * GN_ROW; k += 32)
                        wgn[k] = (k < nvalid) ? a.gnr[row0 + k] : -1;
                }
                __syncwarp();
                int cn[FCG_WARP_TILES * 8];
#pragma unroll
                for (int mm = 0; mm < FCG_WARP_TILES * 8; ++mm) {
                    const int e = lane + 32 * mm;
                    const int cell = e & 63, bx = cell >> 4, by = (cell >> 2) & 3, bz = cell & 3;
                    const int jp = 9 * ((bx + 1) >> 1) + 3 * ((by + 1) >> 1) + ((bz + 1) >> 1);
                    cn[mm] = wgn[(e >> 6) * GN_ROW + jp];
                }
#pragma unroll
                for (int mm = 0; mm < FCG_WARP_TILES * 8; ++mm) {
                    const int e = lane + 32 * mm;
                    const int cell = e & 63, bx = cell >> 4, by = (cell >> 2) & 3, bz = cell & 3;
                    wsp[(e >> 8) * CG_TILE_WORDS + cg_block_base((e >> 6) & 3) + cell] = (cn[mm] != -1)
                                 ? zsrc[cn[mm] + ((((bx + 1) & 1) << 2) | (((by + 1) & 1) << 1) | ((bz + 1) & 1))]
                                 : 0.f;
                }
                __syncwarp();
#pragma unroll
                for (int tt = 0; tt < FCG_WARP_TILES; ++tt) {
                    const i64 g = (tile + tt) * 4 + gl;
                    if (g < ng) {
                        const float* blk = wsp + tt * CG_TILE_WORDS + cg_block_base(gl);
                        float o = 0.f;
                        if (dp.sym) {
#pragma unroll
                            for (int j = 0; j < 27; ++j)
                                o = fmaf(cls[stencil_class(j)],
                                         blk[(sx_ + j / 9) * 16 + (sy + (j / 3) % 3) * 4 + (sz + j % 3)], o);
                        } else {
#pragma unroll
                            for (int j = 0; j < 27; ++j)
                                o = fmaf(sst[j], blk[(sx_ + j / 9) * 16 + (sy + (j / 3) % 3) * 4 + (sz + j % 3)], o);
                        }
                        own_row(lo + 8 * g + ch, blk[(sx_ + 1) * 16 + (sy + 1) * 4 + (sz + 1)], o);
                    }
                }
            }
            __syncthreads();   // the staging buffer is reused by phase B
        }
        v[0] = loc.value();
        v[1] = v[2] = 0.0;
        if (!(ok = reduce(v))) break;
        const double pq = v[0];
        if (!(pq > 0.0) || !isfinite(pq)) {
            if (plain) break;   // breakdown of plain CG: the residual is as small as it gets
            plain = true;       // the learned direction is unusable: restart plain CG from r
            fallback_at = k;
            restart = true;
            rz_prev = rr_prev;
            ++k;
            continue;
        }
        const float al = (float)(rz_prev / pq);
        ok = phase_b(false, al, pnew);
        if (!ok) break;
        const double rr = v[0], zr = v[1], zro = v[2];
        float* tmp = rcur;
        rcur = rnext;
        rnext = tmp;
        if (plain) {
            beta = (float)(rr / rz_prev);
            rz_prev = rr;
            restart = false;
        } else if (!(rr < rr_prev) || !(zr > 0.0) || !isfinite(zr) || !isfinite(zro)) {
            plain = true;       // the learned step did not reduce the residual: plain CG from here
            fallback_at = k;
            beta = 0.f;
            restart = true;
            rz_prev = rr;
        } else {
            beta = (float)((zr - zro) / rz_prev);
            rz_prev = zr;
            restart = false;
        }
        rr_prev = rr;
        ++k;
    }
    if (rank == 0 && threadIdx.x == 0) {
        a.state[d].iters = k - 1;
        a.state[d].fallback_at = fallback_at;
        a.state[d].rr = rr_prev;
        a.state[d].bb = bb;
        a.state[d].rr_true = rr_true;
        a.state[d].refines = refines;
        a.state[d].status = ok ? 0 : PRGPU_ERR_TIMEOUT;
    }
    // every MMA was waited for, except after a wait that gave up: wait (bounded) for it
    if (!mma_ok && lt == 0 && gflag[grp]) mbar_wait(&bars[grp], phase ^ 1u, MBAR_LIMIT);   // the wait that gave up
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(tslot, 512);
}

void stage_solve_learned(Ctx& c) {
    if (!c.lp_params) {
        set_last_error("params.learned is set but no preconditioner was loaded (prgpu_load_preconditioner)");
        throw Error{PRGPU_ERR_ARG, {0}};
    }
    cudaStream_t s = c.stream;
    const int D = c.D;
    const i64 M = c.nodes.M;
    dfree(c.x, s);
    c.x = dalloc<float>(M, s);
    c.x_rows = M;
    float* ra = dalloc<float>(M, s);
    float* rb = dalloc<float>(M, s);
    float* z = dalloc<float>(M, s);
    float* p = dalloc<float>(M, s);
    float* q = dalloc<float>(M, s);
    ensure_group_rows(c);
    std::vector<float> cn(27 * (D + 1)), centre(D + 1);
    for (int d = 0; d <= D; ++d) {
        centre[d] = c.stencil[27 * d + 13];
        for (int j = 0; j < 27; ++j) cn[27 * d + j] = centre[d] != 0.f ? c.stencil[27 * d + j] / centre[d] : 0.f;
    }
    float* dcn = dalloc<float>((i64)cn.size(), s);
    float* dcentre = dalloc<float>(D + 1, s);
    CK(cudaMemcpyAsync(dcn, cn.data(), cn.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dcentre, centre.data(), centre.size() * 4, cudaMemcpyHostToDevice, s));
    // the largest shared-memory carveout: the block holds about 120 KB
    CK(cudaFuncSetAttribute(k_fcg_all, cudaFuncAttributeMaxDynamicSharedMemorySize, FCG_DSMEM));
    CK(cudaFuncSetAttribute(k_fcg_all, cudaFuncAttributePreferredSharedMemoryCarveout,
                            (int)cudaSharedmemCarveoutMaxShared));
    int sms = 0, per_sm = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fcg_all, FCG_THREADS, FCG_DSMEM));
    if (per_sm < 1) {
        set_last_error("the flexible CG kernel cannot be resident on an SM");
        throw Error{PRGPU_ERR_LIMIT, {0}};
    }
    // the block allocates all 512 TMEM columns of its SM: one block per SM
    per_sm = 1;
    c.solver_blocks = sms * per_sm;
    std::vector<CgDepth> deps;
    std::vector<int> block_depth;
    partition_depths(c, 0, D, sms * per_sm, deps, block_depth);
    const int nblk = (int)block_depth.size();
    CgDepth* ddeps = dalloc<CgDepth>(D + 1, s);
    int* dbd = dalloc<int>(nblk, s);
    FcgState* st = dalloc<FcgState>(D + 1, s);
    FcgSync* psync = dalloc<FcgSync>(D + 1, s);
    double* partial = dalloc<double>((i64)nblk * 4, s);
    int* err = dalloc<int>(1, s);
    CK(cudaMemcpyAsync(ddeps, deps.data(), (D + 1) * sizeof(CgDepth), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dbd, block_depth.data(), nblk * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(st, 0, (D + 1) * sizeof(FcgState), s));
    CK(cudaMemsetAsync(psync, 0, (D + 1) * sizeof(FcgSync), s));
    CK(cudaMemsetAsync(err, 0, sizeof(int), s));
    FcgArgs a;
    a.mode = c.params.solve_mode;
    const float tolf = (float)c.params.cg_tol;
    a.tol2 = tolf * tolf;
    a.rel2 = c.params.cg_tol * c.params.cg_tol;
    a.max_iter = c.params.cg_max_iter;
    a.M = M;
    a.neigh = c.nodes.neigh;
    a.gn = c.gn;
    a.gnr = c.gn_rows;
    a.ngroups = (M - 1) / 8;
    a.b = c.divergence;
    a.x = c.x;
    a.ra = ra;
    a.rb = rb;
    a.z = z;
    a.p = p;
    a.q = q;
    a.state = st;
    a.sync = psync;
    a.partial = partial;
    a.err = err;
    const WaitLimits wl = wait_limits();
    a.spin_limit = wl.spin_limit;
    a.extra = wl.extra;
    a.wt.w1 = (const __nv_bfloat16*)c.lp_w1b;
    a.wt.w2 = (const __nv_bfloat16*)c.lp_w2b;
    a.wt.p = c.lp_params;
    a.cnorm = dcn;
    a.centre = dcentre;
    a.refine = c.params.refine;
    void* kargs[] = {(void*)&a, (void*)&ddeps, (void*)&dbd};
    const int kt = c.kbegin("fcg", 0.0);
    CK(cudaLaunchCooperativeKernel((void*)k_fcg_all, dim3((unsigned)nblk), dim3(FCG_THREADS), kargs, FCG_DSMEM, s));
    ++g_kernel_launches;
    c.kend(kt);
    std::vector<FcgState> hs(D + 1);
    int herr = 0;
    CK(cudaMemcpyAsync(hs.data(), st, (D + 1) * sizeof(FcgState), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    c.cg_iters.assign(D + 1, 0);
    c.cg_rr.assign(D + 1, 0.f);
    c.cg_fallback.assign(D + 1, -1);
    c.cg_true_rel.assign(D + 1, 0.0);
    c.cg_fp64_rel.assign(D + 1, -1.0);
    c.cg_refines.assign(D + 1, 0);
    double bytes = 0;
    for (int d = 0; d <= D; ++d) {
        c.cg_iters[d] = hs[d].iters;
        c.cg_rr[d] = (float)hs[d].rr;
        c.cg_fallback[d] = hs[d].fallback_at;
        c.cg_true_rel[d] = hs[d].bb > 0 ? std::sqrt(hs[d].rr / hs[d].bb) : 0.0;
        c.cg_fp64_rel[d] = (hs[d].rr_true >= 0 && hs[d].bb > 0) ? std::sqrt(hs[d].rr_true / hs[d].bb) : -1.0;
        c.cg_refines[d] = hs[d].refines;
        // per row and iteration: the group table twice (product and preconditioner
        // staging), z or r, the previous p, p and q written; r and q staged, x read and
        // written, p read, r' and z written
        bytes += (double)hs[d].iters * (double)c.count[d] * (2 * 13.5 + 4 * 4 + 9 * 4);
    }
    if (kt >= 0) c.kpending[kt].bytes = bytes;
    dfree(ra, s); dfree(rb, s); dfree(z, s); dfree(p, s); dfree(q, s);
    dfree(dcn, s); dfree(dcentre, s); dfree(ddeps, s); dfree(dbd, s); dfree(st, s); dfree(psync, s);
    dfree(partial, s); dfree(err, s);
    if (herr) {
        set_last_error("flexible CG: a device wait timed out");
        throw Error{PRGPU_ERR_TIMEOUT, {0}};
    }
}

}  // namespace prgpu
