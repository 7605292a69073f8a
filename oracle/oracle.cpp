// oracle.cpp -- CPU restatement of the reference Poisson-reconstruction path.
//
// TEST INFRASTRUCTURE.  This file is the parity oracle and the CPU baseline.
// Only tests/, __graft_entry__.smoke() and bench.py (CPU-baseline leg) may load
// it; the product library never calls into it.
//
// Every stage follows the reference (DavidXu-JJ/PoissonRecon_GPU) step by step;
// each function cites the file:line it restates.  Arithmetic is ordered as the
// reference orders it:
//   * host-side reference code (input normalisation, basis functions, inner-
//     product tables) is x86-64 code without fused multiply-add: this file is
//     compiled with -ffp-contract=off so the same IEEE single/double sequence
//     results on any host;
//   * device-side reference code (splat weights, basis evaluation, CG, marching
//     cubes interpolation) was compiled by nvcc, which fuses a*b+c into one FMA;
//     those sites call fmaf()/fma() explicitly.
// Deliberate deviations from the reference (its races and uninitialised reads)
// are marked "canonical" and take the value the reference intends.
//
// Parity status: the inner-product tables are pinned bit-exactly against the
// reference's own host code (oracle/ref_tables_driver.cu); the marching-cubes
// case table is pinned against MarchingCubes.cuh; the remaining stages are a
// restatement checked by the tests against those pins and analytic properties.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../poissonrecon_gpu_gb300/csrc/mc_table.h"

namespace orc {

typedef int64_t i64;
typedef uint64_t u64;

// ---------------------------------------------------------------------------
// Host polynomial arithmetic (Polynomial.inl, PPolynomial.inl), float
// ---------------------------------------------------------------------------
struct SPoly {          // StartingPolynomial<deg<=4>  (PPolynomial.cuh:33)
    float start;
    float c[5];
    int deg;
};
typedef std::vector<SPoly> PPoly;

static SPoly sp_zero(int deg) { SPoly s; s.start = 0; s.deg = deg; for (int i = 0; i < 5; ++i) s.c[i] = 0; return s; }

// Polynomial::shift  (Polynomial.inl:258-268)
static void poly_shift(const float* c, int deg, float t, float* out) {
    for (int i = 0; i <= deg; ++i) out[i] = 0;
    for (int i = 0; i <= deg; ++i) {
        float temp = 1;
        for (int j = i; j >= 0; --j) {
            out[j] += c[i] * temp;
            temp *= -t * j;
            temp /= (i - j + 1);
        }
    }
}
// Polynomial::operator()  (Polynomial.inl:72-80)
static float poly_eval(const float* c, int deg, float t) {
    float temp = 1, v = 0;
    for (int i = 0; i <= deg; ++i) { v += temp * c[i]; temp *= t; }
    return v;
}
// Polynomial::integral(tMin,tMax)  (Polynomial.inl:81-92)
static float poly_integral(const float* c, int deg, float tMin, float tMax) {
    float v = 0, t1 = tMin, t2 = tMax;
    for (int i = 0; i <= deg; ++i) {
        v += c[i] * (t2 - t1) / (i + 1);
        t1 *= tMin;
        t2 *= tMax;
    }
    return v;
}
// PPolynomial::set(sps,count): order by start, merge equal starts (PPolynomial.inl:94-104)
static PPoly pp_set(std::vector<SPoly> sps) {
    std::stable_sort(sps.begin(), sps.end(), [](const SPoly& a, const SPoly& b) { return a.start - b.start < 0; });
    PPoly q;
    for (auto& s : sps) {
        if (q.empty() || s.start != q.back().start) q.push_back(s);
        else for (int k = 0; k < 5; ++k) q.back().c[k] += s.c[k];
    }
    return q;
}
// PPolynomial::scale  (PPolynomial.inl:283-289 with StartingPolynomial::scale :46-52)
static PPoly pp_scale(const PPoly& a, float s) {
    PPoly q = a;
    for (auto& p : q) {
        p.start = p.start * s;
        float s2 = 1.0f;
        for (int i = 0; i <= p.deg; ++i) { p.c[i] *= s2; s2 /= s; }
    }
    return q;
}
// PPolynomial::shift  (PPolynomial.inl:290-296)
static PPoly pp_shift(const PPoly& a, float t) {
    PPoly q = a;
    for (auto& p : q) {
        p.start = p.start + t;
        float o[5];
        poly_shift(p.c, p.deg, t, o);
        for (int i = 0; i < 5; ++i) p.c[i] = (i <= p.deg) ? o[i] : 0.f;
    }
    return q;
}
// PPolynomial::operator*(PPolynomial)  (PPolynomial.inl:256-270)
static PPoly pp_mul(const PPoly& a, const PPoly& b) {
    std::vector<SPoly> sp;
    sp.reserve(a.size() * b.size());
    for (auto& x : a)
        for (auto& y : b) {
            SPoly r = sp_zero(x.deg + y.deg);
            r.start = x.start > y.start ? x.start : y.start;
            for (int i = 0; i <= x.deg; ++i)
                for (int j = 0; j <= y.deg; ++j) r.c[i + j] += x.c[i] * y.c[j];
            sp.push_back(r);
        }
    return pp_set(sp);
}
// PPolynomial::integral(tMin,tMax)  (PPolynomial.inl:158-174)
static float pp_integral(const PPoly& a, float tMin, float tMax) {
    int m = 1;
    float st = tMin, en = tMax, s, v = 0;
    if (tMin > tMax) { m = -1; st = tMax; en = tMin; }
    for (size_t i = 0; i < a.size() && a[i].start < en; ++i) {
        s = st < a[i].start ? a[i].start : st;
        v += poly_integral(a[i].c, a[i].deg, s, en);
    }
    return v * m;
}
// PPolynomial::operator()  (PPolynomial.inl:152-157)
static float pp_eval(const PPoly& a, float t) {
    float v = 0;
    for (size_t i = 0; i < a.size() && t > a[i].start; ++i) v += poly_eval(a[i].c, a[i].deg, t);
    return v;
}
static PPoly pp_derivative(const PPoly& a) {  // PPolynomial.inl:297-305, Polynomial.inl:56-61
    PPoly q = a;
    for (auto& p : q) {
        float o[5] = {0, 0, 0, 0, 0};
        for (int i = 0; i < p.deg; ++i) o[i] = p.c[i + 1] * (i + 1);
        p.deg -= 1;
        memcpy(p.c, o, sizeof o);
    }
    return q;
}
// PPolynomial::MovingAverage  (PPolynomial.inl:406-423)
static PPoly pp_moving_average(const PPoly& a, float radius) {
    std::vector<SPoly> sps;
    for (auto& pi : a) {
        SPoly ip = sp_zero(pi.deg + 1);  // Polynomial::integral(): c[0]=0, c[i+1]=c[i]/(i+1)
        for (int i = 0; i <= pi.deg; ++i) ip.c[i + 1] = pi.c[i] / (i + 1);
        float at = poly_eval(ip.c, ip.deg, pi.start);
        ip.c[0] -= at;
        SPoly lo = sp_zero(ip.deg), hi = sp_zero(ip.deg);
        lo.start = pi.start - radius;
        hi.start = pi.start + radius;
        poly_shift(ip.c, ip.deg, -radius, lo.c);
        poly_shift(ip.c, ip.deg, radius, hi.c);
        for (int i = 0; i <= hi.deg; ++i) hi.c[i] = hi.c[i] * -1.0f;
        sps.push_back(lo);
        sps.push_back(hi);
    }
    PPoly A = pp_set(sps);
    float div = 2 * radius;
    for (auto& p : A)
        for (int i = 0; i <= p.deg; ++i) { p.c[i] *= 1.0f; p.c[i] /= div; }
    return A;
}
// GaussianApproximation<2>(0.5)  (PPolynomial.inl:384-404)
static PPoly gaussian_approximation2() {
    PPoly c;  // ConstantFunction(0.5)
    SPoly a = sp_zero(0), b = sp_zero(0);
    a.start = -0.5f; a.c[0] = 1.0f;
    b.start = 0.5f; b.c[0] = -1.0f;
    c.push_back(a);
    c.push_back(b);
    return pp_moving_average(pp_moving_average(c, 0.5f), 0.5f);
}

// BinaryNode<Real>::CenterAndWidth(idx)  (BinaryNode.cuh:45-60)
static void center_width_d(int idx, double& c, double& w) {
    int i = idx + 1, d = -1;
    while (i) { i >>= 1; d++; }
    int off = (idx + 1) - (1 << d);
    w = 1.0 / (1 << d);
    c = (0.5 + off) * w;
}
static void center_width_f(int idx, float& c, float& w) {
    int i = idx + 1, d = -1;
    while (i) { i >>= 1; d++; }
    int off = (idx + 1) - (1 << d);
    w = float(1.0 / (1 << d));
    c = float((0.5 + off) * (double)w);
}

// ---------------------------------------------------------------------------
// Device-side polynomial evaluation (ConfirmedPPolynomial.cuh:37-91), FMA sites
// ---------------------------------------------------------------------------
struct CPoly {  // ConfirmedPPolynomial<Deg,4>, degree <= 3, 4 pieces
    float start[4];
    float c[4][4];
};
// ConfirmedPPolynomial::shift  (ConfirmedPPolynomial.cuh:37-50)
static CPoly cpoly_shift(const CPoly& p, int deg, float t) {
    CPoly r;
    for (int i = 0; i < 4; ++i) {
        r.start[i] = p.start[i] + t;
        for (int k = 0; k < 4; ++k) r.c[i][k] = 0;
        for (int k = 0; k <= deg; ++k) {
            float temp = 1;
            for (int j = k; j >= 0; --j) {
                r.c[i][j] = fmaf(p.c[i][k], temp, r.c[i][j]);
                temp = temp * (-t * (float)j);
                temp = temp / (float)(k - j + 1);
            }
        }
    }
    return r;
}
// value(ConfirmedPPolynomial, x)  (ConfirmedPPolynomial.cuh:79-91)
static inline float cpoly_value(const CPoly& p, int deg, float x) {
    float res = 0;
    for (int i = 0; i < 4 && x > p.start[i]; ++i) {
        float temp = 1, v = 0;
        for (int j = 0; j <= deg; ++j) { v = fmaf(temp, p.c[i][j], v); temp = temp * x; }
        res = res + v;
    }
    return res;
}
static CPoly to_cpoly(const PPoly& a) {
    CPoly r;
    memset(&r, 0, sizeof r);
    for (size_t i = 0; i < a.size() && i < 4; ++i) {
        r.start[i] = a[i].start;
        for (int k = 0; k <= a[i].deg && k < 4; ++k) r.c[i][k] = a[i].c[k];
    }
    return r;
}

// ---------------------------------------------------------------------------
// Lookup tables derived from their definitions (main.cu:80-99,
// MarchingCubes.cuh:693-744)
// ---------------------------------------------------------------------------
static int LUTparent[8][27], LUTchild[8][27];
static int parentFaceKind[8][6];
static int childrenVertexKind[8];
static int faceEdges[6][4];
static prgpu_mc::Tables MC;
static bool g_tables_ready = false;

static void init_static_tables() {
    if (g_tables_ready) return;
    for (int s = 0; s < 8; ++s) {
        int cx = (s >> 2) & 1, cy = (s >> 1) & 1, cz = s & 1;
        for (int j = 0; j < 27; ++j) {
            int dx = j / 9 - 1, dy = (j / 3) % 3 - 1, dz = j % 3 - 1;
            int tx = cx + dx, ty = cy + dy, tz = cz + dz;
            int px = (tx + 2) / 2 - 1, py = (ty + 2) / 2 - 1, pz = (tz + 2) / 2 - 1;
            LUTparent[s][j] = 9 * (px + 1) + 3 * (py + 1) + (pz + 1);
            LUTchild[s][j] = ((tx & 1) << 2) | ((ty & 1) << 1) | (tz & 1);
        }
    }
    // parentFaceKind is indexed by an (x | y<<1 | z<<2) child code in the
    // reference table; its last row also lists face 0 (MarchingCubes.cuh:708-717).
    for (int s = 0; s < 8; ++s) {
        int xyz[3] = {s & 1, (s >> 1) & 1, (s >> 2) & 1};
        for (int j = 0; j < 6; ++j) parentFaceKind[s][j] = (xyz[j >> 1] == (j & 1)) ? j : -1;
    }
    parentFaceKind[7][0] = 0;
    // childrenVertexKind[j] is the cube-vertex id of corner j (MarchingCubes.cuh:721-723)
    for (int j = 0; j < 8; ++j) childrenVertexKind[j] = prgpu_mc::vertex_id(j & 1, (j >> 1) & 1, (j >> 2) & 1);
    for (int f = 0; f < 6; ++f) {
        int a = f >> 1, s = f & 1, n = 0;
        for (int e = 0; e < 12; ++e) {
            int o = e >> 2;
            if (o == a) continue;
            int a0 = (o == 0) ? 1 : 0, a1 = (o == 2) ? 1 : 2;
            int off = (a == a0) ? (e & 1) : ((e >> 1) & 1);
            (void)a1;
            if (off == s) faceEdges[f][n++] = e;
        }
    }
    prgpu_mc::build(MC);
    g_tables_ready = true;
}

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
struct Mesh {
    std::vector<float> v;   // 3 per vertex, normalised coordinates
    std::vector<int> f;     // 3 per triangle
    std::vector<i64> vkey;  // per vertex: its lattice edge (lattice_edge_key), for the weld check
};

struct Ctx {
    int D = 8;
    int threads = 1;
    i64 N = 0;
    std::vector<float> in_p, in_n;          // raw input
    std::vector<float> P, Nn;               // normalised, sorted
    std::vector<i64> sort_idx;              // input index of each sorted point
    float center[3] = {0, 0, 0}, scale = 1;
    // node arrays (global index = base[d] + slot)
    std::vector<i64> base, count;           // D+2 / D+1
    i64 M = 0;
    std::vector<i64> key;
    std::vector<int> pidx, pnum, parent, didx, dnum, depth;
    std::vector<int> children, neighs;      // 8*M, 27*M
    std::vector<int> point_node;            // sorted point -> global leaf index
    // basis
    int res = 0;
    PPoly base_f, dbase_f, F_norm;
    std::vector<CPoly> basis;               // res basis functions (degree 3 storage, cubic 0)
    CPoly basis_maxdepth;                   // F/F(0) scaled to the finest width (degree 2)
    std::vector<double> dot, ddot, d2dot;   // res*res
    // rhs / solve
    std::vector<float> vfield;              // 3*count[D]
    std::vector<float> divergence;          // M
    std::vector<float> x;                   // M
    std::vector<int> cg_iters;              // D+1
    std::vector<float> cg_rr;               // D+1 final r.r
    std::vector<float> stencil;             // 27*(D+1)
    std::vector<double> stencil64;          // the same entries before the cast to float
    int cascadic = 0;                       // coarse-to-fine solve (not the reference's)
    // FP64 run (precision study)
    std::vector<double> vfield64, divergence64, x64, point_value64;
    std::vector<int> cg_iters64;
    double iso64 = 0;
    // iso
    std::vector<float> point_value;
    float iso = 0;
    // mesh
    Mesh mesh;
    std::vector<int> has_tri, has_int;      // per node at depth < D
    i64 subdivide_roots = 0;
    // timing samples only: subdivide every root_stride-th root (0: none), and
    // the virtual cells of all roots / of the subdivided ones
    int root_stride = 1;
    i64 vcells[2] = {0, 0};
    std::vector<i64> batch_tri;             // triangles per batch (0 = finest real nodes)
    std::vector<float> corner_value_D;      // per depth-D vertex (debug)
};

static int omp_threads(const Ctx& c) { return c.threads > 0 ? c.threads : 1; }

// ---------------------------------------------------------------------------
// a1: normalisation  (main.cu:511-571)
// ---------------------------------------------------------------------------
static void normalise(Ctx& c, std::vector<float>& p, std::vector<float>& n) {
    const i64 N = c.N;
    float mx[3], mn[3];
    for (i64 k = 0; k < N; ++k)
        for (int i = 0; i < 3; ++i) {
            float v = c.in_p[3 * k + i];
            if (!k || v < mn[i]) mn[i] = v;
            if (!k || v > mx[i]) mx[i] = v;
        }
    float scale = 1;
    for (int i = 0; i < 3; ++i) {
        if (!i || scale < mx[i] - mn[i]) scale = float(mx[i] - mn[i]);
        c.center[i] = float(mx[i] + mn[i]) / 2;
    }
    scale *= 1.25f;
    for (int i = 0; i < 3; ++i) c.center[i] -= scale / 2;
    c.scale = scale;
    p.resize(3 * N);
    n.resize(3 * N);
    const float D2 = (float)(2 << c.D);
    for (i64 k = 0; k < N; ++k) {
        for (int i = 0; i < 3; ++i) p[3 * k + i] = (c.in_p[3 * k + i] - c.center[i]) / scale;
        float nx = c.in_n[3 * k], ny = c.in_n[3 * k + 1], nz = c.in_n[3 * k + 2];
        float sq = nx * nx + ny * ny + nz * nz;   // SquareLength in Real=float (Geometry.inl:30)
        float len = float(std::sqrt((double)sq));
        if (len > float(1e-6)) len = 1.0f / len;
        len *= D2;
        n[3 * k] = nx * len;
        n[3 * k + 1] = ny * len;
        n[3 * k + 2] = nz * len;
    }
}

// encodePoint  (main.cu:132-164): D-level key from '>' comparisons
static u64 encode_point(const float* pos, int D) {
    u64 key = 0;
    float cx = 0.5f, cy = 0.5f, cz = 0.5f, w = 0.25f;
    for (int i = D - 1; i >= 0; --i) {
        if (pos[0] > cx) { key |= 1ull << (3 * i + 2); cx += w; } else cx -= w;
        if (pos[1] > cy) { key |= 1ull << (3 * i + 1); cy += w; } else cy -= w;
        if (pos[2] > cz) { key |= 1ull << (3 * i); cz += w; } else cz -= w;
        w /= 2;
    }
    return key;
}

// ---------------------------------------------------------------------------
// a2-a7: octree  (main.cu:166-841)
// ---------------------------------------------------------------------------
static void build_octree(Ctx& c) {
    const int D = c.D;
    const i64 N = c.N;
    std::vector<float> p, n;
    normalise(c, p, n);
    std::vector<u64> code(N);
    for (i64 k = 0; k < N; ++k) code[k] = encode_point(&p[3 * k], D);
    // sort_by_key on (key<<32 | index): order by key, ties by input index (main.cu:596-603)
    std::vector<i64> order(N);
    for (i64 k = 0; k < N; ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](i64 a, i64 b) { return code[a] < code[b]; });
    c.P.resize(3 * N); c.Nn.resize(3 * N); c.sort_idx = order;
    std::vector<u64> skey(N);
    for (i64 k = 0; k < N; ++k) {
        i64 s = order[k];
        for (int i = 0; i < 3; ++i) { c.P[3 * k + i] = p[3 * s + i]; c.Nn[3 * k + i] = n[3 * s + i]; }
        skey[k] = code[s];
    }
    // unique nodes per depth: uk[d], first point, point count
    std::vector<std::vector<u64>> uk(D + 1);
    std::vector<std::vector<int>> upidx(D + 1), upnum(D + 1), uparent(D + 1);
    for (i64 k = 0; k < N; ++k) {
        if (k == 0 || skey[k] != skey[k - 1]) { uk[D].push_back(skey[k]); upidx[D].push_back((int)k); }
    }
    for (size_t r = 0; r < uk[D].size(); ++r)
        upnum[D].push_back((int)((r + 1 < uk[D].size() ? upidx[D][r + 1] : N) - upidx[D][r]));
    for (int d = D - 1; d >= 0; --d) {
        u64 mask = ~((1ull << (3 * (D - d))) - 1);
        for (size_t r = 0; r < uk[d + 1].size(); ++r) {
            u64 pk = uk[d + 1][r] & mask;
            if (uk[d].empty() || uk[d].back() != pk) {
                uk[d].push_back(pk); upidx[d].push_back(upidx[d + 1][r]); upnum[d].push_back(0);
            }
            upnum[d].back() += upnum[d + 1][r];
            uparent[d + 1].push_back((int)uk[d].size() - 1);
        }
    }
    // node array sizes: full sibling groups below every non-empty node
    c.count.assign(D + 1, 0);
    c.base.assign(D + 2, 0);
    c.count[0] = 1;
    for (int d = 1; d <= D; ++d) c.count[d] = 8 * (i64)uk[d - 1].size();
    for (int d = 1; d <= D + 1; ++d) c.base[d] = c.base[d - 1] + c.count[d - 1];
    const i64 M = c.base[D + 1];
    c.M = M;
    c.key.assign(M, 0); c.pidx.assign(M, 0); c.pnum.assign(M, 0); c.parent.assign(M, -1);
    c.didx.assign(M, 0); c.dnum.assign(M, 0); c.depth.assign(M, 0);
    c.children.assign(8 * M, -1); c.neighs.assign(27 * M, -1);
    // slot of every unique node at its depth
    std::vector<std::vector<i64>> uslot(D + 1);
    uslot[0].push_back(0);
    for (int d = 1; d <= D; ++d)
        for (size_t r = 0; r < uk[d].size(); ++r)
            uslot[d].push_back(8 * (i64)uparent[d][r] + (i64)((uk[d][r] >> (3 * (D - d))) & 7));
    // keys, depth, parents of every slot (updateEmptyNodeInfo main.cu:433-490 gives
    // every sibling the key of its slot and the common parent)
    c.key[0] = 0; c.depth[0] = 0; c.parent[0] = -1;
    for (int d = 1; d <= D; ++d) {
        for (size_t g = 0; g < uk[d - 1].size(); ++g) {
            i64 pglobal = c.base[d - 1] + uslot[d - 1][g];
            for (int k = 0; k < 8; ++k) {
                i64 s = c.base[d] + 8 * (i64)g + k;
                c.key[s] = (i64)(uk[d - 1][g] | ((u64)k << (3 * (D - d))));
                c.depth[s] = d;
                c.parent[s] = (int)pglobal;  // canonical: the true parent of every sibling
            }
        }
    }
    // non-empty nodes: pidx/pnum (generateUniqueNodeArrayD_1 main.cu:301-334)
    for (int d = 0; d <= D; ++d)
        for (size_t r = 0; r < uk[d].size(); ++r) {
            i64 s = c.base[d] + uslot[d][r];
            c.pidx[s] = upidx[d][r];
            c.pnum[s] = upnum[d][r];
        }
    // children: contiguous groups of 8 (canonical for every non-empty node above D)
    for (int d = 0; d < D; ++d)
        for (size_t r = 0; r < uk[d].size(); ++r) {
            i64 s = c.base[d] + uslot[d][r];
            for (int k = 0; k < 8; ++k) c.children[8 * s + k] = (int)(c.base[d + 1] + 8 * (i64)r + k);
        }
    // didx/dnum at depth D (initNodeArrayD_DIdxDnum main.cu:267-276)
    for (i64 s = 0; s < c.count[D]; ++s) { c.didx[c.base[D] + s] = (int)s; c.dnum[c.base[D] + s] = 1; }
    // non-empty nodes above D: sum of children dnum, min didx over children with dnum != 0
    for (int d = D - 1; d >= 0; --d)
        for (size_t r = 0; r < uk[d].size(); ++r) {
            i64 s = c.base[d] + uslot[d][r];
            int sum = 0, mn = 0x7fffffff;
            for (int k = 0; k < 8; ++k) {
                i64 ch = c.children[8 * s + k];
                if (c.dnum[ch] != 0) { sum += c.dnum[ch]; mn = std::min(mn, c.didx[ch]); }
            }
            c.dnum[s] = sum;
            c.didx[s] = mn;
        }
    // empty siblings: pidx/didx as running prefixes inside the group (main.cu:457-486)
    for (int d = 1; d <= D; ++d)
        for (i64 g = 0; g < c.count[d] / 8; ++g) {
            i64 s0 = c.base[d] + 8 * g;
            int valid = 0;
            while (valid < 8 && c.pnum[s0 + valid] == 0) ++valid;
            int nowP = c.pidx[s0 + valid], nowD = c.didx[s0 + valid];
            for (int k = 0; k < 8; ++k) {
                c.pidx[s0 + k] = nowP;
                nowP += c.pnum[s0 + k];
                if (d != D) { c.didx[s0 + k] = nowD; nowD += c.dnum[s0 + k]; }
            }
        }
    // point -> leaf map (processPointToNodeArrayD main.cu:252-265)
    c.point_node.assign(N, 0);
    for (size_t r = 0; r < uk[D].size(); ++r) {
        i64 s = c.base[D] + uslot[D][r];
        for (int k = 0; k < upnum[D][r]; ++k) c.point_node[upidx[D][r] + k] = (int)s;
    }
    // neighbours top-down (computeNeighbor main.cu:492-509, root main.cu:803-808)
    c.neighs[13] = 0;
    for (int d = 1; d <= D; ++d) {
#pragma omp parallel for num_threads(omp_threads(c)) schedule(static)
        for (i64 s = c.base[d]; s < c.base[d + 1]; ++s) {
            int son = (int)((c.key[s] >> (3 * (D - d))) & 7);
            int par = c.parent[s];
            for (int j = 0; j < 27; ++j) {
                int np = c.neighs[27 * (i64)par + LUTparent[son][j]];
                c.neighs[27 * s + j] = (np != -1) ? c.children[8 * (i64)np + LUTchild[son][j]] : -1;
            }
        }
    }
}

// per-axis offset of a node at its depth, and its function index (main.cu:861-911)
static inline void node_coords(u64 key, int d, int D, int xyz[3]) {
    xyz[0] = xyz[1] = xyz[2] = 0;
    for (int l = 1; l <= d; ++l) {
        int sh = 3 * (D - l);
        xyz[0] = (xyz[0] << 1) | (int)((key >> (sh + 2)) & 1);
        xyz[1] = (xyz[1] << 1) | (int)((key >> (sh + 1)) & 1);
        xyz[2] = (xyz[2] << 1) | (int)((key >> sh) & 1);
    }
}
static inline void function_index(const Ctx& c, i64 node, int fi[3]) {
    int d = c.depth[node], xyz[3];
    node_coords((u64)c.key[node], d, c.D, xyz);
    for (int a = 0; a < 3; ++a) fi[a] = (1 << d) - 1 + xyz[a];
}

// ---------------------------------------------------------------------------
// a8: basis functions and inner-product tables (FunctionData.inl:112-300,
// main.cu:3306-3359)
// ---------------------------------------------------------------------------
static void build_basis(Ctx& c, bool full_tables) {
    const int D = c.D;
    PPoly F = gaussian_approximation2();
    float f0 = pp_eval(F, 0);
    PPoly baseF = F;
    for (auto& p : baseF) for (int i = 0; i <= p.deg; ++i) p.c[i] /= f0;   // F/F(0)
    c.base_f = baseF;
    c.dbase_f = pp_derivative(baseF);
    c.F_norm = baseF;
    c.res = (1 << (D + 1)) - 1;
    const int res = c.res;
    c.basis.resize(res);
    for (int i = 0; i < res; ++i) {
        double c1, w1;
        center_width_d(i, c1, w1);
        PPoly b = pp_shift(pp_scale(baseF, (float)w1), (float)c1);
        CPoly cp = to_cpoly(b);
        c.basis[i] = cp;   // stored as degree 3 with a zero cubic coefficient
    }
    c.basis_maxdepth = to_cpoly(pp_scale(baseF, (float)(1.0 / (1 << D))));
    // tables (FunctionData::setDotTables, FunctionData.inl:159-205)
    const size_t R2 = (size_t)res * res;
    if (full_tables) { c.dot.assign(R2, 0); c.ddot.assign(R2, 0); c.d2dot.assign(R2, 0); }
    const double t1 = baseF[0].start, t2 = baseF.back().start;
    const double r = std::fabs(baseF[0].start);
    const PPoly& B = c.base_f;
    const PPoly& dB = c.dbase_f;
    // same-depth stencil factors are translation invariant; record them per depth
    c.stencil.assign(27 * (D + 1), 0.f);
    c.stencil64.assign(27 * (D + 1), 0.0);
    std::vector<double> sdot(2 * (D + 1)), sd2(2 * (D + 1));
    for (int d = 0; d <= D; ++d) {
        double w = 1.0 / (1 << d);
        for (int delta = 0; delta <= 1; ++delta) {
            // pair (i, j=i-delta): shift (c2-c1)/w1 = -delta, scale 1
            PPoly g = pp_shift(pp_scale(B, 1.0f), (float)(-delta));
            PPoly dg = pp_shift(pp_scale(dB, 1.0f), (float)(-delta));
            sdot[2 * d + delta] = pp_integral(pp_mul(B, g), (float)(-2 * r), (float)(2 * r)) * w;
            sd2[2 * d + delta] = pp_integral(pp_mul(dB, dg), (float)(-2 * r), (float)(2 * r)) / w;
        }
        // GetLaplacianEntry (main.cu:1143-1158), dropped when |v|<=1e-6 (main.cu:1205)
        for (int j = 0; j < 27; ++j) {
            int dd[3] = {std::abs(j / 9 - 1), std::abs((j / 3) % 3 - 1), std::abs(j % 3 - 1)};
            if (d == 0 && (dd[0] | dd[1] | dd[2])) continue;
            double dt[3], d2[3];
            for (int a = 0; a < 3; ++a) { dt[a] = sdot[2 * d + dd[a]]; d2[a] = sd2[2 * d + dd[a]]; }
            double e = d2[0] * dt[1] * dt[2] + d2[1] * dt[0] * dt[2] + d2[2] * dt[0] * dt[1];
            c.stencil[27 * d + j] = (std::fabs(e) > (double)float(1e-6)) ? (float)e : 0.f;
            c.stencil64[27 * d + j] = (std::fabs(e) > (double)float(1e-6)) ? e : 0.0;
        }
    }
    if (!full_tables) return;
    for (int i = 0; i < res; ++i) {
        double c1, w1;
        center_width_d(i, c1, w1);
        double start1 = t1 * w1 + c1, end1 = t2 * w1 + c1;
        for (int j = 0; j <= i; ++j) {
            double c2, w2;
            center_width_d(j, c2, w2);
            size_t idx1 = (size_t)i + (size_t)res * j, idx2 = (size_t)j + (size_t)res * i;
            double start = t1 * w2 + c2, end = t2 * w2 + c2;
            if (start < start1) start = start1;
            if (end > end1) end = end1;
            if (start >= end) continue;
            PPoly g = pp_shift(pp_scale(B, (float)(w2 / w1)), (float)((c2 - c1) / w1));
            double dv = pp_integral(pp_mul(B, g), (float)(-2 * r), (float)(2 * r)) * w1;
            if (std::fabs(dv) < 1e-15) continue;
            c.dot[idx1] = c.dot[idx2] = dv;
            double dd = pp_integral(pp_mul(dB, g), (float)(-2 * r), (float)(2 * r));
            c.ddot[idx1] = dd;
            c.ddot[idx2] = -c.ddot[idx1];   // on the diagonal this overwrites with -dd
            PPoly dg = pp_shift(pp_scale(dB, (float)(w2 / w1)), (float)((c2 - c1) / w1));
            c.d2dot[idx1] = c.d2dot[idx2] = pp_integral(pp_mul(dB, dg), (float)(-2 * r), (float)(2 * r)) / w2;
        }
    }
}

// ---------------------------------------------------------------------------
// a9: vector field  (main.cu:913-964)
// ---------------------------------------------------------------------------
static void vector_field(Ctx& c) {
    const int D = c.D;
    const i64 lo = c.base[D], hi = c.base[D + 1];
    c.vfield.assign(3 * (hi - lo), 0.f);
    // the shifted splat kernel depends only on the point: hoist it
    std::vector<CPoly> sh(3 * c.N);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(static)
    for (i64 k = 0; k < c.N; ++k)
        for (int a = 0; a < 3; ++a) sh[3 * k + a] = cpoly_shift(c.basis_maxdepth, 2, c.P[3 * k + a]);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 256)
    for (i64 i = lo; i < hi; ++i) {
        int fi[3];
        function_index(c, i, fi);
        float oc[3], w;
        for (int a = 0; a < 3; ++a) center_width_f(fi[a], oc[a], w);
        float v[3] = {0, 0, 0};
        for (int j = 0; j < 27; ++j) {
            int nb = c.neighs[27 * i + j];
            if (nb == -1) continue;
            for (int k = 0; k < c.pnum[nb]; ++k) {
                i64 pt = c.pidx[nb] + k;
                float x = cpoly_value(sh[3 * pt], 2, oc[0]);
                float y = cpoly_value(sh[3 * pt + 1], 2, oc[1]);
                float z = cpoly_value(sh[3 * pt + 2], 2, oc[2]);
                float wgt = x * y * z;
                for (int a = 0; a < 3; ++a) v[a] = fmaf(wgt, c.Nn[3 * pt + a], v[a]);
            }
        }
        for (int a = 0; a < 3; ++a) c.vfield[3 * (i - lo) + a] = v[a];
    }
}

// ---------------------------------------------------------------------------
// a10-a11: divergence  (main.cu:1007-1141, 3383-3462)
// The finer depths accumulate float dot products in double in neighbour order;
// the coarse depths use the same accumulation (the reference reduces the same
// float terms with thrust::reduce in single precision).
// ---------------------------------------------------------------------------
static void divergence(Ctx& c) {
    const int D = c.D, res = c.res;
    const i64 M = c.M, lo = c.base[D];
    c.divergence.assign(M, 0.f);
    std::vector<int> fiD(3 * c.count[D]);
    for (i64 s = 0; s < c.count[D]; ++s) function_index(c, lo + s, &fiD[3 * s]);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 64)
    for (i64 i = 0; i < M; ++i) {
        int fi[3];
        function_index(c, i, fi);
        double val = 0;
        for (int j = 0; j < 27; ++j) {
            int nb = c.neighs[27 * i + j];
            if (nb == -1) continue;
            for (int k = 0; k < c.dnum[nb]; ++k) {
                i64 o = c.didx[nb] + k;
                const float* vo = &c.vfield[3 * o];
                const int* fo = &fiD[3 * o];
                float u0 = (float)c.ddot[(size_t)fi[0] + (size_t)fo[0] * res];
                float u1 = (float)c.ddot[(size_t)fi[1] + (size_t)fo[1] * res];
                float u2 = (float)c.ddot[(size_t)fi[2] + (size_t)fo[2] * res];
                float t = vo[0] * u0;
                t = fmaf(vo[1], u1, t);
                t = fmaf(vo[2], u2, t);
                val += (double)t;
            }
        }
        c.divergence[i] = (float)val;
    }
}

// ---------------------------------------------------------------------------
// Cascadic option (not the reference's, whose depths are independent systems):
// depth d's right-hand side loses the coarser depths' solution,
//   b'_i = b_i - sum_{d' < d} sum_{j in N27(ancestor_d'(i))} <grad B_i, grad B_j> x_j,
// over the 27 neighbours of i's ancestor at each coarser depth (the truncation
// the reference's divergence uses).  <grad B_i, grad B_j> is the product of the
// 1-D tables, dd_x t_y t_z + t_x dd_y t_z + t_x t_y dd_z with t = dot and
// dd = d2dot (the form of the same-depth stencil), so the 3x3x3 sum factors axis
// by axis.  In double with explicit fma, in the library's order (solve.cu,
// k_cascade_rhs): per ancestor d' = 0.., for ox: for oy:
//   zt[oy] = fma(t_z0, X0, fma(t_z1, X1, t_z2 * X2)), zd[oy] likewise with dd_z,
// then ytt, ydt, ytd (the same nesting over oy) and
//   acc = fma(dd_x[ox], ytt, fma(t_x[ox], ydt + ytd, acc)).
// The table entries for one axis depend on the node's and the neighbour's
// function indices only; a missing neighbour contributes X = 0.
// ---------------------------------------------------------------------------
static inline double dot3(double a0, double a1, double a2, double x0, double x1, double x2) {
    return std::fma(a0, x0, std::fma(a1, x1, a2 * x2));
}

static float cascade_rhs(const Ctx& c, i64 i, int d) {
    const size_t res = (size_t)c.res;
    int fi[3];
    function_index(c, i, fi);
    i64 anc[32];
    i64 a = i;
    for (int e = d; e > 0; --e) { a = c.parent[a]; anc[e - 1] = a; }
    double acc = 0;
    for (int e = 0; e < d; ++e) {
        // the ancestor's function index per axis; its neighbour at offset o - 1 has index + o - 1
        int fa[3];
        function_index(c, anc[e], fa);
        double t[3][3], dd[3][3];
        for (int k = 0; k < 3; ++k)
            for (int o = 0; o < 3; ++o) {
                const long fq = (long)fa[k] + o - 1;
                const long lo = (1l << e) - 1, hi = (2l << e) - 1;   // depth e's function indices
                t[k][o] = dd[k][o] = 0.0;
                if (fq >= lo && fq < hi) {
                    const size_t idx = (size_t)fi[k] + res * (size_t)fq;
                    t[k][o] = c.dot[idx];
                    dd[k][o] = c.d2dot[idx];
                }
            }
        for (int ox = 0; ox < 3; ++ox) {
            double zt[3], zd[3];
            for (int oy = 0; oy < 3; ++oy) {
                double X[3];
                for (int oz = 0; oz < 3; ++oz) {
                    const int q = c.neighs[27 * anc[e] + 9 * ox + 3 * oy + oz];
                    X[oz] = q != -1 ? (double)c.x[q] : 0.0;
                }
                zt[oy] = dot3(t[2][0], t[2][1], t[2][2], X[0], X[1], X[2]);
                zd[oy] = dot3(dd[2][0], dd[2][1], dd[2][2], X[0], X[1], X[2]);
            }
            const double ytt = dot3(t[1][0], t[1][1], t[1][2], zt[0], zt[1], zt[2]);
            const double ydt = dot3(dd[1][0], dd[1][1], dd[1][2], zt[0], zt[1], zt[2]);
            const double ytd = dot3(t[1][0], t[1][1], t[1][2], zd[0], zd[1], zd[2]);
            acc = std::fma(dd[0][ox], ytt, std::fma(t[0][ox], ydt + ytd, acc));
        }
    }
    return (float)((double)c.divergence[i] - acc);
}

// ---------------------------------------------------------------------------
// a12-a13: per-depth Laplacian and CG  (main.cu:1143-1332, CG_CUDA.cuh:186-509)
// mode 0: reference schedule (x0=0, stop when float(r.r) <= 1e-5f*1e-5f or after
//         max_iter iterations).  mode 1: relative residual ||r|| <= tol*||b||.
// ---------------------------------------------------------------------------
static int solve(Ctx& c, int mode, double tol, int max_iter) {
    const int D = c.D;
    if (c.cascadic && c.dot.empty()) return -1;   // the cross-depth products need the full tables
    c.x.assign(c.M, 0.f);
    c.cg_iters.assign(D + 1, 0);
    c.cg_rr.assign(D + 1, 0.f);
    for (int d = 0; d <= D; ++d) {
        const i64 lo = c.base[d], n = c.count[d];
        const float* st = &c.stencil[27 * d];
        std::vector<float> r(n), p(n), Ax(n), xx(n, 0.f);
        const float* b = &c.divergence[lo];
        std::vector<float> rhs;
        if (c.cascadic) {
            rhs.resize(n);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(static)
            for (i64 i = 0; i < n; ++i) rhs[i] = cascade_rhs(c, lo + i, d);
            b = rhs.data();
        }
        auto spmv = [&](const std::vector<float>& in, std::vector<float>& out) {
#pragma omp parallel for num_threads(omp_threads(c)) schedule(static)
            for (i64 i = 0; i < n; ++i) {
                float o = 0.f;
                for (int j = 0; j < 27; ++j) {
                    int nb = c.neighs[27 * (lo + i) + j];
                    if (nb == -1 || st[j] == 0.f) continue;
                    o = fmaf(st[j], in[nb - lo], o);
                }
                out[i] = o;
            }
        };
        auto dotd = [&](const std::vector<float>& a, const std::vector<float>& bb) {
            double s = 0;
#pragma omp parallel for num_threads(omp_threads(c)) reduction(+ : s) schedule(static)
            for (i64 i = 0; i < n; ++i) s += (double)(a[i] * bb[i]);
            return s;
        };
        for (i64 i = 0; i < n; ++i) r[i] = b[i];
        // r = b - A*0: A*0 = 0 so r stays b
        float r1 = (float)dotd(r, r), r0 = 0.f;
        const float tol2 = 1e-5f * 1e-5f;
        double bnorm2 = 0;
        for (i64 i = 0; i < n; ++i) bnorm2 += (double)b[i] * (double)b[i];
        auto done = [&](float rr) {
            if (mode == 0) return !(rr > tol2);
            return (double)rr <= tol * tol * bnorm2;
        };
        int k = 1;
        while (!done(r1) && k <= max_iter) {
            if (k > 1) {
                float beta = r1 / r0;
                for (i64 i = 0; i < n; ++i) p[i] = fmaf(beta, p[i], r[i]);
            } else {
                for (i64 i = 0; i < n; ++i) p[i] = r[i];
            }
            spmv(p, Ax);
            double pq = dotd(p, Ax);
            float a = (float)((double)r1 / pq);
            float na = -a;
            for (i64 i = 0; i < n; ++i) { xx[i] = fmaf(a, p[i], xx[i]); r[i] = fmaf(na, Ax[i], r[i]); }
            r0 = r1;
            r1 = (float)dotd(r, r);
            ++k;
        }
        c.cg_iters[d] = k - 1;
        c.cg_rr[d] = r1;
        for (i64 i = 0; i < n; ++i) c.x[lo + i] = xx[i];
    }
    return 0;
}

// ---------------------------------------------------------------------------
// a14: implicit function at the points and the iso-value (main.cu:1334-1381,
// 3480-3499)
// ---------------------------------------------------------------------------
static inline float eval_at(const Ctx& c, i64 node, const float q[3], float val) {
    for (int j = 0; j < 27; ++j) {
        int nb = c.neighs[27 * node + j];
        if (nb == -1) continue;
        int fi[3];
        function_index(c, nb, fi);
        float vx = cpoly_value(c.basis[fi[0]], 3, q[0]);
        float vy = cpoly_value(c.basis[fi[1]], 3, q[1]);
        float vz = cpoly_value(c.basis[fi[2]], 3, q[2]);
        val = fmaf(c.x[nb] * vx * vy, vz, val);
    }
    return val;
}
static void point_values(Ctx& c) {
    c.point_value.assign(c.N, 0.f);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(static)
    for (i64 k = 0; k < c.N; ++k) {
        i64 node = c.point_node[k];
        float val = 0.f;
        const float* q = &c.P[3 * k];
        while (node != -1) {
            val = eval_at(c, node, q, val);
            node = c.parent[node];
        }
        c.point_value[k] = val;
    }
    double s = 0;
    for (i64 k = 0; k < c.N; ++k) s += c.point_value[k];
    c.iso = (float)s / (float)c.N;
}

// ---------------------------------------------------------------------------
// FP64 run (precision study; not a stage of the reference, which computes in
// FP32 apart from its inner-product tables).  The same octree, normalised points
// and FP64 inner-product tables; everything after them in double: the splat
// with the closed-form B-spline F/F(0) (F the quadratic B-spline of support
// [-1.5, 1.5], F(0) = 3/4: the function GaussianApproximation builds,
// PPolynomial.inl:384-423), the divergence (main.cu:1007-1141 semantics), the
// stencil with the same drop rule (main.cu:1143-1213), CG per depth from x0 = 0
// to ||r|| <= tol ||b||, the implicit function at the points and the iso-value.
// ---------------------------------------------------------------------------
static inline double bspline_norm(double t) {
    t = std::fabs(t);
    if (t < 0.5) return (0.75 - t * t) / 0.75;
    if (t < 1.5) {
        const double u = 1.5 - t;
        return 0.5 * u * u / 0.75;
    }
    return 0.0;
}

static void fp64_run(Ctx& c, double tol) {
    const int D = c.D, res = c.res;
    const i64 M = c.M, lo = c.base[D], nD = c.count[D];
    const double sD = (double)(1 << D);
    // splat
    c.vfield64.assign(3 * nD, 0.0);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 256)
    for (i64 i = lo; i < lo + nD; ++i) {
        int fi[3];
        function_index(c, i, fi);
        double oc[3], w;
        for (int a = 0; a < 3; ++a) center_width_d(fi[a], oc[a], w);
        double v[3] = {0, 0, 0};
        for (int j = 0; j < 27; ++j) {
            const int nb = c.neighs[27 * i + j];
            if (nb == -1) continue;
            for (int k = 0; k < c.pnum[nb]; ++k) {
                const i64 pt = c.pidx[nb] + k;
                const double wgt = bspline_norm((oc[0] - c.P[3 * pt]) * sD) * bspline_norm((oc[1] - c.P[3 * pt + 1]) * sD) *
                                   bspline_norm((oc[2] - c.P[3 * pt + 2]) * sD);
                for (int a = 0; a < 3; ++a) v[a] += wgt * (double)c.Nn[3 * pt + a];
            }
        }
        for (int a = 0; a < 3; ++a) c.vfield64[3 * (i - lo) + a] = v[a];
    }
    // divergence
    std::vector<int> fiD(3 * nD);
    for (i64 s = 0; s < nD; ++s) function_index(c, lo + s, &fiD[3 * s]);
    c.divergence64.assign(M, 0.0);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 64)
    for (i64 i = 0; i < M; ++i) {
        int fi[3];
        function_index(c, i, fi);
        double val = 0;
        for (int j = 0; j < 27; ++j) {
            const int nb = c.neighs[27 * i + j];
            if (nb == -1) continue;
            for (int k = 0; k < c.dnum[nb]; ++k) {
                const i64 o = c.didx[nb] + k;
                const int* fo = &fiD[3 * o];
                val += c.vfield64[3 * o] * c.ddot[(size_t)fi[0] + (size_t)fo[0] * res] +
                       c.vfield64[3 * o + 1] * c.ddot[(size_t)fi[1] + (size_t)fo[1] * res] +
                       c.vfield64[3 * o + 2] * c.ddot[(size_t)fi[2] + (size_t)fo[2] * res];
            }
        }
        c.divergence64[i] = val;
    }
    // CG per depth in double
    c.x64.assign(M, 0.0);
    c.cg_iters64.assign(D + 1, 0);
    for (int d = 0; d <= D; ++d) {
        const i64 dlo = c.base[d], n = c.count[d];
        const double* st = &c.stencil64[27 * d];
        std::vector<double> r(n), p(n), q(n), xx(n, 0.0);
        for (i64 i = 0; i < n; ++i) r[i] = c.divergence64[dlo + i];
        auto dot = [&](const std::vector<double>& a, const std::vector<double>& b) {
            double s = 0;
#pragma omp parallel for num_threads(omp_threads(c)) reduction(+ : s) schedule(static)
            for (i64 i = 0; i < n; ++i) s += a[i] * b[i];
            return s;
        };
        const double bb = dot(r, r);
        double rr = bb, rr0 = 0;
        int k = 1;
        while (rr > tol * tol * bb && k <= 100000) {
            if (k == 1) p = r;
            else {
                const double beta = rr / rr0;
                for (i64 i = 0; i < n; ++i) p[i] = r[i] + beta * p[i];
            }
#pragma omp parallel for num_threads(omp_threads(c)) schedule(static)
            for (i64 i = 0; i < n; ++i) {
                double o = 0;
                for (int j = 0; j < 27; ++j) {
                    const int nb = c.neighs[27 * (dlo + i) + j];
                    if (nb != -1 && st[j] != 0.0) o += st[j] * p[nb - dlo];
                }
                q[i] = o;
            }
            const double al = rr / dot(p, q);
            for (i64 i = 0; i < n; ++i) {
                xx[i] += al * p[i];
                r[i] -= al * q[i];
            }
            rr0 = rr;
            rr = dot(r, r);
            ++k;
        }
        c.cg_iters64[d] = k - 1;
        for (i64 i = 0; i < n; ++i) c.x64[dlo + i] = xx[i];
    }
    // implicit function at the points, iso-value
    c.point_value64.assign(c.N, 0.0);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(static)
    for (i64 k = 0; k < c.N; ++k) {
        i64 node = c.point_node[k];
        double val = 0.0;
        const float* q = &c.P[3 * k];
        while (node != -1) {
            for (int j = 0; j < 27; ++j) {
                const int nb = c.neighs[27 * node + j];
                if (nb == -1) continue;
                int fi[3];
                function_index(c, nb, fi);
                double v = c.x64[nb];
                for (int a = 0; a < 3; ++a) {
                    double cc, w;
                    center_width_d(fi[a], cc, w);
                    v *= bspline_norm(((double)q[a] - cc) / w);
                }
                val += v;
            }
            node = c.parent[node];
        }
        c.point_value64[k] = val;
    }
    double s = 0;
    for (i64 k = 0; k < c.N; ++k) s += c.point_value64[k];
    c.iso64 = s / (double)c.N;
}

// ---------------------------------------------------------------------------
// a15-a20: octree vertices/edges/faces, marching cubes, subdivision
// (main.cu:1403-2986, 2994-3245, 3504-4566)
// ---------------------------------------------------------------------------
struct NodeView {     // uniform access to real nodes and rebuilt (virtual) nodes
    const Ctx* c;
    i64 M;            // NodeArray_sz
    // virtual arrays
    std::vector<i64> vkey;
    std::vector<int> vparent, vchildren, vneighs, vdepth, vvertices, vedges;
    std::vector<float> vcenter;
    std::vector<int> is_root, replaced;
    int rootId = -1;  // single-root mode: id of the replaced real node
};

static inline void node_center(u64 key, int d, int D, float cen[3]) {  // getNodeCenterAllDepth
    int xyz[3];
    node_coords(key, d, D, xyz);
    for (int a = 0; a < 3; ++a) cen[a] = (float)(2 * xyz[a] + 1) / (float)(1 << (d + 1));
}
static inline double sqdist(const float* a, const float* b) {
    float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return (double)(dx * dx + dy * dy + dz * dz);
}

// the finest-lattice edge a vertex lies on: its lower corner's lattice coordinates (corner
// positions are node centres +- half widths, dyadic, so pos * 2^D is an exact integer) and
// the edge's axis.  Not a reference quantity: it identifies the vertices that the weld
// option (one vertex per lattice edge across subdivision batches) merges.
static inline i64 lattice_edge_key(const float* p1, const float* p2, int dim, int D) {
    const float s = (float)(1 << D);
    i64 key = 0;
    for (int i = 0; i < 3; ++i) {
        const float lo = (i == dim) ? std::min(p1[i], p2[i]) : p1[i];
        key = (key << 20) | (i64)std::llround((double)lo * s);
    }
    return key * 3 + dim;
}

static void append_batch(Ctx& c, const std::vector<float>& vbuf, const std::vector<int>& tbuf,
                         const std::vector<i64>& kbuf) {
    int prev = (int)(c.mesh.v.size() / 3);
    c.mesh.v.insert(c.mesh.v.end(), vbuf.begin(), vbuf.end());
    c.mesh.vkey.insert(c.mesh.vkey.end(), kbuf.begin(), kbuf.end());
    for (int t : tbuf) c.mesh.f.push_back(t + prev);
    c.batch_tri.push_back((i64)tbuf.size() / 3);
}

// interpolatePoint (main.cu:2584-2597)
static inline void interpolate(const float* p1, const float* p2, int dim, float v1, float v2, float* out) {
    for (int i = 0; i < 3; ++i) if (i != dim) out[i] = p1[i];
    float pivot = v1 / (v1 - v2);
    float another = 1 - pivot;
    out[dim] = fmaf(p2[dim], pivot, p1[dim] * another);
}

static void marching_cubes(Ctx& c) {
    const int D = c.D;
    const i64 M = c.M;
    c.mesh.v.clear(); c.mesh.f.clear(); c.mesh.vkey.clear(); c.batch_tri.clear();
    std::vector<float> cen(3 * M);
    for (i64 i = 0; i < M; ++i) node_center((u64)c.key[i], c.depth[i], D, &cen[3 * i]);
    std::vector<int> nodeVert(8 * M, 0), nodeEdge(12 * M, 0), nodeFace(6 * M, 0);
    // --- vertices of every depth (initVertexOwner main.cu:1438-1495) ---
    struct Vtx { float pos[3]; int owner, kind, depth; };
    std::vector<Vtx> V;
    {
        // owner tests in parallel; collected in node order (the copy_if ordering)
        std::vector<unsigned char> own_mask(M, 0);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 1024)
        for (i64 i = 1; i < M; ++i) {
            int d = c.depth[i];
            float hw = 1.0f / (1 << (d + 1)), W = 1.0f / (1 << d), W2 = W * W;
            const float* nc = &cen[3 * i];
            unsigned m = 0;
            for (int j = 0; j < 8; ++j) {
                float vp[3] = {nc[0] + (2 * (j & 1) - 1) * hw, nc[1] + (2 * ((j & 2) >> 1) - 1) * hw,
                               nc[2] + (2 * ((j & 4) >> 2) - 1) * hw};
                i64 ownK = 0x7fffffff; int own = -1;
                for (int k = 0; k < 27; ++k) {
                    int nb = c.neighs[27 * i + k];
                    if (nb == -1) continue;
                    if (sqdist(vp, &cen[3 * nb]) < W2 && ownK > c.key[nb]) { ownK = c.key[nb]; own = nb; }
                }
                if (own == i) m |= 1u << j;
            }
            own_mask[i] = (unsigned char)m;
        }
        for (i64 i = 1; i < M; ++i) {
            if (!own_mask[i]) continue;
            int d = c.depth[i];
            float hw = 1.0f / (1 << (d + 1));
            const float* nc = &cen[3 * i];
            for (int j = 0; j < 8; ++j) {
                if (!((own_mask[i] >> j) & 1)) continue;
                Vtx v;
                v.pos[0] = nc[0] + (2 * (j & 1) - 1) * hw;
                v.pos[1] = nc[1] + (2 * ((j & 2) >> 1) - 1) * hw;
                v.pos[2] = nc[2] + (2 * ((j & 4) >> 2) - 1) * hw;
                v.owner = (int)i; v.kind = j; v.depth = d;
                V.push_back(v);
            }
        }
    }
    const i64 NV = (i64)V.size();
    // back-links (maintainVertexNodePointerNonAtomic main.cu:1640-1682); every slot has one owner
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 1024)
    for (i64 v = 0; v < NV; ++v) {
        int o = V[v].owner, d = c.depth[o];
        float W = 1.0f / (1 << d), W2 = W * W;
        for (int k = 0; k < 27; ++k) {
            int nb = c.neighs[27 * (i64)o + k];
            if (nb == -1) continue;
            const float* nc = &cen[3 * nb];
            if (!(sqdist(V[v].pos, nc) < W2)) continue;
            int idx = 0;
            if (nc[0] - V[v].pos[0] < 0) idx |= 1;
            if (nc[2] - V[v].pos[2] < 0) idx |= 4;
            if (nc[1] - V[v].pos[1] < 0) idx += (idx & 1) ? 1 : 3;
            nodeVert[8 * (i64)nb + idx] = (int)v + 1;
        }
    }
    // --- edges at depth D (initEdgeArray main.cu:1795-1862) ---
    struct Edg { int kind, owner; };
    std::vector<Edg> E;
    auto edge_center = [](const float* nc, float hw, int kind, float* ec) {
        int o = kind >> 2, off[2] = {kind & 1, (kind & 2) >> 1}, dim = 0;
        for (int k = 0; k < 3; ++k) {
            int m = 0;
            if (o != k) { m = 2 * off[dim] - 1; ++dim; }
            ec[k] = nc[k] + m * hw;
        }
    };
    {
        std::vector<unsigned short> emask(M - c.base[D], 0);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 1024)
        for (i64 i = c.base[D]; i < M; ++i) {
            float hw = 1.0f / (1 << (D + 1)), W = 1.0f / (1 << D), W2 = W * W;
            unsigned m = 0;
            for (int j = 0; j < 12; ++j) {
                float ec[3];
                edge_center(&cen[3 * i], hw, j, ec);
                i64 ownK = 0x7fffffff; int own = -1;
                for (int k = 0; k < 27; ++k) {
                    int nb = c.neighs[27 * i + k];
                    if (nb == -1) continue;
                    if (sqdist(ec, &cen[3 * nb]) < W2 && ownK > c.key[nb]) { ownK = c.key[nb]; own = nb; }
                }
                if (own == i) m |= 1u << j;
            }
            emask[i - c.base[D]] = (unsigned short)m;
        }
        for (i64 i = c.base[D]; i < M; ++i)
            for (int j = 0; j < 12; ++j)
                if ((emask[i - c.base[D]] >> j) & 1) E.push_back({j, (int)i});
    }
    // (maintainEdgeNodePointer main.cu:2021-2082)
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 1024)
    for (i64 e = 0; e < (i64)E.size(); ++e) {
        int o = E[e].owner;
        float hw = 1.0f / (1 << (D + 1)), W = 1.0f / (1 << D), W2 = W * W;
        float ec[3];
        edge_center(&cen[3 * (i64)o], hw, E[e].kind, ec);
        int orient = E[e].kind >> 2;
        for (int k = 0; k < 27; ++k) {
            int nb = c.neighs[27 * (i64)o + k];
            if (nb == -1) continue;
            const float* nc = &cen[3 * nb];
            if (!(sqdist(ec, nc) < W2)) continue;
            int idx = orient << 2, dim = 0;
            for (int a = 0; a < 3; ++a)
                if (a != orient) { if (nc[a] - ec[a] < 0) idx |= (1 << dim); ++dim; }
            nodeEdge[12 * (i64)nb + idx] = (int)e + 1;
        }
    }
    // --- faces of every depth (initFaceArray main.cu:2827-2899) ---
    struct Fac { int kind, owner, hasParent; };
    std::vector<Fac> Fa;
    {
        std::vector<unsigned char> fmask(M, 0);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 1024)
        for (i64 i = 0; i < M; ++i) {
            int d = c.depth[i];
            float hw = 1.0f / (1 << (d + 1)), W = 1.0f / (1 << d), W2 = W * W;
            unsigned m = 0;
            for (int j = 0; j < 6; ++j) {
                float fc[3] = {cen[3 * i], cen[3 * i + 1], cen[3 * i + 2]};
                fc[j >> 1] += (2 * (j & 1) - 1) * hw;
                i64 ownK = 0x7fffffff; int own = -1;
                for (int k = 0; k < 27; ++k) {
                    int nb = c.neighs[27 * i + k];
                    if (nb == -1) continue;
                    if (sqdist(fc, &cen[3 * nb]) < W2 && ownK > c.key[nb]) { ownK = c.key[nb]; own = nb; }
                }
                if (own == i) m |= 1u << j;
            }
            fmask[i] = (unsigned char)m;
        }
        for (i64 i = 0; i < M; ++i) {
            if (!fmask[i]) continue;
            int d = c.depth[i];
            int son = (int)((c.key[i] >> (3 * (D - d))) & 7);
            for (int j = 0; j < 6; ++j) {
                if (!((fmask[i] >> j) & 1)) continue;
                int hp = (c.parent[i] == -1) ? -1 : (parentFaceKind[son][j] != -1 ? 1 : -1);
                Fa.push_back({j, (int)i, hp});
            }
        }
    }
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 1024)
    for (i64 f = 0; f < (i64)Fa.size(); ++f) {  // maintainFaceNodePointer main.cu:2908-2955
        int o = Fa[f].owner, d = c.depth[o];
        float hw = 1.0f / (1 << (d + 1)), W = 1.0f / (1 << d), W2 = W * W;
        float fc[3] = {cen[3 * (i64)o], cen[3 * (i64)o + 1], cen[3 * (i64)o + 2]};
        int orient = Fa[f].kind >> 1;
        fc[orient] += (2 * (Fa[f].kind & 1) - 1) * hw;
        for (int k = 0; k < 27; ++k) {
            int nb = c.neighs[27 * (i64)o + k];
            if (nb == -1) continue;
            const float* nc = &cen[3 * nb];
            if (!(sqdist(fc, nc) < W2)) continue;
            int idx = orient << 1;
            if (nc[orient] - fc[orient] < 0) ++idx;
            nodeFace[6 * (i64)nb + idx] = (int)f + 1;
        }
    }
    std::vector<int> faceHit(Fa.size(), 0);
    // --- vertex values (computeVertexImplicitFunctionValue main.cu:2259-2326) ---
    std::vector<float> vval(NV);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 256)
    for (i64 v = 0; v < NV; ++v) {
        const Vtx& vt = V[v];
        float val = 0.f;
        int node = vt.owner, d = vt.depth;
        int exceed = childrenVertexKind[vt.kind];
        if (node > 0) {
            while (node != -1) { val = eval_at(c, node, vt.pos, val); node = c.parent[node]; }
            node = vt.owner;
            while (d < D) {
                ++d;
                node = c.children[8 * (i64)node + exceed];
                if (node == -1) break;
                val = eval_at(c, node, vt.pos, val);
            }
        }
        vval[v] = val - c.iso;
    }
    // --- marching cubes on the finest nodes ---
    {
        std::vector<int> vexNums(E.size(), 0);
        for (size_t e = 0; e < E.size(); ++e) {
            int o = E[e].owner, k = E[e].kind;
            int v1 = nodeVert[8 * (i64)o + MC.edge_v[k][0]] - 1, v2 = nodeVert[8 * (i64)o + MC.edge_v[k][1]] - 1;
            if (vval[v1] * vval[v2] <= 0) vexNums[e] = 1;
        }
        std::vector<int> vexAddr(E.size());
        int nv = 0;
        for (size_t e = 0; e < E.size(); ++e) { vexAddr[e] = nv; nv += vexNums[e]; }
        std::vector<float> vbuf(3 * (size_t)nv);
        std::vector<i64> kbuf((size_t)nv);
        for (size_t e = 0; e < E.size(); ++e) {
            if (!vexNums[e]) continue;
            int o = E[e].owner, k = E[e].kind;
            int v1 = nodeVert[8 * (i64)o + MC.edge_v[k][0]] - 1, v2 = nodeVert[8 * (i64)o + MC.edge_v[k][1]] - 1;
            interpolate(V[v1].pos, V[v2].pos, k >> 2, vval[v1], vval[v2], &vbuf[3 * (size_t)vexAddr[e]]);
            kbuf[vexAddr[e]] = lattice_edge_key(V[v1].pos, V[v2].pos, k >> 2, D);
        }
        std::vector<int> tbuf;
        for (i64 i = c.base[D]; i < M; ++i) {
            int cat = 0;
            for (int j = 0; j < 8; ++j)
                if (vval[nodeVert[8 * i + j] - 1] < 0) cat |= 1 << j;
            int edgeHas[12] = {0};
            for (int t = 0; t < MC.tri_count[cat]; ++t)
                for (int q = 0; q < 3; ++q) {
                    int e = MC.tri_edges[cat][3 * t + q];
                    edgeHas[e] = 1;
                    tbuf.push_back(vexAddr[nodeEdge[12 * i + e] - 1]);
                }
            // surface-intersection marks up the face chain (main.cu:2736-2755)
            for (int j = 0; j < 6; ++j) {
                int mark = 0;
                for (int q = 0; q < 4; ++q) mark |= edgeHas[faceEdges[j][q]];
                if (!mark) continue;
                int parentNode = c.parent[i];
                int nowFace = nodeFace[6 * i + j] - 1;
                faceHit[nowFace] = 1;
                while (Fa[nowFace].hasParent != -1) {
                    nowFace = nodeFace[6 * (i64)parentNode + j] - 1;
                    parentNode = c.parent[parentNode];
                    faceHit[nowFace] = 1;
                }
            }
        }
        append_batch(c, vbuf, tbuf, kbuf);
    }
    // --- leaves above the finest depth (ProcessLeafNodesAtOtherDepth main.cu:2957-2986) ---
    c.has_tri.assign(c.base[D], 0);
    c.has_int.assign(c.base[D], 0);
    for (i64 i = 1; i < c.base[D]; ++i) {   // node 0 has no vertices of its own
        float v0 = vval[nodeVert[8 * i] - 1];
        int sign = v0 < 0 ? -1 : 1, ht = 0;
        for (int j = 1; j < 8; ++j)
            if (sign * vval[nodeVert[8 * i + j] - 1] < 0) { ht = 1; break; }
        c.has_tri[i] = ht;
        int hi = 0;
        for (int j = 0; j < 6; ++j)
            if (faceHit[nodeFace[6 * i + j] - 1]) { hi = 1; break; }
        c.has_int[i] = hi;
    }
    // ifSubdivide (main.cu:2988-2992): leaves with a sign change or a marked face
    std::vector<int> roots;
    for (i64 i = 0; i < c.base[D]; ++i)
        if (c.children[8 * i] == -1 && (c.has_tri[i] || c.has_int[i])) roots.push_back((int)i);
    c.subdivide_roots = (i64)roots.size();
    c.vcells[0] = c.vcells[1] = 0;
    for (int r : roots) c.vcells[0] += (i64)1 << (3 * (D - c.depth[r]));
    if (c.root_stride != 1) {
        std::vector<int> kept;
        if (c.root_stride > 1)
            for (size_t k = 0; k < roots.size(); k += (size_t)c.root_stride) kept.push_back(roots[k]);
        roots.swap(kept);
    }
    for (int r : roots) c.vcells[1] += (i64)1 << (3 * (D - c.depth[r]));
    if (roots.empty()) return;

    // working copy of the children pointers (the rebuild rewires them)
    std::vector<int> children = c.children;
    const float hwD = 1.0f / (1 << (D + 1)), WD = 1.0f / (1 << D), WD2 = WD * WD;

    // MC over one rebuilt array; 'first_D'..'nv_nodes' are its finest nodes
    auto run_batch = [&](NodeView& nv, i64 first_D, i64 nv_nodes) {
        const i64 MM = nv.M;
        auto is_virtual = [&](int id) { return id >= MM; };
        auto nb_of = [&](int id, int k) -> int {
            return is_virtual(id) ? nv.vneighs[27 * (i64)(id - MM) + k] : c.neighs[27 * (i64)id + k];
        };
        auto center_of = [&](int id) -> const float* {
            return is_virtual(id) ? &nv.vcenter[3 * (i64)(id - MM)] : &cen[3 * (i64)id];
        };
        // vertices owned by rebuilt finest nodes (initSubdivideVertexOwner main.cu:1501-1566)
        std::vector<Vtx> SV;
        std::vector<unsigned char> vmask(nv_nodes - first_D, 0);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 1024)
        for (i64 i = first_D; i < nv_nodes; ++i) {
            const float* ncen = &nv.vcenter[3 * i];
            unsigned m = 0;
            for (int j = 0; j < 8; ++j) {
                float vp[3] = {ncen[0] + (2 * (j & 1) - 1) * hwD, ncen[1] + (2 * ((j & 2) >> 1) - 1) * hwD,
                               ncen[2] + (2 * ((j & 4) >> 2) - 1) * hwD};
                i64 ownK = 0x7fffffff; int own = -1;
                for (int k = 0; k < 27; ++k) {
                    int nb = nv.vneighs[27 * i + k];
                    if (nb == -1 || !is_virtual(nb)) continue;
                    if (sqdist(vp, &nv.vcenter[3 * (i64)(nb - MM)]) < WD2) {
                        i64 kk = nv.vkey[nb - MM];
                        if (ownK > kk) { ownK = kk; own = nb; }
                    }
                }
                if (own == MM + i) m |= 1u << j;
            }
            vmask[i - first_D] = (unsigned char)m;
        }
        for (i64 i = first_D; i < nv_nodes; ++i) {
            const unsigned m = vmask[i - first_D];
            if (!m) continue;
            const float* ncen = &nv.vcenter[3 * i];
            for (int j = 0; j < 8; ++j) {
                if (!((m >> j) & 1)) continue;
                Vtx v;
                v.pos[0] = ncen[0] + (2 * (j & 1) - 1) * hwD;
                v.pos[1] = ncen[1] + (2 * ((j & 2) >> 1) - 1) * hwD;
                v.pos[2] = ncen[2] + (2 * ((j & 4) >> 2) - 1) * hwD;
                v.owner = (int)(MM + i); v.kind = j; v.depth = D;
                SV.push_back(v);
            }
        }
        // (maintainSubdivideVertexNodePointer main.cu:1684-1793)
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 1024)
        for (i64 v = 0; v < (i64)SV.size(); ++v) {
            int o = SV[v].owner;
            for (int k = 0; k < 27; ++k) {
                int nb = nv.vneighs[27 * (i64)(o - MM) + k];
                if (nb == -1) continue;
                const float* nc = center_of(nb);
                if (!(sqdist(SV[v].pos, nc) < WD2)) continue;
                int idx = 0;
                if (nc[0] - SV[v].pos[0] < 0) idx |= 1;
                if (nc[2] - SV[v].pos[2] < 0) idx |= 4;
                if (nc[1] - SV[v].pos[1] < 0) idx += (idx & 1) ? 1 : 3;
                if (is_virtual(nb)) nv.vvertices[8 * (i64)(nb - MM) + idx] = (int)v + 1;
            }
        }
        // edges (initSubdivideEdgeArray main.cu:1868-1943, maintainSubdivideEdgeNodePointer :2085-2153)
        std::vector<Edg> SE;
        std::vector<unsigned short> emask(nv_nodes - first_D, 0);
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 1024)
        for (i64 i = first_D; i < nv_nodes; ++i) {
            unsigned m = 0;
            for (int j = 0; j < 12; ++j) {
                float ec[3];
                edge_center(&nv.vcenter[3 * i], hwD, j, ec);
                i64 ownK = 0x7fffffff; int own = -1;
                for (int k = 0; k < 27; ++k) {
                    int nb = nv.vneighs[27 * i + k];
                    if (nb == -1 || !is_virtual(nb)) continue;
                    if (sqdist(ec, &nv.vcenter[3 * (i64)(nb - MM)]) < WD2) {
                        i64 kk = nv.vkey[nb - MM];
                        if (ownK > kk) { ownK = kk; own = nb; }
                    }
                }
                if (own == MM + i) m |= 1u << j;
            }
            emask[i - first_D] = (unsigned short)m;
        }
        for (i64 i = first_D; i < nv_nodes; ++i)
            for (int j = 0; j < 12; ++j)
                if ((emask[i - first_D] >> j) & 1) SE.push_back({j, (int)(MM + i)});
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 1024)
        for (i64 e = 0; e < (i64)SE.size(); ++e) {
            int o = SE[e].owner;
            float ec[3];
            edge_center(&nv.vcenter[3 * (i64)(o - MM)], hwD, SE[e].kind, ec);
            int orient = SE[e].kind >> 2;
            for (int k = 0; k < 27; ++k) {
                int nb = nv.vneighs[27 * (i64)(o - MM) + k];
                if (nb == -1) continue;
                const float* nc = center_of(nb);
                if (!(sqdist(ec, nc) < WD2)) continue;
                int idx = orient << 2, dim = 0;
                for (int a = 0; a < 3; ++a)
                    if (a != orient) { if (nc[a] - ec[a] < 0) idx |= (1 << dim); ++dim; }
                if (is_virtual(nb)) nv.vedges[12 * (i64)(nb - MM) + idx] = (int)e + 1;
            }
        }
        // values (computeSubdivideVertexImplicitFunctionValue main.cu:2328-2442)
        std::vector<float> sval(SV.size());
#pragma omp parallel for num_threads(omp_threads(c)) schedule(dynamic, 64)
        for (i64 v = 0; v < (i64)SV.size(); ++v) {
            float val = 0.f;
            int node = SV[v].owner;
            if (node > 0) {
                while (node != -1) {
                    for (int k = 0; k < 27; ++k) {
                        int nb = nb_of(node, k);
                        if (nb == -1) continue;
                        if (nv.rootId >= 0) { if (nb == MM) nb = nv.rootId; }
                        else if (nb >= MM && nv.is_root[nb - MM]) nb = nv.replaced[nb - MM];
                        if (nb >= MM) continue;   // rebuilt nodes carry no coefficient
                        int fi[3];
                        function_index(c, nb, fi);
                        float vx = cpoly_value(c.basis[fi[0]], 3, SV[v].pos[0]);
                        float vy = cpoly_value(c.basis[fi[1]], 3, SV[v].pos[1]);
                        float vz = cpoly_value(c.basis[fi[2]], 3, SV[v].pos[2]);
                        val = fmaf(c.x[nb] * vx * vy, vz, val);
                    }
                    node = is_virtual(node) ? nv.vparent[node - MM] : c.parent[node];
                }
            }
            sval[v] = val - c.iso;
        }
        std::vector<int> vexNums(SE.size(), 0), vexAddr(SE.size());
        for (size_t e = 0; e < SE.size(); ++e) {
            i64 o = SE[e].owner - MM; int k = SE[e].kind;
            int v1 = nv.vvertices[8 * o + MC.edge_v[k][0]] - 1, v2 = nv.vvertices[8 * o + MC.edge_v[k][1]] - 1;
            if (sval[v1] * sval[v2] <= 0) vexNums[e] = 1;
        }
        int nvx = 0;
        for (size_t e = 0; e < SE.size(); ++e) { vexAddr[e] = nvx; nvx += vexNums[e]; }
        if (nvx == 0) { c.batch_tri.push_back(0); return; }
        std::vector<float> vbuf(3 * (size_t)nvx);
        std::vector<i64> kbuf((size_t)nvx);
        for (size_t e = 0; e < SE.size(); ++e) {
            if (!vexNums[e]) continue;
            i64 o = SE[e].owner - MM; int k = SE[e].kind;
            int v1 = nv.vvertices[8 * o + MC.edge_v[k][0]] - 1, v2 = nv.vvertices[8 * o + MC.edge_v[k][1]] - 1;
            interpolate(SV[v1].pos, SV[v2].pos, k >> 2, sval[v1], sval[v2], &vbuf[3 * (size_t)vexAddr[e]]);
            kbuf[vexAddr[e]] = lattice_edge_key(SV[v1].pos, SV[v2].pos, k >> 2, D);
        }
        std::vector<int> tbuf;
        for (i64 i = first_D; i < nv_nodes; ++i) {
            int cat = 0;
            for (int j = 0; j < 8; ++j)
                if (sval[nv.vvertices[8 * i + j] - 1] < 0) cat |= 1 << j;
            for (int t = 0; t < MC.tri_count[cat]; ++t)
                for (int q = 0; q < 3; ++q)
                    tbuf.push_back(vexAddr[nv.vedges[12 * i + MC.tri_edges[cat][3 * t + q]] - 1]);
        }
        append_batch(c, vbuf, tbuf, kbuf);
    };

    auto rebuild_neighbours = [&](NodeView& nv, i64 lo, i64 hi, int d) {  // computeRebuildNeighbor
        const i64 MM = nv.M;
#pragma omp parallel for num_threads(omp_threads(c)) schedule(static)
        for (i64 i = lo; i < hi; ++i) {
            int son = (int)((nv.vkey[i] >> (3 * (D - d))) & 7);
            int par = nv.vparent[i];
            for (int j = 0; j < 27; ++j) {
                int np = (par < MM) ? c.neighs[27 * (i64)par + LUTparent[son][j]]
                                    : nv.vneighs[27 * (i64)(par - MM) + LUTparent[son][j]];
                int r = -1;
                if (np != -1)
                    r = (np < MM) ? children[8 * (i64)np + LUTchild[son][j]]
                                  : nv.vchildren[8 * (i64)(np - MM) + LUTchild[son][j]];
                nv.vneighs[27 * i + j] = r;
            }
        }
    };
    auto qpow8 = [](int e) { i64 r = 1; while (e-- > 0) r *= 8; return r; };

    // coarse roots one by one (main.cu:3886-4202)
    const int finerDepth = 3;
    size_t ri = 0;
    for (; ri < roots.size(); ++ri) {
        int root = roots[ri], rd = c.depth[root];
        if (rd >= finerDepth) break;
        i64 sz = (qpow8(D - rd + 1) - 1) / 7;
        NodeView nv; nv.c = &c; nv.M = M; nv.rootId = root;
        nv.vkey.assign(sz, 0); nv.vparent.assign(sz, 0); nv.vchildren.assign(8 * sz, 0);
        nv.vneighs.assign(27 * sz, 0); nv.vdepth.assign(sz, 0); nv.vvertices.assign(8 * sz, 0);
        nv.vedges.assign(12 * sz, 0); nv.vcenter.assign(3 * sz, 0.f);
        int rootParent = c.parent[root];
        int rootSon = (int)((c.key[root] >> (3 * (D - rd))) & 7);
        children[8 * (i64)rootParent + rootSon] = (int)M;
        nv.vparent[0] = rootParent;
        std::vector<i64> addr(D + 2, 0), num(D + 2, 0);
        for (int j = rd; j <= D; ++j) num[j] = qpow8(j - rd);
        for (int j = rd + 1; j <= D; ++j) addr[j] = addr[j - 1] + num[j - 1];
#pragma omp parallel for num_threads(omp_threads(c)) schedule(static)
        for (i64 i = 0; i < sz; ++i) {  // singleRebuildArray main.cu:3114-3155
            int rel = 0; i64 up = i * 7 + 1, b = 8;
            while (b <= up) { ++rel; b <<= 3; }
            int dep = rd + rel;
            i64 off = i - (qpow8(rel) - 1) / 7;
            for (int k = 0; k < 8; ++k)
                nv.vchildren[8 * i + k] = (dep < D) ? (int)(M + (qpow8(rel + 1) - 1) / 7 + (off << 3) + k) : -1;
            if (i != 0) nv.vparent[i] = (int)(M + (qpow8(rel - 1) - 1) / 7 + (off >> 3));
            nv.vkey[i] = c.key[root] | (i64)((u64)off << (3 * (D - dep)));
            nv.vdepth[i] = dep;
            node_center((u64)nv.vkey[i], dep, D, &nv.vcenter[3 * i]);
        }
        for (int j = rd; j <= D; ++j) rebuild_neighbours(nv, addr[j], addr[j] + num[j], j);
        run_batch(nv, addr[D], sz);
        children[8 * (i64)rootParent + rootSon] = root;
    }
    // finer roots, one batch per depth (main.cu:4204-4561)
    for (int bd = finerDepth; bd < D; ++bd) {
        std::vector<int> br;
        for (size_t k = ri; k < roots.size(); ++k) if (c.depth[roots[k]] == bd) br.push_back(roots[k]);
        if (br.empty()) continue;
        const i64 nr = (i64)br.size();
        std::vector<i64> dcount(D + 1, 0), daddr(D + 2, 0);
        for (int j = bd; j <= D; ++j) dcount[j] = nr * qpow8(j - bd);
        for (int j = 1; j <= D + 1; ++j) daddr[j] = daddr[j - 1] + dcount[j - 1];
        const i64 total = daddr[D + 1];
        NodeView nv; nv.c = &c; nv.M = M; nv.rootId = -1;
        nv.vkey.assign(total, 0); nv.vparent.assign(total, 0); nv.vchildren.assign(8 * total, 0);
        nv.vneighs.assign(27 * total, 0); nv.vdepth.assign(total, 0); nv.vvertices.assign(8 * total, 0);
        nv.vedges.assign(12 * total, 0); nv.vcenter.assign(3 * total, 0.f);
        nv.is_root.assign(total, 0); nv.replaced.assign(total, 0);
        for (i64 r = 0; r < nr; ++r) {  // wholeRebuildArray main.cu:3032-3112
            int root = br[r];
            i64 idx = daddr[bd] + r;
            nv.vkey[idx] = c.key[root];
            nv.vparent[idx] = c.parent[root];
            for (int k = 0; k < 8; ++k) nv.vchildren[8 * idx + k] = children[8 * (i64)root + k];
            nv.vdepth[idx] = bd;
            nv.is_root[idx] = 1;
            nv.replaced[idx] = root;
            node_center((u64)c.key[root], bd, D, &nv.vcenter[3 * idx]);
            int son = (int)((c.key[root] >> (3 * (D - bd))) & 7);
            children[8 * (i64)c.parent[root] + son] = (int)(M + idx);
            for (int dep = bd + 1; dep <= D; ++dep) {
                i64 nowIdx = daddr[dep] + r * qpow8(dep - bd);
                i64 cn = qpow8(dep - bd);
                for (i64 j = 0; j < cn; j += 8) {
                    i64 pIdx = daddr[dep - 1] + r * qpow8(dep - 1 - bd) + j / 8;
                    for (int k = 0; k < 8; ++k) {
                        i64 t = nowIdx + j + k;
                        nv.vkey[t] = nv.vkey[pIdx] | (i64)((u64)k << (3 * (D - dep)));
                        nv.vparent[t] = (int)(M + pIdx);
                        nv.vdepth[t] = dep;
                        nv.replaced[t] = root;
                        node_center((u64)nv.vkey[t], dep, D, &nv.vcenter[3 * t]);
                        nv.vchildren[8 * pIdx + k] = (int)(M + t);
                    }
                }
            }
        }
        for (int j = finerDepth; j <= D; ++j) rebuild_neighbours(nv, daddr[j], daddr[j] + dcount[j], j);
        run_batch(nv, daddr[D], total);
    }
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C interface (ctypes)
// ---------------------------------------------------------------------------
using namespace orc;
extern "C" {

void* orc_create(int depth, int threads) {
    init_static_tables();
    Ctx* c = new Ctx();
    c->D = depth;
    c->threads = threads;
    return c;
}
void orc_destroy(void* h) { delete (Ctx*)h; }

int orc_set_points(void* h, const float* xyz, const float* nrm, int64_t n) {
    Ctx* c = (Ctx*)h;
    if (n <= 0 || !xyz || !nrm) return 1;
    c->N = n;
    c->in_p.assign(xyz, xyz + 3 * n);
    c->in_n.assign(nrm, nrm + 3 * n);
    return 0;
}
int orc_build_octree(void* h) { build_octree(*(Ctx*)h); return 0; }
int orc_build_basis(void* h, int full_tables) { build_basis(*(Ctx*)h, full_tables != 0); return 0; }
int orc_vector_field(void* h) { vector_field(*(Ctx*)h); return 0; }
int orc_divergence(void* h) { divergence(*(Ctx*)h); return 0; }
int orc_solve(void* h, int mode, double tol, int max_iter) { return solve(*(Ctx*)h, mode, tol, max_iter); }
int orc_set_cascadic(void* h, int on) { ((Ctx*)h)->cascadic = on != 0; return 0; }
int orc_point_values(void* h) { point_values(*(Ctx*)h); return 0; }
// FP64 run after build_octree and build_basis(full tables): see fp64_run
int orc_fp64_run(void* h, double tol) {
    Ctx* c = (Ctx*)h;
    if (c->ddot.empty()) return -1;
    fp64_run(*c, tol);
    return 0;
}
int orc_marching_cubes(void* h) { marching_cubes(*(Ctx*)h); return 0; }
// timing samples: subdivide every stride-th root only (0: none); the default 1 is the full path
int orc_set_root_stride(void* h, int stride) { ((Ctx*)h)->root_stride = stride; return 0; }

// one call for the whole path, reference CG schedule
int orc_reconstruct(void* h, int mode, double tol, int max_iter) {
    Ctx* c = (Ctx*)h;
    build_octree(*c);
    build_basis(*c, true);
    vector_field(*c);
    divergence(*c);
    if (solve(*c, mode, tol, max_iter)) return -1;
    point_values(*c);
    marching_cubes(*c);
    return 0;
}

// generic array access: returns a pointer to internal storage and its element count
const void* orc_get(void* h, const char* name, int64_t* count) {
    Ctx* c = (Ctx*)h;
    std::string n(name);
#define RET(vec) do { *count = (int64_t)(vec).size(); return (vec).data(); } while (0)
    if (n == "points") RET(c->P);
    if (n == "normals") RET(c->Nn);
    if (n == "sort_idx") RET(c->sort_idx);
    if (n == "base") RET(c->base);
    if (n == "count") RET(c->count);
    if (n == "key") RET(c->key);
    if (n == "pidx") RET(c->pidx);
    if (n == "pnum") RET(c->pnum);
    if (n == "parent") RET(c->parent);
    if (n == "children") RET(c->children);
    if (n == "neighs") RET(c->neighs);
    if (n == "didx") RET(c->didx);
    if (n == "dnum") RET(c->dnum);
    if (n == "point_node") RET(c->point_node);
    if (n == "dot") RET(c->dot);
    if (n == "ddot") RET(c->ddot);
    if (n == "d2dot") RET(c->d2dot);
    if (n == "stencil") RET(c->stencil);
    if (n == "vfield") RET(c->vfield);
    if (n == "divergence") RET(c->divergence);
    if (n == "x") RET(c->x);
    if (n == "cg_iters") RET(c->cg_iters);
    if (n == "cg_rr") RET(c->cg_rr);
    if (n == "point_value") RET(c->point_value);
    if (n == "mesh_v") RET(c->mesh.v);
    if (n == "mesh_f") RET(c->mesh.f);
    if (n == "mesh_vkey") RET(c->mesh.vkey);
    if (n == "has_tri") RET(c->has_tri);
    if (n == "has_int") RET(c->has_int);
    if (n == "batch_tri") RET(c->batch_tri);
    if (n == "vfield64") RET(c->vfield64);
    if (n == "divergence64") RET(c->divergence64);
    if (n == "x64") RET(c->x64);
    if (n == "point_value64") RET(c->point_value64);
    if (n == "cg_iters64") RET(c->cg_iters64);
    if (n == "stencil64") RET(c->stencil64);
#undef RET
    if (n == "center") { *count = 3; return c->center; }
    if (n == "scale") { *count = 1; return &c->scale; }
    if (n == "iso") { *count = 1; return &c->iso; }
    if (n == "iso64") { *count = 1; return &c->iso64; }
    if (n == "subdivide_roots") { *count = 1; return &c->subdivide_roots; }
    if (n == "vcells") { *count = 2; return c->vcells; }
    *count = -1;
    return nullptr;
}

// replace an internal float array (stage-by-stage parity tests feed the same inputs)
int orc_set_f32(void* h, const char* name, const float* data, int64_t count) {
    Ctx* c = (Ctx*)h;
    std::string n(name);
    std::vector<float>* dst = nullptr;
    if (n == "vfield") dst = &c->vfield;
    else if (n == "divergence") dst = &c->divergence;
    else if (n == "x") dst = &c->x;
    else if (n == "iso") { c->iso = data[0]; return 0; }
    if (!dst) return 1;
    dst->assign(data, data + count);
    return 0;
}

// marching-cubes case table as generated for the oracle (tests compare it with
// the reference header and with the library's copy)
int orc_mc_table(int* counts, int* edges) {
    init_static_tables();
    for (int c = 0; c < 256; ++c) {
        counts[c] = MC.tri_count[c];
        for (int k = 0; k < 16; ++k) edges[16 * c + k] = MC.tri_edges[c][k];
    }
    return 0;
}
int orc_luts(int* lut_parent, int* lut_child) {
    init_static_tables();
    memcpy(lut_parent, LUTparent, sizeof LUTparent);
    memcpy(lut_child, LUTchild, sizeof LUTchild);
    return 0;
}

}  // extern "C"
