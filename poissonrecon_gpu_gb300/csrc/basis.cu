// Basis functions and B-spline inner-product tables, computed on the GPU.
// Replaces FunctionData::set / setDotTables (FunctionData.inl:112-205) and the
// host table set-up in main.cu:3306-3359.
//
// The reference evaluates every table entry with single-precision polynomial
// arithmetic and stores the result in double; the kernels below restate that
// arithmetic operation for operation, so the values agree bit for bit.  Only
// the entries that the later stages read are materialised:
//   * the divergence reads <B_a', B_b> for a node a and a finest-depth node b
//     in the 3x3x3 block around a: 3*2^(D-d) entries per function index a at
//     depth d (prgpu "compact rows");
//   * the Laplacian reads same-depth entries with offset 0 or 1, which are
//     translation invariant: 27 stencil coefficients per depth.
// The full res x res tables are built only on request (parity tests).
#include <mutex>
#include <vector>

#include "context.h"
#include "poly.h"
#include "prims.cuh"

namespace prgpu {

// ---------------- host: the base function F/F(0) (PPolynomial.inl:384-423) ----
namespace {
struct HP {  // host piecewise polynomial of small size
    int n = 0, deg = 0;
    SPoly p[8];
};
HP moving_average(const HP& a, float radius) {
    SPoly sps[16];
    int m = 0;
    for (int k = 0; k < a.n; ++k) {
        float ip[5] = {0, 0, 0, 0, 0};
        for (int i = 0; i <= a.deg; ++i) ip[i + 1] = a.p[k].c[i] / (float)(i + 1);
        float at = poly_eval(ip, a.deg + 1, a.p[k].start);
        ip[0] = ip[0] - at;
        SPoly lo, hi;
        for (int i = 0; i < 5; ++i) lo.c[i] = hi.c[i] = 0.f;
        lo.start = a.p[k].start - radius;
        hi.start = a.p[k].start + radius;
        poly_shift(ip, a.deg + 1, -radius, lo.c);
        poly_shift(ip, a.deg + 1, radius, hi.c);
        for (int i = 0; i <= a.deg + 1; ++i) hi.c[i] = hi.c[i] * -1.0f;
        sps[m++] = lo;
        sps[m++] = hi;
    }
    // stable order by start, merge equal starts
    for (int i = 1; i < m; ++i) {
        SPoly t = sps[i];
        int z = i;
        while (z > 0 && (sps[z - 1].start - t.start) > 0.f) { sps[z] = sps[z - 1]; --z; }
        sps[z] = t;
    }
    HP q;
    q.deg = a.deg + 1;
    for (int k = 0; k < m; ++k) {
        if (q.n == 0 || sps[k].start != q.p[q.n - 1].start) q.p[q.n++] = sps[k];
        else for (int i = 0; i < 5; ++i) q.p[q.n - 1].c[i] = q.p[q.n - 1].c[i] + sps[k].c[i];
    }
    float div = 2 * radius;
    for (int k = 0; k < q.n; ++k)
        for (int i = 0; i <= q.deg; ++i) { q.p[k].c[i] = q.p[k].c[i] * 1.0f; q.p[k].c[i] = q.p[k].c[i] / div; }
    return q;
}
float hp_eval(const HP& a, float t) {
    float v = 0.f;
    for (int i = 0; i < a.n && t > a.p[i].start; ++i) v = v + poly_eval(a.p[i].c, a.deg, t);
    return v;
}
PP<4> to_pp(const HP& h) {
    PP<4> r;
    r.n = h.n;
    r.deg = h.deg;
    for (int k = 0; k < h.n; ++k) r.p[k] = h.p[k];
    return r;
}
}  // namespace

static PP<4> g_B, g_dB;
static std::once_flag g_B_once;

static void build_base_function() {
    HP c;  // ConstantFunction(0.5)
    c.n = 2;
    c.deg = 0;
    for (int k = 0; k < 2; ++k) for (int i = 0; i < 5; ++i) c.p[k].c[i] = 0.f;
    c.p[0].start = -0.5f; c.p[0].c[0] = 1.0f;
    c.p[1].start = 0.5f; c.p[1].c[0] = -1.0f;
    HP F = moving_average(moving_average(c, 0.5f), 0.5f);
    float f0 = hp_eval(F, 0.f);
    for (int k = 0; k < F.n; ++k)
        for (int i = 0; i <= F.deg; ++i) F.p[k].c[i] = F.p[k].c[i] / f0;
    g_B = to_pp(F);
    g_dB = g_B;
    g_dB.deg = g_B.deg - 1;
    for (int k = 0; k < g_B.n; ++k) {
        float o[5] = {0, 0, 0, 0, 0};
        for (int i = 0; i < g_B.deg; ++i) o[i] = g_B.p[k].c[i + 1] * (float)(i + 1);
        for (int i = 0; i < 5; ++i) g_dB.p[k].c[i] = o[i];
    }
}

// the base function and its derivative, built once (contexts may run on several host threads)
static void ensure_base_function() { std::call_once(g_B_once, build_base_function); }

static CPoly to_cpoly(const PP<4>& a) {
    CPoly r;
    for (int k = 0; k < 4; ++k) {
        r.start[k] = (k < a.n) ? a.p[k].start : 0.f;
        for (int i = 0; i < 4; ++i) r.c[k][i] = (k < a.n && i <= a.deg) ? a.p[k].c[i] : 0.f;
    }
    return r;
}

// 27 stencil coefficients per depth (GetLaplacianEntry main.cu:1143-1158, drop
// rule main.cu:1205): same-depth inner products depend only on the offset.
void host_stencils(int D, std::vector<float>& st) {
    ensure_base_function();
    st.assign(27 * (D + 1), 0.f);
    for (int d = 0; d <= D; ++d) {
        const double w = 1.0 / (double)(1 << d);
        double sdot[2], sd2[2];
        for (int delta = 0; delta <= 1; ++delta) {
            InnerProducts ip = inner_products(g_B, g_dB, 0.0, w, -delta * w, w, true);
            // inner_products(c1,w1,c2,w2) with c2-c1 = -delta*w gives the shift -delta
            sdot[delta] = ip.dot;
            sd2[delta] = ip.d2dot;
        }
        for (int j = 0; j < 27; ++j) {
            int dd[3] = {abs(j / 9 - 1), abs((j / 3) % 3 - 1), abs(j % 3 - 1)};
            if (d == 0 && (dd[0] | dd[1] | dd[2])) continue;
            double dt[3], d2[3];
            for (int a = 0; a < 3; ++a) { dt[a] = sdot[dd[a]]; d2[a] = sd2[dd[a]]; }
            double e = d2[0] * dt[1] * dt[2] + d2[1] * dt[0] * dt[2] + d2[2] * dt[0] * dt[1];
            st[27 * d + j] = (fabs(e) > (double)1e-6f) ? (float)e : 0.f;
        }
    }
}

// ------------------------------ kernels -------------------------------------
struct BasePack {
    PP<4> B, dB;
};

// baseFunctions[i] = baseFunction.scale(w).shift(c)  (FunctionData.inl:139-152)
__global__ void k_basis_functions(BasePack bp, int res, CPoly* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < res; i += gridDim.x * blockDim.x) {
        double c1, w1;
        center_width_d(i, c1, w1);
        PP<4> t, u;
        pp_scale(bp.B, (float)w1, t);
        pp_shift(t, (float)c1, u);
        CPoly r;
        for (int k = 0; k < 4; ++k) {
            r.start[k] = (k < u.n) ? u.p[k].start : 0.f;
            for (int q = 0; q < 4; ++q) r.c[k][q] = (k < u.n && q <= u.deg) ? u.p[k].c[q] : 0.f;
        }
        out[i] = r;
    }
}

// value of the reference's dDot table at [a + res*b] (FunctionData.inl:176-204):
// computed for the pair (max, min); the mirrored entry is negated and the
// diagonal holds the negated value.
__device__ __host__ inline double ddot_entry(const BasePack& bp, int a, int b, double t1, double t2) {
    int i = a > b ? a : b, j = a > b ? b : a;
    double ci, wi, cj, wj;
    center_width_d(i, ci, wi);
    center_width_d(j, cj, wj);
    if (!supports_overlap(t1, t2, ci, wi, cj, wj)) return 0.0;
    InnerProducts ip = inner_products(bp.B, bp.dB, ci, wi, cj, wj, false);
    if (fabs(ip.dot) < 1e-15) return 0.0;
    return (a > b) ? ip.ddot : -ip.ddot;
}

// compact rows: entry (d, x, u) holds ddot[a + res*b] for a = 2^d-1+x and the
// finest index b = 2^D-1+t, t = (x-1)*2^(D-d)+u, 0 <= u < 3*2^(D-d).  Every depth
// has 2^d rows of 3*2^(D-d) entries, 3*2^D in all, so depth d starts at d*3*2^D;
// all depths in one launch.
__global__ void k_ddot_rows(BasePack bp, int D, double t1, double t2, float* __restrict__ out) {
    const i64 per_depth = 3ll << D;
    const i64 n = (i64)(D + 1) * per_depth;
    for (i64 g = (i64)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (i64)gridDim.x * blockDim.x) {
        const int d = (int)(g / per_depth);
        const i64 e = g - (i64)d * per_depth;
        const i64 W = 3ll << (D - d);
        const i64 x = e / W, u = e - x * W;
        const i64 t = (x - 1) * (1ll << (D - d)) + u;
        float v = 0.f;
        if (t >= 0 && t < (1ll << D)) {
            int a = (int)((1ll << d) - 1 + x), b = (int)((1ll << D) - 1 + t);
            v = (float)ddot_entry(bp, a, b, t1, t2);
        }
        out[g] = v;
    }
}

// full res x res tables (parity output only), one thread per pair j <= i
__global__ void k_full_tables(BasePack bp, int res, double t1, double t2, double* __restrict__ dot,
                              double* __restrict__ ddot, double* __restrict__ d2dot) {
    const i64 npairs = (i64)res * (res + 1) / 2;
    for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < npairs; e += (i64)gridDim.x * blockDim.x) {
        // e -> (i, j) with j <= i
        i64 i = (i64)((sqrt(8.0 * (double)e + 1.0) - 1.0) / 2.0);
        while (i * (i + 1) / 2 > e) --i;
        while ((i + 1) * (i + 2) / 2 <= e) ++i;
        i64 j = e - i * (i + 1) / 2;
        double c1, w1, c2, w2;
        center_width_d((int)i, c1, w1);
        center_width_d((int)j, c2, w2);
        if (!supports_overlap(t1, t2, c1, w1, c2, w2)) continue;
        InnerProducts ip = inner_products(bp.B, bp.dB, c1, w1, c2, w2, true);
        if (fabs(ip.dot) < 1e-15) continue;
        i64 idx1 = i + (i64)res * j, idx2 = j + (i64)res * i;
        dot[idx1] = ip.dot;
        dot[idx2] = ip.dot;
        d2dot[idx1] = ip.d2dot;
        d2dot[idx2] = ip.d2dot;
        ddot[idx1] = ip.ddot;
        ddot[idx2] = -ip.ddot;   // i == j: the negated value, as in the reference
    }
}

// Cross-depth 1-D inner products for the cascadic solve.  For a node at depth d
// and a neighbour of its ancestor at depth e < d (k = d - e levels up), the 1-D
// pair (dot, d2dot) depends only on the node's position a in [0, 2^k) within the
// ancestor along the axis and the neighbour's offset o - 1, o in {0, 1, 2}: the
// centres enter inner_products only through (c2 - c1) / w1 and w2 / w1, which are
// exact in double.  The entry is the full table's value for (finer, coarser)
// (the same overlap test and |dot| < 1e-15 drop as k_full_tables), at
// off[d * (D + 1) + e] + o * 2^k + a.
__global__ void k_cascade_tables(BasePack bp, int D, double t1, double t2, const i64* __restrict__ off, i64 n,
                                 double2* __restrict__ tab) {
    for (i64 g = (i64)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (i64)gridDim.x * blockDim.x) {
        // locate the (d, e) table holding g
        int d = 1, e = 0;
        for (int dd = 1; dd <= D; ++dd)
            for (int ee = 0; ee < dd; ++ee)
                if (off[dd * (D + 1) + ee] <= g) { d = dd; e = ee; }
        const int k = d - e;
        const i64 r = g - off[d * (D + 1) + e];
        const int o = (int)(r >> k);
        const i64 a = r - ((i64)o << k);
        const double w1 = 1.0 / (double)(1ll << d), w2 = 1.0 / (double)(1ll << e);
        // ancestor at position 1, node at 2^k + a below it, neighbour at 1 + o - 1
        const double c1 = ((double)((1ll << k) + a) + 0.5) * w1;
        const double c2 = ((double)o + 0.5) * w2;
        double2 v = make_double2(0.0, 0.0);
        if (supports_overlap(t1, t2, c1, w1, c2, w2)) {
            InnerProducts ip = inner_products(bp.B, bp.dB, c1, w1, c2, w2, true);
            if (!(fabs(ip.dot) < 1e-15)) v = make_double2(ip.dot, ip.d2dot);
        }
        tab[g] = v;
    }
}

void ensure_cascade_tables(Ctx& c) {
    const int D = c.D;
    if (c.cascade_tab && (int)c.cascade_off.size() == (D + 1) * (D + 1) + 1) return;
    ensure_base_function();
    cudaStream_t s = c.stream;
    c.cascade_off.assign((size_t)(D + 1) * (D + 1) + 1, 0);
    i64 n = 0;
    for (int d = 0; d <= D; ++d)
        for (int e = 0; e <= D; ++e) {
            c.cascade_off[(size_t)d * (D + 1) + e] = n;
            if (e < d) n += 3ll << (d - e);
        }
    c.cascade_off[(size_t)(D + 1) * (D + 1)] = n;
    dfree(c.cascade_tab, s);
    c.cascade_tab = dalloc<double2>(std::max<i64>(n, 1), s);
    i64* doff = dalloc<i64>((i64)c.cascade_off.size(), s);
    CK(cudaMemcpyAsync(doff, c.cascade_off.data(), c.cascade_off.size() * sizeof(i64), cudaMemcpyHostToDevice, s));
    BasePack bp;
    bp.B = g_B;
    bp.dB = g_dB;
    const double t1 = g_B.p[0].start, t2 = g_B.p[g_B.n - 1].start;
    if (n > 0) {
        k_cascade_tables<<<grid_for(n, 128, 152 * 16), 128, 0, s>>>(bp, D, t1, t2, doff, n, c.cascade_tab);
        CK_LAUNCH();
    }
    dfree(doff, s);
}

void stage_basis(Ctx& c) {
    ensure_base_function();
    cudaStream_t s = c.stream;
    const int D = c.D;
    c.res = (1 << (D + 1)) - 1;
    // tables of another maxDepth (a batch may change it) are rebuilt on demand
    dfree(c.full_tables, s);
    if ((int)c.cascade_off.size() != (D + 1) * (D + 1) + 1) {
        dfree(c.cascade_tab, s);
        c.cascade_off.clear();
    }
    BasePack bp;
    bp.B = g_B;
    bp.dB = g_dB;
    dfree(c.basis, s);
    c.basis = dalloc<CPoly>(c.res, s);
    k_basis_functions<<<grid_for(c.res, 128), 128, 0, s>>>(bp, c.res, c.basis);
    CK_LAUNCH();
    // splat kernel: (F/F(0)).scale(2^-D)  (main.cu:3355-3359)
    {
        PP<4> sc;
        pp_scale(g_B, (float)(1.0 / (double)(1 << D)), sc);
        c.basis_maxdepth = to_cpoly(sc);
    }
    // compact divergence rows
    c.ddot_row_start.assign(D + 2, 0);
    for (int d = 0; d <= D; ++d) c.ddot_row_start[d + 1] = c.ddot_row_start[d] + (1ll << d) * (3ll << (D - d));
    dfree(c.ddot_div, s);
    c.ddot_div = dalloc<float>(c.ddot_row_start[D + 1], s);
    const double t1 = g_B.p[0].start, t2 = g_B.p[g_B.n - 1].start;
    k_ddot_rows<<<grid_for(c.ddot_row_start[D + 1], 64, 1ll << 20), 64, 0, s>>>(bp, D, t1, t2, c.ddot_div);
    CK_LAUNCH();
    host_stencils(D, c.stencil);
}

void stage_full_tables(Ctx& c) {
    ensure_base_function();
    cudaStream_t s = c.stream;
    const int res = (1 << (c.D + 1)) - 1;
    const i64 R2 = (i64)res * res;
    dfree(c.full_tables, s);
    c.full_tables = dalloc<double>(3 * R2, s);
    CK(cudaMemsetAsync(c.full_tables, 0, (size_t)(3 * R2) * sizeof(double), s));
    BasePack bp;
    bp.B = g_B;
    bp.dB = g_dB;
    const double t1 = g_B.p[0].start, t2 = g_B.p[g_B.n - 1].start;
    i64 npairs = (i64)res * (res + 1) / 2;
    k_full_tables<<<grid_for(npairs, 128, 152 * 32), 128, 0, s>>>(bp, res, t1, t2, c.full_tables, c.full_tables + R2,
                                                                  c.full_tables + 2 * R2);
    CK_LAUNCH();
}

}  // namespace prgpu
