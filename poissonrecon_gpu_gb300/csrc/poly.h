// Piecewise polynomials in "starting polynomial" form with single-precision
// coefficients, restating the reference's host arithmetic (Polynomial.inl,
// PPolynomial.inl, FunctionData.inl).  Usable on host and device; the library
// is built with --fmad=false and host code with -ffp-contract=off, so both
// sides produce the reference's unfused IEEE results.
#pragma once
#include <cmath>

#include "common.cuh"

namespace prgpu {

#ifndef __CUDACC__
#define PRGPU_HD
#else
#define PRGPU_HD __host__ __device__
#endif

struct SPoly {
    float start;
    float c[5];
};

template <int CAP>
struct PP {
    int n = 0;
    int deg = 0;
    SPoly p[CAP];
};

// Polynomial::shift (Polynomial.inl:258-268)
PRGPU_HD inline void poly_shift(const float* c, int deg, float t, float* out) {
    for (int i = 0; i <= deg; ++i) out[i] = 0.f;
    for (int i = 0; i <= deg; ++i) {
        float temp = 1.f;
        for (int j = i; j >= 0; --j) {
            out[j] = out[j] + c[i] * temp;
            temp = temp * (-t * (float)j);
            temp = temp / (float)(i - j + 1);
        }
    }
}
PRGPU_HD inline float poly_eval(const float* c, int deg, float t) {
    float temp = 1.f, v = 0.f;
    for (int i = 0; i <= deg; ++i) { v = v + temp * c[i]; temp = temp * t; }
    return v;
}
// Polynomial::integral(tMin,tMax) (Polynomial.inl:81-92)
PRGPU_HD inline float poly_integral(const float* c, int deg, float tMin, float tMax) {
    float v = 0.f, t1 = tMin, t2 = tMax;
    for (int i = 0; i <= deg; ++i) {
        v = v + c[i] * (t2 - t1) / (float)(i + 1);
        t1 = t1 * tMin;
        t2 = t2 * tMax;
    }
    return v;
}

template <int CAP>
PRGPU_HD inline void pp_scale(const PP<CAP>& a, float s, PP<CAP>& q) {
    q = a;
    for (int k = 0; k < a.n; ++k) {
        q.p[k].start = a.p[k].start * s;
        float s2 = 1.0f;
        for (int i = 0; i <= a.deg; ++i) { q.p[k].c[i] = a.p[k].c[i] * s2; s2 = s2 / s; }
    }
}
template <int CAP>
PRGPU_HD inline void pp_shift(const PP<CAP>& a, float t, PP<CAP>& q) {
    q.n = a.n;
    q.deg = a.deg;
    for (int k = 0; k < a.n; ++k) {
        q.p[k].start = a.p[k].start + t;
        float o[5];
        poly_shift(a.p[k].c, a.deg, t, o);
        for (int i = 0; i < 5; ++i) q.p[k].c[i] = (i <= a.deg) ? o[i] : 0.f;
    }
}
// PPolynomial product: pairwise products, ordered by start (stable), equal starts summed
// (PPolynomial.inl:256-270 with set() at :94-104)
template <int CA, int CB, int CQ>
PRGPU_HD inline void pp_mul(const PP<CA>& a, const PP<CB>& b, PP<CQ>& q) {
    SPoly sp[CQ];
    int m = 0;
    const int dq = a.deg + b.deg;
    for (int x = 0; x < a.n; ++x)
        for (int y = 0; y < b.n; ++y) {
            SPoly r;
            r.start = a.p[x].start > b.p[y].start ? a.p[x].start : b.p[y].start;
            for (int k = 0; k < 5; ++k) r.c[k] = 0.f;
            for (int i = 0; i <= a.deg; ++i)
                for (int j = 0; j <= b.deg; ++j) r.c[i + j] = r.c[i + j] + a.p[x].c[i] * b.p[y].c[j];
            // stable insertion by start
            int z = m;
            while (z > 0 && (sp[z - 1].start - r.start) > 0.f) { sp[z] = sp[z - 1]; --z; }
            sp[z] = r;
            ++m;
        }
    q.n = 0;
    q.deg = dq;
    for (int k = 0; k < m; ++k) {
        if (q.n == 0 || sp[k].start != q.p[q.n - 1].start) q.p[q.n++] = sp[k];
        else for (int i = 0; i < 5; ++i) q.p[q.n - 1].c[i] = q.p[q.n - 1].c[i] + sp[k].c[i];
    }
}
// PPolynomial::integral(tMin,tMax) (PPolynomial.inl:158-174)
template <int CAP>
PRGPU_HD inline float pp_integral(const PP<CAP>& a, float tMin, float tMax) {
    int m = 1;
    float st = tMin, en = tMax, s, v = 0.f;
    if (tMin > tMax) { m = -1; st = tMax; en = tMin; }
    for (int i = 0; i < a.n && a.p[i].start < en; ++i) {
        s = st < a.p[i].start ? a.p[i].start : st;
        v = v + poly_integral(a.p[i].c, a.deg, s, en);
    }
    return v * (float)m;
}

// BinaryNode<double>::CenterAndWidth (BinaryNode.cuh:45-60)
PRGPU_HD inline void center_width_d(int idx, double& c, double& w) {
    int i = idx + 1, d = -1;
    while (i) { i >>= 1; d++; }
    int off = (idx + 1) - (1 << d);
    w = 1.0 / (double)(1 << d);
    c = (0.5 + off) * w;
}

// FunctionData::{dot,dDot,d2Dot}Product with normalize = 0 (FunctionData.inl:266-300)
struct InnerProducts {
    double dot, ddot, d2dot;
};
PRGPU_HD inline InnerProducts inner_products(const PP<4>& B, const PP<4>& dB, double c1, double w1, double c2,
                                             double w2, bool want_d2) {
    const float r = fabsf(B.p[0].start);
    const float lo = (float)(-2.0 * (double)r), hi = (float)(2.0 * (double)r);
    const float sc = (float)(w2 / w1), sh = (float)((c2 - c1) / w1);
    PP<4> g0, g;
    pp_scale(B, sc, g0);
    pp_shift(g0, sh, g);
    PP<16> prod;
    pp_mul(B, g, prod);
    InnerProducts ip;
    ip.dot = (double)pp_integral(prod, lo, hi) * w1;
    pp_mul(dB, g, prod);
    ip.ddot = (double)pp_integral(prod, lo, hi);
    ip.d2dot = 0;
    if (want_d2) {
        PP<4> dg0, dg;
        pp_scale(dB, sc, dg0);
        pp_shift(dg0, sh, dg);
        pp_mul(dB, dg, prod);
        ip.d2dot = (double)pp_integral(prod, lo, hi) / w2;
    }
    return ip;
}

// overlap test of setDotTables (FunctionData.inl:176-186); i is the larger index
PRGPU_HD inline bool supports_overlap(double t1, double t2, double c1, double w1, double c2, double w2) {
    double start1 = t1 * w1 + c1, end1 = t2 * w1 + c1;
    double start = t1 * w2 + c2, end = t2 * w2 + c2;
    if (start < start1) start = start1;
    if (end > end1) end = end1;
    return start < end;
}

}  // namespace prgpu
