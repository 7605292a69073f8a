"""The coarse part of the brick bounds (iso.cu: bern_fit, k_brick_xl, shell_poly, blossom_row,
k_brick_bound), restated on the CPU.

A basis function of depth d has its knots at multiples of its cell width 2^(D-d) (finest-lattice
units).  Over a brick of edge E (aligned to E) every function of width >= E is one quadratic piece
per axis, and over a leaf every ancestor function is one piece.  The bound sums those terms as a
tri-quadratic polynomial in Bernstein form, restricts the leaf's part to the brick by blossoming,
and bounds it by its coefficients' range; the finer shell terms stay as interval sums.  These
tests check each step in float64, and that the whole split encloses the exact corner values of
subdivided leaves of an oracle reconstruction.
"""
import numpy as np
import pytest

U = 2.0 ** -24


def _bspline(t):
    t = np.abs(t)
    return np.where(t < 0.5, (0.75 - t * t) / 0.75, np.where(t < 1.5, 0.5 * (1.5 - t) ** 2 / 0.75, 0.0))


def _basis(D, d, n, u):
    """B_{d,n} at finest-lattice coordinates u (support [(n-1)w, (n+2)w], w = 2^(D-d))."""
    w = 1 << (D - d)
    return _bspline(np.asarray(u, np.float64) / w - n - 0.5)


def _bern(k, K):
    k = np.asarray(k, np.float64)
    return np.stack([(K - k) ** 2, 2 * k * (K - k), k * k]) / float(K * K)


def _fit(v):
    """bern_fit: (b0, b1, b2, delta) of values v[0..K]."""
    K = len(v) - 1
    b = np.array([v[0], 2 * v[K // 2] - 0.5 * (v[0] + v[K]), v[K]])
    q = b @ _bern(np.arange(K + 1), K)
    delta = np.abs(q - v).max() * (1 + 2 ** -20) + 5 * U * np.abs(b).max()
    return b, delta


def _blossom(A, B, S):
    """blossom_row for q = 0, 1, 2: Bernstein coefficients over [0, S] -> over [A, B]."""
    a, b, s = A, B, S
    return np.array([[(s - a) ** 2, 2 * a * (s - a), a * a],
                     [(s - a) * (s - b), a * (s - b) + b * (s - a), a * b],
                     [(s - b) ** 2, 2 * b * (s - b), b * b]], np.float64) / float(S * S)


def test_functions_are_one_piece_where_the_bound_says():
    """Ancestors over the leaf and functions of width >= E over an aligned brick: the fit through
    three points reproduces the function at every lattice point."""
    D = 9
    for r in range(1, D):
        S = 1 << (D - r)
        E = min(S, 8)
        for Lc in (0, 1, (1 << r) // 2, (1 << r) - 1):
            for l in range(r + 1):
                anc = Lc >> (r - l)
                for t in range(3):
                    v = _basis(D, l, anc + t - 1, Lc * S + np.arange(S + 1))
                    b, delta = _fit(v)
                    assert delta <= 1e-12 + 5 * U * np.abs(b).max()
            for d in range(r + 1, D + 1):
                if (1 << (D - d)) < E:
                    continue
                for bb in range(S // E):
                    g0 = Lc * S + bb * E
                    m = g0 >> (D - d)
                    for N in range(m - 2, m + 3):
                        v = _basis(D, d, N, g0 + np.arange(E + 1))
                        b, delta = _fit(v)
                        assert delta <= 1e-12 + 5 * U * np.abs(b).max()


def test_fit_residual_covers_noise():
    """The tabulated values carry float noise; delta bounds the fit's residual at every corner and
    M = max|b| + delta bounds the values (bern_m)."""
    rng = np.random.default_rng(1)
    for K in (2, 4, 8, 64):
        for _ in range(200):
            c = rng.normal(size=3)
            v = c @ _bern(np.arange(K + 1), K) + rng.normal(scale=1e-3, size=K + 1)
            b, delta = _fit(v)
            q = b @ _bern(np.arange(K + 1), K)
            assert np.all(np.abs(q - v) <= delta)
            assert np.all(np.abs(v) <= np.abs(b).max() + delta)


def test_blossom_restriction_and_hull():
    """Blossoming gives the same polynomial over the brick, and the tensor coefficients' range
    encloses it at every corner of the brick."""
    rng = np.random.default_rng(2)
    for S in (16, 64, 1024):
        E = 8
        for _ in range(50):
            C = rng.normal(size=(3, 3, 3))
            b = rng.integers(0, S // E, size=3)
            T = [_blossom(int(bi) * E, (int(bi) + 1) * E, S) for bi in b]
            Cb = np.einsum("ai,bj,ck,ijk->abc", T[0], T[1], T[2], C)
            k = np.arange(E + 1)
            leaf = [_bern(int(bi) * E + k, S) for bi in b]
            brick = _bern(k, E)
            P_leaf = np.einsum("ijk,ia,jb,kc->abc", C, leaf[0], leaf[1], leaf[2])
            P_brick = np.einsum("ijk,ia,jb,kc->abc", Cb, brick, brick, brick)
            assert np.allclose(P_leaf, P_brick, atol=1e-12)
            assert Cb.min() - 1e-12 <= P_brick.min() and P_brick.max() <= Cb.max() + 1e-12
            for t in T:
                assert np.all(t >= 0) and np.allclose(t.sum(1), 1)


def test_separable_contraction_equals_the_term_sum():
    """shell_poly's three contractions over the 4^3 window grid give sum x Qx (x) Qy (x) Qz."""
    rng = np.random.default_rng(3)
    X = rng.normal(size=(4, 4, 4)) * (rng.random((4, 4, 4)) < 0.4)
    Q = [rng.normal(size=(4, 3)) for _ in range(3)]
    T1 = np.einsum("abn,nl->abl", X, Q[2])
    T2 = np.einsum("abl,bj->ajl", T1, Q[1])
    C = np.einsum("ajl,ai->ijl", T2, Q[0])
    direct = np.zeros((3, 3, 3))
    for a, b_, c in zip(*np.nonzero(X)):
        direct += X[a, b_, c] * np.einsum("i,j,l->ijl", Q[0][a], Q[1][b_], Q[2][c])
    assert np.allclose(C, direct)


def _window_axis(g0, B, Lc, r, d, D):
    sh, span = D - d, 1 << (d - r)
    llo = Lc * span
    vlo = (g0 >> sh) if g0 == (llo << sh) else ((g0 - 1) >> sh)
    vhi = (g0 + B - 1) >> sh
    return vlo - 1, vhi - vlo + 3, (vlo - 1 < llo) or (vhi + 1 >= llo + span)


def test_coarse_windows_fit_the_row_table():
    """At the depths of knot spacing >= E a window spans at most PW = 4 cells per axis."""
    n = 0
    for D in (8, 10, 12, 15):
        for r in range(0, D):
            S = 1 << (D - r)
            E = min(S, 8)
            for Lc in sorted({0, 1, (1 << r) - 1}):
                for b in sorted({0, 1, S // E - 1}):
                    g0 = Lc * S + b * E
                    for d in range(r + 1, D + 1):
                        if (1 << (D - d)) < E:
                            continue
                        wlo, ext, _ = _window_axis(g0, E, Lc, r, d, D)
                        assert ext <= 4
                        n += 1
    assert n > 100


@pytest.fixture(scope="module")
def torus_d8(oracle_mod):
    from poissonrecon_gpu_gb300 import shapes
    xyz, nrm = shapes.torus(60_000, seed=3)
    o = oracle_mod.Oracle(8)
    o.set_points(xyz, nrm)
    o.build_octree()
    o.build_basis(True)
    o.vector_field()
    o.divergence()
    o.solve(1, 1e-6, 10000)
    o.point_values()
    return o


def test_split_bound_encloses_the_corner_values(torus_d8):
    """For bricks of sampled coarse leaves of lattice edge >= 8: the coarse polynomial's hull plus
    the finer shell terms' interval sum encloses the exact corner values (float64, closed-form
    basis: the GPU's tabulated values differ by float noise, which bern_fit's residual carries)."""
    o, D = torus_d8, 8
    x = o.get("x").astype(np.float64)
    base, key = o.get("base"), o.get("key").astype(np.uint64)
    children = o.get("children")
    M = len(x)
    ch0 = children.reshape(M, -1)[:, 0] if children.size != M else children
    depth = np.searchsorted(base, np.arange(M), side="right") - 1

    def coords(k, d):
        c = np.zeros(3, np.int64)
        for l in range(1, d + 1):
            sh = 3 * (D - l)
            for a, bit in ((0, 2), (1, 1), (2, 0)):
                c[a] = (c[a] << 1) | int((int(k) >> (sh + bit)) & 1)
        return c

    tables = []
    for d in range(D + 1):
        ks = key[base[d]:base[d + 1]]
        cs = np.zeros((len(ks), 3), np.int64)
        for l in range(1, d + 1):
            sh = np.uint64(3 * (D - l))
            for a, bit in ((0, 2), (1, 1), (2, 0)):
                cs[:, a] = (cs[:, a] << 1) | ((ks >> (sh + np.uint64(bit))) & np.uint64(1)).astype(np.int64)
        xs = x[base[d]:base[d + 1]]
        tables.append((cs[xs != 0], xs[xs != 0]))
    leaves = [i for i in range(base[D]) if ch0[i] == -1 and depth[i] <= D - 3]
    rng = np.random.default_rng(0)
    checked = 0
    for L in rng.permutation(leaves)[:60]:
        r = int(depth[L])
        S = 1 << (D - r)
        E = min(S, 8)
        Lc = coords(key[L], r)
        for b in [rng.integers(0, S // E, size=3) for _ in range(2)]:
            g0 = Lc * S + b * E
            k = np.arange(E + 1)
            Fc = np.zeros((E + 1,) * 3)
            Ff = np.zeros((E + 1,) * 3)
            flo = fhi = 0.0
            for d in range(D + 1):
                w = 1 << (D - d)
                lo_n, hi_n = g0 // w - 2, (g0 + E) // w + 2
                cs, xs = tables[d]
                near = np.all((cs >= lo_n) & (cs <= hi_n), axis=1)
                for N, xv in zip(cs[near], xs[near]):
                    v = [_basis(D, d, N[a], g0[a] + k) for a in range(3)]
                    if not all(vv.any() for vv in v):
                        continue
                    term = xv * np.einsum("i,j,l->ijl", *v)
                    if d <= r or w >= E:
                        Fc += term
                    else:
                        Ff += term
                        lo3 = [vv.min() for vv in v]
                        hi3 = [vv.max() for vv in v]
                        ends = [xv * a * bb * c for a in (lo3[0], hi3[0]) for bb in (lo3[1], hi3[1]) for c in (lo3[2], hi3[2])]
                        flo += min(ends)
                        fhi += max(ends)
            # the coarse part's Bernstein coefficients over the brick from its values at 0, E/2, E
            h = E // 2
            V = Fc[np.ix_([0, h, E], [0, h, E], [0, h, E])]
            Tm = np.array([[1, 0, 0], [-0.5, 2, -0.5], [0, 0, 1]])
            Cb = np.einsum("ai,bj,ck,ijk->abc", Tm, Tm, Tm, V)
            assert np.allclose(np.einsum("ijk,ia,jb,kc->abc", Cb, _bern(k, E), _bern(k, E), _bern(k, E)), Fc,
                               atol=1e-9 * max(1.0, np.abs(Fc).max()))
            F = Fc + Ff
            tol = 1e-9 * max(1.0, np.abs(F).max())
            assert Cb.min() + flo - tol <= F.min() and F.max() <= Cb.max() + fhi + tol
            checked += 1
    assert checked >= 60
