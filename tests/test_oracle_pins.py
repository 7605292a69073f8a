"""The CPU oracle pinned to the reference: golden tables produced by the
reference's own host code, the marching-cubes table and the neighbour LUTs."""
import os
import re

import numpy as np
import pytest

from conftest import reference_file

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("depth", [5, 8])
def test_oracle_tables_match_reference_host_code(oracle_mod, depth):
    g = np.load(os.path.join(GOLDEN, "ref_tables_d%d.npz" % depth))
    o = oracle_mod.Oracle(depth, threads=4)
    xyz = np.array([[0.2, 0.3, 0.4], [0.7, 0.6, 0.5]], np.float32)
    o.set_points(xyz, np.ones_like(xyz))
    o.build_octree()
    o.build_basis(True)
    res = int(g["res"])
    for name in ("dot", "ddot", "d2dot"):
        mine = o.get(name)
        assert mine.size == res * res
        ref = np.zeros(res * res)
        ref[g[name + "_idx"]] = g[name + "_val"]
        # bit-exact, including the reference's negated diagonal of dDotTable
        assert np.array_equal(mine, ref), name


def test_oracle_stencil_matches_reference_tables(oracle_mod):
    """The 27 per-depth Laplacian coefficients equal GetLaplacianEntry on the golden tables."""
    depth = 5
    g = np.load(os.path.join(GOLDEN, "ref_tables_d%d.npz" % depth))
    res = int(g["res"])
    T = {}
    for name in ("dot", "d2dot"):
        t = np.zeros(res * res)
        t[g[name + "_idx"]] = g[name + "_val"]
        T[name] = t
    o = oracle_mod.Oracle(depth, threads=2)
    xyz = np.array([[0.2, 0.3, 0.4], [0.7, 0.6, 0.5]], np.float32)
    o.set_points(xyz, np.ones_like(xyz))
    o.build_octree()
    o.build_basis(False)
    st = o.get("stencil").reshape(depth + 1, 27)
    for d in range(2, depth + 1):
        i = (1 << d) - 1 + (1 << (d - 1))          # an interior index at depth d
        for j in range(27):
            off = (j // 9 - 1, (j // 3) % 3 - 1, j % 3 - 1)
            idx = [i * res + (i + o_) for o_ in off]
            dot = [T["dot"][k] for k in idx]
            d2 = [T["d2dot"][k] for k in idx]
            e = d2[0] * dot[1] * dot[2] + d2[1] * dot[0] * dot[2] + d2[2] * dot[0] * dot[1]
            want = np.float32(e) if abs(e) > float(np.float32(1e-6)) else np.float32(0)
            assert st[d, j] == want, (d, j)


def _parse_constant(src, name):
    i = src.index("__constant__ int %s" % name)
    j = src.index("};", i)
    body = src[src.index("=", i):j]
    return np.array([int(x) for x in re.findall(r"-?\d+", body)])


def test_mc_table_matches_reference_header(oracle_mod):
    path = reference_file("MarchingCubes.cuh")
    if not path:
        pytest.skip("reference tree not mounted")
    src = open(path).read()
    tri = _parse_constant(src, "triangles").reshape(256, 16)
    cnt = _parse_constant(src, "trianglesCount")
    ev = _parse_constant(src, "edgeVertex").reshape(12, 2)
    counts, edges = oracle_mod.mc_table()
    assert np.array_equal(counts, cnt)
    X = np.array([0, 1, 1, 0, 0, 1, 1, 0]); Y = np.array([0, 0, 1, 1, 0, 0, 1, 1]); Z = np.array([0, 0, 0, 0, 1, 1, 1, 1])
    P = np.stack([X, Y, Z], 1).astype(float)
    mid = 0.5 * (P[ev[:, 0]] + P[ev[:, 1]])

    def vector_area(e, n):
        a = np.zeros(3)
        for t in range(n):
            p = mid[e[3 * t:3 * t + 3]]
            a += np.cross(p[1] - p[0], p[2] - p[0])
        return a
    for c in range(256):
        n = cnt[c]
        assert set(edges[c, :3 * n]) == set(tri[c, :3 * n]), c
        # same polygons with the same orientation: equal vector area
        assert np.allclose(vector_area(edges[c], n), vector_area(tri[c], n)), c


def test_neighbour_luts_match_reference(oracle_mod):
    path = reference_file("main.cu")
    if not path:
        pytest.skip("reference tree not mounted")
    src = open(path).read()
    lp = _parse_constant(src, "LUTparent").reshape(8, 27)
    lc = _parse_constant(src, "LUTchild").reshape(8, 27)
    p, c = oracle_mod.luts()
    assert np.array_equal(p, lp)
    assert np.array_equal(c, lc)


def test_base_function_matches_reference(oracle_mod):
    g = np.load(os.path.join(GOLDEN, "ref_tables_d5.npz"))
    bf = g["base_function"]
    # F/F(0) of the degree-2 B-spline: starts -1.5,-0.5,0.5,1.5 and F(0) = 1
    assert np.array_equal(bf[:, 0], [-1.5, -0.5, 0.5, 1.5])
    v0 = sum(p[1] for p in bf if 0 > p[0])
    assert v0 == 1.0
