"""The benchmarked configuration itself against the CPU oracle, stage by stage.

Workload: shapes.torus(1_000_000, seed=0) -- R 0.3, r 0.1, density 1+7x,
position noise 0.001, vMF normal noise kappa 500 -- at maxDepth 10 with per-depth
CG to relative residual 1e-6 (FP64 reductions): exactly what bench.py times.
At this size the keys use 30 bits, the finest depth holds 3.97M nodes and about
10^5 coarse leaves are subdivided, so the depth-10 paths of every stage are
exercised.  The oracle (oracle/oracle.cpp, OpenMP) takes a couple of minutes on
the host cores, most of it in the subdivision, which it evaluates without any
culling.

Bars (as in test_gpu_parity.py):
  * octree arrays, normalised points/normals, inner-product tables, vector
    field, divergence at depths D and D-1: bit-exact; divergence above: 2 ulp;
  * CG (different FP64 reduction order): per depth max|x_gpu - x_orc| <= 1e-4 max|x_orc|;
  * each path on its own solution: implicit values within 1e-4 of max|f|,
    iso-value within 1e-5 relative, triangle counts within 0.5 %, symmetric
    Hausdorff distance <= 1e-3 of the bounding-box diagonal;
  * given the oracle's solution and iso-value: point values bit-exact and the
    identical set of triangles (compared as vertex coordinates).

One depth-10 superquadric of the batched configuration goes through
prgpu_reconstruct_batch (with smaller clouds around it) and is compared with the
oracle in the same way.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NODE_FIELDS = ("key", "pidx", "pnum", "parent", "children", "neighs", "didx", "dnum", "point_node")
D = 10


def _hausdorff(a, b):
    from scipy.spatial import cKDTree
    return max(cKDTree(b).query(a)[0].max(), cKDTree(a).query(b)[0].max())


def _triangle_set(v, f):
    t = np.ascontiguousarray(v[f].reshape(len(f), 9).astype(np.float32))
    return np.sort(t.view([("", np.float32)] * 9).ravel())


@pytest.fixture(scope="module")
def c2(lib_built, oracle_mod):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    xyz, nrm = shapes.torus(1_000_000, seed=0)
    g = pg.Reconstructor(depth=D, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6, cg_max_iter=10000)
    o = oracle_mod.Oracle(D)
    g.set_points(xyz, nrm)
    o.set_points(xyz, nrm)
    g.build_octree()
    o.build_octree()
    yield {"g": g, "o": o, "xyz": xyz}
    g.close()


def test_c2_octree_bit_exact(c2):
    g, o = c2["g"], c2["o"]
    assert np.array_equal(g.get("base"), o.get("base"))
    assert np.array_equal(g.get("count"), o.get("count"))
    assert int(g.get("count")[D]) > 3_900_000
    for f in NODE_FIELDS:
        assert np.array_equal(g.get(f), o.get(f)), f
    for f in ("points", "normals", "center", "scale"):
        assert np.array_equal(g.get(f), o.get(f)), f


def test_c2_rhs(c2):
    g, o = c2["g"], c2["o"]
    g.compute_rhs()
    o.build_basis(True)
    o.vector_field()
    o.divergence()
    for t in ("dot", "ddot", "d2dot"):
        assert np.array_equal(g.get(t), o.get(t)), t
    assert np.array_equal(g.get("stencil"), o.get("stencil"))
    assert np.array_equal(g.get("vfield"), o.get("vfield"))
    a, b = g.get("divergence"), o.get("divergence")
    base = o.get("base")
    fine = slice(base[D - 1], base[D + 1])
    assert np.array_equal(a[fine], b[fine])
    coarse = slice(0, base[D - 1])
    ulp = np.spacing(np.abs(b[coarse]).astype(np.float32))
    assert np.all(np.abs(a[coarse] - b[coarse]) <= 2 * ulp)


def test_c2_solve_and_values(c2):
    g, o = c2["g"], c2["o"]
    # each path solves its own system (the right-hand sides agree to 2 ulp)
    o.solve(1, 1e-6, 10000)
    g.solve()
    xg, xo = g.get("x"), o.get("x")
    base = o.get("base")
    for d in range(D + 1):
        sl = slice(base[d], base[d + 1])
        scale = max(np.abs(xo[sl]).max(), 1e-30)
        assert np.abs(xg[sl] - xo[sl]).max() <= 1e-4 * scale, d
    # implicit values and iso-value, each on its own solution
    iso_g = g.eval_points()
    o.point_values()
    fo, fg = o.get("point_value"), g.get("point_value")
    assert np.abs(fg - fo).max() <= 1e-4 * np.abs(fo).max()
    iso_o = float(o.get("iso")[0])
    assert abs(iso_g - iso_o) <= 1e-5 * abs(iso_o)
    c2["own_iso"] = iso_g


def test_c2_meshes(c2):
    g, o, xyz = c2["g"], c2["o"], c2["xyz"]
    # the GPU path's own mesh (its own x and iso-value)
    g.extract_mesh()
    gv_own, gf_own = g.mesh()
    # the oracle's mesh: full subdivision of every sign-changing coarse leaf, no culling
    o.marching_cubes()
    ov = o.get("mesh_v").reshape(-1, 3)
    of = o.get("mesh_f").reshape(-1, 3)
    c, s = o.get("center"), o.get("scale")[0]
    ov_in = (ov * s).astype(np.float32) + c
    assert abs(len(gf_own) - len(of)) <= 0.005 * len(of)
    diag = float(np.linalg.norm(xyz.max(0) - xyz.min(0)))
    assert _hausdorff(gv_own[np.unique(gf_own)], ov_in[np.unique(of)]) <= 1e-3 * diag
    # given the oracle's solution and iso-value: bit-exact point values, identical triangles
    g.set("x", o.get("x"))
    g.eval_points()
    assert np.array_equal(g.get("point_value"), o.get("point_value"))
    g.set("iso", np.float32([o.get("iso")[0]]))
    g.extract_mesh()
    assert int(g.get("subdivide_roots")[0]) == int(o.get("subdivide_roots")[0])
    assert int(g.get("subdivide_roots")[0]) > 50_000
    gv, gf = g.mesh()
    assert len(gf) == len(of)
    assert np.array_equal(_triangle_set(gv, gf), _triangle_set(ov_in, of))


def test_superquadric_d10_in_a_batch_matches_oracle(lib_built, oracle_mod):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    big = shapes.superquadric(7, n_min=150_000, n_max=150_001)
    small = [shapes.superquadric(200 + k, n_min=5000, n_max=20000) for k in range(3)]
    clouds = [small[0], big, small[1], small[2]]
    depths = [7, 10, 8, 9]
    r = pg.Reconstructor(depth=8)
    out = r.reconstruct_batch(clouds, depths)
    r.close()
    gv, gf = out[1]
    xyz, nrm = big
    o = oracle_mod.Oracle(10)
    o.set_points(xyz, nrm)
    o.reconstruct()
    ov = o.get("mesh_v").reshape(-1, 3) * o.get("scale")[0] + o.get("center")
    of = o.get("mesh_f").reshape(-1, 3)
    assert abs(len(gf) - len(of)) <= 0.005 * len(of)
    diag = float(np.linalg.norm(xyz.max(0) - xyz.min(0)))
    assert _hausdorff(gv[np.unique(gf)], ov[np.unique(of)]) <= 1e-3 * diag
    # a separate reconstruction of the same cloud gives the batch's mesh bit for bit
    s = pg.Reconstructor(depth=10)
    sv, sf = s.reconstruct(xyz, nrm)
    s.close()
    assert np.array_equal(sv, gv) and np.array_equal(sf, gf)


def test_c2_precision_against_fp64_oracle(c2, lib_built, oracle_mod):
    """The torus at maxDepth 10 against the FP64 oracle run (see test_gpu_precision.py): with the
    reference's single-precision basis evaluation, and with params.stable_basis."""
    import os
    import sys
    import poissonrecon_gpu_gb300 as pg
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_gpu_precision import _keep, precision_row
    o, xyz = c2["o"], c2["xyz"]
    nrm = o._nrm
    for stable, (imp, iso) in ((False, (0.15, 2e-2)), (True, (1e-3, 1e-5))):
        row = precision_row(pg, oracle_mod, "torus 1M, maxDepth 10", xyz, nrm, D, o=o, stable=stable)
        _keep(row)
        assert row["implicit_rel_err"] <= imp, row
        assert row["iso_rel_err"] <= iso, row
        assert all(0 <= r <= 1e-6 * 1.0001 for r in row["fp64_residual_per_depth"]), row
