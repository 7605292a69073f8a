"""params.cascadic (coarse-to-fine solve with the cross-depth products; not the reference's
independent depths) through the C ABI, against the oracle's restatement of the same solve.

Tolerances, as for the default solve: per depth max|x_gpu - x_orc| <= 1e-4 * max|x_orc| (the
CG reductions differ in order); implicit values within 1e-4 of max|f|; iso-value within 1e-5
relative; triangle counts within 0.5 %; symmetric Hausdorff distance <= 1e-3 of the bounding-box
diagonal.  Solving the depths one prgpu_solve_depth call each, coarse to fine, repeats
prgpu_solve bit for bit (the same launches with the same partitions).
"""
import numpy as np
import pytest

from conftest import sphere

pytestmark = pytest.mark.gpu


def _hausdorff(a, b):
    from scipy.spatial import cKDTree
    return max(cKDTree(b).query(a)[0].max(), cKDTree(a).query(b)[0].max())


@pytest.mark.parametrize("kind,n,depth", [("sphere", 20000, 7), ("torus", 30000, 8)])
def test_cascadic_matches_oracle(lib_built, oracle_mod, kind, n, depth):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    xyz, nrm = sphere(n, seed=5) if kind == "sphere" else shapes.torus(n, seed=5)
    g = pg.Reconstructor(depth=depth, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6, cascadic=True)
    gv, gf = g.reconstruct(xyz, nrm)
    o = oracle_mod.Oracle(depth)
    o.set_points(xyz, nrm)
    o.set_cascadic(True)
    o.reconstruct(1, 1e-6, 10000)
    base = o.get("base")
    xg, xo = g.get("x"), o.get("x")
    for d in range(depth + 1):
        sl = slice(base[d], base[d + 1])
        assert np.abs(xg[sl] - xo[sl]).max() <= 1e-4 * np.abs(xo[sl]).max(), d
    fo, fg = o.get("point_value"), g.get("point_value")
    assert np.abs(fg - fo).max() <= 1e-4 * np.abs(fo).max()
    iso_o = float(o.get("iso")[0])
    assert abs(float(g.get("iso")[0]) - iso_o) <= 1e-5 * abs(iso_o)
    ov = o.get("mesh_v").reshape(-1, 3) * o.get("scale")[0] + o.get("center")
    of = o.get("mesh_f").reshape(-1, 3)
    assert abs(len(gf) - len(of)) <= 0.005 * len(of)
    diag = np.linalg.norm(xyz.max(0) - xyz.min(0))
    assert _hausdorff(gv[np.unique(gf)], ov[np.unique(of)]) <= 1e-3 * diag
    g.close()


def test_cascadic_solve_depth_sequence(lib_built):
    import poissonrecon_gpu_gb300 as pg
    xyz, nrm = sphere(20000, seed=6)
    depth = 7
    a = pg.Reconstructor(depth=depth, cascadic=True)
    a.set_points(xyz, nrm); a.build_octree(); a.compute_rhs(); a.solve()
    b = pg.Reconstructor(depth=depth, cascadic=True)
    b.set_points(xyz, nrm); b.build_octree(); b.compute_rhs()
    for d in range(depth + 1):
        b.solve_depth(d, pg.SOLVE_REFERENCE)
    assert np.array_equal(a.get("x"), b.get("x"))
    assert np.array_equal(a.get("cg_iters"), b.get("cg_iters"))
    a.close()
    b.close()


def test_cascadic_sphere_mesh_closer(lib_built):
    """On a 200k-point sphere at maxDepth 9 the cascadic mesh lies closer to the true sphere than
    the reference's independent-depth mesh."""
    import poissonrecon_gpu_gb300 as pg
    xyz, nrm = sphere(200_000, seed=0)
    dist = {}
    for casc in (False, True):
        r = pg.Reconstructor(depth=9, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6, cascadic=casc)
        v, f = r.reconstruct(xyz, nrm)
        used = np.unique(f)
        dist[casc] = np.abs(np.linalg.norm(v[used] - 0.5, axis=1) - 0.35)
        r.close()
    assert dist[True].max() < 0.01
    assert dist[True].mean() < 0.75 * dist[False].mean()
