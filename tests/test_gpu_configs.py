"""The remaining benchmark configurations, at sizes the oracle finishes in under a minute:

  * a union of 3-8 ellipsoids at maxDepth 9 (the shapes of the solver-study configuration),
    end to end through both paths: octree arrays bit-exact, implicit values within 1e-4 of
    max|f|, iso-value within 1e-5, triangle counts within 0.5 %, symmetric Hausdorff distance
    <= 1e-3 of the bounding-box diagonal;
  * uneven clouds in one call (the batched configuration): superquadrics of 5k-60k points at
    depths drawn from {7, 8, 9}, through prgpu_reconstruct_batch, give the meshes of separate
    reconstructions bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NODE_FIELDS = ("key", "pidx", "pnum", "parent", "children", "neighs", "didx", "dnum", "point_node")


def _hausdorff(a, b):
    from scipy.spatial import cKDTree
    return max(cKDTree(b).query(a)[0].max(), cKDTree(a).query(b)[0].max())


def test_ellipsoid_union_d9_end_to_end(lib_built, oracle_mod):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    xyz, nrm = shapes.ellipsoid_union(3, n_min=20000, n_max=20001)
    depth = 9
    g = pg.Reconstructor(depth=depth)
    gv, gf = g.reconstruct(xyz, nrm)
    o = oracle_mod.Oracle(depth)
    o.set_points(xyz, nrm)
    o.reconstruct()
    for f in NODE_FIELDS:
        assert np.array_equal(g.get(f), o.get(f)), f
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


def test_superquadric_batch_matches_separate(lib_built):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    rng = np.random.default_rng(11)
    clouds = [shapes.superquadric(100 + k, n_min=5000, n_max=60000) for k in range(12)]
    depths = [int(d) for d in rng.choice([7, 8, 9], len(clouds))]
    single = []
    for (xyz, nrm), d in zip(clouds, depths):
        r = pg.Reconstructor(depth=d)
        single.append(r.reconstruct(xyz, nrm))
        r.close()
    r = pg.Reconstructor(depth=8)
    batch = r.reconstruct_batch(clouds, depths)
    r.close()
    assert len(batch) == len(clouds)
    for (v1, f1), (v2, f2) in zip(single, batch):
        assert len(f1) > 0
        assert np.array_equal(v1, v2) and np.array_equal(f1, f2)
