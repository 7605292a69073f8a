"""Edge-case inputs through the CUDA path, checked against the oracle stage by stage.

For each cloud: the octree arrays are bit-exact; the divergence at the two finest
depths is bit-exact; given the oracle's solution the implicit values at the
points are bit-exact; given the oracle's iso-value the mesh has the same
triangles (compared as sets of vertex coordinates).  Degenerate clouds (one
point, coincident points, non-finite coordinates) are rejected with an error
and leave the context usable.
"""
import numpy as np
import pytest

from conftest import sphere

pytestmark = pytest.mark.gpu

NODE_FIELDS = ("key", "pidx", "pnum", "parent", "children", "neighs", "didx", "dnum", "point_node")


def _disc(n, seed):
    """Coplanar points: a disc in the plane z = 0.5, normals +z."""
    rng = np.random.default_rng(seed)
    r = 0.3 * np.sqrt(rng.random(n))
    t = 2 * np.pi * rng.random(n)
    xyz = np.stack([0.5 + r * np.cos(t), 0.5 + r * np.sin(t), np.full(n, 0.5)], 1)
    nrm = np.tile([0.0, 0.0, 1.0], (n, 1))
    return xyz.astype(np.float32), nrm.astype(np.float32)


def _duplicates(n, seed):
    xyz, nrm = sphere(n, seed=seed)
    k = n // 2
    return np.concatenate([xyz, xyz[:k]]), np.concatenate([nrm, nrm[:k]])


def _zero_normals(n, seed):
    xyz, nrm = sphere(n, seed=seed)
    nrm = nrm.copy()
    nrm[::10] = 0.0
    return xyz, nrm


def _clusters(n, seed):
    """A sphere and a small dense sphere touching it: deep leaves next to coarse ones."""
    from poissonrecon_gpu_gb300 import shapes
    a, an = shapes.sphere(n, seed=seed)
    b, bn = shapes.sphere(n // 2, radius=0.04, center=(0.5, 0.5, 0.89), seed=seed + 1)
    return np.concatenate([a, b]), np.concatenate([an, bn])


def _slab(n, seed):
    """Two parallel squares 0.02 apart with opposite normals (a thin plate)."""
    rng = np.random.default_rng(seed)
    m = n // 2
    uv = 0.2 + 0.6 * rng.random((2 * m, 2))
    z = np.concatenate([np.full(m, 0.49), np.full(m, 0.51)])
    xyz = np.stack([uv[:, 0], uv[:, 1], z], 1)
    nz = np.concatenate([np.full(m, -1.0), np.full(m, 1.0)])
    nrm = np.stack([np.zeros(2 * m), np.zeros(2 * m), nz], 1)
    return xyz.astype(np.float32), nrm.astype(np.float32)


CASES = {"disc": (_disc, 4000, 6), "duplicates": (_duplicates, 3000, 6), "zero-normals": (_zero_normals, 3000, 6),
         "clusters": (_clusters, 4000, 7), "slab": (_slab, 4000, 6)}


@pytest.mark.parametrize("case", list(CASES))
def test_edge_case_parity(lib_built, oracle_mod, case):
    import poissonrecon_gpu_gb300 as pg
    gen, n, depth = CASES[case]
    xyz, nrm = gen(n, 3)
    g = pg.Reconstructor(depth=depth)
    o = oracle_mod.Oracle(depth, threads=4)
    g.set_points(xyz, nrm)
    o.set_points(xyz, nrm)
    g.build_octree()
    o.build_octree()
    for f in NODE_FIELDS:
        assert np.array_equal(g.get(f), o.get(f)), f
    g.compute_rhs()
    o.build_basis(True)
    o.vector_field()
    o.divergence()
    base = o.get("base")
    fine = slice(base[depth - 1], base[depth + 1])
    assert np.array_equal(g.get("vfield"), o.get("vfield"))
    assert np.array_equal(g.get("divergence")[fine], o.get("divergence")[fine])
    o.solve(0, 1e-5, 10000)
    g.solve()
    g.set("x", o.get("x"))
    g.eval_points()
    o.point_values()
    assert np.array_equal(g.get("point_value"), o.get("point_value"))
    g.set("iso", np.float32([o.get("iso")[0]]))
    g.extract_mesh()
    o.marching_cubes()
    gv, gf = g.mesh()
    ov = o.get("mesh_v").reshape(-1, 3) * o.get("scale")[0] + o.get("center")
    of = o.get("mesh_f").reshape(-1, 3)
    assert len(gf) == len(of) and len(gf) > 0
    tg = np.sort(gv[gf].reshape(len(gf), 9).view([("", np.float32)] * 9).ravel())
    to = np.sort(ov[of].reshape(len(of), 9).astype(np.float32).view([("", np.float32)] * 9).ravel())
    assert np.array_equal(tg, to)
    g.close()


def test_degenerate_clouds_rejected(lib_built):
    import poissonrecon_gpu_gb300 as pg
    g = pg.Reconstructor(depth=5)
    one = np.float32([[0.3, 0.4, 0.5]])
    up = np.float32([[0.0, 0.0, 1.0]])
    for xyz, nrm in ((one, up), (np.repeat(one, 100, 0), np.repeat(up, 100, 0))):
        with pytest.raises(pg.PrgpuError, match="degenerate"):
            g.reconstruct(xyz, nrm)
    bad, bn = sphere(500, seed=1)
    bad = bad.copy()
    bad[7, 1] = np.nan
    with pytest.raises(pg.PrgpuError):
        g.reconstruct(bad, bn)
    # the context is still usable
    v, f = g.reconstruct(*sphere(2000, seed=1))
    assert len(f) > 0
    g.close()
