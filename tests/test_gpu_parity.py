"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances:
  * integer stages (octree arrays, subdivision flags, triangle topology): bit-exact;
  * stages whose arithmetic is restated operation for operation (normalised
    points, inner-product tables, vector field, finest-depth divergence, stencil,
    implicit values from the same solution, marching-cubes vertices): bit-exact;
  * divergence at depths < D-1 (FP64 block reduction instead of a sequential
    FP64 sum): |diff| <= 2 ulp of the value;
  * CG solution (different FP64 reduction order): per depth
    max|x_gpu - x_orc| <= 1e-4 * max|x_orc|;
  * end to end: implicit values within 1e-4 of max|f|, iso-value within 1e-5
    relative, symmetric Hausdorff distance <= 1e-3 of the bounding-box diagonal,
    triangle counts within 0.5 %.
"""
import numpy as np
import pytest

from conftest import sphere

pytestmark = pytest.mark.gpu


def _torus(n, seed=0):
    from poissonrecon_gpu_gb300 import shapes
    return shapes.torus(n, seed=seed)


NODE_FIELDS = ("key", "pidx", "pnum", "parent", "children", "neighs", "didx", "dnum", "point_node")


# torus30k-d8 has subdivided leaves of every lattice edge from 2 to 64 (bricks of 8^3 cells, their
# 4^3-brick super-bricks, and the small single-brick leaves), adjacent leaves of the same depth
# batch (corners owned by another leaf) and culled bricks next to live ones
@pytest.fixture(scope="module", params=[("sphere", 5000, 6), ("torus", 30000, 7), ("torus", 30000, 8)],
                ids=["sphere5k-d6", "torus30k-d7", "torus30k-d8"])
def staged(request, lib_built, oracle_mod):
    import poissonrecon_gpu_gb300 as pg
    kind, n, depth = request.param
    xyz, nrm = sphere(n, seed=2) if kind == "sphere" else _torus(n, seed=2)
    g = pg.Reconstructor(depth=depth)
    o = oracle_mod.Oracle(depth)
    g.set_points(xyz, nrm)
    o.set_points(xyz, nrm)
    g.build_octree()
    o.build_octree()
    st = {"g": g, "o": o, "depth": depth, "xyz": xyz}
    yield st
    g.close()


def test_octree_bit_exact(staged):
    g, o = staged["g"], staged["o"]
    assert np.array_equal(g.get("base"), o.get("base"))
    assert np.array_equal(g.get("count"), o.get("count"))
    for f in NODE_FIELDS:
        assert np.array_equal(g.get(f), o.get(f)), f
    assert np.array_equal(g.get("points"), o.get("points"))
    assert np.array_equal(g.get("normals"), o.get("normals"))
    assert np.array_equal(g.get("sort_idx").astype(np.int64), o.get("sort_idx"))
    assert np.array_equal(g.get("center"), o.get("center"))
    assert np.array_equal(g.get("scale"), o.get("scale"))


def test_basis_tables_and_vector_field(staged):
    g, o = staged["g"], staged["o"]
    g.compute_rhs()
    o.build_basis(True)
    o.vector_field()
    for t in ("dot", "ddot", "d2dot"):
        assert np.array_equal(g.get(t), o.get(t)), t
    assert np.array_equal(g.get("stencil"), o.get("stencil"))
    assert np.array_equal(g.get("vfield"), o.get("vfield"))


def test_divergence(staged):
    g, o = staged["g"], staged["o"]
    o.divergence()
    a, b = g.get("divergence"), o.get("divergence")
    base, D = o.get("base"), staged["depth"]
    fine = slice(base[D - 1], base[D + 1])
    assert np.array_equal(a[fine], b[fine])
    coarse = slice(0, base[D - 1])
    ulp = np.spacing(np.abs(b[coarse]).astype(np.float32))
    assert np.all(np.abs(a[coarse] - b[coarse]) <= 2 * ulp)


def test_solve(staged):
    g, o = staged["g"], staged["o"]
    o.set_f32("divergence", g.get("divergence"))
    o.solve(0, 1e-5, 10000)
    g.solve()
    xg, xo = g.get("x"), o.get("x")
    base, D = o.get("base"), staged["depth"]
    for d in range(D + 1):
        sl = slice(base[d], base[d + 1])
        scale = max(np.abs(xo[sl]).max(), 1e-30)
        assert np.abs(xg[sl] - xo[sl]).max() <= 1e-4 * scale, d
    assert np.all(np.abs(g.get("cg_iters") - o.get("cg_iters")) <= 3)
    assert np.all(g.get("cg_rr") <= np.float32(1e-5) * np.float32(1e-5))


def test_point_values_bit_exact(staged):
    g, o = staged["g"], staged["o"]
    g.set("x", o.get("x"))
    iso_g = g.eval_points()
    o.point_values()
    assert np.array_equal(g.get("point_value"), o.get("point_value"))
    iso_o = float(o.get("iso")[0])
    assert abs(iso_g - iso_o) <= 1e-6 * abs(iso_o)


def test_mesh_matches_oracle(staged):
    g, o = staged["g"], staged["o"]
    g.set("iso", np.float32([o.get("iso")[0]]))
    g.extract_mesh()
    o.marching_cubes()
    # the subdivision flags decide which leaves are refined (ifSubdivide main.cu:2988):
    # compared on the leaves above the finest depth, the nodes that use them
    ch = o.get("children").reshape(-1, 8)
    nc = len(g.get("has_tri"))
    leaf = np.nonzero(ch[:nc, 0] == -1)[0]
    leaf = leaf[leaf > 0]
    assert np.array_equal(g.get("has_tri")[leaf], o.get("has_tri")[leaf])
    assert np.array_equal(g.get("has_int")[leaf], o.get("has_int")[leaf])
    assert int(g.get("subdivide_roots")[0]) == int(o.get("subdivide_roots")[0])
    gv, gf = g.mesh()
    ov = o.get("mesh_v").reshape(-1, 3)
    of = o.get("mesh_f").reshape(-1, 3)
    c, s = o.get("center"), o.get("scale")[0]
    ov = (ov * s).astype(np.float32) + c
    assert len(gf) == len(of)
    # same triangles, compared as sets of vertex coordinates
    tg = np.sort(gv[gf].reshape(len(gf), 9).view([("", np.float32)] * 9).ravel())
    to = np.sort(ov[of].reshape(len(of), 9).astype(np.float32).view([("", np.float32)] * 9).ravel())
    assert np.array_equal(tg, to)


def test_weld_matches_oracle(staged, oracle_mod):
    """weld = 1 against the oracle's mesh welded by the same rule (oracle.weld: one vertex per
    finest-lattice edge across subdivision batches, placed where the first triangle corner on that
    edge puts it): given the oracle's solution and iso-value, the same number of vertices, the
    same vertex positions and the same triangles."""
    import poissonrecon_gpu_gb300 as pg
    o = staged["o"]
    w = pg.Reconstructor(depth=staged["depth"], weld=True)
    w.set_points(o._xyz, o._nrm)
    w.build_octree()
    w.compute_rhs()
    w.solve()
    w.set("x", o.get("x"))
    w.eval_points()
    w.set("iso", np.float32([o.get("iso")[0]]))
    w.extract_mesh()
    gv, gf = w.mesh()
    w.close()
    o.marching_cubes()
    ov, of = oracle_mod.weld(o.get("mesh_v"), o.get("mesh_f").reshape(-1, 3), o.get("mesh_vkey"))
    c, s = o.get("center"), o.get("scale")[0]
    ov = (ov * s).astype(np.float32) + c
    # unwelded, the oracle has a vertex per lattice edge and batch: the weld merges some
    assert len(ov) < len(o.get("mesh_v")) // 3
    assert len(gv) == len(ov) and len(gf) == len(of)
    row = [("", np.float32)] * 3
    assert np.array_equal(np.sort(gv.view(row).ravel()), np.sort(ov.view(row).ravel()))
    tg = np.sort(gv[gf].reshape(len(gf), 9).view([("", np.float32)] * 9).ravel())
    to = np.sort(ov[of].reshape(len(of), 9).view([("", np.float32)] * 9).ravel())
    assert np.array_equal(tg, to)


def _hausdorff(a, b):
    from scipy.spatial import cKDTree
    return max(cKDTree(b).query(a)[0].max(), cKDTree(a).query(b)[0].max())


@pytest.mark.parametrize("n,depth", [(50000, 8)], ids=["sphere50k-d8"])
def test_end_to_end(lib_built, oracle_mod, n, depth):
    """Config 1 through both paths, each on its own (no shared intermediates)."""
    import poissonrecon_gpu_gb300 as pg
    xyz, nrm = sphere(n, seed=0)
    g = pg.Reconstructor(depth=depth)
    gv, gf = g.reconstruct(xyz, nrm)
    o = oracle_mod.Oracle(depth)
    o.set_points(xyz, nrm)
    o.reconstruct()
    for f in NODE_FIELDS:
        assert np.array_equal(g.get(f), o.get(f)), f
    fo = o.get("point_value")
    fg = g.get("point_value")
    assert np.abs(fg - fo).max() <= 1e-4 * np.abs(fo).max()
    iso_o = float(o.get("iso")[0])
    assert abs(float(g.get("iso")[0]) - iso_o) <= 1e-5 * abs(iso_o)
    ov = o.get("mesh_v").reshape(-1, 3) * o.get("scale")[0] + o.get("center")
    of = o.get("mesh_f").reshape(-1, 3)
    assert abs(len(gf) - len(of)) <= 0.005 * len(of)
    diag = np.linalg.norm(xyz.max(0) - xyz.min(0))
    assert _hausdorff(gv[np.unique(gf)], ov[np.unique(of)]) <= 1e-3 * diag
    g.close()


def test_small_and_invalid_inputs(lib_built, oracle_mod):
    import poissonrecon_gpu_gb300 as pg
    xyz, nrm = sphere(40, seed=5)
    g = pg.Reconstructor(depth=4)
    v, f = g.reconstruct(xyz, nrm)
    o = oracle_mod.Oracle(4, threads=1)
    o.set_points(xyz, nrm)
    o.reconstruct()
    for fld in NODE_FIELDS:
        assert np.array_equal(g.get(fld), o.get(fld)), fld
    assert len(f) == len(o.get("mesh_f")) // 3
    # empty input and out-of-order calls are rejected, the context stays usable
    with pytest.raises(pg.PrgpuError):
        g.set_points(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32))
    h = pg.Reconstructor(depth=5)
    with pytest.raises(pg.PrgpuError):
        h.solve(allow_not_converged=False)
    v2, f2 = g.reconstruct(xyz, nrm)
    assert np.array_equal(f, f2) and np.array_equal(v, v2)
    g.close()
    h.close()


def test_cg_csr_matches_dense_solve(lib_built):
    torch = pytest.importorskip("torch")
    import poissonrecon_gpu_gb300 as pg
    n = 3000
    rng = np.random.default_rng(0)
    # SPD: 1-D Laplacian plus a positive diagonal
    rows, cols, vals = [], [], []
    for i in range(n):
        for j, v in ((i - 1, -1.0), (i, 2.5), (i + 1, -1.0)):
            if 0 <= j < n:
                rows.append(i); cols.append(j); vals.append(v)
    rowptr = np.searchsorted(rows, np.arange(n + 1)).astype(np.int32)
    b = rng.standard_normal(n).astype(np.float32)
    dev = torch.device("cuda:0")
    tI = torch.tensor(rowptr, device=dev)
    tJ = torch.tensor(np.array(cols, np.int32), device=dev)
    tV = torch.tensor(np.array(vals, np.float32), device=dev)
    tb = torch.tensor(b, device=dev)
    tx = torch.zeros(n, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    ms, it = pg.solverCG_DeviceToDevice(n, len(vals), tI.data_ptr(), tJ.data_ptr(), tV.data_ptr(),
                                        tb.data_ptr(), tx.data_ptr(), 1e-5, 10000)
    A = np.zeros((n, n))
    A[rows, cols] = vals
    x = np.linalg.solve(A, b.astype(np.float64))
    assert it > 0 and ms > 0
    assert np.abs(tx.cpu().numpy() - x).max() <= 1e-4 * np.abs(x).max()


def test_reconstruct_batch_matches_single(lib_built):
    """prgpu_reconstruct_batch: clouds of different sizes and depths in one call give the meshes of
    separate reconstructions; a bad cloud is reported by index and nothing leaks."""
    import poissonrecon_gpu_gb300 as pg
    clouds = [sphere(3000, seed=4), _torus(6000, seed=6), sphere(1500, seed=8)]
    depths = [5, 6, 4]
    single = []
    for (xyz, nrm), d in zip(clouds, depths):
        r = pg.Reconstructor(depth=d)
        single.append(r.reconstruct(xyz, nrm))
        r.close()
    r = pg.Reconstructor(depth=7)
    batch = r.reconstruct_batch(clouds, depths)
    for (v1, f1), (v2, f2) in zip(single, batch):
        assert np.array_equal(v1, v2) and np.array_equal(f1, f2)
    with pytest.raises(pg.PrgpuError, match="cloud 1"):
        r.reconstruct_batch([clouds[0], clouds[1]], [5, 1])
    # the context keeps its own depth
    v, f = r.reconstruct(*clouds[0])
    assert len(f) > 0
    r.close()


def _open_edges(f):
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, cnt = np.unique(e, axis=0, return_counts=True)
    return int((cnt == 1).sum())


@pytest.mark.parametrize("kind,n,depth", [("sphere", 50000, 8), ("torus", 30000, 8)], ids=["sphere50k-d8", "torus30k-d8"])
def test_weld_shares_vertices_across_batches(lib_built, kind, n, depth):
    """weld = 1: one vertex per lattice edge across subdivision batches.  The triangles are the
    same (same count, same emission order); each welded vertex is a vertex of the unwelded mesh
    (the position one of its batches computed), and the batch seams close (open edges remain only
    where the batches on either side disagree on a corner's sign)."""
    import poissonrecon_gpu_gb300 as pg
    xyz, nrm = sphere(n, seed=0) if kind == "sphere" else _torus(n, seed=0)
    meshes = []
    for weld in (False, True):
        r = pg.Reconstructor(depth=depth, weld=weld)
        meshes.append(r.reconstruct(xyz, nrm))
        r.close()
    (v0, f0), (v1, f1) = meshes
    assert len(f1) == len(f0) and len(v1) < len(v0)
    # every welded vertex position occurs in the unwelded mesh
    p0 = np.unique(v0.view([("", np.float32)] * 3).ravel())
    p1 = np.unique(v1.view([("", np.float32)] * 3).ravel())
    assert np.all(np.isin(p1, p0))
    # triangle by triangle, a corner moves along its own lattice edge: less than one finest cell
    # (the batches on either side of a seam compute the crossing from their own corner values)
    cell = 1.25 * float((xyz.max(0) - xyz.min(0)).max()) / (1 << depth)
    assert np.abs(v1[f1] - v0[f0]).max() <= cell
    assert _open_edges(f1) * 50 < _open_edges(f0)


def test_density_weights_remove_sparse_side_sheets(lib_built):
    """density_weights = 1 (Kazhdan's weighting of non-uniform samples, not in the reference): on
    the torus with an 8x sampling gradient the unweighted indicator grows sheets inside the sparse
    half of the tube (vertices up to the tube radius away from the surface, in the oracle's meshes
    as well); weighted, every vertex lies near the surface.  The weights have mean 1 and follow
    the density (larger on the sparse side)."""
    import poissonrecon_gpu_gb300 as pg
    xyz, nrm = _torus(200_000, seed=0)

    def dev(v):
        rho = np.hypot(v[:, 0] - 0.5, v[:, 1] - 0.5)
        return np.abs(np.hypot(rho - 0.3, v[:, 2] - 0.5) - 0.1)

    out = {}
    for dw in (False, True):
        r = pg.Reconstructor(depth=9, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6, density_weights=dw)
        v, f = r.reconstruct(xyz, nrm)
        out[dw] = (dev(v), r.get("point_weight") if dw else None)
        r.close()
    assert (out[False][0] > 0.03).sum() > 1000          # the sheets, without weights
    d, w = out[True]
    assert d.max() < 0.02 and np.quantile(d, 0.99) < 0.005
    assert abs(float(w.astype(np.float64).mean()) - 1.0) < 1e-4 and w.min() > 0
    # the sparse side (small x) weighs more than the dense side
    r = pg.Reconstructor(depth=9)
    r.set_points(xyz, nrm)
    r.build_octree()
    order = r.get("sort_idx")          # sorted position -> input index
    r.close()
    x = xyz[order, 0]
    assert w[x < 0.3].mean() > 3 * w[x > 0.7].mean()


def test_solve_depth_and_node_arrays(lib_built, oracle_mod):
    """prgpu_solve_depth: solving the depths one call each gives the all-depth solve (the depths are
    independent systems; the reduction partitions differ, so within the CG tolerance), and a depth
    solved alone leaves the others' x untouched.  prgpu_get_node_arrays: the reference's OctNode
    fields, equal to the named arrays and to the oracle's."""
    import poissonrecon_gpu_gb300 as pg
    xyz, nrm = sphere(5000, seed=2)
    depth = 6
    a = pg.Reconstructor(depth=depth)
    a.set_points(xyz, nrm); a.build_octree(); a.compute_rhs(); a.solve()
    xa = a.get("x")
    b = pg.Reconstructor(depth=depth)
    b.set_points(xyz, nrm); b.build_octree(); b.compute_rhs()
    base = b.get("base")
    b.solve_depth(depth, pg.SOLVE_REFERENCE)
    xb = b.get("x")
    assert np.all(xb[: base[depth]] == 0.0)          # the other depths are untouched
    for d in range(depth):
        b.solve_depth(d, pg.SOLVE_REFERENCE)
    xb = b.get("x")
    for d in range(depth + 1):
        sl = slice(base[d], base[d + 1])
        assert np.abs(xb[sl] - xa[sl]).max() <= 1e-4 * max(np.abs(xa[sl]).max(), 1e-30), d
    assert np.all(np.abs(b.get("cg_iters") - a.get("cg_iters")) <= 2)
    with pytest.raises(pg.PrgpuError):
        b.solve_depth(depth + 1, pg.SOLVE_REFERENCE)
    na = b.node_arrays()
    for f in ("key", "pidx", "pnum", "parent", "children", "neighs", "didx", "dnum", "base"):
        assert np.array_equal(na[f], b.get(f)), f
    o = oracle_mod.Oracle(depth)
    o.set_points(xyz, nrm)
    o.build_octree()
    for f in ("key", "pidx", "pnum", "parent", "children", "neighs", "didx", "dnum"):
        assert np.array_equal(na[f].astype(np.int64), o.get(f).astype(np.int64)), f
    a.close()
    b.close()
