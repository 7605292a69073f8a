"""Properties of the oracle's restatement on small inputs (CPU only)."""
import numpy as np
import pytest

from conftest import sphere


@pytest.fixture(scope="module")
def small(oracle_mod):
    xyz, nrm = sphere(4000, seed=1)
    o = oracle_mod.Oracle(6, threads=4)
    o.set_points(xyz, nrm)
    o.reconstruct()
    return o, xyz, nrm


def test_octree_invariants(small):
    o, xyz, _ = small
    base, count = o.get("base"), o.get("count")
    M = base[-1]
    key, parent, children = o.get("key"), o.get("parent"), o.get("children").reshape(-1, 8)
    pidx, pnum, neighs = o.get("pidx"), o.get("pnum"), o.get("neighs").reshape(-1, 27)
    D = len(count) - 1
    assert count[0] == 1 and all(c % 8 == 0 for c in count[1:])
    assert pnum[0] == len(xyz)
    for d in range(1, D + 1):
        lo, hi = base[d], base[d + 1]
        par = parent[lo:hi]
        # every slot's parent lies one depth up and lists it as a child
        assert np.all((par >= base[d - 1]) & (par < base[d]))
        k = np.arange(lo, hi)
        son = (key[lo:hi] >> (3 * (D - d))) & 7
        assert np.array_equal(children[par, son], k)
        # point ranges of the 8 siblings tile the parent's range
        g = pnum[lo:hi].reshape(-1, 8).sum(1)
        assert np.array_equal(g, pnum[par[::8]])
    # neighbour 13 is the node itself; neighbour relation is symmetric
    assert np.array_equal(neighs[:, 13], np.arange(M))
    for j in range(27):
        nb = neighs[:, j]
        ok = nb >= 0
        assert np.array_equal(neighs[nb[ok], 26 - j], np.nonzero(ok)[0])


def test_solver_meets_reference_schedule(small):
    o, _, _ = small
    it = o.get("cg_iters")
    rr = o.get("cg_rr")
    assert np.all(it < 10000)
    assert np.all(rr <= np.float32(1e-5) * np.float32(1e-5))


def test_mesh_lies_on_sphere(small):
    o, xyz, _ = small
    v = o.get("mesh_v").reshape(-1, 3)
    f = o.get("mesh_f").reshape(-1, 3)
    assert len(f) > 1000
    used = np.unique(f)
    c, s = o.get("center"), o.get("scale")[0]
    r = np.linalg.norm(v[used] * s + c - 0.5, axis=1)
    assert abs(r.mean() - 0.35) < 0.005
    assert r.min() > 0.3 and r.max() < 0.4


def test_duplicate_points_share_leaves(oracle_mod):
    """Repeated samples land in the same leaf; point ranges still tile the input."""
    xyz, nrm = sphere(500, seed=4)
    xyz2 = np.concatenate([xyz, xyz[:200]])
    nrm2 = np.concatenate([nrm, nrm[:200]])
    o = oracle_mod.Oracle(5, threads=2)
    o.set_points(xyz2, nrm2)
    o.build_octree()
    base, pnum, pidx = o.get("base"), o.get("pnum"), o.get("pidx")
    D = 5
    leaf = slice(base[D], base[D + 1])
    assert pnum[leaf].sum() == len(xyz2)
    nz = pnum[leaf] > 0
    starts = pidx[leaf][nz]
    assert np.all(np.diff(starts) > 0)
    assert np.array_equal(np.sort(o.get("sort_idx")), np.arange(len(xyz2)))


def test_weld_rule(oracle_mod):
    """oracle.weld (the weld option's rule): each vertex lies on the lattice edge its key names;
    welding keeps the triangles, moves each corner at most along its own lattice edge, and
    closes the seams between subdivision batches."""
    from poissonrecon_gpu_gb300 import shapes
    xyz, nrm = shapes.torus(30000, seed=2)
    D = 7
    o = oracle_mod.Oracle(D, threads=4)
    o.set_points(xyz, nrm)
    o.reconstruct()
    v, f, k = o.get("mesh_v").reshape(-1, 3), o.get("mesh_f").reshape(-1, 3), o.get("mesh_vkey")
    assert len(k) == len(v) and len(np.unique(k)) < len(k)
    axis = k % 3
    lat = k // 3
    lc = np.stack([(lat >> 40) & 0xFFFFF, (lat >> 20) & 0xFFFFF, lat & 0xFFFFF], 1).astype(np.float64) / (1 << D)
    t = v.astype(np.float64) - lc
    on = np.ones(len(v), bool)
    for ax in range(3):
        sel = axis == ax
        others = [q for q in range(3) if q != ax]
        on[sel] &= np.all(t[sel][:, others] == 0, axis=1)
        on[sel] &= (t[sel, ax] >= 0) & (t[sel, ax] <= 1.0 / (1 << D))
    assert on.all()
    wv, wf = oracle_mod.weld(v, f, k)
    assert len(wf) == len(f) and len(wv) == len(np.unique(k[f.ravel()]))
    assert np.abs(wv[wf] - v[f]).max() <= 1.0 / (1 << D)

    def open_edges(ff):
        e = np.sort(np.concatenate([ff[:, [0, 1]], ff[:, [1, 2]], ff[:, [2, 0]]]), axis=1)
        _, cnt = np.unique(e, axis=0, return_counts=True)
        return int((cnt == 1).sum())
    assert open_edges(wf) * 50 < open_edges(f)


def test_density_depth_rule(oracle_mod):
    """oracle.occupied_per_depth against the Morton prefixes of the sorted points, and the
    density-based depth rule: sparser clouds (fewer points on the same surface) get coarser."""
    from poissonrecon_gpu_gb300 import shapes
    D = 9
    depths = []
    for n in (2000, 20000, 200000):
        xyz, nrm = shapes.sphere(n, seed=4)
        o = oracle_mod.Oracle(D, threads=4)
        o.set_points(xyz, nrm)
        o.build_octree()
        occ = oracle_mod.occupied_per_depth(o)
        key = o.get("key")[o.get("base")[D]:][o.get("pnum")[o.get("base")[D]:] > 0]
        for d in range(D + 1):
            assert occ[d] == len(np.unique(key >> (3 * (D - d)))), (n, d)
        depths.append(oracle_mod.choose_depth(n, occ, D, 8.0))
        # n / occupied is non-increasing in depth, and the rule picks the last depth meeting it
        dd = depths[-1]
        assert dd == 2 or n / occ[dd] >= 8.0
        assert dd == D or n / occ[dd + 1] < 8.0
    assert depths[0] < depths[1] < depths[2]
