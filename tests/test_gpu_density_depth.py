"""Density-based depth (prgpu_choose_depth) against the oracle's restatement: the occupied nodes
per depth of the octree built at the maximum depth, and the depth the samples-per-node rule picks
from them; a cloud reconstructed at that depth."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,k", [(3000, 8.0), (50000, 8.0), (50000, 2.0), (400000, 8.0)])
def test_choose_depth_matches_oracle(lib_built, oracle_mod, n, k):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    D = 10
    xyz, nrm = shapes.torus(n, seed=5)
    d, occ = pg.choose_depth(xyz, nrm, max_depth=D, samples_per_node=k)
    o = oracle_mod.Oracle(D)
    o.set_points(xyz, nrm)
    o.build_octree()
    occ_o = oracle_mod.occupied_per_depth(o)
    assert np.array_equal(occ, occ_o)
    assert d == oracle_mod.choose_depth(n, occ_o, D, k)
    assert 2 <= d <= D


def test_reconstruct_at_chosen_depth(lib_built):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    xyz, nrm = shapes.sphere(20000, seed=6)
    d, occ = pg.choose_depth(xyz, nrm, max_depth=12, samples_per_node=4.0)
    assert d < 12 and len(xyz) / occ[d] >= 4.0 > len(xyz) / occ[d + 1]
    r = pg.Reconstructor(depth=d)
    v, f = r.reconstruct(xyz, nrm)
    r.close()
    rad = np.linalg.norm(v[np.unique(f)] - 0.5, axis=1)
    assert len(f) > 1000 and abs(float(rad.mean()) - 0.35) < 0.01
    with pytest.raises(pg.PrgpuError):
        pg.choose_depth(xyz, nrm, max_depth=12, samples_per_node=0.0)
