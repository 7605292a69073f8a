"""The seeded synthetic clouds that stand in for the reference's scanned inputs: reproducible per
seed, unit normals, and the geometry their configurations describe."""
import numpy as np

from poissonrecon_gpu_gb300 import shapes


def _unit(n):
    return np.allclose(np.linalg.norm(n.astype(np.float64), axis=1), 1.0, atol=1e-5)


def test_same_seed_same_cloud():
    for gen in (lambda s: shapes.sphere(3000, seed=s), lambda s: shapes.torus(3000, seed=s),
                lambda s: shapes.ellipsoid_union(s, n_min=3000, n_max=4000),
                lambda s: shapes.superquadric(s, n_min=3000, n_max=4000),
                lambda s: shapes.displaced_sphere(3000, seed=s)):
        a, b, c = gen(5), gen(5), gen(6)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        assert not np.array_equal(a[0], c[0])
        assert a[0].dtype == np.float32 and a[1].dtype == np.float32 and _unit(a[1])


def test_sphere_and_torus_geometry():
    p, n = shapes.sphere(5000, seed=0)
    r = np.linalg.norm(p - 0.5, axis=1)
    assert np.allclose(r, 0.35, atol=1e-6)
    assert np.allclose(n, (p - 0.5) / r[:, None], atol=1e-5)
    p, n = shapes.torus(20000, seed=0, sigma=0.0, kappa=1e9)
    rho = np.hypot(p[:, 0] - 0.5, p[:, 1] - 0.5)
    assert np.abs(np.hypot(rho - 0.3, p[:, 2] - 0.5) - 0.1).max() < 1e-5
    # density 1 + 7x: the dense side holds several times the points of the sparse side
    assert (p[:, 0] > 0.7).sum() > 3 * (p[:, 0] < 0.3).sum()


def test_displaced_sphere_band():
    p, n = shapes.displaced_sphere(20000, seed=0)
    r = np.linalg.norm(p - 0.5, axis=1)
    # radius 0.35 + 0.05 h, |h| <= 1
    assert r.min() >= 0.30 - 1e-5 and r.max() <= 0.40 + 1e-5
    # normals point outward
    assert np.all(((p - 0.5) * n).sum(1) > 0)


def test_superquadric_and_ellipsoids_in_the_unit_cube():
    for s in range(4):
        p, _ = shapes.superquadric(s, n_min=2000, n_max=3000)
        assert p.min() > 0.0 and p.max() < 1.0
        p, n = shapes.ellipsoid_union(s, n_min=2000, n_max=3000)
        assert p.min() > 0.0 and p.max() < 1.0 and _unit(n)
