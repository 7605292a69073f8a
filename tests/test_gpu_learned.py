"""The learned preconditioner on the GPU, through the C ABI.

  * the tensor-core network (tcgen05 MMAs, TMEM accumulators) against the FP64
    oracle (oracle/mlp.py): forward outputs with the library's bfloat16 rounding
    points emulated (tight) and in plain FP64 (loose); the training kernel's
    gradient against the emulated analytic gradient (tight) and against FP64
    central finite differences (loose: bf16 activations);
  * residual/error pairs recorded from plain CG, training that lowers the loss,
    and a checkpoint that resumes (parameters, Adam moments, step count);
  * flexible CG with the trained network: every depth reaches the same relative
    residual as plain CG, the mesh matches plain CG's (triangle counts within
    0.5 %, Hausdorff <= 1e-3 of the diagonal), and a network that produces
    useless corrections falls back to plain CG and still converges.
"""
import os

import numpy as np
import pytest

from oracle import mlp

pytestmark = pytest.mark.gpu

TOL_EMULATED = 2e-3   # relative to the largest value: fp32 accumulation order, rare bf16 ties
TOL_FP64 = 5e-2       # bf16 activations against an FP64 network


def _features(rng, n):
    import poissonrecon_gpu_gb300 as pg
    f = np.zeros((n, 64), np.float32)
    f[:, :27] = rng.uniform(-1, 1, (n, 27))
    f[:, 27:54] = rng.choice([0.0, 1.0, -0.25, 0.125], (n, 27))
    f[:, 54] = rng.integers(1, 10, n) / 16.0
    return pg.to_bf16_bits(f)


def test_forward_matches_oracle(lib_built):
    import poissonrecon_gpu_gb300 as pg
    rng = np.random.default_rng(0)
    T = pg.Trainer(seed=3)
    p = T.params()
    p[pg.P_W3:pg.P_B3] = rng.standard_normal(64) * 0.3   # a non-trivial output layer
    p[pg.P_B1:pg.P_W2] = rng.standard_normal(64) * 0.1
    p[pg.P_B2:pg.P_W3] = rng.standard_normal(64) * 0.1
    T.set_params(p)
    for n in (1, 128, 1000, 4099):
        fb = _features(rng, n)
        y = T.forward(fb)
        x = pg.from_bf16_bits(fb).astype(np.float64)
        ye, _ = mlp.forward(p, x, emulate=True)
        yf, _ = mlp.forward(p, x, emulate=False)
        scale = np.abs(ye).max()
        assert np.abs(y - ye).max() <= TOL_EMULATED * scale, n
        assert np.abs(y - yf).max() <= TOL_FP64 * scale, n
    T.close()


def test_gradients_match_oracle_and_finite_differences(lib_built):
    import poissonrecon_gpu_gb300 as pg
    rng = np.random.default_rng(1)
    T = pg.Trainer(seed=5)
    p = T.params()
    p[pg.P_W3:pg.P_B3] = rng.standard_normal(64) * 0.3
    p[pg.P_B1:pg.P_W2] = rng.standard_normal(64) * 0.1
    p[pg.P_B2:pg.P_W3] = rng.standard_normal(64) * 0.1
    T.set_params(p)
    n = 700   # five full tiles and a partial one
    fb = _features(rng, n)
    t = rng.standard_normal(n).astype(np.float32)
    g, loss = T.gradients(fb, t)
    x = pg.from_bf16_bits(fb).astype(np.float64)
    le, ge = mlp.loss_and_grad(p, x, t, emulate=True)
    lf, gf = mlp.loss_and_grad(p, x, t, emulate=False)
    assert abs(loss - le) <= 1e-3 * le
    for lo, hi in ((mlp.P_W1, mlp.P_B1), (mlp.P_B1, mlp.P_W2), (mlp.P_W2, mlp.P_B2), (mlp.P_B2, mlp.P_W3),
                   (mlp.P_W3, mlp.P_B3), (mlp.P_B3, mlp.P_COUNT)):
        a, b = g[lo:hi], ge[lo:hi]
        assert np.linalg.norm(a - b) <= 1e-2 * np.linalg.norm(b) + 1e-7, (lo, hi)
    # against FP64 central differences of the FP64 loss, on a sample of every block
    idx = np.concatenate([rng.choice(np.arange(lo, hi), min(12, hi - lo), replace=False)
                          for lo, hi in ((0, 4096), (4096, 4160), (4160, 8256), (8256, 8320), (8320, 8384),
                                         (8384, 8385))])
    fd = mlp.finite_difference(p, x, t, idx, 1e-6)
    assert np.linalg.norm(g[idx] - fd) <= TOL_FP64 * np.linalg.norm(fd)
    assert np.linalg.norm(gf[idx] - fd) <= 1e-4 * np.linalg.norm(fd)   # the oracle's own backward pass
    cos = float(g[idx] @ fd / (np.linalg.norm(g[idx]) * np.linalg.norm(fd)))
    assert cos >= 0.998
    T.close()


def _system(seed, n=20000, depth=8):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    xyz, nrm = shapes.ellipsoid_union(seed, n_min=n, n_max=n + 1)
    r = pg.Reconstructor(depth=depth, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6)
    r.set_points(xyz, nrm)
    r.build_octree()
    r.compute_rhs()
    return r, (xyz, nrm)


@pytest.fixture(scope="module")
def trained(lib_built, tmp_path_factory):
    import poissonrecon_gpu_gb300 as pg
    T = pg.Trainer(seed=11)
    total = 0
    for seed in range(4):
        r, _ = _system(1000 + seed)
        total += T.record(r, rows_per_depth=256)
        r.close()
    assert total == T.info()["samples"] and total > 20000
    f, t = T.samples(0, 1000)
    assert np.all(np.abs(t) <= 64.0) and np.isfinite(t).all()
    xf = pg.from_bf16_bits(f)
    # features: residuals scaled to [-1, 1], the centre neighbour present with coefficient 1
    assert np.abs(xf[:, :27]).max() <= 1.0 and np.all(xf[:, 27 + 13] == 1.0)
    l0 = T.train(1, batch=8192, lr=1e-3)
    l1 = T.train(400, batch=8192, lr=1e-3)
    assert l1 < 0.8 * l0
    path = str(tmp_path_factory.mktemp("lpc") / "lpc.bin")
    T.save(path)
    return T, path


def test_checkpoint_resume(trained, tmp_path):
    import poissonrecon_gpu_gb300 as pg
    T, path = trained
    p0 = T.params()
    U = pg.Trainer(seed=99)
    U.load(path)
    assert U.info()["step"] == T.info()["step"]
    assert np.array_equal(U.params(), p0)
    # the file holds the parameters and both Adam moments: a second save is identical
    again = str(tmp_path / "again.bin")
    U.save(again)
    assert open(again, "rb").read() == open(path, "rb").read()
    # a damaged file is rejected
    bad = str(tmp_path / "bad.bin")
    open(bad, "wb").write(open(path, "rb").read()[:100])
    with pytest.raises(pg.PrgpuError):
        U.load(bad)
    U.close()


def _hausdorff(a, b):
    from scipy.spatial import cKDTree
    return max(cKDTree(b).query(a)[0].max(), cKDTree(a).query(b)[0].max())


def test_learned_solve_matches_plain(trained):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    _, path = trained
    xyz, nrm = shapes.ellipsoid_union(5000, n_min=30000, n_max=30001)   # held out
    plain = pg.Reconstructor(depth=8, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6)
    vp, fp = plain.reconstruct(xyz, nrm)
    learned = pg.Reconstructor(depth=8, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6, preconditioner=path)
    vl, fl = learned.reconstruct(xyz, nrm)
    st = learned.stats()
    rel = np.array(st["cg_rel_residual"])
    assert np.all(rel <= 1e-6 * 1.0001), rel
    assert abs(len(fl) - len(fp)) <= 0.005 * len(fp)
    diag = float(np.linalg.norm(xyz.max(0) - xyz.min(0)))
    assert _hausdorff(vl[np.unique(fl)], vp[np.unique(fp)]) <= 1e-3 * diag
    plain.close()
    learned.close()


def test_useless_network_falls_back_to_plain_cg(trained, tmp_path):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    T, _ = trained
    U = pg.Trainer(seed=1)
    p = np.zeros(pg.N_PARAMS, np.float32)
    # y = -relu(f13) + relu(-f13) = -r_i / s_i: z_i = -r_i / L[centre], so r.z < 0 at once
    p[pg.P_W1 + 0 * 64 + 13] = 1.0
    p[pg.P_W1 + 1 * 64 + 13] = -1.0
    p[pg.P_W2 + 0 * 64 + 0] = 1.0
    p[pg.P_W2 + 1 * 64 + 1] = 1.0
    p[pg.P_W3 + 0] = -1.0
    p[pg.P_W3 + 1] = 1.0
    U.set_params(p)
    path = str(tmp_path / "neg.bin")
    U.save(path)
    xyz, nrm = shapes.ellipsoid_union(5001, n_min=20000, n_max=20001)
    plain = pg.Reconstructor(depth=7, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6)
    vp, fp = plain.reconstruct(xyz, nrm)
    r = pg.Reconstructor(depth=7, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6, preconditioner=path)
    v, f = r.reconstruct(xyz, nrm)
    st = r.stats()
    fb = st["cg_fallback"]
    cnt = r.get("count")
    # depths of at least 256 rows start with the network and fall back at once; smaller ones
    # run plain CG throughout (-1)
    assert all((k == 0) if cnt[d] >= 256 else (k == -1) for d, k in enumerate(fb) if d > 0), fb
    assert np.all(np.array(st["cg_rel_residual"]) <= 1e-6 * 1.0001)
    # plain CG from the start: the same iterations as the plain solver, within reduction order
    assert np.all(np.abs(np.array(st["cg_iters"]) - np.array(plain.stats()["cg_iters"])) <= 1)
    assert abs(len(f) - len(fp)) <= 0.005 * len(fp)
    r.close()
    plain.close()
    U.close()
