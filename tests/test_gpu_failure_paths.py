"""Failure paths of the C ABI, made to happen without faulting or hanging the GPU.

The reference has no failure handling to compare with: its I/O errors and
missing device features end the process (PointStream.inl:33,
CG_CUDA.cuh:359-373), and its kernels' launch errors go unchecked (Debug.cuh:10-24).
Here every failure is a status code, and these tests reach the failure paths
through prgpu_test_hook:

  * a device allocation that fails (PRGPU_HOOK_FAIL_ALLOC), walked over every
    allocation of a small reconstruction: each call returns PRGPU_ERR_NOMEM,
    the memory pool holds exactly what it held before the call (the context's
    buffers and the failed stage's temporaries are released), and the same
    context then reconstructs the same mesh bit for bit;
  * a solver grid barrier whose last arrival never comes
    (PRGPU_HOOK_BARRIER_WAIT: one block more expected than launched, a limit of
    a few thousand polls): the persistent CG kernels give up, the call returns
    PRGPU_ERR_TIMEOUT, and the context and the CSR solver work again afterwards.
"""
import ctypes

import numpy as np
import pytest

from conftest import sphere

pytestmark = pytest.mark.gpu


def test_allocation_failures_release_everything(lib_built):
    import poissonrecon_gpu_gb300 as pg
    xyz, nrm = sphere(4000, seed=3)
    r = pg.Reconstructor(depth=6)
    v0, f0 = r.reconstruct(xyz, nrm)
    r.close()
    used0 = pg.test_hook(pg.HOOK_POOL_USED)
    r = pg.Reconstructor(depth=6)
    k, failures = 1, 0
    while True:
        pg.test_hook(pg.HOOK_FAIL_ALLOC, k)
        try:
            v, f = r.reconstruct(xyz, nrm)
            ok = True
        except pg.PrgpuError as e:
            assert e.status == 3, str(e)
            ok = False
        finally:
            pg.test_hook(pg.HOOK_CLEAR)
        if ok:
            break
        failures += 1
        assert pg.test_hook(pg.HOOK_POOL_USED) == used0, "allocation %d left memory behind" % k
        k += 1
        assert k < 5000
    # every allocation of the pipeline was made to fail once
    assert failures >= 30
    assert np.array_equal(v, v0) and np.array_equal(f, f0)
    r.close()
    assert pg.test_hook(pg.HOOK_POOL_USED) == used0


def test_barrier_timeout_is_reported_and_the_context_recovers(lib_built):
    import poissonrecon_gpu_gb300 as pg
    xyz, nrm = sphere(20000, seed=4)
    ref = pg.Reconstructor(depth=7)
    v0, f0 = ref.reconstruct(xyz, nrm)
    ref.close()
    for mode in (pg.SOLVE_REFERENCE, pg.SOLVE_RELATIVE):
        r = pg.Reconstructor(depth=7, solve_mode=mode, cg_tol=1e-5 if mode == pg.SOLVE_REFERENCE else 1e-6)
        r.set_points(xyz, nrm)
        r.build_octree()
        r.compute_rhs()
        pg.test_hook(pg.HOOK_BARRIER_WAIT, 4000)
        try:
            with pytest.raises(pg.PrgpuError) as ei:
                r.solve()
            assert ei.value.status == 6
        finally:
            pg.test_hook(pg.HOOK_CLEAR)
        v, f = r.reconstruct(xyz, nrm)
        if mode == pg.SOLVE_REFERENCE:
            assert np.array_equal(v, v0) and np.array_equal(f, f0)
        else:
            assert len(f) > 0.9 * len(f0)
        r.close()


def test_csr_barrier_timeout(lib_built):
    torch = pytest.importorskip("torch")
    import poissonrecon_gpu_gb300 as pg
    L = pg._lib()
    dev = torch.device("cuda:0")
    n = 20000
    # 1-D Laplacian plus a positive diagonal
    rowptr = np.zeros(n + 1, np.int32)
    cols, vals = [], []
    for i in range(n):
        for j, v in ((i - 1, -1.0), (i, 2.5), (i + 1, -1.0)):
            if 0 <= j < n:
                cols.append(j)
                vals.append(v)
        rowptr[i + 1] = len(cols)
    b = np.random.default_rng(0).standard_normal(n).astype(np.float32)
    tI, tJ = torch.tensor(rowptr, device=dev), torch.tensor(np.array(cols, np.int32), device=dev)
    tV, tb = torch.tensor(np.array(vals, np.float32), device=dev), torch.tensor(b, device=dev)
    x = torch.zeros(n, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    it = ctypes.c_int32(0)
    pg.test_hook(pg.HOOK_BARRIER_WAIT, 4000)
    try:
        rc = L.prgpu_cg_csr(n, len(vals), tI.data_ptr(), tJ.data_ptr(), tV.data_ptr(), tb.data_ptr(), x.data_ptr(),
                            1e-5, 10000, ctypes.byref(it), None)
    finally:
        pg.test_hook(pg.HOOK_CLEAR)
    assert rc == 6
    rc = L.prgpu_cg_csr(n, len(vals), tI.data_ptr(), tJ.data_ptr(), tV.data_ptr(), tb.data_ptr(), x.data_ptr(),
                        1e-5, 10000, ctypes.byref(it), None)
    assert rc == 0
    # residual of the recovered solve, on the host
    xs = x.cpu().numpy().astype(np.float64)
    ax = 2.5 * xs
    ax[1:] -= xs[:-1]
    ax[:-1] -= xs[1:]
    assert np.linalg.norm(ax - b) <= 2e-5 * max(1.0, np.linalg.norm(b)) + 1e-4


def test_hook_arguments_are_checked(lib_built):
    import poissonrecon_gpu_gb300 as pg
    L = pg._lib()
    assert L.prgpu_test_hook(pg.HOOK_FAIL_ALLOC, 0, None) == 1
    assert L.prgpu_test_hook(pg.HOOK_BARRIER_WAIT, 0, None) == 1
    assert L.prgpu_test_hook(pg.HOOK_POOL_USED, 0, None) == 1
    assert L.prgpu_test_hook(99, 0, None) == 1
    assert L.prgpu_test_hook(pg.HOOK_CLEAR, 0, None) == 0
