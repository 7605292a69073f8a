"""prgpu_cg_csr_noalloc: the CSR conjugate-gradient solve for callers that cannot
allocate device memory at solve time (a framework's caching allocator owns the
device memory, cudaFree's synchronisation is not affordable, or allocation is
forbidden after start-up).  Its scratch lives in a static device array of the
library, so it is checked here, through the C ABI, against the allocating entry
point prgpu_cg_csr on two calls in a row (the second call reuses the array the
first one left behind), and against the row limit of that array.

This file is collected last so that a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 18


def _spd_csr(n, seed):
    rng = np.random.default_rng(seed)
    diag = 2.5 + rng.random(n)
    rows, cols, vals = [], [], []
    for i in range(n):
        for j, v in ((i - 1, -1.0), (i, diag[i]), (i + 1, -1.0)):
            if 0 <= j < n:
                rows.append(i); cols.append(j); vals.append(v)
    rowptr = np.searchsorted(np.array(rows), np.arange(n + 1)).astype(np.int32)
    b = rng.standard_normal(n).astype(np.float32)
    return rowptr, np.array(cols, np.int32), np.array(vals, np.float32), b


def test_noalloc_cg_matches_allocating_cg(lib_built):
    torch = pytest.importorskip("torch")
    import poissonrecon_gpu_gb300 as pg
    L = pg._lib()
    dev = torch.device("cuda:0")
    for call, (n, seed) in enumerate([(40000, 1), (65536, 2)]):
        rowptr, col, val, b = _spd_csr(n, seed)
        tI = torch.tensor(rowptr, device=dev)
        tJ = torch.tensor(col, device=dev)
        tV = torch.tensor(val, device=dev)
        tb = torch.tensor(b, device=dev)
        x_ref = torch.zeros(n, dtype=torch.float32, device=dev)
        x_new = torch.full((n,), 7.0, dtype=torch.float32, device=dev)   # overwritten by the solve
        torch.cuda.synchronize()
        it_ref = ctypes.c_int32(0)
        rc = L.prgpu_cg_csr(n, len(val), tI.data_ptr(), tJ.data_ptr(), tV.data_ptr(), tb.data_ptr(),
                            x_ref.data_ptr(), 1e-5, 10000, ctypes.byref(it_ref), None)
        assert rc == 0, L.prgpu_last_error()
        it_new = ctypes.c_int32(0)
        rc = L.prgpu_cg_csr_noalloc(n, len(val), tI.data_ptr(), tJ.data_ptr(), tV.data_ptr(), tb.data_ptr(),
                                    x_new.data_ptr(), 1e-5, 10000, None, ctypes.byref(it_new))
        assert rc == 0, L.prgpu_last_error()
        xr, xn = x_ref.cpu().numpy(), x_new.cpu().numpy()
        scale = np.abs(xr).max()
        # both are FP32 CG with FP64 reductions; only the reduction order differs
        assert np.abs(xn - xr).max() <= 1e-4 * scale, call
        assert abs(it_new.value - it_ref.value) <= 2, call


def test_noalloc_rejects_oversized_systems(lib_built):
    torch = pytest.importorskip("torch")
    import poissonrecon_gpu_gb300 as pg
    L = pg._lib()
    dev = torch.device("cuda:0")
    n = MAX_ROWS + 1
    t = torch.zeros(n + 1, dtype=torch.int32, device=dev)
    f = torch.zeros(n, dtype=torch.float32, device=dev)
    rc = L.prgpu_cg_csr_noalloc(n, 1, t.data_ptr(), t.data_ptr(), f.data_ptr(), f.data_ptr(), f.data_ptr(),
                                1e-5, 10, None, None)
    assert rc == 4
    assert b"static scratch limit" in L.prgpu_last_error()


def test_noalloc_refuses_a_capturing_stream(lib_built):
    """The call blocks until its solve ends, so it cannot be part of a CUDA graph: on a capturing
    stream it returns PRGPU_ERR_ARG before touching the stream, the capture stays valid, and a
    call after the capture solves as usual."""
    torch = pytest.importorskip("torch")
    import poissonrecon_gpu_gb300 as pg
    L = pg._lib()
    dev = torch.device("cuda:0")
    n = 4096
    rowptr, col, val, b = _spd_csr(n, 3)
    tI, tJ = torch.tensor(rowptr, device=dev), torch.tensor(col, device=dev)
    tV, tb = torch.tensor(val, device=dev), torch.tensor(b, device=dev)
    x = torch.zeros(n, dtype=torch.float32, device=dev)
    y = torch.ones(16, device=dev)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    it = ctypes.c_int32(0)
    with torch.cuda.graph(g, stream=s):
        y.mul_(2.0)
        rc = L.prgpu_cg_csr_noalloc(n, len(val), tI.data_ptr(), tJ.data_ptr(), tV.data_ptr(), tb.data_ptr(),
                                    x.data_ptr(), 1e-5, 10000, ctypes.c_void_p(s.cuda_stream), ctypes.byref(it))
    assert rc == 1 and b"capturing" in L.prgpu_last_error()
    g.replay()
    torch.cuda.synchronize()
    assert float(y[0]) == 2.0
    rc = L.prgpu_cg_csr_noalloc(n, len(val), tI.data_ptr(), tJ.data_ptr(), tV.data_ptr(), tb.data_ptr(),
                                x.data_ptr(), 1e-5, 10000, None, ctypes.byref(it))
    assert rc == 0 and it.value > 0
