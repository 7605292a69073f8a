"""libprgpu.so loads and exports the C ABI; host-only entry points work without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import REPO


def _declared_symbols():
    src = open(os.path.join(REPO, "include", "prgpu.h")).read()
    return sorted(set(re.findall(r"^(?:int|int64_t|const char\s*\*)\s*(prgpu_[a-z_0-9]+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(lib_built):
    L = ctypes.CDLL(lib_built)
    syms = _declared_symbols()
    assert len(syms) >= 18
    for s in syms:
        assert hasattr(L, s), s
    import poissonrecon_gpu_gb300 as pg
    assert set(pg.SIGNATURES) == set(syms)


def test_params_default(lib_built):
    import poissonrecon_gpu_gb300 as pg
    p = pg.Params()
    assert pg._lib().prgpu_params_default(ctypes.byref(p)) == 0
    assert (p.depth, p.solve_mode, p.cg_max_iter) == (8, 0, 10000)
    assert abs(p.cg_tol - 1e-5) < 1e-20


def test_create_rejects_bad_depth(lib_built):
    import poissonrecon_gpu_gb300 as pg
    p = pg.Params()
    pg._lib().prgpu_params_default(ctypes.byref(p))
    p.depth = 40
    h = ctypes.c_void_p()
    assert pg._lib().prgpu_create(ctypes.byref(p), ctypes.byref(h)) == 4


def test_ply_round_trip(lib_built, tmp_path):
    import poissonrecon_gpu_gb300 as pg
    rng = np.random.default_rng(0)
    v = rng.random((10, 3)).astype(np.float32)
    f = rng.integers(0, 10, (7, 3)).astype(np.int32)
    for binary in (True, False):
        path = str(tmp_path / ("m%d.ply" % binary))
        pg.write_mesh(path, v, f, binary=binary)
        txt = open(path, "rb").read(200)
        assert txt.startswith(b"ply\nformat " + (b"binary_little_endian" if binary else b"ascii"))
    # oriented points: binary and ascii PLY, .bnpts, ascii rows
    xyz = rng.random((25, 3)).astype(np.float32)
    nrm = rng.standard_normal((25, 3)).astype(np.float32)
    p1 = tmp_path / "p.ply"
    with open(p1, "wb") as fh:
        fh.write(b"ply\nformat binary_little_endian 1.0\nelement vertex 25\n")
        for name in ("x", "y", "z", "nx", "ny", "nz"):
            fh.write(b"property float %s\n" % name.encode())
        fh.write(b"end_header\n")
        fh.write(np.concatenate([xyz, nrm], 1).astype("<f4").tobytes())
    a, b = pg.read_points(str(p1))
    assert np.array_equal(a, xyz) and np.array_equal(b, nrm)
    p2 = tmp_path / "p.bnpts"
    np.concatenate([xyz, nrm], 1).astype(np.float32).tofile(p2)
    a, b = pg.read_points(str(p2))
    assert np.array_equal(a, xyz) and np.array_equal(b, nrm)
    p3 = tmp_path / "p_ascii.ply"
    with open(p3, "w") as fh:
        fh.write("ply\nformat ascii 1.0\nelement vertex 25\n")
        for name in ("x", "y", "z", "nx", "ny", "nz"):
            fh.write("property float %s\n" % name)
        fh.write("end_header\n")
        for r in np.concatenate([xyz, nrm], 1):
            fh.write(" ".join("%.9g" % x for x in r) + "\n")
    a, b = pg.read_points(str(p3))
    assert np.allclose(a, xyz) and np.allclose(b, nrm)


def test_read_points_errors(lib_built, tmp_path):
    import poissonrecon_gpu_gb300 as pg
    bad = tmp_path / "bad.ply"
    bad.write_bytes(b"ply\nformat binary_little_endian 1.0\nelement vertex 10\nproperty float x\nend_header\n")
    with pytest.raises(pg.PrgpuError):
        pg.read_points(str(bad))
    with pytest.raises(pg.PrgpuError):
        pg.read_points(str(tmp_path / "missing.ply"))
    trunc = tmp_path / "trunc.ply"
    hdr = b"ply\nformat binary_little_endian 1.0\nelement vertex 10\n" + \
        b"".join(b"property float %s\n" % n for n in (b"x", b"y", b"z", b"nx", b"ny", b"nz")) + b"end_header\n"
    trunc.write_bytes(hdr + b"\0" * 40)
    with pytest.raises(pg.PrgpuError):
        pg.read_points(str(trunc))


def test_cli_usage(lib_built):
    exe = os.path.join(REPO, "poissonrecon_gpu_gb300", "prgpu")
    r = subprocess.run([exe], capture_output=True)
    assert r.returncode == 2 and b"usage" in r.stderr
