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
    for flag in (b"--weld", b"--density", b"--cascadic", b"--relative", b"--binary"):
        assert flag in r.stderr
    r = subprocess.run([exe, "--no-such-flag"], capture_output=True)
    assert r.returncode == 2 and b"usage" in r.stderr


def _ply_header(fmt, n, props, pre=b""):
    h = b"ply\nformat %s 1.0\n" % fmt + pre + b"element vertex %d\n" % n
    for t, name in props:
        h += b"property %s %s\n" % (t, name)
    return h + b"end_header\n"


def test_ply_parallel_reader_matches_sequential(lib_built, tmp_path):
    """Large files take the threaded paths (fixed-size binary records, one ascii record per
    line); layouts they do not cover fall back to the sequential reader.  Both give the
    same points, converted through double as the sequential reader converts them."""
    import poissonrecon_gpu_gb300 as pg
    rng = np.random.default_rng(3)
    n = 300_000
    xyz = rng.random((n, 3)).astype(np.float32)
    nrm = rng.standard_normal((n, 3))                   # stored as double
    red = rng.integers(0, 256, n).astype(np.uint8)
    props = [(b"float", b"x"), (b"uchar", b"red"), (b"float", b"y"), (b"float", b"z"),
             (b"double", b"nx"), (b"double", b"ny"), (b"double", b"nz")]
    want_n = nrm.astype(np.float32)
    for order, fmt in (("<", b"binary_little_endian"), (">", b"binary_big_endian")):
        rec = np.zeros(n, dtype=[("x", order + "f4"), ("red", "u1"), ("y", order + "f4"), ("z", order + "f4"),
                                 ("nx", order + "f8"), ("ny", order + "f8"), ("nz", order + "f8")])
        rec["x"], rec["y"], rec["z"], rec["red"] = xyz[:, 0], xyz[:, 1], xyz[:, 2], red
        rec["nx"], rec["ny"], rec["nz"] = nrm[:, 0], nrm[:, 1], nrm[:, 2]
        fast = tmp_path / ("fast%s.ply" % fmt.decode())
        fast.write_bytes(_ply_header(fmt, n, props) + rec.tobytes())
        # an element with a list property before the vertices: sequential reader
        meta = b"element meta 1\nproperty list uchar int ids\n"
        slow = tmp_path / ("slow%s.ply" % fmt.decode())
        one = np.array([2], np.uint8).tobytes() + np.array([7, 9], order + "i4").tobytes()
        slow.write_bytes(_ply_header(fmt, n, props, pre=meta) + one + rec.tobytes())
        a1, b1 = pg.read_points(str(fast))
        a2, b2 = pg.read_points(str(slow))
        assert np.array_equal(a1, xyz) and np.array_equal(b1, want_n)
        assert np.array_equal(a1, a2) and np.array_equal(b1, b2)
    # ascii: one record per line (threaded), and with a blank line (sequential)
    lines = ["%.9g %d %.9g %.9g %.17g %.17g %.17g" % (x[0], r, x[1], x[2], m[0], m[1], m[2])
             for x, r, m in zip(xyz.astype(np.float64), red, nrm)]
    hdr = _ply_header(b"ascii", n, props).decode()
    fast = tmp_path / "fast_ascii.ply"
    fast.write_text(hdr + "\n".join(lines) + "\n3 0 1 2\n")
    slow = tmp_path / "slow_ascii.ply"
    slow.write_text(hdr + "\n".join(lines[: n // 2]) + "\n\n" + "\n".join(lines[n // 2:]) + "\n")
    a1, b1 = pg.read_points(str(fast))
    a2, b2 = pg.read_points(str(slow))
    assert np.array_equal(a1, xyz) and np.array_equal(b1, want_n)
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)


def test_ply_parallel_writer_bytes(lib_built, tmp_path):
    """The threaded ascii writer produces the bytes of one '%g' line per vertex and face, in order."""
    import poissonrecon_gpu_gb300 as pg
    rng = np.random.default_rng(4)
    v = (rng.standard_normal((200_000, 3)) * 10.0 ** rng.integers(-6, 6, (200_000, 1))).astype(np.float32)
    f = rng.integers(0, len(v), (300_000, 3)).astype(np.int32)
    path = tmp_path / "m.ply"
    pg.write_mesh(str(path), v, f, binary=False)
    body = open(path, "rb").read().split(b"end_header\n", 1)[1]
    want = "".join("%g %g %g\n" % tuple(r) for r in v.astype(np.float64)) + \
        "".join("3 %d %d %d\n" % tuple(t) for t in f)
    assert body == want.encode()
    pb = tmp_path / "mb.ply"
    pg.write_mesh(str(pb), v, f, binary=True)
    raw = open(pb, "rb").read().split(b"end_header\n", 1)[1]
    assert raw[: 12 * len(v)] == v.tobytes()
    faces = np.frombuffer(raw[12 * len(v):], dtype=[("n", "u1"), ("i", "<i4", 3)])
    assert np.all(faces["n"] == 3) and np.array_equal(faces["i"], f)
