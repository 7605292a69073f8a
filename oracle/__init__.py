"""ctypes wrapper of the CPU oracle (oracle/oracle.cpp).

Test infrastructure: only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg use this module.  The product library never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

# element types of the arrays exposed by orc_get()
_DTYPES = {
    "points": np.float32, "normals": np.float32, "sort_idx": np.int64,
    "base": np.int64, "count": np.int64, "key": np.int64,
    "pidx": np.int32, "pnum": np.int32, "parent": np.int32, "children": np.int32,
    "neighs": np.int32, "didx": np.int32, "dnum": np.int32, "point_node": np.int32,
    "dot": np.float64, "ddot": np.float64, "d2dot": np.float64, "stencil": np.float32,
    "vfield": np.float32, "divergence": np.float32, "x": np.float32,
    "cg_iters": np.int32, "cg_rr": np.float32, "point_value": np.float32,
    "mesh_v": np.float32, "mesh_f": np.int32, "mesh_vkey": np.int64, "has_tri": np.int32, "has_int": np.int32,
    "batch_tri": np.int64, "center": np.float32, "scale": np.float32, "iso": np.float32,
    "subdivide_roots": np.int64,
    "vcells": np.int64,
    "vfield64": np.float64, "divergence64": np.float64, "x64": np.float64, "point_value64": np.float64,
    "cg_iters64": np.int32, "stencil64": np.float64, "iso64": np.float64,
}


def occupied_per_depth(o) -> np.ndarray:
    """Nodes of each depth holding at least one point, from the oracle's octree (pnum, base)."""
    base, pnum = o.get("base"), o.get("pnum")
    return np.array([int((pnum[base[d]:base[d + 1]] > 0).sum()) for d in range(len(base) - 1)], np.int64)


def choose_depth(n: int, occupied, max_depth: int, samples_per_node: float) -> int:
    """The density-based depth rule of prgpu_choose_depth: the largest d in 2..max_depth with
    n / occupied[d] >= samples_per_node (2 when none is).  Kazhdan's samples-per-node criterion
    over the whole cloud; the reference fixes maxDepth at compile time (main.cu:69)."""
    best = 2
    for d in range(2, max_depth + 1):
        if occupied[d] > 0 and n / occupied[d] >= samples_per_node:
            best = d
    return best


def weld(v: np.ndarray, f: np.ndarray, vkey: np.ndarray):
    """The weld option's rule on the oracle's mesh: one vertex per finest-lattice edge across
    subdivision batches (the reference keeps one per edge and batch, main.cu:3799-4564).  A
    welded vertex sits where the first triangle corner on its edge, in triangle order, puts it.
    v [nv, 3], f [nt, 3], vkey [nv] (orc_get "mesh_vkey"); returns (vertices in key order, faces)."""
    corners = np.asarray(f, dtype=np.int64).ravel()
    keys, first, inv = np.unique(np.asarray(vkey)[corners], return_index=True, return_inverse=True)
    return np.asarray(v).reshape(-1, 3)[corners[first]], inv.reshape(-1, 3).astype(np.int32)


def build(force: bool = False) -> str:
    """Compile liboracle.so with oracle/build.sh (g++, OpenMP)."""
    src = os.path.join(_HERE, "oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["sh", os.path.join(_HERE, "build.sh")])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, i64, c_int, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        L.orc_create.restype = vp
        L.orc_create.argtypes = [c_int, c_int]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_points.argtypes = [vp, vp, vp, i64]
        for name in ("orc_build_octree", "orc_vector_field", "orc_divergence",
                     "orc_point_values", "orc_marching_cubes"):
            getattr(L, name).argtypes = [vp]
        L.orc_build_basis.argtypes = [vp, c_int]
        L.orc_set_root_stride.argtypes = [vp, c_int]
        L.orc_set_cascadic.argtypes = [vp, c_int]
        L.orc_solve.argtypes = [vp, c_int, dbl, c_int]
        L.orc_fp64_run.argtypes = [vp, dbl]
        L.orc_reconstruct.argtypes = [vp, c_int, dbl, c_int]
        L.orc_get.restype = vp
        L.orc_get.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(i64)]
        L.orc_set_f32.argtypes = [vp, ctypes.c_char_p, vp, i64]
        L.orc_mc_table.argtypes = [vp, vp]
        L.orc_luts.argtypes = [vp, vp]
        _lib = L
    return _lib


class Oracle:
    """One reconstruction on the CPU, stage by stage (reference semantics)."""

    def __init__(self, depth: int, threads: int | None = None):
        self.depth = depth
        self.threads = threads or os.cpu_count() or 1
        self._h = lib().orc_create(depth, self.threads)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def set_points(self, xyz: np.ndarray, nrm: np.ndarray):
        self._xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        self._nrm = np.ascontiguousarray(nrm, dtype=np.float32)
        rc = lib().orc_set_points(self._h, self._xyz.ctypes.data, self._nrm.ctypes.data, len(self._xyz))
        if rc:
            raise ValueError("oracle rejected the point set")

    def build_octree(self):
        lib().orc_build_octree(self._h)

    def build_basis(self, full_tables: bool = True):
        lib().orc_build_basis(self._h, int(full_tables))

    def vector_field(self):
        lib().orc_vector_field(self._h)

    def divergence(self):
        lib().orc_divergence(self._h)

    def solve(self, mode: int = 0, tol: float = 1e-5, max_iter: int = 10000):
        lib().orc_solve(self._h, mode, tol, max_iter)

    def point_values(self):
        lib().orc_point_values(self._h)

    def marching_cubes(self):
        lib().orc_marching_cubes(self._h)

    def set_cascadic(self, on: bool = True):
        """Coarse-to-fine solve: each depth's right-hand side less the coarser solution."""
        lib().orc_set_cascadic(self._h, int(on))

    def fp64_run(self, tol: float = 1e-6):
        """Precision study: the pipeline after the octree and tables in FP64 (needs
        build_basis(True)); results under vfield64, divergence64, x64,
        point_value64, cg_iters64, iso64."""
        if lib().orc_fp64_run(self._h, tol):
            raise RuntimeError("fp64_run needs the full tables (build_basis(True))")

    def set_root_stride(self, stride: int):
        """Timing samples only: subdivide every stride-th root (0: none)."""
        lib().orc_set_root_stride(self._h, stride)

    def reconstruct(self, mode: int = 0, tol: float = 1e-5, max_iter: int = 10000):
        lib().orc_reconstruct(self._h, mode, tol, max_iter)

    def get(self, name: str) -> np.ndarray:
        n = ctypes.c_int64(0)
        ptr = lib().orc_get(self._h, name.encode(), ctypes.byref(n))
        if n.value < 0:
            raise KeyError(name)
        dt = np.dtype(_DTYPES[name])
        if n.value == 0:
            return np.zeros(0, dtype=dt)
        buf = (ctypes.c_char * (n.value * dt.itemsize)).from_address(ptr)
        return np.frombuffer(buf, dtype=dt).copy()

    def set_f32(self, name: str, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=np.float32).ravel()
        if lib().orc_set_f32(self._h, name.encode(), a.ctypes.data, a.size):
            raise KeyError(name)


def mc_table():
    counts = np.zeros(256, np.int32)
    edges = np.zeros((256, 16), np.int32)
    lib().orc_mc_table(counts.ctypes.data, edges.ctypes.data)
    return counts, edges


def luts():
    p = np.zeros((8, 27), np.int32)
    c = np.zeros((8, 27), np.int32)
    lib().orc_luts(p.ctypes.data, c.ctypes.data)
    return p, c
