"""GB300 Poisson surface reconstruction: Python host interface over libprgpu.so.

The compute path is the sm_103a CUDA library built from ``csrc/``; this module
only moves arrays across its C ABI (``include/prgpu.h``).  The stage methods
mirror the reference's stage functions (main.cu):

==========================  ==============================================
``build_octree``            ``pipelineBuildNodeArray`` (main.cu:511)
``compute_rhs``             basis tables, ``computeVectorField``, divergence
``solve``                   ``LaplacianIteration`` / ``solverCG_DeviceToDevice``
``eval_points``             ``calculatePointsImplicitFunctionValue`` + iso
``extract_mesh``            marching cubes + coarse-leaf subdivision
==========================  ==============================================

There is no CPU fallback: constructing a :class:`Reconstructor` without the
compiled library or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libprgpu.so")

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "size limit",
          5: "not converged", 6: "device wait timed out", 7: "I/O error"}
SOLVE_REFERENCE, SOLVE_RELATIVE = 0, 1

# element types of the arrays behind prgpu_get_array
ARRAY_DTYPES = {
    "key": np.int64, "pidx": np.int32, "pnum": np.int32, "didx": np.int32, "dnum": np.int32,
    "parent": np.int32, "children": np.int32, "neighs": np.int32, "point_node": np.int32,
    "points": np.float32, "normals": np.float32, "sort_idx": np.uint32, "base": np.int64,
    "count": np.int64, "center": np.float32, "scale": np.float32, "vfield": np.float32,
    "divergence": np.float32, "stencil": np.float32, "ddot_rows": np.float32, "dot": np.float64,
    "ddot": np.float64, "d2dot": np.float64, "x": np.float32, "cg_iters": np.int32, "cg_rr": np.float32,
    "point_value": np.float32, "point_weight": np.float32, "iso": np.float32, "has_tri": np.int32, "has_int": np.int32,
    "batch_tri": np.int64, "subdivide_roots": np.int64,
}


class PrgpuError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        msg = "%s failed: %s (%s)" % (where, STATUS.get(status, status), _lib().prgpu_last_error().decode())
        super().__init__(msg)


class Params(ctypes.Structure):
    _fields_ = [("depth", ctypes.c_int32), ("solve_mode", ctypes.c_int32), ("cg_tol", ctypes.c_double),
                ("cg_max_iter", ctypes.c_int32), ("device", ctypes.c_int32), ("weld", ctypes.c_int32),
                ("density_weights", ctypes.c_int32), ("cascadic", ctypes.c_int32), ("learned", ctypes.c_int32),
                ("refine", ctypes.c_int32), ("stable_basis", ctypes.c_int32), ("reserved", ctypes.c_int32 * 2)]


class Mesh(ctypes.Structure):
    _fields_ = [("n_vertices", ctypes.c_int64), ("n_triangles", ctypes.c_int64),
                ("vertices", ctypes.POINTER(ctypes.c_float)), ("triangles", ctypes.POINTER(ctypes.c_int32))]


class NodeArrays(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int64), ("max_depth", ctypes.c_int32),
                ("base", ctypes.c_void_p), ("key", ctypes.c_void_p), ("pidx", ctypes.c_void_p),
                ("pnum", ctypes.c_void_p), ("parent", ctypes.c_void_p), ("children", ctypes.c_void_p),
                ("neighs", ctypes.c_void_p), ("didx", ctypes.c_void_p), ("dnum", ctypes.c_void_p)]


# every entry point of include/prgpu.h with its ctypes signature
_VP, _I64, _I32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
SIGNATURES = {
    "prgpu_params_default": (ctypes.c_int, [ctypes.POINTER(Params)]),
    "prgpu_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(_VP)]),
    "prgpu_destroy": (ctypes.c_int, [_VP]),
    "prgpu_set_points": (ctypes.c_int, [_VP, _VP, _VP, _I64]),
    "prgpu_set_points_device": (ctypes.c_int, [_VP, _VP, _VP, _I64]),
    "prgpu_build_octree": (ctypes.c_int, [_VP]),
    "prgpu_compute_rhs": (ctypes.c_int, [_VP]),
    "prgpu_solve": (ctypes.c_int, [_VP]),
    "prgpu_solve_depth": (ctypes.c_int, [_VP, _I32, _I32]),
    "prgpu_get_node_arrays": (ctypes.c_int, [_VP, ctypes.POINTER(NodeArrays)]),
    "prgpu_eval_points": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_float)]),
    "prgpu_extract_mesh": (ctypes.c_int, [_VP]),
    "prgpu_get_mesh": (ctypes.c_int, [_VP, ctypes.POINTER(Mesh)]),
    "prgpu_reconstruct": (ctypes.c_int, [_VP, _VP, _VP, _I64, ctypes.POINTER(Mesh)]),
    "prgpu_reconstruct_batch": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP, ctypes.c_int32, ctypes.POINTER(Mesh)]),
    "prgpu_mesh_free": (ctypes.c_int, [ctypes.POINTER(Mesh)]),
    "prgpu_get_array": (ctypes.c_int, [_VP, ctypes.c_char_p, _VP, _I64, ctypes.POINTER(_I64)]),
    "prgpu_set_array": (ctypes.c_int, [_VP, ctypes.c_char_p, _VP, _I64]),
    "prgpu_stats_json": (ctypes.c_int, [_VP, ctypes.c_char_p, _I64]),
    "prgpu_last_error": (ctypes.c_char_p, []),
    "prgpu_get_stream": (ctypes.c_int, [_VP, ctypes.POINTER(_VP)]),
    "prgpu_set_profiling": (ctypes.c_int, [_VP, _I32]),
    "prgpu_kernel_launches": (ctypes.c_int64, []),
    "prgpu_test_hook": (ctypes.c_int, [_I32, _I64, ctypes.POINTER(_I64)]),
    "prgpu_load_preconditioner": (ctypes.c_int, [_VP, ctypes.c_char_p]),
    "prgpu_trainer_create": (ctypes.c_int, [_I32, ctypes.c_uint64, ctypes.POINTER(_VP)]),
    "prgpu_trainer_destroy": (ctypes.c_int, [_VP]),
    "prgpu_trainer_record": (ctypes.c_int, [_VP, _VP, _I32, ctypes.POINTER(_I64)]),
    "prgpu_trainer_train": (ctypes.c_int, [_VP, _I32, _I32, ctypes.c_float, ctypes.POINTER(ctypes.c_double)]),
    "prgpu_trainer_save": (ctypes.c_int, [_VP, ctypes.c_char_p]),
    "prgpu_trainer_load": (ctypes.c_int, [_VP, ctypes.c_char_p]),
    "prgpu_trainer_info": (ctypes.c_int, [_VP, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "prgpu_trainer_get_params": (ctypes.c_int, [_VP, _VP]),
    "prgpu_trainer_set_params": (ctypes.c_int, [_VP, _VP]),
    "prgpu_trainer_samples": (ctypes.c_int, [_VP, _I64, _I64, _VP, _VP]),
    "prgpu_mlp_forward": (ctypes.c_int, [_VP, _VP, _I64, _VP]),
    "prgpu_mlp_gradients": (ctypes.c_int, [_VP, _VP, _VP, _I64, _VP, ctypes.POINTER(ctypes.c_double)]),
    "prgpu_cg_csr": (ctypes.c_int, [_I32, _I32, _VP, _VP, _VP, _VP, _VP, ctypes.c_float, _I32,
                                    ctypes.POINTER(_I32), ctypes.POINTER(ctypes.c_float)]),
    "prgpu_cg_csr_noalloc": (ctypes.c_int, [_I32, _I32, _VP, _VP, _VP, _VP, _VP, ctypes.c_float, _I32, _VP,
                                            ctypes.POINTER(_I32)]),
    "prgpu_read_points": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_I64), ctypes.POINTER(_VP),
                                         ctypes.POINTER(_VP)]),
    "prgpu_write_mesh_ply": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Mesh), _I32]),
    "prgpu_choose_depth": (ctypes.c_int, [_VP, _VP, _I64, _I32, ctypes.c_double, _I32, ctypes.POINTER(_I32), _VP]),
}

_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libprgpu.so is not built (run poissonrecon_gpu_gb300/builder.py); "
                              "there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def _check(rc, where):
    if rc != 0:
        raise PrgpuError(rc, where)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Reconstructor:
    """One reconstruction context on one GPU (its own CUDA stream)."""

    def __init__(self, depth: int = 8, solve_mode: int = SOLVE_REFERENCE, cg_tol: float = 1e-5,
                 cg_max_iter: int = 10000, device: int = 0, weld: bool = False, density_weights: bool = False,
                 cascadic: bool = False, preconditioner: str | None = None, refine: bool = False,
                 stable_basis: bool = False):
        L = _lib()
        p = Params()
        L.prgpu_params_default(ctypes.byref(p))
        p.depth, p.solve_mode, p.cg_tol, p.cg_max_iter, p.device = depth, solve_mode, cg_tol, cg_max_iter, device
        p.weld = 1 if weld else 0
        p.density_weights = 1 if density_weights else 0
        p.cascadic = 1 if cascadic else 0
        p.learned = 1 if preconditioner else 0
        p.refine = 1 if refine else 0
        p.stable_basis = 1 if stable_basis else 0
        self.params = p
        self._h = _VP()
        _check(L.prgpu_create(ctypes.byref(p), ctypes.byref(self._h)), "prgpu_create")
        self.depth = depth
        if preconditioner:
            self.load_preconditioner(preconditioner)

    def load_preconditioner(self, path: str):
        """Weights of the learned preconditioner from a checkpoint (used when learned=1)."""
        _check(_lib().prgpu_load_preconditioner(self._h, os.fspath(path).encode()), "prgpu_load_preconditioner")

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib().prgpu_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- stages
    def set_points(self, xyz, nrm):
        self._xyz, self._nrm = _f32(xyz), _f32(nrm)
        _check(_lib().prgpu_set_points(self._h, self._xyz.ctypes.data, self._nrm.ctypes.data, len(self._xyz)),
               "prgpu_set_points")

    def set_points_device(self, xyz_ptr: int, nrm_ptr: int, n: int):
        _check(_lib().prgpu_set_points_device(self._h, xyz_ptr, nrm_ptr, n), "prgpu_set_points_device")

    def build_octree(self):
        _check(_lib().prgpu_build_octree(self._h), "prgpu_build_octree")

    def compute_rhs(self):
        _check(_lib().prgpu_compute_rhs(self._h), "prgpu_compute_rhs")

    def solve(self, allow_not_converged: bool = True):
        rc = _lib().prgpu_solve(self._h)
        if rc == 5 and allow_not_converged:
            return False
        _check(rc, "prgpu_solve")
        return True

    def solve_depth(self, depth: int, mode: int = SOLVE_REFERENCE, allow_not_converged: bool = True):
        """One depth's system (prgpu_solve_depth); the other depths' x are kept."""
        rc = _lib().prgpu_solve_depth(self._h, depth, mode)
        if rc == 5 and allow_not_converged:
            return False
        _check(rc, "prgpu_solve_depth")
        return True

    def node_arrays(self) -> dict:
        """The octree as the reference's OctNode fields (prgpu_get_node_arrays)."""
        L = _lib()
        na = NodeArrays()
        _check(L.prgpu_get_node_arrays(self._h, ctypes.byref(na)), "prgpu_get_node_arrays")
        M, D = na.n_nodes, na.max_depth
        out = {"base": np.zeros(D + 2, np.int64), "key": np.zeros(M, np.uint64), "pidx": np.zeros(M, np.int32),
               "pnum": np.zeros(M, np.int32), "parent": np.zeros(M, np.int32),
               "children": np.zeros(8 * M, np.int32), "neighs": np.zeros(27 * M, np.int32),
               "didx": np.zeros(M, np.int32), "dnum": np.zeros(M, np.int32)}
        for k, a in out.items():
            setattr(na, k, a.ctypes.data)
        _check(L.prgpu_get_node_arrays(self._h, ctypes.byref(na)), "prgpu_get_node_arrays")
        return out

    def eval_points(self) -> float:
        iso = ctypes.c_float(0)
        _check(_lib().prgpu_eval_points(self._h, ctypes.byref(iso)), "prgpu_eval_points")
        return iso.value

    def extract_mesh(self):
        _check(_lib().prgpu_extract_mesh(self._h), "prgpu_extract_mesh")

    def mesh(self):
        m = Mesh()
        _check(_lib().prgpu_get_mesh(self._h, ctypes.byref(m)), "prgpu_get_mesh")
        v = np.ctypeslib.as_array(m.vertices, shape=(m.n_vertices * 3,)).reshape(-1, 3).copy() \
            if m.n_vertices else np.zeros((0, 3), np.float32)
        f = np.ctypeslib.as_array(m.triangles, shape=(m.n_triangles * 3,)).reshape(-1, 3).copy() \
            if m.n_triangles else np.zeros((0, 3), np.int32)
        return v, f

    def reconstruct(self, xyz, nrm):
        self.set_points(xyz, nrm)
        self.build_octree()
        self.compute_rhs()
        self.solve()
        self.eval_points()
        self.extract_mesh()
        return self.mesh()

    def reconstruct_batch(self, clouds, depths=None):
        """Reconstruct several (xyz, nrm) clouds in one call (prgpu_reconstruct_batch);
        returns a list of (vertices, triangles)."""
        xyz = np.ascontiguousarray(np.concatenate([np.asarray(c[0], np.float32).reshape(-1, 3) for c in clouds]))
        nrm = np.ascontiguousarray(np.concatenate([np.asarray(c[1], np.float32).reshape(-1, 3) for c in clouds]))
        offsets = np.zeros(len(clouds) + 1, np.int64)
        offsets[1:] = np.cumsum([len(c[0]) for c in clouds])
        dep = None if depths is None else np.ascontiguousarray(depths, dtype=np.int32)
        outs = (Mesh * max(len(clouds), 1))()
        _check(_lib().prgpu_reconstruct_batch(self._h, xyz.ctypes.data, nrm.ctypes.data, offsets.ctypes.data,
                                              None if dep is None else dep.ctypes.data, len(clouds), outs),
               "prgpu_reconstruct_batch")
        result = []
        for k in range(len(clouds)):
            m = outs[k]
            v = np.ctypeslib.as_array(m.vertices, shape=(m.n_vertices * 3,)).reshape(-1, 3).copy() \
                if m.n_vertices else np.zeros((0, 3), np.float32)
            f = np.ctypeslib.as_array(m.triangles, shape=(m.n_triangles * 3,)).reshape(-1, 3).copy() \
                if m.n_triangles else np.zeros((0, 3), np.int32)
            _lib().prgpu_mesh_free(ctypes.byref(m))
            result.append((v, f))
        return result

    # ---- arrays
    def get(self, name: str) -> np.ndarray:
        L = _lib()
        nb = _I64(0)
        _check(L.prgpu_get_array(self._h, name.encode(), None, 0, ctypes.byref(nb)), "prgpu_get_array(%s)" % name)
        dt = np.dtype(ARRAY_DTYPES[name])
        out = np.empty(nb.value // dt.itemsize, dtype=dt)
        _check(L.prgpu_get_array(self._h, name.encode(), out.ctypes.data, nb.value, ctypes.byref(nb)),
               "prgpu_get_array(%s)" % name)
        return out

    def set(self, name: str, arr):
        a = _f32(arr).ravel()
        _check(_lib().prgpu_set_array(self._h, name.encode(), a.ctypes.data, a.nbytes), "prgpu_set_array(%s)" % name)

    def set_profiling(self, enable: bool = True):
        _check(_lib().prgpu_set_profiling(self._h, int(enable)), "prgpu_set_profiling")

    def stream(self) -> int:
        st = _VP()
        _check(_lib().prgpu_get_stream(self._h, ctypes.byref(st)), "prgpu_get_stream")
        return st.value or 0

    def stats(self) -> dict:
        buf = ctypes.create_string_buffer(1 << 16)
        _check(_lib().prgpu_stats_json(self._h, buf, len(buf)), "prgpu_stats_json")
        return json.loads(buf.value.decode())


def choose_depth(xyz, nrm, max_depth: int = 10, samples_per_node: float = 8.0, device: int = 0):
    """Density-based depth (prgpu_choose_depth): the finest depth <= max_depth whose occupied
    nodes hold samples_per_node points each on average.  Returns (depth, occupied nodes per depth)."""
    xyz, nrm = _f32(xyz), _f32(nrm)
    d = ctypes.c_int32(0)
    occ = np.zeros(max_depth + 1, np.int64)
    _check(_lib().prgpu_choose_depth(xyz.ctypes.data, nrm.ctypes.data, len(xyz), max_depth, float(samples_per_node),
                                     device, ctypes.byref(d), occ.ctypes.data), "prgpu_choose_depth")
    return int(d.value), occ


# ---- reference-named helpers -------------------------------------------------
def pipelineBuildNodeArray(xyz, nrm, depth: int, device: int = 0):
    """Octree of an oriented point set; returns the reference OctNode fields as arrays."""
    r = Reconstructor(depth=depth, device=device)
    r.set_points(xyz, nrm)
    r.build_octree()
    out = {k: r.get(k) for k in ("key", "pidx", "pnum", "parent", "children", "neighs", "didx", "dnum",
                                "base", "count", "point_node", "points", "normals", "center", "scale")}
    r.close()
    return out


def solverCG_DeviceToDevice(N: int, nz: int, I: int, J: int, val: int, rhs: int, x: int, tol: float = 1e-5,
                            max_iter: int = 10000):
    """CG on a CSR matrix in device memory (raw device pointers), x0 = 0.  Returns (kernel ms, iterations)."""
    it = _I32(0)
    ms = ctypes.c_float(0)
    rc = _lib().prgpu_cg_csr(N, nz, I, J, val, rhs, x, tol, max_iter, ctypes.byref(it), ctypes.byref(ms))
    if rc not in (0, 5):
        raise PrgpuError(rc, "prgpu_cg_csr")
    return ms.value, it.value


N_PARAMS = 8385
# offsets in the parameter vector: W1 [64 out][64 in], b1, W2 [64][64], b2, w3, b3
P_W1, P_B1, P_W2, P_B2, P_W3, P_B3 = 0, 4096, 4160, 8256, 8320, 8384


def to_bf16_bits(a) -> np.ndarray:
    """float32 -> bfloat16 bit patterns (round to nearest even)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return r.astype(np.uint16)


def from_bf16_bits(b) -> np.ndarray:
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


class Trainer:
    """The learned preconditioner's trainer on one GPU (prgpu_trainer_*): parameters,
    Adam state and the residual/error samples recorded from plain CG."""

    def __init__(self, device: int = 0, seed: int = 0):
        self._h = _VP()
        _check(_lib().prgpu_trainer_create(device, seed, ctypes.byref(self._h)), "prgpu_trainer_create")

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib().prgpu_trainer_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def record(self, rec: "Reconstructor", rows_per_depth: int = 256) -> int:
        n = _I64(0)
        _check(_lib().prgpu_trainer_record(self._h, rec._h, rows_per_depth, ctypes.byref(n)), "prgpu_trainer_record")
        return n.value

    def train(self, steps: int, batch: int = 8192, lr: float = 1e-3) -> float:
        loss = ctypes.c_double(0)
        _check(_lib().prgpu_trainer_train(self._h, steps, batch, lr, ctypes.byref(loss)), "prgpu_trainer_train")
        return loss.value

    def save(self, path: str):
        _check(_lib().prgpu_trainer_save(self._h, os.fspath(path).encode()), "prgpu_trainer_save")

    def load(self, path: str):
        _check(_lib().prgpu_trainer_load(self._h, os.fspath(path).encode()), "prgpu_trainer_load")

    def info(self):
        ns, st = _I64(0), _I64(0)
        _check(_lib().prgpu_trainer_info(self._h, ctypes.byref(ns), ctypes.byref(st)), "prgpu_trainer_info")
        return {"samples": ns.value, "step": st.value}

    def params(self) -> np.ndarray:
        out = np.zeros(N_PARAMS, np.float32)
        _check(_lib().prgpu_trainer_get_params(self._h, out.ctypes.data), "prgpu_trainer_get_params")
        return out

    def set_params(self, p):
        a = np.ascontiguousarray(p, dtype=np.float32)
        assert a.size == N_PARAMS
        _check(_lib().prgpu_trainer_set_params(self._h, a.ctypes.data), "prgpu_trainer_set_params")

    def samples(self, first: int = 0, n: int | None = None):
        """Recorded samples: (features as bf16 bit patterns [n, 64], targets [n])."""
        if n is None:
            n = self.info()["samples"] - first
        f = np.zeros((n, 64), np.uint16)
        t = np.zeros(n, np.float32)
        _check(_lib().prgpu_trainer_samples(self._h, first, n, f.ctypes.data, t.ctypes.data), "prgpu_trainer_samples")
        return f, t

    def forward(self, feat_bits) -> np.ndarray:
        f = np.ascontiguousarray(feat_bits, dtype=np.uint16).reshape(-1, 64)
        y = np.zeros(len(f), np.float32)
        _check(_lib().prgpu_mlp_forward(self._h, f.ctypes.data, len(f), y.ctypes.data), "prgpu_mlp_forward")
        return y

    def gradients(self, feat_bits, targets):
        f = np.ascontiguousarray(feat_bits, dtype=np.uint16).reshape(-1, 64)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.zeros(N_PARAMS, np.float32)
        loss = ctypes.c_double(0)
        _check(_lib().prgpu_mlp_gradients(self._h, f.ctypes.data, t.ctypes.data, len(f), g.ctypes.data,
                                          ctypes.byref(loss)), "prgpu_mlp_gradients")
        return g, loss.value


def kernel_launches() -> int:
    return int(_lib().prgpu_kernel_launches())


HOOK_CLEAR, HOOK_FAIL_ALLOC, HOOK_BARRIER_WAIT, HOOK_POOL_USED = 0, 1, 2, 3


def test_hook(what: int, arg: int = 0) -> int:
    """Failure-path hooks (prgpu_test_hook): returns the hook's output value (pool bytes
    for HOOK_POOL_USED, else 0)."""
    out = _I64(0)
    _check(_lib().prgpu_test_hook(what, arg, ctypes.byref(out)), "prgpu_test_hook")
    return out.value


def read_points(path: str):
    n = _I64(0)
    px, pn = _VP(), _VP()
    _check(_lib().prgpu_read_points(path.encode(), ctypes.byref(n), ctypes.byref(px), ctypes.byref(pn)),
           "prgpu_read_points")
    xyz = np.ctypeslib.as_array(ctypes.cast(px, ctypes.POINTER(ctypes.c_float)), shape=(n.value * 3,))
    nrm = np.ctypeslib.as_array(ctypes.cast(pn, ctypes.POINTER(ctypes.c_float)), shape=(n.value * 3,))
    return xyz.reshape(-1, 3).copy(), nrm.reshape(-1, 3).copy()


def write_mesh(path: str, vertices, triangles, binary: bool = True):
    v = _f32(vertices)
    f = np.ascontiguousarray(triangles, dtype=np.int32)
    m = Mesh(len(v), len(f), v.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
             f.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    _check(_lib().prgpu_write_mesh_ply(path.encode(), ctypes.byref(m), int(binary)), "prgpu_write_mesh_ply")


def build(force: bool = False):
    from . import builder
    return builder.build(force=force)
