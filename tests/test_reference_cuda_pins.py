"""Pins of the oracle and the library to the reference's own CUDA build.

tests/golden/ref_cuda_sphere50k_d8.{npz,json} come from
tests/golden/gen_reference_cuda.py, which runs the reference's
pipelineBuildNodeArray (main.cu:511-841) and its stock main()
(main.cu:3247-4573), built from the unchanged sources by oracle/ref_cuda.sh, on
a GB300, on the 50,000-point sphere (shapes.sphere(50000, seed=0)) at the
reference's maxDepth 8.  The npz holds a SHA-256 digest of each reference
array, every position where its pidx differs from this project's (with both
values), and, for the children, the digest with the reference's uninitialised
finest-depth entries set to -1 plus a sample of the raw differences.

For each node field the test requires that
  * this project's array has exactly the recorded values at the recorded
    positions, and patching the reference's values in reproduces the
    reference's digest (so the two arrays agree everywhere else, bit for bit);
  * every difference is a documented reference defect:
      - pidx: the hash insertMin race (Hash.cuh:53-69) -- the slot winner's
        atomicExch(value, INT_MAX) can land after another point's atomicMin, so a
        leaf of 2-3 points whose points straddle lanes keeps a later point's
        index; empty siblings (pidx filled from the preceding sibling) and
        parents (minimum over children) carry the same shift.  Canonical: the
        first point;
      - children of finest-depth nodes: uninitialised in the reference
        (updateEmptyNodeInfo, main.cu:466-472); canonical -1;
  * keys, pnum, parent, neighbours, didx, dnum, the sorted normalised points and
    normals have no difference; the point-to-leaf map agrees once the
    reference's index within the finest depth is made global (+ base[D]);
  * the reference's three runs agree with each other in every field but pidx,
    whose racy entries change from run to run.
The mesh comparison (json): the same triangle count, and the symmetric Hausdorff
distance and iso-value difference recorded.
"""
import hashlib
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
NPZ = os.path.join(HERE, "golden", "ref_cuda_sphere50k_d8.npz")
JSN = os.path.join(HERE, "golden", "ref_cuda_sphere50k_d8.json")
D = 8
EXACT = ("key", "pnum", "parent", "neighs", "didx", "dnum", "points", "normals")


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _as_ref(arrays, base):
    """This project's arrays in the reference's dtypes and conventions."""
    out = {}
    for f in ("pidx", "pnum", "parent", "children", "neighs", "didx", "dnum"):
        out[f] = np.asarray(arrays[f], dtype=np.int32).ravel()
    out["key"] = np.asarray(arrays["key"], dtype=np.int64).ravel()
    out["points"] = np.asarray(arrays["points"], dtype=np.float32).ravel()
    out["normals"] = np.asarray(arrays["normals"], dtype=np.float32).ravel()
    out["point_node"] = (np.asarray(arrays["point_node"], dtype=np.int64) - int(base[D])).astype(np.int32)
    return out


def _check(arrays):
    z = np.load(NPZ)
    info = json.load(open(JSN))
    base = z["base"]
    ours = _as_ref(arrays, np.append(base, 0))
    for f in EXACT + ("point_node",):
        assert _digest(ours[f]) == str(z["sha256_" + f]), f
    idx, ref, rec = z["diff_pidx_idx"], z["diff_pidx_ref"], z["diff_pidx_ours"]
    assert np.array_equal(ours["pidx"][idx], rec)
    b = ours["pidx"].copy()
    b[idx] = ref
    assert _digest(b) == str(z["sha256_pidx"])
    # children: the reference's array with its uninitialised finest-depth rows set to -1
    # is this project's array; a sample of the raw differences sits at finest nodes
    assert _digest(ours["children"]) == str(z["sha256_children_canonical"])
    assert np.all(ours["children"].reshape(-1, 8)[int(base[D]):] == -1)
    idx = z["diff_children_idx"]
    assert np.all(idx // 8 >= base[D]) and np.all(ours["children"][idx] == -1)
    # pidx: insertMin race
    pidx, pnum = ours["pidx"], ours["pnum"]
    idx, ref = z["diff_pidx_idx"], z["diff_pidx_ref"]
    assert len(idx) <= 100
    shift = ref - pidx[idx]
    assert np.all((shift >= 1) & (shift <= 2))
    groups = np.unique((idx[idx >= base[D]] - 1) // 8)
    for g in groups:   # each affected finest group holds a leaf whose reference pidx is one of its own later points
        sl = slice(1 + 8 * g, 9 + 8 * g)
        m = dict(zip(idx.tolist(), ref.tolist()))
        racy = [i for i in range(sl.start, sl.stop)
                if pnum[i] >= 2 and i in m and pidx[i] < m[i] <= pidx[i] + pnum[i] - 1]
        assert racy, g
    # the reference's own runs: every field repeats except pidx, which the race changes
    r2r = info["run_to_run_differences"]
    assert all(v == [0, 0] for f, v in r2r.items() if f != "pidx")
    assert max(r2r["pidx"]) > 0
    return info


@pytest.fixture(scope="module")
def oracle_arrays(oracle_mod):
    from poissonrecon_gpu_gb300 import shapes
    xyz, nrm = shapes.sphere(50000, seed=0)
    o = oracle_mod.Oracle(D)
    o.set_points(xyz, nrm)
    o.build_octree()
    return {f: o.get(f) for f in ("key", "pidx", "pnum", "parent", "children", "neighs", "didx", "dnum", "points",
                                  "normals", "point_node")}


def test_oracle_pinned_to_reference_build(oracle_arrays):
    info = _check(oracle_arrays)
    assert info["reference"]["mesh"]["triangles"] > 0


@pytest.mark.gpu
def test_library_pinned_to_reference_build(lib_built):
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    xyz, nrm = shapes.sphere(50000, seed=0)
    r = pg.Reconstructor(depth=D)
    r.set_points(xyz, nrm)
    r.build_octree()
    arrays = {f: r.get(f) for f in ("key", "pidx", "pnum", "parent", "children", "neighs", "didx", "dnum",
                                    "points", "normals", "point_node")}
    info = _check(arrays)
    # the same points and solver schedule end to end: mesh against the reference's mesh
    v, f = r.reconstruct(xyz, nrm)
    ref_tri = info["reference"]["mesh"]["triangles"]
    assert abs(len(f) - ref_tri) <= 0.005 * ref_tri
    # the reference's iso-value changes by about 1e-4 from run to run (its CG sums with
    # FP64 atomics in arrival order, CG_CUDA.cuh:212-240): compare with the mean of its runs
    runs = info["reference"]["iso_printed_runs"]
    iso_ref = float(np.mean(runs))
    spread = max(runs) - min(runs)
    assert abs(float(r.get("iso")[0]) - iso_ref) <= 2e-4 * abs(iso_ref)
    assert spread > 0
    r.close()
