"""bench.py's host-side helpers, on the CPU: the workload and config naming, the roofline
arithmetic, the DRAM traffic read from the committed ncu summary, and the clock summary."""
import argparse
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

import bench  # noqa: E402


def _args(**kw):
    a = argparse.Namespace(gpus=1, steps=5, warmup=3, impl="prgpu", points=1_000_000, depth=10, tol=1e-6,
                           shape="torus")
    for k, v in kw.items():
        setattr(a, k, v)
    return a


def test_config_names_the_workload():
    c = bench.config(_args(), "flushed")
    assert c["workload"] == "torus 1000000 points, maxDepth 10, CG to relative residual 1e-06"
    assert c["parallelism"] == "single GPU" and c["l2"] == "flushed"
    c = bench.config(_args(shape="displaced_sphere", points=30_000_000, depth=12, gpus=2), "flushed")
    assert c["workload"].startswith("displaced sphere 30000000 points, maxDepth 12")
    assert c["parallelism"] == "replicas"


def test_workload_shapes():
    for shape in ("torus", "sphere", "displaced_sphere"):
        xyz, nrm = bench.workload(_args(shape=shape, points=2000))
        assert xyz.shape == (2000, 3) and nrm.shape == (2000, 3)
        assert xyz.dtype == np.float32 and np.all(np.isfinite(xyz))
        assert np.allclose(np.linalg.norm(nrm, axis=1), 1.0, atol=1e-5)


def test_measured_traffic_reads_the_committed_table():
    t = bench.measured_traffic(_args())
    assert {"cg", "divergence", "brick_bound", "splat"} <= set(t)
    assert all(isinstance(v, int) and v > 0 for v in t.values())
    # only for the workload the table was measured on
    assert bench.measured_traffic(_args(points=200_000)) == {}
    assert bench.measured_traffic(_args(shape="sphere")) == {}


def test_roofline_of_the_dominant_timer():
    stats = {"kernels": {"cg": {"ms": 30.0, "launches": 10, "bytes": 5.0e10},
                         "splat": {"ms": 8.0, "launches": 10, "bytes": 7.0e9}}}
    r = bench.roofline(stats, {"hbm_gbs": 6772.9}, {"cg": 123})
    assert r["kernel"] == "cg" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    # 5 GB per launch in 3 ms
    assert abs(r["achieved"] - 5.0e9 / 3.0e-3 / 1e9) < 0.1
    assert abs(r["frac"] - r["achieved"] / 6772.9) < 1e-4
    assert r["traffic"] == 123 and r["peak_source"].startswith("measured")
    assert bench.roofline({"kernels": {}}, {}, {}) is None
    # a timer spanning several kernels is not the dominant kernel
    agg = {"kernels": dict(stats["kernels"], divergence={"ms": 40.0, "launches": 10, "bytes": 1e9},
                           divergence_groups={"ms": 20.0, "launches": 10, "bytes": 0})}
    assert bench.roofline(agg, {"hbm_gbs": 6772.9}, {})["kernel"] == "cg"
    assert bench.roofline(stats, {}, {})["peak_source"] == "fallback"


def test_clock_summary(tmp_path):
    p = tmp_path / "clocks.csv"
    p.write_text("0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active\n"
                 "0, 2060, 2070, 1400.0, 0x4, Not Active, Not Active, Not Active, Active\n"
                 "garbage line\n")
    c = bench.Clocks(str(p))
    c.proc = object()   # as if sampling had run
    s = c.summary()
    assert s["sm_max_mhz"] == 2070.0 and s["samples"] == 2
    assert s["sm_mhz"] == 2065.0 and s["reasons"] == ["sw_power_cap"]


def test_kernel_roofline_covers_every_timer():
    stats = {"kernels": {"cg": {"ms": 30.0, "launches": 10, "bytes": 5.0e10},
                         "splat": {"ms": 8.0, "launches": 10, "bytes": 7.0e9},
                         "lists": {"ms": 1.0, "launches": 5, "bytes": 0}}}
    k = bench.kernel_roofline(stats, {"hbm_gbs": 6000.0}, 20.0)
    assert set(k["kernels"]) == {"cg", "splat"}
    assert abs(k["kernels"]["splat"]["achieved_gbs"] - 0.7e9 / 0.8e-3 / 1e9) < 0.1
    # the step's algorithmic bytes (5.7 GB per step) over the step time
    assert abs(k["step_algorithmic_gb"] - 5.7) < 1e-6
    assert abs(k["step_frac"] - 5.7 / 20e-3 / 6000.0) < 1e-4


def test_displaced_sphere_on_a_torch_device():
    torch = __import__("pytest").importorskip("torch")
    from poissonrecon_gpu_gb300 import shapes
    xyz, nrm = shapes.displaced_sphere(5000, seed=1, device=torch.device("cpu"))
    assert xyz.shape == (5000, 3) and xyz.dtype == np.float32
    r = np.linalg.norm(xyz - 0.5, axis=1)
    assert r.min() > 0.35 - 0.05 - 1e-3 and r.max() < 0.35 + 0.05 + 1e-3
    assert np.allclose(np.linalg.norm(nrm, axis=1), 1.0, atol=1e-5)
    # the normal leans away from the radial direction only as far as the displacement slopes
    radial = (xyz - 0.5) / r[:, None]
    assert np.all((nrm * radial).sum(1) > 0.3)
    # the same distribution as the host generator's sample
    xh, _ = shapes.displaced_sphere(5000, seed=1)
    rh = np.linalg.norm(xh - 0.5, axis=1)
    assert np.all(np.abs(np.quantile(r, [0.1, 0.5, 0.9]) - np.quantile(rh, [0.1, 0.5, 0.9])) < 3e-3)
