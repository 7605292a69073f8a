"""Benchmark: end-to-end Poisson reconstruction throughput (points/s) on GB300.

Workload (default): the precision-study configuration -- 1,000,000 seeded
synthetic points on a torus (R=0.3, r=0.1, density 1+7x, position noise
sigma=0.001, von Mises-Fisher normal noise kappa=500), maxDepth 10, per-depth CG
to relative residual 1e-6 with FP64 reductions.  One step is one complete
reconstruction: normalise, octree, tables, splat, divergence, solve, implicit
values + iso-value, marching cubes with subdivision, mesh to host.

  value : points/s with the input already resident in HBM (prgpu_set_points_device)
  e2e   : points/s through prgpu_reconstruct with pinned host buffers, host->device
          copy of the points and device->host copy of the mesh inside the timed region
  solver_study : solve ms to relative residual 1e-6, learned-preconditioned
          flexible CG against plain CG, on held-out unions of ellipsoids at maxDepth 9
  reference_cuda_build : the reference's own CUDA program on the 50,000-point sphere at
          maxDepth 8 (its compile-time depth), beside this library on the same file
  kernel_roofline : every kernel timer's algorithmic bytes over its time, as a fraction of
          the measured HBM copy bandwidth, and the whole step's
  large_config : the 30M-point displaced sphere at maxDepth 12 (--large 1, the default):
          throughput, stages, per-kernel rooflines, plain against learned solve
Timing: CUDA events on the library's stream, per step, L2 flushed (256 MiB
write) between steps; clocks sampled with nvidia-smi during the timed steps.

--impl reference runs the reference path on the host cores: the CPU oracle
(oracle/oracle.cpp, a restatement of the reference pipeline, OpenMP over all
host cores) on a bounded sample of the same workload.  Every stage runs on the
full point set except the subdivision of coarse leaves, which processes every
ROOT_STRIDE-th subdivided leaf; its time is scaled up by the ratio of all
virtual cells to the sampled ones.  The marching-cubes time without any
subdivision is measured once (untimed) to separate the two parts.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

PEAKS = os.path.join(REPO, "MEASURED_PEAKS.json")
ROOT_STRIDE = 400              # CPU sample: subdivide every 400th subdivided leaf


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)   # enough timed work for the 200 ms clock samples
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="prgpu", choices=["prgpu", "reference"])
    ap.add_argument("--points", type=int, default=1_000_000)
    ap.add_argument("--depth", type=int, default=10)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--solver-seeds", type=int, default=200, help="held-out shapes of the learned-vs-plain "
                    "solver study (0: skip)")
    ap.add_argument("--large", type=int, default=1, help="1: also run the 30M-point, maxDepth-12 configuration "
                    "once (large_config object); 0: skip it")
    ap.add_argument("--solver-only", action="store_true", help="run only the learned-vs-plain solver study "
                    "(--solver-seeds shapes) and print it as one JSON line")
    ap.add_argument("--clocks-csv", default=None, help="where to keep the nvidia-smi clock samples "
                    "(default: a temporary directory)")
    ap.add_argument("--shape", default="torus", choices=["torus", "sphere", "displaced_sphere"],
                    help="torus: density 1+7x, noise (default workload); sphere: uniform; displaced_sphere: "
                         "4-octave value-noise displacement (the 30M-point, maxDepth 12 configuration)")
    return ap.parse_args()


def workload(args):
    from poissonrecon_gpu_gb300 import shapes
    if args.shape == "sphere":
        return shapes.sphere(args.points, seed=0)
    if args.shape == "displaced_sphere":
        return shapes.displaced_sphere(args.points, seed=0)
    return shapes.torus(args.points, seed=0)


def config(args, l2):
    shape = args.shape.replace("_", " ")
    return {"workload": "%s %d points, maxDepth %d, CG to relative residual %g" % (shape, args.points, args.depth,
                                                                                   args.tol),
            "points": args.points, "depth": args.depth, "solve": "per-depth CG, rel residual %g, FP64 dots" % args.tol,
            "l2": l2, "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_reference(args, steps, warmup):
    """The reference path on the host cores: the oracle, subdivision sampled."""
    import oracle
    oracle.build()
    xyz, nrm = workload(args)
    threads = os.cpu_count() or 1
    o = oracle.Oracle(args.depth, threads=threads)
    o.set_points(xyz, nrm)

    def stages():
        o.build_octree()
        o.build_basis(True)
        o.vector_field()
        o.divergence()
        o.solve(1, args.tol, 10000)
        o.point_values()

    # marching cubes without subdivision, once: the part the sample does not scale
    stages()
    o.set_root_stride(0)
    t = time.perf_counter()
    o.marching_cubes()
    t_real = time.perf_counter() - t
    o.set_root_stride(ROOT_STRIDE)
    runs = []
    for it in range(warmup + steps):
        t0 = time.perf_counter()
        stages()
        t1 = time.perf_counter()
        o.marching_cubes()
        t2 = time.perf_counter()
        total, kept = (int(v) for v in o.get("vcells"))
        scale = total / kept if kept else 1.0
        t_full = (t1 - t0) + t_real + max(t2 - t1 - t_real, 0.0) * scale
        if it >= warmup:
            runs.append((t2 - t0, t_full, kept, total))
    wall = float(np.mean([r[0] for r in runs]))
    per = float(np.mean([r[1] for r in runs]))
    kept, total = runs[-1][2], runs[-1][3]
    return {"value": len(xyz) / per, "unit": "points/s", "cores": threads, "kind": "port",
            "measured_s_per_step": wall, "estimated_full_s_per_step": per,
            "measured_sample_points_per_s": len(xyz) / wall,
            "sample": "CPU oracle (OpenMP restatement of the reference pipeline, %d threads) on the full %d-point "
                      "torus at maxDepth %d, relative-residual CG; subdivision of every %dth subdivided leaf "
                      "(%d of %d virtual cells), its time scaled by the cell ratio; %.1f s measured per step, "
                      "%.1f s estimated for the whole path" % (threads, len(xyz), args.depth, ROOT_STRIDE, kept,
                                                              total, wall, per)}, per


TRAFFIC = os.path.join(REPO, "profiles", "dram_traffic_torus1M_d10.md")


def measured_table(args):
    """Per kernel timer, from the committed ncu summary of this workload: DRAM bytes per launch
    ('traffic') and, where a full-section capture measured it, the issue-slot use ('issue')."""
    if args.shape != "torus" or args.points != 1_000_000 or args.depth != 10 or not os.path.exists(TRAFFIC):
        return {}
    out = {}
    for line in open(TRAFFIC):
        cols = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cols) >= 6 and cols[4].isdigit():
            row = {"traffic": int(cols[4])}
            if len(cols) >= 7:
                try:
                    row["issue"] = float(cols[6]) / 100.0
                except ValueError:
                    pass
            out[cols[0]] = row
    return out


def measured_traffic(args):
    """DRAM bytes per launch of each kernel timer, from the committed ncu summary of this workload."""
    return {k: v["traffic"] for k, v in measured_table(args).items()}


def file_io_pass(r, xyz, nrm, steps):
    """The same reconstruction from a binary PLY file to a PLY file through the C ABI
    (prgpu_read_points, prgpu_reconstruct, prgpu_write_mesh_ply): host wall time per step,
    file I/O included; the mesh is written binary (timed) and ascii (timed apart)."""
    import shutil
    import tempfile
    import poissonrecon_gpu_gb300 as pg
    L = pg._lib()
    d = tempfile.mkdtemp(prefix="prgpu_bench_")
    try:
        src = os.path.join(d, "points.ply")
        with open(src, "wb") as fh:
            fh.write(b"ply\nformat binary_little_endian 1.0\nelement vertex %d\n" % len(xyz))
            for k in ("x", "y", "z", "nx", "ny", "nz"):
                fh.write(b"property float %s\n" % k.encode())
            fh.write(b"end_header\n")
            fh.write(np.concatenate([xyz, nrm], 1).astype("<f4").tobytes())
        out_b, out_a = os.path.join(d, "mesh_bin.ply"), os.path.join(d, "mesh_ascii.ply")
        rd, rc_, wb, wa = [], [], [], []
        for _ in range(steps):
            t0 = time.perf_counter()
            n = ctypes.c_int64(0)
            px, pn = ctypes.c_void_p(), ctypes.c_void_p()
            if L.prgpu_read_points(src.encode(), ctypes.byref(n), ctypes.byref(px), ctypes.byref(pn)):
                raise pg.PrgpuError(1, "prgpu_read_points")
            t1 = time.perf_counter()
            m = pg.Mesh()
            rc = L.prgpu_reconstruct(r._h, px, pn, n.value, ctypes.byref(m))
            if rc not in (0, 5):
                raise pg.PrgpuError(rc, "prgpu_reconstruct")
            t2 = time.perf_counter()
            if L.prgpu_write_mesh_ply(out_b.encode(), ctypes.byref(m), 1):
                raise pg.PrgpuError(1, "prgpu_write_mesh_ply")
            t3 = time.perf_counter()
            if L.prgpu_write_mesh_ply(out_a.encode(), ctypes.byref(m), 0):
                raise pg.PrgpuError(1, "prgpu_write_mesh_ply")
            t4 = time.perf_counter()
            rd.append(t1 - t0); rc_.append(t2 - t1); wb.append(t3 - t2); wa.append(t4 - t3)
        med = lambda v: float(np.median(v)) * 1e3
        total = med(np.array(rd) + np.array(rc_) + np.array(wb))
        return {"value": len(xyz) / (total * 1e-3), "unit": "points/s", "ms_per_step": total,
                "read_ms": med(rd), "reconstruct_ms": med(rc_), "write_binary_ms": med(wb),
                "write_ascii_ms": med(wa), "host_threads": os.cpu_count(),
                "path": "binary PLY in, binary PLY out (ascii output timed apart), host wall time"}
    finally:
        shutil.rmtree(d, ignore_errors=True)


CHECKPOINT = os.path.join(REPO, "poissonrecon_gpu_gb300", "weights", "lpc_ellipsoids_d9.bin")
REF_CUDA = os.path.join(REPO, "oracle", "_ref", "ref_cuda")


def solver_study(seeds, device):
    """Learned-preconditioned flexible CG against plain CG on held-out shapes of the
    solver-study configuration: unions of 3-8 ellipsoids (20k-200k points), maxDepth 9,
    every depth solved to relative residual 1e-6 checked on the FP64 true residual
    (params.refine).  Solve time: the library's CUDA-event timer around the solve stage,
    median of 3 solves per shape."""
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    if not os.path.exists(CHECKPOINT):
        return {"unavailable": "no checkpoint at %s" % os.path.relpath(CHECKPOINT, REPO)}
    kw = dict(depth=9, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6, refine=True, device=device)
    plain = pg.Reconstructor(**kw)
    lrn = pg.Reconstructor(preconditioner=CHECKPOINT, **kw)
    rows = []
    for k in range(seeds):
        xyz, nrm = shapes.ellipsoid_union(100000 + k)
        row = {"points": len(xyz)}
        for name, r in (("plain", plain), ("learned", lrn)):
            r.set_points(xyz, nrm)
            r.build_octree()
            r.compute_rhs()
            ts = []
            for _ in range(3):
                r.solve()
                ts.append(r.stats()["ms"]["solve"])
            st = r.stats()
            row[name] = {"ms": float(np.median(ts)), "iters": st["cg_iters"], "fallback": st["cg_fallback"],
                         "fp64": max(st["cg_fp64_residual"])}
        rows.append(row)
    plain.close()
    lrn.close()
    pm = np.array([r["plain"]["ms"] for r in rows])
    lm = np.array([r["learned"]["ms"] for r in rows])
    it_p = np.array([sum(r["plain"]["iters"]) for r in rows])
    it_l = np.array([sum(r["learned"]["iters"]) for r in rows])
    return {"workload": "unions of 3-8 ellipsoids, held-out seeds 100000-%d, 20k-200k points, maxDepth 9, relative "
                        "residual 1e-6 (FP64 true residual)" % (100000 + seeds - 1),
            "shapes": seeds, "points_mean": float(np.mean([r["points"] for r in rows])),
            "plain_solve_ms_mean": float(pm.mean()), "learned_solve_ms_mean": float(lm.mean()),
            "ratio_learned_over_plain": float(lm.mean() / pm.mean()),
            "iterations_sum_over_depths_mean": {"plain": float(it_p.mean()), "learned": float(it_l.mean())},
            "depths_falling_back": int(sum(sum(1 for v in r["learned"]["fallback"] if v >= 0) for r in rows)),
            "max_fp64_residual": {"plain": float(max(r["plain"]["fp64"] for r in rows)),
                                  "learned": float(max(r["learned"]["fp64"] for r in rows))},
            "checkpoint": os.path.relpath(CHECKPOINT, REPO)}


def reference_cuda_anchor(device, runs=3):
    """The reference's own CUDA program (built unchanged by oracle/ref_cuda.sh; maxDepth 8
    fixed by its main.cu:69) on the 50,000-point sphere, timed by its own clock ("The whole
    project takes", PLY in to ASCII PLY out), beside this library file to file on the same
    file (binary PLY read, reconstruction with the reference's CG schedule, ASCII PLY write)."""
    import re
    import shutil
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    if not os.path.exists(REF_CUDA):
        return {"unavailable": "the reference's CUDA program is not built here (oracle/ref_cuda.sh)"}
    work = tempfile.mkdtemp(prefix="prgpu_refcuda_")
    try:
        xyz, nrm = shapes.sphere(50000, seed=0)
        src = os.path.join(work, "bunny.points.ply")   # the file name the reference's main() opens
        with open(src, "wb") as fh:
            fh.write(b"ply\nformat binary_little_endian 1.0\nelement vertex %d\n" % len(xyz))
            for k in ("x", "y", "z", "nx", "ny", "nz"):
                fh.write(b"property float %s\n" % k.encode())
            fh.write(b"end_header\n")
            fh.write(np.concatenate([xyz, nrm], 1).astype("<f4").tobytes())
        ref_s, ref_stage = [], {}
        for _ in range(runs):
            p = subprocess.run([REF_CUDA, "pipeline"], env=dict(os.environ, PRGPU_REF_IO_DIR=work),
                               capture_output=True, text=True, timeout=300)
            m = re.search(r"The whole project takes ([0-9.]+)s", p.stdout)
            if not m:
                return {"unavailable": "the reference's program did not finish: %s" % p.stderr[-200:]}
            ref_s.append(float(m.group(1)))
            for ln in p.stdout.splitlines():
                mm = re.match(r"(.*?) takes:? ?([0-9.]+)(ms|s)", ln.strip())
                if mm:
                    ref_stage[mm.group(1)] = float(mm.group(2)) * (1e-3 if mm.group(3) == "ms" else 1.0)
        r = pg.Reconstructor(depth=8, device=device)
        out_ply = os.path.join(work, "ours.ply")
        ours = []
        for _ in range(max(runs, 3)):
            t0 = time.perf_counter()
            px, pn = pg.read_points(src)
            v, f = r.reconstruct(px, pn)
            pg.write_mesh(out_ply, v, f, binary=False)
            ours.append(time.perf_counter() - t0)
        r.close()
        t_ref, t_ours = float(np.median(ref_s)), float(np.median(ours))
        return {"workload": "sphere 50000 points, maxDepth 8, reference CG schedule, PLY in to ASCII PLY out",
                "reference_s": t_ref, "reference_runs_s": ref_s, "reference_stages_s": ref_stage,
                "ours_s": t_ours, "ours_points_per_s": len(xyz) / t_ours, "reference_points_per_s": len(xyz) / t_ref,
                "speedup": t_ref / t_ours,
                "note": "the reference's own clock, which starts after CUDA initialisation; its process then "
                        "crashes in host-side teardown after printing it"}
    finally:
        shutil.rmtree(work, ignore_errors=True)


class Steps:
    """One reconstruction as a step: device-resident (input already in HBM) or through
    prgpu_reconstruct with pinned host buffers; timed with CUDA events on the library's stream,
    L2 flushed before each step."""

    def __init__(self, r, xyz, nrm, dev, flush):
        import torch
        self.r, self.n, self.dev, self.flush = r, len(xyz), dev, flush
        self.h_xyz = torch.from_numpy(xyz).pin_memory()
        self.h_nrm = torch.from_numpy(nrm).pin_memory()
        self.d_xyz = self.h_xyz.to(dev)
        self.d_nrm = self.h_nrm.to(dev)
        self.stream = torch.cuda.ExternalStream(r.stream(), device=dev)

    def device_step(self):
        r = self.r
        r.set_points_device(self.d_xyz.data_ptr(), self.d_nrm.data_ptr(), self.n)
        r.build_octree()
        r.compute_rhs()
        r.solve()
        r.eval_points()
        r.extract_mesh()

    def host_step(self):
        import poissonrecon_gpu_gb300 as pg
        m = pg.Mesh()
        rc = pg._lib().prgpu_reconstruct(self.r._h, self.h_xyz.data_ptr(), self.h_nrm.data_ptr(), self.n,
                                         ctypes.byref(m))
        if rc not in (0, 5):
            raise pg.PrgpuError(rc, "prgpu_reconstruct")
        return m.n_vertices, m.n_triangles

    def timed(self, step, k):
        import torch
        ms, out = [], None
        for _ in range(k):
            self.flush.fill_(1.0)
            torch.cuda.synchronize(self.dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            out = step()
            e1.record(self.stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms, out


def kernel_roofline(stats, peaks, ms_per_step):
    """Every kernel timer's algorithmic bytes per launch over its CUDA-event time, as a fraction of
    the measured HBM copy bandwidth, and the whole step's algorithmic bytes over its time."""
    peak = peaks.get("hbm_gbs", 6800.0)
    out, total = {}, 0.0
    for name, k in (stats.get("kernels") or {}).items():
        if k["bytes"] <= 0 or k["ms"] <= 0:
            continue
        gbs = k["bytes"] / (k["ms"] * 1e-3) / 1e9
        out[name] = {"ms_per_launch": round(k["ms"] / max(k["launches"], 1), 4),
                     "gb_per_launch": round(k["bytes"] / max(k["launches"], 1) / 1e9, 4),
                     "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}
        total += k["bytes"] / max(k["launches"], 1)
    step_gbs = total / (ms_per_step * 1e-3) / 1e9
    return {"kernels": out, "step_algorithmic_gb": round(total / 1e9, 3), "step_achieved_gbs": round(step_gbs, 1),
            "step_frac": round(step_gbs / peak, 4), "peak": peak}


def large_config(device, peaks, steps=2, warmup=1):
    """The 30M-point displaced sphere (4-octave value-noise displacement, amplitude 0.05) at maxDepth
    12, every depth to relative residual 1e-6: device-resident and end-to-end throughput, stage
    times, per-kernel rooflines, and the solve with plain CG against the learned preconditioner
    (the shipped checkpoint, trained at maxDepth 9; plain CG takes over any depth where the
    network's steps do not reduce the residual)."""
    import torch
    import poissonrecon_gpu_gb300 as pg
    from poissonrecon_gpu_gb300 import shapes
    dev = torch.device("cuda", device)
    t0 = time.perf_counter()
    xyz, nrm = shapes.displaced_sphere(30_000_000, seed=0, device=dev)
    t_gen = time.perf_counter() - t0
    n = len(xyz)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    kw = dict(depth=12, solve_mode=pg.SOLVE_RELATIVE, cg_tol=1e-6, cg_max_iter=10000, device=device)
    r = pg.Reconstructor(**kw)
    run = Steps(r, xyz, nrm, dev, flush)
    for _ in range(warmup):
        run.device_step()
    dev_ms, _ = run.timed(run.device_step, steps)
    e2e_ms, (nv, nt) = run.timed(run.host_step, 1)
    r.set_profiling(True)
    prof_ms, _ = run.timed(run.device_step, 1)
    st = r.stats()
    r.set_profiling(False)
    solve = {}
    for name in ("plain", "learned"):
        if name == "learned":
            if not os.path.exists(CHECKPOINT):
                break
            r.close()
            r = pg.Reconstructor(preconditioner=CHECKPOINT, **kw)
            r.set_points_device(run.d_xyz.data_ptr(), run.d_nrm.data_ptr(), n)
            r.build_octree()
            r.compute_rhs()
        ts = []
        for _ in range(3):
            r.solve()
            ts.append(r.stats()["ms"]["solve"])
        s2 = r.stats()
        solve[name] = {"ms": float(np.median(ts)), "iters": s2["cg_iters"], "fallback": s2.get("cg_fallback"),
                       "rel_residual_max": float(max(s2["cg_rel_residual"]))}
    r.close()
    t_dev = float(np.mean(dev_ms))
    return {"workload": "displaced sphere 30000000 points, maxDepth 12, CG to relative residual 1e-06",
            "value": n / (t_dev * 1e-3), "unit": "points/s", "ms_per_step": t_dev, "steps": steps,
            "e2e": {"value": n / (e2e_ms[0] * 1e-3), "ms_per_step": e2e_ms[0], "h2d_bytes_per_step": 24 * n,
                    "d2h_bytes_per_step": int(12 * nv + 12 * nt)},
            "nodes": st.get("nodes"), "mesh": {"vertices": nv, "triangles": nt}, "stages_ms": st.get("ms"),
            "profiled_ms_per_step": prof_ms[0], "roofline": kernel_roofline(st, peaks, prof_ms[0]),
            "solve": solve, "generate_s": round(t_gen, 2),
            "data": "synthetic, generated on the GPU with torch (shapes.displaced_sphere, device=)"}


def max_over_ranks(values, device):
    """Replicas: every rank times its own reconstruction; the job's time is the slowest rank's."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


# library timers that span several kernels, each of which also has its own timer
AGGREGATE_TIMERS = {"divergence"}   # divergence_d, divergence_d1, divergence_groups, divergence_root


def roofline(stats, peaks, traffic, issue=None):
    """The dominant kernel's roofline (an aggregate timer is not a kernel; its kernels are).
    issue: per timer, the fraction of issue slots ncu saw busy (an issue-bound kernel shows a
    low HBM fraction and a high issue fraction)."""
    ks = {n: k for n, k in stats.get("kernels", {}).items() if n not in AGGREGATE_TIMERS}
    if not ks:
        return None
    name, k = max(ks.items(), key=lambda kv: kv[1]["ms"])
    per_launch_ms = k["ms"] / max(k["launches"], 1)
    bytes_per_launch = k["bytes"] / max(k["launches"], 1)
    achieved = bytes_per_launch / (per_launch_ms * 1e-3) / 1e9 if per_launch_ms > 0 else 0.0
    peak = peaks.get("hbm_gbs", 6800.0)
    return {"kernel": name, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic.get(name),
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks else "fallback",
            "launch_ms": round(per_launch_ms, 4), "algorithmic_bytes_per_launch": bytes_per_launch,
            "sm_issue_active": (issue or {}).get(name)}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        cpu, per = cpu_reference(args, args.steps, args.warmup)
        # ms_per_step is the measured time of one sampled step (what the run's wall clock
        # holds); value is the whole path's throughput estimated from that sample
        out = {"metric": "points/s end-to-end", "value": cpu["value"], "unit": "points/s", "n_gpus": args.gpus,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": cpu["measured_s_per_step"] * 1e3,
               "estimated_full_ms_per_step": per * 1e3, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": config(args, "n/a (host)"), "impl": "reference", "cpu_baseline": cpu,
               "e2e": {"value": cpu["value"], "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return

    if args.solver_only:
        if rank == 0:
            print(json.dumps({"solver_study": solver_study(max(args.solver_seeds, 1), local)}))
        return

    import torch
    import poissonrecon_gpu_gb300 as pg
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}

    xyz, nrm = workload(args)
    n = len(xyz)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)   # 256 MiB > L2
    r = pg.Reconstructor(depth=args.depth, solve_mode=pg.SOLVE_RELATIVE, cg_tol=args.tol, cg_max_iter=10000,
                         device=local)
    run = Steps(r, xyz, nrm, dev, flush)
    device_step, host_step, timed = run.device_step, run.host_step, run.timed

    for _ in range(args.warmup):
        device_step()
        host_step()
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()

    clock_csv = args.clocks_csv or os.path.join(tempfile.mkdtemp(prefix="prgpu_clocks_"), "clocks.csv")
    with Clocks(clock_csv) as clk:
        launches0 = pg.kernel_launches()
        dev_ms, _ = timed(device_step, args.steps)
        launches = pg.kernel_launches() - launches0
        e2e_ms, (nv, nt) = timed(host_step, args.steps)
    # per-kernel timers (CUDA events around each kernel) in a separate pass of the same
    # steps, so that the timed steps above carry no profiling events
    r.set_profiling(True)
    prof_ms, _ = timed(device_step, args.steps)
    stats = r.stats()
    r.set_profiling(False)
    torch.cuda.synchronize(dev)
    t_dev = float(np.mean(dev_ms))
    t_e2e = float(np.mean(e2e_ms))
    if world > 1:
        t_dev, t_e2e = max_over_ranks([t_dev, t_e2e], dev)
    if rank != 0:
        return
    out = {
        "metric": "points/s end-to-end", "value": n * world / (t_dev * 1e-3), "unit": "points/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_dev,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config(args, "flushed between steps (256 MiB write)"),
        "e2e": {"value": n * world / (t_e2e * 1e-3), "unit": "points/s", "ms_per_step": t_e2e,
                "h2d_bytes_per_step": int(24 * n), "d2h_bytes_per_step": int(12 * nv + 12 * nt)},
        "gpu_launches": int(launches),
        "roofline": roofline(stats, peaks, measured_traffic(args),
                             {k: v["issue"] for k, v in measured_table(args).items() if "issue" in v}),
        "kernel_roofline": kernel_roofline(stats, peaks, float(np.mean(prof_ms))),
        "profiled_ms_per_step": float(np.mean(prof_ms)),
        "clocks": clk.summary(),
        "stages_ms": stats.get("ms"),
        "cg_iters": stats.get("cg_iters"),
        "kernels": stats.get("kernels"),
        "subdivision": {k: stats.get(k) for k in ("roots_per_depth", "virtual_cells", "bricks", "live_bricks",
                                                  "foreign_corners", "foreign_evaluated", "super_bricks",
                                                  "super_decided")},
        "nodes": stats.get("nodes"),
        "mesh": {"vertices": nv, "triangles": nt},
    }
    if world == 1:
        out["file_e2e"] = file_io_pass(r, xyz, nrm, max(args.steps, 3))
        if args.solver_seeds > 0:
            out["solver_study"] = solver_study(args.solver_seeds, local)
        out["reference_cuda_build"] = reference_cuda_anchor(local)
        if args.large:
            r.close()
            r = None
            torch.cuda.empty_cache()
            out["large_config"] = large_config(local, peaks)
    if os.environ.get("PRGPU_BENCH_NO_CPU") != "1":
        cpu, _ = cpu_reference(args, 1, 0)
        out["cpu_baseline"] = cpu
    print(json.dumps(out))
    if r is not None:
        r.close()


if __name__ == "__main__":
    main()
