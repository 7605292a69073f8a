"""Trains the learned preconditioner on the GPU and writes its checkpoint.

Data: seeded unions of 3-8 ellipsoids (shapes.ellipsoid_union: centres uniform in
[0.2, 0.8]^3, semi-axes 0.05-0.25, random rotations, 20k-200k points, exact
normals), each reconstructed up to its right-hand side at maxDepth 9; plain CG
on every depth then supplies residual/error pairs (prgpu_trainer_record: the
solution to relative 1e-7, the iterates after 1, 2, 3, 5, 8, 12 and 20
iterations, a fixed number of random rows per depth and iterate).  Training:
Adam on minibatches of the mean squared error, forward and backward on the
tensor cores (prgpu_trainer_train).  The checkpoint holds the parameters, the
Adam moments, the step count and the seed; --resume continues from one.

  python -m poissonrecon_gpu_gb300.train_preconditioner --out lpc.bin
      [--shapes 2000] [--first-seed 0] [--depth 9] [--rows 64] [--steps 20000]
      [--batch 16384] [--lr 1e-3] [--resume lpc.bin] [--device 0]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import SOLVE_RELATIVE, Reconstructor, Trainer, shapes


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", required=True)
    ap.add_argument("--shapes", type=int, default=2000)
    ap.add_argument("--first-seed", type=int, default=0)
    ap.add_argument("--depth", type=int, default=9)
    ap.add_argument("--rows", type=int, default=64, help="rows per depth and recorded iterate")
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--resume", default=None)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)

    T = Trainer(device=a.device, seed=a.seed)
    if a.resume:
        T.load(a.resume)
    r = Reconstructor(depth=a.depth, solve_mode=SOLVE_RELATIVE, cg_tol=1e-6, device=a.device)
    t0 = time.perf_counter()
    points = 0
    for k in range(a.shapes):
        xyz, nrm = shapes.ellipsoid_union(a.first_seed + k)
        points += len(xyz)
        r.set_points(xyz, nrm)
        r.build_octree()
        r.compute_rhs()
        T.record(r, rows_per_depth=a.rows)
    t_rec = time.perf_counter() - t0
    r.close()
    log = []
    t1 = time.perf_counter()
    done = 0
    while done < a.steps:
        n = min(1000, a.steps - done)
        loss = T.train(n, batch=a.batch, lr=a.lr)
        done += n
        log.append((T.info()["step"], loss))
    t_train = time.perf_counter() - t1
    T.save(a.out)
    info = T.info()
    print(json.dumps({"checkpoint": a.out, "shapes": a.shapes, "points": points, "samples": info["samples"],
                      "step": info["step"], "record_s": round(t_rec, 2), "train_s": round(t_train, 2),
                      "loss": [(s, round(l, 5)) for s, l in log[:: max(1, len(log) // 10)]] + [log[-1]]}))
    T.close()


if __name__ == "__main__":
    main()
