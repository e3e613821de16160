"""Train the learned warm start on the GPU and write its parameter file.

    python -m chm_gb300.train_warmstart [--out chm_gb300/data/warmstart_mlp.npz]

Training data: plain FP64 solutions of the suspension system from the
1M-face generator (524,288 points in a 70 km square, 10 layers), on seeds
held out from the benchmark's (which uses seed 1 and up): by default 20
seeds x 100 hourly steps = 2,000 solutions, each step's forcing evolving as
in the benchmark and its snow state advanced by the step's drift_mass.
Rows are sampled from every solution.  Training: Adam on the library's
tensor-core forward/backward kernels.  The meshes are generated in a
spawn-started process pool before CUDA is touched.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import multiprocessing as mp
import os
import time

import numpy as np

from . import synth, warmstart


def _workload(spec):
    n_points, side, seed, wind = spec
    return synth.Workload(n_points, side, seed=seed, wind_scale=wind)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(warmstart.WEIGHTS_FILE))
    ap.add_argument("--seeds", default=",".join(str(s) for s in range(1001, 1021)))
    ap.add_argument("--config", default="tri1m")
    ap.add_argument("--steps-per-seed", type=int, default=100)
    ap.add_argument("--rows-per-step", type=int, default=20000)
    ap.add_argument("--train-steps", type=int, default=12000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--wind", type=float, default=8.0)
    args = ap.parse_args()
    cfg = synth.CONFIGS[args.config]
    t0 = time.time()
    seeds = [int(s) for s in args.seeds.split(",")]
    specs = [(cfg["n_points"], cfg["side"], s, args.wind) for s in seeds]
    with cf.ProcessPoolExecutor(max_workers=min(len(specs), os.cpu_count() or 1),
                                mp_context=mp.get_context("spawn")) as ex:
        workloads = list(ex.map(_workload, specs))
    t_mesh = time.time() - t0
    params, mean, scale, losses, n = warmstart.train_from_solutions(
        seeds, cfg["n_points"], cfg["side"], cfg["nLayer"], args.steps_per_seed, args.rows_per_step,
        args.train_steps, lr=args.lr, batch=args.batch, seed=0, wind=args.wind, workloads=workloads)
    warmstart.save(args.out, params, mean, scale, losses=losses, rows=n, seeds=np.array(seeds),
                   config=args.config, nLayer=cfg["nLayer"], steps_per_seed=args.steps_per_seed,
                   solutions=len(seeds) * args.steps_per_seed)
    print(f"trained on {n} rows from {len(seeds)} seeds x {args.steps_per_seed} steps "
          f"({len(seeds) * args.steps_per_seed} solutions) in {time.time() - t0:.1f} s "
          f"(meshes {t_mesh:.1f} s); loss {losses[:50].mean():.4f} -> {losses[-100:].mean():.4f}; wrote {args.out}")


if __name__ == "__main__":
    main()
