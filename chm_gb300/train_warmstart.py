"""Train the learned warm start on the GPU and write its parameter file.

    python -m chm_gb300.train_warmstart [--out chm_gb300/data/warmstart_mlp.npz]

Training data: plain FP64 solutions of the suspension system on seeded
synthetic meshes of the benchmark's point density (held-out seeds: the
benchmark uses seed 1 and up), rows sampled from every step.  Training:
Adam on the library's tensor-core forward/backward kernels.
"""
from __future__ import annotations

import argparse
import time

import numpy as np

from . import synth, warmstart


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(warmstart.WEIGHTS_FILE))
    ap.add_argument("--seeds", default="1001,1002,1003")
    ap.add_argument("--config", default="tri262k")
    ap.add_argument("--steps-per-seed", type=int, default=8)
    ap.add_argument("--rows-per-step", type=int, default=250000)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    args = ap.parse_args()
    cfg = synth.CONFIGS[args.config]
    t0 = time.time()
    seeds = [int(s) for s in args.seeds.split(",")]
    params, mean, scale, losses, n = warmstart.train_from_solutions(
        seeds, cfg["n_points"], cfg["side"], cfg["nLayer"], args.steps_per_seed, args.rows_per_step,
        args.train_steps, lr=args.lr, batch=args.batch, seed=0)
    warmstart.save(args.out, params, mean, scale, losses=losses, rows=n, seeds=np.array(seeds),
                   config=args.config, nLayer=cfg["nLayer"])
    print(f"trained on {n} rows from {len(seeds)} seeds x {args.steps_per_seed} steps in {time.time() - t0:.1f} s; "
          f"loss {losses[:50].mean():.4f} -> {losses[-100:].mean():.4f}; wrote {args.out}")


if __name__ == "__main__":
    main()
