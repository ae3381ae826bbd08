"""Trains the learned preconditioner on the GPU and saves its weights.

    python -m autopdex_gb300.train_preconditioner --n 256 --problems 2000 --steps 6000 \
        --out autopdex_gb300/weights/heat_unet_n256.npz
    python -m autopdex_gb300.train_preconditioner --problem membrane --n 128 --steps 3000 \
        --out autopdex_gb300/weights/membrane_unet_n128.npz
    python -m autopdex_gb300.train_preconditioner --problem brick --n 128 --problems 2 \
        --rhs-per-state 4 --factor 4 --steps 1500 --batch 4

heat: training pairs (residual, error) come from the iterates of the plain float64 Jacobi-PCG
solver on heat-conduction problems -div(k grad T) = b with k = exp(Gaussian random field) seeded
0 .. problems-1 (length 0.05, std 1, the 1024 x 1024 heat workload's family at n x n), one
constant and one random right-hand side each.
membrane: the nearly incompressible Cook membrane (the 512 x 512 membrane workload's geometry
at n x n), tangents at converged load states, random vector right-hand sides after the
Chebyshev pre-smoothing of the native FCG, error energies from the banded Cholesky factor.
brick: the 3-D network (UNet3D) on the 128^3 backward-Euler heat workload's family: tangents
of the first Newton step from seeded random temperature fields, right-hand sides the Newton
residual and random fields, pairs from the plain float64 Jacobi-PCG iterates; the network
works on the grid coarsened by --factor.
"""
import argparse
import json
import os
import time

import torch

from . import learned


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--problems", type=int, default=2000)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--problem", default="heat", choices=["heat", "membrane", "brick"])
    ap.add_argument("--rhs-per-state", type=int, default=400)
    ap.add_argument("--factor", type=int, default=1, help="membrane: train the network on the grid coarsened by this")
    ap.add_argument("--degree", type=int, default=3, help="membrane: Chebyshev pre-smoothing degree")
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    if args.out is None:
        args.out = os.path.join(learned.WEIGHTS_DIR, f"{args.problem}_unet_n{args.n}.npz")
    t0 = time.time()
    if args.problem == "heat":
        ts = learned.make_training_set(args.problems, n=args.n, seed0=args.seed, verbose=True)
        net = learned.UNet(seed=args.seed)
    elif args.problem == "brick":
        ts = learned.make_brick_training_set(n=args.n, states=args.problems, rhs_per_state=args.rhs_per_state,
                                             seed0=args.seed, factor=args.factor, verbose=True)
        net = learned.UNet3D(seed=args.seed)
    else:
        ts = learned.make_membrane_training_set(n=args.n, rhs_per_state=args.rhs_per_state, seed=args.seed,
                                                factor=args.factor, degree=args.degree, verbose=True)
        net = learned.UNet(seed=args.seed, n_in=ts.nd + ts.naux)
    t1 = time.time()
    fit = learned.train3d if args.problem == "brick" else learned.train
    losses = fit(net, ts, steps=args.steps, batch=args.batch, lr=args.lr, verbose=True)
    torch.cuda.synchronize()
    t2 = time.time()
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    net.save(args.out)
    meta = {"train_n": args.n, "problems": args.problems, "steps": args.steps, "batch": args.batch,
            "samples": len(ts), "data_seconds": round(t1 - t0, 1), "train_seconds": round(t2 - t1, 1),
            "loss_first50": round(sum(losses[:50]) / 50, 4), "loss_last50": round(sum(losses[-50:]) / 50, 4),
            "loss_per_100_steps": [round(sum(losses[i:i + 100]) / len(losses[i:i + 100]), 4)
                                   for i in range(0, len(losses), 100)],
            "problem": args.problem,
            "command": f"python -m autopdex_gb300.train_preconditioner --problem {args.problem} --n {args.n} "
                       f"--problems {args.problems} --rhs-per-state {args.rhs_per_state} --factor {args.factor} "
                       f"--degree {args.degree} --steps {args.steps}"}
    with open(os.path.splitext(args.out)[0] + ".json", "w") as fh:
        json.dump(meta, fh, indent=1)
    print(f"data {t1 - t0:.1f} s ({len(ts)} pairs), training {t2 - t1:.1f} s, "
          f"loss {sum(losses[:50]) / 50:.4f} -> {sum(losses[-50:]) / 50:.4f}; saved {args.out}")


if __name__ == "__main__":
    main()
