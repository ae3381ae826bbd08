"""Trains the learned preconditioner on the GPU and saves its weights.

    python -m autopdex_gb300.train_preconditioner --n 256 --problems 2000 --steps 3000 \
        --out autopdex_gb300/weights/heat_unet_n256.npz

Training pairs (r, K^-1 r) come from the plain float64 Jacobi-PCG solver on heat-conduction
problems -div(k grad T) = r with k = exp(Gaussian random field) seeded 0 .. problems-1
(length 0.05, std 1, the config-4 family), one constant and one random right-hand side each.
"""
import argparse
import os
import time

import torch

from . import learned


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--problems", type=int, default=2000)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=os.path.join(learned.WEIGHTS_DIR, "heat_unet_n256.npz"))
    args = ap.parse_args()
    t0 = time.time()
    R, A, E = learned.make_training_set(args.problems, n=args.n, seed0=args.seed, verbose=True)
    t1 = time.time()
    net = learned.UNet(seed=args.seed)
    losses = learned.train(net, R, A, E, args.n, steps=args.steps, batch=args.batch, lr=args.lr, verbose=True)
    torch.cuda.synchronize()
    t2 = time.time()
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    net.save(args.out)
    print(f"data {t1 - t0:.1f} s ({R.shape[0]} pairs), training {t2 - t1:.1f} s, "
          f"loss {sum(losses[:50]) / 50:.4f} -> {sum(losses[-50:]) / 50:.4f}; saved {args.out}")


if __name__ == "__main__":
    main()
