"""Train the learned initial guess and evaluate it against the plain solve.

    python -m flowfpmpp_gb300.train_learned --count 2000 --epochs 8 \
        --out flowfpmpp_gb300/data/learned_guess.npy

Training set: `count` random bodies on 128x128x64 grids (1-4 ellipsoids and
boxes, FP64 PCG targets to 1e-8); evaluation: `eval_count` unseen bodies on
256x256x128 grids, FP64 PCG to 1e-10 from phi = 0 and from the learned guess.
Prints one JSON line with the timings, the loss history, the iteration
counts and the fallback count.
"""
from __future__ import annotations

import argparse
import json
import sys
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--train-grid", type=int, nargs=3, default=[128, 128, 64])
    ap.add_argument("--eval-grid", type=int, nargs=3, default=[256, 256, 128])
    ap.add_argument("--eval-count", type=int, default=64)
    ap.add_argument("--eval-method", default="pcg")
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", default=None)
    ap.add_argument("--init", default=None, help="start from these parameters (.npy)")
    a = ap.parse_args(argv)

    import numpy as np
    import torch
    from flowfpmpp_gb300 import learned as lg

    log = lambda m: print(m, file=sys.stderr, flush=True)
    t0 = time.perf_counter()
    data = lg.make_dataset(a.count, *a.train_grid, seed=a.seed, log=log)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    net = lg.LearnedGuess(seed=a.seed) if a.init is None else lg.LearnedGuess(params=np.load(a.init))
    t0 = time.perf_counter()
    hist = lg.train(net, data, epochs=a.epochs, lr=a.lr, log=log) if a.epochs > 0 else []
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    if a.out:
        net.save(a.out)
    del data
    torch.cuda.empty_cache()

    rng = np.random.default_rng(a.seed + 100000)
    rows = []
    for s in range(a.eval_count):
        ax, ay, az = lg.training_grid(*a.eval_grid)
        axis = int(rng.integers(0, 3))
        p = lg.DeviceProblem(lg.frame_for(lg.random_bodies(rng, ax, ay, az), ax, ay, az, axis))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        _, sw0, r0, _ = p.solve(a.eval_method, tol=1e-10)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        _, sw1, r1, fb = p.solve(a.eval_method, tol=1e-10, net=net)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        rows.append(dict(plain_its=sw0, plain_s=t2 - t1, plain_res=r0, learned_its=sw1, learned_s=t3 - t2,
                         learned_res=r1, fallback=fb))
        log(f"eval {s + 1}/{a.eval_count}: plain {sw0} its {t2 - t1:.3f} s, learned {sw1} its {t3 - t2:.3f} s, "
            f"fallback {fb}")
    its0 = sum(r["plain_its"] for r in rows)
    its1 = sum(r["learned_its"] for r in rows)
    t0s = sum(r["plain_s"] for r in rows)
    t1s = sum(r["learned_s"] for r in rows)
    print(json.dumps(dict(train_count=a.count, train_grid=a.train_grid, epochs=a.epochs, dataset_s=t_data,
                          train_s=t_train, loss_history=hist, eval_grid=a.eval_grid, eval_count=a.eval_count,
                          eval_method=a.eval_method, plain_iterations=its0, learned_iterations=its1,
                          plain_seconds=t0s, learned_seconds=t1s,
                          fallbacks=sum(r["fallback"] for r in rows),
                          max_residual=max([r["learned_res"] for r in rows] or [0.0]))))


if __name__ == "__main__":
    main()
