"""Trains the shift-predicting MLP on the GPU and writes its weights.

    python -m mpk_gb300.train_shifts --count 2000 --out shift_mlp.npz

Training data: `count` seeded synthetic diffusion matrices
(mpk_gb300.shifts.training_matrix), their features and the normalised
Ritz values of an s-step Lanczos run, all computed by the library's GPU
kernels; the MLP (NFEAT -> 64 -> 64 -> s) is trained by the library's own
forward/backward/Adam kernels.  The file holds the flat parameters, the
dimensions, the loss curve and the held-out error."""
import argparse
import json
import time

import numpy as np

from . import shifts as S


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=2000)
    ap.add_argument("--holdout", type=int, default=200)
    ap.add_argument("--s", type=int, default=8)
    ap.add_argument("--width", type=int, default=64)
    ap.add_argument("--epochs", type=int, default=600)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default="shift_mlp.npz")
    args = ap.parse_args()
    t0 = time.time()
    X, T = S.training_set(args.count + args.holdout, s=args.s, seed=args.seed)
    t1 = time.time()
    Xtr, Ttr, Xte, Tte = X[:args.count], T[:args.count], X[args.count:], T[args.count:]
    mlp, curve = S.train(Xtr, Ttr, width=args.width, epochs=args.epochs, seed=args.seed)
    t2 = time.time()
    pred = mlp.forward(Xte)
    test_mse = float(np.mean((np.sort(np.clip(pred, 0, 1), axis=1) - Tte) ** 2))
    base_mse = float(np.mean((Tte - Ttr.mean(0)) ** 2))  # predicting the mean target
    np.savez(args.out, params=mlp.params(), nin=X.shape[1], width=args.width, nout=args.s,
             curve=curve, test_mse=test_mse, mean_predictor_mse=base_mse, count=args.count, seed=args.seed)
    print(json.dumps({"data_s": t1 - t0, "train_s": t2 - t1, "loss_first": float(curve[0]),
                      "loss_last": float(curve[-1]), "test_mse": test_mse, "mean_predictor_mse": base_mse}))


def load(path):
    """The trained MLP stored by main()."""
    from . import Mlp
    d = np.load(path)
    m = Mlp(int(d["nin"]), int(d["width"]), int(d["nout"]))
    m.set_params(d["params"])
    return m


if __name__ == "__main__":
    main()
