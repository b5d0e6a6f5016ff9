"""Training of the learned starting radius (needs a GPU).

The model (csrc/radius_model.cuh) predicts, per query, a high quantile of
log(r_K / eps0): r_K is the distance to the query's (k+1)-th nearest point
(itself included) and eps0 the BETA starting radius of the join.  Training
data are exact joins of seeded synthetic datasets (2-6-D, mixed uniform and
Gaussian-mixture skews) run with this library's plain path; the features
come from knnsj_radius_features and the network is trained by the library's
own CUDA forward / backward / Adam kernels (knnsj_radius_train).

usage:
  python -m hybrid_k_nearest_neighbor_self_join_gb300.train_radius \
      [--sets 32] [--points 1000000] [--per 40000] [--epochs 8] [--out DIR]

Writes DIR/radius_model.npz (model, loss curve, held-out figures) and
DIR/radius_model_weights.inc, the C array the library is built with
(copy it to csrc/ to make it the built-in model).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import time

import numpy as np

from . import _lib, datasets

KS = (8, 16, 32, 64, 128)
BETAS = (0.0, 0.025, 0.05)


def training_sets(n_sets: int, n: int, seed: int):
    """Seeded sets: d in 2..6, uniform-heavy to clustered, sizes log-uniform
    in [n/5, 2n]."""
    rng = np.random.default_rng(seed)
    for i in range(n_sets):
        d = int(rng.integers(2, 7))
        comps = int(rng.integers(1, 60))
        ufrac = float(rng.choice([0.05, 0.2, 0.5, 1.0]))
        sd_hi = float(rng.choice([0.02, 0.05, 0.1]))
        m = int(np.exp(rng.uniform(np.log(n / 5), np.log(2 * n))))
        x = datasets.gmm(m, d, comps, ufrac, seed * 1000 + i, sd_lo=0.002, sd_hi=sd_hi, dtype=np.float32)
        yield i, x, float(rng.choice(BETAS))


def radius_features(x: np.ndarray, k: int, beta: float):
    lib = _lib.load()
    n, d = x.shape
    out = np.empty((n, _lib.RADIUS_FEATURES), np.float32)
    eps0 = ctypes.c_double(0.0)
    opts = _lib.Options.make(beta=beta)
    _lib.check(lib.knnsj_radius_features(x.ctypes.data, _lib.KNNSJ_F32, n, d, k, ctypes.byref(opts),
                                         out.ctypes.data, ctypes.byref(eps0)), "features")
    return out, eps0.value


def targets(dists_k: np.ndarray, eps0: float) -> np.ndarray:
    r = np.maximum(dists_k.astype(np.float64), eps0 / 256.0)
    return np.log(r / eps0).astype(np.float32)


def collect(x: np.ndarray, beta: float, per: int, rng) -> tuple[np.ndarray, np.ndarray]:
    from . import selfjoin
    n = x.shape[0]
    _, dists = selfjoin(x, max(KS), beta=beta)
    Xs, Ys = [], []
    for k in KS:
        feats, eps0 = radius_features(x, k, beta)
        rows = rng.choice(n, min(per, n), replace=False)
        Xs.append(feats[rows])
        Ys.append(targets(dists[rows, k], eps0))
    return np.concatenate(Xs), np.concatenate(Ys)


def train(X: np.ndarray, Y: np.ndarray, epochs: int = 8, batch: int = 8192, lr: float = 1e-3,
          quantile: float = 0.9, seed: int = 1):
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    model = np.empty(_lib.RADIUS_MODEL_FLOATS, np.float32)
    loss = np.zeros(epochs, np.float32)
    o = _lib.TrainOptions()
    o.struct_size = ctypes.sizeof(o)
    o.epochs, o.batch, o.lr, o.quantile, o.seed = epochs, batch, lr, quantile, seed
    _lib.check(_lib.load().knnsj_radius_train(X.ctypes.data, Y.ctypes.data, X.shape[0], ctypes.byref(o),
                                              model.ctypes.data, loss.ctypes.data), "train")
    return model, loss


def predict(model: np.ndarray, X: np.ndarray) -> np.ndarray:
    X = np.ascontiguousarray(X, np.float32)
    out = np.empty(X.shape[0], np.float32)
    _lib.check(_lib.load().knnsj_radius_predict(np.ascontiguousarray(model, np.float32).ctypes.data,
                                                X.ctypes.data, X.shape[0], out.ctypes.data), "predict")
    return out


def write_weights_inc(model: np.ndarray, path: str, note: str) -> None:
    vals = ", ".join(f"{float(v):.9e}f" for v in np.asarray(model, np.float32))
    lines = ["// Radius model weights, generated by train_radius.py -- do not edit.",
             f"// {note}",
             f"static const float kRadiusModelDefault[{_lib.RADIUS_MODEL_FLOATS}] = {{"]
    line = ""
    for tok in vals.split(", "):
        if len(line) + len(tok) > 108:
            lines.append(line.rstrip())
            line = ""
        line += tok + ", "
    lines.append(line.rstrip().rstrip(","))
    lines.append("};")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def placeholder_model() -> np.ndarray:
    """log(r/eps0) = 0 for every query: the first pass starts at eps0."""
    m = np.zeros(_lib.RADIUS_MODEL_FLOATS, np.float32)
    m[24:48] = 1.0
    return m


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--sets", type=int, default=32)
    ap.add_argument("--points", type=int, default=1_000_000)
    ap.add_argument("--per", type=int, default=40_000)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--quantile", type=float, default=0.9)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--holdout", type=int, default=4)
    ap.add_argument("--out", default="radius_model_out")
    a = ap.parse_args(argv)
    os.makedirs(a.out, exist_ok=True)
    rng = np.random.default_rng(a.seed)
    t0 = time.time()
    Xtr, Ytr, Xte, Yte = [], [], [], []
    for i, x, beta in training_sets(a.sets + a.holdout, a.points, a.seed):
        X, Y = collect(x, beta, a.per, rng)
        (Xtr if i < a.sets else Xte).append(X)
        (Ytr if i < a.sets else Yte).append(Y)
        print(f"set {i}: d={x.shape[1]} beta={beta} samples={len(Y)} ({time.time() - t0:.1f}s)", flush=True)
    Xtr, Ytr = np.concatenate(Xtr), np.concatenate(Ytr)
    Xte, Yte = np.concatenate(Xte), np.concatenate(Yte)
    t1 = time.time()
    model, loss = train(Xtr, Ytr, epochs=a.epochs, quantile=a.quantile, seed=a.seed)
    t_train = time.time() - t1
    pred = predict(model, Xte)
    cover = float(np.mean(pred >= Yte))
    report = {
        "train_samples": int(len(Ytr)), "holdout_samples": int(len(Yte)), "epochs": a.epochs,
        "quantile": a.quantile, "loss_per_epoch": [float(v) for v in loss], "train_seconds": t_train,
        "holdout_coverage": cover, "holdout_mean_log_ratio": float(np.mean(pred - Yte)),
        "holdout_target_mean": float(np.mean(Yte)),
    }
    print(json.dumps(report), flush=True)
    np.savez(os.path.join(a.out, "radius_model.npz"), model=model, loss=loss, report=json.dumps(report))
    note = (f"{a.sets} sets x {a.points} points, {len(KS)} k values, {a.epochs} epochs, quantile {a.quantile}, "
            f"held-out coverage {cover:.3f}")
    write_weights_inc(model, os.path.join(a.out, "radius_model_weights.inc"), note)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
