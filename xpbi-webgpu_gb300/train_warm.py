"""Train the warm-start network on multipliers the plain solver produces.

Data: seeded dam-breach scenes (PBF water beside Drucker-Prager sand, the
benchmark's scene mix) at reduced size with varied sand parameters. Each
scene runs the plain solve (every iteration from lambda = 0) for a random
number of substeps, then logs a few substeps: per solid particle the 16
features at iteration 0 and alpha_tilde * lambda after the full iteration
budget. The network learns the increment of that over the previous
substep's multiplier (feature 4): the warm start is the previous multiplier
plus the prediction, so a network that predicts nothing is the
previous-multiplier start and the BF16 rounding only touches the increment.

Training: Adam with the library's own tensor-core forward / backward
kernels (xpbi_mlp_train). Inputs and target are standardised for training;
the affine maps are folded into the first and last layers afterwards, so
the stored network takes raw features and returns alpha_tilde times the
multiplier increment.

    python -m xpbi-webgpu_gb300.train_warm --out weights.bin
"""
from __future__ import annotations

import argparse
import importlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "weights", "warm_start_dam.bin")


def _pkg():
    root = os.path.dirname(HERE)
    if root not in sys.path:
        sys.path.insert(0, root)
    return importlib.import_module("xpbi-webgpu_gb300")


def load_weights(path: str = WEIGHTS) -> np.ndarray:
    return np.fromfile(path, dtype=np.float32)


def training_scene(xp, seed: int, scale: float):
    rng = np.random.default_rng(10_000 + seed)
    sc = xp.scenes.config_dam_breach(seed=1000 + seed, scale=scale)
    sand = sc["materials"][0]
    sand["E"] = float(np.exp(rng.uniform(np.log(1e5), np.log(4e5))))
    sand["p0"] = xp.scenes.dp_alpha(float(rng.uniform(28, 40)))
    return sc


def generate(n_scenes: int = 512, scale: float = 0.05, max_warm: int = 120, logged: int = 4,
             rows_per_substep: int = 1024, seed: int = 0, verbose: bool = True):
    xp = _pkg()
    rng = np.random.default_rng(seed)
    X, Y = [], []
    t0 = time.time()
    for s in range(n_scenes):
        sc = training_scene(xp, s, scale)
        it = sc["iterations"]
        with xp.Simulation(sc) as sim:
            sim.write_params(xp.params_for(sc))
            sim.set_solver(0, 0.0, False, True)
            w = int(rng.integers(0, max_warm + 1))
            if w:
                sim.step(w, it, True)
            for _ in range(logged):
                sim.encode_substep(it, True)
                f, t, _ = sim.read_training()
                solid = f[:, 8:15].sum(axis=1) > 0
                idx = np.flatnonzero(solid)
                if len(idx) > rows_per_substep:
                    idx = rng.choice(idx, rows_per_substep, replace=False)
                X.append(f[idx])
                Y.append(t[idx])
        if verbose and (s + 1) % 64 == 0:
            print(f"scenes {s + 1}/{n_scenes}  rows {sum(len(y) for y in Y)}  {time.time() - t0:.1f}s", flush=True)
    return np.concatenate(X), np.concatenate(Y)


def _he_init(seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    parts = [rng.standard_normal((64, 16)) * np.sqrt(2.0 / 16), np.zeros(64),
             rng.standard_normal((64, 64)) * np.sqrt(2.0 / 64), np.zeros(64),
             rng.standard_normal((64, 64)) * np.sqrt(2.0 / 64), np.zeros(64),
             rng.standard_normal(64) * np.sqrt(1.0 / 64), np.zeros(1)]
    return np.concatenate([p.reshape(-1) for p in parts]).astype(np.float32)


def fit_network(X, Y, steps: int = 3000, batch: int = 8192, lr: float = 2e-3, seed: int = 0):
    """Standardise, train on the GPU, fold the standardisation back in."""
    net = importlib.import_module("xpbi-webgpu_gb300.net")
    rng = np.random.default_rng(seed)
    X = np.asarray(X, np.float64)
    Y = np.asarray(Y, np.float64)
    mx = X.mean(0)
    sx = X.std(0)
    sx[sx < 1e-12] = 1.0
    my, sy = Y.mean(), max(Y.std(), 1e-30)
    perm = rng.permutation(len(X))
    Xs = ((X[perm] - mx) / sx).astype(np.float32)
    Ys = ((Y[perm] - my) / sy).astype(np.float32)
    p, hist = net.train(Xs, Ys, _he_init(seed), steps=steps, batch=min(batch, len(Xs)), lr=lr)
    # fold: z1 = W1 ((x - mx) / sx) + b1 = (W1 / sx) x + (b1 - (W1 / sx) mx)
    p = p.astype(np.float64)
    W1 = p[:1024].reshape(64, 16)
    b1 = p[1024:1088]
    W1f = W1 / sx
    b1f = b1 - W1f @ mx
    p[:1024] = W1f.reshape(-1)
    p[1024:1088] = b1f
    # y = sy * y_s + my
    p[9408:9472] *= sy
    p[9472] = p[9472] * sy + my
    return p.astype(np.float32), hist


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=512)
    ap.add_argument("--scale", type=float, default=0.05)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--out", default=WEIGHTS)
    args = ap.parse_args()
    X, Y = generate(args.scenes, args.scale)
    Y = Y - X[:, 4]  # increment over the previous substep's multiplier
    print("rows", len(X), "target mean/std", float(Y.mean()), float(Y.std()), flush=True)
    p, hist = fit_network(X, Y, steps=args.steps)
    print("loss (standardised) first / last", float(hist[:20].mean()), float(hist[-20:].mean()), flush=True)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    p.tofile(args.out)
    print("wrote", args.out)


if __name__ == "__main__":
    main()
