"""Train the learned-rank MLP from exact kept ranks logged by the plain FP64 path.

Training data: every update of a seeded ensemble run with an exact FP64
split (the rank from the tail rule) is logged by the engine as
(16 features, k / k_max):

* depth-10 runs of the 64-qubit Haar brickwork ensemble (chi_max 1024,
  cutoff 1e-8, complex128), split by cuSOLVER's exact FP64 SVD, the faster
  exact path at the 1024 x 1024 theta' of the tenth layer;
* brickwork circuits of depth 10 with Haar gates on 16-40 qubits,
  chi_max in {16, 32, 64, 128}, cutoffs 1e-10 .. 1e-4 (the engine's FP64
  Jacobi);
* single-bond updates of decaying-spectrum bonds theta = Q1 diag(d^k) Q2^H
  (d in 0.80 .. 0.98, chi 64 .. 512) under Haar gates, cutoffs 1e-8 .. 1e-3,
  the bond's spectrum supplied as the previous spectrum.

The network is then trained on the GPU with the engine's forward/backward
and Adam kernels.  Parameters go to rank_model_params.npy next to this file
and a summary to rank_model_train.json.

    python qaintensor.jl_gb300/train_rank_model.py [--c3-circuits 24] [--circuits 48] [--bonds 96]
"""

from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def haar(rng):
    z = (rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))) / math.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))[None, :]


def decay_bond(chi, d, rng):
    n = 2 * chi
    g1 = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(2)
    g2 = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(2)
    q1, _ = np.linalg.qr(g1)
    q2, _ = np.linalg.qr(g2)
    s = d ** np.arange(chi, dtype=np.float64)
    s /= np.linalg.norm(s)
    a = (q1[:, :chi] * s[None, :]).reshape((chi, 2, chi), order="F")
    b = q2[:, :chi].conj().T.reshape((chi, 2, chi), order="F")
    return a, b, s


def collect(eng, circuits: int, bonds: int, seed: int, c3_circuits: int = 0, log=print):
    rng = np.random.default_rng(seed)
    eng.set_rank_logging(True)
    eng.clear_rank_log()
    t0 = time.time()
    for c in range(c3_circuits):
        n, depth = 64, 10
        mps = eng.product_state(n)
        for layer in range(1, depth + 1):
            mps.set_circuit_position(layer, depth)
            for w in range(1 if layer % 2 else 2, n, 2):
                mps.apply_2q(haar(rng), w, 1e-8, 1024, mode="cusolver")
        mps.free()
        log(f"  64-qubit circuits {c + 1}/{c3_circuits}: {eng.rank_log()[1].size} samples, {time.time() - t0:.0f}s")
    for c in range(circuits):
        n = int(rng.integers(16, 41))
        chi_max = int(rng.choice([16, 32, 64, 128]))
        cutoff = float(10.0 ** rng.uniform(-10, -4))
        depth = 10
        mps = eng.product_state(n)
        for layer in range(1, depth + 1):
            mps.set_circuit_position(layer, depth)
            for w in range(1 if layer % 2 else 2, n, 2):
                mps.apply_2q(haar(rng), w, cutoff, chi_max, mode="plain")
        mps.free()
        if c % 8 == 7:
            log(f"  circuits {c + 1}/{circuits}: {eng.rank_log()[1].size} samples, {time.time() - t0:.0f}s")
    for j in range(bonds):
        chi = int(rng.choice([64, 128, 256, 512]))
        d = float(rng.uniform(0.80, 0.98))
        cutoff = float(10.0 ** rng.uniform(-8, -3))
        a, b, s = decay_bond(chi, d, rng)
        mps = eng.mps([a, b])
        mps.set_bond_spectrum(1, s)
        mps.apply_2q(haar(rng), 1, cutoff, 2 * chi, mode="plain")
        mps.free()
        if j % 16 == 15:
            log(f"  bonds {j + 1}/{bonds}: {eng.rank_log()[1].size} samples, {time.time() - t0:.0f}s")
    X, Y = eng.rank_log()
    eng.set_rank_logging(False)
    return X, Y


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--c3-circuits", type=int, default=24)
    ap.add_argument("--circuits", type=int, default=48)
    ap.add_argument("--bonds", type=int, default=96)
    ap.add_argument("--epochs", type=int, default=200)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--out", default=os.path.join(HERE, "rank_model_params.npy"))
    ap.add_argument("--summary", default=os.path.join(HERE, "rank_model_train.json"))
    ap.add_argument("--log", default="", help="also save the logged (features, rank) samples to this .npz")
    args = ap.parse_args()
    import __graft_entry__ as g
    qt = g.load_package()
    eng = qt.Engine(mode="plain")
    t0 = time.time()
    X, Y = collect(eng, args.circuits, args.bonds, args.seed, args.c3_circuits)
    t_log = time.time() - t0
    rng = np.random.default_rng(args.seed + 1)
    idx = rng.permutation(len(Y))
    nval = max(1, len(Y) // 10)
    val, tr = idx[:nval], idx[nval:]
    t1 = time.time()
    loss = eng.train_rank_model(X[tr], Y[tr], epochs=args.epochs, batch=256, lr=1e-3, seed=args.seed)
    t_train = time.time() - t1
    pred = eng.mlp_forward(X[val])
    val_rmse = float(np.sqrt(np.mean((pred - Y[val]) ** 2)))
    np.save(args.out, eng.rank_params())
    summary = {"samples": int(len(Y)), "train": int(len(tr)), "val": int(nval), "train_mse": loss,
               "val_rmse_fraction": val_rmse, "log_seconds": t_log, "train_seconds": t_train,
               "epochs": args.epochs, "seed": args.seed, "c3_circuits": args.c3_circuits,
               "c3_samples": int(args.c3_circuits * sum(len(range(1 if l % 2 else 2, 64, 2)) for l in range(1, 11))),
               "circuits": args.circuits, "bonds": args.bonds}
    with open(args.summary, "w") as f:
        json.dump(summary, f, indent=1)
    if args.log:
        np.savez_compressed(args.log, X=X, Y=Y)
    print(json.dumps(summary))
    eng.close()


if __name__ == "__main__":
    main()
