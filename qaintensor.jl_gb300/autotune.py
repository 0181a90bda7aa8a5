"""Autotuner of the engine's launch and sketch parameters, with a JSON cache.

Two choices are tuned on the GPU the engine runs on:

* the launch shape of the batched path's persistent layer kernel, per
  bond-cap bucket (caps 16, 32, 64, 128): threads per CTA (128 to 1024)
  and CTAs per SM (1 or 2).  Each candidate runs the same seeded ensemble
  of Haar brickwork circuits (qubits uniform in [8, 40], depths uniform in
  [4, 24], every circuit at the bucket's cap) as a captured CUDA graph;
  the fastest replay wins.  Every candidate computes the same updates -- a
  launch shape changes which CTA takes which task, not the arithmetic of a
  task -- so the choice is by time alone.
* the sketch width of a rank pinned at the chi_max cap in the chosen split
  (``cap_sketch``, a multiple of chi_max), per chi_max: each candidate
  updates the same decaying-spectrum bond; the fastest sketch whose
  truncation error stays within ``tol`` of the exact FP64 split's (cuSOLVER
  on the same complex64 input) wins.

The cache maps the device name to its tuned values:

    {"NVIDIA GB300": {"batch": {"16": {"threads": 128, "ctas_per_sm": 4,
                                       "updates_per_s": ..., "candidates": [...]}, ...},
                      "sketch": {"1024": {"cap_sketch": 1.125, "ms": ..., "ratio": ...}}}}

``tune_*`` measure and return entries, ``save``/``load`` keep the cache,
``apply_batch`` and ``engine_options`` turn it into launch shapes and engine
options.  The tuner is host code over the engine's public API.
"""

from __future__ import annotations

import json
import math
import os
from typing import Dict, Iterable, List, Sequence, Tuple

import numpy as np

BUCKETS = (16, 32, 64, 128)
BATCH_CANDIDATES: Tuple[Tuple[int, int], ...] = ((128, 2), (256, 1), (256, 2), (512, 1), (512, 2), (1024, 1))
SKETCH_CANDIDATES: Tuple[float, ...] = (1.0625, 1.125, 1.1875, 1.25)


def default_cache_path() -> str:
    """``QT_AUTOTUNE_CACHE``, else ``~/.cache/qaintensor_gb300/autotune.json``."""
    return os.environ.get("QT_AUTOTUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache",
                                                               "qaintensor_gb300", "autotune.json")


def device_name(device: int = 0) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:  # no torch or no device: one entry for every device
        return "default"


def load(path: str | None = None) -> Dict:
    path = path or default_cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save(cache: Dict, path: str | None = None) -> str:
    path = path or default_cache_path()
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    return path


# --------------------------------------------------------------------------
# synthetic workloads (seeded)
# --------------------------------------------------------------------------

def _haar(rng: np.random.Generator) -> np.ndarray:
    z = (rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))) / math.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))[None, :]


def ensemble(rng: np.random.Generator, ncirc: int, cap: int, qubits=(8, 40), depths=(4, 24)):
    """Brickwork circuits at one bond cap: (nqubits, caps, layers)."""
    nq, caps, circuits = [], [], []
    for _ in range(ncirc):
        n = int(rng.integers(qubits[0], qubits[1] + 1))
        depth = int(rng.integers(depths[0], depths[1] + 1))
        gates = []
        for layer in range(1, depth + 1):
            for w in range(1 if layer % 2 else 2, n, 2):
                gates.append((layer, w, _haar(rng)))
        nq.append(n)
        caps.append(cap)
        circuits.append(gates)
    layers = [[] for _ in range(max((g[-1][0] for g in circuits if g), default=0))]
    for ci, gates in enumerate(circuits):
        for (layer, w, g) in gates:
            layers[layer - 1].append((ci, w, g))
    return nq, caps, layers


# --------------------------------------------------------------------------
# the batched kernel's launch shape
# --------------------------------------------------------------------------

def time_batch(qt, eng, nq, caps, layers, bucket: int, shape: Tuple[int, int], cutoff: float, reps: int) -> Dict:
    b = qt.Batch(eng, nq, caps)
    try:
        b.set_launch(bucket, shape[0], shape[1])
        b.run(layers, cutoff, use_graph=True)  # capture + first run
        best = float("inf")
        for _ in range(reps):
            b.reset()
            eng.sync()
            eng.timer_record(0)
            b.replay()
            eng.timer_record(1)
            best = min(best, eng.timer_elapsed(0, 1))
        return {"threads": shape[0], "ctas_per_sm": shape[1], "ms": best, "updates_per_s": b.ntask / (best / 1e3),
                "tasks": b.ntask}
    finally:
        b.free()


def tune_batch(qt, eng, bucket: int, ncirc: int = 256, reps: int = 2, cutoff: float = 1e-8, seed: int = 4242,
               candidates: Sequence[Tuple[int, int]] = BATCH_CANDIDATES, qubits=(8, 40), depths=(4, 24)) -> Dict:
    """Time every launch shape on one seeded ensemble at cap ``bucket``."""
    nq, caps, layers = ensemble(np.random.default_rng(seed + bucket), ncirc, bucket, qubits, depths)
    rows = [time_batch(qt, eng, nq, caps, layers, bucket, c, cutoff, reps) for c in candidates]
    best = min(rows, key=lambda r: r["ms"])
    return {"threads": best["threads"], "ctas_per_sm": best["ctas_per_sm"], "updates_per_s": best["updates_per_s"],
            "ncirc": ncirc, "candidates": rows}


# --------------------------------------------------------------------------
# the sketch width at the chi_max cap
# --------------------------------------------------------------------------

def _decay_pair(chi: int, rng: np.random.Generator, decay: float = 0.97):
    n = 2 * chi
    g1 = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(2)
    g2 = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(2)
    q1, _ = np.linalg.qr(g1)
    q2, _ = np.linalg.qr(g2)
    s = decay ** np.arange(chi, dtype=np.float64)
    s /= np.linalg.norm(s)
    a = (q1[:, :chi] * s[None, :]).reshape((chi, 2, chi), order="F")
    b = q2[:, :chi].conj().T.reshape((chi, 2, chi), order="F")
    return a.astype(np.complex64), b.astype(np.complex64), s


def _product(sites) -> np.ndarray:
    a, b = (x.astype(np.complex128) for x in sites)
    return a.reshape((-1, a.shape[2]), order="F") @ b.reshape((b.shape[0], -1), order="F")


def tune_sketch(qt, chi: int, device: int = 0, reps: int = 2, tol: float = 1e-3, seed: int = 99,
                candidates: Sequence[float] = SKETCH_CANDIDATES, rank_model=None) -> Dict:
    """The fastest cap_sketch whose truncation error is within (1 + tol) of
    the exact FP64 split's on a 0.97^k bond at chi (truncated to chi)."""
    rng = np.random.default_rng(seed + chi)
    a, b, s = _decay_pair(chi, rng)
    g = _haar(rng)
    ref = qt.Engine(mode="cusolver", device=device)
    m = ref.mps([a.astype(np.complex128), b.astype(np.complex128)], dtype=np.complex128)
    m.apply_2q(g, 1, 1e-12, chi)
    exact_t = _product([m.site(1), m.site(2)])
    m.free()
    ref.close()
    # the exact theta' of the complex64 inputs
    th = _product([a, b]).reshape((chi, 2, 2, chi), order="F")
    g4 = np.asarray(g).reshape((2, 2, 2, 2), order="F")
    th = np.einsum("pqrs,arsb->apqb", g4, th).reshape((2 * chi, 2 * chi), order="F")
    exact_err = float(np.linalg.norm(th - exact_t))
    rows = []
    for cs in candidates:
        eng = qt.Engine(mode="chosen", device=device, tc_gemm=1, cap_sketch=float(cs))
        if rank_model is None:
            # the width tuned here is the one of a rank predicted at the cap:
            # a model whose output is the constant 1 (k = k_max) stands in
            rank_model = np.zeros(eng.n_params, dtype=np.float32)
            rank_model[-1] = 1.0
        eng.set_rank_params(rank_model, enable=True)
        tmpl = eng.mps([a, b], dtype=np.complex64)
        tmpl.set_bond_spectrum(1, s)
        best, st, err = float("inf"), None, None
        for r in range(reps + 1):
            x = tmpl.clone()
            eng.sync()
            eng.timer_record(0)
            st = x.apply_2q(g, 1, 1e-12, chi)
            eng.timer_record(1)
            if r > 0:  # the first update warms up
                best = min(best, eng.timer_elapsed(0, 1))
            if r == reps:
                err = float(np.linalg.norm(th - _product([x.site(1), x.site(2)])))
            x.free()
        tmpl.free()
        eng.close()
        rows.append({"cap_sketch": cs, "ms": best, "ratio": err / exact_err if exact_err > 0 else None,
                     "sketch_size": st["sketch_size"], "fallback": st["fallback"]})
    ok = [r for r in rows if r["ratio"] is not None and r["ratio"] <= 1.0 + tol and not r["fallback"]]
    pick = min(ok, key=lambda r: r["ms"]) if ok else max(rows, key=lambda r: r["cap_sketch"])
    return {"cap_sketch": pick["cap_sketch"], "ms": pick["ms"], "ratio": pick["ratio"], "tol": tol,
            "candidates": rows}


# --------------------------------------------------------------------------
# the whole tuning pass and its use
# --------------------------------------------------------------------------

def tune(qt, path: str | None = None, device: int = 0, buckets: Iterable[int] = BUCKETS,
         sketch_chis: Iterable[int] = (), ncirc: int = 256, reps: int = 2, **kw) -> Dict:
    """Tune the given buckets and sketch widths, merge them into the cache
    for this device, save it and return the device's entry."""
    cache = load(path)
    entry = cache.setdefault(device_name(device), {})
    eng = qt.Engine(mode="chosen", device=device)
    try:
        for bk in buckets:
            entry.setdefault("batch", {})[str(bk)] = tune_batch(qt, eng, bk, ncirc=ncirc, reps=reps, **kw)
    finally:
        eng.close()
    for chi in sketch_chis:
        entry.setdefault("sketch", {})[str(chi)] = tune_sketch(qt, chi, device=device, reps=reps)
    save(cache, path)
    return entry


def device_entry(cache: Dict, device: int = 0) -> Dict:
    return cache.get(device_name(device)) or cache.get("default") or {}


def apply_batch(batch, cache: Dict, device: int = 0) -> List[Tuple[int, int, int]]:
    """Set the tuned launch shape of every tuned bucket on ``batch``; returns
    the (bucket, threads, ctas_per_sm) applied."""
    applied = []
    for bk, e in sorted(device_entry(cache, device).get("batch", {}).items(), key=lambda kv: int(kv[0])):
        batch.set_launch(int(bk), int(e["threads"]), int(e["ctas_per_sm"]))
        applied.append((int(bk), int(e["threads"]), int(e["ctas_per_sm"])))
    return applied


def engine_options(cache: Dict, chi_max: int, device: int = 0) -> Dict:
    """Engine options for a workload at ``chi_max``: the cap_sketch tuned at
    the nearest tuned chi_max (none when nothing is tuned)."""
    sk = device_entry(cache, device).get("sketch", {})
    if not sk:
        return {}
    near = min(sk, key=lambda c: abs(math.log(int(c) / max(chi_max, 1))))
    return {"cap_sketch": float(sk[near]["cap_sketch"])}
