"""The autotuner: it times launch shapes of the batched kernel and sketch
widths of the chosen split on the GPU, writes its JSON cache, a load of that
cache reproduces the choice, and a tuned batch gives the same results as the
default launch shape (a launch shape moves tasks between CTAs, not their
arithmetic)."""
import importlib.util
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def autotune_module():
    path = os.path.join(ROOT, "qaintensor.jl_gb300", "autotune.py")
    spec = importlib.util.spec_from_file_location("qaintensor_gb300_autotune", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_tune_save_load_and_reuse(engine, tmp_path):
    at = autotune_module()
    cache_path = str(tmp_path / "autotune.json")
    eng = engine.Engine(mode="chosen")
    entry = {"batch": {"16": at.tune_batch(engine, eng, 16, ncirc=24, reps=1, candidates=((128, 2), (256, 1)),
                                           qubits=(6, 12), depths=(3, 8))}}
    eng.close()
    entry["sketch"] = {"256": at.tune_sketch(engine, 256, reps=1, candidates=(1.125, 1.25))}
    at.save({at.device_name(0): entry}, cache_path)
    cache = at.load(cache_path)
    assert cache[at.device_name(0)] == entry  # the JSON round trip keeps every field
    b16 = entry["batch"]["16"]
    assert (b16["threads"], b16["ctas_per_sm"]) in ((128, 2), (256, 1)) and b16["updates_per_s"] > 0
    sk = entry["sketch"]["256"]
    assert sk["ratio"] <= 1.0 + sk["tol"], sk
    assert at.engine_options(cache, 256) == {"cap_sketch": sk["cap_sketch"]}

    # reuse: a new batch takes the tuned shape and computes what the default shape does
    rng = np.random.default_rng(77)
    circuits = []
    for _ in range(8):
        n = int(rng.integers(5, 10))
        circuits.append((n, O.brickwork_gates(n, 5, rng)))
    layers = [[] for _ in range(5)]
    for ci, (_, gates) in enumerate(circuits):
        for (layer, w, g) in gates:
            layers[layer - 1].append((ci, w, g))
    results = []
    for tuned in (False, True):
        eng = engine.Engine(mode="chosen")
        b = engine.Batch(eng, [c[0] for c in circuits], [16] * len(circuits))
        if tuned:
            applied = at.apply_batch(b, cache)
            assert applied == [(16, b16["threads"], b16["ctas_per_sm"])]
            assert b.get_launch(16) == (b16["threads"], b16["ctas_per_sm"])
        b.run(layers, 1e-8, use_graph=True)
        results.append((b.expect_z(1), [list(b.bond_dims(c)) for c in range(len(circuits))], b.task_stats()[0]))
        b.free()
        eng.close()
    (z0, d0, r0), (z1, d1, r1) = results
    assert d0 == d1 and list(r0) == list(r1)
    np.testing.assert_allclose(z0, z1, atol=1e-6)
    for ci, (n, gates) in enumerate(circuits):
        sites, _ = O.run_brickwork(n, gates, 1e-8, 16)
        assert abs(z1[ci] - O.expect_z(sites, 1)) <= 5e-5
