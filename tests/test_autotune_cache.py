"""The autotuner's host logic without a GPU: the JSON cache round trip, the
device entry lookup, the launch shapes handed to a batch and the engine
options chosen for a chi_max, and the seeded tuning ensemble."""
import importlib.util
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_autotune():
    spec = importlib.util.spec_from_file_location("qt_autotune", os.path.join(ROOT, "qaintensor.jl_gb300", "autotune.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["qt_autotune"] = mod
    spec.loader.exec_module(mod)
    return mod


class FakeBatch:
    def __init__(self):
        self.calls = []

    def set_launch(self, bucket, threads, ctas_per_sm):
        self.calls.append((bucket, threads, ctas_per_sm))


def sample_cache(at):
    return {at.device_name(): {
        "batch": {"64": {"threads": 512, "ctas_per_sm": 1}, "16": {"threads": 128, "ctas_per_sm": 2}},
        "sketch": {"1024": {"cap_sketch": 1.125}, "256": {"cap_sketch": 1.25}}}}


def test_cache_round_trip_and_missing_file(tmp_path):
    at = load_autotune()
    path = str(tmp_path / "sub" / "autotune.json")
    assert at.load(path) == {}  # no file yet: an empty cache, not an error
    cache = sample_cache(at)
    assert at.save(cache, path) == path
    assert at.load(path) == cache
    with open(path, "w") as f:
        f.write("{not json")
    assert at.load(path) == {}  # a damaged file reads as an empty cache


def test_cache_path_from_the_environment(monkeypatch, tmp_path):
    at = load_autotune()
    monkeypatch.setenv("QT_AUTOTUNE_CACHE", str(tmp_path / "c.json"))
    assert at.default_cache_path() == str(tmp_path / "c.json")


def test_launch_shapes_applied_in_bucket_order():
    at = load_autotune()
    batch = FakeBatch()
    applied = at.apply_batch(batch, sample_cache(at))
    assert applied == [(16, 128, 2), (64, 512, 1)]
    assert batch.calls == applied
    assert at.apply_batch(FakeBatch(), {}) == []  # nothing tuned: the kernel's defaults stay


def test_engine_options_take_the_nearest_tuned_chi():
    at = load_autotune()
    cache = sample_cache(at)
    assert at.engine_options(cache, 1024) == {"cap_sketch": 1.125}
    assert at.engine_options(cache, 700) == {"cap_sketch": 1.125}  # log-nearest of 256 and 1024
    assert at.engine_options(cache, 300) == {"cap_sketch": 1.25}
    assert at.engine_options({}, 1024) == {}
    # an entry stored under "default" serves any device
    assert at.engine_options({"default": cache[at.device_name()]}, 256) == {"cap_sketch": 1.25}


def test_tuning_ensemble_is_seeded_and_brickwork():
    at = load_autotune()
    a = at.ensemble(np.random.default_rng(7), 12, 32)
    b = at.ensemble(np.random.default_rng(7), 12, 32)
    nq, caps, layers = a
    assert nq == b[0] and caps == [32] * 12 and len(layers) == len(b[2])
    for la, lb in zip(layers, b[2]):
        assert [(c, w) for c, w, _ in la] == [(c, w) for c, w, _ in lb]
        assert all(np.array_equal(g, h) for (_, _, g), (_, _, h) in zip(la, lb))
    for li, layer in enumerate(layers, start=1):
        for ci, w, g in layer:
            assert 8 <= nq[ci] <= 40 and 1 <= w < nq[ci]
            assert w % 2 == (1 if li % 2 else 0)  # odd layers on (1,2),(3,4)..., even on (2,3),...
            assert np.allclose(g.conj().T @ g, np.eye(4), atol=1e-12)  # Haar gates are unitary
