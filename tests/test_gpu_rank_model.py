"""What the learned-rank MLP gains: trained on exact ranks logged by the plain
path, it sizes the randomized sketch; without it the chosen mode must sketch
at full size.  Ranks stay exact (fallback covers misses) and the update gets
cheaper."""
import math
import time

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def decay_bond(chi, d, rng):
    a, b, s = O.decay_theta_factors(chi, rng, decay=d)
    return a, b, s


def test_trained_rank_model_shrinks_the_sketch(engine):
    rng = np.random.default_rng(99)
    cutoff = 1e-4
    # --- log exact ranks from the plain FP64 path ---
    plain = engine.Engine(mode="plain")
    plain.set_rank_logging(True)
    for _ in range(40):
        chi = int(rng.choice([64, 96, 128]))
        d = float(rng.uniform(0.55, 0.9))
        a, b, s = decay_bond(chi, d, rng)
        m = plain.mps([a, b])
        m.set_bond_spectrum(1, s)
        m.apply_2q(O.haar_unitary(rng), 1, cutoff, 2 * chi)
        m.free()
    X, Y = plain.rank_log()
    assert X.shape == (40, 16)
    plain.close()
    # --- train on the GPU ---
    with_model = engine.Engine(mode="chosen")
    loss = with_model.train_rank_model(X, Y, epochs=400, batch=16, lr=2e-3, seed=3)
    assert loss < 0.01
    without = engine.Engine(mode="chosen", use_rank_model=0)
    # --- held-out bonds ---
    sk_with, sk_without, t_with, t_without, n_fb = [], [], 0.0, 0.0, 0
    for _ in range(6):
        chi = 128
        d = float(rng.uniform(0.6, 0.8))
        a, b, s = decay_bond(chi, d, rng)
        g = O.haar_unitary(rng)
        ex = O.apply_2q([a.copy(), b.copy()], g, 1, cutoff, 0)
        for eng, sk, which in ((with_model, sk_with, "with"), (without, sk_without, "without")):
            m = eng.mps([a.astype(np.complex64), b.astype(np.complex64)], dtype=np.complex64)
            m.set_bond_spectrum(1, s)
            t0 = time.perf_counter()
            st = m.apply_2q(g, 1, cutoff, 0)
            dt = time.perf_counter() - t0
            # FP32-level spectra may move the rank by one at a near-tie of the
            # tail rule; the truncation itself must stay as good as the exact one
            assert abs(st["rank"] - ex.rank) <= 1, (which, st, ex.rank)
            th = O.apply_gate_to_theta(O.theta_of(a.astype(np.complex64).astype(complex),
                                                  b.astype(np.complex64).astype(complex)), g, chi, chi)
            err = np.linalg.norm(th - O.theta_of(m.site(1).astype(complex), m.site(2).astype(complex)))
            assert err <= 1.1 * np.sqrt(ex.discarded_weight) + 2e-6, (which, err, np.sqrt(ex.discarded_weight))
            sk.append(st["sketch_size"] or 2 * chi)
            if which == "with":
                t_with += dt
                n_fb += st["fallback"]
            else:
                t_without += dt
            m.free()
    # the model sizes the sketch well below the full 2*chi the method without it needs
    assert np.mean(sk_with) < 0.8 * np.mean(sk_without), (sk_with, sk_without)
    assert n_fb <= 2
    print(f"sketch with model {np.mean(sk_with):.0f} vs {np.mean(sk_without):.0f}; "
          f"time {t_with:.3f}s vs {t_without:.3f}s; fallbacks {n_fb}")
    with_model.close()
    without.close()
