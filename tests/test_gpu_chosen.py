"""GPU tests of the mixed-precision ("chosen") mode and the learned-rank MLP."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def const_model(eng, frac):
    """A rank model whose output is the constant `frac` (all weights zero)."""
    p = np.zeros(eng.n_params, dtype=np.float32)
    p[-1] = frac
    eng.set_rank_params(p, enable=True)


def exact_theta(a, b, g):
    chil, chir = a.shape[0], b.shape[2]
    return O.apply_gate_to_theta(O.theta_of(a, b), g, chil, chir)


@pytest.mark.parametrize("chi", [128, 256])
def test_randomized_path_matches_exact_truncation(engine, chi):
    # decaying spectrum; cutoff far above the FP32-level noise floor: the
    # sketched split keeps the exact rank and its truncation error is within
    # 1.1x of the exact SVD's
    rng = np.random.default_rng(chi)
    a, b, s = O.decay_theta_factors(chi, rng, decay=0.6)
    g = O.haar_unitary(rng)
    cutoff = 1e-3
    ex = O.apply_2q([a.copy(), b.copy()], g, 1, cutoff, 0)
    eng = engine.Engine(mode="chosen")
    const_model(eng, min(1.0, 1.3 * ex.rank / (2 * chi)))
    m = eng.mps([a.astype(np.complex64), b.astype(np.complex64)], dtype=np.complex64)
    st = m.apply_2q(g, 1, cutoff, 0)
    assert st["sketch_size"] > 0 and not st["fallback"], st
    assert st["rank"] == ex.rank, (st, ex.rank)
    th = exact_theta(a.astype(np.complex64).astype(complex), b.astype(np.complex64).astype(complex), g)
    approx = O.theta_of(m.site(1).astype(complex), m.site(2).astype(complex))
    err = np.linalg.norm(th - approx)
    assert err <= 1.1 * np.sqrt(ex.discarded_weight), (err, np.sqrt(ex.discarded_weight))
    A = m.site(1).reshape((2 * chi, -1), order="F").astype(complex)
    np.testing.assert_allclose(A.conj().T @ A, np.eye(A.shape[1]), atol=2e-5)
    m.free()
    eng.close()


def test_undersized_sketch_falls_back_to_exact(engine):
    rng = np.random.default_rng(11)
    chi = 64
    a, b, s = O.decay_theta_factors(chi, rng, decay=0.97)
    g = O.haar_unitary(rng)
    cutoff = 1e-4
    ex = O.apply_2q([a.copy(), b.copy()], g, 1, cutoff, 0)
    eng = engine.Engine(mode="chosen")
    const_model(eng, 0.05)  # far below the rank the cutoff needs
    m = eng.mps([a.astype(np.complex64), b.astype(np.complex64)], dtype=np.complex64)
    st = m.apply_2q(g, 1, cutoff, 0)
    assert st["fallback"] == 1 and st["rank"] == ex.rank, (st, ex.rank)
    m.free()
    eng.close()


def test_chosen_brickwork_expectations_within_1e6(engine):
    rng = np.random.default_rng(5)
    n, depth, cutoff, chi_max = 10, 8, 1e-8, 16
    gates = O.brickwork_gates(n, depth, rng)
    eng = engine.Engine(mode="chosen")
    mps = eng.product_state(n, dtype=np.complex64)
    for (_, w, g) in gates:
        mps.apply_2q(g, w, cutoff, chi_max)
    sites, _ = O.run_brickwork(n, gates, cutoff, chi_max)
    for i in range(1, n):
        assert abs(mps.expect_zz(i) - O.expect_zz(sites, i)) <= 1e-6
    assert abs(mps.expect_z(1) - O.expect_z(sites, 1)) <= 1e-6
    mps.free()
    eng.close()


def test_mlp_forward_and_gradients_match_fp64_oracle(engine):
    rng = np.random.default_rng(3)
    X = rng.random((300, 16))
    Y = rng.random(300)
    params = O.mlp_init(rng)
    flat = np.concatenate([params[0].ravel(), params[1], params[2].ravel(), params[3], params[4].ravel(), params[5]])
    eng = engine.Engine()
    assert flat.size == eng.n_params
    eng.set_rank_params(flat.astype(np.float32), enable=False)
    pred = eng.mlp_forward(X.astype(np.float32))
    ref, cache = O.mlp_forward(params, X)
    np.testing.assert_allclose(pred, ref, rtol=1e-4, atol=1e-4)
    loss, g = eng.mlp_loss_grad(X, Y, flat)
    gref = O.mlp_backward(params, cache, ref, Y)
    gflat = np.concatenate([gref[0].ravel(), gref[1], gref[2].ravel(), gref[3], gref[4].ravel(), gref[5]])
    assert abs(loss - O.mlp_loss(ref, Y)) <= 1e-4 * max(1.0, loss)
    np.testing.assert_allclose(g, gflat, rtol=2e-3, atol=2e-5 * np.abs(gflat).max())
    eng.close()


def test_mlp_training_reduces_loss(engine):
    rng = np.random.default_rng(4)
    X = rng.random((4000, 16)).astype(np.float32)
    Y = (0.2 + 0.5 * X[:, 0] - 0.3 * X[:, 5] * X[:, 9]).astype(np.float32)
    eng = engine.Engine()
    params0 = np.concatenate([p.ravel() for p in O.mlp_init(np.random.default_rng(9))]).astype(np.float32)
    loss0, _ = eng.mlp_loss_grad(X, Y, params0)
    loss = eng.train_rank_model(X, Y, epochs=20, batch=128, lr=2e-3, seed=1, init=params0)
    assert loss < 0.05 * loss0, (loss, loss0)
    pred = eng.mlp_forward(X[:100])
    assert np.sqrt(np.mean((pred - Y[:100]) ** 2)) < 0.05
    eng.close()


def test_rank_features_match_oracle(engine):
    rng = np.random.default_rng(6)
    eng = engine.Engine()
    n = 6
    mps = eng.product_state(n)
    gates = O.brickwork_gates(n, 3, rng)
    sites = O.product_state(n)
    kept = {}  # bond -> spectrum kept by its last update
    for (layer, w, g) in gates[:-1]:
        mps.apply_2q(g, w, 1e-10, 8)
        st = O.apply_2q(sites, g, w, 1e-10, 8)
        kept[w] = st.spectrum[: st.rank]
    layer, w, g = gates[-1]
    mps.set_circuit_position(layer, 3)
    f = mps.rank_features(g, w, 1e-10, 8)
    a, b = sites[w - 1], sites[w]
    s_prev = kept.get(w, np.ones(a.shape[2]))
    fr = O.rank_features(s_prev, g, w - 1, n, layer, 3, a.shape[0], b.shape[2], 8, 1e-10)
    np.testing.assert_allclose(f, fr, rtol=1e-5, atol=1e-6)
    eng.close()


@pytest.mark.parametrize("scale", [1e11, 1e-13])
def test_chosen_split_is_scale_invariant(engine, scale):
    """complex64 storage keeps squared norms in FP32: theta' of norm ~1e22 (or
    ~1e-26) would overflow (underflow) them.  The FP32 splits scale by a power
    of two first, so the sketched and the direct split give the scaled
    results of the unit-norm problem: same rank, values and error relative to
    the scale, no fallback."""
    rng = np.random.default_rng(3)
    chi = 128
    a, b, s = O.decay_theta_factors(chi, rng, decay=0.6)
    g = O.haar_unitary(rng)
    cutoff = 1e-3
    ex = O.apply_2q([a.copy(), b.copy()], g, 1, cutoff, 0)
    th = exact_theta(a.astype(np.complex64).astype(complex), b.astype(np.complex64).astype(complex), g)
    for frac in (1.3 * ex.rank / (2 * chi), 1.0):  # sketched split, then the direct one
        eng = engine.Engine(mode="chosen")
        const_model(eng, min(1.0, frac))
        m = eng.mps([(a * scale).astype(np.complex64), (b * scale).astype(np.complex64)], dtype=np.complex64)
        st = m.apply_2q(g, 1, cutoff * scale * scale, 0)
        assert not st["fallback"] and st["rank"] == ex.rank, (st, ex.rank)
        approx = O.theta_of(m.site(1).astype(complex), m.site(2).astype(complex)) / (scale * scale)
        err = np.linalg.norm(th - approx)
        assert err <= 1.1 * np.sqrt(ex.discarded_weight), (err, np.sqrt(ex.discarded_weight))
        m.free()
        eng.close()
    # the bare truncated SVD through the same FP32 split
    M = (th * scale * scale).astype(np.complex64)
    eng = engine.Engine(mode="chosen")
    U, S, Vh, k, _ = eng.truncated_svd(M, cutoff * scale * scale, mode="chosen")
    ref = np.linalg.svd(th, compute_uv=False)
    assert k == ex.rank
    np.testing.assert_allclose(S[:k] / (scale * scale), ref[:k], rtol=1e-4, atol=1e-6 * ref[0])
    eng.close()


@pytest.mark.parametrize("chil,chir", [(96, 160), (160, 96)])
def test_sketch_path_on_rectangular_theta(engine, chil, chir):
    """The sketched split on a rectangular theta' (2 chiL x 2 chiR, both
    orientations): the row-space sketch, the tall C = theta' Y and the
    projection B' = A'^H theta' keep the exact rank and the truncation
    error within 1.1x of the exact SVD's."""
    rng = np.random.default_rng(chil + 3 * chir)
    chim = 48
    a = (rng.standard_normal((chil, 2, chim)) + 1j * rng.standard_normal((chil, 2, chim))) * 0.7 ** np.arange(chim)
    b = rng.standard_normal((chim, 2, chir)) + 1j * rng.standard_normal((chim, 2, chir))
    nrm = np.linalg.norm(O.theta_of(a, b))
    a /= np.sqrt(nrm)
    b /= np.sqrt(nrm)
    g = O.haar_unitary(rng)
    cutoff = 1e-3
    a64, b64 = a.astype(np.complex64).astype(complex), b.astype(np.complex64).astype(complex)
    ex = O.apply_2q([a64.copy(), b64.copy()], g, 1, cutoff, 0)
    eng = engine.Engine(mode="chosen")
    const_model(eng, min(1.0, 1.3 * ex.rank / (2 * min(chil, chir))))
    m = eng.mps([a.astype(np.complex64), b.astype(np.complex64)], dtype=np.complex64)
    st = m.apply_2q(g, 1, cutoff, 0)
    assert st["sketch_size"] > 0 and not st["fallback"], st
    assert st["rank"] == ex.rank, (st, ex.rank)
    th = exact_theta(a64, b64, g)
    approx = O.theta_of(m.site(1).astype(complex), m.site(2).astype(complex))
    err = np.linalg.norm(th - approx)
    assert err <= 1.1 * np.sqrt(ex.discarded_weight), (err, np.sqrt(ex.discarded_weight))
    A = m.site(1).reshape((2 * chil, -1), order="F").astype(complex)
    np.testing.assert_allclose(A.conj().T @ A, np.eye(A.shape[1]), atol=2e-5)
    m.free()
    eng.close()
