"""The tcgen05 split-TF32x3 complex GEMM against FP64 numpy, and the chosen
update running its products on the tensor cores."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tc(engine):
    e = engine.Engine(mode="chosen", tc_gemm=1)
    yield e
    e.close()


def rand_c64(rng, *shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize("mnk", [(128, 64, 32), (200, 100, 70), (300, 257, 129), (1024, 512, 256), (64, 32, 32)])
def test_tc_gemm_matches_fp64(tc, mnk):
    M, N, K = mnk
    rng = np.random.default_rng(M + N + K)
    A, B = rand_c64(rng, M, K), rand_c64(rng, K, N)
    got = tc.contract_pair(A, B, [1], [0])
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    # split-TF32x3 with FP32 accumulation: FP32-level error, ~2^-22 sqrt(K) |A||B|
    bound = 4e-7 * np.sqrt(K) * np.abs(A).max() * np.abs(B).max() * np.sqrt(K)
    assert np.abs(got - ref).max() <= bound, (np.abs(got - ref).max(), bound)


def test_tc_chosen_update_matches_exact_truncation(engine):
    rng = np.random.default_rng(21)
    chi = 128
    a, b, s = O.decay_theta_factors(chi, rng, decay=0.6)
    g = O.haar_unitary(rng)
    cutoff = 1e-3
    ex = O.apply_2q([a.copy(), b.copy()], g, 1, cutoff, 0)
    eng = engine.Engine(mode="chosen", tc_gemm=1)
    p = np.zeros(eng.n_params, dtype=np.float32)
    p[-1] = min(1.0, 1.3 * ex.rank / (2 * chi))
    eng.set_rank_params(p, enable=True)
    m = eng.mps([a.astype(np.complex64), b.astype(np.complex64)], dtype=np.complex64)
    st = m.apply_2q(g, 1, cutoff, 0)
    assert st["sketch_size"] > 0 and not st["fallback"] and st["rank"] == ex.rank, (st, ex.rank)
    th = O.apply_gate_to_theta(O.theta_of(a.astype(np.complex64).astype(complex), b.astype(np.complex64).astype(complex)),
                               g, chi, chi)
    err = np.linalg.norm(th - O.theta_of(m.site(1).astype(complex), m.site(2).astype(complex)))
    assert err <= 1.1 * np.sqrt(ex.discarded_weight)
    m.free()
    eng.close()
