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


@pytest.mark.parametrize("ops", [("N", "N"), ("C", "N"), ("N", "C"), ("C", "C")])
@pytest.mark.parametrize("mnk", [(64, 32, 32), (2048, 32, 2048), (300, 257, 129), (1024, 1040, 2048),
                                 (2048, 2048, 64), (2048, 2048, 2048)])
def test_tc_gemm_ops_and_beta(tc, ops, mnk):
    """Every operand orientation the SVD path uses, with beta = 1 accumulation
    (the Gram-Schmidt projection update), up to 2048 in each dimension."""
    M, N, K = mnk
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rand_c64(rng, *((M, K) if ops[0] == "N" else (K, M)))
    B = rand_c64(rng, *((K, N) if ops[1] == "N" else (N, K)))
    C0 = rand_c64(rng, M, N)
    got = tc.gemm(A, B, ops[0], ops[1], alpha=-1.0, beta=1.0, out=C0)
    opa = A.astype(np.complex128) if ops[0] == "N" else A.astype(np.complex128).conj().T
    opb = B.astype(np.complex128) if ops[1] == "N" else B.astype(np.complex128).conj().T
    ref = C0.astype(np.complex128) - opa @ opb
    # split-TF32x3 with FP32 accumulation: a few 2^-21 relative per product,
    # growing like sqrt(K) over the sum (measured ~4e-6 sqrt(K) at unit entries)
    err = np.abs(got - ref).max() / np.sqrt(K)
    assert err <= 2e-5, err


@pytest.mark.parametrize("ops", [("N", "N"), ("C", "N"), ("N", "C")])
def test_fp64_gemm_ops(engine, ops):
    eng = engine.Engine(mode="plain")
    rng = np.random.default_rng(3)
    M, N, K = 130, 70, 90
    A = rng.standard_normal((M, K) if ops[0] == "N" else (K, M)) + 1j * rng.standard_normal((M, K) if ops[0] == "N" else (K, M))
    B = rng.standard_normal((K, N) if ops[1] == "N" else (N, K)) + 1j * rng.standard_normal((K, N) if ops[1] == "N" else (N, K))
    got = eng.gemm(A, B, ops[0], ops[1])
    opa = A if ops[0] == "N" else A.conj().T
    opb = B if ops[1] == "N" else B.conj().T
    assert np.abs(got - opa @ opb).max() <= 1e-13 * np.sqrt(K) * 4
    eng.close()
