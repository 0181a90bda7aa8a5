"""GPU parity of the engine's plain FP64 path with the FP64 oracle (through the C ABI)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(engine):
    e = engine.Engine(mode="plain")
    yield e
    e.close()


def rand_c(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("shape", [(1, 1), (2, 1), (1, 3), (5, 3), (3, 5), (16, 16), (17, 33), (64, 40),
                                   (40, 64), (128, 128), (130, 70)])
def test_truncated_svd_matches_lapack(eng, shape):
    rng = np.random.default_rng(sum(shape))
    m = rand_c(rng, *shape)
    U, S, Vh, k, disc = eng.truncated_svd(m, 0.0)
    s_ref = np.linalg.svd(m, compute_uv=False)
    assert k == O.tail_rank(s_ref, 0.0)
    np.testing.assert_allclose(S, s_ref[:k], rtol=1e-12, atol=1e-13 * s_ref[0])
    np.testing.assert_allclose(U @ np.diag(S) @ Vh, m, atol=1e-12 * np.linalg.norm(m))
    np.testing.assert_allclose(U.conj().T @ U, np.eye(k), atol=1e-12)
    np.testing.assert_allclose(Vh @ Vh.conj().T, np.eye(k), atol=1e-12)


def test_truncated_svd_graded_spectrum_and_cutoff(eng):
    # singular values spanning 14 decades: absolute accuracy and the tail rule
    rng = np.random.default_rng(3)
    n = 96
    q1, _ = np.linalg.qr(rand_c(rng, n, n))
    q2, _ = np.linalg.qr(rand_c(rng, n, n))
    s = np.exp(-np.linspace(0, 32, n))
    m = (q1 * s) @ q2.conj().T
    for er in (0.0, 1e-12, 1e-10, 1e-6, 1e-2):
        U, S, Vh, k, disc = eng.truncated_svd(m, er)
        s_ref = O.svd_gesdd(m)[1]
        assert k == O.tail_rank(s_ref, er, clamp=True), er
        # two backward-stable SVDs agree to O(n eps ||m||)
        np.testing.assert_allclose(S, s_ref[:k], rtol=0, atol=n * 2.2e-16 * s_ref[0] * 4)


def test_truncated_svd_rank_deficient_exact_zeros(eng):
    rng = np.random.default_rng(4)
    a = rand_c(rng, 20, 3) @ rand_c(rng, 3, 12)
    U, S, Vh, k, _ = eng.truncated_svd(a, 0.0)
    np.testing.assert_allclose(U @ np.diag(S) @ Vh, a, atol=1e-12 * np.linalg.norm(a))
    assert k >= 3


@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
def test_contract_pair_matches_ncon(eng, dt):
    rng = np.random.default_rng(5)
    A = rand_c(rng, 3, 4, 5).astype(dt)
    B = rand_c(rng, 5, 2, 4).astype(dt)
    got = eng.contract_pair(A, B, [1, 2], [2, 0])
    ref = np.tensordot(A.astype(np.complex128), B.astype(np.complex128), axes=([1, 2], [2, 0]))
    tol = 1e-12 if dt == np.complex128 else 1e-5
    np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.abs(ref).max())


def test_contract_svd_reference_cases(eng):
    # test/test_svd.jl:8-25 through the engine
    rng = np.random.default_rng(6)
    t1, t2 = rand_c(rng, 4, 4), rand_c(rng, 4, 4)
    np.testing.assert_allclose(eng.contract_svd(t1, t2, (2, 1)), t1 @ t2, rtol=1e-10)
    t1, t2 = rand_c(rng, 2, 3, 4, 6), rand_c(rng, 1, 5, 2, 4)
    np.testing.assert_allclose(eng.contract_svd(t1, t2, (1, 3)), O.contract_svd(t1, t2, (1, 3)), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(eng.contract_svd(t1, t2, (3, 4)), O.contract_svd(t1, t2, (3, 4)), rtol=1e-10, atol=1e-12)
    with pytest.raises(ValueError, match="^Error must be positive$"):
        eng.contract_svd(t1, t2, (1, 3), er=-0.3)
    with pytest.raises(ValueError, match="^Dimensions of contraction legs do not match$"):
        eng.contract_svd(t1, rand_c(rng, 8, 8), (1, 3))


@pytest.mark.parametrize("chis", [(1, 1, 1), (1, 2, 2), (3, 5, 4), (8, 8, 8), (16, 9, 33), (37, 64, 29), (64, 64, 64)])
def test_apply_2q_matches_oracle(eng, chis):
    cl, cm, cr = chis
    rng = np.random.default_rng(cl * 1000 + cm * 10 + cr)
    a, b = rand_c(rng, cl, 2, cm), rand_c(rng, cm, 2, cr)
    g = O.haar_unitary(rng)
    for cutoff, chi_max in ((0.0, 0), (1e-1, 0), (0.0, max(1, min(cl, cr)))):
        mps = eng.mps([a, b])
        st = mps.apply_2q(g, 1, cutoff, chi_max)
        sites = [a.copy(), b.copy()]
        ref = O.apply_2q(sites, g, 1, cutoff, chi_max)
        assert st["rank"] == ref.rank and st["rank_cutoff"] == ref.rank_cutoff
        np.testing.assert_allclose(st["discarded_weight"], ref.discarded_weight, rtol=1e-9, atol=1e-14 * ref.norm2)
        got = O.theta_of(mps.site(1), mps.site(2))
        np.testing.assert_allclose(got, O.theta_of(*sites), atol=1e-11 * np.sqrt(ref.norm2))
        A2 = mps.site(1).reshape((2 * cl, -1), order="F")
        np.testing.assert_allclose(A2.conj().T @ A2, np.eye(A2.shape[1]), atol=1e-12)
        mps.free()


def test_brickwork_12_qubits_parity_and_dense(eng):
    # 12-qubit brickwork of depth 8, Haar gates, cutoff 1e-10, chi_max 32
    rng = np.random.default_rng(2024)
    n, depth, cutoff, chi_max = 12, 8, 1e-10, 32
    gates = O.brickwork_gates(n, depth, rng)
    mps = eng.product_state(n)
    ranks = [mps.apply_2q(g, w, cutoff, chi_max)["rank"] for (_, w, g) in gates]
    sites, stats = O.run_brickwork(n, gates, cutoff, chi_max)
    assert ranks == [s.rank for s in stats]
    for i in (1, 6, 12):
        z, zr = mps.expect_z(i), O.expect_z(sites, i)
        assert abs(z - zr) <= 1e-10 * max(abs(zr), 1e-3), (i, z, zr)
    zz, zzr = mps.expect_zz(5), O.expect_zz(sites, 5)
    assert abs(zz - zzr) <= 1e-10 * max(abs(zzr), 1e-3)
    psi = O.mps_to_state(mps.sites())
    np.testing.assert_allclose(psi, O.mps_to_state(sites), atol=1e-10)


def test_switch_matches_reference_permutation(eng):
    # test/test_mps.jl:253-273 (switch neighbouring qubits) through the engine
    rng = np.random.default_rng(8)
    b = [rand_c(rng, 2) for _ in range(6)]
    psi = b[0]
    for v in b[1:]:
        psi = np.kron(psi, v)
    ref_mps = O.mps_from_state(psi)
    mps = eng.mps(ref_mps.tensors)
    for i in (4, 3, 2, 1):
        mps.switch(i)
    order = [1, 3, 4, 5, 6, 2]
    perm = b[order[0] - 1]
    for o in order[1:]:
        perm = np.kron(perm, b[o - 1])
    np.testing.assert_allclose(O.mps_to_state(mps.sites()), perm, atol=1e-12 * np.linalg.norm(perm))


def test_errors_are_reported(eng, engine):
    mps = eng.product_state(3)
    g = np.eye(4)
    with pytest.raises(engine.QaintensorBoundsError):
        mps.apply_2q(g, 3, 0.0, 0)
    bad = np.eye(4, dtype=complex)
    bad[0, 0] = np.nan
    with pytest.raises(engine.EngineError):
        mps.apply_2q(bad, 1, 0.0, 0)


@pytest.mark.parametrize("chi", [256, 1024])
def test_plain_single_bond_sweep_matches_oracle(eng, chi):
    # the single-bond workload in complex128 (theta = Q1 diag(0.97^k) Q2^H,
    # Haar gate, truncation back to chi) in plain mode against the oracle's
    # update (src/switch.jl:26-54 split, src/svd.jl:29-33 rule): identical
    # ranks, and theta' rebuilt from the new sites within 1e-10 ||theta'||
    rng = np.random.default_rng(7 + chi)
    a, b, _ = O.decay_theta_factors(chi, rng)
    g = O.haar_unitary(rng)
    cutoff = 1e-10
    mps = eng.mps([a, b])
    st = mps.apply_2q(g, 1, cutoff, chi)
    sites = [a.copy(), b.copy()]
    ref = O.apply_2q(sites, g, 1, cutoff, chi)
    tail = np.sqrt(np.cumsum(ref.spectrum[::-1] ** 2))[::-1]
    near = np.abs(tail / cutoff - 1.0).min()  # a tie of the tail rule would show here
    assert st["rank"] == ref.rank, (st, ref.rank, near)
    assert st["rank_cutoff"] == ref.rank_cutoff, (st, ref.rank_cutoff, near)
    np.testing.assert_allclose(st["discarded_weight"], ref.discarded_weight, rtol=1e-9)
    got = O.theta_of(mps.site(1), mps.site(2))
    want = O.theta_of(*sites)
    assert np.linalg.norm(got - want) <= 1e-10 * np.sqrt(ref.norm2)
    mps.free()


def test_chosen_single_bond_at_chi_64_complex64(engine):
    # the same workload at chi = 64 in complex64, chosen mode: the exact rank
    # and a truncation error within 1.1x of the exact FP64 split's
    rng = np.random.default_rng(71)
    chi = 64
    a, b, _ = O.decay_theta_factors(chi, rng)
    g = O.haar_unitary(rng)
    a32, b32 = a.astype(np.complex64), b.astype(np.complex64)
    ex = O.apply_2q([a32.astype(complex), b32.astype(complex)], g, 1, 1e-10, chi)
    ch = engine.Engine(mode="chosen", tc_gemm=1)
    m = ch.mps([a32, b32], dtype=np.complex64)
    st = m.apply_2q(g, 1, 1e-10, chi)
    assert st["rank"] == ex.rank == chi
    th = O.apply_gate_to_theta(O.theta_of(a32.astype(complex), b32.astype(complex)), g, chi, chi)
    err = np.linalg.norm(th - O.theta_of(m.site(1).astype(complex), m.site(2).astype(complex)))
    assert err <= 1.1 * np.sqrt(ex.discarded_weight), (err, np.sqrt(ex.discarded_weight))
    m.free()
    ch.close()
