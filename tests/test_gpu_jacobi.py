"""One-sided block Jacobi SVD against LAPACK on graded spectra, in FP64 and
FP32 storage, for every round implementation: the one-launch cluster round
(pair rows held in the shared memory of 1, 2, 4 or 8 CTAs), the three-kernel
round, and for FP32 the cooperative sweep kernel (jacobi_kernel 0, one launch
per sweep) and the two-launch round (3)."""

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def crandn(rng, *shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def graded(rng, m, n, decay):
    k = min(m, n)
    q1, _ = np.linalg.qr(crandn(rng, m, k))
    q2, _ = np.linalg.qr(crandn(rng, n, k))
    s = decay ** np.arange(k, dtype=np.float64)
    return (q1 * s) @ q2.conj().T, s


# shapes covering cluster sizes 1..8 of the FP64 round (rows per CTA <= ~390)
# and 1..4 of the FP32 round, column counts not a multiple of the 8-column
# block, tall and wide
SHAPES = [(40, 24), (24, 40), (300, 201), (701, 513), (1100, 1003), (1536, 1536)]


@pytest.mark.parametrize("kernel", [0, 1, 2])
@pytest.mark.parametrize("shape", SHAPES)
def test_fp64_jacobi_matches_lapack(engine, shape, kernel):
    rng = np.random.default_rng(sum(shape) + kernel)
    m, n = shape
    M, _ = graded(rng, m, n, 0.985)
    eng = engine.Engine(mode="plain", jacobi_kernel=kernel)
    U, S, Vh, k, _ = eng.truncated_svd(M, 0.0)
    ref = np.linalg.svd(M, compute_uv=False)
    assert k == min(m, n)
    # M itself is known to ~u ||M|| (it is a rounded product), so the values
    # agree with LAPACK's to a multiple of that, not relatively
    assert np.abs(S - ref).max() <= 1e-12 * ref[0], np.abs(S - ref).max()
    assert np.linalg.norm((U * S) @ Vh - M) <= 1e-12 * np.sqrt(max(m, n)) * np.linalg.norm(M)
    assert np.abs(U.conj().T @ U - np.eye(k)).max() <= 1e-11
    eng.close()


@pytest.mark.parametrize("kernel", [0, 1, 2, 3])
@pytest.mark.parametrize("shape", SHAPES)
def test_fp32_jacobi_matches_lapack(engine, shape, kernel):
    rng = np.random.default_rng(7 * sum(shape) + kernel)
    m, n = shape
    M, _ = graded(rng, m, n, 0.97)
    M32 = M.astype(np.complex64)
    ref = np.linalg.svd(M32.astype(np.complex128), compute_uv=False)
    nrm = np.linalg.norm(ref)
    floor = 4 * np.sqrt(max(m, n)) * 5.96e-8 * nrm  # the chosen-mode noise floor
    tail = np.sqrt(np.cumsum(ref[::-1] ** 2))[::-1]

    def rank_at(cut):
        return int(np.argmax(np.append(tail[1:], 0.0) <= cut)) + 1

    eng = engine.Engine(mode="chosen", jacobi_kernel=kernel)
    # a cutoff well above the floor: the exact rank (+-1 at a tie)
    cut = 50 * floor
    U, S, Vh, k, _ = eng.truncated_svd(M32, cut, mode="chosen")
    assert abs(k - rank_at(cut)) <= 1, (k, rank_at(cut))
    err = np.linalg.norm((U * S) @ Vh - M32)
    assert err <= 1.1 * np.sqrt(np.sum(ref[k:] ** 2)) + floor, (err, floor)
    # FP32 storage: values to ~sqrt(rows) u_fp32 of ||M|| absolutely
    assert np.abs(S[:k] - ref[:k]).max() <= 2 * floor, (np.abs(S[:k] - ref[:k]).max(), floor)
    # one Newton-Schulz step leaves the left factor orthonormal to FP32 rounding
    assert np.abs(U.conj().T @ U - np.eye(k)).max() <= 2e-6 * np.sqrt(m)
    # cutoff 0 lies below the FP32 resolution and nothing certifies the rank
    # (no cap, no rank bound for a bare matrix): the exact FP64 split of the
    # same complex64 input decides, with LAPACK's rank and values
    c0 = eng.cert_counters()
    U, S, Vh, k, _ = eng.truncated_svd(M32, 0.0, mode="chosen")
    assert eng.cert_counters()["fallback"] == c0["fallback"] + 1
    assert k == rank_at(0.0), (k, rank_at(0.0))
    assert np.abs(S[:k] - ref[:k]).max() <= 1e-12 * ref[0]
    eng.close()


def test_one_launch_round_equals_three_kernel_round_fp64(engine):
    """The two round implementations reach the same factorisation to FP64
    accuracy on one matrix (different summation orders, same fixed point)."""
    rng = np.random.default_rng(11)
    M, _ = graded(rng, 512, 384, 0.98)
    out = []
    for kernel in (0, 1):
        eng = engine.Engine(mode="plain", jacobi_kernel=kernel)
        out.append(eng.truncated_svd(M, 1e-9))
        eng.close()
    (U0, S0, V0, k0, d0), (U1, S1, V1, k1, d1) = out
    assert k0 == k1
    assert np.abs(S0 - S1).max() <= 1e-13 * S0[0] * 384
    assert np.linalg.norm((U0 * S0) @ V0 - (U1 * S1) @ V1) <= 1e-11 * np.linalg.norm(M)


@pytest.mark.parametrize("chi", [256, 1024])
def test_fp32_split_of_rank_deficient_theta(engine, chi):
    """theta' = G (A.B) with a 0.97^k spectrum: half of its values at chi = 1024
    lie below FP32 resolution.  The FP32 split must still reproduce the exact
    truncation to chi (error within 1.1x, unit left factor to FP32 level)."""
    import oracle as O
    rng = np.random.default_rng(chi)
    a, b, _ = O.decay_theta_factors(chi, rng, 0.97)
    g = O.haar_unitary(rng)
    th = O.apply_gate_to_theta(O.theta_of(a.astype(np.complex64).astype(complex), b.astype(np.complex64).astype(complex)),
                               g, chi, chi).astype(np.complex64)
    ref = np.linalg.svd(th.astype(complex), compute_uv=False)
    exact = np.sqrt(np.sum(ref[chi:] ** 2))
    eng = engine.Engine(mode="chosen", tc_gemm=1)
    U, S, Vh, k, _ = eng.truncated_svd(th, 1e-6, chi_max=chi, mode="chosen")
    assert k == chi
    err = np.linalg.norm((U * S) @ Vh - th.astype(complex))
    assert err <= 1.1 * exact, (err, exact)
    assert np.abs(U.conj().T @ U - np.eye(k)).max() <= 1e-4
    assert np.abs(S[:k] - ref[:k]).max() <= 1e-4 * ref[0]
    eng.close()


@pytest.mark.parametrize("shape", [(1100, 1003), (333, 517)])
def test_sweep_kernel_equals_two_launch_round_fp32(engine, shape):
    """The cooperative sweep kernel (rotation folded into the next round's
    Gram, ping-pong buffers, per-pair round flags) and the two-launch round
    reach the same truncation: same rank, values within the FP32 floor."""
    rng = np.random.default_rng(sum(shape))
    m, n = shape
    M, _ = graded(rng, m, n, 0.97)
    M32 = M.astype(np.complex64)
    floor = 4 * np.sqrt(max(m, n)) * 5.96e-8 * np.linalg.norm(M32)
    out = []
    for kernel in (0, 3):
        eng = engine.Engine(mode="chosen", jacobi_kernel=kernel)
        out.append(eng.truncated_svd(M32, 50 * floor, mode="chosen"))
        eng.close()
    (U0, S0, V0, k0, _), (U1, S1, V1, k1, _) = out
    assert abs(k0 - k1) <= 1
    k = min(k0, k1)
    assert np.abs(S0[:k] - S1[:k]).max() <= 2 * floor
    ref = np.linalg.svd(M32.astype(np.complex128), compute_uv=False)
    for U, S, Vh, kk in ((U0, S0, V0, k0), (U1, S1, V1, k1)):
        err = np.linalg.norm((U * S) @ Vh - M32)
        assert err <= 1.1 * np.sqrt(np.sum(ref[kk:] ** 2)) + floor, (err, floor)


# the orthonormalisations of an FP32 sketch: (QT_ORTH_ONE_LAUNCH, QT_CHOLQR_CLUSTER)
ORTH_VARIANTS = {"one-launch": ("1", "1"), "cluster16": ("0", "1"), "cluster8": ("0", "8"), "four-kernel": ("0", "0")}


def capped_update(engine, a, b, g, chi, env, monkeypatch):
    """One chosen-mode update of the bond (a, b) at the chi_max = chi cap (the
    sketched split) under the given environment; returns (stats, site 1, site 2)."""
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    eng = engine.Engine(mode="chosen", tc_gemm=1)
    # a rank model predicting the cap: the update is cap-bound and sketched
    p = np.zeros(eng.n_params, dtype=np.float32)
    p[-1] = 1.0
    eng.set_rank_params(p, enable=True)
    m = eng.mps([a.astype(np.complex64), b.astype(np.complex64)], dtype=np.complex64)
    st = m.apply_2q(g, 1, 1e-6, chi)
    out = (st, m.site(1).astype(complex), m.site(2).astype(complex))
    m.free()
    eng.close()
    return out


@pytest.mark.parametrize("chi", [200, 512, 1024])
def test_orthonormalisations_give_the_same_truncation(engine, monkeypatch, chi):
    """The sketch bases of a capped update orthonormalised in one cooperative
    launch (16 rows per CTA in shared memory, grid barriers between the
    Gram-Schmidt phases), by the cluster CholeskyQR per block (the block's
    rows in the shared memory of 16 CTAs, or of 8) with the three projection
    kernels, and by the four-kernel passes: the same rank, truncation errors
    within 1.1x of the exact SVD's, unit left factors, kept values within
    1e-4 of the largest.  chi = 200 sketches 264 columns (a last block of 8)
    over 400 rows (the last CTA's rows padded)."""
    rng = np.random.default_rng(5 * chi)
    a, b, _ = O.decay_theta_factors(chi, rng, 0.97)
    g = O.haar_unitary(rng)
    a64, b64 = a.astype(np.complex64).astype(complex), b.astype(np.complex64).astype(complex)
    th = O.apply_gate_to_theta(O.theta_of(a64, b64), g, chi, chi)
    ref = np.linalg.svd(th, compute_uv=False)
    exact = np.sqrt(np.sum(ref[chi:] ** 2))
    out = {}
    for name, (one, cluster) in ORTH_VARIANTS.items():
        if chi == 1024 and name == "four-kernel":
            continue  # the slowest variant adds nothing at this size
        st, s1, s2 = capped_update(engine, a, b, g, chi, {"QT_ORTH_ONE_LAUNCH": one, "QT_CHOLQR_CLUSTER": cluster},
                                   monkeypatch)
        assert st["sketch_size"] > 0 and not st["fallback"] and st["rank"] == chi, (name, st)
        err = np.linalg.norm(th - O.theta_of(s1, s2))
        assert err <= 1.1 * exact, (name, err, exact)
        A = s1.reshape((2 * chi, -1), order="F")
        # one Newton-Schulz step on FP32 columns, half of them below FP32
        # resolution at chi = 1024: orthonormal to ~1e-4 there
        assert np.abs(A.conj().T @ A - np.eye(chi)).max() <= 4e-6 * np.sqrt(2 * chi), name
        out[name] = np.linalg.norm(s2.reshape((chi, -1), order="F"), axis=1)
    for name, sv in out.items():
        assert np.abs(out["one-launch"] - sv).max() <= 1e-4 * ref[0], name


def test_one_launch_orthonormalisation_is_reproducible(engine, monkeypatch):
    """Fixed summation orders: two capped updates of the same bond give the
    same sites bit for bit."""
    rng = np.random.default_rng(77)
    a, b, _ = O.decay_theta_factors(256, rng, 0.97)
    g = O.haar_unitary(rng)
    r0 = capped_update(engine, a, b, g, 256, {}, monkeypatch)
    r1 = capped_update(engine, a, b, g, 256, {}, monkeypatch)
    assert r0[0]["sketch_size"] > 0 and r0[0]["rank"] == r1[0]["rank"]
    assert np.array_equal(r0[1], r1[1]) and np.array_equal(r0[2], r1[2])


@pytest.mark.parametrize("shape", [(2048, 1152), (1100, 1003), (700, 1400)])
def test_sweep_kernel_row_halves_equal_one_cta_per_pair(engine, monkeypatch, shape):
    """Two CTAs per pair (each holding half of the rows, the pair's partial
    Grams exchanged every round) against one CTA per pair
    (QT_JACOBI_HALVES=1): the same truncation -- rank, values within the
    FP32 floor, errors within 1.1x of the exact SVD's."""
    rng = np.random.default_rng(3 * sum(shape))
    m, n = shape
    M, _ = graded(rng, m, n, 0.97)
    M32 = M.astype(np.complex64)
    floor = 4 * np.sqrt(max(m, n)) * 5.96e-8 * np.linalg.norm(M32)
    ref = np.linalg.svd(M32.astype(np.complex128), compute_uv=False)
    out = []
    for halves in ("1", "2"):
        monkeypatch.setenv("QT_JACOBI_HALVES", halves)
        eng = engine.Engine(mode="chosen", jacobi_kernel=0)
        out.append(eng.truncated_svd(M32, 50 * floor, mode="chosen"))
        eng.close()
    (U0, S0, V0, k0, _), (U1, S1, V1, k1, _) = out
    assert abs(k0 - k1) <= 1
    k = min(k0, k1)
    assert np.abs(S0[:k] - S1[:k]).max() <= 2 * floor
    for U, S, Vh, kk in ((U0, S0, V0, k0), (U1, S1, V1, k1)):
        err = np.linalg.norm((U * S) @ Vh - M32)
        assert err <= 1.1 * np.sqrt(np.sum(ref[kk:] ** 2)) + floor, (err, floor)
        assert np.abs(U.conj().T @ U - np.eye(kk)).max() <= 2e-6 * np.sqrt(m)


@pytest.mark.parametrize("shape,halves", [((2048, 1152), "2"), ((1024, 1536), "2"), ((1024, 1536), "1")])
def test_sweep_kernel_is_reproducible(engine, monkeypatch, shape, halves):
    """Two chosen-mode splits of the same matrix give the same factors bit
    for bit: the round protocol has no race (a tall matrix, whose Jacobi
    carries no V and runs two CTAs per pair, and a wide one, whose right
    factor V the rounds rotate too)."""
    monkeypatch.setenv("QT_JACOBI_HALVES", halves)
    rng = np.random.default_rng(sum(shape))
    m, n = shape
    M, _ = graded(rng, m, n, 0.995)
    M32 = M.astype(np.complex64)
    outs = []
    for _ in range(2):
        eng = engine.Engine(mode="chosen", jacobi_kernel=0)
        outs.append(eng.truncated_svd(M32, 1e-6, chi_max=min(m, n) // 2, mode="chosen"))
        eng.close()
    (U0, S0, V0, k0, _), (U1, S1, V1, k1, _) = outs
    assert k0 == k1
    assert np.array_equal(S0, S1) and np.array_equal(U0, U1) and np.array_equal(V0, V1)


@pytest.mark.parametrize("shape", [(2, 600), (8, 600), (31, 1024), (40, 600)])
def test_two_cta_rounds_with_a_short_v(engine, monkeypatch, shape):
    """A wide matrix whose right factor V has fewer rows than the 32-row
    granule of the row split (the small splits at the ends of an MPS
    compression): half 0 owns all of V's rows and half 1 none, and the split
    matches LAPACK and the one-CTA rounds."""
    rng = np.random.default_rng(sum(shape))
    m, n = shape
    M, _ = graded(rng, m, n, 0.9)
    M32 = M.astype(np.complex64)
    ref = np.linalg.svd(M32.astype(np.complex128), compute_uv=False)
    floor = 4 * np.sqrt(max(m, n)) * 5.96e-8 * np.linalg.norm(M32)
    out = []
    for halves in ("2", "1"):
        monkeypatch.setenv("QT_JACOBI_HALVES", halves)
        eng = engine.Engine(mode="chosen", jacobi_kernel=0)
        U, S, Vh, k, _ = eng.truncated_svd(M32, 50 * floor, mode="chosen")
        eng.close()
        err = np.linalg.norm((U * S) @ Vh - M32)
        assert err <= 1.1 * np.sqrt(np.sum(ref[k:] ** 2)) + floor, (halves, err, floor)
        assert np.abs(S[:k] - ref[:k]).max() <= 2 * floor, halves
        assert np.abs(U.conj().T @ U - np.eye(k)).max() <= 2e-6 * np.sqrt(max(m, n)), halves
        out.append((k, S))
    assert out[0][0] == out[1][0]
