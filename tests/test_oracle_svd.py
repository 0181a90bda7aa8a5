"""Oracle pins ported from test/test_svd.jl (contract_svd, its errors, truncation bound)."""
import numpy as np
import pytest

import oracle as O

RTOL = np.sqrt(np.finfo(float).eps)  # Julia's default isapprox rtol


def rand_c(rng, *shape):
    return rng.random(shape) + 1j * rng.random(shape)


def test_contract_svd_matrix_product():
    # test/test_svd.jl:8-11
    rng = np.random.default_rng(11)
    t1, t2 = rand_c(rng, 4, 4), rand_c(rng, 4, 4)
    np.testing.assert_allclose(O.contract_svd(t1, t2, (2, 1)), t1 @ t2, rtol=RTOL)


def test_contract_svd_rank4_open_leg_order():
    # test/test_svd.jl:13-25
    rng = np.random.default_rng(12)
    t1, t2 = rand_c(rng, 2, 3, 4, 6), rand_c(rng, 1, 5, 2, 4)
    con1 = O.Summation([(1, 1), (2, 3)])
    con2 = O.Summation([(1, 3), (2, 4)])
    open1 = [(1, 2), (1, 3), (1, 4), (2, 1), (2, 2), (2, 4)]
    open2 = [(1, 1), (1, 2), (1, 4), (2, 1), (2, 2), (2, 3)]
    tn1 = O.Network([t1, t2], [con1], open1)
    tn2 = O.Network([t1, t2], [con2], open2)
    np.testing.assert_allclose(O.contract(tn1), O.contract_svd(t1, t2, (1, 3)), rtol=RTOL, atol=1e-13)
    np.testing.assert_allclose(O.contract(tn2), O.contract_svd(t1, t2, (3, 4)), rtol=RTOL, atol=1e-13)


def test_contract_svd_exceptions():
    # test/test_svd.jl:28-50
    rng = np.random.default_rng(13)
    t1, t2 = rand_c(rng, 2, 3, 4, 2), rand_c(rng, 1, 5, 2, 4)
    with pytest.raises(O.QaintensorError, match="^Error must be positive$"):
        O.contract_svd(t1, t2, (1, 3), er=-0.3)
    t2_short = rand_c(rng, 8, 8)
    # Julia's size(A, 3) of a matrix is 1, so the legs (2 vs 1) mismatch
    with pytest.raises(O.QaintensorError, match="^Dimensions of contraction legs do not match$"):
        O.contract_svd(t1, t2_short, (1, 3))
    con2 = O.Summation([(1, 3), (2, 4)])
    open2 = [(1, 1), (1, 2), (1, 4), (2, 1), (2, 2), (2, 3)]
    np.testing.assert_allclose(O.contract(O.Network([t1, t2], [con2], open2)),
                               O.contract_svd(t1, t2, (3, 4)), rtol=RTOL, atol=1e-13)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_contract_svd_truncation_bound(seed):
    # test/test_svd.jl:53-83 (seeded)
    rng = np.random.default_rng(seed)
    s = np.exp(-np.arange(100.0))
    u1, _ = np.linalg.qr(rng.random((100, 100)))
    v1, _ = np.linalg.qr(rng.random((100, 100)))
    u2, _ = np.linalg.qr(rng.random((100, 100)))
    v2, _ = np.linalg.qr(rng.random((100, 100)))
    T1 = u1 @ np.diag(s) @ v1
    T2 = u2 @ np.diag(s) @ v2
    er = 1e-10
    mps = O.ClosedMPS([T1, T2])
    psi_approx = O.contract_svd_mps(mps, er=er)
    psi = O.contract(mps)
    k = O.tail_rank(s, er)
    n = np.linalg.norm(s)
    nt = np.linalg.norm(s[k:])
    assert np.linalg.norm(psi_approx - psi) < 2 * n * nt + nt ** 2


def test_tail_rank_rule_edges():
    # src/svd.jl:29-33: strict '>' on the sqrt of the reversed cumulative sum
    s = np.array([1.0, 0.5, 0.0, 0.0])
    assert O.tail_rank(s, 0.0) == 2          # exact zeros dropped at er = 0
    assert O.tail_rank(s, 0.5) == 1          # tail sqrt(0.25) = 0.5 is not > 0.5
    assert O.tail_rank(s, 0.49) == 2
    with pytest.raises(O.QaintensorError):
        O.tail_rank(s, 2.0)                  # findfirst -> nothing in the reference
    assert O.tail_rank(s, 2.0, clamp=True) == 1
