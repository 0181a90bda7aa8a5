"""CPU model of the cluster CholeskyQR's schedule (cholqr_cluster_kernel in
k_rsvd.cu): the maps from threads to Gram tiles and entries, the ownership of
the cluster reduce-scatter, the rows each CTA stages, and the blocked 8-column
Cholesky and inverse with their register windows, clamped indices and
skipped pivots past b.  The model follows the kernel's index arithmetic
step by step (lanes as numpy vectors) and is checked against numpy's
Cholesky and inverse; entries the kernel never writes are NaN here, so any
read of them shows up."""
import numpy as np
import pytest

BW, TILES, E, GROUPS = 32, 36, 576, 7


def tile(T):
    ti, tj = T, 0
    while ti > tj:
        ti -= tj + 1
        tj += 1
    return ti, tj


def entry_ij(e):
    """Entry e = 36 (4 (i & 3) + (j & 3)) + tile of the stored Gram."""
    ti, tj = tile(e % TILES)
    k = e // TILES
    return 4 * ti + (k >> 2), 4 * tj + (k & 3)


def test_tiles_cover_the_upper_triangle_once():
    seen = np.zeros((BW, BW), int)
    for e in range(E):
        i, j = entry_ij(e)
        seen[i, j] += 1
    assert (seen[np.triu_indices(BW)] == 1).all()
    # the diagonal tiles also hold their lower entries, nothing else below
    low = np.tril(np.ones((BW, BW), bool), -1)
    blk = (np.arange(BW)[:, None] // 4) == (np.arange(BW)[None, :] // 4)
    assert (seen[low & ~blk] == 0).all() and (seen[low & blk] == 1).all()
    # thread t < 252 -> (row group t / 36, tile t % 36)
    assert sorted({(t // TILES, t % TILES) for t in range(GROUPS * TILES)}) == \
        [(g, T) for g in range(GROUPS) for T in range(TILES)]


@pytest.mark.parametrize("cs", [8, 16])
def test_reduce_scatter_owns_every_entry_once(cs):
    owned = np.zeros(E, int)
    for crank in range(cs):
        for t in range(256):
            e = crank + cs * t
            if e < E:
                owned[e] += 1
                assert e % cs == crank  # the gather reads rank e % cs
    assert (owned == 1).all()


def shape(m, cs):
    for nrb in (1, 2, 4, 8):
        if cs * 32 * nrb >= m:
            return nrb
    return 0


@pytest.mark.parametrize("m", [33, 256, 400, 1000, 2048, 4096])
@pytest.mark.parametrize("cs", [8, 16])
def test_rows_are_staged_once(m, cs):
    nrb = shape(m, cs)
    if nrb == 0:
        assert m > cs * 256
        return
    rows = 32 * nrb
    arows = (rows + GROUPS - 1) // GROUPS * GROUPS
    # warp w loads columns 4w .. 4w+3, lane l the rows l + 32 u of its CTA
    hit = np.zeros((m, BW), int)
    for crank in range(cs):
        for w in range(8):
            for cc in range(4):
                for lane in range(32):
                    for u in range(nrb):
                        r = crank * rows + lane + 32 * u
                        if r < m:
                            hit[r, 4 * w + cc] += 1
    assert (hit == 1).all()
    # the Gram's row groups read rows g + 7 q < arows (padding rows are zero)
    assert max(g + GROUPS * q for g in range(GROUPS) for q in range(arows // GROUPS)) == arows - 1


def blocked_cholesky_inverse(G, b, shift_tr=0.0):
    """The kernel's (E): R in place of the upper triangle, then X = R^{-1}."""
    Gl = np.full((BW, BW), np.nan, complex)
    iu = np.triu_indices(BW)
    Gl[iu] = G[iu]
    tr = np.sum(np.real(np.diag(G))[:b])
    for l in range(b):
        Gl[l, l] = G[l, l].real + shift_tr * tr
    Ry = np.zeros(BW)
    lanes = np.arange(32)
    for k0 in range(0, b, 8):
        col = k0 + lanes
        c = np.zeros((32, 8), complex)
        for r in range(8):
            ok = (col < BW) & (k0 + r <= col)
            c[ok, r] = Gl[k0 + r, col[ok]]
        dn = c[:, 0].real.copy()
        for kk in range(8):
            k = k0 + kk
            if k >= b:
                continue
            d = dn[kk]
            assert d > 0
            y = 1.0 / np.sqrt(d)
            rk = np.where(lanes == kk, d * y, np.where(lanes > kk, c[:, 0] * y, 0))
            dn = c[:, 1].real - np.abs(rk) ** 2
            ok = col < BW
            Gl[k, col[ok]] = rk[ok]
            Ry[k] = y
            for r in range(1, 8):
                rkr = rk[min(kk + r, 31)]
                c[:, r - 1] = c[:, r] - np.conj(rkr) * rk
        for w in range(8):
            for i in range(k0 + 8 + w, BW, 8):
                j = lanes[lanes >= i]
                v0 = Gl[i, j].copy()
                v1 = np.zeros_like(v0)
                for q in range(0, 8, 2):
                    v0 -= np.conj(Gl[k0 + q, i]) * Gl[k0 + q, j]
                    v1 -= np.conj(Gl[k0 + q + 1, i]) * Gl[k0 + q + 1, j]
                Gl[i, j] = v0 + v1
    Xs = np.full((BW, BW), np.nan, complex)
    for w in range(4):
        k0 = 8 * w
        for lane in range(8):
            x = np.zeros(8, complex)
            x[lane] = 1
            for kk in range(7, -1, -1):
                x[kk] *= Ry[k0 + kk]
                for i in range(kk):
                    x[i] -= Gl[k0 + i, k0 + kk] * x[kk]
            Xs[k0:k0 + 8, k0 + lane] = x
    for e in range(BW * BW):
        if (e // BW) // 8 > (e % BW) // 8:
            Xs[e // BW, e % BW] = 0
    for d in range(1, 4):
        Tb = {}
        for t in range(256):
            bi, a, cc = t // 64, (t // 8) % 8, t % 8
            bj = bi + d
            if bj < 4:
                i, j = 8 * bi + a, 8 * bj + cc
                Tb[t] = sum(Gl[i, l] * Xs[l, j] for l in range(8 * (bi + 1), 8 * (bj + 1)))
        for t in range(256):
            bi, a, cc = t // 64, (t // 8) % 8, t % 8
            bj = bi + d
            if bj < 4:
                i, j = 8 * bi + a, 8 * bj + cc
                Xs[i, j] = -sum(Xs[i, 8 * bi + q] * Tb[64 * bi + 8 * q + cc] for q in range(8))
    R = np.where(np.triu(np.ones((BW, BW), bool)), Gl, 0)
    return R, Xs


@pytest.mark.parametrize("b", [32, 29, 8, 7, 1])
def test_blocked_cholesky_and_inverse(b):
    rng = np.random.default_rng(b)
    Y = rng.standard_normal((96, BW)) + 1j * rng.standard_normal((96, BW))
    Y[:, b:] = 0  # a partial block: zero columns past b
    Y[:, :b] *= 0.7 ** np.arange(b)  # graded, as the sketch blocks are
    G = Y.conj().T @ Y
    R, X = blocked_cholesky_inverse(G, b)
    Rb = R[:b, :b]
    assert np.isfinite(R).all() and np.isfinite(X).all()
    np.testing.assert_allclose(Rb.conj().T @ Rb, G[:b, :b], atol=1e-12 * np.abs(G).max())
    np.testing.assert_allclose(Rb @ X[:b, :b], np.eye(b), atol=1e-9)
    assert (X[b:, :] == 0).all() and (X[:, b:][:b] == 0).all()
    np.testing.assert_allclose(np.abs(np.diag(Rb)), np.abs(np.diag(np.linalg.cholesky(G[:b, :b]).conj().T)),
                               rtol=1e-10)


def test_shifted_pass_factors_the_shifted_gram():
    rng = np.random.default_rng(3)
    Y = rng.standard_normal((64, BW)) + 1j * rng.standard_normal((64, BW))
    Y[:, 1] = Y[:, 0]  # exactly dependent: the shift keeps the pivots positive
    G = Y.conj().T @ Y
    shift = 11.0 * (64 * BW + BW * (BW + 1)) * 5.96e-8
    R, X = blocked_cholesky_inverse(G, BW, shift)
    Gs = G + shift * np.trace(G).real * np.eye(BW)
    np.testing.assert_allclose(R.conj().T @ R, Gs, atol=1e-12 * np.abs(Gs).max())
    np.testing.assert_allclose(R @ X, np.eye(BW), atol=1e-8)
