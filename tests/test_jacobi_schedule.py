"""Host-side model of the FP32 Jacobi sweep kernel's round protocol
(jacobi_sweep32_kernel in qaintensor.jl_gb300/csrc/k_jacobi.cu).

CTA q owns table q of every round of the circle tournament.  Round g rebuilds
its two blocks from round g-1's columns (buffer (g-1)&1) and unitaries (slot
(g-1)&1), writes them to buffer g&1 and its own unitary to slot g&1, then
publishes done[q] = g.  Before round g it waits until done[] >= g-1 for six
CTAs: the two round g-1 pairs that held its blocks (read after write), the
round g-1 readers of its blocks' round g-2 columns and the round g-1 readers
of unitary slot q of round g-2 (write after read).

The model runs every CTA as three steps (wait+read, write, publish)
interleaved in random orders and checks that each read sees the intended
version, that no write hits a location another CTA is still reading, that no
schedule deadlocks, and that the ping-pong rebuild applies the same products
as rotating the pairs in place round after round."""

import random

import numpy as np
import pytest

JW = 8


def tournament(r, q, n):
    if q == 0:
        a, b = r % (n - 1), n - 1
    else:
        a, b = (r + q) % (n - 1), (r - q + (n - 1)) % (n - 1)
    return (a, b) if a < b else (b, a)


def pair_of(r, blk, n):
    """Table and side of block blk in round r (the kernel's pair_of)."""
    if blk == n - 1:
        return 0, 1
    rr = r % (n - 1)
    if blk == rr:
        return 0, 0
    d = (blk - rr + (n - 1)) % (n - 1)
    if d <= n // 2 - 1:
        q, partner = d, (rr - d + (n - 1)) % (n - 1)
    else:
        q, partner = n - 1 - d, (rr + n - 1 - d) % (n - 1)
    return q, (1 if blk > partner else 0)


def inner_partner(ir, y, n=16):
    """The pair solver's partner of column y in inner round ir (the circle
    tournament over the pair's 16 columns)."""
    if y == n - 1:
        return ir
    if y == ir:
        return n - 1
    return (2 * ir - y + (n - 1)) % (n - 1)


def wait_targets(g, r, q, nb):
    R = nb - 1
    if g == 0:
        return []
    rp, rpp = (r - 1) % R, (r - 2) % R
    bi, bj = tournament(r, q, nb)
    t = [pair_of(rp, b, nb)[0] for b in (bi, bj)]
    if g >= 2:
        for b in (bi, bj):
            qq, _ = pair_of(rpp, b, nb)
            a2, b2 = tournament(rpp, qq, nb)
            t.append(pair_of(rp, b2 if a2 == b else a2, nb)[0])
        for b in tournament(rpp, q, nb):
            t.append(pair_of(rp, b, nb)[0])
    return t


@pytest.mark.parametrize("n", [2, 4, 6, 16, 34, 256])
def test_inverse_tournament(n):
    for r in range(n - 1):
        seen = set()
        for q in range(n // 2):
            a, b = tournament(r, q, n)
            assert pair_of(r, a, n) == (q, 0) and pair_of(r, b, n) == (q, 1)
            seen |= {a, b}
        assert seen == set(range(n))


def test_inner_partner_is_the_16_column_tournament():
    for ir in range(15):
        for q in range(8):
            a, b = tournament(ir, q, 16)
            assert inner_partner(ir, a) == b and inner_partner(ir, b) == a


def run_schedule(nb, sweeps, seed):
    rnd = random.Random(seed)
    P, R = nb // 2, nb - 1
    G = sweeps * R
    buf = [{b: 0 for b in range(nb)}, {b: -1 for b in range(nb)}]
    wslot = [[-1] * P, [-1] * P]
    done = [-1] * P
    state = [(0, "A")] * P
    active, reads_of = {}, {}
    sweep_end = R  # one launch per sweep: a kernel boundary every R rounds
    while True:
        cand = []
        for q in range(P):
            g, st = state[q]
            if g >= min(G, sweep_end):
                continue
            if st != "A" or all(done[t] >= g - 1 for t in wait_targets(g, g % R, q, nb)):
                cand.append(q)
        if not cand:
            if any(state[q][0] < G for q in range(P)):
                assert all(state[q][0] == sweep_end for q in range(P)), "deadlock"
                sweep_end += R
                continue
            break
        q = rnd.choice(cand)
        g, st = state[q]
        r = g % R
        bi, bj = tournament(r, q, nb)
        if st == "A":
            locs = []
            for b in (bi, bj):
                if g > 0:
                    qq, _ = pair_of((r - 1) % R, b, nb)
                    assert wslot[(g - 1) & 1][qq] == g - 1, "unitary read before it was written"
                    locs.append(("w", (g - 1) & 1, qq))
                    for c in tournament((r - 1) % R, qq, nb):
                        assert buf[(g - 1) & 1][c] == g - 1, "columns read before they were written"
                        locs.append(("x", (g - 1) & 1, c))
                else:
                    locs.append(("x", 0, b))
            reads_of[q] = locs
            for loc in locs:
                active.setdefault(loc, set()).add(q)
            state[q] = (g, "B")
        elif st == "B":
            writes = [("w", g & 1, q)] + ([("x", g & 1, bi), ("x", g & 1, bj)] if g > 0 else [])
            for w in writes:
                assert not (active.get(w, set()) - {q}), "write while another CTA reads"
            for kind, sl, idx in writes:
                (buf[sl] if kind == "x" else wslot[sl])[idx] = g
            state[q] = (g, "C")
        else:
            for loc in reads_of.pop(q):
                active[loc].discard(q)
            done[q] = g
            state[q] = (g + 1, "A")
    assert done == [G - 1] * P


@pytest.mark.parametrize("nb", [2, 4, 6, 8, 16, 34])
@pytest.mark.parametrize("sweeps", [1, 3])
def test_round_protocol_random_schedules(nb, sweeps):
    for seed in range(60 if nb <= 16 else 15):
        run_schedule(nb, sweeps, seed)


def test_pingpong_rebuild_equals_in_place_rotation():
    rng = np.random.default_rng(5)
    for nn in (16, 37, 100):
        nb = (nn + JW - 1) // JW
        nb += nb % 2
        R = nb - 1
        G = 2 * R
        X = rng.standard_normal((40, nn))
        Ws = [[None if rng.random() < 0.3 else np.linalg.qr(rng.standard_normal((16, 16)))[0]
               for _ in range(nb // 2)] for _ in range(G)]

        def cols(r, q):
            a, b = tournament(r, q, nb)
            return [c if c < nn else -1 for c in list(range(a * JW, a * JW + JW)) + list(range(b * JW, b * JW + JW))]

        def stack(M, cs):
            return np.stack([M[:, c] if c >= 0 else np.zeros(M.shape[0]) for c in cs], 1)

        seq = X.copy()
        for g in range(G):
            for q in range(nb // 2):
                if Ws[g][q] is not None:
                    cs = cols(g % R, q)
                    out = stack(seq, cs) @ Ws[g][q]
                    for i, c in enumerate(cs):
                        if c >= 0:
                            seq[:, c] = out[:, i]
        buf = [X.copy(), np.full_like(X, np.nan)]
        for g in range(1, G):
            r, rp = g % R, (g - 1) % R
            for q in range(nb // 2):
                for b in tournament(r, q, nb):
                    qq, side = pair_of(rp, b, nb)
                    own = [c for c in range(b * JW, b * JW + JW) if c < nn]
                    if Ws[g - 1][qq] is not None:
                        out = stack(buf[(g - 1) & 1], cols(rp, qq)) @ Ws[g - 1][qq][:, side * JW:side * JW + JW]
                    else:
                        out = buf[(g - 1) & 1][:, own]
                    buf[g & 1][:, own] = out[:, :len(own)]
        fin = buf[(G - 1) & 1].copy()
        for q in range(nb // 2):
            if Ws[G - 1][q] is not None:
                cs = cols((G - 1) % R, q)
                out = stack(fin, cs) @ Ws[G - 1][q]
                for i, c in enumerate(cs):
                    if c >= 0:
                        fin[:, c] = out[:, i]
        assert np.allclose(fin, seq)


def run_schedule_halves(nb, sweeps, seed):
    """The protocol with two CTAs per pair (row halves): each half runs the
    rounds above on its own copies of the columns' rows, the unitaries and the
    round flags, and the two halves of a pair exchange partial Grams once per
    round (publish its partial into slot g&1 of the pair, then wait for the
    other half's).  Checks the same properties, plus that an exchange reads
    the partner's partial of the same round and that a partial is never
    overwritten before the partner has read it."""
    rnd = random.Random(seed)
    P, R = nb // 2, nb - 1
    G = sweeps * R
    H = 2
    buf = [[{b: 0 for b in range(nb)}, {b: -1 for b in range(nb)}] for _ in range(H)]
    wslot = [[[-1] * P, [-1] * P] for _ in range(H)]
    done = [[-1] * P for _ in range(H)]
    xflag = [[-1] * P for _ in range(H)]
    gx = {}          # (slot, q, h) -> round of the partial held
    consumed = {}    # (slot, q, h) -> whether the partner has read it
    state = {(q, h): (0, "A") for q in range(P) for h in range(H)}
    active, reads_of = {}, {}
    sweep_end = R
    while True:
        cand = []
        for (q, h), (g, st) in state.items():
            if g >= min(G, sweep_end):
                continue
            if st == "A" and not all(done[h][t] >= g - 1 for t in wait_targets(g, g % R, q, nb)):
                continue
            if st == "Y" and xflag[1 - h][q] < g:
                continue
            cand.append((q, h))
        if not cand:
            if any(g < G for (g, _) in state.values()):
                assert all(g == sweep_end for (g, _) in state.values()), "deadlock"
                sweep_end += R
                continue
            break
        q, h = rnd.choice(cand)
        g, st = state[(q, h)]
        r = g % R
        bi, bj = tournament(r, q, nb)
        if st == "A":
            locs = []
            for b in (bi, bj):
                if g > 0:
                    qq, _ = pair_of((r - 1) % R, b, nb)
                    assert wslot[h][(g - 1) & 1][qq] == g - 1, "unitary read before it was written"
                    locs.append(("w", h, (g - 1) & 1, qq))
                    for c in tournament((r - 1) % R, qq, nb):
                        assert buf[h][(g - 1) & 1][c] == g - 1, "rows read before they were written"
                        locs.append(("x", h, (g - 1) & 1, c))
                else:
                    locs.append(("x", h, 0, b))
            reads_of[(q, h)] = locs
            for loc in locs:
                active.setdefault(loc, set()).add((q, h))
            state[(q, h)] = (g, "X")
        elif st == "X":
            key = (g & 1, q, h)
            assert key not in gx or consumed[key], "partial overwritten before the partner read it"
            gx[key], consumed[key] = g, False
            xflag[h][q] = g
            state[(q, h)] = (g, "Y")
        elif st == "Y":
            key = (g & 1, q, 1 - h)
            assert gx.get(key) == g, "exchange read a partial of another round"
            consumed[key] = True
            state[(q, h)] = (g, "B")
        elif st == "B":
            writes = [("w", h, g & 1, q)] + ([("x", h, g & 1, bi), ("x", h, g & 1, bj)] if g > 0 else [])
            for w in writes:
                assert not (active.get(w, set()) - {(q, h)}), "write while another CTA reads"
            for kind, hh, sl, idx in writes:
                (buf[hh][sl] if kind == "x" else wslot[hh][sl])[idx] = g
            state[(q, h)] = (g, "C")
        else:
            for loc in reads_of.pop((q, h)):
                active[loc].discard((q, h))
            done[h][q] = g
            state[(q, h)] = (g + 1, "A")
    assert done == [[G - 1] * P] * H


@pytest.mark.parametrize("nb", [2, 4, 6, 16, 34])
@pytest.mark.parametrize("sweeps", [1, 3])
def test_row_halves_protocol_random_schedules(nb, sweeps):
    for seed in range(40 if nb <= 16 else 10):
        run_schedule_halves(nb, sweeps, seed)
