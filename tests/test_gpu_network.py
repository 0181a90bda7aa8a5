"""Network-level drivers (src/contract.jl:242-264, src/mps.jl:190-201) over the
GPU pairwise contraction, against the oracle's ncon restatement."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def crandn(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def test_closed_mps_overlap_network(engine):
    rng = np.random.default_rng(3)
    n, chi = 6, 4
    dims = [1] + [chi] * (n - 1) + [1]
    sites = [crandn(rng, dims[i], 2, dims[i + 1]) for i in range(n)]
    tensors = [s.reshape(s.shape) for s in sites] + [s.conj() for s in sites]
    contractions = []
    for i in range(1, n):
        contractions.append([(i, 3), (i + 1, 1)])
        contractions.append([(n + i, 3), (n + i + 1, 1)])
    for i in range(1, n + 1):
        contractions.append([(i, 2), (n + i, 2)])
    openidx = [(1, 1), (n + 1, 1), (n, 3), (2 * n, 3)]
    net = O.Network(tensors, [O.Summation(s) for s in contractions], openidx)
    eng = engine.Engine(mode="plain")
    got = engine.contract(eng, tensors, contractions, openidx)
    ref = O.contract(net)
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    eng.close()


def test_trace_and_disconnected_parts(engine):
    rng = np.random.default_rng(4)
    a = crandn(rng, 3, 4, 3)          # legs 1 and 3 traced
    b, c = crandn(rng, 4, 5), crandn(rng, 2, 2)
    contractions = [[(1, 1), (1, 3)], [(1, 2), (2, 1)]]
    openidx = [(3, 2), (2, 2), (3, 1)]
    net = O.Network([a, b, c], [O.Summation(s) for s in contractions], openidx)
    eng = engine.Engine(mode="plain")
    got = engine.contract(eng, [a, b, c], contractions, openidx)
    ref = O.contract(net)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    eng.close()


def test_contract_svd_mps_matches_oracle(engine):
    rng = np.random.default_rng(5)
    n, chi = 5, 3
    tensors = [crandn(rng, 2, chi)] + [crandn(rng, chi, 2, chi) for _ in range(n - 2)] + [crandn(rng, chi, 2)]
    contractions = [[(1, 2), (2, 1)]] + [[(i, 3), (i + 1, 1)] for i in range(2, n)]
    openidx = [(1, 1)] + [(i, 2) for i in range(2, n + 1)]
    net = O.Network(tensors, [O.Summation(s) for s in contractions], openidx, kind="mps")
    eng = engine.Engine(mode="plain")
    for er in (0.0, 1e-2):
        got = engine.contract_svd_mps(eng, tensors, contractions, er=er)
        ref = O.contract_svd_mps(net, er=er)
        assert got.shape == ref.shape
        assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()
    eng.close()


def test_switch_wires_and_permute_match_oracle(engine):
    """switch!(mps, i, j) and permute!(mps, order) (src/switch.jl) as ladders
    of GPU switches, against the oracle's restatement."""
    rng = np.random.default_rng(9)
    n = 6
    psi = crandn(rng, 2 ** n)
    psi /= np.linalg.norm(psi)
    eng = engine.Engine(mode="plain")
    for op, arg in (("wires", (2, 5)), ("wires", (6, 1)), ("perm", [3, 1, 6, 2, 5, 4])):
        ref = O.mps_from_state(psi)
        mps = eng.mps(ref.tensors)
        if op == "wires":
            O.switch_wires(ref, *arg)
            mps.switch_wires(*arg)
        else:
            O.permute_mps(ref, arg)
            mps.permute(arg)
        got = O.mps_to_state(mps.sites())
        want = O.mps_to_state(O.sites_from_reference_mps(ref.tensors))
        assert np.abs(got - want).max() <= 1e-11, (op, arg)
        mps.free()
    with pytest.raises(engine.QaintensorError, match="repeat values"):
        m = eng.product_state(3)
        m.permute([1, 1, 2])
    eng.close()
