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


def test_optimised_order_network(engine):
    """contract(net, optimize=true) (src/contract.jl:249-258): the planned
    order on the GPU gives the oracle's tensor (test/test_tensor_circuit.jl:58
    checks the same against the default order)."""
    rng = np.random.default_rng(8)
    n, chi = 5, 6
    dims = [1] + [chi] * (n - 1) + [1]
    sites = [crandn(rng, dims[i], 2, dims[i + 1]) for i in range(n)]
    tensors = sites + [s.conj() for s in sites]
    contractions = []
    for i in range(1, n):
        contractions.append([(i, 3), (i + 1, 1)])
        contractions.append([(n + i, 3), (n + i + 1, 1)])
    for i in range(2, n + 1):
        contractions.append([(i, 2), (n + i, 2)])
    openidx = [(1, 1), (n + 1, 1), (n, 3), (2 * n, 3), (1, 2), (n + 1, 2)]
    net = O.Network(tensors, [O.Summation(s) for s in contractions], openidx)
    eng = engine.Engine(mode="plain")
    got = engine.contract(eng, tensors, contractions, openidx, optimize=True)
    ref = O.contract(net)
    np.testing.assert_allclose(got, O.contract(net, True), rtol=0, atol=1e-12 * np.abs(ref).max())
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    eng.close()


@pytest.mark.parametrize("nq", [1, 2, 5, 8])
def test_mps_from_state_on_gpu(engine, nq):
    """MPS(psi) (src/mps.jl:55-89) with the SVDs on the GPU: the device MPS
    contracts back to psi (test/test_mps.jl:34-49) and its bonds are the
    oracle's."""
    rng = np.random.default_rng(nq)
    psi = crandn(rng, 2 ** nq)
    eng = engine.Engine(mode="plain")
    if nq == 1:
        with pytest.raises(engine.QaintensorError, match=r"^Input state must have length 2\^N$"):
            engine.mps_from_state(eng, crandn(rng, 3))
        eng.close()
        return
    m = engine.mps_from_state(eng, psi)
    sites = m.sites()
    back = O.mps_to_state([s.astype(complex) for s in sites])
    assert np.abs(back - psi).max() <= 1e-12 * np.abs(psi).max()
    ref = O.mps_from_state(psi)
    assert [s.shape[-1] for s in sites[:-1]] == [t.shape[-1] for t in ref.tensors[:-1]]
    m.free()
    eng.close()


@pytest.mark.parametrize("nq", [1, 2, 3, 4])
def test_mpo_from_matrix_on_gpu(engine, nq):
    """MPO(m) (src/mpo.jl:27-90) with the SVDs on the GPU: the chain
    contracts back to m the way the oracle's network does."""
    rng = np.random.default_rng(10 + nq)
    mat = crandn(rng, 2 ** nq, 2 ** nq)
    eng = engine.Engine(mode="plain")
    sites = engine.mpo_from_matrix(eng, mat)
    ref = O.mpo_from_matrix(mat)
    assert [s.shape for s in sites] == [t.shape for t in ref.tensors]
    got = O.contract(O.Network(sites, ref.contractions, ref.openidx, "mpo"))
    want = O.contract(ref)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    eng.close()
