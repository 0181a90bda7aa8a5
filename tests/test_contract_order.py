"""contract(net, optimize=true) of src/contract.jl:242-258: the reference's
breadth-first contraction-order search (contract_order, :183-235, after
arXiv:1304.6112) restated in the oracle and in the package's host logic.
Both give the same sequence and cost on random connected networks, the
ordered contraction gives the same tensor as the default order, and the
known-answer case is a chain whose cheapest order is fixed by its sizes."""
import itertools

import numpy as np
import pytest

import oracle as O


def random_network(rng, ntens, nopen):
    """A connected network of ntens tensors: a random spanning tree of bonds,
    a few extra bonds, and nopen open legs."""
    legs = [[] for _ in range(ntens)]
    bonds = []
    for i in range(1, ntens):
        bonds.append((int(rng.integers(0, i)), i))
    for _ in range(int(rng.integers(0, ntens))):
        a, b = rng.choice(ntens, 2, replace=False)
        bonds.append((int(a), int(b)))
    dims = []
    contractions = []
    for a, b in bonds:
        d = int(rng.integers(2, 5))
        legs[a].append(d)
        legs[b].append(d)
        contractions.append(O.Summation([(a + 1, len(legs[a])), (b + 1, len(legs[b]))]))
        dims.append(d)
    openidx = []
    for _ in range(nopen):
        t = int(rng.integers(0, ntens))
        legs[t].append(int(rng.integers(2, 4)))
        openidx.append((t + 1, len(legs[t])))
    tensors = [(rng.standard_normal(tuple(l)) + 1j * rng.standard_normal(tuple(l))) for l in legs]
    return O.Network(tensors, contractions, openidx)


def test_known_chain_order():
    # A(2x100) - B(100x3) - C(3x100): contracting B with C first costs
    # 100*3*100 + 2*100*100 ... the search picks the cheaper (A.B) first
    rng = np.random.default_rng(1)
    A, B, C = (rng.standard_normal(s) for s in ((2, 100), (100, 3), (3, 100)))
    net = O.Network([A, B, C], [O.Summation([(1, 2), (2, 1)]), O.Summation([(2, 2), (3, 1)])], [(1, 1), (3, 2)])
    costs, labels = O.contract_rep_costs(net)
    seq, cost = O.contract_order(costs, labels)
    assert seq == [1, 2] and cost == 2 * 100 * 3 + 2 * 3 * 100
    np.testing.assert_allclose(O.contract(net, True), A @ B @ C)


@pytest.mark.parametrize("ntens", [3, 4, 5, 6])
def test_package_planner_matches_oracle_and_order_keeps_the_tensor(ntens):
    import __graft_entry__ as g
    qt = g.load_package()
    rng = np.random.default_rng(ntens)
    for _ in range(6):
        net = random_network(rng, ntens, int(rng.integers(1, 4)))
        costs, labels = O.contract_rep_costs(net)
        seq_o, cost_o = O.contract_order(costs, labels)
        seq_p, cost_p = qt.contract_order([t.shape for t in net.tensors],
                                          qt.contract_rep(net.tensors, [s.idx for s in net.contractions], net.openidx))
        assert (seq_p, cost_p) == (seq_o, cost_o)
        assert sorted(seq_o) == list(range(1, len(net.contractions) + 1))
        ref = O.contract(net)
        np.testing.assert_allclose(O.contract(net, True), ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())


def test_disconnected_network_is_refused():
    rng = np.random.default_rng(2)
    net = O.Network([rng.standard_normal((2, 3)), rng.standard_normal((3, 2)), rng.standard_normal((2,))],
                    [O.Summation([(1, 2), (2, 1)])], [(1, 1), (2, 2), (3, 1)])
    costs, labels = O.contract_rep_costs(net)
    with pytest.raises(O.QaintensorError, match="not connected"):
        O.contract_order(costs, labels)
