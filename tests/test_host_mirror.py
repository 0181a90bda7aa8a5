"""Host logic of the reference-facing mirror (no GPU): network labels as
src/contract.jl:39-60 assigns them."""
import numpy as np

import oracle as O


def test_contract_rep_matches_reference_labels(engine):
    rng = np.random.default_rng(1)
    a, b, c = rng.standard_normal((2, 3, 4)), rng.standard_normal((4, 3)), rng.standard_normal((2, 5))
    contractions = [[(1, 2), (2, 2)], [(1, 3), (2, 1)]]
    openidx = [(3, 2), (1, 1), (3, 1)]
    net = O.Network([a, b, c], [O.Summation(s) for s in contractions], openidx)
    assert engine.contract_rep([a, b, c], contractions, openidx) == O.contract_rep(net)


def test_contract_svd_mps_rejects_periodic_and_negative_er(engine):
    import pytest
    t = [np.zeros((2, 3)), np.zeros((3, 2, 3)), np.zeros((3, 2))]
    with pytest.raises(engine.QaintensorError, match="Error must be positive"):
        engine.contract_svd_mps(None, t, [], er=-1.0)
    with pytest.raises(engine.QaintensorError, match="periodic"):
        engine.contract_svd_mps(None, t, [[(3, 3), (1, 1)]], er=0.0)
