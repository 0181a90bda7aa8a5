"""The FP64 oracle still reproduces the committed golden fixtures
(tests/golden/make_golden.py made them from the oracle pinned by the ported
reference tests)."""
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def test_tail_rule_fixture():
    f = load("tail_rule")
    for s, er, k in zip(f["spectra"], f["cutoffs"], f["k"]):
        assert O.tail_rank(s[~np.isnan(s)], er, clamp=True) == k


def test_brickwork12_fixture():
    f = load("brickwork12")
    gates = list(zip(f["gate_layers"], f["gate_wires"], f["gates"]))
    sites, stats = O.run_brickwork(int(f["n"]), gates, float(f["cutoff"]), int(f["chi_max"]))
    assert [s.rank for s in stats] == list(f["ranks"])
    assert [s.rank_cutoff for s in stats] == list(f["ranks_cutoff"])
    z = [O.expect_z(sites, w) for w in range(1, int(f["n"]) + 1)]
    assert np.allclose(z, f["z"], rtol=1e-12, atol=1e-14)
    assert np.abs(O.mps_to_state(sites) - f["psi"]).max() <= 1e-12
    # the truncated MPS state is the dense circuit state up to the discarded weight
    assert abs(np.vdot(f["psi"], f["dense"])) ** 2 > 1 - 10 * max(f["discarded"].sum(), 1e-15)


def test_decay_bond_fixture():
    f = load("decay_bond")
    sites = [f["a"].copy(), f["b"].copy()]
    st = O.apply_2q(sites, f["gate"], 1, float(f["cutoff"]), 0)
    assert st.rank == int(f["rank"])
    assert np.abs(st.spectrum - f["spectrum"]).max() <= 1e-14
    got = O.theta_of(sites[0], sites[1])
    ref = O.theta_of(f["a_new"], f["b_new"])
    assert np.abs(got - ref).max() <= 1e-13


@pytest.mark.slow
def test_tfim10_fixture():
    f = load("tfim10")
    n, chi, cutoff = int(f["n"]), int(f["chi"]), float(f["cutoff"])
    mpo = O.tfim_mpo(n, 1.0, f["h"])
    ref, _, _ = O.compress_sweep([f[f"site{i}"].copy() for i in range(n)], cutoff, chi)
    for step in range(3):
        ref, r, _ = O.compress_sweep(O.apply_mpo_sites(ref, mpo), cutoff, chi)
        assert list(r) == list(f["ranks"][step])
        assert abs(O.mpo_energy(ref, mpo) - f["energies"][step]) <= 1e-10 * abs(f["energies"][step])
