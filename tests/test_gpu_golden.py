"""The engine against the committed golden fixtures (made by the FP64 oracle;
no oracle code runs here): plain FP64 mode, kept ranks identical,
expectation values to 1e-10 relative."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def contract_state(sites):
    psi = np.ones((1, 1), dtype=np.complex128)
    for s in sites:
        cl, _, cr = s.shape
        psi = (psi @ s.reshape((cl, 2 * cr), order="F")).reshape((-1, cr), order="F")
    return psi.reshape(-1, order="F")


def test_tail_rule_against_fixture(engine):
    f = load("tail_rule")
    eng = engine.Engine(mode="plain")
    for s, er, k in zip(f["spectra"], f["cutoffs"], f["k"]):
        s = s[~np.isnan(s)]
        _, S, _, kk, _ = eng.truncated_svd(np.diag(s).astype(np.complex128), float(er))
        assert kk == k, (s, er, kk, k)
        assert np.abs(S - s[:kk]).max() <= 1e-14
    eng.close()


def test_brickwork12_against_fixture(engine):
    f = load("brickwork12")
    n = int(f["n"])
    eng = engine.Engine(mode="plain")
    mps = eng.product_state(n)
    ranks = [mps.apply_2q(g, int(w), float(f["cutoff"]), int(f["chi_max"]))["rank"]
             for w, g in zip(f["gate_wires"], f["gates"])]
    assert ranks == list(f["ranks"])
    z = np.array([mps.expect_z(w) for w in range(1, n + 1)])
    assert np.all(np.abs(z - f["z"]) <= 1e-10 * np.maximum(np.abs(f["z"]), 1e-3))
    psi = contract_state(mps.sites())
    assert np.abs(psi - f["psi"]).max() <= 1e-10
    mps.free()
    eng.close()


@pytest.mark.parametrize("mode", ["plain", "cusolver"])
def test_decay_bond_against_fixture(engine, mode):
    f = load("decay_bond")
    eng = engine.Engine(mode=mode)
    m = eng.mps([f["a"], f["b"]])
    st = m.apply_2q(f["gate"], 1, float(f["cutoff"]), 0)
    assert st["rank"] == int(f["rank"])
    assert abs(st["discarded_weight"] - float(f["discarded"])) <= 1e-14
    a, b = m.site(1), m.site(2)
    chi = a.shape[0]
    got = a.reshape((2 * chi, -1), order="F") @ b.reshape((b.shape[0], -1), order="F")
    ref = f["a_new"].reshape((2 * chi, -1), order="F") @ f["b_new"].reshape((f["b_new"].shape[0], -1), order="F")
    assert np.abs(got - ref).max() <= 1e-12
    m.free()
    eng.close()


def test_tfim10_against_fixture(engine):
    f = load("tfim10")
    n, chi, cutoff = int(f["n"]), int(f["chi"]), float(f["cutoff"])
    # TFIM MPO restated here from its definition (bond dimension 3):
    # W = [[I, 0, 0], [Z, 0, 0], [-h X, -J Z, I]] on the (left, right) bond legs
    I2, X, Z = np.eye(2), np.array([[0, 1], [1, 0]], float), np.diag([1.0, -1.0])
    mpo = []
    for i in range(n):
        W = np.zeros((3, 2, 2, 3), dtype=np.complex128)
        W[0, :, :, 0] = I2
        W[1, :, :, 0] = Z
        W[2, :, :, 0] = -f["h"][i] * X
        W[2, :, :, 1] = -Z
        W[2, :, :, 2] = I2
        if i == 0:
            W = W[2:3]
        if i == n - 1:
            W = W[:, :, :, 0:1]
        mpo.append(W)
    eng = engine.Engine(mode="plain")
    m = eng.mps([f[f"site{i}"] for i in range(n)])
    m.compress(cutoff, chi, mode="plain")
    for step in range(3):
        m.apply_mpo(mpo)
        ranks, _ = m.compress(cutoff, chi, mode="plain")
        assert list(ranks) == list(f["ranks"][step])
        e = m.expect_mpo(mpo)
        assert abs(e - f["energies"][step]) <= 1e-10 * abs(f["energies"][step]), (step, e, f["energies"][step])
    m.free()
    eng.close()
