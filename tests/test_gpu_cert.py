"""The chosen mode honours the caller's cutoff of src/svd.jl:29-33 below its
FP32 resolution: a rank decision there is certified (the chi_max cap binds
with margin, or exactly as many values lie above the resolution as the exact
rank bound allows) or taken by the exact FP64 split.  Ranks therefore equal
the FP64 oracle's, and the counters say how each decision was made."""
import numpy as np
import pytest
import scipy.linalg as sla

import oracle as O

pytestmark = pytest.mark.gpu

_X = np.array([[0, 1], [1, 0]], dtype=complex)
_Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
_Z = np.diag([1.0, -1.0]).astype(complex)
_HXXZ = np.kron(_X, _X) + np.kron(_Y, _Y) + np.kron(_Z, _Z)


def weak_gate(rng, tau):
    """A weakly entangling gate (u2 (x) u1) exp(-i tau (XX + YY + ZZ)): its
    circuits have Schmidt values spread over many decades, many of them
    between a 1e-10 cutoff and the FP32 resolution."""
    u1, u2 = O.haar_unitary(rng, 2), O.haar_unitary(rng, 2)
    return np.kron(u2, u1) @ sla.expm(-1j * tau * _HXXZ)


def weak_brickwork(rng, n, depth, tau=0.08):
    gates = []
    for layer in range(1, depth + 1):
        for w in range(1 if layer % 2 else 2, n, 2):
            gates.append((layer, w, weak_gate(rng, tau)))
    return gates


def test_cutoff_below_resolution_takes_the_exact_split(engine):
    # a decaying spectrum whose rank at cutoff 1e-9 lies far below the FP32
    # resolution (~2e-6 ||theta||), no cap: no certificate, the FP64 split decides
    rng = np.random.default_rng(5)
    chi = 64
    a, b, _ = O.decay_theta_factors(chi, rng, decay=0.8)
    g = O.haar_unitary(rng)
    a32, b32 = a.astype(np.complex64), b.astype(np.complex64)
    cutoff = 1e-9
    ex = O.apply_2q([a32.astype(complex), b32.astype(complex)], g, 1, cutoff, 0)
    eng = engine.Engine(mode="chosen")
    m = eng.mps([a32, b32], dtype=np.complex64)
    c0 = eng.cert_counters()
    st = m.apply_2q(g, 1, cutoff, 0)
    c1 = eng.cert_counters()
    assert st["fallback"] == 4 and c1["fallback"] == c0["fallback"] + 1, (st, c0, c1)
    assert st["rank"] == ex.rank, (st, ex.rank)
    th = O.apply_gate_to_theta(O.theta_of(a32.astype(complex), b32.astype(complex)), g, chi, chi)
    approx = O.theta_of(m.site(1).astype(complex), m.site(2).astype(complex))
    # the exact split's own truncation error, plus complex64 rounding of the sites
    err = np.linalg.norm(th - approx)
    assert err <= np.sqrt(ex.discarded_weight) + 4e-7 * np.linalg.norm(th), (err, np.sqrt(ex.discarded_weight))
    m.free()
    eng.close()


def test_cap_certificate_keeps_the_fp32_split(engine):
    # the chi_max cap binds with a tail far above cutoff + resolution
    rng = np.random.default_rng(6)
    chi = 64
    a, b, _ = O.decay_theta_factors(chi, rng, decay=0.97)
    g = O.haar_unitary(rng)
    eng = engine.Engine(mode="chosen")
    m = eng.mps([a.astype(np.complex64), b.astype(np.complex64)], dtype=np.complex64)
    c0 = eng.cert_counters()
    st = m.apply_2q(g, 1, 1e-12, 48)
    c1 = eng.cert_counters()
    assert st["fallback"] == 0 and st["rank"] == 48, st
    assert c1["cap"] == c0["cap"] + 1, (c0, c1)
    m.free()
    eng.close()


def test_structural_certificate_on_haar_brickwork(engine):
    # Haar brickwork from |0...0>: theta' has exactly (operator-Schmidt rank
    # 4) x (inner bond) values, or the Hilbert-space dimension, above zero;
    # every decision at cutoff 1e-10 is certified and equals the oracle's
    rng = np.random.default_rng(7)
    n, depth, cutoff = 8, 5, 1e-10
    gates = O.brickwork_gates(n, depth, rng)
    ref_sites, ref_stats = O.run_brickwork(n, gates, cutoff, 0)
    eng = engine.Engine(mode="chosen")
    mps = eng.product_state(n, dtype=np.complex64)
    stats = [mps.apply_2q(g, w, cutoff, 0) for (_, w, g) in gates]
    cert = eng.cert_counters()
    assert cert["fallback"] == 0 and cert["struct"] + cert["resolved"] + cert["cap"] == len(gates), cert
    assert [s["rank"] for s in stats] == [s.rank for s in ref_stats]
    assert abs(mps.expect_z(1) - O.expect_z(ref_sites, 1)) <= 1e-6
    mps.free()
    eng.close()


def test_weakly_entangling_chain_matches_fp64_ranks(engine):
    # many Schmidt values between the cutoff and the FP32 resolution: some
    # decisions fall back; every kept rank equals the FP64 oracle's and <Z_i>
    # agrees to 1e-6
    rng = np.random.default_rng(8)
    n, depth, cutoff = 10, 8, 1e-10
    gates = weak_brickwork(rng, n, depth)
    ref_sites, ref_stats = O.run_brickwork(n, gates, cutoff, 16)
    eng = engine.Engine(mode="chosen")
    mps = eng.product_state(n, dtype=np.complex64)
    stats = [mps.apply_2q(g, w, cutoff, 16) for (_, w, g) in gates]
    cert = eng.cert_counters()
    assert cert["fallback"] > 0 and cert["struct"] > 0, cert
    assert [s["rank"] for s in stats] == [s.rank for s in ref_stats]
    for i in (1, n // 2, n):
        assert abs(mps.expect_z(i) - O.expect_z(ref_sites, i)) <= 1e-6
    mps.free()
    eng.close()


def test_batch_certifies_or_takes_the_fp64_split(engine):
    # the persistent batched kernel applies the same rule per task: weakly
    # entangling circuits at cutoff 1e-10 need the in-kernel FP64 split for
    # some tasks; bond dimensions equal the FP64 oracle's.  <Z_1> agrees to
    # 1e-5: the certified tasks keep FP32 products and Jacobi over up to 8
    # layers (5.6e-6 measured at worst)
    rng = np.random.default_rng(9)
    circuits = []
    for _ in range(10):
        n = int(rng.integers(4, 11))
        depth = int(rng.integers(2, 9))
        chi = int(rng.choice([4, 8, 16]))
        circuits.append((n, depth, chi, weak_brickwork(rng, n, depth)))
    layers = [[] for _ in range(max(c[1] for c in circuits))]
    for ci, (_, _, _, gates) in enumerate(circuits):
        for (layer, w, g) in gates:
            layers[layer - 1].append((ci, w, g))
    cutoff = 1e-10
    eng = engine.Engine(mode="chosen")
    b = engine.Batch(eng, [c[0] for c in circuits], [c[2] for c in circuits])
    b.run(layers, cutoff, use_graph=True)
    cert = b.cert_counts()
    assert cert["fallback"] > 0 and cert["struct"] > 0, cert
    assert sum(cert.values()) == sum(len(l) for l in layers)
    z = b.expect_z(1)
    for ci, (n, depth, chi, gates) in enumerate(circuits):
        sites, _ = O.run_brickwork(n, gates, cutoff, chi)
        assert list(b.bond_dims(ci)) == [1] + [s.shape[2] for s in sites], ci
        assert abs(z[ci] - O.expect_z(sites, 1)) <= 1e-5, (ci, z[ci], O.expect_z(sites, 1))
    b.free()
    eng.close()
