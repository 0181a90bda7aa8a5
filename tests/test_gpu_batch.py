"""The batched persistent-kernel path against the FP64 oracle on a small
ensemble of uneven circuits (qubits, depths, bond caps)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def ensemble(rng, ncirc):
    circuits = []
    for c in range(ncirc):
        n = int(rng.integers(4, 11))
        depth = int(rng.integers(2, 7))
        chi = int(rng.choice([2, 4, 8, 16]))
        circuits.append((n, depth, chi, O.brickwork_gates(n, depth, rng)))
    return circuits


def to_layers(circuits):
    depth = max(c[1] for c in circuits)
    layers = [[] for _ in range(depth)]
    for ci, (_, _, _, gates) in enumerate(circuits):
        for (layer, w, g) in gates:
            layers[layer - 1].append((ci, w, g))
    return layers


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_oracle(engine, use_graph):
    rng = np.random.default_rng(41)
    circuits = ensemble(rng, 24)
    eng = engine.Engine(mode="chosen")
    b = engine.Batch(eng, [c[0] for c in circuits], [c[2] for c in circuits])
    cutoff = 1e-8
    b.run(to_layers(circuits), cutoff, use_graph=use_graph)
    z = b.expect_z(1)
    ranks, sweeps, _ = b.task_stats()
    assert ranks.min() >= 1 and sweeps.max() > 0
    for ci, (n, depth, chi, gates) in enumerate(circuits):
        sites, stats = O.run_brickwork(n, gates, cutoff, chi)
        # complex64 storage: |<Z>| error <= 2 ||psi - ref|| (the state bound below)
        assert abs(z[ci] - O.expect_z(sites, 1)) <= 5e-5, (ci, z[ci], O.expect_z(sites, 1))
        dims = b.bond_dims(ci)
        assert list(dims) == [1] + [s.shape[2] for s in sites], (ci, dims)
        psi = O.mps_to_state([b.site(ci, i).astype(np.complex128) for i in range(1, n + 1)])
        ref = O.mps_to_state(sites)
        assert np.linalg.norm(psi - ref) <= 5e-5 * np.linalg.norm(ref)  # FP32 over <= 6 layers
    b.free()
    eng.close()


def test_batch_replay_reproduces_the_run(engine):
    rng = np.random.default_rng(42)
    circuits = ensemble(rng, 12)
    eng = engine.Engine(mode="chosen")
    b = engine.Batch(eng, [c[0] for c in circuits], [c[2] for c in circuits])
    b.run(to_layers(circuits), 1e-8, use_graph=True)
    z1 = b.expect_z(2)
    b.reset()
    b.replay()
    z2 = b.expect_z(2)
    np.testing.assert_allclose(z1, z2, atol=1e-6)
    b.free()
    eng.close()
