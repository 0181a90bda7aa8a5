"""Generate the golden input/output fixtures of the parity tests from the FP64
oracle (test infrastructure; run from the repository root):

    python tests/golden/make_golden.py

The reference publishes no golden vectors (its tests are equivalence tests,
ported in tests/test_oracle_*.py, which pin the oracle); these fixtures freeze
the pinned oracle's outputs on seeded inputs so the GPU tests compare against
stored numbers, and tests/test_golden.py checks that the oracle still
reproduces them.

brickwork12.npz  12 qubits from |0...0>, brickwork depth 8, Haar gates (seed
                 2024), cutoff 1e-10, chi_max 32: gates, kept rank, rank at
                 the cutoff and discarded weight per update, <Z_w> for every
                 wire, the MPS amplitudes and the dense-statevector amplitudes.
decay_bond.npz   one update at chi = 32: A, B (spectrum 0.97^k), Haar gate,
                 cutoff 1e-4; spectrum of theta', kept rank, new sites.
tail_rule.npz    spectra and cutoffs with the tail rule's kept rank (clamped
                 at 1, as the engine does).
tfim10.npz       10-site TFIM MPO (J = 1, h seeded in [0.5, 1.5]), a seeded
                 chi = 12 MPS, compression then 3 rounds of MPO application +
                 compression (cutoff 1e-9, chi_max 12): ranks and <H> per round.

Two more fixtures come from the workload-config runner, because one run of
each takes about twenty minutes on four host cores:

c3_zz_fp64_c128.json  <Z_i Z_i+1> on all 63 bonds of the 64-qubit, depth-20
                      Haar brickwork (seed 64, chi_max 1024, cutoff 1e-8) run
                      by the FP64 oracle:
                      python tests/run_configs.py c3ref --c3-ref-storage c128
c3_zz_fp64_c64.json   the same with every updated site rounded to complex64:
                      python tests/run_configs.py c3ref --c3-ref-storage c64
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402


def brickwork12():
    rng = np.random.default_rng(2024)
    n, depth, cutoff, chi_max = 12, 8, 1e-10, 32
    gates = O.brickwork_gates(n, depth, rng)
    sites, stats = O.run_brickwork(n, gates, cutoff, chi_max)
    dense = np.zeros(2 ** n, dtype=complex)
    dense[0] = 1
    for (_, w, g) in gates:
        dense = O.apply_statevector(dense, g, (w, w + 1))
    return dict(n=n, depth=depth, cutoff=cutoff, chi_max=chi_max,
                gate_wires=np.array([w for (_, w, _) in gates]), gate_layers=np.array([l for (l, _, _) in gates]),
                gates=np.stack([g for (_, _, g) in gates]),
                ranks=np.array([s.rank for s in stats]), ranks_cutoff=np.array([s.rank_cutoff for s in stats]),
                discarded=np.array([s.discarded_weight for s in stats]),
                z=np.array([O.expect_z(sites, w) for w in range(1, n + 1)]),
                psi=O.mps_to_state(sites), dense=dense)


def decay_bond():
    rng = np.random.default_rng(32)
    chi, cutoff = 32, 1e-4
    a, b = O.decay_theta_factors(chi, rng, 0.97)[:2]
    g = O.haar_unitary(rng, 4)
    sites = [a.copy(), b.copy()]
    st = O.apply_2q(sites, g, 1, cutoff, 0)
    return dict(a=a, b=b, gate=g, cutoff=cutoff, spectrum=st.spectrum, rank=st.rank,
                discarded=st.discarded_weight, a_new=sites[0], b_new=sites[1])


def tail_rule():
    rng = np.random.default_rng(5)
    spectra, cutoffs, ks = [], [], []
    for case in range(24):
        n = int(rng.integers(1, 40))
        s = np.sort(rng.uniform(0, 1, n) ** (1 + case % 4))[::-1]
        if case % 5 == 0:
            s[n // 2:] = 0.0  # exact zeros
        for er in (0.0, 1e-12, 1e-3, 0.05, 0.3, 10.0):
            spectra.append(np.pad(s, (0, 40 - n), constant_values=np.nan))
            cutoffs.append(er)
            ks.append(O.tail_rank(s, er, clamp=True))
    return dict(spectra=np.array(spectra), cutoffs=np.array(cutoffs), k=np.array(ks))


def tfim10():
    rng = np.random.default_rng(17)
    n, chi, cutoff = 10, 12, 1e-9
    h = rng.uniform(0.5, 1.5, n)
    mpo = O.tfim_mpo(n, 1.0, h)
    dims = [1] + [chi] * (n - 1) + [1]
    sites = [(rng.standard_normal((dims[i], 2, dims[i + 1])) + 1j * rng.standard_normal((dims[i], 2, dims[i + 1])))
             for i in range(n)]
    out = dict(n=n, chi=chi, cutoff=cutoff, h=h)
    for i, s in enumerate(sites):
        out[f"site{i}"] = s
    ref, _, _ = O.compress_sweep([s.copy() for s in sites], cutoff, chi)
    ranks, energies = [], []
    for step in range(3):
        ref, r, _ = O.compress_sweep(O.apply_mpo_sites(ref, mpo), cutoff, chi)
        ranks.append(r)
        energies.append(O.mpo_energy(ref, mpo))
    out["ranks"] = np.array(ranks)
    out["energies"] = np.array(energies)
    return out


MAKERS = {"brickwork12": brickwork12, "decay_bond": decay_bond, "tail_rule": tail_rule, "tfim10": tfim10}


def main():
    for name, fn in MAKERS.items():
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **fn())
        print(f"{path}: {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
