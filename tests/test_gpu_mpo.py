"""MPO application, compression sweep and <H> on the device MPS against the FP64 oracle."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def random_sites(rng, n, chi):
    dims = [1] + [chi] * (n - 1) + [1]
    sites = [(rng.standard_normal((dims[i], 2, dims[i + 1])) + 1j * rng.standard_normal((dims[i], 2, dims[i + 1])))
             for i in range(n)]
    return sites


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-10), (np.complex64, 2e-5)])
def test_tfim_power_steps_match_oracle(engine, dtype, tol):
    rng = np.random.default_rng(17)
    n, chi, cutoff = 10, 12, 1e-9
    h = rng.uniform(0.5, 1.5, n)
    mpo = O.tfim_mpo(n, 1.0, h)
    sites = random_sites(rng, n, chi)
    eng = engine.Engine(mode="plain" if dtype == np.complex128 else "chosen")
    m = eng.mps([s.astype(dtype) for s in sites], dtype=dtype)
    ref, _, _ = O.compress_sweep([s.astype(dtype).astype(np.complex128) for s in sites], cutoff, chi)
    m.compress(cutoff, chi, mode="plain" if dtype == np.complex128 else "chosen")
    for step in range(3):
        m.apply_mpo(mpo)
        ranks, disc = m.compress(cutoff, chi, mode="plain" if dtype == np.complex128 else "chosen")
        ref, rranks, rdisc = O.compress_sweep(O.apply_mpo_sites(ref, mpo), cutoff, chi)
        e_gpu, e_ref = m.expect_mpo(mpo), O.mpo_energy(ref, mpo)
        assert abs(e_gpu - e_ref) <= tol * max(1.0, abs(e_ref)), (step, e_gpu, e_ref)
        if dtype == np.complex128:
            assert list(ranks) == list(rranks)
    psi = O.mps_to_state([s.astype(np.complex128) for s in m.sites()])
    ref_psi = O.mps_to_state(ref)
    ov = abs(np.vdot(psi, ref_psi)) / (np.linalg.norm(psi) * np.linalg.norm(ref_psi))
    assert ov > 1 - 10 * tol
    m.free()
    eng.close()


def test_tfim_energy_against_dense_hamiltonian(engine):
    rng = np.random.default_rng(18)
    n = 6
    h = rng.uniform(0.5, 1.5, n)
    mpo = O.tfim_mpo(n, 1.0, h)
    sites = random_sites(rng, n, 4)
    psi = O.mps_to_state(sites)
    Z = np.diag([1.0, -1.0])
    X = np.array([[0, 1], [1, 0]], dtype=float)
    H = np.zeros((2 ** n, 2 ** n), dtype=complex)
    for i in range(n):
        e = np.zeros(2 ** n, dtype=complex)
        for c in range(2 ** n):
            e[:] = 0
            e[c] = 1
            H[:, c] -= h[i] * O.apply_statevector(e, X, (i + 1,))
            if i + 1 < n:
                H[:, c] -= O.apply_statevector(O.apply_statevector(e, Z, (i + 1,)), Z, (i + 2,))
    ref = np.vdot(psi, H @ psi).real / np.vdot(psi, psi).real
    eng = engine.Engine(mode="plain")
    m = eng.mps(sites)
    assert abs(m.expect_mpo(mpo) - ref) <= 1e-10 * max(1, abs(ref))
    assert abs(O.mpo_energy(sites, mpo) - ref) <= 1e-10 * max(1, abs(ref))
    m.free()
    eng.close()
