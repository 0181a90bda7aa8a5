"""Oracle pins ported from test/test_mpo.jl (the strongest gate/wire convention pins)."""
import itertools

import numpy as np
import pytest

import oracle as O

RTOL = np.sqrt(np.finfo(float).eps)


def randn_c(rng, *shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def random_mps(rng, n):
    # test/test_mpo.jl:14-23
    ts = [randn_c(rng, 2, 2)] + [randn_c(rng, 2, 2, 2) for _ in range(n - 2)] + [randn_c(rng, 2, 2)]
    return O.ClosedMPS(ts)


def rand_unitary(rng, d):
    q, _ = np.linalg.qr(rng.random((d, d)) + 1j * rng.random((d, d)))
    return q


def full_operator(m, iwire, n):
    """The 2^n x 2^n matrix of gate m on wires iwire (Qaintessent sparse_matrix)."""
    out = np.zeros((2 ** n, 2 ** n), dtype=np.complex128)
    for c in range(2 ** n):
        e = np.zeros(2 ** n, dtype=np.complex128)
        e[c] = 1
        out[:, c] = O.apply_statevector(e, m, iwire)
    return out


def test_mpo_construction():
    # test/test_mpo.jl:25-36
    rng = np.random.default_rng(1)
    u = rand_unitary(rng, 4)
    mpo = O.mpo_from_matrix(u)
    assert len(mpo.tensors) == 2
    # the chain reproduces the operator; openidx lists the highest site first
    # (src/mpo.jl:73-82), so reverse the bit order before flattening
    t = np.transpose(O.contract(mpo), [1, 0, 3, 2]).reshape((4, 4), order="F")
    np.testing.assert_allclose(t, u, rtol=RTOL, atol=1e-13)


def test_extend_mpo_self_consistency():
    # test/test_mpo.jl:38-45
    rng = np.random.default_rng(2)
    a, b = rng.random((2, 2)) + 1j * rng.random((2, 2)), rng.random((2, 2)) + 1j * rng.random((2, 2))
    u1 = np.kron(np.kron(a, np.eye(2)), b)
    u2 = np.kron(a, b)
    ref = O.contract(O.mpo_from_matrix(u1))
    np.testing.assert_allclose(ref, O.contract(O.extend_mpo(u2, (3, 1))), rtol=RTOL, atol=1e-12)
    np.testing.assert_allclose(ref, O.contract(O.extend_mpo(O.mpo_from_matrix(u2), (3, 1))), rtol=RTOL, atol=1e-12)


def test_extend_mpo_against_circuit_gate():
    # test/test_mpo.jl:47-59
    rng = np.random.default_rng(3)
    qa, qb = rand_unitary(rng, 2), rand_unitary(rng, 2)
    u = np.kron(qa, qb)
    ref = full_operator(u, (3, 1), 3).reshape((2,) * 6, order="F")
    np.testing.assert_allclose(ref, O.contract(O.extend_mpo(u, (3, 1))), rtol=RTOL, atol=1e-12)
    np.testing.assert_allclose(ref, O.contract(O.extend_mpo(O.mpo_from_matrix(u), (3, 1))), rtol=RTOL, atol=1e-12)


@pytest.mark.parametrize("seed", range(6))
def test_apply_mpo_cnot(seed):
    # test/test_mpo.jl:62-86
    rng = np.random.default_rng(seed)
    n = 5
    psi = np.ones(1, dtype=np.complex128)
    for _ in range(n):
        psi = np.kron(psi, rng.standard_normal(2) + 1j * rng.standard_normal(2))
    cntrl = int(rng.integers(1, n + 1))
    targ = int(rng.integers(1, n))
    if targ >= cntrl:
        targ += 1
    ucnot = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)
    ref = O.apply_statevector(psi, ucnot, (targ, cntrl))
    got = O.contract(O.apply_mpo(O.mps_from_state(psi), O.mpo_from_matrix(ucnot), (targ, cntrl))).reshape(-1, order="F")
    np.testing.assert_allclose(got, ref, rtol=RTOL, atol=1e-12)


def test_apply_mpo_multi_qubit_all_wire_sets():
    # test/test_mpo.jl:88-121: a random 4-qubit unitary on every sorted wire set
    # of 8 qubits, plus an unsorted sample through the matrix overload
    rng = np.random.default_rng(4)
    n, m = 8, 4
    u = rand_unitary(rng, 2 ** m)
    mps = random_mps(rng, n)
    psi = O.contract(mps).reshape(-1, order="F")
    mpo = O.mpo_from_matrix(u)
    for com in itertools.combinations(range(1, n + 1), m):
        ref = O.apply_statevector(psi, u, com)
        got = O.contract(O.apply_mpo(mps, mpo, com)).reshape(-1, order="F")
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=1e-11)
        iw = tuple(int(x) for x in rng.choice(np.arange(1, n + 1), m, replace=False))
        ref = O.apply_statevector(psi, u, iw)
        got = O.contract(O.apply_mpo_matrix(mps, u, iw)).reshape(-1, order="F")
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=1e-11)


def test_apply_mpo_exceptions():
    # test/test_mpo.jl:124-140
    rng = np.random.default_rng(5)
    u = rand_unitary(rng, 8)
    mps = random_mps(rng, 5)
    mpo = O.mpo_from_matrix(u)
    with pytest.raises(O.QaintensorError, match="^Repeated wires are not valid.$"):
        O.apply_mpo(mps, mpo, (1, 3, 3))
    with pytest.raises(O.QaintensorError, match="between 1 and n"):
        O.apply_mpo(mps, mpo, (1, -2, 4))
    with pytest.raises(O.QaintensorError, match="between 1 and n"):
        O.apply_mpo(mps, mpo, (1, 3, 6))
