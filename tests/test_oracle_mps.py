"""Oracle pins ported from test/test_mps.jl and test/test_tensor_circuit.jl."""
import math
from functools import reduce

import numpy as np
import pytest

import oracle as O

RTOL = np.sqrt(np.finfo(float).eps)


def randn_c(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def kron_all(vs):
    return reduce(np.kron, vs)


def close(a, b):
    np.testing.assert_allclose(a, b, rtol=RTOL, atol=1e-12)


def test_contract_svd_mps_open_and_errors():
    # test/test_mps.jl:9-19
    rng = np.random.default_rng(1)
    T = rng.random((2, 2, 2))
    mps = O.OpenMPS(T, 3)
    g = O.Network(mps.tensors, mps.contractions, mps.openidx)
    close(O.contract(g), O.contract_svd_mps(mps, er=0.0))
    with pytest.raises(O.QaintensorError, match="periodic boundary"):
        O.contract_svd_mps(O.PeriodicMPS(T, 3), er=0.0)
    with pytest.raises(O.QaintensorError, match="^Error must be positive$"):
        O.contract_svd_mps(mps, er=-0.5)


def test_check_mps_exceptions():
    # test/test_mps.jl:21-33
    rng = np.random.default_rng(2)
    mps = O.OpenMPS(rng.random((2, 2, 2)), 3)
    mps.contractions[0] = O.Summation([(1, 2), (2, 1)])
    with pytest.raises(O.QaintensorError, match="first leg must contract with last leg"):
        O.check_mps(mps)
    mps.contractions[0] = O.Summation([(1, 3), (2, 2)])
    with pytest.raises(O.QaintensorError, match="last leg must contract with first leg"):
        O.check_mps(mps)
    mps.tensors[1] = rng.random((2, 2, 2, 2))
    with pytest.raises(O.QaintensorError, match="can only have 2 or 3 legs"):
        O.check_mps(mps)


def test_statevector_round_trip():
    # test/test_mps.jl:34-49 (wire 1 = fastest index)
    rng = np.random.default_rng(3)
    b = [randn_c(rng, 2) for _ in range(5)]
    ref = kron_all(b)
    mps = O.mps_from_state(ref)
    close(O.contract(mps).reshape(-1, order="F"), ref)
    with pytest.raises(O.QaintensorError, match=r"^Input state must have length 2\^N$"):
        O.mps_from_state(randn_c(rng, 6))


def qft_gates(n):
    """A QFT-shaped gate list (Hadamards and controlled phases: symmetric matrices)."""
    h = np.array([[1, 1], [1, -1]]) / math.sqrt(2)
    out = []
    for i in range(n, 0, -1):
        out.append((h, (i,)))
        for j in range(i - 1, 0, -1):
            ph = np.diag([1, 1, 1, np.exp(1j * math.pi / 2 ** (i - j))])
            out.append((ph, (i, j)))
    return out


def test_tensor_circuit_qft_on_general_network():
    # test/test_mps.jl:57-88 and test/test_tensor_circuit.jl:32-60
    rng = np.random.default_rng(4)
    psi = O.Network([randn_c(rng, 2, 6), randn_c(rng, 2, 6, 7), randn_c(rng, 2, 7)],
                    [O.Summation([(1, 2), (2, 2)]), O.Summation([(2, 3), (3, 2)])],
                    [(1, 1), (2, 1), (3, 1)])
    ref = O.contract(psi).reshape(-1, order="F")
    for m, w in qft_gates(3):
        ref = O.apply_statevector(ref, m, w)
    for m, w in qft_gates(3):
        O.tensor_circuit(psi, m, w)
    close(O.contract(psi).reshape(-1, order="F"), ref)
    # test/test_tensor_circuit.jl:58: the optimised contraction order
    close(O.contract(psi, True).reshape(-1, order="F"), ref)


def test_mps_constructor_exceptions():
    # test/test_mps.jl:90-104
    rng = np.random.default_rng(5)
    ts = [rng.random((2, 2, 2)), rng.random((2, 2, 2))]
    op = [(1, 2), (2, 2)]
    with pytest.raises(O.QaintensorError, match="first leg must contract with last leg"):
        O.make_mps(ts, [O.Summation([(1, 1), (2, 3)])], op)
    with pytest.raises(O.QaintensorError, match="last leg must contract with first leg"):
        O.make_mps(ts, [O.Summation([(1, 3), (2, 3)])], op)
    with pytest.raises(O.QaintensorError, match="can only have 2 or 3 legs"):
        O.make_mps([rng.random((2, 2, 2, 2)), rng.random((2, 2, 2))], [O.Summation([(1, 4), (2, 1)])], op)


def test_open_closed_mps_and_exceptions():
    # test/test_mps.jl:106-150
    rng = np.random.default_rng(6)
    mps = O.OpenMPS(rng.random((2, 2, 2)), 3)
    close(O.contract(O.Network(mps.tensors, mps.contractions, mps.openidx)), O.contract_svd_mps(mps))
    with pytest.raises(O.QaintensorError, match="^Tensors must have 3 legs$"):
        O.OpenMPS([rng.random((2, 2, 2, 2))] * 2)
    mps = O.ClosedMPS([rng.random((2, 5)), rng.random((5, 2, 3)), rng.random((3, 2))])
    close(O.contract(O.Network(mps.tensors, mps.contractions, mps.openidx)), O.contract_svd_mps(mps))
    T1, T2, T3 = rng.random((2, 2, 2)), rng.random((2, 2, 2, 2)), rng.random((2, 2))
    with pytest.raises(O.QaintensorError, match="^First tensor must have 2 legs$"):
        O.ClosedMPS([T1, T1, T3])
    with pytest.raises(O.QaintensorError, match="except the first and last one"):
        O.ClosedMPS([T3, T2, T3])
    with pytest.raises(O.QaintensorError, match="^Last tensor must have 2 legs$"):
        O.ClosedMPS([T3, T1, T2])


def test_single_tensor_network_contracts_to_itself():
    # test/test_tensor_circuit.jl:21-31: one tensor, both legs open
    rng = np.random.default_rng(13)
    t = rng.standard_normal((2, 6)) + 1j * rng.standard_normal((2, 6))
    net = O.Network([t], [], [(1, 1), (1, 2)])
    np.testing.assert_allclose(O.contract(net), t, rtol=0, atol=1e-15)


def test_copy_is_independent():
    # test/test_mps.jl:275-288: a copy equals the original, and replacing a
    # tensor of the original leaves the copy alone
    rng = np.random.default_rng(12)
    mps = O.ClosedMPS([rng.random((2, 5)), rng.random((5, 2, 3)), rng.random((3, 2))])
    cp = mps.copy()
    assert all(np.array_equal(x, y) for x, y in zip(cp.tensors, mps.tensors))
    assert cp.contractions == mps.contractions and cp.openidx == mps.openidx
    mps.tensors[0] = rng.random((2, 5))
    assert not np.array_equal(mps.tensors[0], cp.tensors[0])


@pytest.mark.parametrize("seed", [7, 8, 9])
def test_permute_mps(seed):
    # test/test_mps.jl:157-174
    rng = np.random.default_rng(seed)
    n = 6
    b = [randn_c(rng, 2) for _ in range(n)]
    order = list(rng.permutation(n) + 1)
    mps = O.mps_from_state(kron_all(b))
    O.permute_mps(mps, order)
    close(O.contract(mps).reshape(-1, order="F"), kron_all([b[o - 1] for o in order]))


def test_permute_exceptions():
    # test/test_mps.jl:176-199
    rng = np.random.default_rng(10)
    mps = O.mps_from_state(kron_all([randn_c(rng, 2) for _ in range(6)]))
    with pytest.raises(O.QaintensorError, match="same length"):
        O.permute_mps(mps, [1, 2, 3])
    with pytest.raises(O.QaintensorError, match="repeat values"):
        O.permute_mps(mps, [1] * 6)
    with pytest.raises(O.QaintensorError, match="only contain positive"):
        O.permute_mps(mps, [1, -2, 3, 4, -5, 6])
    with pytest.raises(O.QaintensorError, match="cannot exceed"):
        O.permute_mps(mps, [1, 2, 8, 4, 5, 6])


def test_switch_wires():
    # test/test_mps.jl:202-222
    rng = np.random.default_rng(11)
    b = [randn_c(rng, 2) for _ in range(6)]
    order = [1, 3, 2, 5, 6, 4]
    ref, perm = kron_all(b), kron_all([b[o - 1] for o in order])
    mps = O.mps_from_state(ref)
    O.switch_pairs(mps, [(2, 3), (4, 6), (4, 5)])
    close(O.contract(mps).reshape(-1, order="F"), perm)
    mps = O.mps_from_state(ref)
    O.switch_wires(mps, 2, 3)
    O.switch_wires(mps, 4, 6)
    O.switch_wires(mps, 4, 5)
    close(O.contract(mps).reshape(-1, order="F"), perm)


def test_switch_exceptions_and_neighbours():
    # test/test_mps.jl:224-273
    rng = np.random.default_rng(12)
    b = [randn_c(rng, 2) for _ in range(6)]
    mps = O.mps_from_state(kron_all(b))
    with pytest.raises(O.QaintensorError, match="must be positive"):
        O.switch_wires(mps.copy(), 1, -2)
    with pytest.raises(O.QaintensorError, match="less than or equal"):
        O.switch_wires(mps.copy(), 7, 4)
    with pytest.raises(O.QaintensorError, match="must be positive"):
        O.switch_pairs(mps.copy(), [(3, 4), (1, -2)])
    order = [1, 3, 4, 5, 6, 2]
    mps = O.mps_from_state(kron_all(b))
    for i in (4, 3, 2, 1):
        O.switch_adjacent(mps, i)
    close(O.contract(mps).reshape(-1, order="F"), kron_all([b[o - 1] for o in order]))
    with pytest.raises(IndexError):
        O.switch_adjacent(mps, 7)
    with pytest.raises(IndexError):
        O.switch_adjacent(mps, -2)


def controlled(u, nctrl=1):
    d = u.shape[0]
    m = np.eye(d * 2 ** nctrl, dtype=np.complex128)
    m[-d:, -d:] = u
    return m


X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
Z = np.diag([1, -1]).astype(np.complex128)
SWAP = np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


def net3(rng):
    return O.Network([randn_c(rng, 2, 6), randn_c(rng, 2, 6, 7), randn_c(rng, 2, 7)],
                     [O.Summation([(1, 2), (2, 2)]), O.Summation([(2, 3), (3, 2)])],
                     [(1, 1), (2, 1), (3, 1)])


def test_decompose_two_qubit_gates():
    # test/test_tensor_circuit.jl:62-91: controlled X/Y/Z through decompose!,
    # the non-symmetric controlled-Y pins "U acts on the input legs"
    rng = np.random.default_rng(13)
    psi = net3(rng)
    gates = [(controlled(X), (3, 1)), (controlled(Y), (3, 1)), (controlled(Y), (1, 2)), (controlled(Z), (2, 1))]
    ref = O.contract(psi).reshape(-1, order="F")
    for m, w in gates:
        ref = O.apply_statevector(ref, m, w)
    for m, w in gates:
        O.tensor_circuit(psi, m, w, is_decompose=True)
    close(O.contract(psi).reshape(-1, order="F"), ref)


def test_decompose_three_qubit_gates():
    # test/test_tensor_circuit.jl:93-126
    rng = np.random.default_rng(14)
    psi = O.Network([randn_c(rng, 2, 6), randn_c(rng, 2, 6, 7), randn_c(rng, 2, 7, 5), randn_c(rng, 2, 5)],
                    [O.Summation([(1, 2), (2, 2)]), O.Summation([(2, 3), (3, 2)]), O.Summation([(3, 3), (4, 2)])],
                    [(1, 1), (2, 1), (3, 1), (4, 1)])
    gates = [(controlled(SWAP), (4, 1, 3)), (Y, (2,)), (controlled(X), (3, 1)), (Y, (2,)),
             (controlled(X, 2), (4, 1, 2)), (Z, (3,))]
    ref = O.contract(psi).reshape(-1, order="F")
    for m, w in gates:
        ref = O.apply_statevector(ref, m, w)
    for m, w in gates:
        O.tensor_circuit(psi, m, w, is_decompose=True)
    close(O.contract(psi).reshape(-1, order="F"), ref)
