"""Networks built by lazy gate insertion (tensor_circuit!, src/tensor_circuit.jl:14-52,
with and without decompose!) contracted on the GPU by the device-resident ncon
driver, against the oracle's ncon restatement and the dense statevector: the
GPU counterparts of test/test_tensor_circuit.jl:32-126 and test/test_mps.jl:57-88.
Every pairwise step, trace and the final leg order run on the device."""
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
Z = np.diag([1, -1]).astype(np.complex128)
SWAP = np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


def randn_c(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def controlled(u, nctrl=1):
    d = u.shape[0]
    m = np.eye(d * 2 ** nctrl, dtype=np.complex128)
    m[-d:, -d:] = u
    return m


def qft_gates(n):
    h = np.array([[1, 1], [1, -1]]) / math.sqrt(2)
    out = []
    for i in range(n, 0, -1):
        out.append((h, (i,)))
        for j in range(i - 1, 0, -1):
            out.append((np.diag([1, 1, 1, np.exp(1j * math.pi / 2 ** (i - j))]), (i, j)))
    return out


def net_chain(rng, bonds):
    """A general network of len(bonds)+1 tensors with the physical leg first
    (the layout of test/test_tensor_circuit.jl's states)."""
    n = len(bonds) + 1
    tensors, contractions = [], []
    for i in range(n):
        legs = [2] + ([bonds[i - 1]] if i > 0 else []) + ([bonds[i]] if i < n - 1 else [])
        tensors.append(randn_c(rng, *legs))
    for i in range(1, n):
        contractions.append(O.Summation([(i, 3 if i > 1 else 2), (i + 1, 2)]))
    return O.Network(tensors, contractions, [(i, 1) for i in range(1, n + 1)])


def gpu_contract(engine, eng, net, optimize=False):
    return engine.contract(eng, net.tensors, [s.idx for s in net.contractions], net.openidx, optimize=optimize)


def check(got, ref):
    assert got.shape == ref.shape, (got.shape, ref.shape)
    assert np.abs(got - ref).max() <= 1e-11 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("optimize", [False, True])
def test_qft_without_decompose(engine, optimize):
    # test/test_mps.jl:57-88 / test/test_tensor_circuit.jl:32-60: symmetric
    # gates appended as single tensors; plain and optimised order
    rng = np.random.default_rng(21)
    psi = net_chain(rng, [6, 7, 5])
    state = O.contract(psi).reshape(-1, order="F")
    for m, w in qft_gates(4):
        state = O.apply_statevector(state, m, w)
        O.tensor_circuit(psi, m, w)
    eng = engine.Engine(mode="plain")
    got = gpu_contract(engine, eng, psi, optimize)
    check(got, O.contract(psi, optimize))
    np.testing.assert_allclose(got.reshape(-1, order="F"), state, rtol=1e-10, atol=1e-10 * np.abs(state).max())
    eng.close()


def test_decomposed_two_and_three_qubit_gates(engine):
    # test/test_tensor_circuit.jl:62-126: decompose! chains of non-symmetric
    # gates (controlled-Y pins "U acts on the input legs").  A one-qubit gate
    # has no chain: it is inserted as one tensor whose row leg meets the state
    # (src/tensor_circuit.jl:44-51), i.e. as its transpose -- Y^T = -Y here,
    # which the dense reference must apply too
    rng = np.random.default_rng(22)
    psi = net_chain(rng, [6, 7, 5])
    gates = [(controlled(X), (3, 1)), (controlled(Y), (3, 1)), (controlled(Y), (1, 2)), (controlled(Z), (2, 1)),
             (controlled(SWAP), (4, 1, 3)), (Y, (2,)), (controlled(X, 2), (4, 1, 2)), (Z, (3,))]
    state = O.contract(psi).reshape(-1, order="F")
    for m, w in gates:
        state = O.apply_statevector(state, m.T if len(w) == 1 else m, w)
        O.tensor_circuit(psi, m, w, is_decompose=True)
    eng = engine.Engine(mode="plain")
    got = gpu_contract(engine, eng, psi)
    check(got, O.contract(psi))
    np.testing.assert_allclose(got.reshape(-1, order="F"), state, rtol=1e-10, atol=1e-10 * np.abs(state).max())
    eng.close()


def test_undecomposed_nonsymmetric_gate_applies_the_transpose(engine):
    # the reference's lazy insertion without decompose! contracts the gate
    # matrix's row legs with the state (src/tensor_circuit.jl:44-51), i.e.
    # applies U^T; the device contraction of that network does the same
    rng = np.random.default_rng(23)
    psi = net_chain(rng, [4, 4])
    u = O.haar_unitary(rng)
    state = O.contract(psi).reshape(-1, order="F")
    O.tensor_circuit(psi, u, (1, 3))
    eng = engine.Engine(mode="plain")
    got = gpu_contract(engine, eng, psi).reshape(-1, order="F")
    np.testing.assert_allclose(got, O.apply_statevector(state, u.T, (1, 3)), rtol=1e-10, atol=1e-12)
    assert np.abs(got - O.apply_statevector(state, u, (1, 3))).max() > 1e-3
    eng.close()


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_permuted_pairwise_step_on_tensor_cores(engine, dtype):
    # a pairwise step whose operands need real permutes (contracted legs in
    # the middle and at the end, in swapped order), large enough for the
    # complex64 tensor-core path: the permutes are folded into the operand
    # gathers (no permuted copy); complex128 takes the gather + FP64 GEMM
    rng = np.random.default_rng(24)
    A = randn_c(rng, 12, 16, 10, 8).astype(dtype)
    B = randn_c(rng, 8, 9, 16, 6).astype(dtype)
    eng = engine.Engine(mode="chosen" if dtype == np.complex64 else "plain", tc_gemm=1)
    tc0 = eng.work_counters()["tc_launches"]
    ta, tb = eng.tensor(A), eng.tensor(B)
    tcd = ta.contract(tb, [1, 3], [2, 0], out_perm=[3, 0, 2, 1])
    got = tcd.numpy(dtype)
    # natural leg order: A's free legs (a, b), then B's (c, d)
    natural = np.einsum("aibj,jcid->abcd", A.astype(np.complex128), B.astype(np.complex128))
    ref = np.transpose(natural, [3, 0, 2, 1])
    tol = 2e-6 if dtype == np.complex64 else 1e-12
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max() * math.sqrt(128)
    if dtype == np.complex64:
        assert eng.work_counters()["tc_launches"] == tc0 + 1  # the tcgen05 GEMM ran
    # the host-buffer entry point gives the same natural-order product
    np.testing.assert_allclose(eng.contract_pair(A, B, [1, 3], [2, 0]), natural.astype(dtype),
                               rtol=0, atol=tol * np.abs(natural).max() * math.sqrt(128))
    for t in (ta, tb, tcd):
        t.free()
    eng.close()


def test_trace_permute_and_outer_product_on_device(engine):
    rng = np.random.default_rng(25)
    A = randn_c(rng, 3, 5, 3, 4)
    B = randn_c(rng, 2, 3)
    eng = engine.Engine(mode="plain")
    ta, tb = eng.tensor(A), eng.tensor(B)
    tr = ta.trace(0, 2)
    np.testing.assert_allclose(tr.numpy(np.complex128), np.einsum("aiab->ib", A), rtol=1e-13, atol=1e-13)
    pm = ta.permute([2, 0, 3, 1])
    np.testing.assert_allclose(pm.numpy(np.complex128), np.transpose(A, [2, 0, 3, 1]))
    op = tr.contract(tb, [], [])
    np.testing.assert_allclose(op.numpy(np.complex128), np.einsum("ib,cd->ibcd", np.einsum("aiab->ib", A), B),
                               rtol=1e-13, atol=1e-13)
    for t in (ta, tb, tr, pm, op):
        t.free()
    eng.close()
