"""The allocation-free truncated SVD against the regular entry point.

Callers that own all device memory (an embedding framework with its own
arena, code that must not call cudaMalloc) hand the library only their input
and output buffers; here torch plays that caller: it owns the device
buffers, the library uses nothing but its fixed scratch array.  Two calls in
a row (a tall then a wide matrix) must each agree with qt_truncated_svd
within the parity tolerance of the plain FP64 path (1e-12 relative), leave
both factors orthonormal, and change neither the device's free memory nor
torch's allocator.  The largest supported size (256 x 256) works and one row
more is refused with QT_ENOTSUP."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    """Column-major complex128 numpy array -> flat float64 CUDA tensor (interleaved)."""
    flat = np.asfortranarray(a).reshape(-1, order="F").view(np.float64).copy()
    return torch.from_numpy(flat).cuda()


def _host(t, shape):
    return t.cpu().numpy().view(np.complex128).reshape(shape, order="F")


def _graded(rng, m, n, decay):
    q1, _ = np.linalg.qr(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
    q2, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    r = min(m, n)
    return (q1[:, :r] * decay ** np.arange(r)) @ q2[:, :r].conj().T


def test_no_alloc_svd_matches_regular_entry_point(engine):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    rng = np.random.default_rng(2027)
    eng = engine.Engine(mode="plain")
    stream = torch.cuda.current_stream().cuda_stream
    inputs = []
    for (m, n, cutoff, chi_max) in ((96, 80, 1e-10, 0), (64, 130, 1e-3, 40)):
        M = _graded(rng, m, n, 0.85)
        r = min(m, n)
        U0, S0, Vh0, k0, _ = eng.truncated_svd(M, cutoff, chi_max)
        bufs = (_dev(torch, M), torch.zeros(2 * m * r, dtype=torch.float64, device="cuda"),
                torch.zeros(r, dtype=torch.float64, device="cuda"),
                torch.zeros(2 * r * n, dtype=torch.float64, device="cuda"))
        inputs.append((m, n, cutoff, chi_max, M, (U0, S0, Vh0, k0), bufs))
    torch.cuda.synchronize()

    def call_all():
        ks = []
        for (m, n, cutoff, chi_max, M, _, (dM, dU, dS, dVh)) in inputs:
            ks.append(engine.truncated_svd_noalloc(m, n, dM.data_ptr(), cutoff, chi_max, dU.data_ptr(),
                                                   dS.data_ptr(), dVh.data_ptr(), stream))
        torch.cuda.synchronize()
        return ks

    # the first pass loads the kernels and looks up the array's address; the
    # next two calls (the two shapes in a row) must not allocate
    call_all()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    ks = call_all()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert torch.cuda.memory_allocated() == alloc0
    for k, (m, n, cutoff, chi_max, M, (U0, S0, Vh0, k0), (dM, dU, dS, dVh)) in zip(ks, inputs):
        assert k == k0
        S = dS.cpu().numpy()[:k]
        U = _host(dU[: 2 * m * k], (m, k))
        Vh = _host(dVh[: 2 * k * n], (k, n))
        np.testing.assert_allclose(S, S0, rtol=0, atol=1e-12 * S0[0])
        np.testing.assert_allclose(U @ np.diag(S) @ Vh, U0 @ np.diag(S0) @ Vh0, atol=1e-12 * np.linalg.norm(M))
        np.testing.assert_allclose(U.conj().T @ U, np.eye(k), atol=1e-12)
        np.testing.assert_allclose(Vh @ Vh.conj().T, np.eye(k), atol=1e-12)
        np.testing.assert_allclose(_host(dM, (m, n)), M)  # the input is not modified
    eng.close()


def test_no_alloc_limits(engine):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2028)
    stream = torch.cuda.current_stream().cuda_stream
    eng = engine.Engine(mode="plain")
    m = n = 256  # the largest supported shape
    M = _graded(rng, m, n, 0.95)
    U0, S0, Vh0, k0, _ = eng.truncated_svd(M, 1e-9, 0)
    dM, dU = _dev(torch, M), torch.zeros(2 * m * n, dtype=torch.float64, device="cuda")
    dS = torch.zeros(n, dtype=torch.float64, device="cuda")
    dVh = torch.zeros(2 * m * n, dtype=torch.float64, device="cuda")
    k = engine.truncated_svd_noalloc(m, n, dM.data_ptr(), 1e-9, 0, dU.data_ptr(), dS.data_ptr(), dVh.data_ptr(),
                                     stream)
    torch.cuda.synchronize()
    assert k == k0
    np.testing.assert_allclose(dS.cpu().numpy()[:k], S0, rtol=0, atol=1e-12 * S0[0])
    # one row more than the array holds: refused before any work
    big = torch.zeros(2 * 257 * n, dtype=torch.float64, device="cuda")
    with pytest.raises(engine.EngineError) as e:
        engine.truncated_svd_noalloc(257, n, big.data_ptr(), 1e-9, 0, big.data_ptr(), dS.data_ptr(), big.data_ptr(),
                                     stream)
    assert e.value.code == engine.QT_ENOTSUP
    eng.close()
