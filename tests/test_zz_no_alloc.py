"""The allocation-free truncated SVD against the regular entry point.

Callers that own all device memory (an embedding framework with its own
arena, code that must not call cudaMalloc) hand the library only their input
and output buffers; here torch plays that caller: it owns the device
buffers, the library uses nothing but its fixed scratch array.  Two calls in
a row (a tall then a wide matrix) must each agree with qt_truncated_svd
within the parity tolerance of the plain FP64 path (1e-12 relative)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    """Column-major complex128 numpy array -> flat float64 CUDA tensor (interleaved)."""
    flat = np.asfortranarray(a).reshape(-1, order="F").view(np.float64).copy()
    return torch.from_numpy(flat).cuda()


def _host(t, shape):
    return t.cpu().numpy().view(np.complex128).reshape(shape, order="F")


@pytest.mark.parametrize("repeat", [0])
def test_no_alloc_svd_matches_regular_entry_point(engine, repeat):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    rng = np.random.default_rng(2027)
    eng = engine.Engine(mode="plain")
    stream = torch.cuda.current_stream().cuda_stream
    for (m, n, cutoff, chi_max) in ((96, 80, 1e-10, 0), (64, 130, 1e-3, 40)):
        q1, _ = np.linalg.qr(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
        q2, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
        r = min(m, n)
        s = 0.85 ** np.arange(r)
        M = (q1[:, :r] * s) @ q2[:, :r].conj().T
        U0, S0, Vh0, k0, _ = eng.truncated_svd(M, cutoff, chi_max)
        dM = _dev(torch, M)
        dU = torch.zeros(2 * m * r, dtype=torch.float64, device="cuda")
        dS = torch.zeros(r, dtype=torch.float64, device="cuda")
        dVh = torch.zeros(2 * r * n, dtype=torch.float64, device="cuda")
        k = engine.truncated_svd_noalloc(m, n, dM.data_ptr(), cutoff, chi_max, dU.data_ptr(), dS.data_ptr(),
                                         dVh.data_ptr(), stream)
        torch.cuda.synchronize()
        assert k == k0
        S = dS.cpu().numpy()[:k]
        U = _host(dU[: 2 * m * k], (m, k))
        Vh = _host(dVh[: 2 * k * n], (k, n))
        np.testing.assert_allclose(S, S0, rtol=0, atol=1e-12 * S0[0])
        np.testing.assert_allclose(U @ np.diag(S) @ Vh, U0 @ np.diag(S0) @ Vh0, atol=1e-12 * np.linalg.norm(M))
        np.testing.assert_allclose(U.conj().T @ U, np.eye(k), atol=1e-12)
        np.testing.assert_allclose(_host(dM, (m, n)), M)  # the input is not modified
    eng.close()
