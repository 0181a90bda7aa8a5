"""The bounded device waits end in an error status, not a hang: with the
test hooks QT_JACOBI_STALL_TEST / QT_ORTH_STALL_TEST the Jacobi sweep
kernel's or the one-launch orthonormalisation's CTA 0 waits on a word that
nothing sets; the wait gives up after the given polls, the other CTAs leave
through the abort word, the call returns QT_ETIMEOUT, and the same handle
then computes normally."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def graded(rng, m, n, decay):
    k = min(m, n)
    q1, _ = np.linalg.qr(rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k)))
    q2, _ = np.linalg.qr(rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k)))
    return (q1 * decay ** np.arange(k)) @ q2.conj().T


def test_sweep_kernel_wait_times_out_and_the_handle_recovers(engine, monkeypatch):
    rng = np.random.default_rng(31)
    m, n = 1100, 1003  # FP32 storage, 63 pairs: the one-launch sweep kernel
    M = graded(rng, m, n, 0.97).astype(np.complex64)
    cut = 50 * 4 * np.sqrt(m) * 5.96e-8 * np.linalg.norm(M)  # well above the FP32 resolution
    eng = engine.Engine(mode="chosen", jacobi_kernel=0)
    monkeypatch.setenv("QT_JACOBI_STALL_TEST", "20000")
    with pytest.raises(engine.EngineError) as e:
        eng.truncated_svd(M, cut, mode="chosen")
    assert e.value.code == engine.QT_ETIMEOUT
    monkeypatch.delenv("QT_JACOBI_STALL_TEST")
    U, S, Vh, k, _ = eng.truncated_svd(M, cut, mode="chosen")
    ref = np.linalg.svd(M.astype(np.complex128), compute_uv=False)
    assert k > 0 and np.abs(S - ref[:k]).max() <= 1e-4 * ref[0]
    eng.close()


def test_orthonormalisation_barrier_times_out_and_the_handle_recovers(engine, monkeypatch):
    import oracle as O
    rng = np.random.default_rng(32)
    chi = 512
    a, b, _ = O.decay_theta_factors(chi, rng, 0.97)
    g = O.haar_unitary(rng)
    eng = engine.Engine(mode="chosen", tc_gemm=1)
    p = np.zeros(eng.n_params, dtype=np.float32)
    p[-1] = 1.0  # a rank model predicting the cap: the update is sketched
    eng.set_rank_params(p, enable=True)
    sites = [a.astype(np.complex64), b.astype(np.complex64)]
    m = eng.mps(sites, dtype=np.complex64)
    monkeypatch.setenv("QT_ORTH_STALL_TEST", "20000")
    with pytest.raises(engine.EngineError) as e:
        m.apply_2q(g, 1, 1e-6, chi)
    assert e.value.code == engine.QT_ETIMEOUT
    m.free()
    monkeypatch.delenv("QT_ORTH_STALL_TEST")
    m = eng.mps(sites, dtype=np.complex64)
    st = m.apply_2q(g, 1, 1e-6, chi)
    assert st["sketch_size"] > 0 and st["rank"] == chi and not st["fallback"], st
    m.free()
    eng.close()
