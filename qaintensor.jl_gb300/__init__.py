"""Host-side mirror of Qaintensor.jl's contraction / truncated-SVD API over the
GB300 engine's C ABI (``libqaintensor_gb300.so``, declared in
``include/qaintensor_gb300.h``).

Names, argument meaning and error messages follow the Julia entry points:
``contract_svd(T1, T2, (i1, i2); er)`` (src/svd.jl:7-38), ``switch!``
(src/switch.jl), and the eager two-qubit update ``apply_2q!`` that the
engine adds on top of ``tensor_circuit!``'s gate convention.  Wire and site
numbers are 1-based here, as in Julia; the C ABI is 0-based.

There is no CPU fallback: importing works anywhere, but creating an
``Engine`` loads the CUDA library and raises if it is missing or no GPU is
usable.
"""

from __future__ import annotations

import ctypes as C
import math
import os
from typing import List, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libqaintensor_gb300.so")

QT_OK, QT_EINVAL_ERR_NEG, QT_EDIM_MISMATCH, QT_ENOMEM, QT_ECUDA, QT_ETIMEOUT, QT_ENUMERIC, \
    QT_EFALLBACK_FAILED, QT_EINVAL, QT_EPERIODIC, QT_EBOUNDS, QT_ENOTSUP = 0, -1, -2, -3, -4, -5, -6, -7, -8, -9, -10, -11
QT_C64, QT_C128 = 0, 1
MODES = {"plain": 0, "chosen": 1, "cusolver": 2}

# the reference's own messages for the codes that have one
REFERENCE_MESSAGES = {
    QT_EINVAL_ERR_NEG: "Error must be positive",                                  # src/svd.jl:9, src/mps.jl:192
    QT_EDIM_MISMATCH: "Dimensions of contraction legs do not match",              # src/svd.jl:16
    QT_EPERIODIC: "Function doesn't support periodic boundary conditions for now",  # src/mps.jl:195
}


class QaintensorError(ValueError):
    """An error the reference raises as ErrorException(msg); ``str(e)`` is msg."""

    def __init__(self, msg: str, code: int = QT_EINVAL):
        super().__init__(msg)
        self.code = code


class QaintensorBoundsError(IndexError):
    """Out-of-range site (the reference's BoundsError)."""


class EngineError(RuntimeError):
    """A device-side failure (CUDA, allocation, numerics)."""

    def __init__(self, msg: str, code: int):
        super().__init__(msg)
        self.code = code


CERT_NAMES = ("fallback", "resolved", "cap", "struct")


class QtConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("mode", C.c_int), ("cutoff", C.c_double), ("chi_max", C.c_int),
                ("oversample", C.c_int), ("power_iters", C.c_int), ("renormalize", C.c_int),
                ("use_rank_model", C.c_int), ("max_sweeps", C.c_int), ("jacobi_tol", C.c_double),
                ("noise_floor", C.c_double), ("seed", C.c_uint64), ("tc_gemm", C.c_int),
                ("jacobi_kernel", C.c_int), ("cap_sketch", C.c_double)]


class QtUpdateStats(C.Structure):
    _fields_ = [("rank", C.c_int), ("rank_cutoff", C.c_int), ("predicted_rank", C.c_int), ("sketch_size", C.c_int),
                ("fallback", C.c_int), ("sweeps", C.c_int), ("discarded_weight", C.c_double),
                ("norm2", C.c_double), ("residual", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def library() -> C.CDLL:
    """Load the engine library (once).  Raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"CUDA engine not built: {LIB_PATH} is missing (run __graft_entry__.build())")
    lib = C.CDLL(LIB_PATH)
    P, I, D, L = C.c_void_p, C.c_int, C.c_double, C.c_int64
    sig = {
        "qt_config_default": (I, [C.POINTER(QtConfig)]),
        "qt_create": (I, [C.POINTER(P), C.POINTER(QtConfig)]),
        "qt_destroy": (I, [P]),
        "qt_last_error": (C.c_char_p, [P]),
        "qt_abi_version": (I, []),
        "qt_launch_count": (L, [P]),
        "qt_work_counters": (I, [P, C.POINTER(D)]),
        "qt_cert_counters": (I, [P, C.POINTER(L)]),
        "qt_gemm": (I, [P, I, I, I, L, L, L, C.POINTER(D), P, L, P, L, C.POINTER(D), P, L]),
        "qt_contract_pair": (I, [P, I, I, C.POINTER(L), P, I, C.POINTER(L), P, I, C.POINTER(I), C.POINTER(I), P]),
        "qt_tensor_create": (I, [P, I, I, C.POINTER(L), P, C.POINTER(P)]),
        "qt_tensor_free": (I, [P, P]),
        "qt_tensor_ndims": (I, [P]),
        "qt_tensor_dims": (I, [P, C.POINTER(L)]),
        "qt_tensor_download": (I, [P, P, P]),
        "qt_tensor_contract": (I, [P, P, P, I, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(P)]),
        "qt_tensor_permute": (I, [P, P, C.POINTER(I), C.POINTER(P)]),
        "qt_tensor_trace": (I, [P, P, I, I, C.POINTER(P)]),
        "qt_truncated_svd": (I, [P, I, L, L, P, D, I, I, P, C.POINTER(D), P, C.POINTER(I), C.POINTER(D)]),
        "qt_contract_svd": (I, [P, I, I, C.POINTER(L), P, I, C.POINTER(L), P, I, I, D, P]),
        "qt_mps_create": (I, [P, I, C.POINTER(L), C.POINTER(P), I, C.POINTER(P)]),
        "qt_mps_free": (I, [P, P]),
        "qt_mps_nsites": (I, [P]),
        "qt_mps_site_dims": (I, [P, I, C.POINTER(L)]),
        "qt_mps_download": (I, [P, P, I, P]),
        "qt_mps_upload_site": (I, [P, P, I, C.POINTER(L), P]),
        "qt_apply_2q": (I, [P, P, I, C.POINTER(D), D, I, I, C.POINTER(QtUpdateStats)]),
        "qt_switch": (I, [P, P, I]),
        "qt_expect_z": (I, [P, P, I, C.POINTER(D)]),
        "qt_expect_zz": (I, [P, P, I, C.POINTER(D)]),
        "qt_mps_norm2": (I, [P, P, C.POINTER(D)]),
        "qt_rank_model_set_logging": (I, [P, I]),
        "qt_rank_model_log_size": (L, [P]),
        "qt_rank_model_get_log": (I, [P, P, P]),
        "qt_rank_model_clear_log": (I, [P]),
        "qt_rank_model_set_params": (I, [P, P, I, I]),
        "qt_rank_model_get_params": (I, [P, P, I]),
        "qt_rank_model_enable": (I, [P, I]),
        "qt_rank_model_set_margin": (I, [P, D]),
        "qt_rank_model_nparams": (I, []),
        "qt_rank_model_train": (I, [P, L, P, P, P, I, I, D, C.c_uint64, C.POINTER(D)]),
        "qt_mlp_forward": (I, [P, L, P, P]),
        "qt_mlp_loss_grad": (I, [P, L, P, P, P, P, C.POINTER(D)]),
        "qt_rank_features_of": (I, [P, I, C.POINTER(D), D, I, P]),
        "qt_mps_set_bond_spectrum": (I, [P, I, C.POINTER(D), I]),
        "qt_mps_set_circuit_position": (I, [P, I, I]),
        "qt_mps_clone": (I, [P, P, C.POINTER(P)]),
        "qt_timer_record": (I, [P, I]),
        "qt_timer_elapsed": (I, [P, I, I, C.POINTER(D)]),
        "qt_sync": (I, [P]),
        "qt_l2_flush": (I, [P]),
        "qt_profile_enable": (I, [P, I]),
        "qt_profile_collect": (I, [P]),
        "qt_profile_get": (I, [I, C.c_char_p, I, C.POINTER(L), C.POINTER(D)]),
        "qt_host_alloc": (P, [C.c_size_t]),
        "qt_host_free": (I, [P]),
        "qt_batch_create": (I, [P, I, P, P, C.POINTER(P)]),
        "qt_batch_free": (I, [P, P]),
        "qt_batch_run": (I, [P, P, I, P, P, P, P, D, I]),
        "qt_batch_replay": (I, [P, P]),
        "qt_batch_reset": (I, [P, P]),
        "qt_batch_task_stats": (I, [P, P, P, P, P]),
        "qt_batch_cert_counts": (I, [P, P, C.POINTER(L)]),
        "qt_batch_set_launch": (I, [P, P, I, I, I]),
        "qt_batch_get_launch": (I, [P, I, C.POINTER(I), C.POINTER(I)]),
        "qt_batch_bond_dims": (I, [P, P, I, P]),
        "qt_batch_download_site": (I, [P, P, I, I, P]),
        "qt_batch_expect_z": (I, [P, P, I, P]),
        "qt_truncated_svd_noalloc": (I, [L, L, P, D, I, P, P, P, C.POINTER(I), P]),
        "qt_mps_apply_mpo": (I, [P, P, C.POINTER(P), C.POINTER(L)]),
        "qt_mps_compress": (I, [P, P, D, I, I, I, P, P]),
        "qt_mps_expect_mpo": (I, [P, P, C.POINTER(P), C.POINTER(L), C.POINTER(D)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _dtype_code(dt) -> int:
    dt = np.dtype(dt)
    if dt == np.complex64:
        return QT_C64
    if dt == np.complex128:
        return QT_C128
    raise QaintensorError(f"unsupported dtype {dt}: use complex64 or complex128")


def _np_dtype(code: int):
    return np.complex64 if code == QT_C64 else np.complex128


def _gate_arg(g) -> C.Array:
    g = np.asfortranarray(np.asarray(g, dtype=np.complex128))
    if g.shape != (4, 4):
        raise QaintensorError("a two-qubit gate must be a 4x4 matrix")
    flat = np.empty(32, dtype=np.float64)
    gf = g.reshape(-1, order="F")
    flat[0::2], flat[1::2] = gf.real, gf.imag
    return (C.c_double * 32)(*flat)


class Engine:
    """One engine handle: one CUDA stream on one device (not thread-safe)."""

    def __init__(self, mode: str = "plain", cutoff: float = 0.0, chi_max: int = 0, device: int = 0, **kw):
        lib = library()
        cfg = QtConfig()
        lib.qt_config_default(C.byref(cfg))
        cfg.device, cfg.mode, cfg.cutoff, cfg.chi_max = device, MODES[mode], cutoff, chi_max
        for k, v in kw.items():
            if not hasattr(cfg, k):
                raise TypeError(f"unknown engine option {k}")
            setattr(cfg, k, v)
        self._lib = lib
        self._h = C.c_void_p()
        rc = lib.qt_create(C.byref(self._h), C.byref(cfg))
        if rc != QT_OK:
            raise EngineError(f"qt_create failed with status {rc} (is a CUDA GPU visible?)", rc)
        self.config = cfg

    # -- plumbing -------------------------------------------------------------
    def _check(self, rc: int):
        if rc == QT_OK:
            return
        msg = self._lib.qt_last_error(self._h).decode()
        if rc in REFERENCE_MESSAGES:
            raise QaintensorError(REFERENCE_MESSAGES[rc], rc)
        if rc == QT_EBOUNDS:
            raise QaintensorBoundsError(msg)
        if rc in (QT_EINVAL,):
            raise QaintensorError(msg, rc)
        raise EngineError(f"{msg} (status {rc})", rc)

    def close(self):
        if self._h:
            self._lib.qt_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        """Kernel launches issued by this handle so far."""
        return int(self._lib.qt_launch_count(self._h))

    # -- measurement ----------------------------------------------------------
    def timer_record(self, slot: int):
        """Record CUDA event `slot` (0..7) on the handle's stream."""
        self._check(self._lib.qt_timer_record(self._h, slot))

    def timer_elapsed(self, a: int, b: int) -> float:
        ms = C.c_double()
        self._check(self._lib.qt_timer_elapsed(self._h, a, b, C.byref(ms)))
        return ms.value

    def work_counters(self) -> dict:
        """Cumulative algorithmic work: Jacobi bytes/rounds, tensor-core TF32 flops/launches."""
        out = (C.c_double * 8)()
        self._check(self._lib.qt_work_counters(self._h, out))
        return {"jacobi_bytes": out[0], "jacobi_rounds": out[1], "tc_flops": out[2], "tc_launches": out[3],
                "jacobi_pairs": out[4], "jacobi_inner_sweeps": out[5], "jacobi_gram_bytes": out[6],
                "jacobi_rot_bytes": out[7]}

    def cert_counters(self) -> dict:
        """Chosen-mode rank decisions since creation, by how they were decided:
        ``fallback`` (exact FP64 split, no certificate), ``resolved`` (cutoff at
        or above the FP32 resolution), ``cap`` (chi_max binds with margin),
        ``struct`` (the exact rank bound is met)."""
        out = (C.c_int64 * 4)()
        self._check(self._lib.qt_cert_counters(self._h, out))
        return dict(zip(CERT_NAMES, (int(v) for v in out)))

    def sync(self):
        self._check(self._lib.qt_sync(self._h))

    def l2_flush(self):
        """Write 256 MiB on the device (evicts L2) on the handle's stream."""
        self._check(self._lib.qt_l2_flush(self._h))

    def profile_enable(self, on: bool = True):
        self._check(self._lib.qt_profile_enable(self._h, int(on)))

    def profile_collect(self):
        """[(kernel name, launches, total device ms)] of the launches recorded
        since profile_enable(True), longest first."""
        n = self._lib.qt_profile_collect(self._h)
        if n < 0:
            self._check(n)
        out = []
        buf = C.create_string_buffer(256)
        for i in range(n):
            cnt, ms = C.c_int64(), C.c_double()
            self._lib.qt_profile_get(i, buf, 256, C.byref(cnt), C.byref(ms))
            out.append((buf.value.decode(), cnt.value, ms.value))
        return sorted(out, key=lambda r: -r[2])

    def pinned_empty(self, shape, dtype, order="F") -> np.ndarray:
        """A numpy array over pinned (page-locked) host memory, freed with the array."""
        dt = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dt.itemsize
        p = self._lib.qt_host_alloc(nbytes)
        if not p:
            raise EngineError("pinned host allocation failed", QT_ENOMEM)
        buf = (C.c_byte * nbytes).from_address(p)
        arr = np.frombuffer(buf, dtype=dt).reshape(shape, order=order)
        lib = self._lib

        class _Owner:
            def __del__(self_inner):
                lib.qt_host_free(C.c_void_p(p))

        arr_base = _Owner()
        arr = arr.view(_PinnedArray)
        arr._owner = arr_base
        return arr

    # -- MPS ------------------------------------------------------------------
    def mps(self, sites: Sequence[np.ndarray], dtype=np.complex128) -> "DeviceMPS":
        """Upload 3-leg sites (chiL, 2, chiR); 2-leg end tensors (2, chi) /
        (chi, 2) of the reference's MPS are accepted and reshaped."""
        n = len(sites)
        arrs = []
        for i, t in enumerate(sites):
            t = np.asarray(t)
            if t.ndim == 2:
                t = t.reshape((1,) + t.shape, order="F") if i == 0 else t.reshape(t.shape + (1,), order="F")
            arrs.append(np.asfortranarray(t.astype(dtype, copy=False)))
        dims = (C.c_int64 * (3 * n))(*[d for t in arrs for d in t.shape])
        ptrs = (C.c_void_p * n)(*[t.ctypes.data for t in arrs])
        out = C.c_void_p()
        self._check(self._lib.qt_mps_create(self._h, n, dims, ptrs, _dtype_code(dtype), C.byref(out)))
        return DeviceMPS(self, out, _dtype_code(dtype))

    def product_state(self, n: int, dtype=np.complex128) -> "DeviceMPS":
        """|0...0> on n sites of bond dimension 1."""
        dims = (C.c_int64 * (3 * n))(*([1, 2, 1] * n))
        out = C.c_void_p()
        self._check(self._lib.qt_mps_create(self._h, n, dims, None, _dtype_code(dtype), C.byref(out)))
        return DeviceMPS(self, out, _dtype_code(dtype))

    # -- dense primitives -----------------------------------------------------
    def contract_pair(self, A: np.ndarray, B: np.ndarray, axesA: Sequence[int], axesB: Sequence[int]) -> np.ndarray:
        """ncon pairwise step: contract axesA of A with axesB of B (0-based);
        the result's legs are A's free legs then B's (column-major)."""
        dt = np.result_type(A.dtype, B.dtype, np.complex64)
        A = np.asfortranarray(A.astype(dt))
        B = np.asfortranarray(B.astype(dt))
        nc = len(axesA)
        free = [A.shape[i] for i in range(A.ndim) if i not in axesA] + [B.shape[i] for i in range(B.ndim) if i not in axesB]
        out = np.zeros(free if free else [1], dtype=dt, order="F")
        dA = (C.c_int64 * A.ndim)(*A.shape)
        dB = (C.c_int64 * B.ndim)(*B.shape)
        self._check(self._lib.qt_contract_pair(self._h, _dtype_code(dt), A.ndim, dA, _ptr(A), B.ndim, dB, _ptr(B), nc,
                                               (C.c_int * nc)(*axesA), (C.c_int * nc)(*axesB), _ptr(out)))
        return out

    def tensor(self, data, dtype=None) -> "DeviceTensor":
        """A device-resident copy of a host tensor (column-major)."""
        return DeviceTensor(self, data, dtype)

    def gemm(self, A: np.ndarray, B: np.ndarray, opA: str = "N", opB: str = "N", alpha=1.0, beta=0.0, out=None):
        """alpha op(A) op(B) + beta out on the device (op "N" or "C"); complex64 or complex128."""
        dt = np.result_type(A.dtype, B.dtype, np.complex64)
        A = np.asfortranarray(A.astype(dt))
        B = np.asfortranarray(B.astype(dt))
        M = A.shape[0] if opA == "N" else A.shape[1]
        K = A.shape[1] if opA == "N" else A.shape[0]
        N = B.shape[1] if opB == "N" else B.shape[0]
        R = np.zeros((M, N), dtype=dt, order="F") if out is None else np.array(out, dtype=dt, order="F")
        alp = (C.c_double * 2)(float(np.real(alpha)), float(np.imag(alpha)))
        bet = (C.c_double * 2)(float(np.real(beta)), float(np.imag(beta)))
        ops = {"N": 0, "C": 2}
        self._check(self._lib.qt_gemm(self._h, _dtype_code(dt), ops[opA], ops[opB], M, N, K, alp, _ptr(A), A.shape[0],
                                      _ptr(B), B.shape[0], bet, _ptr(R), M))
        return R

    def truncated_svd(self, M: np.ndarray, cutoff: float = 0.0, chi_max: int = 0, mode: str = "plain"):
        """Exact truncated SVD (tail rule of src/svd.jl:29-33): (U, S, Vh, k, discarded)."""
        M = np.asarray(M)
        dt = M.dtype if M.dtype in (np.complex64, np.complex128) else np.complex128
        M = np.asfortranarray(M.astype(dt))
        m, n = M.shape
        kc = min(m, n)
        U = np.zeros((m, kc), dtype=dt, order="F")
        Vh = np.zeros((kc, n), dtype=dt, order="F")
        S = np.zeros(kc)
        k = C.c_int()
        disc = C.c_double()
        self._check(self._lib.qt_truncated_svd(self._h, _dtype_code(dt), m, n, _ptr(M), float(cutoff), int(chi_max),
                                               MODES[mode], _ptr(U), S.ctypes.data_as(C.POINTER(C.c_double)),
                                               _ptr(Vh), C.byref(k), C.byref(disc)))
        kk = k.value
        return U[:, :kk], S[:kk], Vh[:kk, :], kk, disc.value

    def contract_svd(self, T1: np.ndarray, T2: np.ndarray, indx, er: float = 0.0) -> np.ndarray:
        """``contract_svd(T1, T2, (i1, i2); er)`` of src/svd.jl:7-38 (1-based legs)."""
        if not er >= 0:
            raise QaintensorError("Error must be positive", QT_EINVAL_ERR_NEG)
        i1, i2 = indx
        dt = np.result_type(T1.dtype, T2.dtype, np.complex64)
        T1 = np.asfortranarray(T1.astype(dt))
        T2 = np.asfortranarray(T2.astype(dt))
        d1 = T1.shape[i1 - 1] if i1 <= T1.ndim else 1
        d2 = T2.shape[i2 - 1] if i2 <= T2.ndim else 1
        if d1 != d2:
            raise QaintensorError("Dimensions of contraction legs do not match", QT_EDIM_MISMATCH)
        newdim = list(T1.shape[: i1 - 1]) + list(T1.shape[i1:]) + list(T2.shape[: i2 - 1]) + list(T2.shape[i2:])
        out = np.zeros(newdim, dtype=dt, order="F")
        self._check(self._lib.qt_contract_svd(self._h, _dtype_code(dt), T1.ndim, (C.c_int64 * T1.ndim)(*T1.shape),
                                              _ptr(T1), T2.ndim, (C.c_int64 * T2.ndim)(*T2.shape), _ptr(T2),
                                              int(i1), int(i2), float(er), _ptr(out)))
        return out

    # -- learned rank ---------------------------------------------------------
    def set_rank_logging(self, on: bool = True):
        self._check(self._lib.qt_rank_model_set_logging(self._h, int(on)))

    def rank_log(self):
        n = int(self._lib.qt_rank_model_log_size(self._h))
        X = np.zeros((n, 16), dtype=np.float32)
        Y = np.zeros(n, dtype=np.float32)
        if n:
            self._check(self._lib.qt_rank_model_get_log(self._h, _ptr(X), _ptr(Y)))
        return X, Y

    def clear_rank_log(self):
        self._check(self._lib.qt_rank_model_clear_log(self._h))

    @property
    def n_params(self) -> int:
        return int(self._lib.qt_rank_model_nparams())

    def set_rank_params(self, p: np.ndarray, enable: bool = True):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self._lib.qt_rank_model_set_params(self._h, _ptr(p), p.size, int(enable)))

    def rank_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, dtype=np.float32)
        self._check(self._lib.qt_rank_model_get_params(self._h, _ptr(p), p.size))
        return p

    def enable_rank_model(self, on: bool = True):
        self._check(self._lib.qt_rank_model_enable(self._h, int(on)))

    def set_rank_margin(self, margin: float):
        self._check(self._lib.qt_rank_model_set_margin(self._h, float(margin)))

    def train_rank_model(self, X, Y, epochs=30, batch=256, lr=1e-3, seed=0, init=None) -> float:
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        init_p = None if init is None else np.ascontiguousarray(init, dtype=np.float32)
        loss = C.c_double()
        self._check(self._lib.qt_rank_model_train(self._h, X.shape[0], _ptr(X), _ptr(Y),
                                                  None if init_p is None else _ptr(init_p), int(epochs), int(batch),
                                                  float(lr), int(seed), C.byref(loss)))
        return loss.value

    def mlp_forward(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros(X.shape[0], dtype=np.float32)
        self._check(self._lib.qt_mlp_forward(self._h, X.shape[0], _ptr(X), _ptr(out)))
        return out

    def mlp_loss_grad(self, X, Y, params):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        p = np.ascontiguousarray(params, dtype=np.float32)
        g = np.zeros_like(p)
        loss = C.c_double()
        self._check(self._lib.qt_mlp_loss_grad(self._h, X.shape[0], _ptr(X), _ptr(Y), _ptr(p), _ptr(g), C.byref(loss)))
        return loss.value, g


class _PinnedArray(np.ndarray):
    """ndarray view that keeps its pinned host allocation alive."""
    pass


class DeviceMPS:
    """An MPS resident in device memory; sites are (chiL, 2, chiR)."""

    def __init__(self, eng: Engine, ptr: C.c_void_p, dtype_code: int):
        self.eng, self._p, self.dtype_code = eng, ptr, dtype_code

    @property
    def nsites(self) -> int:
        return int(self.eng._lib.qt_mps_nsites(self._p))

    def dims(self, i: int):
        """Dims of site i (1-based)."""
        d = (C.c_int64 * 3)()
        rc = self.eng._lib.qt_mps_site_dims(self._p, i - 1, d)
        if rc == QT_EBOUNDS:
            raise QaintensorBoundsError(f"site {i} out of range")
        return tuple(d)

    def clone(self) -> "DeviceMPS":
        """Device-to-device copy."""
        out = C.c_void_p()
        self.eng._check(self.eng._lib.qt_mps_clone(self.eng._h, self._p, C.byref(out)))
        return DeviceMPS(self.eng, out, self.dtype_code)

    def download_into(self, i: int, out: np.ndarray):
        """Download site i (1-based) into a preallocated column-major array."""
        self.eng._check(self.eng._lib.qt_mps_download(self.eng._h, self._p, i - 1, _ptr(out)))

    def site(self, i: int) -> np.ndarray:
        """Download site i (1-based) as a (chiL, 2, chiR) column-major array."""
        out = np.zeros(self.dims(i), dtype=_np_dtype(self.dtype_code), order="F")
        self.eng._check(self.eng._lib.qt_mps_download(self.eng._h, self._p, i - 1, _ptr(out)))
        return out

    def sites(self) -> List[np.ndarray]:
        return [self.site(i) for i in range(1, self.nsites + 1)]

    def upload_site(self, i: int, t: np.ndarray):
        t = np.asfortranarray(np.asarray(t, dtype=_np_dtype(self.dtype_code)))
        self.eng._check(self.eng._lib.qt_mps_upload_site(self.eng._h, self._p, i - 1, (C.c_int64 * 3)(*t.shape), _ptr(t)))

    def apply_2q(self, gate, i: int, cutoff: Optional[float] = None, chi_max: Optional[int] = None,
                 mode: Optional[str] = None) -> dict:
        """``apply_2q!(mps, G, i)``: gate G on wires (i, i+1), truncated SVD split."""
        st = QtUpdateStats()
        rc = self.eng._lib.qt_apply_2q(self.eng._h, self._p, i - 1, _gate_arg(gate),
                                       -1.0 if cutoff is None else float(cutoff),
                                       -1 if chi_max is None else int(chi_max),
                                       -1 if mode is None else MODES[mode], C.byref(st))
        self.eng._check(rc)
        return st.as_dict()

    def switch(self, i: int):
        """``switch!(mps, i)`` (src/switch.jl:18-56): swap the physical legs of sites i, i+1."""
        self.eng._check(self.eng._lib.qt_switch(self.eng._h, self._p, i - 1))

    def switch_wires(self, i: int, j: int):
        """``switch!(mps, i, j)`` (src/switch.jl:63-86): wire
        numbers count from the far end (i -> L - i + 1) and the swap runs as a
        ladder of adjacent swaps up, then down."""
        if not (i > 0 and j > 0):
            raise QaintensorError("Wire indices `i` and `j` must be positive")
        L = self.nsites
        if not (i <= L and j <= L):
            raise QaintensorError("Indices to swap `i` and `j` must be less than or equal to the number of open "
                                  "wires in MPS")
        if i == j:
            return
        i, j = L - i + 1, L - j + 1
        lo, hi = min(i, j), max(i, j)
        for s in range(lo, hi):
            self.switch(s)
        for s in range(hi - 2, lo - 1, -1):
            self.switch(s)

    def permute(self, order):
        """``Base.permute!(mps, order)`` (src/switch.jl:94-106)."""
        order = list(order)
        n = self.nsites
        if len(order) != n:
            raise QaintensorError("Given permutation must be same length as number of Tensors in MPS")
        if len(set(order)) != len(order):
            raise QaintensorError("Permutation order cannot contain repeat values")
        if not all(x > 0 for x in order):
            raise QaintensorError("Permutation order can only contain positive values")
        if max(order) != len(order):
            raise QaintensorError("Wire numbers in permutation order cannot exceed number of wires in MPS")
        seq = list(range(1, n + 1))
        for i in range(1, n + 1):
            loc = seq.index(order[i - 1]) + 1
            self.switch_wires(i, loc)
            seq[loc - 1], seq[i - 1] = seq[i - 1], seq[loc - 1]

    def expect_z(self, i: int) -> float:
        out = C.c_double()
        self.eng._check(self.eng._lib.qt_expect_z(self.eng._h, self._p, i - 1, C.byref(out)))
        return out.value

    def expect_zz(self, i: int) -> float:
        out = C.c_double()
        self.eng._check(self.eng._lib.qt_expect_zz(self.eng._h, self._p, i - 1, C.byref(out)))
        return out.value

    def norm2(self) -> float:
        out = C.c_double()
        self.eng._check(self.eng._lib.qt_mps_norm2(self.eng._h, self._p, C.byref(out)))
        return out.value

    def set_bond_spectrum(self, bond: int, s):
        s = np.ascontiguousarray(s, dtype=np.float64)
        rc = self.eng._lib.qt_mps_set_bond_spectrum(self._p, bond - 1, s.ctypes.data_as(C.POINTER(C.c_double)), s.size)
        self.eng._check(rc)

    def set_circuit_position(self, layer: int, depth: int):
        self.eng._check(self.eng._lib.qt_mps_set_circuit_position(self._p, int(layer), int(depth)))

    @staticmethod
    def _mpo_args(mpo):
        ws = [np.asfortranarray(np.asarray(w, dtype=np.complex128)) for w in mpo]
        dims = (C.c_int64 * (4 * len(ws)))(*[d for w in ws for d in w.shape])
        ptrs = (C.c_void_p * len(ws))(*[w.ctypes.data for w in ws])
        return ws, ptrs, dims

    def apply_mpo(self, mpo):
        """Contract MPO sites (bL, out, in, bR) into this MPS (bond chi*b)."""
        ws, ptrs, dims = self._mpo_args(mpo)
        self.eng._check(self.eng._lib.qt_mps_apply_mpo(self.eng._h, self._p, ptrs, dims))

    def compress(self, cutoff: float, chi_max: int, mode: str = "plain", normalize: bool = True):
        """QR left-canonicalisation, optional normalisation, right-to-left truncation."""
        n = self.nsites
        ranks = np.zeros(max(n - 1, 1), dtype=np.int32)
        disc = np.zeros(max(n - 1, 1), dtype=np.float64)
        self.eng._check(self.eng._lib.qt_mps_compress(self.eng._h, self._p, float(cutoff), int(chi_max), MODES[mode],
                                                      int(normalize), _ptr(ranks), _ptr(disc)))
        return ranks[: n - 1], disc[: n - 1]

    def expect_mpo(self, mpo) -> float:
        ws, ptrs, dims = self._mpo_args(mpo)
        out = C.c_double()
        self.eng._check(self.eng._lib.qt_mps_expect_mpo(self.eng._h, self._p, ptrs, dims, C.byref(out)))
        return out.value

    def rank_features(self, gate, i: int, cutoff: float, chi_max: int) -> np.ndarray:
        f = np.zeros(16, dtype=np.float32)
        self.eng._check(self.eng._lib.qt_rank_features_of(self._p, i - 1, _gate_arg(gate), float(cutoff),
                                                          int(chi_max), _ptr(f)))
        return f

    def free(self):
        if self._p:
            self.eng._lib.qt_mps_free(self.eng._h, self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            if self.eng._h:
                self.free()
        except Exception:
            pass


class DeviceTensor:
    """A column-major complex tensor resident in the engine's device memory
    (``qt_tensor``): the operand of ncon's pairwise steps on the GPU."""

    def __init__(self, eng: "Engine", data=None, dtype=None, _handle=None):
        self.eng = eng
        if _handle is not None:
            self._p = _handle
        else:
            a = np.asarray(data)
            dt = np.dtype(dtype) if dtype is not None else np.result_type(a.dtype, np.complex64)
            a = np.asfortranarray(a.astype(dt))
            dims = (C.c_int64 * max(a.ndim, 1))(*a.shape)
            self._p = C.c_void_p()
            eng._check(eng._lib.qt_tensor_create(eng._h, _dtype_code(dt), a.ndim, dims, _ptr(a), C.byref(self._p)))
        nd = eng._lib.qt_tensor_ndims(self._p)
        dims = (C.c_int64 * max(nd, 1))()
        eng._lib.qt_tensor_dims(self._p, dims)
        self.shape = tuple(int(dims[i]) for i in range(nd))

    @property
    def ndim(self) -> int:
        return len(self.shape)

    def contract(self, other: "DeviceTensor", axes_self: Sequence[int], axes_other: Sequence[int],
                 out_perm: Optional[Sequence[int]] = None) -> "DeviceTensor":
        """The ncon pairwise step on the device: legs axes_self of this
        tensor with axes_other of ``other`` (0-based); result legs: this
        tensor's free legs then ``other``'s, reordered by ``out_perm``."""
        nc = len(axes_self)
        p = C.c_void_p()
        perm = None if out_perm is None else (C.c_int * max(len(out_perm), 1))(*out_perm)
        self.eng._check(self.eng._lib.qt_tensor_contract(self.eng._h, self._p, other._p, nc,
                                                         (C.c_int * max(nc, 1))(*axes_self),
                                                         (C.c_int * max(nc, 1))(*axes_other), perm, C.byref(p)))
        return DeviceTensor(self.eng, _handle=p)

    def trace(self, ax1: int, ax2: int) -> "DeviceTensor":
        p = C.c_void_p()
        self.eng._check(self.eng._lib.qt_tensor_trace(self.eng._h, self._p, ax1, ax2, C.byref(p)))
        return DeviceTensor(self.eng, _handle=p)

    def permute(self, perm: Sequence[int]) -> "DeviceTensor":
        p = C.c_void_p()
        self.eng._check(self.eng._lib.qt_tensor_permute(self.eng._h, self._p,
                                                        (C.c_int * max(len(perm), 1))(*perm), C.byref(p)))
        return DeviceTensor(self.eng, _handle=p)

    def numpy(self, dtype) -> np.ndarray:
        out = np.zeros(self.shape if self.shape else (1,), dtype=dtype, order="F")
        self.eng._check(self.eng._lib.qt_tensor_download(self.eng._h, self._p, _ptr(out)))
        return out if self.shape else out.reshape(())

    def free(self):
        if self._p and self.eng._h:
            self.eng._lib.qt_tensor_free(self.eng._h, self._p)
        self._p = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Batch:
    """Many independent circuits' MPS (complex64) updated layer by layer by
    one persistent kernel per layer (optionally replayed from a CUDA graph)."""

    def __init__(self, eng: Engine, nqubits, chi_max):
        self.eng = eng
        nq = np.ascontiguousarray(nqubits, dtype=np.int32)
        cm = np.ascontiguousarray(chi_max, dtype=np.int32)
        self.nqubits = nq.copy()
        self._p = C.c_void_p()
        eng._check(eng._lib.qt_batch_create(eng._h, nq.size, _ptr(nq), _ptr(cm), C.byref(self._p)))
        self.ntask = 0

    def run(self, layers, cutoff: float, use_graph: bool = True):
        """layers: list of lists of (circuit, wire 1-based, 4x4 gate)."""
        starts, circ, site, gates = [0], [], [], []
        for layer in layers:
            for (c, w, g) in layer:
                circ.append(c)
                site.append(w - 1)
                gf = np.asarray(g, dtype=np.complex128).reshape(-1, order="F")
                gates.append(np.stack([gf.real, gf.imag], axis=1).ravel())
            starts.append(len(circ))
        st = np.asarray(starts, dtype=np.int32)
        ci = np.asarray(circ, dtype=np.int32)
        si = np.asarray(site, dtype=np.int32)
        ga = np.ascontiguousarray(np.concatenate(gates) if gates else np.zeros(32), dtype=np.float64)
        self.ntask = len(circ)
        self.eng._check(self.eng._lib.qt_batch_run(self.eng._h, self._p, len(layers), _ptr(st), _ptr(ci), _ptr(si),
                                                   _ptr(ga), float(cutoff), int(use_graph)))

    def replay(self):
        self.eng._check(self.eng._lib.qt_batch_replay(self.eng._h, self._p))

    def reset(self):
        self.eng._check(self.eng._lib.qt_batch_reset(self.eng._h, self._p))

    def task_stats(self):
        n = self.ntask
        r, sw, d = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.float32)
        if n:
            self.eng._check(self.eng._lib.qt_batch_task_stats(self.eng._h, self._p, _ptr(r), _ptr(sw), _ptr(d)))
        return r, sw, d

    def set_launch(self, bucket_cap: int, threads: int, ctas_per_sm: int):
        """Launch shape of the layer kernel for circuits with bond caps in the
        bucket ``bucket_cap`` (16, 32, 64, 128); takes effect at the next run."""
        self.eng._check(self.eng._lib.qt_batch_set_launch(self.eng._h, self._p, int(bucket_cap), int(threads),
                                                          int(ctas_per_sm)))

    def get_launch(self, bucket_cap: int):
        t, c = C.c_int(), C.c_int()
        self.eng._check(self.eng._lib.qt_batch_get_launch(self._p, int(bucket_cap), C.byref(t), C.byref(c)))
        return t.value, c.value

    def cert_counts(self) -> dict:
        """Rank decisions of the last program's tasks, as Engine.cert_counters."""
        out = (C.c_int64 * 4)()
        self.eng._check(self.eng._lib.qt_batch_cert_counts(self.eng._h, self._p, out))
        return dict(zip(CERT_NAMES, (int(v) for v in out)))

    def bond_dims(self, c: int):
        out = np.zeros(int(self.nqubits[c]) + 1, dtype=np.int32)
        self.eng._check(self.eng._lib.qt_batch_bond_dims(self.eng._h, self._p, c, _ptr(out)))
        return out

    def site(self, c: int, i: int) -> np.ndarray:
        d = self.bond_dims(c)
        out = np.zeros((d[i - 1], 2, d[i]), dtype=np.complex64, order="F")
        self.eng._check(self.eng._lib.qt_batch_download_site(self.eng._h, self._p, c, i - 1, _ptr(out)))
        return out

    def expect_z(self, i: int) -> np.ndarray:
        out = np.zeros(self.nqubits.size, dtype=np.float64)
        self.eng._check(self.eng._lib.qt_batch_expect_z(self.eng._h, self._p, i - 1, _ptr(out)))
        return out

    def free(self):
        if self._p:
            self.eng._lib.qt_batch_free(self.eng._h, self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            if self.eng._h:
                self.free()
        except Exception:
            pass


def truncated_svd_noalloc(m: int, n: int, dM: int, cutoff: float, chi_max: int, dU: int, dS: int, dVh: int,
                          stream: int = 0) -> int:
    """Truncated SVD of a complex128 device matrix for callers that cannot
    allocate device memory: every pointer (integers, device addresses) is the
    caller's; the scratch is the library's fixed device array.  Returns k.
    m, n <= 256; calls must not overlap on the GPU."""
    k = C.c_int()
    rc = library().qt_truncated_svd_noalloc(int(m), int(n), C.c_void_p(dM), float(cutoff), int(chi_max),
                                             C.c_void_p(dU), C.c_void_p(dS), C.c_void_p(dVh), C.byref(k),
                                             C.c_void_p(stream))
    if rc != QT_OK:
        if rc in REFERENCE_MESSAGES:
            raise QaintensorError(REFERENCE_MESSAGES[rc], rc)
        raise EngineError(f"qt_truncated_svd_noalloc failed with status {rc}", rc)
    return k.value


# ---------------------------------------------------------------------------
# Julia-named entry points (module level, explicit engine)
# ---------------------------------------------------------------------------

def contract_svd(engine: Engine, T1, T2, indx, er: float = 0.0):
    """src/svd.jl:7-38 on the engine."""
    return engine.contract_svd(T1, T2, indx, er)


def switch_(mps: DeviceMPS, i: int):
    """``switch!(mps, i)``."""
    mps.switch(i)


def apply_2q_(mps: DeviceMPS, gate, i: int, cutoff=None, chi_max=None, mode=None) -> dict:
    """``apply_2q!(mps, G, i; cutoff, chi_max, mode)``."""
    return mps.apply_2q(gate, i, cutoff, chi_max, mode)


# ---------------------------------------------------------------------------
# Network-level drivers of the reference over the engine's GPU primitives
# ---------------------------------------------------------------------------

def contract_rep(tensors, contractions, openidx) -> List[List[int]]:
    """``contract_rep`` of src/contract.jl:39-60: ``contractions[i]`` (a list of
    1-based (tensor, leg) pairs) gets label i + 1, open leg i gets
    -(i + 1 + #contractions)."""
    labels = [[0] * np.ndim(t) for t in tensors]
    for i, summ in enumerate(contractions, 1):
        for (t, leg) in summ:
            labels[t - 1][leg - 1] = i
    nc = len(contractions)
    for i, (t, leg) in enumerate(openidx, 1):
        if labels[t - 1][leg - 1] != 0:
            raise QaintensorError("an open leg is also contracted")
        labels[t - 1][leg - 1] = -i - nc
    if any(v == 0 for l in labels for v in l):
        raise QaintensorError("a leg is neither contracted nor open")
    return labels


def contract_order(shapes, labels):
    """``contract_order`` of src/contract.jl:183-235: the cheapest pairwise
    contraction sequence by the breadth-first search with a rising cost cap
    of Pfeifer, Haegeman and Verstraete (arXiv:1304.6112), as the reference
    ports it from opt_einsum.  Objects are bitmasks (tensors, legs by |label|);
    the cost of joining two objects that share a leg is the product of the
    dimensions of all their legs plus both build costs.  Same visiting order,
    tie-breaking and cap updates as the reference, so the same sequence.
    Returns (sequence of contracted labels, cost)."""
    dim = {}
    for shp, lab in zip(shapes, labels):
        for d, v in zip(shp, lab):
            dim[abs(v)] = int(d)
    n = len(labels)
    # level c holds objects built from c tensors: [legmask, tensormask, seq, cost, new]
    level = [[] for _ in range(n + 1)]
    for i, lab in enumerate(labels):
        legs = 0
        for v in lab:
            legs |= 1 << abs(v)
        level[1].append([legs, 1 << i, [], 0, True])
    lo, cap, nxt = 0, 1, math.inf
    while not level[n]:
        for c in range(2, n + 1):
            for d in range(1, c // 2 + 1):
                dst = level[c]
                for A in level[d]:
                    for B in level[c - d]:
                        if A[1] & B[1]:
                            continue
                        shared = A[0] & B[0]
                        if not shared:
                            continue
                        cost = 1
                        both, bit = A[0] | B[0], 0
                        while both:
                            if both & 1:
                                cost *= dim[bit]
                            both >>= 1
                            bit += 1
                        cost += A[3] + B[3]
                        if cost > cap:
                            nxt = min(nxt, cost)
                            continue
                        if not (A[4] or B[4]) and cost <= lo:
                            continue
                        tmask = A[1] | B[1]
                        seq = A[2] + B[2] + [b for b in range(shared.bit_length()) if shared >> b & 1]
                        hit = next((o for o in dst if o[1] == tmask), None)
                        if hit is None:
                            dst.append([A[0] ^ B[0], tmask, seq, cost, True])
                        elif hit[3] > cost:
                            hit[:] = [A[0] ^ B[0], tmask, seq, cost, True]
        if not level[n] and nxt == math.inf:
            raise QaintensorError("contract_order: the network is not connected")
        lo, cap, nxt = cap, nxt, math.inf
        for lv in level:
            for o in lv:
                o[4] = False
    return level[n][0][2], level[n][0][3]


def contract(engine: "Engine", tensors, contractions, openidx, optimize: bool = False, order=None) -> np.ndarray:
    """``contract(net, optimize)`` of src/contract.jl:242-264 on the GPU.  The
    network's tensors are uploaded once and stay in device memory; every
    pairwise product, trace and the final leg order run on the device
    (``qt_tensor_contract``, ``qt_tensor_trace``, ``qt_tensor_permute``) and
    only the result is downloaded.  The schedule is TensorOperations.ncon's:
    positive labels in ascending order (or in ``order``), each step
    contracting every label the two operands share; a label repeated on one
    tensor is traced; disconnected parts are joined by outer products; the
    result's axes run -1, -2, ...  With ``optimize`` the labels are
    renumbered by their position in ``contract_order``'s sequence and
    contracted with ``order=sequence``, as the reference does."""
    dt = np.result_type(*[np.asarray(t).dtype for t in tensors], np.complex64)
    if len(tensors) == 1:  # src/contract.jl:243-245: permutedims only
        t = engine.tensor(tensors[0], dt)
        out = t.permute([leg - 1 for (_, leg) in openidx]) if t.ndim else t
        res = out.numpy(dt)
        t.free()
        out.free()
        return res
    labels = contract_rep(tensors, contractions, openidx)
    if optimize and order is None:
        if any(len({v for v in l if v > 0}) != sum(1 for v in l if v > 0) for l in labels):
            raise QaintensorError("contract_order: a leg contracted with its own tensor (a trace) is not supported")
        sequence, _ = contract_order([np.shape(t) for t in tensors], labels)
        pos = {lab: k for k, lab in enumerate(sequence, 1)}
        labels = [[pos[v] if v > 0 else v for v in l] for l in labels]
        order = list(sequence)
    work = [(engine.tensor(t, dt), list(l)) for t, l in zip(tensors, labels)]
    for lab in (order if order is not None else sorted({v for l in labels for v in l if v > 0})):
        holders = [k for k, (_, l) in enumerate(work) if lab in l]
        if not holders:
            continue  # consumed by an earlier multi-label step
        if len(holders) == 1:
            t, l = work[holders[0]]
            a, b = [i for i, v in enumerate(l) if v == lab]
            work[holders[0]] = (t.trace(a, b), [v for i, v in enumerate(l) if i not in (a, b)])
            t.free()
            continue
        ka, kb = holders
        (ta, la), (tb, lb) = work[ka], work[kb]
        common = [v for v in la if v > 0 and v in lb]
        t = ta.contract(tb, [la.index(v) for v in common], [lb.index(v) for v in common])
        ta.free()
        tb.free()
        l = [v for v in la if v not in common] + [v for v in lb if v not in common]
        work = [w for k, w in enumerate(work) if k not in (ka, kb)] + [(t, l)]
    t, l = work[0]
    for tb, lb in work[1:]:
        t2 = t.contract(tb, [], [])
        t.free()
        tb.free()
        t, l = t2, l + lb
    if l:
        out = t.permute(sorted(range(len(l)), key=lambda i: -l[i]))
        t.free()
        t = out
    res = t.numpy(dt)
    t.free()
    return res


def contract_svd_mps(engine: "Engine", tensors, contractions=(), er: float = 0.0) -> np.ndarray:
    """``contract_svd_mps(tn; er)`` of src/mps.jl:190-201: the left-to-right
    chain of ``contract_svd`` over the MPS sites, each on the GPU."""
    if not er >= 0:
        raise QaintensorError("Error must be positive", QT_EINVAL_ERR_NEG)
    n = len(tensors)
    for summ in contractions:
        if sorted(map(tuple, summ)) == sorted([(n, 3), (1, 1)]):
            raise QaintensorError("Function doesn't support periodic boundary conditions for now", QT_EPERIODIC)
    t = np.asarray(tensors[0])
    for j in range(1, n):
        t = engine.contract_svd(t, tensors[j], (t.ndim, 1), er)
    return t


def mps_from_state(engine: "Engine", psi, dtype=np.complex128) -> "DeviceMPS":
    """``MPS(psi)`` of src/mps.jl:55-89 with every SVD on the GPU
    (``qt_truncated_svd``, cutoff 0: only exactly-zero values are dropped): the
    statevector (wire 1 = fastest index) is split site by site, U becoming
    the site and diag(S) V^H carried to the next; returns the device MPS
    (end sites (1,2,chi) / (chi,2,1), the reference's (2,chi) / (chi,2))."""
    psi = np.asarray(psi)
    n = psi.size
    if n < 2 or n & (n - 1):
        raise QaintensorError("Input state must have length 2^N")
    M = n.bit_length() - 1
    mode = "plain" if np.dtype(dtype) == np.complex128 else "chosen"
    p = psi.astype(dtype).reshape((2, n // 2), order="F")
    sites = []
    lbond = 1
    for bit in range(1, M):
        U, S, Vh, k, _ = engine.truncated_svd(p.reshape((lbond * 2, -1), order="F"), 0.0, mode=mode)
        sites.append(U.reshape((lbond, 2, k), order="F"))
        p = (S[:, None] * Vh).astype(dtype)
        lbond = k
    sites.append(p.reshape((lbond, 2, 1), order="F"))
    return engine.mps(sites, dtype=dtype)


def mpo_from_matrix(engine: "Engine", m) -> List[np.ndarray]:
    """``MPO(m)`` of src/mpo.jl:27-90 with every SVD on the GPU: the 2^M x 2^M
    operator is reshaped to (o1,i1,o2,i2,...) (src/mpo.jl:41-51) and split
    site by site.  Returns the reference's site tensors: first (out,in,b),
    middle (b,out,in,b'), last (b,out,in); one qubit: the 2x2 matrix."""
    m = np.asarray(m, dtype=np.complex128)
    if m.ndim != 2 or m.shape[0] != m.shape[1]:
        raise QaintensorError("MPO: the operator must be square")
    M = m.shape[0].bit_length() - 1
    if M < 1 or m.shape[0] != 1 << M:
        raise QaintensorError("Need at least one qubit to act on.")
    if M == 1:
        return [m.reshape((2, 2), order="F")]
    perm = [k for i in range(M) for k in (i, i + M)]
    t = np.transpose(m.reshape((2,) * (2 * M), order="F"), perm).reshape((4, -1), order="F")
    U, S, Vh, k, _ = engine.truncated_svd(t, 0.0)
    sites = [U.reshape((2, 2, k), order="F")]
    t = S[:, None] * Vh
    for _ in range(2, M):
        U, S, Vh, nk, _ = engine.truncated_svd(t.reshape((k * 4, -1), order="F"), 0.0)
        sites.append(U.reshape((k, 2, 2, nk), order="F"))
        t = S[:, None] * Vh
        k = nk
    sites.append(t.reshape((k, 2, 2), order="F"))
    return sites
