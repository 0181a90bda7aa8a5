"""FP64 oracle for the engine's documented extensions (test oracle only).

The reference has no eager two-qubit gate + truncated-SVD update; it is
composed here from reference pieces, each cited:

* two-site contraction   -- src/switch.jl:26 (the contract_svd call) / src/svd.jl:35
* gate acts as U on the input legs, iwire[k] = bit k-1 -- src/decompose.jl:16-31, src/mpo.jl:41-57
* matrix view (2*chiL, 2*chiR), rows (a,s1), columns (s2,b) -- src/switch.jl:35-36
* rank by the absolute tail rule              -- src/svd.jl:29-33
* split U -> left site, diag(S)V' -> right     -- src/switch.jl:50-52

Sites use a uniform 3-leg layout (chiL, 2, chiR); the first site has chiL=1
and the last chiR=1 (the same memory as the reference's 2-leg end tensors).
Site and wire numbers are 1-based, as in the Julia API.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

from .reference_path import svd_gesdd, tail_rank

__all__ = [
    "haar_unitary", "brickwork_gates", "product_state", "sites_from_reference_mps",
    "UpdateStats", "theta_of", "apply_gate_to_theta", "apply_2q", "run_brickwork",
    "mps_to_state", "mps_norm2", "expect_z", "expect_zz", "operator_schmidt",
    "tfim_mpo", "apply_mpo_sites", "canonicalize_left", "compress_sweep", "mpo_energy",
    "randomized_svd", "decay_theta_factors", "MLP_SIZES", "mlp_init", "mlp_forward",
    "mlp_backward", "mlp_loss", "rank_features", "N_FEATURES",
]


# --------------------------------------------------------------------------
# inputs
# --------------------------------------------------------------------------

def haar_unitary(rng: np.random.Generator, n: int = 4) -> np.ndarray:
    """Haar-random U(n): QR of a complex Ginibre matrix with the diagonal-phase
    fix of Mezzadri (2007), so the distribution is exactly Haar."""
    z = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(2.0)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))[None, :]


def brickwork_gates(n_qubits: int, depth: int, rng: np.random.Generator):
    """Brickwork circuit: layer l (1-based) acts on wire pairs (1,2),(3,4),...
    when l is odd and (2,3),(4,5),... when l is even.  Returns a list of
    (layer, first_wire, 4x4 unitary); gates are drawn layer by layer, left to right."""
    out = []
    for layer in range(1, depth + 1):
        start = 1 if layer % 2 == 1 else 2
        for w in range(start, n_qubits, 2):
            out.append((layer, w, haar_unitary(rng, 4)))
    return out


def product_state(n_qubits: int, dtype=np.complex128) -> List[np.ndarray]:
    """|0...0> as bond-1 sites (1,2,1)."""
    s = np.zeros((1, 2, 1), dtype=dtype)
    s[0, 0, 0] = 1.0
    return [s.copy() for _ in range(n_qubits)]


def sites_from_reference_mps(tensors: Sequence[np.ndarray]) -> List[np.ndarray]:
    """Reference MPS tensors (first (2,chi), middle (chiL,2,chiR), last (chi,2))
    -> uniform 3-leg sites.  Pure reshapes: the memory is unchanged."""
    out = []
    n = len(tensors)
    for i, t in enumerate(tensors):
        if t.ndim == 3:
            out.append(t)
        elif i == 0:
            out.append(t.reshape((1,) + t.shape, order="F"))
        elif i == n - 1:
            out.append(t.reshape(t.shape + (1,), order="F"))
        else:
            raise ValueError("2-leg tensor in the middle of an MPS")
    return out


def decay_theta_factors(chi: int, rng: np.random.Generator, decay: float = 0.97):
    """Single-bond workload: theta = Q1 diag(decay^k) Q2^H normalised to unit
    Frobenius norm, with Q1, Q2 from QR of i.i.d. complex Gaussian (2chi x 2chi)
    matrices, returned as two sites A (chi,2,chi), B (chi,2,chi) with
    theta = A.B (the spectrum beyond index chi, below decay^chi, is dropped so
    the bond between A and B is chi)."""
    n = 2 * chi
    g1 = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(2)
    g2 = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(2)
    q1, _ = np.linalg.qr(g1)
    q2, _ = np.linalg.qr(g2)
    s = decay ** np.arange(chi, dtype=np.float64)
    s /= np.linalg.norm(s)
    a = (q1[:, :chi] * s[None, :]).reshape((chi, 2, chi), order="F")
    b = q2[:, :chi].conj().T.reshape((chi, 2, chi), order="F")
    return a, b, s


# --------------------------------------------------------------------------
# the composed two-qubit gate + truncated-SVD update
# --------------------------------------------------------------------------

@dataclass
class UpdateStats:
    rank: int                 # kept rank k
    rank_cutoff: int          # rank from the tail rule alone (before chi_max)
    discarded_weight: float   # sum_{i>k} s_i^2 of the full spectrum
    norm2: float              # sum_i s_i^2
    spectrum: np.ndarray      # full descending spectrum


def theta_of(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """theta (2chiL x 2chiR) = A_mat (2chiL x chiM) . B_mat (chiM x 2chiR)."""
    chil, _, chim = a.shape
    _, _, chir = b.shape
    return a.reshape((2 * chil, chim), order="F") @ b.reshape((chim, 2 * chir), order="F")


def apply_gate_to_theta(theta: np.ndarray, g: np.ndarray, chil: int, chir: int) -> np.ndarray:
    """theta'(a,o1,o2,b) = sum G[o1+2o2, i1+2i2] theta(a,i1,i2,b)."""
    t4 = theta.reshape((chil, 2, 2, chir), order="F")
    g4 = np.asarray(g, dtype=np.complex128).reshape((2, 2, 2, 2), order="F")
    out = np.einsum("pqrs,arsb->apqb", g4, t4)
    return out.reshape((2 * chil, 2 * chir), order="F")


def apply_2q(sites: List[np.ndarray], g: np.ndarray, i: int, cutoff: float = 0.0,
             chi_max: int = 0, renormalize: bool = False) -> UpdateStats:
    """Apply the 4x4 gate ``g`` to wires (i, i+1) (1-based) and re-split with a
    truncated SVD; ``sites`` is updated in place.  ``chi_max <= 0`` means no cap.
    With ``renormalize`` the kept values are rescaled to the full spectrum's norm."""
    a, b = sites[i - 1], sites[i]
    chil, chir = a.shape[0], b.shape[2]
    th = apply_gate_to_theta(theta_of(a, b), g, chil, chir)
    u, s, vh = svd_gesdd(th)
    kc = tail_rank(s, cutoff, clamp=True)
    k = min(kc, chi_max) if chi_max > 0 else kc
    sk = s[:k].copy()
    if renormalize:
        sk *= math.sqrt(float(np.sum(s * s))) / math.sqrt(float(np.sum(sk * sk)))
    sites[i - 1] = u[:, :k].reshape((chil, 2, k), order="F")
    sites[i] = (sk[:, None] * vh[:k, :]).reshape((k, 2, chir), order="F")
    return UpdateStats(k, kc, float(np.sum(s[k:] ** 2)), float(np.sum(s * s)), s)


def run_brickwork(n_qubits: int, gates, cutoff: float, chi_max: int, sites=None):
    """Run a brickwork gate list (from ``brickwork_gates``) through ``apply_2q``.
    Returns (sites, list of UpdateStats in gate order)."""
    sites = product_state(n_qubits) if sites is None else sites
    stats = [apply_2q(sites, g, w, cutoff, chi_max) for (_, w, g) in gates]
    return sites, stats


# --------------------------------------------------------------------------
# observables
# --------------------------------------------------------------------------

def mps_to_state(sites: Sequence[np.ndarray]) -> np.ndarray:
    """Dense statevector with wire 1 as the fastest index (column-major)."""
    psi = np.ones((1, 1), dtype=np.complex128)
    for a in sites:
        p = np.einsum("pa,asb->psb", psi, a)
        psi = p.reshape((p.shape[0] * 2, p.shape[2]), order="F")
    return psi.reshape(-1, order="F") if psi.shape[1] == 1 else psi


def _transfer(sites, ops):
    env = np.ones((1, 1), dtype=np.complex128)
    for a, o in zip(sites, ops):
        if o is None:
            env = np.einsum("ab,asc,bsd->cd", env, a.conj(), a)
        else:
            env = np.einsum("ab,asc,st,btd->cd", env, a.conj(), o, a)
    return env[0, 0]


_Z = np.diag([1.0, -1.0]).astype(np.complex128)
_X = np.array([[0, 1], [1, 0]], dtype=np.complex128)


def mps_norm2(sites) -> float:
    return float(np.real(_transfer(sites, [None] * len(sites))))


def expect_z(sites, i: int) -> float:
    """<psi|Z_i|psi>/<psi|psi> (wire i, 1-based)."""
    ops = [None] * len(sites)
    ops[i - 1] = _Z
    return float(np.real(_transfer(sites, ops))) / mps_norm2(sites)


def expect_zz(sites, i: int) -> float:
    """<psi|Z_i Z_{i+1}|psi>/<psi|psi> (wires i, i+1, 1-based)."""
    ops = [None] * len(sites)
    ops[i - 1] = _Z
    ops[i] = _Z
    return float(np.real(_transfer(sites, ops))) / mps_norm2(sites)


def operator_schmidt(g: np.ndarray) -> np.ndarray:
    """Operator-Schmidt values of a 2-qubit gate: the singular values of the
    interleaved (o1 i1) x (o2 i2) reshape, exactly the 4x4 SVD that
    src/decompose.jl:16-26 (and src/mpo.jl:41-53) take for M = 2."""
    m = np.asarray(g, dtype=np.complex128).reshape((2, 2, 2, 2), order="F")
    m = np.transpose(m, [0, 2, 1, 3]).reshape((4, 4), order="F")
    return np.linalg.svd(m, compute_uv=False)


# --------------------------------------------------------------------------
# MPO workload: transverse-field Ising model, application and compression
# --------------------------------------------------------------------------

def tfim_mpo(n: int, J: float, h: Sequence[float]) -> List[np.ndarray]:
    """H = -J sum Z_i Z_{i+1} - sum h_i X_i as bond-3 MPO sites (bL, out, in, bR),
    the reference's middle-site leg order (src/mpo.jl:66).  Ends have bond 1."""
    eye = np.eye(2, dtype=np.complex128)
    sites = []
    for i in range(n):
        w = np.zeros((3, 2, 2, 3), dtype=np.complex128)
        w[0, :, :, 0] = eye
        w[1, :, :, 0] = _Z
        w[2, :, :, 0] = -h[i] * _X
        w[2, :, :, 1] = -J * _Z
        w[2, :, :, 2] = eye
        if i == 0:
            w = w[2:3]
        if i == n - 1:
            w = w[..., 0:1]
        sites.append(w)
    return sites


def apply_mpo_sites(sites, mpo):
    """Exact MPO x MPS: new site (chiL*bL, 2, chiR*bR), fused index a + chiL*alpha."""
    out = []
    for a, w in zip(sites, mpo):
        cl, _, cr = a.shape
        bl, _, _, br = w.shape
        t = np.einsum("aib,xoiy->axoby", a, w)
        out.append(t.reshape((cl * bl, 2, cr * br), order="F"))
    return out


def canonicalize_left(sites):
    """Left-to-right QR sweep; returns the norm carried by the last site."""
    sites = list(sites)
    for i in range(len(sites) - 1):
        cl, _, cr = sites[i].shape
        q, r = np.linalg.qr(sites[i].reshape((cl * 2, cr), order="F"))
        k = q.shape[1]
        sites[i] = q.reshape((cl, 2, k), order="F")
        nxt = sites[i + 1]
        sites[i + 1] = (r @ nxt.reshape((nxt.shape[0], -1), order="F")).reshape((k, 2, nxt.shape[2]), order="F")
    return sites


def compress_sweep(sites, cutoff: float, chi_max: int, normalize: bool = True):
    """SVD compression: left-canonicalise, optionally normalise, then sweep
    right to left truncating each bond by the tail rule and chi_max, absorbing
    U*S into the left neighbour.  Returns (sites, kept ranks, discarded weights)."""
    sites = canonicalize_left(sites)
    if normalize:
        nrm = np.linalg.norm(sites[-1])
        sites[-1] = sites[-1] / nrm
    ranks, disc = [], []
    for i in range(len(sites) - 1, 0, -1):
        cl, _, cr = sites[i].shape
        u, s, vh = svd_gesdd(sites[i].reshape((cl, 2 * cr), order="F"))
        kc = tail_rank(s, cutoff, clamp=True)
        k = min(kc, chi_max) if chi_max > 0 else kc
        sites[i] = vh[:k].reshape((k, 2, cr), order="F")
        us = u[:, :k] * s[None, :k]
        prev = sites[i - 1]
        pl = prev.shape[0]
        sites[i - 1] = (prev.reshape((pl * 2, cl), order="F") @ us).reshape((pl, 2, k), order="F")
        ranks.append(k)
        disc.append(float(np.sum(s[k:] ** 2)))
    return sites, ranks[::-1], disc[::-1]


def mpo_energy(sites, mpo) -> float:
    """<psi|H|psi>/<psi|psi> by an MPO transfer sweep."""
    env = np.ones((1, 1, 1), dtype=np.complex128)
    for a, w in zip(sites, mpo):
        env = np.einsum("axb,asc,xsty,btd->cyd", env, a.conj(), w, a)
    return float(np.real(env[0, 0, 0])) / mps_norm2(sites)


# --------------------------------------------------------------------------
# randomized truncated SVD (FP64 reference of the algorithm)
# --------------------------------------------------------------------------

def randomized_svd(m: np.ndarray, l: int, power_iters: int, rng: np.random.Generator):
    """Range finder with ``l`` Gaussian probes and ``power_iters`` subspace
    iterations, QR re-orthogonalisation, then the SVD of B = Q^H M.
    Returns (U, S, Vh, residual_norm) with residual = ||M - Q Q^H M||_F."""
    n = m.shape[1]
    om = (rng.standard_normal((n, l)) + 1j * rng.standard_normal((n, l))) / math.sqrt(2)
    y = m @ om
    q, _ = np.linalg.qr(y)
    for _ in range(power_iters):
        z, _ = np.linalg.qr(m.conj().T @ q)
        q, _ = np.linalg.qr(m @ z)
    b = q.conj().T @ m
    ub, s, vh = np.linalg.svd(b, full_matrices=False)
    res = np.linalg.norm(m - q @ b)
    return q @ ub, s, vh, float(res)


# --------------------------------------------------------------------------
# the learned-rank MLP (FP64 reference of forward / backward)
# --------------------------------------------------------------------------

N_FEATURES = 16
MLP_SIZES = (N_FEATURES, 64, 64, 1)


def rank_features(prev_spectrum, gate, site: int, n_sites: int, layer: int, depth: int,
                  chil: int, chir: int, chi_max: int, cutoff: float) -> np.ndarray:
    """The 16 input features of one bond update.

    0      k_prev / k_max         (previous kept rank at this bond)
    1..8   fraction of the previous (unit-normalised) spectrum above 10^-j, j=1..8
    9..12  the gate's operator-Schmidt values / 2
    13     site / n_sites
    14     layer / depth
    15     -log10(cutoff) / 16
    with k_max = min(2 chiL, 2 chiR, chi_max)."""
    kmax = min(2 * chil, 2 * chir, chi_max if chi_max > 0 else 1 << 30)
    s = np.asarray(prev_spectrum, dtype=np.float64)
    nrm = math.sqrt(float(np.sum(s * s))) or 1.0
    s = s / nrm
    f = np.zeros(N_FEATURES)
    f[0] = s.size / kmax
    for j in range(1, 9):
        f[j] = float(np.count_nonzero(s > 10.0 ** (-j))) / kmax
    f[9:13] = operator_schmidt(gate) / 2.0
    f[13] = site / max(n_sites, 1)
    f[14] = layer / max(depth, 1)
    f[15] = -math.log10(max(cutoff, 1e-300)) / 16.0
    return f


def mlp_init(rng: np.random.Generator, sizes=MLP_SIZES):
    """He-style initialisation; returns [W1, b1, W2, b2, W3, b3] with W (out x in)."""
    params = []
    for i in range(len(sizes) - 1):
        fan_in = sizes[i]
        params.append(rng.standard_normal((sizes[i + 1], fan_in)) * math.sqrt(2.0 / fan_in))
        params.append(np.zeros(sizes[i + 1]))
    return params


def mlp_forward(params, x):
    """x (batch x 16) -> (prediction (batch,), cache). ReLU hidden layers, linear output."""
    w1, b1, w2, b2, w3, b3 = params
    z1 = x @ w1.T + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ w2.T + b2
    h2 = np.maximum(z2, 0.0)
    y = (h2 @ w3.T + b3)[:, 0]
    return y, (x, z1, h1, z2, h2)


def mlp_loss(pred, target) -> float:
    """Mean squared error."""
    return float(np.mean((pred - target) ** 2))


def mlp_backward(params, cache, pred, target):
    """Gradients of the mean squared error w.r.t. [W1, b1, W2, b2, W3, b3]."""
    w1, b1, w2, b2, w3, b3 = params
    x, z1, h1, z2, h2 = cache
    n = x.shape[0]
    dy = (2.0 / n) * (pred - target)[:, None]
    gw3 = dy.T @ h2
    gb3 = dy.sum(0)
    dh2 = dy @ w3
    dz2 = dh2 * (z2 > 0)
    gw2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dh1 = dz2 @ w2
    dz1 = dh1 * (z1 > 0)
    gw1 = dz1.T @ x
    gb1 = dz1.sum(0)
    return [gw1, gb1, gw2, gb2, gw3, gb3]
