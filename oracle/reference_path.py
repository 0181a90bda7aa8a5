"""FP64 restatement of the reference's hot-path algorithms (test oracle only).

Every array is a *logical* numpy array whose axis ``k`` is Julia dimension
``k+1``; every reshape uses ``order='F'`` so that flattening follows Julia's
column-major rule.  Leg and tensor numbers in ``Summation``/``openidx`` are
1-based, exactly as in the reference.  Error messages are the reference's.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Sequence, Tuple

import numpy as np
import scipy.linalg as sla

__all__ = [
    "QaintensorError", "Summation", "Network", "contract_rep", "contract_rep_costs", "contract_order", "ncon",
    "contract",
    "svd_gesdd", "tail_rank", "contract_svd", "check_mps", "make_mps", "OpenMPS",
    "ClosedMPS", "PeriodicMPS", "contract_svd_mps", "mps_from_state", "switch_adjacent",
    "switch_wires", "switch_pairs", "permute_mps", "mpo_from_matrix", "decompose",
    "extend_mpo", "apply_mpo", "apply_mpo_matrix", "tensor_circuit", "apply_statevector",
    "is_power_two",
    "shift_pair",
    "shift_summation",
]


class QaintensorError(ValueError):
    """Raised where the reference raises ``ErrorException(msg)``; ``str(e)`` is msg."""


class QaintensorBoundsError(IndexError):
    """Raised where the reference constructs a ``BoundsError``."""


@dataclass
class Summation:
    """src/tensor_network.jl:7-10 -- one contraction: list of (tensor, leg), 1-based."""
    idx: List[Tuple[int, int]]

    def __eq__(self, other):
        return [tuple(p) for p in self.idx] == [tuple(p) for p in other.idx]


@dataclass
class Network:
    """GeneralTensorNetwork / MPS / MPO container (src/tensor_network.jl:26-33,
    src/mps.jl:7-29, src/mpo.jl:8-19).  ``kind`` is "general", "mps" or "mpo"."""
    tensors: List[np.ndarray]
    contractions: List[Summation] = field(default_factory=list)
    openidx: List[Tuple[int, int]] = field(default_factory=list)
    kind: str = "general"

    def copy(self):
        return Network(list(self.tensors), [Summation(list(s.idx)) for s in self.contractions],
                       list(self.openidx), self.kind)


def is_power_two(i: int) -> bool:
    """src/helper.jl:24-27."""
    return i != 0 and (i & (i - 1)) == 0


def shift_pair(p: Tuple[int, int], step: int) -> Tuple[int, int]:
    """src/helper.jl:15-17: the (tensor, leg) pair with the tensor moved by step."""
    return (p[0] + step, p[1])


def shift_summation(s: "Summation", step: int) -> "Summation":
    """src/helper.jl:6-8: both pairs of a contraction shifted by step."""
    return Summation([shift_pair(s.idx[i], step) for i in range(2)])


# --------------------------------------------------------------------------
# contraction (src/contract.jl:39-60, 242-264; TensorOperations.ncon semantics)
# --------------------------------------------------------------------------

def contract_rep(net: Network) -> List[List[int]]:
    """src/contract.jl:39-60: contraction i gets label i, open leg i gets -(i + #contractions)."""
    indexlist = [[0] * t.ndim for t in net.tensors]
    for i, s in enumerate(net.contractions, 1):
        for (t, leg) in s.idx:
            assert 1 <= leg <= net.tensors[t - 1].ndim
            indexlist[t - 1][leg - 1] = i
    j = len(net.contractions)
    for i, (t, leg) in enumerate(net.openidx, 1):
        assert indexlist[t - 1][leg - 1] == 0
        indexlist[t - 1][leg - 1] = -i - j
    for idx in indexlist:
        for v in idx:
            assert v != 0
    return indexlist


def contract_rep_costs(net: Network):
    """src/contract.jl:8-32 (``contract_rep(net, optimize=true)``): the labels of
    ``contract_rep`` plus each label's dimension (open legs under |label|)."""
    indexlist = contract_rep(net)
    costs = {}
    for t, labels in zip(net.tensors, indexlist):
        for leg, lab in enumerate(labels):
            costs[abs(lab)] = t.shape[leg]
    return costs, indexlist


def contract_order(leg_costs, indexlist):
    """src/contract.jl:183-235 (``contract_order``): the breadth-first search
    for the cheapest pairwise contraction sequence of Pfeifer, Haegeman and
    Verstraete (arXiv:1304.6112), with its cost cap, as the reference ports it
    (``check_contraction!`` at :94-160, ``getBuildCost`` at :65-85).  An object
    is (legs, tensors, sequence, cost); a pair of disjoint objects sharing a
    leg builds the object of their union at cost prod(dims of all legs of
    both) + both costs.  Returns (sequence of contracted labels, cost)."""
    n = len(indexlist)
    S = [[] for _ in range(n + 1)]
    new = [[] for _ in range(n + 1)]
    for i, labels in enumerate(indexlist):
        S[1].append((frozenset(abs(x) for x in labels), frozenset([i]), [], 0))
        new[1].append(True)
    mu_old, mu_cap, mu_next = 0, 1, math.inf
    while not S[n]:
        for c in range(2, n + 1):
            for d in range(1, c // 2 + 1):
                a, b = d, c - d
                for i, (la, ta, qa, ca) in enumerate(S[a]):
                    for j, (lb, tb, qb, cb) in enumerate(S[b]):
                        if ta & tb:
                            continue
                        common = la & lb
                        if not common:
                            continue
                        free = la ^ lb
                        cost = 1
                        for leg in free | common:
                            cost *= leg_costs[leg]
                        cost += ca + cb
                        if cost > mu_cap:
                            mu_next = min(mu_next, cost)
                            continue
                        if not (new[a][i] or new[b][j]) and cost <= mu_old:
                            continue
                        tens = ta | tb
                        seq = qa + qb + sorted(common)
                        ptr = next((k for k, o in enumerate(S[a + b]) if o[1] == tens), None)
                        if ptr is None:
                            S[a + b].append((free, tens, seq, cost))
                            new[a + b].append(True)
                        elif S[a + b][ptr][3] > cost:
                            S[a + b][ptr] = (free, tens, seq, cost)
                            new[a + b][ptr] = True
        if not S[n] and mu_next == math.inf:
            raise QaintensorError("contract_order: the network is not connected")
        mu_old, mu_cap, mu_next = mu_cap, mu_next, math.inf
        for flags in new:
            flags[:] = [False] * len(flags)
    return S[n][0][2], S[n][0][3]


def ncon(tensors: Sequence[np.ndarray], indexlist: Sequence[Sequence[int]], order=None) -> np.ndarray:
    """TensorOperations 3.1 ``ncon`` (called at src/contract.jl:257,263).

    Positive labels are contracted pairwise in ascending label order, or in
    ``order`` when given (each pairwise step contracts every label the two
    operands share); negative labels stay open and the result's axes are
    ordered -1, -2, ...
    """
    work = [(np.asarray(t), list(l)) for t, l in zip(tensors, indexlist)]
    for lab in (order if order is not None else sorted({v for l in indexlist for v in l if v > 0})):
        holders = [k for k, (_, l) in enumerate(work) if lab in l]
        if not holders:
            continue  # already consumed by an earlier multi-label pairwise step
        if len(holders) == 1:
            t, l = work[holders[0]]
            a, b = [i for i, v in enumerate(l) if v == lab]
            t = np.trace(t, axis1=a, axis2=b)
            l = [v for i, v in enumerate(l) if i not in (a, b)]
            work[holders[0]] = (t, l)
            continue
        ka, kb = holders
        ta, la = work[ka]
        tb, lb = work[kb]
        common = [v for v in la if v > 0 and v in lb]
        ax_a = [la.index(v) for v in common]
        ax_b = [lb.index(v) for v in common]
        t = np.tensordot(ta, tb, axes=(ax_a, ax_b))
        l = [v for v in la if v not in common] + [v for v in lb if v not in common]
        work = [w for k, w in enumerate(work) if k not in (ka, kb)] + [(t, l)]
    t, l = work[0]
    for tb, lb in work[1:]:
        t = np.tensordot(t, tb, axes=0)
        l = l + lb
    order = sorted(range(len(l)), key=lambda i: -l[i])
    return np.transpose(t, order) if l else t


def contract(net: Network, optimize: bool = False) -> np.ndarray:
    """src/contract.jl:242-264.  With ``optimize`` (:249-258) the labels are
    renumbered by their position in ``contract_order``'s sequence and ncon
    runs with ``order=sequence``, as the reference does."""
    if len(net.tensors) == 1:
        return np.transpose(net.tensors[0], [leg - 1 for (_, leg) in net.openidx])
    if optimize:
        costs, indexlist = contract_rep_costs(net)
        sequence, _ = contract_order(costs, indexlist)
        pos = {lab: k for k, lab in enumerate(sequence, 1)}
        indexlist = [[pos[v] if v > 0 else v for v in l] for l in indexlist]
        return ncon([t for t in net.tensors], indexlist, order=list(sequence))
    return ncon([t for t in net.tensors], contract_rep(net))


# --------------------------------------------------------------------------
# truncated SVD (src/svd.jl:7-38)
# --------------------------------------------------------------------------

def svd_gesdd(m: np.ndarray):
    """Thin SVD with LAPACK ``?gesdd`` -- Julia LinearAlgebra.svd's default driver."""
    return sla.svd(np.asarray(m), full_matrices=False, lapack_driver="gesdd")


def tail_rank(s: np.ndarray, er: float, clamp: bool = False) -> int:
    """The absolute tail-norm rule of src/svd.jl:29-33.

    ``cumsum = sqrt.(cumsum(reverse(S.^2)))``; ``k = len - findfirst(x -> x > er) + 1``:
    the smallest k with sqrt(sum_{i>k} s_i^2) <= er.  The cumulative sum runs
    sequentially from the smallest value (numpy's cumsum is sequential, like
    Julia's).  When no tail exceeds ``er`` Julia's ``findfirst`` returns
    ``nothing`` and the reference throws; ``clamp=True`` returns 1 instead
    (the engine's documented behaviour).
    """
    s = np.asarray(s, dtype=np.float64)
    c = np.sqrt(np.cumsum(s[::-1] ** 2))
    hit = np.nonzero(c > er)[0]
    if hit.size == 0:
        if clamp:
            return 1
        raise QaintensorError("findfirst returned nothing: cutoff exceeds the norm of the spectrum")
    return int(s.size - hit[0])


def contract_svd(t1: np.ndarray, t2: np.ndarray, indx: Tuple[int, int], er: float = 0.0) -> np.ndarray:
    """src/svd.jl:7-38: contract legs (i1, i2) (1-based) through two truncated SVDs."""
    if not er >= 0:
        raise QaintensorError("Error must be positive")
    i1, i2 = indx
    n1, n2 = t1.ndim, t2.ndim
    # Julia's size(A, d) is 1 for d > ndims(A)
    d1 = t1.shape[i1 - 1] if i1 <= n1 else 1
    d2 = t2.shape[i2 - 1] if i2 <= n2 else 1
    newdim = list(t1.shape[: i1 - 1]) + list(t1.shape[i1:]) + list(t2.shape[: i2 - 1]) + list(t2.shape[i2:])
    if d1 != d2:
        raise QaintensorError("Dimensions of contraction legs do not match")
    p1 = np.transpose(t1, list(range(i1 - 1)) + list(range(i1, n1)) + [i1 - 1])
    p2 = np.transpose(t2, [i2 - 1] + list(range(i2 - 1)) + list(range(i2, n2)))
    p1 = p1.reshape((-1, d1), order="F")
    p2 = p2.reshape((d1, -1), order="F")
    u1, s1, v1h = svd_gesdd(p1)
    u2, s2, v2h = svd_gesdd(p2)
    k1 = tail_rank(s1, er)
    k2 = tail_rank(s2, er)
    t = u1[:, :k1] @ np.diag(s1[:k1]) @ v1h[:k1, :] @ u2[:, :k2] @ np.diag(s2[:k2]) @ v2h[:k2, :]
    return t.reshape(newdim, order="F")


# --------------------------------------------------------------------------
# MPS (src/mps.jl)
# --------------------------------------------------------------------------

def check_mps(mps: Network) -> None:
    """src/mps.jl:37-48."""
    for t in mps.tensors:
        if t.ndim not in (2, 3):
            raise QaintensorError("Each Tensor object in MPS form can only have 2 or 3 legs")
    for s in mps.contractions:
        assert len(s.idx) == 2
        if s.idx[0][1] != mps.tensors[s.idx[0][0] - 1].ndim:
            raise QaintensorError("Tensor objects first leg must contract with last leg of previous Tensor object")
        if s.idx[1][1] != 1:
            raise QaintensorError("Tensor objects last leg must contract with first leg of next Tensor object")


def make_mps(tensors, contractions, openidx) -> Network:
    """The inner constructor of src/mps.jl:15-28 (same checks, same messages)."""
    for s in contractions:
        assert len(s.idx) == 2
        if s.idx[0][1] != tensors[s.idx[0][0] - 1].ndim:
            raise QaintensorError("Tensor objects first leg must contract with last leg of previous Tensor object")
        if s.idx[1][1] != 1:
            raise QaintensorError("Tensor objects last leg must contract with first leg of next Tensor object")
    for t in tensors:
        # the reference's check parses as `length <= (3 & length) >= 2`; it is
        # effective for 4-leg tensors (4 <= 0 is false), which is what its tests use
        if not (t.ndim <= (3 & t.ndim) >= 2):
            raise QaintensorError("Each Tensor object in MPS form can only have 2 or 3 legs")
    return Network(list(tensors), list(contractions), list(openidx), "mps")


def OpenMPS(T, N: int | None = None) -> Network:
    """src/mps.jl:99-121."""
    tensors = [T] * N if N is not None else list(T)
    for t in tensors:
        if t.ndim != 3:
            raise QaintensorError("Tensors must have 3 legs")
    l = len(tensors)
    contractions = [Summation([(i, 3), (i + 1, 1)]) for i in range(1, l)]
    openidx = [(1, 1)] + [(i, 2) for i in range(1, l + 1)] + [(l, 3)]
    return make_mps(tensors, contractions, openidx)


def ClosedMPS(T) -> Network:
    """src/mps.jl:130-154."""
    T = list(T)
    l = len(T)
    if T[0].ndim != 2:
        raise QaintensorError("First tensor must have 2 legs")
    for i in range(1, l - 1):
        if T[i].ndim != 3:
            raise QaintensorError("Tensors must have 3 legs, except the first and last one")
    if T[-1].ndim != 2:
        raise QaintensorError("Last tensor must have 2 legs")
    contractions = [Summation([(1, 2), (2, 1)])] + [Summation([(i, 3), (i + 1, 1)]) for i in range(2, l)]
    openidx = [(1, 1)] + [(i, 2) for i in range(2, l + 1)]
    return make_mps(T, contractions, openidx)


def PeriodicMPS(T, N: int | None = None) -> Network:
    """src/mps.jl:162-182."""
    tensors = [T] * N if N is not None else list(T)
    for t in tensors:
        assert t.ndim == 3
    l = len(tensors)
    contractions = [Summation([(i, 3), (i + 1, 1)]) for i in range(1, l)] + [Summation([(l, 3), (1, 1)])]
    openidx = [(i, 2) for i in range(1, l + 1)]
    return make_mps(tensors, contractions, openidx)


def contract_svd_mps(tn: Network, er: float = 0.0) -> np.ndarray:
    """src/mps.jl:190-201: left-to-right chain of ``contract_svd``."""
    if not er >= 0:
        raise QaintensorError("Error must be positive")
    l = len(tn.tensors)
    if any(s == Summation([(l, 3), (1, 1)]) for s in tn.contractions) or \
            any(s == Summation([(1, 1), (l, 3)]) for s in tn.contractions):
        raise QaintensorError("Function doesn't support periodic boundary conditions for now")
    t = tn.tensors[0]
    for j in range(1, l):
        t = contract_svd(t, tn.tensors[j], (t.ndim, 1), er=er)
    return t


def mps_from_state(psi: np.ndarray) -> Network:
    """src/mps.jl:55-89: statevector (wire 1 = fastest index) -> MPS by untruncated SVDs."""
    psi = np.asarray(psi, dtype=np.complex128)
    if not is_power_two(psi.size):
        raise QaintensorError("Input state must have length 2^N")
    M = int(round(math.log2(psi.size)))
    tensors, contractions, openidx = [], [], []
    p = psi.reshape((2, 2 ** (M - 1)), order="F")
    u, s, vh = svd_gesdd(p)
    tensors.append(u)
    openidx.append((1, 1))
    lbond = s.size
    p = np.diag(s) @ vh
    lastbit = 2
    for bit in range(2, M):
        p = p.reshape((lbond * 2, 2 ** (M - bit)), order="F")
        u, s, vh = svd_gesdd(p)
        rbond = s.size
        p = np.diag(s) @ vh
        tensors.append(u.reshape((lbond, 2, rbond), order="F"))
        contractions.append(Summation([(bit - 1, lastbit), (bit, 1)]))
        openidx.append((bit, 2))
        lbond = rbond
        lastbit = 3
    tensors.append(p)
    contractions.append(Summation([(M - 1, lastbit), (M, 1)]))
    openidx.append((M, 2))
    return make_mps(tensors, contractions, openidx)


# --------------------------------------------------------------------------
# switch! / permute! (src/switch.jl)
# --------------------------------------------------------------------------

def switch_adjacent(mps: Network, i: int) -> None:
    """``switch!(mps, i)``: swap the physical legs of sites i and i+1 (1-based).

    Follows src/switch.jl:18-56: the two sites are
    contracted with ``contract_svd(..., er=0)``, the physical legs swapped,
    then one untruncated SVD split with U to the left and diag(S)V' to the right.
    """
    if not (0 < i < len(mps.tensors)):
        raise QaintensorBoundsError(f"switch! site {i} out of range")
    t1, t2 = mps.tensors[i - 1], mps.tensors[i]
    d1, d2 = t1.shape, t2.shape
    t = contract_svd(t1, t2, (t1.ndim, 1))
    if t1.ndim == 2:
        t = np.transpose(t, [1, 0, 2]).reshape((2, 2 * d2[-1]), order="F")
    elif t2.ndim == 2:
        t = np.transpose(t, [0, 2, 1]).reshape((2 * d1[0], 2), order="F")
    else:
        t = np.transpose(t, [0, 2, 1, 3]).reshape((2 * d1[0], 2 * d2[-1]), order="F")
    u, s, vh = svd_gesdd(t)
    bond = s.size
    v = np.diag(s) @ vh
    if t1.ndim == 2:
        u = u.reshape((2, bond), order="F")
        v = v.reshape((bond, 2, d2[-1]), order="F")
    elif t2.ndim == 2:
        u = u.reshape((d1[0], 2, bond), order="F")
    else:
        u = u.reshape((d1[0], 2, bond), order="F")
        v = v.reshape((bond, 2, d2[-1]), order="F")
    mps.tensors[i - 1] = u
    mps.tensors[i] = v


def switch_wires(mps: Network, i: int, j: int) -> None:
    """``switch!(mps, i, j)`` (src/switch.jl:63-86): wire numbers
    count from the far end (``i -> L - i + 1``) and the swap runs as a ladder of
    adjacent swaps up then down."""
    check_mps(mps)
    if not (i > 0 and j > 0):
        raise QaintensorError("Wire indices `i` and `j` must be positive")
    L = len(mps.tensors)
    if not (i <= L and j <= L):
        raise QaintensorError("Indices to swap `i` and `j` must be less than or equal to the number of open wires in MPS")
    if i == j:
        return
    i, j = L - i + 1, L - j + 1
    lo, hi = (i, j) if i < j else (j, i)
    for s in range(lo, hi):
        switch_adjacent(mps, s)
    for s in range(hi - 2, lo - 1, -1):
        switch_adjacent(mps, s)


def switch_pairs(mps: Network, pairs) -> None:
    """``switch!(mps, indices::Vector{Tuple})`` (src/switch.jl:6-11)."""
    check_mps(mps)
    for a, b in pairs:
        switch_wires(mps, a, b)


def permute_mps(mps: Network, order: Sequence[int]) -> None:
    """``Base.permute!(mps, order)`` (src/switch.jl:94-106)."""
    check_mps(mps)
    order = list(order)
    n = len(mps.tensors)
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
        switch_wires(mps, i, loc)
        seq[loc - 1], seq[i - 1] = seq[i - 1], seq[loc - 1]


# --------------------------------------------------------------------------
# MPO / decompose! (src/mpo.jl, src/decompose.jl)
# --------------------------------------------------------------------------

def _operator_chain(m: np.ndarray, M: int):
    """The sequential factorisation shared by src/mpo.jl:41-70 and
    src/decompose.jl:14-41: interleave (o1,i1,o2,i2,...), then SVD site by site."""
    m = m.reshape((2,) * (2 * M), order="F")
    dims = []
    for i in range(M):
        dims += [i, i + M]
    m = np.transpose(m, dims).reshape((4, -1), order="F")
    u, s, vh = svd_gesdd(m)
    bond = s.size
    m = np.diag(s) @ vh
    ts = [u.reshape((2, 2, bond), order="F")]
    for _ in range(2, M):
        m = m.reshape((bond * 4, -1), order="F")
        u, s, vh = svd_gesdd(m)
        m = np.diag(s) @ vh
        nb = s.size
        ts.append(u.reshape((bond, 2, 2, nb), order="F"))
        bond = nb
    ts.append(m.reshape((bond, 2, 2), order="F"))
    return ts


def mpo_from_matrix(m: np.ndarray) -> Network:
    """``MPO(m)`` (src/mpo.jl:27-90).  Site legs: first (out,in,b), middle
    (b,out,in,b'), last (b,out,in); openidx lists outputs then inputs, highest
    site first.  A one-qubit MPO lists leg 2 as output and leg 1 as input."""
    m = np.asarray(m, dtype=np.complex128)
    assert m.shape[0] == m.shape[1]
    M = int(round(math.log2(m.shape[0])))
    if not M >= 1:
        raise QaintensorError("Need at least one qubit to act on.")
    if M > 1:
        ts = _operator_chain(m, M)
        con = [Summation([(1, 3), (2, 1)])] + [Summation([(i, 4), (i + 1, 1)]) for i in range(2, M)]
        openidx = [(M - i + 1, 2) for i in range(1, M)] + [(1, 1)]
        openidx += [(M - i + 1, 3) for i in range(1, M)] + [(1, 2)]
    else:
        ts = [m.reshape((2, 2), order="F")]
        con = []
        openidx = [(1, 2), (1, 1)]
    return Network(ts, con, openidx, "mpo")


def decompose(m: np.ndarray, iwire: Sequence[int]):
    """``decompose!(cg)`` (src/decompose.jl:6-52) for the gate matrix ``m`` on
    wires ``iwire``: returns (tensors, bond-leg codes, wires)."""
    M = len(iwire)
    if not M > 1:
        raise QaintensorError("Only decompose Circuit Gates that apply to multiple wires")
    ts = _operator_chain(np.asarray(m, dtype=np.complex128), M)
    c = [0, 3] + [4] * (M - 2)
    return ts, c, list(iwire)


def extend_mpo(mpo, iwire: Sequence[int]) -> Network:
    """``extend_MPO`` (src/mpo.jl:122-173); ``mpo`` may be an MPO network or a matrix."""
    iwire = tuple(iwire)
    if len(set(iwire)) != len(iwire):
        raise QaintensorError("Repeated wires are not valid.")
    if not isinstance(mpo, Network):
        if not all(w > 0 for w in iwire):
            raise QaintensorError("Wires must be positive integers.")
        if list(iwire) != sorted(iwire, reverse=True):
            raise QaintensorError("Wires not sorted")
        mpo = mpo_from_matrix(mpo)
    if list(iwire) != sorted(iwire, reverse=True):
        raise QaintensorError("Wires not sorted")
    if not all(w > 0 for w in iwire):
        raise QaintensorError("Wires must be positive integers.")
    mpo = mpo.copy()
    iw = tuple(reversed(iwire))
    M = len(iw)
    N = iw[-1] - iw[0] + 1
    assert len(mpo.tensors) == M
    if M == N:
        raise QaintensorError("MPO is already decomposed in N tensors")
    qwire = tuple(range(iw[0], iw[-1] + 1))
    pipes = sorted(set(qwire) - set(iw))
    qwire = tuple(reversed(qwire))
    for w in pipes:
        ind = qwire.index(w) + 1
        bond = mpo.tensors[ind - 2].shape[-1]
        vpipe = np.kron(np.eye(bond), np.eye(2)).reshape((bond, 2, bond, 2), order="F")
        vpipe = np.transpose(vpipe, [0, 1, 3, 2]).astype(np.complex128)
        mpo.tensors.insert(ind - 1, vpipe)
    for i in range(M, N):
        mpo.contractions.append(Summation([(i, 4), (i + 1, 1)]))
        mpo.openidx.insert(0, (i + 1, 2))
        mpo.openidx.insert(i + 1, (i + 1, 3))
    return mpo


def apply_mpo(psi: Network, mpo: Network, iwire: Sequence[int]) -> Network:
    """``apply_MPO(psi, mpo, iwire)`` (src/mpo.jl:184-216): lazy wiring."""
    iwire = tuple(iwire)
    if len(set(iwire)) != len(iwire):
        raise QaintensorError("Repeated wires are not valid.")
    n = len(psi.openidx)
    if not all(0 < w <= n for w in iwire):
        raise QaintensorError("Wires must be integers between 1 and n (total number of qudits).")
    step = len(psi.tensors)
    N = len(iwire)
    iwire = tuple(reversed(iwire))
    # The reference's `if M < N` extension branch compares the tuple length
    # with itself (M is iwire's type parameter), so it never runs: the MPO's
    # own bonds carry it across non-adjacent wires.
    out = Network(list(psi.tensors) + list(mpo.tensors),
                  [Summation(list(s.idx)) for s in psi.contractions]
                  + [shift_summation(s, step) for s in mpo.contractions],
                  list(psi.openidx), "general")
    for i, w in enumerate(iwire, 1):
        out.contractions.append(Summation([psi.openidx[w - 1], shift_pair(mpo.openidx[i + N - 1], step)]))
    for i, q in enumerate(iwire, 1):
        out.openidx[q - 1] = shift_pair(mpo.openidx[i - 1], step)
    return out


def apply_mpo_matrix(psi: Network, m: np.ndarray, iwire: Sequence[int]) -> Network:
    """``apply_MPO(psi, m::AbstractMatrix, iwire)`` (src/mpo.jl:228-241): unsorted
    wires are handled by permuting the operator's legs."""
    iwire = tuple(iwire)
    if len(set(iwire)) != len(iwire):
        raise QaintensorError("Repeated wires are not valid.")
    if not all(w > 0 for w in iwire):
        raise QaintensorError("Wires must be positive integers.")
    M = len(iwire)
    srt = sorted(iwire)
    m = np.asarray(m, dtype=np.complex128)
    if srt != list(iwire):
        sw = list(np.argsort(iwire, kind="stable"))
        perm = sw + [p + M for p in sw]
        m = np.transpose(m.reshape((2,) * (2 * M), order="F"), perm).reshape((2 ** M, 2 ** M), order="F")
    return apply_mpo(psi, mpo_from_matrix(m), tuple(srt))


# --------------------------------------------------------------------------
# tensor_circuit! (src/tensor_circuit.jl:14-80) and the statevector oracle
# --------------------------------------------------------------------------

def tensor_circuit(psi: Network, m: np.ndarray, iwire: Sequence[int], is_decompose: bool = False) -> None:
    """Lazily append gate matrix ``m`` on wires ``iwire`` (src/tensor_circuit.jl:14-52).

    With ``is_decompose=False`` the reference contracts the state with the
    gate tensor's legs 1..M (the matrix's row bits), i.e. it applies the
    transpose of ``m``; this restatement does the same.  The decomposed path
    applies ``m`` itself.
    """
    M = len(iwire)
    m = np.asarray(m, dtype=np.complex128)
    if M > 1 and is_decompose:
        ts, cs, ws = decompose(m, iwire)
        for i, (t, c, w) in enumerate(zip(ts, cs, ws), 1):
            psi.tensors.append(t)
            L = len(psi.tensors)
            psi.contractions.append(Summation([psi.openidx[w - 1], (L, 2 if i == 1 else 3)]))
            if c > 0:
                psi.contractions.append(Summation([(L - 1, c), (L, 1)]))
            psi.openidx[w - 1] = (L, 1) if i == 1 else (L, 2)
        return
    psi.tensors.append(m.reshape((2,) * (2 * M), order="F"))
    L = len(psi.tensors)
    for i, w in enumerate(iwire, 1):
        psi.contractions.append(Summation([psi.openidx[w - 1], (L, i)]))
        psi.openidx[w - 1] = (L, M + i)


def apply_statevector(psi: np.ndarray, m: np.ndarray, iwire: Sequence[int]) -> np.ndarray:
    """Dense ``apply(psi, CircuitGate(iwire, m))`` (Qaintessent 0.1.1 convention
    as pinned by test/test_mpo.jl:88-121): wire w is bit w-1 of the state index,
    and iwire[k] is bit k-1 of the gate-matrix index."""
    psi = np.asarray(psi, dtype=np.complex128)
    n = int(round(math.log2(psi.size)))
    M = len(iwire)
    t = psi.reshape((2,) * n, order="F")
    g = np.asarray(m, dtype=np.complex128).reshape((2,) * (2 * M), order="F")
    axes = [w - 1 for w in iwire]
    r = np.tensordot(g, t, axes=(list(range(M, 2 * M)), axes))
    # r axes: gate outputs (bits of iwire order) then the untouched wires in order
    rest = [a for a in range(n) if a not in axes]
    cur = axes + rest
    inv = [cur.index(a) for a in range(n)]
    return np.transpose(r, inv).reshape(-1, order="F")
