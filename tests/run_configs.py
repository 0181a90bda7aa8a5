"""Run the workload configurations of the benchmark plan and print one JSON
object per configuration (seeded synthetic inputs throughout).  The script
sits with the tests because the oracle is its checker.

    python tests/run_configs.py c1 c2 c4 c5 [--c3-depth 20] [--c4-circuits 4096]
    python tests/run_configs.py cpu [--cpu-reps 5]        (no GPU needed)

c1  12-qubit brickwork, depth 8, Haar gates, cutoff 1e-10, chi_max 32, plain
    FP64: ranks and <Z_1> against the FP64 oracle, amplitudes against the dense
    statevector, wall time.
c2  single-bond sweep chi in {64, 256, 1024}: theta spectrum 0.97^k, Haar gate,
    truncation back to chi; plain (complex128) and chosen (complex64): time
    per update and truncation error against the exact FP64 split.
c3  64-qubit brickwork, complex64, chi_max 1024, cutoff 1e-8, chosen mode:
    updates/s, kept ranks, <Z_i Z_i+1> on all bonds.
c4  batched ensemble: circuits with qubits U[8,40], depth U[4,24], chi_max in
    {16,32,64,128}, complex64, cutoff 1e-8, one persistent kernel per layer in
    a CUDA graph: aggregate updates/s, <Z_1> error against the oracle on a sample.
c5  40-site TFIM MPO (J=1, h ~ U[0.5,1.5]) applied 10 times to a random
    normalised chi=512 complex64 MPS, each followed by a compression sweep to
    chi 512 at cutoff 1e-9 and a renormalisation: <H> against an FP64 device
    run (cuSOLVER splits) on the same inputs, wall time.
cpu the CPU restatement of the reference path (the oracle's update: theta,
    gate fold, gesdd, tail rule) at chi in {64, 256, 1024} on the c2 inputs,
    complex128 (the oracle itself) and complex64 (the same steps in single
    precision, cgesdd), with OpenBLAS on all host threads and on one thread:
    updates/s as the median of --cpu-reps timed updates after one warm-up.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def haar(rng):
    z = (rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))) / math.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))[None, :]


def brickwork(n, depth, rng):
    out = []
    for layer in range(1, depth + 1):
        for w in range(1 if layer % 2 else 2, n, 2):
            out.append((layer, w, haar(rng)))
    return out


def decay_pair(chi, rng, decay=0.97):
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


def theta_prime(a, b, g):
    chi_l, chi_m, chi_r = a.shape[0], a.shape[2], b.shape[2]
    th = a.reshape((2 * chi_l, chi_m), order="F") @ b.reshape((chi_m, 2 * chi_r), order="F")
    g4 = np.asarray(g).reshape((2, 2, 2, 2), order="F")
    th = np.einsum("pqrs,arsb->apqb", g4, th.reshape((chi_l, 2, 2, chi_r), order="F"))
    return th.reshape((2 * chi_l, 2 * chi_r), order="F")


def load_rank_model(eng):
    p = os.path.join(HERE, "rank_model_params.npy")
    if os.path.exists(p):
        eng.set_rank_params(np.load(p), enable=True)
        return True
    return False


def c1(qt, args):
    import oracle as O
    rng = np.random.default_rng(2024)
    n, depth, cutoff, chi_max = 12, 8, 1e-10, 32
    gates = brickwork(n, depth, rng)
    eng = qt.Engine(mode="plain")
    mps = eng.product_state(n)
    t0 = time.perf_counter()
    ranks = [mps.apply_2q(g, w, cutoff, chi_max)["rank"] for (_, w, g) in gates]
    dt = time.perf_counter() - t0
    sites, stats = O.run_brickwork(n, gates, cutoff, chi_max)
    psi = O.mps_to_state([s for s in mps.sites()])
    dense = np.zeros(2 ** n, dtype=complex)
    dense[0] = 1
    for (_, w, g) in gates:
        dense = O.apply_statevector(dense, g, (w, w + 1))
    z, zr = mps.expect_z(1), O.expect_z(sites, 1)
    return {"config": "c1", "updates": len(gates), "seconds": dt, "ranks_identical": ranks == [s.rank for s in stats],
            "Z1_gpu": z, "Z1_oracle": zr, "Z1_rel_err": abs(z - zr) / abs(zr),
            "amp_err_vs_oracle": float(np.abs(psi - O.mps_to_state(sites)).max()),
            "fidelity_vs_dense": float(abs(np.vdot(psi, dense)) ** 2),
            "truncated": int(sum(1 for s in stats if s.rank < s.rank_cutoff))}


def c2(qt, args):
    rng = np.random.default_rng(7)
    out = []
    for chi in args.c2_chis:
        a, b, s = decay_pair(chi, rng)
        g = haar(rng)
        row = {"chi": chi}
        th64 = theta_prime(a.astype(np.complex64).astype(complex), b.astype(np.complex64).astype(complex), g)
        for mode, dt, tc in (("plain", np.complex128, 0), ("chosen", np.complex64, 1)):
            eng = qt.Engine(mode=mode, tc_gemm=tc)
            if mode == "chosen":
                load_rank_model(eng)
            tmpl = eng.mps([a.astype(np.complex64).astype(dt), b.astype(np.complex64).astype(dt)], dtype=dt)
            tmpl.set_bond_spectrum(1, s)
            m = tmpl.clone()
            m.apply_2q(g, 1, 1e-10, chi)  # warm-up
            m.free()
            reps = 1 if (mode == "plain" and chi >= 512) else 3
            eng.sync()
            t0 = time.perf_counter()
            for _ in range(reps):
                m = tmpl.clone()
                st = m.apply_2q(g, 1, 1e-10, chi)
                if _ < reps - 1:
                    m.free()
            eng.sync()
            dt_s = (time.perf_counter() - t0) / reps
            A = m.site(1).astype(complex)
            B = m.site(2).astype(complex)
            approx = A.reshape((2 * chi, -1), order="F") @ B.reshape((B.shape[0], -1), order="F")
            row[mode] = {"ms_per_update": dt_s * 1e3, "rank": st["rank"], "sketch": st["sketch_size"],
                         "fallback": st["fallback"], "trunc_err": float(np.linalg.norm(th64 - approx))}
            m.free()
            tmpl.free()
            eng.close()
        row["trunc_err_ratio_chosen_vs_plain"] = row["chosen"]["trunc_err"] / max(row["plain"]["trunc_err"], 1e-300)
        row["speedup_chosen_vs_plain"] = row["plain"]["ms_per_update"] / row["chosen"]["ms_per_update"]
        out.append(row)
    return {"config": "c2", "rows": out}


def c3(qt, args):
    rng = np.random.default_rng(64)
    n, depth, chi_max, cutoff = 64, args.c3_depth, 1024, 1e-8
    gates = brickwork(n, depth, rng)
    eng = qt.Engine(mode="chosen", tc_gemm=1)
    model = load_rank_model(eng)
    mps = eng.product_state(n, dtype=np.complex64)
    t0 = time.perf_counter()
    stats = []
    for (layer, w, g) in gates:
        mps.set_circuit_position(layer, depth)
        stats.append(mps.apply_2q(g, w, cutoff, chi_max))
    dt = time.perf_counter() - t0
    zz = [mps.expect_zz(i) for i in range(1, n)] if args.c3_observables else []
    return {"config": "c3", "depth": depth, "updates": len(gates), "seconds": dt, "updates_per_s": len(gates) / dt,
            "max_rank": max(s["rank"] for s in stats), "fallbacks": sum(1 for s in stats if s["fallback"]),
            "sketched": sum(1 for s in stats if s["sketch_size"] > 0), "rank_model": model, "ZZ": zz}


def c4_circuits(nc, rng):
    """The ensemble: (qubits, depth, chi_max, brickwork gates) per circuit."""
    circuits = []
    for c in range(nc):
        n = int(rng.integers(8, 41))
        depth = int(rng.integers(4, 25))
        chi = int(rng.choice([16, 32, 64, 128]))
        circuits.append((n, depth, chi, brickwork(n, depth, rng)))
    return circuits


def lpt_shards(costs, world):
    """Circuits to ranks, longest estimated cost first, each to the least
    loaded rank (ties to the lower rank).  Every rank computes the same
    assignment from the same costs; returns each rank's sorted indices."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    shards = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        shards[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in shards]


def gather_by_circuit(dist, idx, vals, nc):
    """Every rank's per-circuit values in global circuit order (the one
    collective of the sharded ensemble, after the timed region)."""
    parts = [(idx, vals)]
    if dist is not None and dist.world > 1:
        parts = [None] * dist.world
        dist.dist.all_gather_object(parts, (list(idx), list(vals)))
    out = [None] * nc
    for ids, vs in parts:
        for i, v in zip(ids, vs):
            out[i] = v
    return out


def c4(qt, args):
    """The batched ensemble, sharded by circuit over the ranks when launched
    with one process per GPU (RANK, WORLD_SIZE, LOCAL_RANK): each rank runs
    its circuits on its own GPU with no collective in the timed region; the
    rate is all ranks' updates over the slowest rank's time."""
    import oracle as O
    dist = getattr(args, "dist", None)
    world, rank, local = (dist.world, dist.rank, dist.local) if dist is not None else (1, 0, 0)
    rng = np.random.default_rng(4096)
    nc = args.c4_circuits
    circuits = c4_circuits(nc, rng)
    # cost estimate: bond updates (depth (n-1)/2) times chi_max^3
    mine = lpt_shards([c[1] * (c[0] - 1) / 2 * c[2] ** 3 for c in circuits], world)[rank]
    layers = [[] for _ in range(max([circuits[ci][1] for ci in mine], default=0))]
    for j, ci in enumerate(mine):
        for (layer, w, g) in circuits[ci][3]:
            layers[layer - 1].append((j, w, g))
    ntask = sum(len(l) for l in layers)
    eng = qt.Engine(mode="chosen", device=local)
    b = qt.Batch(eng, [circuits[ci][0] for ci in mine], [circuits[ci][2] for ci in mine])
    b.run(layers, 1e-8, use_graph=True)  # capture + first run (warm-up)
    b.reset()
    eng.sync()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    b.replay()
    eng.sync()
    dt = time.perf_counter() - t0
    if dist is not None:
        dt, ntask_all = dist.max(dt), int(dist.sum(ntask))
    else:
        ntask_all = ntask
    z = gather_by_circuit(dist, mine, [float(v) for v in b.expect_z(1)], nc)
    b.free()
    eng.close()
    errs = []
    if rank == 0:
        for ci in rng.choice(nc, size=min(nc, args.c4_check), replace=False):
            n, depth, chi, gates = circuits[ci]
            if chi > 32 or n > 24:
                continue
            sites, _ = O.run_brickwork(n, gates, 1e-8, chi)
            errs.append(abs(z[ci] - O.expect_z(sites, 1)))
    return {"config": "c4", "circuits": nc, "ranks": world, "updates": ntask_all, "seconds": dt,
            "updates_per_s": ntask_all / dt, "Z1_err_max_sample": max(errs) if errs else None,
            "checked": len(errs)}


def c5(qt, args):
    rng = np.random.default_rng(40)
    n, chi, steps, cutoff = 40, args.c5_chi, args.c5_steps, 1e-9
    import oracle as O
    h = rng.uniform(0.5, 1.5, n)
    mpo = O.tfim_mpo(n, 1.0, h)
    dims = [1] + [chi] * (n - 1) + [1]
    # a random MPS with entries of variance 1/(2 chiL): each transfer step
    # keeps the expected norm, and the state is normalised exactly below
    sites = [((rng.standard_normal((dims[i], 2, dims[i + 1])) + 1j * rng.standard_normal((dims[i], 2, dims[i + 1])))
              / math.sqrt(2 * 2 * dims[i])).astype(np.complex64) for i in range(n)]
    res = {"config": "c5", "chi": chi, "steps": steps}

    def normalise(m):
        # the power iteration's norm grows by up to ||H|| per application;
        # <H> is scale-invariant, the storage is not
        first = m.site(1)
        m.upload_site(1, first / math.sqrt(m.norm2()))

    # the FP64 reference run splits with cuSOLVER (FP64, the faster of the
    # two FP64 paths at bond 3 chi)
    for mode, dt in (("chosen", np.complex64), ("cusolver", np.complex128)):
        eng = qt.Engine(mode=mode, tc_gemm=1 if mode == "chosen" else 0)
        m = eng.mps([s.astype(dt) for s in sites], dtype=dt)
        normalise(m)
        m.compress(cutoff, chi, mode=mode)
        t0 = time.perf_counter()
        for _ in range(steps):
            m.apply_mpo(mpo)
            m.compress(cutoff, chi, mode=mode)
            normalise(m)
        sec = time.perf_counter() - t0
        res[mode] = {"seconds": sec, "energy": m.expect_mpo(mpo)}
        m.free()
        eng.close()
    res["dE"] = abs(res["chosen"]["energy"] - res["cusolver"]["energy"])
    return res


def _cpu_update(O, a, b, g, chi, dtype):
    """One update of the oracle's path in `dtype`: for complex128 the oracle's
    own apply_2q; for complex64 its steps with every array in complex64."""
    if dtype == np.complex128:
        sites = [a.copy(), b.copy()]
        O.apply_2q(sites, g, 1, 1e-6, chi)
        return sites[0], sites[1]
    chil, chir = a.shape[0], b.shape[2]
    th = O.theta_of(a, b)
    t4 = th.reshape((chil, 2, 2, chir), order="F")
    g4 = np.asarray(g, dtype=np.complex64).reshape((2, 2, 2, 2), order="F")
    th = np.einsum("pqrs,arsb->apqb", g4, t4).reshape((2 * chil, 2 * chir), order="F")
    u, s, vh = O.svd_gesdd(th)
    k = min(O.tail_rank(s.astype(np.float64), 1e-6, clamp=True), chi)
    a2 = u[:, :k].reshape((chil, 2, k), order="F")
    b2 = (s[:k, None] * vh[:k, :]).reshape((k, 2, chir), order="F")
    return a2, b2


def cpu1(qt, args):
    """Timings at the thread count this process was started with."""
    import oracle as O
    rows = []
    for chi in args.c2_chis:
        for dtype in (np.complex128, np.complex64):
            rng = np.random.default_rng(chi)
            a, b, _ = O.decay_theta_factors(chi, rng)
            g = O.haar_unitary(rng)
            a, b = a.astype(dtype), b.astype(dtype)
            _cpu_update(O, a, b, g, chi, dtype)
            ts = []
            for _ in range(args.cpu_reps):
                t0 = time.perf_counter()
                _cpu_update(O, a, b, g, chi, dtype)
                ts.append(time.perf_counter() - t0)
            ts.sort()
            med = ts[len(ts) // 2]
            rows.append({"chi": chi, "dtype": "c128" if dtype == np.complex128 else "c64",
                         "ms_per_update": 1e3 * med, "updates_per_s": 1.0 / med})
    return {"config": "cpu1", "threads": os.environ.get("OPENBLAS_NUM_THREADS", "default"), "rows": rows}


def cpu(qt, args):
    """cpu1 in child processes with OpenBLAS on all host threads and on one."""
    import subprocess
    out = {"config": "cpu", "host_cores": os.cpu_count(), "runs": []}
    for threads in (os.cpu_count(), 1):
        env = dict(os.environ, OPENBLAS_NUM_THREADS=str(threads), OMP_NUM_THREADS=str(threads))
        cmd = [sys.executable, os.path.abspath(__file__), "cpu1", "--cpu-reps", str(args.cpu_reps), "--c2-chis"] + \
            [str(c) for c in args.c2_chis]
        res = subprocess.run(cmd, env=env, capture_output=True, text=True, check=True)
        out["runs"].append(json.loads(res.stdout.strip().splitlines()[-1]))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("configs", nargs="+")
    ap.add_argument("--c2-chis", type=int, nargs="+", default=[64, 256, 1024])
    ap.add_argument("--c3-depth", type=int, default=20)
    ap.add_argument("--c3-observables", action="store_true")
    ap.add_argument("--c4-circuits", type=int, default=4096)
    ap.add_argument("--c4-check", type=int, default=24)
    ap.add_argument("--c5-chi", type=int, default=512)
    ap.add_argument("--c5-steps", type=int, default=10)
    ap.add_argument("--cpu-reps", type=int, default=5)
    args = ap.parse_args()
    qt = None
    if any(c not in ("cpu", "cpu1") for c in args.configs):
        import __graft_entry__ as g
        qt = g.load_package()
    # one process per GPU (torchrun): only c4 shards; rank 0 prints
    args.dist = None
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import bench
        args.dist = bench.Dist()
    rank = args.dist.rank if args.dist is not None else 0
    for c in args.configs:
        if c != "c4" and rank != 0:
            continue
        t0 = time.perf_counter()
        r = {"c1": c1, "c2": c2, "c3": c3, "c4": c4, "c5": c5, "cpu": cpu, "cpu1": cpu1}[c](qt, args)
        r["wall_seconds"] = time.perf_counter() - t0
        if rank == 0:
            print(json.dumps(r), flush=True)
    if args.dist is not None:
        args.dist.close()


if __name__ == "__main__":
    main()
