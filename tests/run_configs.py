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


RANK_MODEL = os.path.join(ROOT, "qaintensor.jl_gb300", "rank_model_params.npy")


def load_rank_model(eng, path=None):
    """Enable the shipped rank model (or the one at `path`); returns its path or None."""
    p = path or RANK_MODEL
    if os.path.exists(p):
        eng.set_rank_params(np.load(p), enable=True)
        return os.path.relpath(p, ROOT)
    return None


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


def zz_all_bonds(sites):
    """<Z_i Z_i+1>/<psi|psi> on every bond from one left and one right
    environment sweep (FP64, the oracle's transfer convention)."""
    n = len(sites)
    z = np.diag([1.0, -1.0]).astype(np.complex128)
    left = [np.ones((1, 1), dtype=np.complex128)]
    for a in sites:
        left.append(np.einsum("ab,asc,bsd->cd", left[-1], a.conj(), a, optimize=True))
    right = [np.ones((1, 1), dtype=np.complex128)]
    for a in reversed(sites):
        right.append(np.einsum("asc,bsd,cd->ab", a.conj(), a, right[-1], optimize=True))
    right = right[::-1]  # right[i]: environment of sites i..n-1 (0-based)
    norm = float(np.real(left[n][0, 0]))
    out = []
    for i in range(n - 1):
        a, b = sites[i], sites[i + 1]
        e = np.einsum("ab,asc,st,btd->cd", left[i], a.conj(), z, a, optimize=True)
        e = np.einsum("ab,asc,st,btd->cd", e, b.conj(), z, b, optimize=True)
        out.append(float(np.real(np.einsum("cd,cd->", e, right[i + 2]))) / norm)
    return out


def run_reference_chain(n, gates, cutoff, chi_max, storage):
    """The FP64 oracle's update chain (src/switch.jl split, src/svd.jl:29-33
    rule, chi_max cap); storage "c64" rounds every updated site to complex64,
    the storage of the chosen mode, so the run isolates what the FP64 split
    achieves on that storage.  Returns the sites."""
    import oracle as O
    sites = O.product_state(n)
    for (_, w, g) in gates:
        O.apply_2q(sites, g, w, cutoff, chi_max)
        if storage == "c64":
            sites[w - 1] = sites[w - 1].astype(np.complex64).astype(np.complex128)
            sites[w] = sites[w].astype(np.complex64).astype(np.complex128)
    return sites


def c3_gates(args):
    return brickwork(args.c3_n, args.c3_depth, np.random.default_rng(64))


def c3ref(qt, args):
    """The FP64 oracle run of the c3 circuit on the CPU (complex128 storage,
    or complex64 storage with --c3-ref-storage c64): <Z_i Z_i+1> on every bond."""
    sites = run_reference_chain(args.c3_n, c3_gates(args), 1e-8, args.c3_chi_max, args.c3_ref_storage)
    return {"config": "c3ref", "storage": args.c3_ref_storage, "n": args.c3_n, "depth": args.c3_depth,
            "chi_max": args.c3_chi_max, "ZZ": zz_all_bonds(sites)}


def c3(qt, args):
    """64-qubit brickwork, complex64, chi_max 1024, cutoff 1e-8, chosen mode:
    updates/s, the rank decisions and <Z_i Z_i+1> on every bond, compared with
    the FP64 oracle runs given by --c3-ref-json (made by c3ref on the CPU);
    --c3-ablate also runs without the rank model."""
    n, depth, chi_max, cutoff = args.c3_n, args.c3_depth, args.c3_chi_max, 1e-8
    gates = c3_gates(args)
    out = {"config": "c3", "n": n, "depth": depth, "chi_max": chi_max, "updates": len(gates)}
    refs = {}
    for path in args.c3_ref_json or []:
        with open(path) as f:
            r = json.load(f)
        if (r["n"], r["depth"], r["chi_max"]) == (n, depth, chi_max):
            refs[r["storage"]] = np.array(r["ZZ"])
    opts = {"jacobi_tol": args.c3_jacobi_tol} if args.c3_jacobi_tol else {}
    out["jacobi_tol"] = args.c3_jacobi_tol or "default"
    for use_model in ((True, False) if args.c3_ablate else (True,)):
        eng = qt.Engine(mode="chosen", tc_gemm=1, **opts)
        model = load_rank_model(eng, args.rank_model) if use_model else None
        mps = eng.product_state(n, dtype=np.complex64)
        eng.sync()
        t0 = time.perf_counter()
        stats = []
        for (layer, w, g) in gates:
            mps.set_circuit_position(layer, depth)
            stats.append(mps.apply_2q(g, w, cutoff, chi_max))
        eng.sync()
        dt = time.perf_counter() - t0
        row = {"seconds": dt, "updates_per_s": len(gates) / dt, "rank_model": model,
               "max_rank": max(s["rank"] for s in stats), "fallbacks": sum(1 for s in stats if s["fallback"]),
               "sketched": sum(1 for s in stats if s["sketch_size"] > 0), "cert": eng.cert_counters()}
        pr = [(s["predicted_rank"], s["rank"]) for s in stats if s["predicted_rank"] > 0]
        if pr:
            p, k = np.array(pr, dtype=float).T
            row["predicted_vs_rank"] = {"updates": len(pr), "exact": int(np.sum(p == k)),
                                        "mean_abs_rel": float(np.mean(np.abs(p - k) / k)),
                                        "under": int(np.sum(p < k))}
        if args.c3_observables or refs:
            zz = np.array([mps.expect_zz(i) for i in range(1, n)])
            row["ZZ"] = zz.tolist()
            for st, zr in refs.items():
                row["dZZ_max_vs_fp64_" + st] = float(np.abs(zz - zr).max())
                row["dZZ_median_vs_fp64_" + st] = float(np.median(np.abs(zz - zr)))
        out["with_model" if use_model else "without_model"] = row
        mps.free()
        eng.close()
    if "c128" in refs and "c64" in refs:
        d = np.abs(refs["c64"] - refs["c128"])
        out["dZZ_fp64_split_c64_storage"] = {"max": float(d.max()), "median": float(np.median(d))}
    return out


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
    rate is all ranks' updates over the slowest rank's time.  With
    --c4-autotune the tuned launch shapes are timed beside the defaults;
    --c4-dump writes every circuit's <Z_1> for c4check (the oracle check on
    the CPU, off the GPU machine)."""
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
    variants = [("default", None)]
    tuned_entry = None
    if getattr(args, "c4_autotune", None):
        import importlib.util
        spec = importlib.util.spec_from_file_location(
            "qaintensor_gb300_autotune", os.path.join(ROOT, "qaintensor.jl_gb300", "autotune.py"))
        at = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(at)
        cache = at.load(args.c4_autotune)
        if not at.device_entry(cache, local).get("batch"):
            at.tune(qt, args.c4_autotune, device=local, ncirc=args.c4_tune_circuits, reps=2)
            cache = at.load(args.c4_autotune)
        tuned_entry = at.device_entry(cache, local).get("batch")
        variants.append(("tuned", lambda bb: at.apply_batch(bb, cache, local)))
    rates, ntask_all, z, cert = {}, ntask, None, None
    for name, apply in variants:
        b = qt.Batch(eng, [circuits[ci][0] for ci in mine], [circuits[ci][2] for ci in mine])
        if apply is not None:
            apply(b)
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
        rates[name] = {"seconds": dt, "updates_per_s": ntask_all / dt}
        z = gather_by_circuit(dist, mine, [float(v) for v in b.expect_z(1)], nc)
        cert = b.cert_counts()
        b.free()
    eng.close()
    dt = rates[variants[-1][0]]["seconds"]
    res = {"config": "c4", "circuits": nc, "ranks": world, "updates": ntask_all, "seconds": dt,
           "updates_per_s": ntask_all / dt, "launch_shapes": rates, "cert": cert}
    if tuned_entry:
        res["tuned"] = {k: {"threads": v["threads"], "ctas_per_sm": v["ctas_per_sm"]} for k, v in tuned_entry.items()}
    if rank == 0 and getattr(args, "c4_dump", None):
        with open(args.c4_dump, "w") as f:
            json.dump({"circuits": nc, "Z1": z}, f)
    if rank == 0 and args.c4_check > 0:
        res.update(c4_errors(O, circuits, z, args, rng))
    return res


def c4_errors(O, circuits, z, args, rng):
    """<Z_1> of a sample of circuits against the FP64 oracle (and, with
    --c4-storage-ref, the FP64 split on complex64 storage against it)."""
    errs, errs_c64 = [], []
    for ci in rng.choice(len(circuits), size=min(len(circuits), args.c4_check), replace=False):
        n, depth, chi, gates = circuits[ci]
        zr = O.expect_z(run_reference_chain(n, gates, 1e-8, chi, "c128"), 1)
        errs.append(abs(z[ci] - zr))
        if getattr(args, "c4_storage_ref", False):
            errs_c64.append(abs(O.expect_z(run_reference_chain(n, gates, 1e-8, chi, "c64"), 1) - zr))
    out = {"checked": len(errs)}
    if errs:
        out["Z1_err"] = {"max": max(errs), "median": float(np.median(errs)),
                         "le_1e-6": int(sum(e <= 1e-6 for e in errs))}
    if errs_c64:
        out["Z1_err_fp64_split_c64_storage"] = {"max": max(errs_c64), "median": float(np.median(errs_c64))}
    return out


def c4check(qt, args):
    """The oracle check of a c4 run's dumped <Z_1> values, on the CPU."""
    import oracle as O
    with open(args.c4_dump) as f:
        d = json.load(f)
    rng = np.random.default_rng(4096)
    circuits = c4_circuits(d["circuits"], rng)
    return dict({"config": "c4check", "circuits": d["circuits"]}, **c4_errors(O, circuits, d["Z1"], args, rng))


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
    # two FP64 paths at bond 3 chi) on complex128 storage; --c5-storage-ref
    # adds the same FP64 splits on complex64 storage (the floor of that storage)
    runs = [("chosen", np.complex64), ("cusolver", np.complex128)]
    if args.c5_storage_ref:
        runs.append(("cusolver", np.complex64))
    for mode, dt in runs:
        eng = qt.Engine(mode=mode, tc_gemm=1 if mode == "chosen" else 0)
        m = eng.mps([s.astype(dt) for s in sites], dtype=dt)
        normalise(m)
        m.compress(cutoff, chi, mode=mode)
        t0 = time.perf_counter()
        energies = []
        for _ in range(steps):
            m.apply_mpo(mpo)
            m.compress(cutoff, chi, mode=mode)
            normalise(m)
            energies.append(m.expect_mpo(mpo))
        sec = time.perf_counter() - t0
        key = mode if (dt == np.complex128 or mode == "chosen") else mode + "_c64"
        res[key] = {"seconds": sec, "energy": energies[-1], "energies": energies}
        if mode == "chosen":
            res[key]["cert"] = eng.cert_counters()
        m.free()
        eng.close()
    res["dE"] = abs(res["chosen"]["energy"] - res["cusolver"]["energy"])
    res["dE_max_over_steps"] = max(abs(x - y) for x, y in zip(res["chosen"]["energies"], res["cusolver"]["energies"]))
    if "cusolver_c64" in res:
        res["dE_max_fp64_split_c64_storage"] = max(abs(x - y) for x, y in zip(res["cusolver_c64"]["energies"],
                                                                               res["cusolver"]["energies"]))
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
    ap.add_argument("--c3-n", type=int, default=64)
    ap.add_argument("--c3-chi-max", type=int, default=1024)
    ap.add_argument("--c3-ref-json", nargs="*", default=[], help="c3ref outputs (JSON) to compare <ZZ> with")
    ap.add_argument("--c3-ref-storage", default="c128", choices=["c128", "c64"])
    ap.add_argument("--c3-ablate", action="store_true", help="also run c3 without the rank model")
    ap.add_argument("--c3-jacobi-tol", type=float, default=0.0, help="FP32 Jacobi tolerance (0: the engine's default)")
    ap.add_argument("--rank-model", default=None, help="rank-model parameters (.npy) instead of the shipped ones")
    ap.add_argument("--c4-dump", default=None, help="write the per-circuit <Z_1> to this JSON (for c4check)")
    ap.add_argument("--c4-storage-ref", action="store_true")
    ap.add_argument("--c4-autotune", default=None, help="autotuner cache (JSON): time the tuned launch shapes too")
    ap.add_argument("--c4-tune-circuits", type=int, default=256)
    ap.add_argument("--c5-storage-ref", action="store_true")
    ap.add_argument("--c4-circuits", type=int, default=4096)
    ap.add_argument("--c4-check", type=int, default=24)
    ap.add_argument("--c5-chi", type=int, default=512)
    ap.add_argument("--c5-steps", type=int, default=10)
    ap.add_argument("--cpu-reps", type=int, default=5)
    args = ap.parse_args()
    qt = None
    if any(c not in ("cpu", "cpu1", "c3ref", "c4check") for c in args.configs):
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
        r = {"c1": c1, "c2": c2, "c3": c3, "c3ref": c3ref, "c4": c4, "c4check": c4check, "c5": c5, "cpu": cpu,
             "cpu1": cpu1}[c](qt, args)
        r["wall_seconds"] = time.perf_counter() - t0
        if rank == 0:
            print(json.dumps(r), flush=True)
    if args.dist is not None:
        args.dist.close()


if __name__ == "__main__":
    main()
