#!/usr/bin/env python
"""Two-qubit gate + truncated-SVD updates per second at chi = 1024 on one GB300.

Workload (one step = one update of one bond): theta = A.B with A, B of shape
(1024, 2, 1024); theta's singular spectrum is 0.97^k normalised to unit norm
(A = Q1[:, :chi] diag(s), B = Q2[:, :chi]^H with Q1, Q2 from QR of seeded
complex Gaussian 2048 x 2048 matrices); a seeded Haar-random gate on the two
physical legs; truncation by the tail rule at cutoff 1e-6 and chi_max = 1024.
Storage complex64, the mixed-precision ("chosen") mode.  Beside it the plain
FP64 GPU path and the cuSOLVER FP64 cross-check are timed on the same inputs.

`value` is updates/s with the inputs resident in HBM (each step clones the
resident input MPS on the device, flushes L2 by writing a 256 MiB buffer and
runs the update); `e2e` is the same metric through the host-buffer API
(pinned host arrays uploaded, updated, downloaded every step).

Multi-GPU: replicas only (one independent bond stream per GPU, no collective
on the data path); value = all ranks' updates / max-over-ranks time.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "2q gate+SVD updates/s at \u03c7=1024: chosen vs plain FP64 GPU at |\u0394E|\u22641e-6"
CHI = 1024
CUTOFF = 1e-6
DECAY = 0.97
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")


def workload_config(chi: int, world: int) -> dict:
    return {"workload": f"single-bond 2q gate+SVD update, theta (chi,2,2,chi) chi={chi}, spectrum {DECAY}^k unit "
                        f"norm, Haar gate, cutoff {CUTOFF}, chi_max {chi}",
            "parallelism": f"replicas x{world}", "l2": "256 MiB device write between steps"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--chi", type=int, default=CHI)
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--no-baselines", action="store_true",
                    help="skip the plain FP64 / cuSOLVER / CPU legs and the accuracy check (profiling runs)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------

def decay_pair(chi: int, seed: int):
    rng = np.random.default_rng(seed)
    n = 2 * chi
    g1 = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(2)
    g2 = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(2)
    q1, _ = np.linalg.qr(g1)
    q2, _ = np.linalg.qr(g2)
    s = DECAY ** np.arange(chi, dtype=np.float64)
    s /= np.linalg.norm(s)
    a = (q1[:, :chi] * s[None, :]).reshape((chi, 2, chi), order="F")
    b = q2[:, :chi].conj().T.reshape((chi, 2, chi), order="F")
    return a, b, s


def haar(rng):
    z = (rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))) / math.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))[None, :]


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        # QT_CLOCKS_DIR keeps the samples (the system temporary directory by default)
        out = os.environ.get("QT_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out, f"clocks_bench_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, fl in rows for i, f in enumerate(fl) if f.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)
# ---------------------------------------------------------------------------

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


# ---------------------------------------------------------------------------
# the engine arm
# ---------------------------------------------------------------------------

def load_engine():
    import __graft_entry__ as g
    return g.load_package()


def load_rank_model(eng):
    p = os.path.join(ROOT, "qaintensor.jl_gb300", "rank_model_params.npy")
    if os.path.exists(p):
        eng.set_rank_params(np.load(p), enable=True)
        return p
    return None


def run_updates(eng, templates, gates, steps, flush):
    """steps updates; returns (device ms, list of stats)."""
    stats = []
    eng.sync()
    eng.timer_record(0)
    for i in range(steps):
        flush()
        m = templates[i % len(templates)].clone()
        stats.append(m.apply_2q(gates[i % len(gates)], 1))
        m.free()
    eng.timer_record(1)
    return eng.timer_elapsed(0, 1), stats


def bench_ours(args, dist: Dist):
    qt = load_engine()
    dev = dist.local
    chi = args.chi
    seeds = [1001 + 2 * dist.rank, 1002 + 2 * dist.rank]
    pairs = [decay_pair(chi, s) for s in seeds]
    rng = np.random.default_rng(77 + dist.rank)
    gates = [haar(rng) for _ in range(max(8, args.steps + args.warmup))]

    eng = qt.Engine(mode="chosen", cutoff=CUTOFF, chi_max=chi, device=dev, tc_gemm=1)
    model_path = load_rank_model(eng)
    templates = []
    for a, b, s in pairs:
        t = eng.mps([a.astype(np.complex64), b.astype(np.complex64)], dtype=np.complex64)
        t.set_bond_spectrum(1, s)
        templates.append(t)
    flush = eng.l2_flush
    # warm-up
    for i in range(args.warmup):
        m = templates[i % 2].clone()
        m.apply_2q(gates[i], 1)
        m.free()
    dist.barrier()
    eng.sync()
    clocks = ClockSampler(dev)
    clocks.start()
    l0 = eng.launches
    ms, stats = run_updates(eng, templates, gates[args.warmup:], args.steps, flush)
    launches = eng.launches - l0
    clk = clocks.stop()
    dist.barrier()
    ms_max = dist.max(ms)
    total_updates = dist.sum(args.steps)
    value = total_updates / (ms_max / 1e3)

    # per-kernel device times over the same workload (events around every launch)
    eng.profile_enable(True)
    w0 = eng.work_counters()
    n_prof = min(args.steps, 3)
    run_updates(eng, templates, gates[args.warmup:], n_prof, flush)
    w1 = eng.work_counters()
    prof = eng.profile_collect()
    eng.profile_enable(False)
    work = {k: (w1[k] - w0[k]) / n_prof for k in w0}  # per update

    out = {"value": value, "ms": ms_max, "stats": stats, "launches": launches, "clocks": clk, "profile": prof,
           "model": model_path, "work": work, "n_prof": n_prof}

    # end-to-end through the host-buffer API
    a64 = [eng.pinned_empty((chi, 2, chi), np.complex64) for _ in range(2)]
    b64 = [eng.pinned_empty((chi, 2, chi), np.complex64) for _ in range(2)]
    for j, (a, b, _) in enumerate(pairs):
        a64[j][...] = a
        b64[j][...] = b
    outA = eng.pinned_empty((chi, 2, chi), np.complex64)
    outB = eng.pinned_empty((chi, 2, chi), np.complex64)
    h2d = d2h = 0
    e2e_steps = max(2, min(args.steps, 5))
    dist.barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        j = i % 2
        m = eng.mps([a64[j], b64[j]], dtype=np.complex64)
        m.set_bond_spectrum(1, pairs[j][2])
        st = m.apply_2q(gates[args.warmup + i], 1)
        k = st["rank"]
        oa = np.ndarray((chi, 2, k), dtype=np.complex64, buffer=outA, order="F")
        ob = np.ndarray((k, 2, chi), dtype=np.complex64, buffer=outB, order="F")
        m.download_into(1, oa)
        m.download_into(2, ob)
        m.free()
        h2d += a64[j].nbytes + b64[j].nbytes
        d2h += oa.nbytes + ob.nbytes
    t1 = time.perf_counter()
    e2e_s = dist.max(t1 - t0)
    out["e2e"] = {"value": dist.sum(e2e_steps) / e2e_s, "unit": "updates/s", "h2d_bytes_per_step": h2d // e2e_steps,
                  "d2h_bytes_per_step": d2h // e2e_steps}

    # accuracy of one chosen update against the engine's exact FP64 path
    if not args.no_baselines:
        out["accuracy"] = accuracy_check(qt, dev, pairs[0], gates[args.warmup])

    # plain FP64 GPU and cuSOLVER FP64 denominators (same inputs, fewer steps)
    if not args.no_baselines:
        out["plain"] = time_mode(qt, dev, pairs, gates[args.warmup:], "plain", args.plain_steps)
        out["cusolver"] = time_mode(qt, dev, pairs, gates[args.warmup:], "cusolver", args.plain_steps)
    for t in templates:
        t.free()
    eng.close()
    return out


def time_mode(qt, dev, pairs, gates, mode, steps):
    eng = qt.Engine(mode=mode, cutoff=CUTOFF, chi_max=CHI, device=dev)
    tmpl = [eng.mps([a, b], dtype=np.complex128) for a, b, _ in pairs]
    m = tmpl[0].clone()
    m.apply_2q(gates[0], 1)  # warm-up
    m.free()
    ms, stats = run_updates(eng, tmpl, gates[1:], steps, lambda: None)
    for t in tmpl:
        t.free()
    eng.close()
    return {"updates_per_s": steps / (ms / 1e3), "ms_per_update": ms / steps, "rank": stats[0]["rank"],
            "sweeps": stats[0]["sweeps"]}


def accuracy_check(qt, dev, pair, gate):
    a, b, s = pair
    chi = a.shape[0]
    ex = qt.Engine(mode="plain", cutoff=CUTOFF, chi_max=chi, device=dev)
    ch = qt.Engine(mode="chosen", cutoff=CUTOFF, chi_max=chi, device=dev, tc_gemm=1)
    load_rank_model(ch)
    m1 = ex.mps([a.astype(np.complex64).astype(np.complex128), b.astype(np.complex64).astype(np.complex128)])
    st1 = m1.apply_2q(gate, 1)
    m2 = ch.mps([a.astype(np.complex64), b.astype(np.complex64)], dtype=np.complex64)
    m2.set_bond_spectrum(1, s)
    st2 = m2.apply_2q(gate, 1)
    A1, B1 = m1.site(1), m1.site(2)
    A2, B2 = m2.site(1).astype(np.complex128), m2.site(2).astype(np.complex128)
    t1 = A1.reshape((2 * chi, -1), order="F") @ B1.reshape((B1.shape[0], -1), order="F")
    t2 = A2.reshape((2 * chi, -1), order="F") @ B2.reshape((B2.shape[0], -1), order="F")
    # exact theta' in FP64 from the same complex64 inputs
    a64, b64 = a.astype(np.complex64).astype(np.complex128), b.astype(np.complex64).astype(np.complex128)
    th = a64.reshape((2 * chi, chi), order="F") @ b64.reshape((chi, 2 * chi), order="F")
    g4 = np.asarray(gate).reshape((2, 2, 2, 2), order="F")
    th = np.einsum("pqrs,arsb->apqb", g4, th.reshape((chi, 2, 2, chi), order="F")).reshape((2 * chi, 2 * chi), order="F")
    err_exact = np.linalg.norm(th - t1)
    err_chosen = np.linalg.norm(th - t2)
    # <Z_1> and <Z_2> of the two-site state (theta'/||theta'||)
    def zexp(t, which):
        t4 = t.reshape((chi, 2, 2, chi), order="F")
        w = np.sum(np.abs(t4) ** 2, axis=(0, 3))
        z = np.array([1.0, -1.0])
        return float((z @ w.sum(1)) / w.sum()) if which == 1 else float((w.sum(0) @ z) / w.sum())
    dz = max(abs(zexp(t1, 1) - zexp(t2, 1)), abs(zexp(t1, 2) - zexp(t2, 2)))
    for o in (m1, m2):
        o.free()
    ex.close()
    ch.close()
    return {"rank_exact": st1["rank"], "rank_chosen": st2["rank"], "predicted_rank": st2["predicted_rank"],
            "sketch_size": st2["sketch_size"], "fallback": st2["fallback"],
            "trunc_err_exact": err_exact, "trunc_err_chosen": err_chosen,
            "trunc_err_ratio": err_chosen / err_exact if err_exact > 0 else None, "dZ_vs_exact": dz}


def cpu_baseline(chi, pair, gate):
    """The oracle (numpy/scipy gesdd on OpenBLAS) on one update of the same workload."""
    import oracle
    a, b, _ = pair
    t0 = time.perf_counter()
    n = 0
    while True:
        oracle.apply_2q([a.copy(), b.copy()], gate, 1, CUTOFF, chi)
        n += 1
        if time.perf_counter() - t0 > 10.0 or n >= 3:
            break
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "updates/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{n} update(s) of the chi={chi} workload (numpy gesdd, OpenBLAS on all host threads)"}


# ---------------------------------------------------------------------------
# roofline
# ---------------------------------------------------------------------------

def load_peaks():
    try:
        with open(PEAKS_FILE) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profiled_traffic(kernel):
    """DRAM bytes per launch of `kernel` from its committed ncu summary
    (profiles/<kernel>_chi1024_bench.md, line `traffic_per_launch_bytes: N`,
    captured on this bench's workload), or None."""
    base = kernel.split("<")[0].split("(")[-1].strip()
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", f"{base}_chi1024_bench.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_per_launch_bytes:"):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def roofline(prof, work, n_prof, sm_mhz=2070.0):
    """Roofline of the dominant kernel (largest total device time in the
    profiled updates), from the engine's algorithmic work counters:
      Jacobi round kernels (FP32 storage): bound by the FP32 FMA pipe they run
        on.  Algorithmic FMAs of a round: per row of a rotated pair, 1024
        complex-as-real FMAs of the rebuild (16 columns x a 16 x 8 block of
        the pair unitary, twice) and 544 of the pair Gram (its upper 4 x 4
        tiles of the 16 x 16 complex Gram); the counters give them as
        8 x rot_bytes and 4.25 x gram_bytes.  Peak = 152 SMs x 128 FP32
        FMA/clock x 2 flops at the SM clock sampled during the run (the
        measured peaks hold no FP32 figure).  Their bytes stay in L2 (the
        ping-pong columns of a 2048 x 1152 complex64 matrix are 19 MB), so
        the DRAM traffic of the ncu capture is reported beside it;
      tc_gemm_kernel: tensor bound; 24 M N K TF32 flops per complex product,
        peak = half the measured dense bf16 rate (TF32 runs at half the bf16
        tensor rate)."""
    if not prof:
        return None
    peaks, src = load_peaks()
    name, launches, ms = prof[0]
    per_launch_s = ms / 1e3 / launches
    fp32_kernels = ("pair_round_kernel", "jacobi_sweep32_kernel", "(gram_kernel", "pair_eig32_kernel",
                    "apply_kernel", "pair_apply32_kernel")
    if name.startswith(fp32_kernels):
        if work["jacobi_rounds"] <= 0:
            return {"kernel": name, "note": "no Jacobi work recorded"}
        fma = 8.0 * work["jacobi_rot_bytes"] + 4.25 * work["jacobi_gram_bytes"]
        if name.startswith("pair_eig32_kernel") or name.startswith("(gram_kernel"):
            fma = 4.25 * work["jacobi_gram_bytes"]
        elif name.startswith("pair_apply32_kernel") or name.startswith("apply_kernel"):
            fma = 8.0 * work["jacobi_rot_bytes"]
        # work counters are per update; the profile covers n_prof updates
        flops_per_launch = 2.0 * fma * n_prof / launches
        achieved = flops_per_launch / per_launch_s / 1e12
        peak = 2.0 * 152 * 128 * sm_mhz * 1e6 / 1e12
        return {"kernel": name, "bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": profiled_traffic(name), "flops_per_launch": flops_per_launch,
                "l2_bytes_per_launch": work["jacobi_bytes"] * n_prof / launches,
                "peak_source": f"152 SMs x 128 FMA/clock x 2 at the sampled SM clock {sm_mhz:.0f} MHz",
                "note": "traffic = DRAM bytes per launch of the committed ncu capture of this workload"}
    if name.startswith("tc_gemm_kernel"):
        n_launch = work["tc_launches"]
        flops_per_launch = work["tc_flops"] / max(n_launch, 1)
        achieved = flops_per_launch / per_launch_s / 1e12
        peak = peaks["bf16_tflops"] / 2
        return {"kernel": name, "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": profiled_traffic(name),
                "peak_source": f"{src} bf16_tflops / 2 (TF32)"}
    return {"kernel": name, "note": "no work model for this kernel"}


# ---------------------------------------------------------------------------
# the reference arm: the CPU restatement of the reference path
# ---------------------------------------------------------------------------

def bench_reference(args, dist: Dist):
    if dist.rank != 0:
        return None
    import oracle
    chi = args.chi
    pair = decay_pair(chi, 1001)
    rng = np.random.default_rng(77)
    # the same K and W as the engine's arm, unless the steps would take more
    # than about three minutes of host time (then as many as fit)
    gates = [haar(rng) for _ in range(args.steps + args.warmup + 8)]
    warm = args.warmup
    t0 = time.perf_counter()
    for i in range(warm):
        oracle.apply_2q([pair[0].copy(), pair[1].copy()], gates[i], 1, CUTOFF, chi)
    per = (time.perf_counter() - t0) / max(warm, 1)
    steps = max(1, min(args.steps, int(180.0 / max(per, 1e-9)))) if warm else max(1, args.steps)
    t0 = time.perf_counter()
    for i in range(steps):
        oracle.apply_2q([pair[0].copy(), pair[1].copy()], gates[warm + i], 1, CUTOFF, chi)
    dt = time.perf_counter() - t0
    v = steps / dt
    return {"metric": METRIC, "value": v, "unit": "updates/s", "n_gpus": 0,
            "steps": steps, "warmup": warm, "ms_per_step": dt / steps * 1e3, "higher_is_better": True,
            "impl": "reference", "dtype": "c128", "data": "synthetic",
            "config": workload_config(chi, 1),
            "cpu_baseline": {"value": v, "unit": "updates/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{steps} timed update(s) of the chi={chi} workload after {warm} warm-up "
                                       f"(numpy gesdd, OpenBLAS on all host threads)"},
            "e2e": {"value": v, "unit": "updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "vs_baseline": None}


def free_port() -> int:
    import socket
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def launch_command(argv, gpus: int, port: int):
    """The one-process-per-GPU launch of this script on `gpus` local GPUs."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={gpus}",
            "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + list(argv)


def check_world(args, env):
    """None when this process should run the bench itself; otherwise the exit
    status of the launch it made.  `--gpus N` without a launcher (WORLD_SIZE
    unset) starts N local ranks through torch.distributed.run; under a
    launcher, a WORLD_SIZE other than N is refused."""
    world = env.get("WORLD_SIZE")
    if world is None:
        if args.gpus > 1:
            return subprocess.call(launch_command(sys.argv[1:], args.gpus, free_port()))
        return None
    if int(world) != args.gpus:
        print(json.dumps({"error": f"--gpus {args.gpus} but WORLD_SIZE={world}: launch one rank per GPU"}),
              file=sys.stderr)
        return 2
    return None


def main():
    args = parse()
    rc = check_world(args, os.environ)
    if rc is not None:
        sys.exit(rc)
    dist = Dist()
    if args.impl == "reference":
        line = bench_reference(args, dist)
        if line is not None:
            print(json.dumps(line))
        dist.close()
        return
    res = bench_ours(args, dist)
    if dist.rank == 0:
        stats = res["stats"]
        prof = res["profile"]
        line = {
            "metric": METRIC,
            "value": res["value"], "unit": "updates/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64",
            "data": "synthetic (seeded decaying-spectrum theta, Haar gates)",
            "config": dict(workload_config(args.chi, dist.world),
                           rank_model=os.path.relpath(res["model"], ROOT) if res["model"] else None),
            "gpu_launches": res["launches"],
            "clocks": res["clocks"],
            "e2e": res["e2e"],
            "update_stats": {k: stats[0][k] for k in ("rank", "predicted_rank", "sketch_size", "fallback", "sweeps")},
            "accuracy": res.get("accuracy"),
            "kernels": [{"name": n, "launches": c, "ms": round(t, 3)} for n, c, t in prof[:8]],
        }
        line["roofline"] = roofline(prof, res["work"], res["n_prof"],
                                    (res["clocks"] or {}).get("sm_mhz") or 2070.0)
        if "plain" in res:
            line["plain_fp64_gpu"] = res["plain"]
            line["cusolver_fp64_gpu"] = res["cusolver"]
            best = max(res["plain"]["updates_per_s"], res["cusolver"]["updates_per_s"])
            line["speedup_vs_best_plain_fp64"] = res["value"] / best
            pair = decay_pair(args.chi, 1001)
            rng = np.random.default_rng(77)
            line["cpu_baseline"] = cpu_baseline(args.chi, pair, haar(rng))
        print(json.dumps(line))
    dist.close()


if __name__ == "__main__":
    main()
