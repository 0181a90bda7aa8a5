"""The N > 1 plumbing as two gloo ranks on the CPU (one process per GPU, no
collective on the data path):
- bench.py: the max and sum reductions every rank sees, the whole-job value
  (updates of all ranks over the slowest rank's time), per-rank inputs, and
  the reference arm that rank 0 alone runs and prints;
- the sharded batched ensemble of tests/run_configs.py (c4): the
  circuit-to-rank assignment, the summed update count and the final gather
  of per-circuit values, with a stand-in engine in place of the GPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import argparse, json, sys
sys.path.insert(0, %(root)r)
import bench
d = bench.Dist()
r = d.rank
out = {"rank": r, "world": d.world, "max": d.max(float(r + 1)), "sum": d.sum(float(r + 1))}
# timing as bench_ours aggregates it: 5 updates per rank, rank r took 100 (r + 1) ms
out["value"] = d.sum(5) / (d.max(100.0 * (r + 1)) / 1e3)
# per-rank inputs: the seeds bench_ours uses
a0, _, _ = bench.decay_pair(4, 1001 + 2 * r)
out["a0"] = [float(a0.real.sum()), float(a0.imag.sum())]
line = bench.bench_reference(argparse.Namespace(chi=8, steps=2, warmup=1), d)
out["ref"] = line
d.barrier()
d.close()
print(json.dumps(out))
"""


def free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks():
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER % {"root": ROOT}], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    res = []
    for p in procs:
        try:
            out, err = p.communicate(timeout=180)
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
        assert p.returncode == 0, err[-2000:]
        res.append(json.loads(out.strip().splitlines()[-1]))
    res.sort(key=lambda x: x["rank"])
    for x in res:
        assert x["world"] == 2
        assert x["max"] == 2.0 and x["sum"] == 3.0
        assert x["value"] == pytest.approx(10 / 0.2)  # 10 updates over the slower rank's 200 ms
    assert res[0]["a0"] != res[1]["a0"]  # each replica runs its own inputs
    ref = res[0]["ref"]
    assert res[1]["ref"] is None  # the other ranks do no work in the reference arm
    assert ref["impl"] == "reference" and ref["value"] > 0 and ref["steps"] == 2
    assert ref["e2e"]["h2d_bytes_per_step"] == 0 and ref["cpu_baseline"]["kind"] == "port"


C4_WORKER = r"""
import argparse, json, sys, types
import numpy as np
sys.path.insert(0, %(root)r)
sys.path.insert(0, %(tests)r)
import bench
import run_configs as R
d = bench.Dist()

class Engine:
    def __init__(self, mode, device=0):
        self.device = device
    def sync(self):
        pass
    def close(self):
        pass

class Batch:
    def __init__(self, eng, nqubits, chi_max):
        self.nq = list(nqubits)
    def run(self, layers, cutoff, use_graph=True):
        self.ntask = sum(len(l) for l in layers)
    def reset(self):
        pass
    def replay(self):
        pass
    def expect_z(self, i):
        return np.asarray(self.nq, dtype=float)  # stand-in value per circuit: its qubit count
    def cert_counts(self):
        return {"fallback": 0, "resolved": 0, "cap": 0, "struct": self.ntask}
    def free(self):
        pass

nc = 40
res = R.c4(types.SimpleNamespace(Engine=Engine, Batch=Batch), argparse.Namespace(c4_circuits=nc, c4_check=0, dist=d))
circuits = R.c4_circuits(nc, np.random.default_rng(4096))
costs = [c[1] * (c[0] - 1) / 2 * c[2] ** 3 for c in circuits]
shards = R.lpt_shards(costs, d.world)
z = R.gather_by_circuit(d, shards[d.rank], [float(circuits[i][0]) for i in shards[d.rank]], nc)
d.close()
print(json.dumps({"rank": d.rank, "res": res, "shards": shards, "z": z, "n": [c[0] for c in circuits],
                  "tasks": sum(len(c[3]) for c in circuits), "costs": costs}))
"""


def test_sharded_ensemble_two_gloo_ranks():
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", C4_WORKER % {"root": ROOT, "tests": os.path.join(ROOT, "tests")}],
                                      env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    res = []
    for p in procs:
        try:
            out, err = p.communicate(timeout=180)
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
        assert p.returncode == 0, err[-2000:]
        res.append(json.loads(out.strip().splitlines()[-1]))
    res.sort(key=lambda x: x["rank"])
    shards = res[0]["shards"]
    assert shards == res[1]["shards"]  # every rank computes the same assignment
    assert sorted(shards[0] + shards[1]) == list(range(40))  # disjoint, complete
    load = [sum(res[0]["costs"][i] for i in s) for s in shards]
    assert max(load) - min(load) <= max(res[0]["costs"])  # LPT: within one circuit of balance
    for x in res:
        assert x["res"]["ranks"] == 2
        assert x["res"]["updates"] == x["tasks"]  # the ranks' update counts add up to the ensemble's
        assert x["z"] == [float(n) for n in x["n"]]  # the gather puts every circuit's value in its place


def test_bench_gpus_flag_starts_one_rank_per_gpu():
    """`bench.py --gpus 2` with no launcher starts two local ranks through
    torch.distributed.run (here on the reference arm, which needs no GPU):
    rank 0 alone prints the line; a WORLD_SIZE that disagrees with --gpus is
    refused."""
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--chi", "16",
           "--steps", "2", "--warmup", "1"]
    p = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [json.loads(x) for x in p.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["steps"] == 2, p.stdout
    bad = dict(env, WORLD_SIZE="3", RANK="0", LOCAL_RANK="0")
    p = subprocess.run(cmd, env=bad, capture_output=True, text=True, timeout=120)
    assert p.returncode == 2 and "WORLD_SIZE=3" in p.stderr
