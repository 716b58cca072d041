"""The reference arm of bench.py on the host CPU: one JSON line with the benchmark contract's
keys, timed on a small synthetic workload (the oracle restatement of the reference path)."""

import json
import subprocess
import sys

from conftest import REPO


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--workload", "rhf_nao24",
                          "--steps", "2", "--warmup", "3", "--cpu-sample", "3"],
                         capture_output=True, text=True, timeout=600, cwd=str(REPO))
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 3
    assert d["extrapolated"] is True and d["measured_step_s"] > 0
    assert d["value"] > 0 and d["higher_is_better"] is False
    assert d["config"]["workload"] == "rhf_nao24"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_two_ranks_gloo():
    """Under torchrun with two ranks (gloo on CPU) only rank 0 runs and prints its line."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), str(REPO / "bench.py"),
           "--impl", "reference", "--workload", "rhf_nao24", "--gpus", "2", "--steps", "1", "--warmup", "3",
           "--cpu-sample", "3"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=str(REPO))
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2


def _max_worker(rank, world, port, q):
    import os
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    sys.path.insert(0, str(REPO))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        q.put((rank, bench.max_over_ranks(world, 1.5 + rank)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    """The step time reported is the maximum over ranks (two gloo ranks on CPU)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_max_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
    assert all(p.exitcode == 0 for p in procs)
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 2.5, 1: 2.5}
