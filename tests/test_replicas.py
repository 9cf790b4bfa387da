"""CPU: bench.py's multi-process path (one rank per GPU, replicas of the
foam) with the gloo backend and two ranks on 127.0.0.1.

  * the rank helpers: process-group set-up from the torchrun environment, the
    barrier, and the reductions the line uses (sum of bubble-steps over ranks,
    maximum of the timed region);
  * the reference arm launched through torchrun for N = 2: rank 0
    alone runs the CPU restatement and prints one JSON line, rank 1 exits 0
    without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    total = bench.allreduce(1000.0 * (r + 1), bench._op("sum"), w)
    slowest = bench.allreduce(0.5 + r, bench._op("max"), w)
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.json" % r), "w") as f:
        json.dump({"world": w, "rank": r, "total": total, "slowest": slowest}, f)


def test_rank_helpers_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        d = json.load(open(tmp_path / ("rank%d.json" % r)))
        assert d["world"] == 2 and d["rank"] == r
        assert d["total"] == 3000.0      # bubble-steps summed over the replicas
        assert d["slowest"] == 1.5       # the line's time is the slowest rank's


def test_reference_arm_under_torchrun():
    pytest.importorskip("oracle.oracle")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--workload", "c1", "--steps", "4",
           "--warmup", "3", "--ref-steps", "4"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 only
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
