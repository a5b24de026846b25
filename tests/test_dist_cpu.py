"""The multi-process plumbing of bench.py on CPU: two gloo ranks agree on
the max-over-ranks timing, and the reference arm launched as two ranks
prints exactly one JSON line (from rank 0) while the other rank exits 0."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    class A:
        impl = "reference"

    ws, r, _ = bench.dist_setup(A)
    assert (ws, r) == (world, rank)
    bench.barrier(ws)
    m = bench.all_max(ws, 1.5 + rank)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(m))
    dist.destroy_process_group()


def test_all_max_over_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    vals = [float((tmp_path / f"rank{r}.txt").read_text()) for r in range(2)]
    assert vals == [2.5, 2.5]


def test_reference_arm_under_two_ranks():
    pytest.importorskip("torch")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--workload", "0"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=240, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
