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


def _clock_summary(tmp_path, lines):
    sys.path.insert(0, ROOT)
    import bench
    s = bench.ClockSampler(0)
    s.path = str(tmp_path / "clocks.csv")
    with open(s.path, "w") as f:
        f.write("".join(ln + "\n" for ln in lines))
    return s.summary()


def test_clock_summary_reads_the_timed_region(tmp_path):
    """The bench's clock record: the median SM clock over the loaded samples
    (idle ones, below half the maximum, are left out), the maximum, and the
    throttle reasons seen Active in any sample."""
    idle = "0, 345, 2070, 150.2, 0x0000000000000001, Not Active, Not Active, Not Active, Not Active"
    busy = "0, 2070, 2070, 1100.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
    capped = "0, 1980, 2070, 1400.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
    s = _clock_summary(tmp_path, [idle, busy, busy, capped, busy, "garbage"])
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 5
    assert s["reasons"] == ["sw_power_cap"]
    hot = busy.replace("Not Active, Not Active, Not Active, Not Active", "Not Active, Active, Not Active, Not Active")
    assert _clock_summary(tmp_path, [busy, hot])["reasons"] == ["hw_thermal_slowdown"]
    # no nvidia-smi (or no sample): the line says so instead of inventing clocks
    s = _clock_summary(tmp_path, [])
    assert s["sm_mhz"] is None and s["samples"] == 0 and s["reasons"] == ["clock sampling unavailable"]


def test_error_summary_and_work_count():
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench
    from xrd_tomography_gb300 import synth
    e = bench.err_summary([1.0, 2.0, 1e-12], [1.0, 2.0, 0.0])
    # the zero reference entry is compared against 1e-6 of the largest (2.0)
    assert abs(e["max_rel"] - 5e-7) < 1e-15 and abs(e["mean_rel"] - 5e-7 / 3) < 1e-15 and e["n"] == 3
    e = bench.err_summary([1.0, 2.0 * (1 + 1e-6)], [1.0, 2.0])
    assert abs(e["max_rel"] - 1e-6) < 1e-12
    inp = synth.make_inputs(synth.tiny_problem(), 1)
    p = inp.problem
    nv = int((np.asarray(inp.seg) > 0).sum())
    # reference-equivalent terms: every (ray, non-empty voxel, window energy, fine q bin)
    assert bench.ref_equiv_terms(inp, 10) == 10.0 * nv * (2 * p.dnrg + 1) * p.nqf
    assert bench.ref_equiv_terms(inp) == float(p.rays) * nv * (2 * p.dnrg + 1) * p.nqf
