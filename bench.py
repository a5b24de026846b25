#!/usr/bin/env python
"""Throughput benchmark of the XRD forward projector (one JSON line).

Workload (N=1): the single-phantom forward model of the 256x256 synthetic
phantom -- 8 materials, 180 views, 512 detector pixels x 64 energy bins,
64-bin source spectrum, 128 fine q bins -- computing the coherent and Compton
counts of all 5.9 M rays (the model matrix is not stored: matrix-free).
A step is one forward projection.

Metric: G ray-voxel-q/s, counted in reference-equivalent units: one
(ray, non-empty voxel, source energy of the ray's window, fine q bin) term
of the Nphotons sum, i.e. rays * voxels * (2*DNRG+1) * NQF per projection,
the dense term count the reference evaluates (integrate_diffraction.cu:266-308).

  value  -- device-resident inputs and outputs, CUDA events on the stream
            the library launches on, L2 flushed (a 256 MB write) between steps
  e2e    -- the same projection through the C ABI with host buffers: the
            inputs are copied from pinned host memory and both outputs back
            to pinned host memory inside the timed region
  cpu_baseline -- the FP64 oracle (the reference's algorithm restated in C,
            OpenMP over rays) on a bounded sample of rays on the host cores
  plain_fp64_gpu -- the FP64 kernel at the reference's launch shape
            (one block per ray) timed on a ray subset

--impl reference times the CPU restatement of the reference's algorithm (the
reference itself needs MATLAB and a removed CUDA texture API) with every host
thread, each step a bounded sample of rays, in the same unit.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = 1            # index of the synthetic configuration
FLUSH_BYTES = 256 << 20
# DRAM bytes (read + write) of k_fwd per (pair, non-empty voxel), from one
# ncu capture of a single launch on the 128x128 workload (4096 pairs x 5009
# voxels); the traffic is the launch's walk table plus a fixed part, so the
# 256x256 figure below is that rate times the pair-voxels of its mean launch
K_FWD_DRAM_BYTES_PER_PAIR_VOXEL = (166727936 + 4232704) / (4096 * 5009)   # 8.33 B (read + write)
# issue slots busy in k_fwd (ncu, the same capture): the kernel is bound by
# instruction issue, not by the SFU rate of the roofline below
K_FWD_ISSUE_BUSY = 0.8392


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU baseline sample")
    ap.add_argument("--no-baselines", action="store_true", help="skip the CPU and plain-FP64 baselines")
    ap.add_argument("--workload", type=int, default=WORKLOAD, choices=[0, 1, 2, 3, 4],
                    help="synthetic configuration (1 is the benchmark; 0 and 2 are small profiling cases; "
                         "3 runs batched MLEM on the 64 phantoms of the batched configuration at their stated "
                         "sizes, several minutes per iteration)")
    ap.add_argument("--batch", type=int, default=None,
                    help="--workload 3: number of phantoms (64); --workload 4 --mlem: number of slices (16)")
    ap.add_argument("--iters", type=int, default=1, help="--workload 3, --workload 4 --mlem: timed MLEM iterations")
    ap.add_argument("--mlem", action="store_true",
                    help="--workload 4: per-voxel MLEM on slices of the 384x384 stack instead of the forward "
                         "projection")
    ap.add_argument("--basis", action="store_true",
                    help="time only the tensor-core basis expansion (the default run includes it)")
    return ap.parse_args()


def ref_equiv_terms(inp, rays=None) -> float:
    p = inp.problem
    nv = int((inp.seg > 0).sum())
    r = p.rays if rays is None else rays
    return float(r) * nv * (2 * p.dnrg + 1) * p.nqf


def workload_config(inp, **extra):
    p = inp.problem
    cfg = {
        "workload": f"single-phantom forward projection, {p.nx}x{p.ny} voxels, {p.n_mat} materials, "
                    f"{p.n_src} views, {p.n_col} px x {p.nrg_det} energy bins, {p.nrg_src}-bin source spectrum, "
                    f"{p.nqf} fine q bins; Nphotons + Cphotons, matrix-free",
        "rays": p.rays,
        "nonempty_voxels": int((inp.seg > 0).sum()),
        "energy_window": 2 * p.dnrg + 1,
        "nqf": p.nqf,
        "seed": inp.meta.get("seed"),
    }
    cfg.update(extra)
    return cfg


# ---- distributed plumbing (one process per GPU; weak scaling) --------------

def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def all_max(ws, x, device=None):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---- clocks sampled during the timed region ---------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


# ---- CPU leg: the oracle on a bounded ray sample ------------------------------

def cpu_sample_rate(inp, budget_s: float, rng_seed: int = 0):
    """G ray-voxel-q/s of the FP64 oracle with all host threads, on a ray
    sample sized to about budget_s seconds."""
    from oracle import pyoracle
    pyoracle.build(ref=False)
    p = inp.problem
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(rng_seed)
    calib = rng.choice(p.rays, threads, replace=False)
    t0 = time.perf_counter()
    pyoracle.forward_rays(inp, calib, threads=threads)
    t_calib = time.perf_counter() - t0
    n = int(max(threads, min(p.rays, threads * max(1.0, budget_s / max(t_calib, 1e-3)))))
    rays = np.sort(rng.choice(p.rays, n, replace=False))
    t0 = time.perf_counter()
    No, Co, _, _ = pyoracle.forward_rays(inp, rays, threads=threads)
    dt = time.perf_counter() - t0
    return ref_equiv_terms(inp, n) / dt / 1e9, threads, n, dt, rays, No, Co


def err_summary(got, ref, floor=1e-6):
    """Max and mean relative error of got against the FP64 values ref; an
    entry below floor times the largest is compared against that floor."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.maximum(np.abs(ref), floor * max(float(np.abs(ref).max()), 1e-300))
    e = np.abs(got - ref) / den
    return {"max_rel": float(e.max()), "mean_rel": float(e.mean()), "n": int(e.size)}


def run_reference(args):
    """--impl reference: the CPU restatement of the reference's algorithm."""
    from xrd_tomography_gb300 import synth
    ws, rank, _ = dist_setup(args)
    if rank != 0:
        barrier(ws)
        return
    inp = synth.config_inputs(args.workload)
    from oracle import pyoracle
    pyoracle.build(ref=False)
    p = inp.problem
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(1)
    step_rays = max(threads, 2 * threads)
    for _ in range(args.warmup):
        pyoracle.forward_rays(inp, rng.choice(p.rays, step_rays, replace=False), threads=threads)
    t_total = 0.0
    for _ in range(args.steps):
        rays = rng.choice(p.rays, step_rays, replace=False)
        t0 = time.perf_counter()
        pyoracle.forward_rays(inp, rays, threads=threads)
        t_total += time.perf_counter() - t0
    v = ref_equiv_terms(inp, step_rays) * args.steps / t_total / 1e9
    sample = (f"{step_rays} randomly drawn rays of the {p.rays}-ray projection per step "
              f"(all {int((inp.seg > 0).sum())} voxels, every fine q bin, FP64)")
    line = {
        "impl": "reference", "metric": "forward projector throughput (reference-equivalent ray-voxel-q terms)",
        "value": v, "unit": "G ray-voxel-q/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": workload_config(inp, sample_rays_per_step=step_rays),
        "cpu_baseline": {"value": v, "unit": "G ray-voxel-q/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "G ray-voxel-q/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    barrier(ws)


# ---- GPU leg -------------------------------------------------------------------

def plain_wave(dev) -> int:
    """Rays for timing the FP64 kernel at the reference's launch shape: 16
    one-warp blocks per SM, enough to keep every SM's FP64 pipe busy, so
    that the sample's rate is the kernel's full-GPU rate (a few blocks would
    leave most SMs idle and understate it)."""
    import torch
    return 16 * torch.cuda.get_device_properties(dev).multi_processor_count


def hbm_peak_gbs():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["hbm_gbs"]), "measured (MEASURED_PEAKS.json)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def mlem_stored_bench(xt, synth, ctx, stream, dev, iters=200):
    """MLEM of main.m:154-176 with the explicit model matrix of the 64x64
    workload (131072 rays x 256 coefficients, 134 MB): iterations per second
    and the HBM throughput of its passes (each iteration reads A once)."""
    import torch
    inp = synth.config_inputs(0)
    p = inp.problem
    K = p.nwt * p.n_mat
    N = torch.empty(p.rays, dtype=torch.float32, device=dev)
    C = torch.empty_like(N)
    A = torch.empty(p.amatrix_elems, dtype=torch.float32, device=dev)
    xt.forward(p, *inp.args(), Nphotons=N, Cphotons=C, Amatrix=A, ctx=ctx)
    torch.cuda.synchronize(dev)
    gen = torch.Generator(device="cpu").manual_seed(7)
    y = torch.poisson((N + C).cpu(), generator=gen).to(dev)
    x = torch.full((K,), 10.0, dtype=torch.float32, device=dev)
    xt.mlem_matrix(A, y, C, x, 3, ctx=ctx)           # warm-up (and graph capture)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record(stream)
    xt.mlem_matrix(A, y, C, x, 0, ctx=ctx)           # sensitivity pass only
    ev[1].record(stream)
    ev[2].record(stream)
    xt.mlem_matrix(A, y, C, x, iters, ctx=ctx)
    ev[3].record(stream)
    torch.cuda.synchronize(dev)
    t0 = ev[0].elapsed_time(ev[1])
    t1 = ev[2].elapsed_time(ev[3])
    per_iter_ms = (t1 - t0) / iters
    a_bytes = A.numel() * 4
    traffic = a_bytes + 2 * p.rays * 4               # A, y and c per iteration
    peak, src = hbm_peak_gbs()
    gbs = traffic / (per_iter_ms * 1e-3) / 1e9
    return {"workload": f"explicit model matrix of the 64x64 workload: {p.rays} rays x {K} coefficients "
                        f"({a_bytes / 1e6:.0f} MB), {iters} iterations, CUDA-graph replay",
            "iter_per_s": 1e3 / per_iter_ms, "ms_per_iter": per_iter_ms,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "traffic": None, "algorithmic_bytes_per_iter": traffic, "peak_source": src}}


def basis_bench(xt, ctx, dev, launches=20):
    """xrdt_basis_expand (I = C B, 3xTF32 on tcgen05) on inputs larger than
    L2, for two shapes: K = N = 32 (a dense basis of 32 coefficients onto 32
    coarse bins, as the basis operator expands per voxel) and K = 64, N = 256.
    Kernel time from CUDA events on the library's stream, mean over
    `launches` launches; bytes are the algorithmic ones (C and B read, I
    written once); flops count the three TF32 products."""
    import torch
    peak, src = hbm_peak_gbs()
    out = {}
    for K, N, M in ((32, 32, 152 * 128 * 64), (64, 256, 152 * 128 * 8)):
        g = torch.Generator(device="cpu").manual_seed(K * 1000 + N)
        C = torch.rand(M, K, generator=g).to(dev)
        B = torch.rand(K, N, generator=g).to(dev)
        I = torch.empty(M, N, device=dev)
        xt.basis_expand(C, B, I, ctx=ctx)
        ctx.set_profiling(True)
        for _ in range(launches):
            xt.basis_expand(C, B, I, ctx=ctx)
        n, ms, _ = ctx.kernel_stats(xt.api.KERNEL_BASIS)
        ctx.set_profiling(False)
        torch.cuda.synchronize(dev)
        t = ms / max(1, n) * 1e-3
        byts = 4.0 * (M * K + K * N + M * N)
        gbs = byts / t / 1e9
        # spot check against FP64 on a few rows
        rows = torch.arange(0, M, max(1, M // 64), device=dev)
        ref = (C[rows].double() @ B.double())
        err = float(((I[rows].double() - ref).abs() / ref.abs().clamp_min(1e-30)).max())
        out[f"M{M}_K{K}_N{N}"] = {
            "ms_per_launch": t * 1e3, "launches": int(n), "tflops_3xtf32": 6.0 * M * N * K / t / 1e12,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "traffic": None, "algorithmic_bytes_per_launch": byts, "peak_source": src},
            "max_rel_err_vs_fp64": err}
        del C, B, I
    return out


def vox_mlem_bench(xt, synth, ctx, stream, dev, iters=50):
    """Per-voxel-coefficient MLEM (main.m:162-176 with one coarse-q pattern per
    voxel) on the 128x128 workload: counts drawn from a seeded ground truth
    (Poisson, peak 1e3 per pixel-bin, flat 5% incoherent bias), 50 iterations
    of the captured forward/adjoint/update graph.  The plain FP64 kernel at
    the reference's launch shape is timed forward and adjoint on a ray subset
    and scaled to all rays for the per-iteration comparison."""
    import torch
    inp = synth.config_inputs(2)
    p = inp.problem
    op = xt.Operator(p, inp.spectrum, inp.seg, inp.a1, inp.a2, ctx=ctx)
    xtrue = torch.from_numpy(synth.vox_truth(inp)).to(dev)
    ybar = op.forward(xtrue, torch.empty(p.rays, device=dev)).double()
    scale = 1e3 / float(ybar.max())
    c = torch.full((p.rays,), 0.05 * float(ybar.mean()) * scale, dtype=torch.float32, device=dev)
    gen = torch.Generator(device="cpu").manual_seed(17)
    y = torch.poisson((ybar * scale + c.double()).cpu(), generator=gen).float().to(dev)
    on = torch.from_numpy(np.repeat(np.asarray(inp.seg).reshape(-1) > 0, p.nwt)).to(dev)
    x = torch.where(on, 1.0, 0.0).float()
    op.mlem(y, c, x.clone(), 2)                        # sensitivity and graph capture
    torch.cuda.synchronize(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record(stream)
    op.mlem(y, c, x, iters)
    ev[1].record(stream)
    torch.cuda.synchronize(dev)
    ms_iter = ev[0].elapsed_time(ev[1]) / iters
    yv = op.forward(x, torch.empty(p.rays, device=dev)).double() + c.double()
    loglik = float((y.double() * torch.log(yv) - yv).sum())
    # separate forward and adjoint calls, device buffers
    w = torch.rand(p.rays, generator=torch.Generator(device="cpu").manual_seed(5)).to(dev)
    yb = torch.empty(p.rays, device=dev)
    gb = torch.empty(op.unknowns, device=dev)
    op.forward(x, yb)
    op.adjoint(w, gb)
    ctx.set_profiling(True)
    for _ in range(3):
        op.forward(x, yb)
        op.adjoint(w, gb)
    f = ctx.kernel_stats(xt.api.KERNEL_VOX_FORWARD)
    a = ctx.kernel_stats(xt.api.KERNEL_VOX_ADJOINT)
    ctx.set_profiling(False)
    # plain FP64 path on a ray subset, its kernels timed with CUDA events
    rng = np.random.default_rng(3)
    sub = np.sort(rng.choice(p.rays, min(p.rays, plain_wave(dev)), replace=False))
    xh = x.cpu().numpy()
    wh = w[torch.from_numpy(sub).to(dev)].cpu().numpy()
    plain_iter_ms = plain_vox_ms(xt, ctx, op, xh, wh, sub) * p.rays / sub.size
    # the operator's forward against the oracle on sampled rays
    err = vox_err_vs_oracle(inp, x.cpu().numpy(), op.forward(x, torch.empty(p.rays, device=dev)).cpu().numpy(),
                            n=64, seed=4)
    op.close()
    return {"workload": f"{p.nx}x{p.ny} phantom, {p.nwt} coarse-q coefficients per voxel "
                        f"({int((np.asarray(inp.seg) > 0).sum())} non-empty voxels), {p.rays} rays, "
                        f"{iters} MLEM iterations (forward + adjoint + update, one CUDA graph each)",
            "iter_per_s": 1e3 / ms_iter, "ms_per_iter": ms_iter,
            "forward_ms": f[1] / max(1, f[0]), "adjoint_ms": a[1] / max(1, a[0]),
            "poisson_loglik_after": loglik,
            "plain_fp64_ms_per_iter": plain_iter_ms,
            "plain_fp64_sample": f"forward and adjoint on {sub.size} of {p.rays} rays (kernel time, CUDA events), "
                                 f"scaled to all rays",
            "speedup_vs_plain_fp64": plain_iter_ms / ms_iter,
            "forward_err_vs_oracle": err}


def plain_vox_ms(xt, ctx, op, x_host, w_host, rays):
    """Device milliseconds of the FP64 kernel at the reference's launch shape
    for the forward and the adjoint of the listed rays (CUDA events around
    each launch; the host-side staging of the call is not counted)."""
    ctx.set_profiling(True)
    op.forward_rays_fp64(x_host, rays)
    op.adjoint_rays_fp64(w_host, rays)
    n, ms, _ = ctx.kernel_stats(xt.api.KERNEL_PLAIN)
    ctx.set_profiling(False)
    return ms


def vox_err_vs_oracle(inp, x_host, y_gpu, n, seed):
    """The per-voxel operator's forward against the FP64 oracle on n sampled rays."""
    from oracle import pyoracle
    pyoracle.build(ref=False)
    rays = np.sort(np.random.default_rng(seed).choice(inp.problem.rays, n, replace=False))
    y_ref, _ = pyoracle.vox_rays(inp, rays, x=x_host)
    return err_summary(np.asarray(y_gpu)[rays], y_ref)


def batch_mlem_bench(xt, synth, ctx, stream, dev, n=8, iters=10, side=(64, 160), views=(24, 64), px=(64, 160)):
    """Batched MLEM over phantoms of uneven size (the batched configuration's
    generator with its ranges scaled down so that the section takes seconds:
    by default sides 64-160 voxels, 24-64 views, 64-160 px, 64 energy bins,
    128 fine q bins, 32 coefficients per voxel): one persistent launch per
    kernel and one CUDA graph per iteration for the whole batch, against the
    same operators run one after another and the plain FP64 kernel."""
    import torch
    inps = synth.batch_inputs(n, side=side, views=views, px=px)
    ops = [xt.Operator(i.problem, i.spectrum, i.seg, i.a1, i.a2, ctx=ctx) for i in inps]
    ys, cs, x0 = [], [], []
    for k, (inp, op) in enumerate(zip(inps, ops)):
        xtrue = torch.from_numpy(synth.vox_truth(inp)).to(dev)
        ybar = op.forward(xtrue, torch.empty(inp.problem.rays, device=dev)).double()
        scale = 1e3 / max(float(ybar.max()), 1e-30)
        c = torch.full((inp.problem.rays,), 0.05 * float(ybar.mean()) * scale, dtype=torch.float32, device=dev)
        gen = torch.Generator(device="cpu").manual_seed(100 + k)
        ys.append(torch.poisson((ybar * scale + c.double()).cpu(), generator=gen).float().to(dev))
        cs.append(c)
        on = torch.from_numpy(np.repeat(np.asarray(inp.seg).reshape(-1) > 0, inp.problem.nwt)).to(dev)
        x0.append(torch.where(on, 1.0, 0.0).float())
    batch = xt.Batch(ops, ctx=ctx)
    warps, tiles, fgrid, agrid = batch.tune()
    xb = [x.clone() for x in x0]
    batch.mlem(ys, cs, xb, 1)                          # sensitivity and graph capture
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize(dev)
    ev[0].record(stream)
    batch.mlem(ys, cs, xb, iters)
    ev[1].record(stream)
    torch.cuda.synchronize(dev)
    ms_batch = ev[0].elapsed_time(ev[1]) / iters
    # the same operators one after another
    ms_seq = 0.0
    for k, op in enumerate(ops):
        x = x0[k].clone()
        op.mlem(ys[k], cs[k], x, 1)
        torch.cuda.synchronize(dev)
        ev[0].record(stream)
        op.mlem(ys[k], cs[k], x, iters)
        ev[1].record(stream)
        torch.cuda.synchronize(dev)
        ms_seq += ev[0].elapsed_time(ev[1]) / iters
    # plain FP64 forward + adjoint on a few rays of every problem (kernel time)
    plain_ms = 0.0
    rng = np.random.default_rng(9)
    for k, (inp, op) in enumerate(zip(inps, ops)):
        sub = np.sort(rng.choice(inp.problem.rays, min(inp.problem.rays, plain_wave(dev)), replace=False))
        plain_ms += plain_vox_ms(xt, ctx, op, x0[k].cpu().numpy(), np.ones(sub.size, np.float32), sub) * \
            inp.problem.rays / sub.size
    pv = sum(int((i.seg > 0).sum()) * i.problem.n_src * i.problem.n_col * i.problem.n_row for i in inps)
    sizes = [f"{i.problem.nx}^2/{i.problem.n_src}v/{i.problem.n_col}px" for i in inps]
    batch.close()
    for op in ops:
        op.close()
    return {"workload": f"{n} phantoms ({', '.join(sizes)}), 64 energy bins, 32 coefficients per voxel, "
                        f"{iters} MLEM iterations, one graph per iteration",
            "ms_per_iter": ms_batch, "iter_per_s": 1e3 / ms_batch,
            "pair_voxels_per_iter": pv, "g_pair_voxels_per_s": pv / (ms_batch * 1e-3) / 1e9,
            "sequential_ms_per_iter": ms_seq, "batching_speedup": ms_seq / ms_batch,
            "plain_fp64_ms_per_iter": plain_ms, "speedup_vs_plain_fp64": plain_ms / ms_batch,
            "plain_fp64_sample": f"forward and adjoint on {plain_wave(dev)} rays of every problem (16 blocks per SM, "
                                 f"kernel time from CUDA events), scaled to all rays",
            "autotuned": {"adjoint_warps": warps, "adjoint_tiles": tiles, "forward_grid": fgrid,
                          "adjoint_grid": agrid}}


def run_batched_stated(args):
    """--workload 3: batched per-voxel MLEM on the batched configuration at its
    stated sizes (--workload 4 --mlem: on slices of the 384x384 stack instead)
    -- args.batch phantoms (64) with sides uniform in 64-384
    voxels, 60-360 views, 128-768 px, 64 energy bins, 32 coefficients per
    voxel -- as one xrdt_batch: every operator streams its detector-side
    table in tiles inside each iteration, one CUDA graph per iteration.  One
    warm-up call (the sensitivity, the graph capture and one iteration), then
    args.iters timed iterations.  The counts are seeded Poisson draws around
    a flat level (the iteration's work does not depend on their values)."""
    import torch
    import xrd_tomography_gb300 as xt
    from xrd_tomography_gb300 import synth
    from xrd_tomography_gb300 import build as lib_build

    ws, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib_build.build()
    os.environ.setdefault("XRDT_WALK_CACHE", "0")
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx = xt.Context(local, stream=stream.cuda_stream)
    t_setup = time.perf_counter()
    if args.workload == 4:
        # slices of the scanner stack: 384x384 at 1.5 mm, 12 materials, 720
        # views, 1024 px x 96 energy bins, each slice its own seeded phantom
        n = args.batch or 16
        inps = [synth.make_inputs(synth.config_problem(4), synth.SEED_BASE + 4 + 1000 * k) for k in range(n)]
        what = (f"{n} slice(s) of the 384x384 stack (1.5 mm, 12 materials, 720 views, 1024 px x 96 energy "
                f"bins), {inps[0].problem.nwt} coefficients per voxel")
    else:
        n = args.batch or 64
        inps = synth.batch_inputs(n)
        what = (f"{n} phantoms of the batched configuration at its stated sizes (sides 64-384, 60-360 views, "
                f"128-768 px), 64 energy bins, {inps[0].problem.nwt} coefficients per voxel")
    ops = [xt.Operator(i.problem, i.spectrum, i.seg, i.a1, i.a2, ctx=ctx) for i in inps]
    gen = torch.Generator(device=dev).manual_seed(23)
    ys, cs, xs = [], [], []
    for inp, op in zip(inps, ops):
        r = inp.problem.rays
        ys.append(torch.poisson(torch.full((r,), 100.0, device=dev), generator=gen))
        cs.append(torch.full((r,), 5.0, device=dev))
        on = torch.from_numpy(np.repeat(np.asarray(inp.seg).reshape(-1) > 0, inp.problem.nwt)).to(dev)
        xs.append(torch.where(on, 1.0, 0.0).float())
    batch = xt.Batch(ops, ctx=ctx)
    warps, tiles, fgrid, agrid = batch.tune()
    batch.mlem(ys, cs, xs, 1)
    torch.cuda.synchronize(dev)
    t_setup = time.perf_counter() - t_setup
    launches0 = ctx.launches
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    barrier(ws)
    with ClockSampler(local) as clk:
        ev[0].record(stream)
        batch.mlem(ys, cs, xs, args.iters)
        ev[1].record(stream)
        torch.cuda.synchronize(dev)
    ms_iter = all_max(ws, ev[0].elapsed_time(ev[1]) / args.iters, dev)
    gpu_launches = ctx.launches - launches0
    pv = [int((np.asarray(i.seg) > 0).sum()) * i.problem.n_src * i.problem.n_col * i.problem.n_row for i in inps]
    # plain FP64 path on four problems (smallest, largest, two others), scaled
    # by pair-voxels to the batch
    order = np.argsort(pv)
    picks = sorted({int(order[0]), int(order[-1]), int(order[len(order) // 3]), int(order[2 * len(order) // 3])})
    rng = np.random.default_rng(9)
    plain_ms, plain_pv = 0.0, 0
    for k in picks:
        inp, op = inps[k], ops[k]
        sub = np.sort(rng.choice(inp.problem.rays, min(inp.problem.rays, plain_wave(dev)), replace=False))
        plain_ms += plain_vox_ms(xt, ctx, op, xs[k].cpu().numpy(), np.ones(sub.size, np.float32), sub) * \
            inp.problem.rays / sub.size
        plain_pv += pv[k]
    plain_iter_ms = plain_ms * sum(pv) / plain_pv
    # the operators' forward against the oracle on sampled rays of three problems
    errs = {}
    for k in (int(order[0]), int(order[len(order) // 2]), int(order[-1])):
        inp, op = inps[k], ops[k]
        y = op.forward(xs[k], torch.empty(inp.problem.rays, device=dev))
        errs[f"{inp.problem.nx}^2/{inp.problem.n_src}v/{inp.problem.n_col}px"] = \
            vox_err_vs_oracle(inp, xs[k].cpu().numpy(), y.cpu().numpy(), n=8, seed=k)
    clocks = clk.summary()
    if rank == 0:
        line = {
            "metric": "batched per-voxel MLEM iterations per second (forward + adjoint + update)",
            "value": 1e3 / ms_iter, "unit": "iter/s", "n_gpus": ws, "steps": args.iters, "warmup": 1,
            "ms_per_step": ms_iter, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (FP64 geometry decisions and global sums)", "data": "synthetic (seeded)",
            "config": {"workload": f"{what}, one xrdt_batch, detector-side tables streamed in tiles",
                       "pair_voxels_per_iter": int(sum(pv)), "rays": int(sum(i.problem.rays for i in inps)),
                       "sizes": [f"{i.problem.nx}^2/{i.problem.n_src}v/{i.problem.n_col}px" for i in inps]},
            "g_pair_voxels_per_s": sum(pv) / (ms_iter * 1e-3) / 1e9,
            "plain_fp64_ms_per_iter": plain_iter_ms,
            "speedup_vs_plain_fp64": plain_iter_ms / ms_iter,
            "plain_fp64_sample": f"forward and adjoint of {plain_wave(dev)} rays of problems {picks} "
                                 f"(kernel time, CUDA events), scaled by pair-voxels to the batch",
            "forward_err_vs_oracle": errs,
            "autotuned": {"adjoint_warps": warps, "adjoint_tiles": tiles, "forward_grid": fgrid,
                          "adjoint_grid": agrid},
            "setup_s": t_setup, "gpu_launches": gpu_launches, "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    barrier(ws)
    batch.close()
    ctx.close()


def run_ours(args):
    import torch
    import xrd_tomography_gb300 as xt
    from xrd_tomography_gb300 import synth
    from xrd_tomography_gb300 import build as lib_build

    ws, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib_build.build()
    lib_build.build_probe()
    inp = synth.config_inputs(args.workload)
    p = inp.problem
    stream = torch.cuda.Stream(dev)          # the library launches on this stream
    torch.cuda.set_stream(stream)
    ctx = xt.Context(local, stream=stream.cuda_stream)

    host = [np.ascontiguousarray(x) for x in (inp.spectrum, inp.Ifine, inp.seg, inp.a1, inp.a2, inp.S2)]
    d_in = [torch.from_numpy(x).to(dev) for x in host]
    Nd = torch.empty(p.rays, dtype=torch.float32, device=dev)
    Cd = torch.empty_like(Nd)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    tables = (inp.q_min, inp.q_max, inp.a_min, inp.a_max)

    def step_dev():
        xt.forward(p, *d_in, *tables, Nphotons=Nd, Cphotons=Cd, want_amatrix=False, ctx=ctx,
                   flags=xt.FWD_NO_SYNC)

    for _ in range(args.warmup):
        step_dev()
    torch.cuda.synchronize(dev)

    # device-resident timed region (profiling on: per-kernel events)
    ctx.set_profiling(True)
    launches0 = ctx.launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(ws)
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            step_dev()
            ev[i][1].record(stream)
        torch.cuda.synchronize(dev)
    barrier(ws)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    gpu_launches = ctx.launches - launches0
    total_s = all_max(ws, sum(step_ms) / 1e3, dev)
    units = ref_equiv_terms(inp) * args.steps * ws
    value = units / total_s / 1e9
    fwd_n, fwd_ms, fwd_work = ctx.kernel_stats(xt.api.KERNEL_FORWARD)
    kstats = {name: ctx.kernel_stats(k)[:2] for name, k in
              (("prep_map", xt.api.KERNEL_PREP_MAP), ("prep_voxels", xt.api.KERNEL_PREP_VOXELS),
               ("src_atten", xt.api.KERNEL_SRC_ATTEN), ("walk", xt.api.KERNEL_WALK),
               ("forward", xt.api.KERNEL_FORWARD))}
    ctx.set_profiling(False)
    clocks = clk.summary()

    # end-to-end through the C ABI with host buffers
    pin = [torch.from_numpy(x).pin_memory() for x in host]
    Nh = torch.empty(p.rays, dtype=torch.float32).pin_memory()
    Ch = torch.empty_like(Nh).pin_memory()
    h2d = sum(int(x.numel() * x.element_size()) for x in pin)
    d2h = int(Nh.numel() * 4 + Ch.numel() * 4)

    def step_e2e():
        xt.forward(p, *pin, *tables, Nphotons=Nh, Cphotons=Ch, want_amatrix=False, ctx=ctx)

    step_e2e()
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(ws)
    for i in range(args.steps):
        flush.fill_(float(i))
        ev2[i][0].record(stream)
        step_e2e()
        ev2[i][1].record(stream)
    torch.cuda.synchronize(dev)
    e2e_s = all_max(ws, sum(a.elapsed_time(b) for a, b in ev2) / 1e3, dev)
    e2e_value = units / e2e_s / 1e9

    line = {
        "metric": "forward projector throughput (reference-equivalent ray-voxel-q terms)",
        "value": value, "unit": "G ray-voxel-q/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64 geometry and integer decisions)",
        "data": "synthetic (seeded phantom, patterns, spectrum)",
        "config": workload_config(inp, parallelism=f"replicas x{ws}" if ws > 1 else "single GPU",
                                  l2="flushed between steps (256 MB write)"),
        "e2e": {"value": e2e_value, "unit": "G ray-voxel-q/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": gpu_launches,
        "clocks": clocks,
        "kernel_ms_per_step": {k: v[1] / max(1, args.steps) for k, v in kstats.items()},
    }

    if rank == 0 and not args.no_baselines:
        line["mlem"] = mlem_stored_bench(xt, synth, ctx, stream, dev)
        line["vox_mlem"] = vox_mlem_bench(xt, synth, ctx, stream, dev)
        line["batch_mlem"] = batch_mlem_bench(xt, synth, ctx, stream, dev)
        # many small problems, each of which alone leaves most of the GPU idle
        line["batch_mlem_small"] = batch_mlem_bench(xt, synth, ctx, stream, dev, n=48, side=(24, 48),
                                                    views=(8, 16), px=(16, 32))
        line["basis"] = basis_bench(xt, ctx, dev)
    if rank == 0:
        # roofline of the dominant kernel: the forward kernel's exponentials
        # (Gaussian q terms, attenuation and Compton factors) on the SFU
        probe = __import__("ctypes").CDLL(lib_build.PROBE_LIB)
        probe.xrdt_probe_peak.restype = __import__("ctypes").c_double
        ex2_peak = probe.xrdt_probe_peak(1)
        fma_peak = probe.xrdt_probe_peak(0)
        fp64_peak = probe.xrdt_probe_peak(2)
        pair_voxels = float(p.n_src) * p.n_col * p.n_row * int((inp.seg > 0).sum())
        per_launch_ms = fwd_ms / max(1, fwd_n)
        work = fwd_work / max(1, fwd_n)
        achieved = work / (per_launch_ms * 1e-3) / 1e9
        line["roofline"] = {
            "bound": "sfu", "achieved": achieved, "peak": ex2_peak / 1e9, "unit": "G exp2/s",
            "frac": achieved / (ex2_peak / 1e9) if ex2_peak > 0 else None,
            "traffic": (K_FWD_DRAM_BYTES_PER_PAIR_VOXEL * pair_voxels / max(1, fwd_n / args.steps)
                        if K_FWD_DRAM_BYTES_PER_PAIR_VOXEL else None),
            "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one k_fwd launch on the 128x128 "
                              "workload (ncu), per (pair, voxel), scaled to this workload's mean launch",
            "issue_slots_busy": K_FWD_ISSUE_BUSY,
            "issue_source": "ncu Issue Slots Busy of k_fwd on the 128x128 workload",
            "kernel": "k_fwd (factored forward projector)",
            "work": "exp2 evaluations the kernel performs (q bins inside its 7.5-sigma windows, one attenuation "
                    "and one Compton factor per (voxel, source energy)), counted by the kernel itself: the "
                    "implemented algorithm's count, not the dense reference-equivalent one of the metric",
            "work_per_launch": work, "launch_ms": per_launch_ms,
            "peak_source": "measured on this GPU by xrdt_probe_peak (ex2.approx, all SMs)",
        }
        line["measured_peaks"] = {"fp32_tflops": fma_peak / 1e12, "sfu_ex2_gops": ex2_peak / 1e9,
                                  "fp64_tflops": fp64_peak / 1e12}
        if not args.no_baselines:
            # plain FP64 kernel at the reference launch shape, on a ray subset
            rng = np.random.default_rng(2)
            sub = rng.choice(p.rays, min(p.rays, plain_wave(dev)), replace=False)
            t0 = time.perf_counter()
            xt.forward_rays(p, sub, *host, *tables, plain=True, ctx=ctx)
            dt = time.perf_counter() - t0
            plain_v = ref_equiv_terms(inp, sub.size) / dt / 1e9
            line["plain_fp64_gpu"] = {"value": plain_v, "unit": "G ray-voxel-q/s", "sample_rays": int(sub.size),
                                      "speedup_of_value": value / plain_v}
            cv, cores, n, dt, srays, No, Co = cpu_sample_rate(inp, args.cpu_seconds)
            line["cpu_baseline"] = {"value": cv, "unit": "G ray-voxel-q/s", "cores": cores, "kind": "port",
                                    "sample": f"{n} randomly drawn rays of the {p.rays}-ray projection "
                                              f"({dt:.1f} s, FP64 oracle, OpenMP over rays)"}
            # the timed projection's outputs against the oracle on the same rays
            idx = torch.from_numpy(srays).to(dev)
            line["err_vs_oracle"] = {
                "N": err_summary(Nd[idx].cpu().numpy(), No), "C": err_summary(Cd[idx].cpu().numpy(), Co),
                "rays": f"the {n} rays of the CPU sample; relative error, entries below 1e-6 of the "
                        f"sample's largest compared against that floor"}
        print(json.dumps(line), flush=True)
    barrier(ws)
    ctx.close()


def run_basis_only(args):
    import torch
    import xrd_tomography_gb300 as xt
    from xrd_tomography_gb300 import build as lib_build
    lib_build.build()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx = xt.Context(0, stream=stream.cuda_stream)
    print(json.dumps({"metric": "basis expansion (3xTF32 on tcgen05)", "basis": basis_bench(xt, ctx, dev)}),
          flush=True)
    ctx.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.basis:
        run_basis_only(args)
    elif args.workload == 3 or (args.workload == 4 and args.mlem):
        run_batched_stated(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
