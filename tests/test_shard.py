"""View-sharded projection and MLEM (xrd_tomography_gb300/shard.py).

On CPU: a shard's problem places its sources where the full scanner does
(the FP64 oracle gives the same rays either way), the shards' rays cover the
full problem once, and MLEM over two gloo ranks -- each holding the rays of
its views of the oracle's dense per-voxel matrix, one all-reduce of the
back-projection per iteration -- equals MLEM of the whole matrix on one rank.
On the GPU: the sharded loop with the library's operator on one rank against
the operator's own fused MLEM."""
import os
import socket
import sys

import numpy as np
import pytest

from xrd_tomography_gb300 import synth
from xrd_tomography_gb300.shard import ShardedMLEM, shard_rays, view_range, view_shard_problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_view_ranges_cover_all_views():
    for n, w in ((32, 2), (33, 4), (5, 5), (180, 8)):
        r = [view_range(n, k, w) for k in range(w)]
        assert r[0][0] == 0 and r[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
        assert max(b - a for a, b in r) - min(b - a for a, b in r) <= 1


def test_shard_rays_partition_the_rays():
    p = synth.tiny_problem()
    idx = np.concatenate([shard_rays(p, *view_range(p.n_src, k, 3)) for k in range(3)])
    assert np.array_equal(np.sort(idx), np.arange(p.rays))


def test_shard_problem_places_sources_as_the_full_scanner(oracle_lib):
    inp = synth.make_inputs(synth.tiny_problem(), 5)
    p = inp.problem
    s0, s1 = 1, 3
    q = view_shard_problem(p, s0, s1)
    sub = synth.Inputs(q, inp.spectrum, inp.Ifine, inp.seg, inp.a1, inp.a2, inp.S2,
                       inp.q_min, inp.q_max, inp.a_min, inp.a_max)
    Ns, Cs, _, _ = oracle_lib.forward_rays(sub, np.arange(q.rays))
    Nf, Cf, _, _ = oracle_lib.forward_rays(inp, shard_rays(p, s0, s1))
    assert np.abs(Ns - Nf).max() <= 1e-12 * np.abs(Nf).max()
    assert np.abs(Cs - Cf).max() <= 1e-12 * np.abs(Cf).max()


def mlem_fp64(A, y, c, x0, iters):
    x = x0.copy()
    s = A.sum(0)
    for _ in range(iters):
        with np.errstate(divide="ignore", invalid="ignore"):
            x = x * (A.T @ (y / (A @ x + c + 1e-20))) / (s + 1e-7)
        x[~np.isfinite(x)] = 0.0
        x[x < 0] = 0.0
    return x


def dense_problem():
    from oracle import pyoracle
    pyoracle.build(ref=False)
    inp = synth.make_inputs(synth.tiny_problem(), 9)
    p = inp.problem
    _, _, _, Av = pyoracle.forward_rays(inp, np.arange(p.rays), want_av=True)
    A = Av.reshape(p.rays, -1)
    xt_true = synth.vox_truth(inp).astype(np.float64)
    ybar = A @ xt_true
    y = np.random.default_rng(1).poisson(ybar / ybar.max() * 1e3).astype(np.float64) * (ybar.max() / 1e3)
    c = np.full(p.rays, 0.05 * ybar.mean())
    x0 = np.where(np.repeat(np.asarray(inp.seg).reshape(-1) > 0, p.nwt), 1.0, 0.0)
    return p, A, y, c, x0


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p, A, y, c, x0 = dense_problem()
    rows = shard_rays(p, *view_range(p.n_src, rank, world))
    Ar = torch.from_numpy(A[rows])
    if len(rows):
        mlem = ShardedMLEM(lambda x: Ar @ x, lambda w: Ar.T @ w, lambda t: dist.all_reduce(t))
    else:   # more ranks than views: this rank holds none
        mlem = ShardedMLEM(None, None, lambda t: dist.all_reduce(t))
    x = torch.from_numpy(x0.copy())
    mlem.run(torch.from_numpy(y[rows]), torch.from_numpy(c[rows]), x, 20)
    np.save(os.path.join(out_dir, f"x{rank}.npy"), x.numpy())
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 5])
def test_sharded_mlem_equals_one_rank(tmp_path, world):
    """Two ranks of two views each; and five ranks over the tiny problem's
    four views, the fifth without views (it adds zeros to the all-reduces)."""
    mp = pytest.importorskip("torch.multiprocessing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.spawn(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    xs = [np.load(tmp_path / f"x{r}.npy") for r in range(world)]
    for xr in xs[1:]:
        assert np.array_equal(xs[0], xr)     # every rank holds the same estimate
    p, A, y, c, x0 = dense_problem()
    ref = mlem_fp64(A, y, c, x0, 20)
    assert np.abs(xs[0] - ref).max() <= 1e-10 * np.abs(ref).max()


def test_rank_without_views():
    p = synth.tiny_problem()
    assert view_range(p.n_src, p.n_src, p.n_src + 1) == (p.n_src, p.n_src)
    assert shard_rays(p, p.n_src, p.n_src).size == 0
    with pytest.raises(ValueError):
        view_shard_problem(p, 2, 2)
    torch = pytest.importorskip("torch")
    with pytest.raises(ValueError):
        ShardedMLEM(None, None, lambda t: None).run(torch.ones(3), torch.ones(3), torch.ones(4), 1)


@pytest.mark.gpu
def test_sharded_loop_with_the_operator_on_one_rank():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xrd_tomography_gb300 as xt
    from xrd_tomography_gb300.shard import operator_shard
    from tests.tolerances import MLEM_FLOOR, max_rel_err
    inp = synth.config_inputs(2)
    p = inp.problem
    ctx = xt.Context(0)
    try:
        op, rows = operator_shard(p, inp.spectrum, inp.seg, inp.a1, inp.a2, 0, 1, ctx=ctx)
        assert np.array_equal(rows, np.arange(p.rays))
        xtrue = torch.from_numpy(synth.vox_truth(inp)).cuda()
        ybar = op.forward(xtrue, torch.empty(p.rays, device="cuda"))
        y = (ybar * (1e3 / float(ybar.max()))).round() + 1.0
        c = torch.full_like(y, 2.0)
        x0 = torch.where(xtrue > 0, 1.0, 0.0).float()
        loop = ShardedMLEM(lambda x: op.forward(x, torch.empty(p.rays, device="cuda")),
                           lambda w: op.adjoint(w, torch.empty(op.unknowns, device="cuda")), lambda t: None)
        xs = loop.run(y, c, x0.clone(), 5)
        xf = x0.clone()
        op.mlem(y, c, xf, 5)
        torch.cuda.synchronize()
        assert max_rel_err(xs.cpu().numpy(), xf.cpu().numpy(), floor=MLEM_FLOOR) < 1e-5
        op.close()
    finally:
        ctx.close()
