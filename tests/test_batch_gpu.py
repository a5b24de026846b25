"""Batches of per-voxel operators (xrdt_batch_*): problems of uneven size in
one persistent launch per kernel must give what each operator gives alone,
and the oracle's per-voxel model on the smallest problem."""
import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth
from tests.tolerances import FAST_RTOL, MLEM_FLOOR, MLEM_RTOL, max_rel_err

pytestmark = pytest.mark.gpu



@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def ctx(torch_cuda, tmp_path_factory):
    import os
    os.environ["XRDT_TUNE_CACHE"] = str(tmp_path_factory.mktemp("tune") / "tune.txt")
    c = xt.Context(0)
    yield c
    c.close()


def problems():
    inps = [synth.make_inputs(synth.tiny_problem(), 21)]
    inps += synth.batch_inputs(3, seed=5, side=(20, 44), views=(6, 14), px=(16, 40))
    return inps


def rand_x(inp, seed):
    p = inp.problem
    x = np.random.default_rng(seed).uniform(0.0, 1.0, (p.nx * p.ny, p.nwt)).astype(np.float32)
    x[np.asarray(inp.seg).reshape(-1) == 0] = 0.0
    return x.reshape(-1)


def test_batch_matches_single_operators_and_oracle(ctx, torch_cuda, oracle_lib):
    torch = torch_cuda
    inps = problems()
    ops = [xt.Operator(i.problem, i.spectrum, i.seg, i.a1, i.a2, ctx=ctx) for i in inps]
    batch = xt.Batch(ops, ctx=ctx)
    xs = [torch.from_numpy(rand_x(inp, 3 + k)).cuda() for k, inp in enumerate(inps)]
    ws = [torch.rand(inp.problem.rays, generator=torch.Generator().manual_seed(k)).cuda() for k, inp in enumerate(inps)]
    ys = [torch.empty(inp.problem.rays, device="cuda") for inp in inps]
    gs = [torch.empty(op.unknowns, device="cuda") for op in ops]
    batch.forward(xs, ys)
    batch.adjoint(ws, gs)
    torch.cuda.synchronize()
    for k, (inp, op) in enumerate(zip(inps, ops)):
        y1 = op.forward(xs[k], torch.empty(inp.problem.rays, device="cuda"))
        g1 = op.adjoint(ws[k], torch.empty(op.unknowns, device="cuda"))
        torch.cuda.synchronize()
        # the forward does the same arithmetic per pair in either launch
        assert torch.equal(ys[k], y1), k
        # the adjoint's pair groups differ: the partial sums add in another order
        assert max_rel_err(gs[k].cpu().numpy(), g1.cpu().numpy()) < FAST_RTOL, k
    # every problem of the batch against the oracle: the batch forward on
    # sampled rays (all of the tiny problem's), and the batch adjoint of
    # weights that are zero off those rays
    sel = [np.arange(inps[0].problem.rays)]
    sel += [np.sort(np.random.default_rng(40 + k).choice(inp.problem.rays, 48, replace=False))
            for k, inp in enumerate(inps[1:], 1)]
    wsp = []
    for k, inp in enumerate(inps):
        idx = torch.from_numpy(sel[k]).cuda()
        w = torch.zeros(inp.problem.rays, device="cuda")
        w[idx] = ws[k][idx]
        wsp.append(w)
    gsp = [torch.empty(op.unknowns, device="cuda") for op in ops]
    batch.adjoint(wsp, gsp)
    torch.cuda.synchronize()
    for k, inp in enumerate(inps):
        y_ref, g_ref = oracle_lib.vox_rays(inp, sel[k], x=xs[k].cpu().numpy(), w=wsp[k].cpu().numpy()[sel[k]])
        assert max_rel_err(ys[k].cpu().numpy()[sel[k]], y_ref) < FAST_RTOL, k
        assert max_rel_err(gsp[k].cpu().numpy(), g_ref.reshape(-1)) < FAST_RTOL, k
    warps, tiles, fgrid, agrid = batch.tune()
    assert warps in (1, 2, 4) and tiles >= 1 and fgrid >= 1 and agrid >= 1
    # a second batch of the same shapes reads the choice from the cache file
    again = xt.Batch(ops, ctx=ctx)
    assert again.tune()[:2] == (warps, tiles)
    again.close()
    batch.close()
    for op in ops:
        op.close()


def test_batch_mlem_matches_single_operators(ctx, torch_cuda):
    torch = torch_cuda
    inps = problems()
    ops = [xt.Operator(i.problem, i.spectrum, i.seg, i.a1, i.a2, ctx=ctx) for i in inps]
    ys, cs, x0 = [], [], []
    for k, (inp, op) in enumerate(zip(inps, ops)):
        xt_true = torch.from_numpy(synth.vox_truth(inp)).cuda()
        ybar = op.forward(xt_true, torch.empty(inp.problem.rays, device="cuda")).double()
        scale = 1e3 / max(float(ybar.max()), 1e-30)
        c = torch.full_like(ybar, 0.05 * float(ybar.mean()) * scale).float()
        y = torch.poisson(ybar * scale + c.double(), generator=torch.Generator(device="cuda").manual_seed(k)).float()
        on = torch.from_numpy(np.repeat(np.asarray(inp.seg).reshape(-1) > 0, inp.problem.nwt)).cuda()
        ys.append(y)
        cs.append(c)
        x0.append(torch.where(on, 1.0, 0.0).float())
    singles = []
    for k, op in enumerate(ops):
        x = x0[k].clone()
        op.mlem(ys[k], cs[k], x, 4)
        singles.append(x)
    batch = xt.Batch(ops, ctx=ctx)
    xb = [x.clone() for x in x0]
    batch.mlem(ys, cs, xb, 2)
    batch.mlem(ys, cs, xb, 2)      # continues from the current estimates
    torch.cuda.synchronize()
    for k in range(len(ops)):
        assert max_rel_err(xb[k].cpu().numpy(), singles[k].cpu().numpy(), floor=MLEM_FLOOR) < MLEM_RTOL, k
    with pytest.raises(ValueError):
        batch.forward([x.cpu() for x in x0], ys)
    batch.close()
    for op in ops:
        op.close()


def test_mixed_batch_streams_the_operators_without_tables(ctx, torch_cuda, monkeypatch):
    """A batch whose operators partly keep their detector-side tables and
    partly walk them in tiles (a walk buffer of a few pixel columns, so the
    streamed problems span several tiles, some shared): forward, adjoint and
    MLEM against the same operators run alone with their tables kept."""
    torch = torch_cuda
    inps = problems()
    kept = [xt.Operator(i.problem, i.spectrum, i.seg, i.a1, i.a2, ctx=ctx) for i in inps]
    monkeypatch.setenv("XRDT_WALK_CACHE", "0")
    nv_max = max(op.voxels for op in kept)
    src_max = max(i.problem.n_src for i in inps)
    monkeypatch.setenv("XRDT_WALK_TILE_BYTES", str(8 * nv_max * src_max * 5))
    streamed = [xt.Operator(i.problem, i.spectrum, i.seg, i.a1, i.a2, ctx=ctx) for i in inps[1:3]]
    monkeypatch.delenv("XRDT_WALK_CACHE")
    mixed = [kept[0], streamed[0], streamed[1], kept[3]]
    batch = xt.Batch(mixed, ctx=ctx)
    xs = [torch.from_numpy(rand_x(inp, 40 + k)).cuda() for k, inp in enumerate(inps)]
    ws = [torch.rand(inp.problem.rays, generator=torch.Generator().manual_seed(50 + k)).cuda()
          for k, inp in enumerate(inps)]
    ys = [torch.empty(inp.problem.rays, device="cuda") for inp in inps]
    gs = [torch.empty(op.unknowns, device="cuda") for op in mixed]
    batch.forward(xs, ys)
    batch.adjoint(ws, gs)
    torch.cuda.synchronize()
    for k, (inp, op) in enumerate(zip(inps, kept)):
        y1 = op.forward(xs[k], torch.empty(inp.problem.rays, device="cuda"))
        g1 = op.adjoint(ws[k], torch.empty(op.unknowns, device="cuda"))
        torch.cuda.synchronize()
        assert torch.equal(ys[k], y1), k
        assert max_rel_err(gs[k].cpu().numpy(), g1.cpu().numpy()) < 1e-6, k
    yms = [(y.double() * (1e3 / float(y.max()))).float() + 1.0 for y in ys]
    cs = [torch.full_like(y, 0.5) for y in yms]
    x0s = [torch.where(x > 0, 1.0, 0.0).float() for x in xs]
    xb = [x.clone() for x in x0s]
    batch.mlem(yms, cs, xb, 4)
    for k, op in enumerate(kept):
        x1 = x0s[k].clone()
        op.mlem(yms[k], cs[k], x1, 4)
        torch.cuda.synchronize()
        assert max_rel_err(xb[k].cpu().numpy(), x1.cpu().numpy(), floor=MLEM_FLOOR) < 1e-6, k
    batch.close()
