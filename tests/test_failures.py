"""Failure detection, in the forms that fault no GPU: errors made on the host
(a forced allocation failure, damaged checkpoint files), a device wait made
to run out on a barrier that nothing signals, and checkpoint/resume of MLEM.
The reference detects nothing (no CUDA error checks, Forward_XRD.cu:210-259)
and keeps its MLEM state in MATLAB memory (main.m:154-176)."""
import os

import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth


# ---- checkpoints (host memory: no GPU needed) -------------------------------

def test_checkpoint_round_trip_and_damage(tmp_path):
    x = np.random.default_rng(1).uniform(0, 1, 1000).astype(np.float32)
    path = str(tmp_path / "mlem.ckpt")
    xt.mlem_checkpoint_write(path, x, 37)
    y, it = xt.mlem_checkpoint_read(path, np.empty(1000, np.float32))
    assert it == 37
    np.testing.assert_array_equal(x, y)
    assert not os.path.exists(path + ".tmp")
    # wrong size, a flipped bit, a truncated file, trailing bytes, no file
    with pytest.raises(xt.XrdtError) as e:
        xt.mlem_checkpoint_read(path, np.empty(999, np.float32))
    assert e.value.status == 4
    raw = bytearray(open(path, "rb").read())
    for bad in (raw[:100] + bytes([raw[100] ^ 1]) + raw[101:], raw[:-3], raw + b"\0"):
        open(path, "wb").write(bytes(bad))
        with pytest.raises(xt.XrdtError) as e:
            xt.mlem_checkpoint_read(path, np.empty(1000, np.float32))
        assert e.value.status == 4
    with pytest.raises(xt.XrdtError) as e:
        xt.mlem_checkpoint_read(str(tmp_path / "missing"), np.empty(1000, np.float32))
    assert e.value.status == 9
    with pytest.raises(xt.XrdtError) as e:
        xt.mlem_checkpoint_write(str(tmp_path / "no" / "dir" / "f"), x, 1)
    assert e.value.status == 9


# ---- on the GPU ---------------------------------------------------------------

@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.gpu
def test_basis_wait_times_out_and_context_survives(torch_cuda, monkeypatch):
    """The tensor-core accumulator wait is bounded: made to wait on a barrier
    nothing arrives at, every block gives up, flags the error, lets its own
    MMAs finish and frees its tensor memory; the call returns
    XRDT_ERR_TIMEOUT and the same context computes correctly afterwards."""
    ctx = xt.Context(0)
    try:
        rng = np.random.default_rng(2)
        C = rng.standard_normal((300, 32)).astype(np.float32)
        B = rng.standard_normal((32, 128)).astype(np.float32)
        monkeypatch.setenv("XRDT_TEST_BASIS_TIMEOUT", "1")
        with pytest.raises(xt.XrdtError) as e:
            xt.basis_expand(C, B, ctx=ctx)
        assert e.value.status == 8
        monkeypatch.delenv("XRDT_TEST_BASIS_TIMEOUT")
        I = xt.basis_expand(C, B, ctx=ctx)
        ref = C.astype(np.float64) @ B.astype(np.float64)
        assert np.abs(I - ref).max() <= 1e-5 * np.abs(ref).max()
    finally:
        ctx.close()


@pytest.mark.gpu
def test_forced_allocation_failure_reports_and_recovers(torch_cuda, monkeypatch):
    """While allocations fail (XRDT_TEST_FAIL_ALLOC=1), a forward call on a
    fresh context and an operator's creation return XRDT_ERR_ALLOC; once
    they succeed again the same context runs both."""
    inp = synth.make_inputs(synth.tiny_problem(), 5)
    p = inp.problem
    ctx = xt.Context(0)
    try:
        monkeypatch.setenv("XRDT_TEST_FAIL_ALLOC", "1")
        with pytest.raises(xt.XrdtError) as e:
            xt.forward(p, *inp.args(), ctx=ctx)
        assert e.value.status == 6
        with pytest.raises(xt.XrdtError) as e:
            xt.Operator(p, inp.spectrum, inp.seg, inp.a1, inp.a2, ctx=ctx)
        assert e.value.status == 6
        monkeypatch.delenv("XRDT_TEST_FAIL_ALLOC")
        N, C, A = xt.forward(p, *inp.args(), ctx=ctx)
        assert np.isfinite(N).all() and N.max() > 0
        op = xt.Operator(p, inp.spectrum, inp.seg, inp.a1, inp.a2, ctx=ctx)
        assert op.forward(np.ones(op.unknowns, np.float32)).max() > 0
        op.close()
    finally:
        ctx.close()


@pytest.mark.gpu
def test_mlem_resumed_from_checkpoint_equals_uninterrupted(torch_cuda, tmp_path):
    """Ten iterations in one run against four, a checkpoint, and six more on
    a new operator reading it back: the same bits."""
    torch = torch_cuda
    inp = synth.config_inputs(2)
    p = inp.problem
    ctx = xt.Context(0)
    try:
        op = xt.Operator(p, inp.spectrum, inp.seg, inp.a1, inp.a2, ctx=ctx)
        xtrue = torch.from_numpy(synth.vox_truth(inp)).cuda()
        ybar = op.forward(xtrue, torch.empty(p.rays, device="cuda"))
        y = (ybar * (1e3 / float(ybar.max()))).round() + 1.0
        c = torch.full_like(y, 2.0)
        x0 = torch.where(xtrue > 0, 1.0, 0.0).float()
        x_full = x0.clone()
        op.mlem(y, c, x_full, 10)
        x_part = x0.clone()
        op.mlem(y, c, x_part, 4)
        path = str(tmp_path / "run.ckpt")
        xt.mlem_checkpoint_write(path, x_part, 4)
        op.close()
        op2 = xt.Operator(p, inp.spectrum, inp.seg, inp.a1, inp.a2, ctx=ctx)
        x_res, done = xt.mlem_checkpoint_read(path, torch.empty_like(x0))
        assert done == 4
        op2.mlem(y, c, x_res, 10 - done)
        torch.cuda.synchronize()
        assert torch.equal(x_res, x_full)
        op2.close()
    finally:
        ctx.close()
