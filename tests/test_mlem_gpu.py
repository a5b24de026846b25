"""MLEM with an explicit model matrix (main.m:154-176) against its FP64
restatement (oracle/mlem.py), through the C ABI."""
import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth
from oracle.mlem import mlem_matrix as mlem_ref
from tests.tolerances import MLEM_FLOOR, MLEM_RTOL, max_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def ctx(torch_cuda):
    c = xt.Context(0)
    yield c
    c.close()


def measured(N, C, seed):
    """Poisson counts of the noise-free model (main.m:141)."""
    rng = np.random.default_rng(seed)
    return rng.poisson(np.asarray(N, np.float64) + np.asarray(C, np.float64)).astype(np.float32)


def rel(a, b):
    """Element-wise relative error above MLEM_FLOOR of the largest entry."""
    return max_rel_err(a, b, floor=MLEM_FLOOR)


def test_tiny_mlem_matches_reference_loop(ctx):
    inp = synth.make_inputs(synth.tiny_problem(), 31)
    p = inp.problem
    N, C, A = xt.forward(p, *inp.args(), ctx=ctx)
    K = p.nwt * p.n_mat
    A = A.reshape(p.rays, K)
    y = measured(N, C, 1)
    x0 = np.full(K, 10.0, np.float32)            # main.m:154
    for iters in (1, 5, 50):
        x = xt.mlem_matrix(A, y, C, x0, iters, ctx=ctx)
        xr = mlem_ref(A, y, C, x0, iters)
        assert rel(x, xr) < MLEM_RTOL, iters


def test_config0_mlem_device_buffers(ctx, torch_cuda):
    torch = torch_cuda
    inp = synth.config_inputs(0)
    p = inp.problem
    K = p.nwt * p.n_mat
    Nd = torch.empty(p.rays, dtype=torch.float32, device="cuda")
    Cd = torch.empty_like(Nd)
    Ad = torch.empty(p.amatrix_elems, dtype=torch.float32, device="cuda")
    xt.forward(p, *inp.args(), Nphotons=Nd, Cphotons=Cd, Amatrix=Ad, ctx=ctx)
    torch.cuda.synchronize()
    y = measured(Nd.cpu().numpy(), Cd.cpu().numpy(), 2)
    yd = torch.from_numpy(y).cuda()
    xd = torch.full((K,), 10.0, dtype=torch.float32, device="cuda")
    xt.mlem_matrix(Ad, yd, Cd, xd, 20, ctx=ctx)
    torch.cuda.synchronize()
    xr = mlem_ref(Ad.view(p.rays, K).cpu().numpy(), y, Cd.cpu().numpy(), np.full(K, 10.0), 20)
    assert rel(xd.cpu().numpy(), xr) < MLEM_RTOL
    # a second call continues from the current estimate (in place)
    xt.mlem_matrix(Ad, yd, Cd, xd, 5, ctx=ctx)
    torch.cuda.synchronize()
    xr2 = mlem_ref(Ad.view(p.rays, K).cpu().numpy(), y, Cd.cpu().numpy(), xr, 5)
    assert rel(xd.cpu().numpy(), xr2) < MLEM_RTOL


def test_mlem_zero_iterations_and_fixups(ctx):
    rng = np.random.default_rng(3)
    rays, K = 1000, 64
    A = rng.uniform(0, 1, (rays, K)).astype(np.float32)
    A[:, 5] = 0.0                                   # a column no ray sees
    y = rng.poisson(20, rays).astype(np.float32)
    c = np.full(rays, 0.5, np.float32)
    x0 = np.full(K, 10.0, np.float32)
    np.testing.assert_array_equal(xt.mlem_matrix(A, y, c, x0, 0, ctx=ctx), x0)
    x = xt.mlem_matrix(A, y, c, x0, 10, ctx=ctx)
    assert x[5] == 0.0 and np.all(np.isfinite(x)) and np.all(x >= 0)
    assert rel(x, mlem_ref(A, y, c, x0, 10)) < MLEM_RTOL
    y0 = np.zeros(rays, np.float32)                 # no counts: everything goes to 0
    assert not xt.mlem_matrix(A, y0, c, x0, 1, ctx=ctx).any()
    ynan = y.copy()
    ynan[7] = np.nan                                # non-finite results are zeroed (main.m:163)
    xn = xt.mlem_matrix(A, ynan, c, x0, 1, ctx=ctx)
    assert np.all(np.isfinite(xn)) and not xn.any()


def test_mlem_rejects_bad_shapes(ctx):
    A = np.ones((10, 6), np.float32)
    y = np.ones(10, np.float32)
    with pytest.raises(xt.XrdtError) as e:
        xt.mlem_matrix(A, y, y, np.ones(6, np.float32), 3, ctx=ctx)
    assert e.value.status == 2
