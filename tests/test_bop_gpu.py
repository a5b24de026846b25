"""The per-voxel operator with a dense q basis (xrdt_bop_*): J coefficients
per voxel expanded onto the NWT coarse q bins on the tensor cores (tcgen05,
3xTF32), the back-projection contracted with the basis likewise.  Checked
against the plain operator with the expansion and contraction done in FP64,
against the FP64 oracle on sampled rays, by the dot-product identity, and
MLEM on the coefficients against a dense FP64 restatement."""
import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth
from tests.tolerances import FAST_RTOL, MLEM_FLOOR, MLEM_RTOL, max_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = xt.Context(0)
    yield c
    c.close()


def gaussian_basis(J, K):
    """J non-negative Gaussian bumps spread over the K coarse bins."""
    k = np.arange(K)[None, :]
    mu = np.linspace(0, K - 1, J)[:, None]
    w = 0.8 * K / J
    return np.exp(-0.5 * ((k - mu) / w) ** 2).astype(np.float32)


def rand_c(inp, J, seed):
    p = inp.problem
    c = np.random.default_rng(seed).uniform(0.0, 1.0, (p.nx * p.ny, J)).astype(np.float32)
    c[np.asarray(inp.seg).reshape(-1) == 0] = 0.0
    return c


@pytest.mark.parametrize("J", [16, 32])
def test_basis_forward_adjoint_against_fp64_expansion_and_oracle(ctx, oracle_lib, J):
    inp = synth.sub_phantom_inputs()
    p = inp.problem
    B = gaussian_basis(J, p.nwt)
    op = xt.Operator(p, inp.spectrum, inp.seg, inp.a1, inp.a2, ctx=ctx)
    bop = xt.BasisOperator(op, B)
    c = rand_c(inp, J, 3)
    x = (c.astype(np.float64) @ B.astype(np.float64))          # FP64 expansion
    y = bop.forward(c.reshape(-1))
    assert max_rel_err(y, op.forward(x.astype(np.float32).reshape(-1))) < FAST_RTOL
    rng = np.random.default_rng(4)
    rays = np.sort(rng.choice(p.rays, 48, replace=False))
    y_ref, _ = oracle_lib.vox_rays(inp, rays, x=x.reshape(-1))
    assert max_rel_err(y[rays], y_ref) < FAST_RTOL
    w = rng.uniform(0.0, 1.0, p.rays).astype(np.float32)
    g = bop.adjoint(w).astype(np.float64).reshape(-1, J)
    gx = op.adjoint(w).astype(np.float64).reshape(-1, p.nwt)
    assert max_rel_err(g, gx @ B.astype(np.float64).T) < FAST_RTOL
    assert not g[np.asarray(inp.seg).reshape(-1) == 0].any()
    # <A B c, w> = <c, B^T A^T w>
    lhs = float(y.astype(np.float64) @ w.astype(np.float64))
    rhs = float(c.reshape(-1).astype(np.float64) @ g.reshape(-1))
    assert abs(lhs - rhs) <= 1e-5 * abs(rhs)
    bop.close()
    op.close()


def test_basis_mlem_matches_dense_restatement(ctx, oracle_lib):
    inp = synth.make_inputs(synth.tiny_problem(), 9)
    p = inp.problem
    J = 16
    B = gaussian_basis(J, p.nwt).astype(np.float64)
    _, _, _, Av = oracle_lib.forward_rays(inp, np.arange(p.rays), want_av=True)
    nvox = p.nx * p.ny
    A = Av.reshape(p.rays, nvox, p.nwt)
    Ac = np.einsum("rvk,jk->rvj", A, B).reshape(p.rays, nvox * J)   # the operator A B^T
    on = np.repeat(np.asarray(inp.seg).reshape(-1) > 0, J)
    ctrue = np.where(on, 1.0, 0.0)
    ybar = Ac @ ctrue
    y = (np.random.default_rng(1).poisson(ybar / ybar.max() * 1e3) * (ybar.max() / 1e3)).astype(np.float32)
    cb = np.full(p.rays, 0.05 * ybar.mean(), np.float32)
    op = xt.Operator(p, inp.spectrum, inp.seg, inp.a1, inp.a2, ctx=ctx)
    bop = xt.BasisOperator(op, B.astype(np.float32))
    x0 = np.where(on, 0.5, 0.0)
    s = Ac.sum(0)
    for iters in (1, 5, 20):
        x = bop.mlem(y, cb, x0.astype(np.float32), iters)
        xr = x0.copy()
        for _ in range(iters):
            with np.errstate(divide="ignore", invalid="ignore"):
                xr = xr * (Ac.T @ (y / (Ac @ xr + cb + 1e-20))) / (s + 1e-7)
            xr[~np.isfinite(xr)] = 0
            xr[xr < 0] = 0
        assert max_rel_err(x, xr, floor=MLEM_FLOOR) < MLEM_RTOL, iters
    bop.close()
    op.close()


def test_basis_rejects_bad_input(ctx):
    inp = synth.make_inputs(synth.tiny_problem(), 9)
    p = inp.problem
    op = xt.Operator(p, inp.spectrum, inp.seg, inp.a1, inp.a2, ctx=ctx)
    B = gaussian_basis(16, p.nwt)
    B[3, 5] = -1.0
    with pytest.raises(xt.XrdtError) as e:
        xt.BasisOperator(op, B)
    assert e.value.status == 4
    with pytest.raises(xt.XrdtError) as e:
        xt.BasisOperator(op, gaussian_basis(24, p.nwt))
    assert e.value.status == 2
    op.close()
