"""Basis expansion on the tensor cores (xrdt_basis_expand): I = C B in FP32
via 3xTF32 tcgen05 MMAs, against numpy in FP64, and as the Ifine input of
the forward projector."""
import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth
from tests.tolerances import FAST_RTOL, max_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = xt.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("M,K,N", [(1, 8, 16), (128, 32, 128), (300, 32, 128), (129, 64, 256), (1000, 16, 48)])
def test_basis_expand_matches_fp64(ctx, M, K, N):
    rng = np.random.default_rng(M + K + N)
    C = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    I = xt.basis_expand(C, B, ctx=ctx)
    ref = C.astype(np.float64) @ B.astype(np.float64)
    bound = np.abs(C.astype(np.float64)) @ np.abs(B.astype(np.float64))
    # 3xTF32: each product to about 2^-21, the sum in FP32
    assert np.all(np.abs(I - ref) <= 4e-6 * bound + 1e-30), float(np.max(np.abs(I - ref) / bound))


def test_basis_expand_rejects_bad_shapes(ctx):
    with pytest.raises(xt.XrdtError) as e:
        xt.basis_expand(np.ones((4, 12), np.float32), np.ones((12, 16), np.float32), ctx=ctx)
    assert e.value.status == 2
    with pytest.raises(xt.XrdtError):
        xt.basis_expand(np.ones((4, 8), np.float32), np.ones((8, 24), np.float32), ctx=ctx)


def test_expanded_patterns_drive_the_forward(ctx):
    """Material patterns given as coefficients of a Gaussian-bump basis on the
    fine q grid: the tensor-core expansion feeds xrdt_forward as Ifine and
    gives the projection of the numpy expansion."""
    inp = synth.make_inputs(synth.tiny_problem(), 13)
    p = inp.problem
    K = 16
    q = p.q_lo + (p.q_hi - p.q_lo) / p.nqf * (np.arange(p.nqf) + 0.5)
    centres = np.linspace(p.q_lo, p.q_hi, K)
    B = np.exp(-0.5 * ((q[None, :] - centres[:, None]) / 0.15) ** 2).astype(np.float32)
    C = np.random.default_rng(2).uniform(0.0, 1.0, (p.n_mat, K)).astype(np.float32)
    I = xt.basis_expand(C, B, ctx=ctx)
    I_ref = (C.astype(np.float64) @ B.astype(np.float64)).astype(np.float32)
    assert max_rel_err(I, I_ref) < 1e-6
    args = list(inp.args())
    args[1] = I.reshape(-1)
    N1, C1, _ = xt.forward(p, *args, want_amatrix=False, ctx=ctx)
    args[1] = I_ref.reshape(-1)
    N2, C2, _ = xt.forward(p, *args, want_amatrix=False, ctx=ctx)
    assert max_rel_err(N1, N2) < FAST_RTOL
    np.testing.assert_array_equal(C1, C2)
