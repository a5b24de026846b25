"""xrdt_mlem_matrix_noalloc: the MLEM entry point for callers that cannot
allocate device memory (its scratch is a fixed array inside the library).

It must give what xrdt_mlem_matrix gives, within the MLEM tolerance of the
other tests, on two calls in a row -- the second call reuses the scratch the
first one left behind.  This file is collected last so that a run stopping at
the first failure has run every other test before it.
"""
import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth

from tests.tolerances import MLEM_FLOOR, MLEM_RTOL, max_rel_err

pytestmark = pytest.mark.gpu


def test_noalloc_mlem_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = xt.Context(0)
    try:
        inp = synth.config_inputs(0)
        p = inp.problem
        K = p.nwt * p.n_mat
        N = torch.empty(p.rays, dtype=torch.float32, device="cuda")
        C = torch.empty_like(N)
        A = torch.empty(p.amatrix_elems, dtype=torch.float32, device="cuda")
        xt.forward(p, *inp.args(), Nphotons=N, Cphotons=C, Amatrix=A, ctx=ctx)
        torch.cuda.synchronize()
        gen = torch.Generator(device="cpu").manual_seed(11)
        y = torch.poisson((N + C).cpu(), generator=gen).cuda()
        x_ref = torch.full((K,), 10.0, dtype=torch.float32, device="cuda")
        x_na = x_ref.clone()
        # a call with no iterations leaves x as it is; it is the first use of
        # the library's device code here, which the driver may load (with the
        # fixed scratch array) only now
        xt.mlem_matrix_noalloc(A, y, C, x_na, 0)
        torch.cuda.synchronize()
        assert torch.equal(x_na, x_ref)
        for iters in (7, 13):   # two calls in a row, continuing from the current estimate
            xt.mlem_matrix(A, y, C, x_ref, iters, ctx=ctx)
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            xt.mlem_matrix_noalloc(A, y, C, x_na, iters)
            torch.cuda.synchronize()
            # the point of the entry point: the call took no device memory
            assert torch.cuda.mem_get_info()[0] >= free_before
            a, b = x_na.cpu().numpy().astype(np.float64), x_ref.cpu().numpy().astype(np.float64)
            assert np.all(np.isfinite(a))
            assert max_rel_err(a, b, floor=MLEM_FLOOR) < MLEM_RTOL, iters
    finally:
        ctx.close()


def test_noalloc_rejects_host_memory_and_bad_sizes():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = xt.lib()
    A = torch.ones(64, dtype=torch.float32, device="cuda")
    y = torch.ones(8, dtype=torch.float32, device="cuda")
    x = torch.ones(8, dtype=torch.float32, device="cuda")
    xh = np.ones(8, np.float32)
    assert L.xrdt_mlem_matrix_noalloc(A.data_ptr(), 8, 8, y.data_ptr(), y.data_ptr(), xh.ctypes.data, 1, None) == 7
    assert L.xrdt_mlem_matrix_noalloc(A.data_ptr(), 8, 2048, y.data_ptr(), y.data_ptr(), x.data_ptr(), 1, None) == 2
    assert L.xrdt_mlem_matrix_noalloc(A.data_ptr(), 8, 6, y.data_ptr(), y.data_ptr(), x.data_ptr(), 1, None) == 2
    # a view that starts 4 bytes into its storage cannot be read as 16-byte vectors
    A2 = torch.ones(65, dtype=torch.float32, device="cuda")[1:]
    assert L.xrdt_mlem_matrix_noalloc(A2.data_ptr(), 8, 8, y.data_ptr(), y.data_ptr(), x.data_ptr(), 1, None) == 7
    # the Python wrapper checks sizes and types before anything reaches the device
    with pytest.raises(ValueError):
        xt.mlem_matrix_noalloc(A[:56], y, y, x, 1)
    with pytest.raises(ValueError):
        xt.mlem_matrix_noalloc(A, y, y[:7], x, 1)
    with pytest.raises(ValueError):
        xt.mlem_matrix_noalloc(A.double(), y, y, x, 1)
