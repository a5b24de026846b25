"""The cross-section table path (xrdt_forward_tables): the coherent term read
from the tabulated cross-section S1 instead of the materials' fine-q patterns,
the form the reference keeps commented out after its kernel
(integrate_diffraction.cu:416-418, 479-494, 701-719), with nearest-bin or
bilinear lookups of both tables, against the FP64 oracle's restatement of the
same lines (the commented-out code itself does not compile: it names an
energy_channel function and NPSI spectra the reference does not define)."""
import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth
from tests.tolerances import FAST_RTOL, max_rel_err

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


def run(inp, S1, ctx, bilinear):
    return xt.forward_tables(inp.problem, inp.spectrum, inp.seg, inp.a1, inp.a2, S1, inp.S2,
                             inp.q_min, inp.q_max, inp.a_min, inp.a_max, bilinear=bilinear, ctx=ctx)


@pytest.mark.parametrize("bilinear", [False, True])
@pytest.mark.parametrize("quirks", [xt.QUIRK_STALE_VOXEL_A, 0])
def test_tiny_every_ray(ctx, oracle_lib, bilinear, quirks):
    inp = synth.make_inputs(synth.tiny_problem(), 7)
    inp.problem.quirks = quirks
    S1 = synth.coherent_table(inp)
    N, C = run(inp, S1, ctx, bilinear)
    rays = np.arange(inp.problem.rays)
    No, Co = oracle_lib.forward_tables(inp, S1, rays, bilinear=bilinear)
    assert max_rel_err(N, No) < FAST_RTOL
    assert max_rel_err(C, Co) < FAST_RTOL


@pytest.mark.parametrize("bilinear", [False, True])
def test_64x64_workload_sampled_rays(ctx, oracle_lib, bilinear):
    inp = synth.config_inputs(0)
    S1 = synth.coherent_table(inp, 1)
    N, C = run(inp, S1, ctx, bilinear)
    rays = np.sort(np.random.default_rng(31).choice(inp.problem.rays, 192, replace=False))
    No, Co = oracle_lib.forward_tables(inp, S1, rays, bilinear=bilinear)
    assert max_rel_err(N[rays], No) < FAST_RTOL
    assert max_rel_err(C[rays], Co) < FAST_RTOL


def test_nearest_compton_equals_the_forward(ctx):
    """With nearest lookups the Compton counts are those of xrdt_forward, bit
    for bit (the same kernel code), and a constant S1 gives the same coherent
    counts either way."""
    inp = synth.config_inputs(0)
    p = inp.problem
    S1 = synth.coherent_table(inp, 2)
    _, C = run(inp, S1, ctx, False)
    _, Cf, _ = xt.forward(p, *inp.args(), want_amatrix=False, ctx=ctx)
    assert np.array_equal(C, Cf)
    Sc = np.full(p.nq * p.na, 117.5, np.float32)
    Nn, _ = run(inp, Sc, ctx, False)
    Nb, _ = run(inp, Sc, ctx, True)
    assert max_rel_err(Nb, Nn) < 1e-6


def test_device_buffers_and_errors(ctx, torch_cuda):
    torch = torch_cuda
    inp = synth.make_inputs(synth.tiny_problem(), 3)
    p = inp.problem
    S1 = synth.coherent_table(inp)
    Nh, Ch = run(inp, S1, ctx, True)
    d = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (inp.spectrum, inp.seg, inp.a1, inp.a2, S1, inp.S2)]
    Nd = torch.empty(p.rays, device="cuda")
    Cd = torch.empty(p.rays, device="cuda")
    xt.forward_tables(p, *d, inp.q_min, inp.q_max, inp.a_min, inp.a_max, Nphotons=Nd, Cphotons=Cd,
                      bilinear=True, ctx=ctx)
    assert np.array_equal(Nd.cpu().numpy(), Nh) and np.array_equal(Cd.cpu().numpy(), Ch)
    with pytest.raises(xt.XrdtError):
        xt.forward_tables(p, inp.spectrum, inp.seg, inp.a1, inp.a2, S1, inp.S2, inp.q_min, inp.q_max,
                          inp.a_min, inp.a_max, ctx=ctx, flags=0x1)    # the FP64 kernel has no table path
