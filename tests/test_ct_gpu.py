"""The transmission CT sinogram (xrdt_ct_sinogram) against its FP64
restatement in the oracle, and its no-phantom limit."""
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


@pytest.mark.parametrize("which", ["tiny", "c0"])
def test_ct_matches_oracle(ctx, oracle_lib, which):
    inp = synth.make_inputs(synth.tiny_problem(), 4) if which == "tiny" else synth.config_inputs(0)
    p = inp.problem
    T, G = xt.ct_sinogram(p, inp.spectrum, inp.a1, inp.a2, ctx=ctx)
    rays = np.arange(p.rays) if which == "tiny" else np.random.default_rng(1).choice(p.rays, 2048, replace=False)
    Tr, Gr = oracle_lib.ct_rays(inp, rays)
    assert max_rel_err(T[rays], Tr) < FAST_RTOL
    assert max_rel_err(G[rays], Gr) < 1e-6
    assert np.all(T <= G * (1 + 1e-6)) and np.all(T > 0)


def test_ct_without_phantom_transmits_everything(ctx):
    inp = synth.make_inputs(synth.tiny_problem(), 4)
    z = np.zeros_like(inp.a1)
    T, G = xt.ct_sinogram(inp.problem, inp.spectrum, z, z, ctx=ctx)
    np.testing.assert_allclose(T, G, rtol=1e-6)
