"""The integer decisions of the fast forward path, bit-exact against the FP64
oracle (xrdt_debug_decisions vs oracle.pyoracle.decisions).

The float outputs are compared under a tolerance, which would hide a one-bin
flip of an integer decision: a Compton table bin nq or column na moves one
voxel's Compton term by a table step, a sample count adds or drops one
attenuation sample.  So the decisions themselves are compared with
np.array_equal, per listed ray and every non-empty voxel:

* the source-energy window (find_src_nrg_range.cu:8-25);
* ROI edge and sample count of both line integrals (GetIntersection.cu:9-57,
  attenuator.cu:44-52; detector side decided in FP32 with an FP64 fallback
  near a threshold, source side in FP64);
* the Compton table bin nq for every window energy (integrate_diffraction.cu:331-337,
  FP32 with an FP64 fallback within 2e-4 of a bin edge);
* the Compton table column na per voxel (integrate_diffraction.cu:177-189) and
  the u8 quantisation of S2 (integrate_diffraction.cu:66-74).

No exception is allowed.
"""
import os

import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth
from xrd_tomography_gb300.problem import QUIRK_STALE_VOXEL_A, reference_problem

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = xt.Context(0)
    yield c
    c.close()


def golden_inputs(name):
    g = np.load(os.path.join(GOLDEN, name))
    p = reference_problem(int(g["nx"]), int(g["ny"]))
    t = g["tables"]
    return synth.Inputs(p, g["spectrum"], g["Ifine"], g["seg"], g["a1"], g["a2"], g["S2"],
                        float(t[0]), float(t[1]), float(t[2]), float(t[3]))


def compare(inp, rays, ctx, oracle_lib):
    got = xt.debug_decisions(inp.problem, rays, inp.spectrum, inp.seg, inp.a1, inp.a2, inp.S2,
                             inp.q_min, inp.q_max, inp.a_min, inp.a_max, ctx=ctx)
    ref = oracle_lib.decisions(inp, rays)
    nv = int((np.asarray(inp.seg) > 0).sum())
    assert got["walk"].shape == (rays.size, nv, 4)
    report = []
    for key in ("win", "walk", "nq", "na", "s2u8"):
        a, b = got[key], ref[key]
        assert a.shape == b.shape, key
        bad = np.argwhere(a != b)
        for idx in bad[:20]:
            report.append(f"{key}{tuple(int(i) for i in idx)}: gpu {a[tuple(idx)]} oracle {b[tuple(idx)]}")
        if bad.size:
            report.append(f"{key}: {len(bad)} of {a.size} differ")
    assert not report, "\n".join(report)
    # the comparison covers real decisions: rays enter the ROI and take samples
    assert (got["walk"][..., 0] > 0).any() and (got["walk"][..., 2] > 0).any()
    assert (got["walk"][..., 1] >= 0).all() and (got["walk"][..., 3] >= 0).all()
    return got


@pytest.mark.parametrize("quirk", [True, False])
def test_tiny_every_ray(ctx, oracle_lib, quirk):
    inp = synth.make_inputs(synth.tiny_problem(), 5)
    p = inp.problem
    p.quirks = QUIRK_STALE_VOXEL_A if quirk else 0
    got = compare(inp, np.arange(p.rays), ctx, oracle_lib)
    # several Compton bins and columns are in play, not one constant
    assert np.unique(got["nq"]).size > 3 and np.unique(got["na"]).size > 1


@pytest.mark.parametrize("name", ["ref_forward_16.npz", "ref_forward_20x12.npz"])
def test_reference_configuration_golden_inputs(ctx, oracle_lib, name):
    """The reference's compiled configuration on the inputs of the golden
    fixtures (made from the reference's own kernel files)."""
    inp = golden_inputs(name)
    rng = np.random.default_rng(40)
    rays = np.sort(rng.choice(inp.problem.rays, 96, replace=False))
    compare(inp, rays, ctx, oracle_lib)


def test_64x64_workload(ctx, oracle_lib):
    inp = synth.config_inputs(0)
    rng = np.random.default_rng(41)
    rays = np.sort(rng.choice(inp.problem.rays, 256, replace=False))
    compare(inp, rays, ctx, oracle_lib)


def test_256x256_workload(ctx, oracle_lib):
    inp = synth.config_inputs(1)
    rng = np.random.default_rng(42)
    rays = np.sort(rng.choice(inp.problem.rays, 48, replace=False))
    compare(inp, rays, ctx, oracle_lib)


def test_axis_aligned_rays(ctx, oracle_lib):
    """Views at multiples of 90 degrees send rays along the voxel grid, where
    a length lands exactly on a multiple of the sample step and an entry
    point on an ROI corner: the cases the FP32 guard bands exist for."""
    inp = synth.make_inputs(synth.tiny_problem(), 6)
    p = inp.problem
    p.n_col = 9      # an odd count puts the middle pixel on the axis through the centre
    inp = synth.make_inputs(p, 6)
    rays = np.arange(p.rays)
    compare(inp, rays, ctx, oracle_lib)
