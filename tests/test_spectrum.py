"""The spectrum-response builder (spectrum_builder.m:64-95): the oracle's
matrix form against the reference's literal double loop, a conservation
property (CPU), and the CUDA builder against the oracle (GPU)."""
import os

import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth
from oracle import spectrum as osp
from tests.tolerances import max_rel_err

SPEC_RTOL = 1e-6   # FP64 build, output rounded to float once


def irregular_fine(rng, n=120, lo=15.0, hi=85.0):
    e = np.sort(rng.uniform(lo, hi, n - 1))
    e = np.concatenate([[lo], e, [hi]]).astype(np.float32)
    counts = rng.uniform(0.0, 5.0, n).astype(np.float32)
    return e, counts


def test_oracle_matrix_form_equals_reference_loops():
    rng = np.random.default_rng(1)
    e, n = irregular_fine(rng)
    src = np.linspace(20.0, 80.0, 8)
    det = np.array([14.0, 22.5, 30.0, 41.0, 55.0, 63.0, 90.0])
    a = osp.response(e, n, src, det)
    b = osp.response_loops(e, n, src, det)
    assert np.max(np.abs(a - b)) <= 1e-13 * np.abs(a).max()
    assert np.all(a >= 0.0)


def conservation_rows(e, n, src, resp, sigma0=osp.SIGMA0, sigma1=osp.SIGMA1, margin=12.0):
    """Rows of source bins at least `margin` widths inside the fine grid, and
    their photon counts sum_h ws[h, s] n[h]."""
    e = np.asarray(e, np.float64)
    left, right = e[:-1], e[1:]
    ws = osp._overlap(left, right, src)
    counts = ws.T @ np.asarray(n, np.float64)
    rows = [s for s in range(len(src) - 1)
            if src[s] - margin * (sigma0 + sigma1 * src[s]) > e[0]
            and src[s + 1] + margin * (sigma0 + sigma1 * src[s + 1]) < e[-1]]
    return rows, counts


def test_oracle_conserves_photons_away_from_the_ends():
    """A detector grid covering the whole fine range catches every photon of
    a source bin whose Gaussian stays inside it (the fine bins sample the
    Gaussian 0.05 keV apart, far below its width)."""
    e, n = synth.hd_spectrum()
    src = np.linspace(8.0, 80.0, 37)
    det = np.linspace(8.0, 80.0, 49)
    resp = osp.response(e, n, src, det)
    rows, counts = conservation_rows(e, n, src, resp)
    assert rows
    got = resp.sum(axis=1)[rows]
    assert np.max(np.abs(got - counts[rows]) / counts[rows]) < 1e-9


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = xt.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("grids", ["reference", "rectangular", "irregular", "measured"])
def test_spectrum_build_matches_oracle(ctx, grids):
    rng = np.random.default_rng(3)
    if grids == "measured":
        # the reference's measured 80 kVp spectrum (Spectrum_80kVp/spectral_data_HD.mat,
        # read by xrd_tomography_gb300.matfile into tests/golden/real_inputs.npz): its
        # 1441 edges and the counts of the 1440 bins (spectrum_builder.m:26-30)
        fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "real_inputs.npz"))
        e = fx["spectrum_energy"].astype(np.float32)
        n = fx["spectrum_counts"][:-1].astype(np.float32)
        src = det = np.linspace(8.0, 80.0, 65).astype(np.float32)
    elif grids == "reference":
        # the reference's grid: 1440 bins of 0.05 keV, 64 coarse bins over 8-80 keV
        e, n = synth.hd_spectrum()
        src = det = np.linspace(8.0, 80.0, 65).astype(np.float32)
    elif grids == "rectangular":
        # the 64x64 workload's grids: 40 source and 32 detector bins over 20-80 keV
        e, n = synth.hd_spectrum(e_min=20.0, n=1200)
        src = np.linspace(20.0, 80.0, 41).astype(np.float32)
        det = np.linspace(20.0, 80.0, 33).astype(np.float32)
    else:
        e, n = irregular_fine(rng, n=500)
        src = np.sort(rng.uniform(10.0, 90.0, 23)).astype(np.float32)
        det = np.sort(rng.uniform(10.0, 90.0, 17)).astype(np.float32)
    got = xt.spectrum_build(e, n, src, det, ctx=ctx)
    ref = osp.flat(osp.response(e, n, src, det))
    assert got.shape == ref.shape
    assert max_rel_err(got, ref) < SPEC_RTOL


@pytest.mark.gpu
def test_spectrum_build_device_buffers_conservation_and_errors(ctx):
    torch = pytest.importorskip("torch")
    e, n = synth.hd_spectrum()
    src = np.linspace(8.0, 80.0, 129).astype(np.float32)
    det = np.linspace(8.0, 80.0, 97).astype(np.float32)
    d = [torch.from_numpy(x).cuda() for x in (e, n, src, det)]
    out = torch.empty((len(src) - 1) * (len(det) - 1), device="cuda")
    xt.spectrum_build(*d, out=out, ctx=ctx)
    got = out.cpu().numpy()
    host = xt.spectrum_build(e, n, src, det, ctx=ctx)
    np.testing.assert_array_equal(got, host)
    resp = got.reshape(len(det) - 1, len(src) - 1).T.astype(np.float64)
    rows, counts = conservation_rows(e, n, src.astype(np.float64), resp)
    assert max_rel_err(resp.sum(axis=1)[rows], counts[rows]) < 1e-5
    with pytest.raises(xt.XrdtError) as err:
        xt.spectrum_build(e[::-1].copy(), n, src, det, ctx=ctx)
    assert err.value.status == 4
    with pytest.raises(xt.XrdtError) as err:
        xt.spectrum_build(e, n, src, det, sigma0=-5.0, sigma1=0.0, ctx=ctx)
    assert err.value.status == 4
    with pytest.raises(ValueError):
        xt.spectrum_build(e[:-1], n, src, det, ctx=ctx)
