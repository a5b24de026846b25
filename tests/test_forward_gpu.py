"""Parity of the CUDA forward projector with the FP64 oracle (GPU).

Every call goes through the C ABI (libxrdt.so).  The oracle is the checker;
the golden fixtures hold outputs of the reference's own kernel files.
"""
import os

import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth
from xrd_tomography_gb300.problem import reference_problem
from tests.tolerances import FAST_RTOL, PLAIN_RTOL, max_rel_err

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


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


def golden_inputs(name):
    g = np.load(os.path.join(GOLD, name))
    p = reference_problem(int(g["nx"]), int(g["ny"]))
    t = g["tables"]
    inp = synth.Inputs(p, g["spectrum"], g["Ifine"], g["seg"], g["a1"], g["a2"], g["S2"],
                       float(t[0]), float(t[1]), float(t[2]), float(t[3]))
    return inp, g


def tiny(seed=5, **kw):
    inp = synth.make_inputs(synth.tiny_problem(), seed)
    if kw:
        inp.problem = inp.problem.copy(**kw)
    return inp


def rows(A, p):
    return np.asarray(A).reshape(-1, p.n_mat, p.nwt)


# ---- small problem, every ray -------------------------------------------

@pytest.mark.parametrize("quirks", [1, 0])
def test_tiny_fast_matches_oracle(ctx, oracle_lib, quirks):
    inp = tiny(quirks=quirks)
    p = inp.problem
    N, C, A = xt.forward(p, *inp.args(), ctx=ctx)
    rays = np.arange(p.rays)
    No, Co, Ao, _ = oracle_lib.forward_rays(inp, rays, want_a=True)
    assert max_rel_err(N, No) < FAST_RTOL
    assert max_rel_err(C, Co) < FAST_RTOL
    assert max_rel_err(rows(A, p), Ao) < FAST_RTOL


@pytest.mark.parametrize("quirks", [1, 0])
def test_tiny_plain_matches_oracle(ctx, oracle_lib, quirks):
    inp = tiny(quirks=quirks)
    p = inp.problem
    N, C, A = xt.forward(p, *inp.args(), plain=True, ctx=ctx)
    No, Co, Ao, _ = oracle_lib.forward_rays(inp, np.arange(p.rays), want_a=True)
    assert max_rel_err(N, No) < PLAIN_RTOL
    assert max_rel_err(C, Co) < PLAIN_RTOL
    assert max_rel_err(rows(A, p), Ao) < PLAIN_RTOL


def test_tiny_ray_subset_equals_full(ctx):
    inp = tiny(seed=9)
    p = inp.problem
    N, C, A = xt.forward(p, *inp.args(), ctx=ctx)
    rays = np.random.default_rng(1).choice(p.rays, 50, replace=False)
    for plain in (False, True):
        Ns, Cs, As = xt.forward_rays(p, rays, *inp.args(), want_amatrix=True, plain=plain, ctx=ctx)
        tol = PLAIN_RTOL if plain else FAST_RTOL
        if not plain:
            np.testing.assert_array_equal(Ns, N[rays])
            np.testing.assert_array_equal(Cs, C[rays])
        else:
            assert max_rel_err(Ns, N[rays]) < 2 * tol + FAST_RTOL
        assert max_rel_err(As, rows(A, p)[rays]) < tol + FAST_RTOL


def test_host_and_device_buffers_agree(ctx, torch_cuda):
    torch = torch_cuda
    inp = tiny(seed=13)
    p = inp.problem
    N, C, A = xt.forward(p, *inp.args(), ctx=ctx)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in
           (inp.spectrum, inp.Ifine, inp.seg, inp.a1, inp.a2, inp.S2)]
    Nd = torch.empty(p.rays, dtype=torch.float32, device="cuda")
    Cd = torch.empty_like(Nd)
    Ad = torch.empty(p.amatrix_elems, dtype=torch.float32, device="cuda")
    xt.forward(p, *dev, inp.q_min, inp.q_max, inp.a_min, inp.a_max, Nphotons=Nd, Cphotons=Cd, Amatrix=Ad,
               ctx=ctx)
    torch.cuda.synchronize()
    assert max_rel_err(Nd.cpu().numpy(), N) < FAST_RTOL
    assert max_rel_err(Cd.cpu().numpy(), C) < FAST_RTOL
    assert max_rel_err(Ad.cpu().numpy(), A) < FAST_RTOL


def test_repeat_calls_agree(ctx):
    inp = tiny(seed=17)
    p = inp.problem
    a = xt.forward(p, *inp.args(), ctx=ctx)
    b = xt.forward(p, *inp.args(), ctx=ctx)
    # N and C: no atomics and a fixed summation order, the same bits every time
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    # the model matrix adds the warps' voxel chunks with shared-memory
    # atomics, whose order varies: a few ulps at most
    np.testing.assert_array_max_ulp(a[2], b[2], maxulp=4)


# ---- reference configuration, against the reference's own outputs --------

@pytest.mark.parametrize("name", ["ref_forward_16.npz", "ref_forward_20x12.npz"])
def test_reference_preset_rays_match_golden(ctx, name):
    inp, g = golden_inputs(name)
    p = inp.problem
    for plain, tol in ((False, FAST_RTOL), (True, PLAIN_RTOL)):
        N, C, _ = xt.forward_rays(p, g["rays"], *inp.args(), plain=plain, ctx=ctx)
        assert max_rel_err(N, g["N"]) < tol, plain
        assert max_rel_err(C, g["C"]) < tol, plain
        _, _, A = xt.forward_rays(p, g["A_rays"], *inp.args(), want_amatrix=True, plain=plain, ctx=ctx)
        assert max_rel_err(A, g["A"]) < tol, plain


def test_reference_preset_full_call(ctx, torch_cuda):
    # the whole Forward_XRD output set (2M rays, a 6.4 GB model matrix) on the device
    torch = torch_cuda
    inp, g = golden_inputs("ref_forward_16.npz")
    p = inp.problem
    Nd = torch.empty(p.rays, dtype=torch.float32, device="cuda")
    Cd = torch.empty_like(Nd)
    Ad = torch.empty(p.amatrix_elems, dtype=torch.float32, device="cuda")
    xt.forward(p, *inp.args(), Nphotons=Nd, Cphotons=Cd, Amatrix=Ad, ctx=ctx)
    torch.cuda.synchronize()
    rays = torch.from_numpy(g["rays"]).cuda()
    assert max_rel_err(Nd[rays].cpu().numpy(), g["N"]) < FAST_RTOL
    assert max_rel_err(Cd[rays].cpu().numpy(), g["C"]) < FAST_RTOL
    arays = torch.from_numpy(g["A_rays"]).cuda()
    A = Ad.view(-1, p.n_mat, p.nwt)[arays].cpu().numpy()
    assert max_rel_err(A, g["A"]) < FAST_RTOL
    del Ad
    torch.cuda.empty_cache()


def test_forward_xrd_mex_shapes(ctx):
    inp, g = golden_inputs("ref_forward_20x12.npz")
    p = inp.problem
    small = p.copy(n_col=64)   # keep the host model matrix small
    seg2d = inp.seg.reshape((p.nx, p.ny), order="F")
    N, C, A = xt.Forward_XRD(inp.spectrum.reshape((64, 64), order="F"), inp.Ifine, seg2d,
                             inp.a1.reshape((p.nx, p.ny), order="F"), inp.a2.reshape((p.nx, p.ny), order="F"),
                             inp.S2.reshape((64, 64), order="F"), inp.q_min, inp.q_max, inp.a_min, inp.a_max,
                             problem=small, ctx=ctx)
    assert N.shape == (32, 64, 1, 64) and C.shape == N.shape
    assert A.shape == (256, 3, 32, 64, 1, 64)
    Nf, Cf, Af = xt.forward(small, *inp.args(), ctx=ctx)
    np.testing.assert_array_equal(N.reshape(-1, order="F"), Nf)
    np.testing.assert_array_equal(A.reshape(-1, order="F"), Af)


# ---- synthetic workloads ---------------------------------------------------

def test_config0_matches_oracle(ctx, oracle_lib, torch_cuda):
    torch = torch_cuda
    inp = synth.config_inputs(0)
    p = inp.problem
    Nd = torch.empty(p.rays, dtype=torch.float32, device="cuda")
    Cd = torch.empty_like(Nd)
    Ad = torch.empty(p.amatrix_elems, dtype=torch.float32, device="cuda")
    xt.forward(p, *inp.args(), Nphotons=Nd, Cphotons=Cd, Amatrix=Ad, ctx=ctx)
    torch.cuda.synchronize()
    rng = np.random.default_rng(0)
    rays = np.sort(rng.choice(p.rays, 256, replace=False))
    No, Co, _, _ = oracle_lib.forward_rays(inp, rays)
    t = torch.from_numpy(rays).cuda()
    assert max_rel_err(Nd[t].cpu().numpy(), No) < FAST_RTOL
    assert max_rel_err(Cd[t].cpu().numpy(), Co) < FAST_RTOL
    ar = rays[:32]
    _, _, Ao, _ = oracle_lib.forward_rays(inp, ar, want_a=True)
    A = Ad.view(-1, p.n_mat, p.nwt)[torch.from_numpy(ar).cuda()].cpu().numpy()
    assert max_rel_err(A, Ao) < FAST_RTOL


def test_config0_plain_rays(ctx, oracle_lib):
    inp = synth.config_inputs(0)
    p = inp.problem
    rays = np.random.default_rng(3).choice(p.rays, 64, replace=False)
    N, C, A = xt.forward_rays(p, rays, *inp.args(), want_amatrix=True, plain=True, ctx=ctx)
    No, Co, Ao, _ = oracle_lib.forward_rays(inp, rays, want_a=True)
    assert max_rel_err(N, No) < PLAIN_RTOL
    assert max_rel_err(C, Co) < PLAIN_RTOL
    assert max_rel_err(A, Ao) < PLAIN_RTOL


def test_config1_rays_match_oracle(ctx, oracle_lib):
    """384 random rays of the 256x256 workload (the FP64 oracle takes about
    half a second per ray and core here)."""
    inp = synth.config_inputs(1)
    p = inp.problem
    rays = np.random.default_rng(4).choice(p.rays, 384, replace=False)
    N, C, _ = xt.forward_rays(p, rays, *inp.args(), ctx=ctx)
    No, Co, _, _ = oracle_lib.forward_rays(inp, rays)
    assert max_rel_err(N, No) < FAST_RTOL
    assert max_rel_err(C, Co) < FAST_RTOL


def test_config1_full_linear_in_patterns(ctx, torch_cuda):
    # full-size properties: Nphotons is linear in Ifine, Cphotons does not
    # depend on it, and the full call agrees with the ray-subset call
    torch = torch_cuda
    inp = synth.config_inputs(1)
    p = inp.problem
    rng = np.random.default_rng(8)
    I2 = rng.uniform(0, 1, inp.Ifine.size).astype(np.float32)
    outs = []
    for I in (inp.Ifine, I2, inp.Ifine + I2):
        Nd = torch.empty(p.rays, dtype=torch.float32, device="cuda")
        Cd = torch.empty_like(Nd)
        args = list(inp.args())
        args[1] = I
        xt.forward(p, *args, Nphotons=Nd, Cphotons=Cd, want_amatrix=False, ctx=ctx)
        torch.cuda.synchronize()
        outs.append((Nd.cpu().numpy(), Cd.cpu().numpy()))
    (N1, C1), (N2, C2), (N3, C3) = outs
    assert max_rel_err(N3, N1 + N2) < 1e-5
    np.testing.assert_array_equal(C1, C2)
    np.testing.assert_array_equal(C1, C3)
    rays = rng.choice(p.rays, 100, replace=False)
    Ns, Cs, _ = xt.forward_rays(p, rays, *inp.args(), ctx=ctx)
    np.testing.assert_array_equal(Ns, N1[rays])
    np.testing.assert_array_equal(Cs, C1[rays])


# ---- edge cases --------------------------------------------------------------

def test_empty_phantom_gives_zeros(ctx):
    inp = tiny()
    inp.seg = np.zeros_like(inp.seg)
    for plain in (False, True):
        N, C, A = xt.forward(inp.problem, *inp.args(), plain=plain, ctx=ctx)
        assert not N.any() and not C.any() and not A.any()


def test_single_voxel_phantom(ctx, oracle_lib):
    inp = tiny(seed=23)
    seg = np.zeros_like(inp.seg)
    seg[5 + 7 * inp.problem.nx] = 2
    inp.seg = seg
    p = inp.problem
    N, C, A = xt.forward(p, *inp.args(), ctx=ctx)
    No, Co, Ao, _ = oracle_lib.forward_rays(inp, np.arange(p.rays), want_a=True)
    assert max_rel_err(N, No) < FAST_RTOL and max_rel_err(C, Co) < FAST_RTOL
    assert max_rel_err(rows(A, p), Ao) < FAST_RTOL
    assert not rows(A, p)[:, [0, 2], :].any()


def test_bad_material_id_rejected(ctx):
    inp = tiny()
    inp.seg = inp.seg.copy()
    inp.seg[3] = inp.problem.n_mat + 1
    for plain in (False, True):
        with pytest.raises(xt.XrdtError) as e:
            xt.forward(inp.problem, *inp.args(), plain=plain, ctx=ctx)
        assert e.value.status == 4


def test_geometry_inside_phantom_rejected(ctx):
    inp = tiny()
    inp.problem = inp.problem.copy(r_src=2.0)
    with pytest.raises(xt.XrdtError) as e:
        xt.forward(inp.problem, *inp.args(), ctx=ctx)
    assert e.value.status == 3


def test_no_sync_needs_device_outputs(ctx):
    inp = tiny()
    with pytest.raises(xt.XrdtError) as e:
        xt.forward(inp.problem, *inp.args(), ctx=ctx, flags=xt.FWD_NO_SYNC)
    assert e.value.status == 7


def test_ray_out_of_range_rejected(ctx):
    inp = tiny()
    with pytest.raises(xt.XrdtError) as e:
        xt.forward_rays(inp.problem, [inp.problem.rays], *inp.args(), ctx=ctx)
    assert e.value.status == 4


def test_launches_are_counted(ctx):
    inp = tiny()
    before = ctx.launches
    xt.forward(inp.problem, *inp.args(), ctx=ctx)
    assert ctx.launches - before >= 4


def wide_window_problem(n_src_bins):
    """The tiny problem's phantom and scanner with n_src_bins source energy
    bins over 16 detector bins (windows of 11 source bins 8 apart): the
    detector windows together span all source bins."""
    p = synth._base(12, 12, 4, 8, 1, n_src_bins, 16, (20.0, 80.0), (20.0, 80.0), 5,
                    32, 64, 3, 16, 16, (0.5, 4.0), 0.03)
    return synth.scanner(p, vox_mm=4.0, r_src_mm=150.0, r_det_mm=120.0, col_mm=4.0, row_mm=2.0,
                         z0_mm=12.0, focal_mm=1.0)


def test_widest_energy_windows(ctx, oracle_lib):
    """128 source bins inside the detector windows, the most the projector
    and the per-voxel operator take (one shared-memory row per bin): every
    ray against the oracle; 130 bins are rejected."""
    inp = synth.make_inputs(wide_window_problem(128), 13)
    p = inp.problem
    N, C, A = xt.forward(p, *inp.args(), ctx=ctx)
    rays = np.arange(p.rays)
    No, Co, Ao, _ = oracle_lib.forward_rays(inp, rays, want_a=True)
    assert max_rel_err(N, No) < FAST_RTOL
    assert max_rel_err(C, Co) < FAST_RTOL
    assert max_rel_err(np.asarray(A).reshape(Ao.shape), Ao) < FAST_RTOL
    op = xt.Operator(p, inp.spectrum, inp.seg, inp.a1, inp.a2, ctx=ctx)
    x = np.random.default_rng(5).uniform(0.0, 1.0, (p.nx * p.ny, p.nwt)).astype(np.float32)
    x[np.asarray(inp.seg).reshape(-1) == 0] = 0.0
    y_ref, _ = oracle_lib.vox_rays(inp, rays, x=x.reshape(-1))
    assert max_rel_err(op.forward(x.reshape(-1)), y_ref) < FAST_RTOL
    op.close()
    wide = synth.make_inputs(wide_window_problem(130), 13)
    with pytest.raises(xt.XrdtError):
        xt.forward(wide.problem, *wide.args(), want_amatrix=False, ctx=ctx)
