"""The FP64 oracle against the reference itself (CPU only).

tests/golden holds outputs of the reference's own Forward_projector_kernels,
compiled unmodified for the host in FP64 (tests/golden/make_golden.py).  The
oracle must reproduce them: integer results exactly, counts to 1e-10.
"""
import os

import numpy as np
import pytest

from xrd_tomography_gb300.problem import reference_problem, src_nrg_range, coarse_q_grid
from xrd_tomography_gb300 import synth
from tests.tolerances import max_rel_err

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name))


def inputs_from(g):
    p = reference_problem(int(g["nx"]), int(g["ny"]))
    t = g["tables"]
    return synth.Inputs(p, g["spectrum"], g["Ifine"], g["seg"], g["a1"], g["a2"], g["S2"],
                        float(t[0]), float(t[1]), float(t[2]), float(t[3]))


def test_config_of_golden_matches_reference_preset():
    g = load("ref_helpers.npz")
    p = reference_problem(100)
    assert list(g["config"]) == [p.n_src, p.n_col, p.n_row, p.nrg_det, p.dnrg, p.nwt, p.nqf, p.n_mat, p.nq, p.na]


def test_wvt_value_bit_exact(oracle_lib):
    g = load("ref_helpers.npz")
    p = reference_problem(100)
    for n in range(p.nwt):
        q, dq = oracle_lib.wvt_value(p, n)
        assert q == g["wvt_q"][n] and dq == g["wvt_dq"][n], n
    # the numpy grid used by the host code agrees to rounding
    qc, dqc = coarse_q_grid(p)
    np.testing.assert_allclose(qc, g["wvt_q"], rtol=1e-15)
    np.testing.assert_allclose(dqc, g["wvt_dq"], rtol=1e-12)


def test_wvt_value_known_answer(oracle_lib):
    # nwt = 255 -> q = 5.98353806, dq = 0.03292389 (to 8 digits; the ninth depends on
    # whether the int*float products of wvt_value.cu:14-19 round to float first)
    q, dq = oracle_lib.wvt_value(reference_problem(100), 255)
    assert abs(q - 5.98353806) < 2e-8 and abs(dq - 0.03292389) < 2e-8


def test_src_nrg_range_bit_exact(oracle_lib):
    g = load("ref_helpers.npz")
    p = reference_problem(100)
    for n in range(p.nrg_det):
        assert oracle_lib.src_nrg_range(p, n) == (g["nrg_lo"][n], g["nrg_hi"][n])
        assert src_nrg_range(p, n) == (g["nrg_lo"][n], g["nrg_hi"][n])
    assert oracle_lib.src_nrg_range(p, 0) == (0, 10)
    assert oracle_lib.src_nrg_range(p, 63) == (53, 63)


def test_src_nrg_range_rectangular(oracle_lib):
    p = synth.config_problem(0)   # 40 source bins, 32 detector bins
    for n in range(p.nrg_det):
        lo, hi = oracle_lib.src_nrg_range(p, n)
        assert (lo, hi) == src_nrg_range(p, n)
        assert hi - lo == 2 * p.dnrg and 0 <= lo and hi < p.nrg_src
        e_centre = p.e_det_min + (n + 0.5) * (p.e_det_max - p.e_det_min) / p.nrg_det
        dEs = (p.e_src_max - p.e_src_min) / p.nrg_src
        assert p.e_src_min + lo * dEs <= e_centre <= p.e_src_min + (hi + 1) * dEs


def test_get_intersection_bit_exact(oracle_lib):
    g = load("ref_helpers.npz")
    for s, rx, ry in zip(g["segs"], g["int_x"], g["int_y"]):
        x, y = oracle_lib.get_intersection(*s[:4], int(s[4]), int(s[5]))
        if np.isnan(rx):
            assert np.isnan(x) and np.isnan(y)
        else:
            assert (x, y) == (rx, ry)


def test_get_intersection_known_answer(oracle_lib):
    x, y = oracle_lib.get_intersection(-50.0, 50.0, 50.5, 50.5, 100, 100)
    assert x == 0.0 and abs(y - 50.2488) < 1e-4


def test_attenuation_uniform_map(oracle_lib):
    # uniform map, nearly vertical ray entering at y = 0: the sample on the
    # border reads a/2 and the next a*3/4 (bilinear against the zero border),
    # every later one reads a, so A1 = DQ * a * (n - 0.75)
    p = reference_problem(16)
    a = 0.01
    inp = synth.Inputs(p, None, None, np.ones(256, np.int32), np.full(256, a, np.float32),
                       np.full(256, 2 * a, np.float32), None, 0, 0, 0, 0)
    A1, A2, n = oracle_lib.attenuator(inp, 8.3, -40.0, 8.5, 8.5)
    Lr = np.hypot(8.5 - (8.3 + 0.2 * 40.0 / 48.5), 8.5)
    assert n == int(np.floor(Lr / 0.25)) + 1
    assert abs(A2 - 2 * A1) < 1e-15
    assert abs(A1 - 0.25 * a * (n - 0.75)) < 1e-4 * A1


@pytest.mark.parametrize("name", ["ref_forward_16.npz", "ref_forward_20x12.npz"])
def test_forward_matches_reference_kernel(oracle_lib, name):
    g = load(name)
    inp = inputs_from(g)
    N, C, _, _ = oracle_lib.forward_rays(inp, g["rays"])
    assert max_rel_err(N, g["N"], floor=0) < 1e-10
    assert max_rel_err(C, g["C"], floor=0) < 1e-10
    _, _, A, _ = oracle_lib.forward_rays(inp, g["A_rays"], want_a=True)
    assert max_rel_err(A, g["A"], floor=1e-12) < 1e-10


def test_per_voxel_rows_sum_to_amatrix(oracle_lib):
    inp = synth.make_inputs(synth.tiny_problem(), 11)
    p = inp.problem
    rays = np.arange(0, p.rays, 7)
    _, _, A, Av = oracle_lib.forward_rays(inp, rays, want_a=True, want_av=True)
    seg = inp.seg
    for m in range(p.n_mat):
        mask = seg == m + 1
        np.testing.assert_allclose(Av[:, mask, :].sum(1), A[:, m, :], rtol=1e-12, atol=1e-300)
    assert np.all(Av[:, seg == 0, :] == 0)


def test_empty_phantom_gives_zeros(oracle_lib):
    inp = synth.make_inputs(synth.tiny_problem(), 3)
    inp.seg = np.zeros_like(inp.seg)
    N, C, A, _ = oracle_lib.forward_rays(inp, np.arange(40), want_a=True)
    assert not N.any() and not C.any() and not A.any()


def test_material_id_above_range_rejected(oracle_lib):
    inp = synth.make_inputs(synth.tiny_problem(), 3)
    inp.seg = inp.seg.copy()
    inp.seg[5] = inp.problem.n_mat + 1
    with pytest.raises(ValueError):
        oracle_lib.forward_rays(inp, np.arange(4))


def test_stale_voxel_quirk_only_changes_compton(oracle_lib):
    inp = synth.make_inputs(synth.tiny_problem(), 21)
    rays = np.arange(0, inp.problem.rays, 5)
    N1, C1, A1, _ = oracle_lib.forward_rays(inp, rays, want_a=True)
    inp.problem = inp.problem.copy(quirks=0)
    N0, C0, A0, _ = oracle_lib.forward_rays(inp, rays, want_a=True)
    assert np.array_equal(N0, N1) and np.array_equal(A0, A1)
    assert not np.array_equal(C0, C1)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLD), "..", "oracle", "_ref", "libxrdt_ref.so")),
                    reason="reference build absent (its sources are not on this machine)")
def test_forward_matches_reference_kernel_fresh_inputs(oracle_lib):
    from oracle import pyoracle as po
    p = reference_problem(14, 18)
    inp = synth.make_inputs(p, 99, n_ellipses=5)
    rays = np.random.default_rng(5).choice(p.rays, 12, replace=False)
    N, C, A, _ = po.forward_rays(inp, rays, want_a=True)
    Nr, Cr, Ar = po.ref_forward_rays(inp, rays)
    assert max_rel_err(N, Nr, floor=0) < 1e-10
    assert max_rel_err(C, Cr, floor=0) < 1e-10
    assert max_rel_err(A, Ar, floor=1e-12) < 1e-10


def test_oracle_ct_limits(oracle_lib):
    """CT restatement: without a phantom every channel transmits its whole
    spectrum weight; doubling the attenuation lowers every transmission."""
    from xrd_tomography_gb300 import synth
    inp = synth.make_inputs(synth.tiny_problem(), 4)
    rays = np.arange(inp.problem.rays)
    T, G = oracle_lib.ct_rays(inp, rays)
    z = synth.make_inputs(synth.tiny_problem(), 4)
    z.a1 = np.zeros_like(z.a1)
    z.a2 = np.zeros_like(z.a2)
    T0, G0 = oracle_lib.ct_rays(z, rays)
    np.testing.assert_array_equal(T0, G0)
    np.testing.assert_array_equal(G, G0)
    d = synth.make_inputs(synth.tiny_problem(), 4)
    d.a1 = 2 * d.a1
    d.a2 = 2 * d.a2
    T2, _ = oracle_lib.ct_rays(d, rays)
    hit = T < G
    assert hit.any() and np.all(T2[hit] < T[hit]) and np.all(T2[~hit] == T[~hit])


def test_table_path_restatement(oracle_lib):
    """The oracle's cross-section table path (integrate_diffraction.cu:701-719,
    commented out in the reference): with nearest lookups its Compton counts
    are the forward's; a constant coherent table gives the same coherent
    counts by nearest and bilinear lookup; and a coherent table that is
    linear along the wavevector axis is read exactly by the bilinear lookup,
    so the counts are linear in the table."""
    inp = synth.make_inputs(synth.tiny_problem(), 7)
    p = inp.problem
    rays = np.arange(p.rays)
    S1 = synth.coherent_table(inp)
    _, C_tab = oracle_lib.forward_tables(inp, S1, rays)
    _, C_fwd, _, _ = oracle_lib.forward_rays(inp, rays)
    assert np.array_equal(C_tab, C_fwd)
    Sc = np.full(p.nq * p.na, 99.0, np.float32)
    Nn, _ = oracle_lib.forward_tables(inp, Sc, rays)
    Nb, _ = oracle_lib.forward_tables(inp, Sc, rays, bilinear=True)
    assert np.allclose(Nn, Nb, rtol=1e-13, atol=0)
    # integer-valued tables a + b*i along q (no u8 rounding): bilinear counts
    # are affine in (a, b)
    iq = np.tile(np.arange(p.nq, dtype=np.float32), p.na)
    N1, _ = oracle_lib.forward_tables(inp, 10.0 + 2.0 * iq, rays, bilinear=True)
    N2, _ = oracle_lib.forward_tables(inp, 30.0 + 6.0 * iq, rays, bilinear=True)
    N0, _ = oracle_lib.forward_tables(inp, np.full(p.nq * p.na, 10.0, np.float32), rays, bilinear=True)
    assert np.allclose(N2, 3.0 * N1, rtol=1e-12, atol=0)
    assert np.all(N1 >= N0)
