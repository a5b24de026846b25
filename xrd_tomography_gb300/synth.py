"""Seeded synthetic inputs for the forward projector and MLEM.

The reference builds its inputs from measured data files (MATLAB v7.3 .mat
files of XRD patterns, a SpekCalc spectrum, Hubbell tables:
builder_functions/*.m).  Those are not used here.  These generators produce
inputs with the same shapes, units and value ranges:

* phantom: random ellipses painted in order, later ones overwriting earlier
  ones (as builder_functions/phantom_generator.m:71-78 paints its objects),
  each with a material id and a density; a1, a2 = density x per-material base;
* XRD pattern per material: Gaussian peaks on the fine q grid plus a floor
  (the role of XRD_builder.m's output Iaxis_fine, concatenated per material,
  XRD_builder.m:187);
* spectrum: Kramers' law plus tungsten K lines, smeared by a Gaussian detector
  response sigma(E) = 0.5*(1.61 + 0.025 E) and integrated over source x
  detector bin pairs (the construction of spectrum_builder.m:64-95);
* S2 table: a smooth surface on [NQ, NA] scaled to about 0..255 with a few
  entries outside that range (the quantisation of integrate_diffraction.cu:66-74
  clamps them).

All arrays are flat, in the reference's column-major order.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .problem import Problem, QUIRK_STALE_VOXEL_A, f32, fine_q_grid, reference_problem

SEED_BASE = 20261203


@dataclass
class Inputs:
    problem: Problem
    spectrum: np.ndarray   # f32 [nrg_src * nrg_det], index e_src + nrg*nrg_src
    Ifine: np.ndarray      # f32 [nqf * n_mat], index qf + m*nqf
    seg: np.ndarray        # i32 [nx * ny], index x + y*nx, 1-based material id, 0 empty
    a1: np.ndarray         # f32 [nx * ny]
    a2: np.ndarray         # f32 [nx * ny]
    S2: np.ndarray         # f32 [nq * na], index q + a*nq
    q_min: float
    q_max: float
    a_min: float
    a_max: float
    meta: dict = field(default_factory=dict)

    def args(self):
        """Arguments of xrdt_forward / Forward_XRD in prhs order."""
        return (self.spectrum, self.Ifine, self.seg, self.a1, self.a2, self.S2,
                self.q_min, self.q_max, self.a_min, self.a_max)


def _phantom(rng, nx, ny, n_ellipses, n_mat, a1_base, a2_base, density=(0.8, 2.7)):
    x = (np.arange(nx) + 0.5)[:, None] * np.ones((1, ny))
    y = np.ones((nx, 1)) * (np.arange(ny) + 0.5)[None, :]
    seg = np.zeros((nx, ny), np.int32)
    a1 = np.zeros((nx, ny), np.float64)
    a2 = np.zeros((nx, ny), np.float64)
    side = min(nx, ny)
    for _ in range(n_ellipses):
        x0 = rng.uniform(0.15, 0.85) * nx
        y0 = rng.uniform(0.15, 0.85) * ny
        a = rng.uniform(0.05, 0.30) * side
        b = rng.uniform(0.05, 0.30) * side
        t = rng.uniform(0.0, math.pi)
        m = int(rng.integers(1, n_mat + 1))
        rho = rng.uniform(*density)
        u = ((x - x0) * math.cos(t) - (y - y0) * math.sin(t)) / a
        v = ((x - x0) * math.sin(t) + (y - y0) * math.cos(t)) / b
        inside = u * u + v * v < 1.0
        seg[inside] = m
        a1[inside] = rho * a1_base[m - 1]
        a2[inside] = rho * a2_base[m - 1]
    # column-major flatten: index x + y*nx
    return (seg.flatten(order="F"), a1.astype(np.float32).flatten(order="F"),
            a2.astype(np.float32).flatten(order="F"))


def _patterns(rng, p: Problem, n_peaks=6, width=(0.03, 0.08), floor=0.02):
    q = fine_q_grid(p)
    out = np.zeros((p.n_mat, p.nqf), np.float64)
    for m in range(p.n_mat):
        I = np.full_like(q, floor)
        for _ in range(n_peaks):
            c = rng.uniform(p.q_lo, p.q_hi)
            w = rng.uniform(*width)
            h = rng.uniform(0.0, 1.0)
            I += h * np.exp(-0.5 * ((q - c) / w) ** 2)
        out[m] = I
    return out.astype(np.float32).reshape(-1)


def kramers_spectrum(p: Problem, kvp=80.0, lines=((59.3, 0.35), (67.2, 0.12)),
                     total=1.0e9, sub=24):
    """Response matrix spectrum[e_src, nrg_det] (column-major flat).

    Source bin e gets sub-samples E of a Kramers spectrum (kvp - E)/E plus
    Gaussian K lines (relative heights given per line, 0.5 keV wide); each
    photon is spread over detector bins with a Gaussian of width
    0.5*(1.61 + 0.025 E) keV (spectrum_builder.m:65) integrated over the bin.
    """
    dEs = (p.e_src_max - p.e_src_min) / p.nrg_src
    dEd = (p.e_det_max - p.e_det_min) / p.nrg_det
    det_edges = p.e_det_min + dEd * np.arange(p.nrg_det + 1)
    S = np.zeros((p.nrg_src, p.nrg_det), np.float64)
    for e in range(p.nrg_src):
        E = p.e_src_min + dEs * (np.arange(sub) + 0.5) / sub + e * dEs
        N = np.clip(kvp - E, 0.0, None) / E
        for (El, h) in lines:
            N = N + h * np.exp(-0.5 * ((E - El) / 0.5) ** 2) * (kvp / El)
        sig = 0.5 * (1.61 + 0.025 * E)
        z = (det_edges[None, :] - E[:, None]) / (sig[:, None] * math.sqrt(2.0))
        cdf = 0.5 * (1.0 + np.vectorize(math.erf)(z))
        frac = np.diff(cdf, axis=1)                       # [sub, nrg_det]
        S[e] = (N[:, None] * frac).sum(0) * dEs / sub
    S *= total / max(S.sum(), 1e-300)
    return S.astype(np.float32).flatten(order="F")


def hd_spectrum(kvp=80.0, e_min=8.0, de=0.05, n=1440, lines=((59.3, 0.35), (67.2, 0.12)), total=1.0e9):
    """A fine source spectrum in the form spectrum_builder.m:22-30 reads its
    measured one: bin edges [n+1] (keV) and photons per keV [n].  Kramers
    bremsstrahlung (kvp - E)/E plus Gaussian K lines (0.5 keV wide, heights
    relative to the continuum at the line), scaled to total photons; the
    default grid is the reference's 1440 bins of 0.05 keV from 8 to 80 keV."""
    edges = e_min + de * np.arange(n + 1)
    E = 0.5 * (edges[:-1] + edges[1:])
    N = np.clip(kvp - E, 0.0, None) / E
    for (El, h) in lines:
        N = N + h * np.exp(-0.5 * ((E - El) / 0.5) ** 2) * (kvp / El)
    N *= total / max(float((N * de).sum()), 1e-300)
    return edges.astype(np.float32), N.astype(np.float32)


def coherent_table(inp: "Inputs", seed: int = 0) -> np.ndarray:
    """A synthetic coherent cross-section table S1 [NQ, NA] (index q + a*NQ)
    on the 0..255 scale of XSection_builder.m:113-119: the form-factor-like
    fall with the wavevector transfer of coherent scattering, modulated along
    the a-ratio axis, with a little noise and one entry below and one above
    the u8 range."""
    p = inp.problem
    rng = np.random.default_rng(SEED_BASE + 500 + seed)
    qq = np.linspace(0.0, 1.0, p.nq)[:, None]
    aa = np.linspace(0.0, 1.0, p.na)[None, :]
    ph = rng.uniform(0, 2 * math.pi, 2)
    t = np.exp(-2.5 * qq) * (0.75 + 0.2 * np.cos(2.7 * aa + ph[0])) + 0.05 * np.sin(7.0 * qq + ph[1]) * aa
    S = 255.0 * np.clip(t, 0.0, None) + rng.uniform(-0.5, 0.5, (p.nq, p.na))
    S[1, 0] = -2.0
    S[0, -1] = 258.5
    return S.astype(np.float32).flatten(order="F")


def _s2_table(rng, nq, na):
    qq = np.linspace(0.0, 1.0, nq)[:, None]
    aa = np.linspace(0.0, 1.0, na)[None, :]
    ph = rng.uniform(0, 2 * math.pi, 3)
    t = 0.55 + 0.3 * np.sin(3.1 * qq + ph[0]) * np.cos(2.3 * aa + ph[1]) + 0.15 * np.sin(5.0 * qq * aa + ph[2])
    S = 255.0 * t + rng.uniform(-0.5, 0.5, (nq, na))
    S[0, 0] = -3.5      # below range: clamps to 0
    S[-1, -1] = 261.25  # above range: clamps to 255
    return S.astype(np.float32).flatten(order="F")


def make_inputs(p: Problem, seed: int, n_ellipses=6, a1_range=(3e-6, 3e-5),
                a2_range=(0.01, 0.04), q_tab=(-14.0, -2.0), a_tab=(-16.0, -9.0),
                total_photons=1.0e9) -> Inputs:
    rng = np.random.default_rng(seed)
    a1_base = np.exp(rng.uniform(math.log(a1_range[0]), math.log(a1_range[1]), p.n_mat))
    a2_base = np.exp(rng.uniform(math.log(a2_range[0]), math.log(a2_range[1]), p.n_mat))
    seg, a1, a2 = _phantom(rng, p.nx, p.ny, n_ellipses, p.n_mat, a1_base, a2_base)
    Ifine = _patterns(rng, p)
    spectrum = kramers_spectrum(p, total=total_photons)
    S2 = _s2_table(rng, p.nq, p.na)
    return Inputs(p, spectrum, Ifine, seg, a1, a2, S2,
                  f32(q_tab[0]), f32(q_tab[1]), f32(a_tab[0]), f32(a_tab[1]),
                  meta={"seed": seed, "a1_base": a1_base, "a2_base": a2_base})


def scanner(p: Problem, vox_mm: float, r_src_mm: float, r_det_mm: float,
            col_mm: float, row_mm: float = 1.0, z0_mm: float = 10.0,
            focal_mm: float = 0.5) -> Problem:
    """A scanner of the reference's form (integrate_diffraction.cu:84-126),
    centred on the phantom, with lengths given in mm for vox_mm voxels."""
    s = 1.0 / vox_mm
    p.cx, p.cy = p.nx / 2.0, p.ny / 2.0
    p.r_src, p.r_det = r_src_mm * s, r_det_mm * s
    p.src_arc, p.src_phi0 = 2.0 * math.pi, 0.0
    p.col_pitch, p.row_pitch, p.z0 = col_mm * s, row_mm * s, z0_mm * s
    p.focal_spot = focal_mm * s
    p.target_angle = math.radians(30.0)
    p.wedge_angle = math.radians(0.5)
    p.vox_side = 1.0
    return p


def _base(nx, ny, n_src, n_col, n_row, nrg_src, nrg_det, e_src, e_det, dnrg,
          nwt, nqf, n_mat, nq, na, q_range, dq0) -> Problem:
    p = reference_problem(nx, ny)
    p.n_src, p.n_col, p.n_row = n_src, n_col, n_row
    p.nrg_src, p.nrg_det, p.dnrg = nrg_src, nrg_det, dnrg
    p.e_src_min, p.e_src_max = e_src
    p.e_det_min, p.e_det_max = e_det
    p.nwt, p.nqf, p.n_mat, p.nq, p.na = nwt, nqf, n_mat, nq, na
    p.q_lo, p.q_hi = q_range
    p.dq0 = dq0
    p.quirks = QUIRK_STALE_VOXEL_A
    return p


def tiny_problem() -> Problem:
    """A few-second case for exhaustive oracle checks: 12x12 voxels, 4 views,
    8 pixels, 12 energy bins, 32 coarse and 64 fine q bins, 3 materials."""
    p = _base(12, 12, 4, 8, 1, 12, 12, (20.0, 80.0), (20.0, 80.0), 2,
              32, 64, 3, 16, 16, (0.5, 4.0), 0.03)
    return scanner(p, vox_mm=4.0, r_src_mm=150.0, r_det_mm=120.0, col_mm=4.0, row_mm=2.0,
                   z0_mm=12.0, focal_mm=1.0)


def config_problem(index: int) -> Problem:
    """Problems of the five synthetic workloads (sizes in the docstrings of
    the bench).  0: 64^2 phantom, 32 views, 128 px x 32 energy bins, 40-bin
    source spectrum over 20-80 keV; 1: 256^2, 180 views, 512 px x 64 bins,
    8 materials, 128 fine q bins, 32 coarse bins; 2: 128^2 phantom with the
    scanner of 0; 4: one 384^2 slice of the 16-slice stack, 720 views,
    1024 px x 96 bins, 12 materials, 256 fine q bins."""
    if index == 0:
        p = _base(64, 64, 32, 128, 1, 40, 32, (20.0, 80.0), (20.0, 80.0), 5,
                  64, 64, 4, 64, 64, (0.5, 4.0), 0.02)
        return scanner(p, 2.0, 300.0, 200.0, 1.0)
    if index == 1:
        p = _base(256, 256, 180, 512, 1, 64, 64, (20.0, 80.0), (20.0, 80.0), 5,
                  32, 128, 8, 64, 64, (0.5, 4.0), 0.05)
        return scanner(p, 2.0, 600.0, 500.0, 1.0)
    if index == 2:
        p = _base(128, 128, 32, 128, 1, 40, 32, (20.0, 80.0), (20.0, 80.0), 5,
                  32, 64, 4, 64, 64, (0.5, 4.0), 0.05)
        return scanner(p, 2.0, 300.0, 200.0, 1.0)
    if index == 4:
        p = _base(384, 384, 720, 1024, 1, 96, 96, (20.0, 80.0), (20.0, 80.0), 5,
                  32, 256, 12, 64, 64, (0.5, 4.0), 0.05)
        return scanner(p, 1.5, 700.0, 600.0, 0.75)
    raise ValueError(f"no single-phantom problem for config {index}")


def config_inputs(index: int) -> Inputs:
    return make_inputs(config_problem(index), SEED_BASE + index)


def sub_phantom_inputs(side: int = 16, seed: int = SEED_BASE + 20) -> Inputs:
    """A side x side phantom in the scanner of the 128^2 adjoint workload
    (32 views, 128 px x 32 energy bins, 32 coarse bins): the size the adjoint
    is checked on against the oracle."""
    p = config_problem(2).copy(nx=side, ny=side)
    p = scanner(p, 2.0, 300.0, 200.0, 1.0)
    return make_inputs(p, seed, n_ellipses=3)


def vox_truth(inp: Inputs) -> np.ndarray:
    """Per-voxel coarse-q coefficients of the phantom: each non-empty voxel
    carries its material's pattern averaged over the fine bins of each
    coarse bin (wvt_value.cu:8-22 edges), times the voxel's density proxy
    a2 / median(a2).  Layout [NX*NY*NWT], voxel index ix + NX*iy."""
    p = inp.problem
    nw = p.nwt
    k = np.arange(nw + 1, dtype=np.float64)
    a = (p.q_hi - p.q_lo - p.dq0 * nw) / (nw * nw)
    edges = p.q_lo + p.dq0 * k + a * k * k
    qf = p.q_lo + (p.q_hi - p.q_lo) / p.nqf * (np.arange(p.nqf) + 0.5)
    I = np.asarray(inp.Ifine, np.float64).reshape(p.n_mat, p.nqf)
    coarse = np.zeros((p.n_mat, nw))
    for j in range(nw):
        sel = (qf >= edges[j]) & (qf < edges[j + 1])
        if sel.any():
            coarse[:, j] = I[:, sel].mean(axis=1)
        else:
            coarse[:, j] = np.array([np.interp(0.5 * (edges[j] + edges[j + 1]), qf, I[m]) for m in range(p.n_mat)])
    seg = np.asarray(inp.seg).reshape(-1)
    a2 = np.asarray(inp.a2, np.float64).reshape(-1)
    x = np.zeros((seg.size, nw))
    on = seg > 0
    dens = a2[on] / np.median(a2[on]) if on.any() else a2[on]
    x[on] = coarse[seg[on] - 1] * dens[:, None]
    return x.astype(np.float32).reshape(-1)


def batch_inputs(n: int, seed: int = SEED_BASE + 3, side=(64, 384), views=(60, 360), px=(128, 768),
                 nwt: int = 32, nqf: int = 128, nrg: int = 64, n_mat: int = 4) -> list:
    """Independent problems of the batched workload: phantom sides, view
    counts and detector widths drawn uniformly from the given ranges (the
    batched configuration uses 64-384 voxels, 60-360 views, 128-768 px),
    a q grid of nqf fine bins, nrg energy bins, 2 mm voxels, and a fan
    scanner that keeps sources and detectors outside the phantom."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        sd = int(rng.integers(side[0], side[1] + 1))
        nv = int(rng.integers(views[0], views[1] + 1))
        npx = int(rng.integers(px[0], px[1] + 1))
        p = _base(sd, sd, nv, npx, 1, nrg, nrg, (20.0, 80.0), (20.0, 80.0), 5,
                  nwt, nqf, n_mat, 64, 64, (0.5, 4.0), 0.05)
        vox_mm = 2.0
        r_src = 1.5 * sd * vox_mm
        r_det = 1.1 * sd * vox_mm
        col = 2.6 * sd * vox_mm / npx
        p = scanner(p, vox_mm, r_src, r_det, col)
        out.append(make_inputs(p, seed * 1000 + i, n_ellipses=6))
    return out
