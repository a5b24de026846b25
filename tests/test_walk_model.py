"""The algebra of the cell-by-cell walk (walk_cells in walk.cuh, used by
k_det_walk): the samples of a run inside one bilinear cell add up in closed
form, so stepping cell by cell gives the per-sample sum of the attenuator
(attenuator.cu:9-109) up to rounding.  A numpy restatement of the stepping
rule is checked against per-sample sums, including axis-aligned and diagonal
rays whose samples land on cell edges.  (The CUDA walk itself is checked
against the oracle in the GPU tests.)"""
import math

import numpy as np

NX = NY = 40


def cell_coeffs(f, ix, iy):
    """Centre-frame coefficients of cell (ix+1, iy+1) of the zero-bordered
    map f (the layout k_build_cells writes)."""
    ci, cj = min(max(ix + 1, 0), NX), min(max(iy + 1, 0), NY)
    def tex(i, j):
        return f[j, i] if 0 <= i < NX and 0 <= j < NY else 0.0
    f00, f10, f01, f11 = tex(ci - 1, cj - 1), tex(ci, cj - 1), tex(ci - 1, cj), tex(ci, cj)
    return (0.25 * (f00 + f10 + f01 + f11), 0.5 * ((f10 - f00) + (f11 - f01)),
            0.5 * ((f01 - f00) + (f11 - f10)), (f11 - f01) - (f10 - f00))


def sample(f, P):
    ix, iy = int(np.rint(P[0])), int(np.rint(P[1]))
    c00, c10, c01, c11 = cell_coeffs(f, ix, iy)
    u, v = P[0] - ix, P[1] - iy
    return c00 + c10 * u + c01 * v + c11 * u * v


def walk_samples(f, R, L, n):
    return sum(sample(f, R + k * L) for k in range(n))


def walk_cells(f, R, L, n):
    """The stepping rule of walk_cells: from the last sample back to the
    first, each step takes the cell of its first sample and the run up to the
    first sample past that cell's exit edge (at least one).  Positions are
    anchored at the voxel end: sample j from the last sits at
    v + (dlt + j DQ) u, with v the point one step past the last sample in
    this restatement."""
    DQ = float(np.hypot(*L))
    u = -L / DQ
    v = R + (n - 1) * L - 0.3 * DQ * u          # the voxel lies beyond the last sample
    dlt = 0.3 * DQ
    Ls = u * DQ
    inv = [(-1.0 / c if abs(c) > 1e-4 else (1e4 if c < 0 else -1e4)) for c in Ls]
    hinv = [(0.5 * inv[a] if Ls[a] < 0 else -0.5 * inv[a]) for a in range(2)]
    acc, k0, steps = 0.0, 0, 0
    while k0 < n:
        P0 = v + (dlt + k0 * DQ) * u
        ix, iy = int(np.rint(P0[0])), int(np.rint(P0[1]))
        u0, v0 = P0[0] - ix, P0[1] - iy
        s = min(u0 * inv[0] + hinv[0], v0 * inv[1] + hinv[1])
        m = int(min(max(np.rint(s + 0.5), 1), n - k0))
        S1 = 0.5 * m * (m - 1)
        S2 = S1 * (2 * m - 1) / 3.0
        su, sv = m * u0 + Ls[0] * S1, m * v0 + Ls[1] * S1
        suv = m * u0 * v0 + (u0 * Ls[1] + v0 * Ls[0]) * S1 + Ls[0] * Ls[1] * S2
        c00, c10, c01, c11 = cell_coeffs(f, ix, iy)
        acc += m * c00 + c10 * su + c01 * sv + c11 * suv
        k0 += m
        steps += 1
    return acc, steps


def test_cell_walk_equals_sample_sums():
    rng = np.random.default_rng(5)
    f = rng.uniform(0.0, 1.0, (NY, NX))
    f[rng.uniform(size=f.shape) < 0.3] = 0.0          # empty space and sharp edges
    n_total = steps_total = 0
    worst = 0.0
    for trial in range(600):
        th = rng.uniform(0, 2 * math.pi) if trial % 5 else rng.integers(0, 8) * math.pi / 4
        L = 0.25 * np.array([math.cos(th), math.sin(th)])
        R = rng.uniform(0, NX - 1, 2)
        if trial % 7 == 0:
            R = np.rint(R) + 0.5                     # samples on cell edges
        n = int(rng.integers(1, 120))
        end = R + n * L
        if not (-1 <= end[0] <= NX - 1 and -1 <= end[1] <= NY - 1):
            continue
        a = walk_samples(f, R, L, n)
        b, steps = walk_cells(f, R, L, n)
        worst = max(worst, abs(a - b) / max(abs(a), 1e-12))
        n_total += n
        steps_total += steps
    assert worst < 1e-12
    # about one cell load per 3 samples at DQ = 1/4 voxel
    assert 2.5 < n_total / steps_total < 4.0


# ---- FP32 accuracy of the anchored offsets ----------------------------------

f32 = np.float32


def fma32(a, b, c):
    """fmaf: the float64 product of two floats is exact."""
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum32(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def anchored_offset32(vx, dlt, u, k0, DQ):
    """walk_cells' cell centre and offset along one axis in FP32: the
    distance dlt + k0 DQ and its product with u formed without error."""
    kq = f32(f32(k0) * f32(DQ))
    kqe = fma32(k0, DQ, -kq)
    sh, e1 = two_sum32(f32(dlt[0]), kq)
    sl = f32(e1 + f32(kqe + f32(dlt[1])))
    px = f32(sh * f32(u[0]))
    ex = f32(fma32(sh, u[0], -px) + fma32(sh, u[1], f32(sl * f32(u[0]))))
    r = f32(np.rint(f32(vx + px)))
    return r, f32(f32(f32(vx - r) + px) + ex)


def split(x):
    hi = f32(x)
    return (hi, f32(x - np.float64(hi)))


def test_anchored_offsets_hold_1e7_at_a_256_voxel_map():
    """Sample positions hundreds of voxels from the origin: the anchored
    offsets from their cell centres stay within a few 1e-8 voxel of the FP64
    positions (a position formed directly in FP32 is off by up to ulp(256)/2
    = 1.5e-5), and the cell choice is the nearest centre or a neighbour whose
    offset just exceeds one half."""
    rng = np.random.default_rng(7)
    worst = 0.0
    for _ in range(4000):
        vx = rng.integers(0, 256) + 0.5
        th = rng.uniform(0, 2 * math.pi)
        u = math.cos(th)
        n = int(rng.integers(1, 1400))
        dlt = rng.uniform(0, 0.25)
        k0 = int(rng.integers(0, n))
        x = vx + (dlt + k0 * 0.25) * u              # FP64 position
        r, d = anchored_offset32(f32(vx), split(dlt), split(u), k0, 0.25)
        worst = max(worst, abs(float(r) + float(d) - x))
        assert abs(float(d)) < 0.5 + 1e-4
    assert worst < 1e-7, worst
