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
    first sample past that cell's exit edge (at least one)."""
    R = R + (n - 1) * L
    L = -L
    inv = [(-1.0 / c if abs(c) > 1e-4 else (1e4 if c < 0 else -1e4)) for c in L]
    hinv = [(0.5 * inv[a] if L[a] < 0 else -0.5 * inv[a]) for a in range(2)]
    acc, k0, steps = 0.0, 0, 0
    while k0 < n:
        P0 = R + k0 * L
        ix, iy = int(np.rint(P0[0])), int(np.rint(P0[1]))
        u0, v0 = P0[0] - ix, P0[1] - iy
        s = min(u0 * inv[0] + hinv[0], v0 * inv[1] + hinv[1])
        m = int(min(max(np.rint(s + 0.5), 1), n - k0))
        S1 = 0.5 * m * (m - 1)
        S2 = S1 * (2 * m - 1) / 3.0
        su, sv = m * u0 + L[0] * S1, m * v0 + L[1] * S1
        suv = m * u0 * v0 + (u0 * L[1] + v0 * L[0]) * S1 + L[0] * L[1] * S2
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
