"""Problem description shared by the C ABI, the oracle and the Python API.

`Problem` mirrors `xrdt_problem` of include/xrdt.h field for field (ctypes).
The reference keeps these values as compile-time #defines
(Forward_XRD.cu:16-53) and hard-coded scanner constants
(integrate_diffraction.cu:81-143); here they are runtime fields.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

QUIRK_STALE_VOXEL_A = 0x1

_INT_FIELDS = [
    "nx", "ny", "n_src", "n_col", "n_row", "nrg_src", "nrg_det", "dnrg",
    "nwt", "nqf", "n_mat", "nq", "na",
]
_DOUBLE_FIELDS = [
    "e_src_min", "e_src_max", "e_det_min", "e_det_max",
    "q_lo", "q_hi", "dq0",
    "hbarc", "mec2", "kn0", "kn1", "kn2", "rsqrt2pi", "dq_step",
    "cx", "cy", "r_src", "r_det", "src_arc", "src_phi0",
    "col_pitch", "row_pitch", "z0", "focal_spot", "target_angle",
    "wedge_angle", "vox_side",
]


class Problem(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int32) for n in _INT_FIELDS]
                + [("quirks", ctypes.c_uint32), ("reserved0", ctypes.c_int32)]
                + [(n, ctypes.c_double) for n in _DOUBLE_FIELDS])

    # ---- derived sizes -------------------------------------------------
    @property
    def n_det(self) -> int:
        return self.n_col * self.n_row

    @property
    def rays(self) -> int:
        return self.n_src * self.n_det * self.nrg_det

    @property
    def amatrix_elems(self) -> int:
        return self.nwt * self.n_mat * self.rays

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}

    def copy(self, **overrides) -> "Problem":
        q = Problem()
        ctypes.pointer(q)[0] = self
        for k, v in overrides.items():
            setattr(q, k, v)
        return q

    def __repr__(self) -> str:  # pragma: no cover - debugging aid
        return "Problem(%s)" % ", ".join(f"{k}={v}" for k, v in self.as_dict().items())


def f32(x: float) -> float:
    """Value of a float-suffixed literal of the reference (float-rounded)."""
    return float(np.float32(x))


def reference_problem(nx: int = 100, ny: int | None = None) -> Problem:
    """The reference's compiled configuration for an nx x ny phantom.

    Dimensions: Forward_XRD.cu:17-25,47-48.  Constants: Forward_XRD.cu:34-53,
    integrate_diffraction.cu:117,126,278.  Scanner: integrate_diffraction.cu:81-128,
    every length scaled by mm_over_vox = NX/100 (:81) and evaluated in double
    from the float-rounded literals, the way the FP64 oracle evaluates them.
    Must agree with xrdt_problem_reference() of the C library.
    """
    ny = nx if ny is None else ny
    p = Problem()
    p.nx, p.ny = nx, ny
    p.n_src, p.n_col, p.n_row = 32, 1024, 1
    p.nrg_src = p.nrg_det = 64
    p.dnrg = 5
    p.nwt, p.nqf, p.n_mat = 256, 768, 3
    p.nq, p.na = 64, 64
    p.quirks = QUIRK_STALE_VOXEL_A
    p.e_src_min = p.e_det_min = 8.0
    p.e_src_max = p.e_det_max = 80.0
    p.q_lo, p.q_hi, p.dq0 = f32(0.5), f32(6.0), f32(0.01)
    p.hbarc = f32(1.973269804)
    p.mec2 = f32(510.99895)
    p.kn0, p.kn1, p.kn2 = f32(0.751691286166726), f32(1.4599683207703), f32(-0.64597532690936)
    p.rsqrt2pi = f32(0.398942280401433)
    p.dq_step = 0.25
    mmv = float(nx) / 100.0
    Lx = 200.0 * mmv
    Ly = 200.0 * mmv
    p.cx, p.cy = Lx / 2.0, Ly / 2.0
    p.r_src, p.r_det = 150.0 * mmv, 170.0 * mmv
    p.src_arc, p.src_phi0 = f32(6.28318530717959), 0.0
    p.col_pitch, p.row_pitch, p.z0 = 0.5 * mmv, 1.0 * mmv, 10.0 * mmv
    p.focal_spot = 0.5 * mmv
    p.target_angle = f32(0.523598775598299)
    p.wedge_angle = f32(0.00872664625997165)
    p.vox_side = 1.0
    return p


def coarse_q_grid(p: Problem) -> tuple[np.ndarray, np.ndarray]:
    """Centres and widths of the NWT parabolic q bins (wvt_value.cu:8-22)."""
    n = np.arange(p.nwt, dtype=np.float64)
    NWT = float(p.nwt)
    c = p.q_hi - p.q_lo - p.dq0 * NWT
    e1 = p.q_lo + n * p.dq0 + c * (n * n) / (NWT * NWT)
    e2 = p.q_lo + (n + 1) * p.dq0 + c * ((n + 1) * (n + 1)) / (NWT * NWT)
    return 0.5 * (e1 + e2), e2 - e1


def fine_q_grid(p: Problem) -> np.ndarray:
    """Fine q-axis of Ifine (integrate_diffraction.cu:302)."""
    dq = (p.q_hi - p.q_lo) / p.nqf
    return p.q_lo + dq * (0.5 + np.arange(p.nqf, dtype=np.float64))


def src_nrg_range(p: Problem, nrg: int) -> tuple[int, int]:
    """find_src_nrg_range.cu:8-25 generalised to two energy grids."""
    if (p.nrg_src == p.nrg_det and p.e_src_min == p.e_det_min
            and p.e_src_max == p.e_det_max):
        c = nrg
    else:
        dEs = (p.e_src_max - p.e_src_min) / p.nrg_src
        dEd = (p.e_det_max - p.e_det_min) / p.nrg_det
        c = int(math.floor((p.e_det_min + (nrg + 0.5) * dEd - p.e_src_min) / dEs))
    lo = max(0, c - p.dnrg)
    hi = lo + 2 * p.dnrg
    if hi >= p.nrg_src:
        hi = p.nrg_src - 1
        lo = hi - 2 * p.dnrg
    return lo, hi
