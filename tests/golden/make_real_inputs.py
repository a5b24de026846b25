"""Extracts the reference's measured inputs from its MATLAB data files into
tests/golden/real_inputs.npz, read by xrd_tomography_gb300.matfile (the
MAT-file reader this fixture also pins: tests/test_matfile.py reads the same
files again when the reference tree is present and compares).

Run from the repository root, with the reference checkout beside the
repository (or XRDT_REF_SRC naming it):

    python tests/golden/make_real_inputs.py

Stored arrays:
  spectrum_energy, spectrum_counts  Spectrum_80kVp/spectral_data_HD.mat, the
                                    fine 80 kVp source spectrum that
                                    spectrum_builder.m:9-30 loads
  D_<material>                      open_source_data/<material>.mat, the
                                    measured patterns [2-theta (deg),
                                    intensity] that XRD_builder.m loads
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from xrd_tomography_gb300.matfile import load_mat  # noqa: E402

REF = os.environ.get("XRDT_REF_SRC") or os.path.abspath(os.path.join(ROOT, "..", "reference"))
MATERIALS = ("cellulose", "TNT", "ammoniumnitrate", "aluminum_alloy")


def main():
    out = {}
    s = load_mat(os.path.join(REF, "Spectrum_80kVp", "spectral_data_HD.mat"))["spectrum"]
    out["spectrum_energy"] = np.asarray(s["energy"], np.float64).ravel()
    out["spectrum_counts"] = np.asarray(s["counts"], np.float64).ravel()
    for m in MATERIALS:
        out["D_" + m] = np.asarray(load_mat(os.path.join(REF, "open_source_data", m + ".mat"))["D"], np.float64)
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "real_inputs.npz"), **out)


if __name__ == "__main__":
    main()
