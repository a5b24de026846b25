"""Generates the golden fixtures of tests/golden from the reference itself.

Run from the repository root, where the reference sources are present:

    python tests/golden/make_golden.py

It builds oracle/_ref/libxrdt_ref.so (the reference's Forward_projector_kernels
compiled unmodified for the host in FP64, see oracle/ref_emulator.cpp), runs
the reference's device functions and its integrate_diffraction kernel on
seeded synthetic inputs, and stores inputs and outputs:

  ref_helpers.npz   wvt_value for every nwt, find_src_nrg_range for every nrg,
                    GetIntersection on a set of segments (reference config)
  ref_forward_16.npz   integrate_diffraction on a 16x16 phantom, 48 rays
                       (N, C, and the Amatrix rows of 16 of them)
  ref_forward_20x12.npz  the same on a non-square 20x12 phantom, 24 rays

The fixtures hold the inputs too, so the tests do not depend on the synthetic
generators staying unchanged.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402
from xrd_tomography_gb300.problem import reference_problem  # noqa: E402
from xrd_tomography_gb300.synth import make_inputs  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def helpers():
    ref = po.ref_lib()
    cfg = (ctypes.c_int32 * 10)()
    ref.xrdt_ref_config(cfg)
    nwt, nrg = cfg[5], cfg[3]
    q = np.zeros(nwt)
    dq = np.zeros(nwt)
    qq, dd = ctypes.c_double(), ctypes.c_double()
    for n in range(nwt):
        ref.xrdt_ref_wvt_value(n, ctypes.byref(qq), ctypes.byref(dd))
        q[n], dq[n] = qq.value, dd.value
    lo = np.zeros(nrg, np.int32)
    hi = np.zeros(nrg, np.int32)
    a, b = ctypes.c_int32(), ctypes.c_int32()
    for n in range(nrg):
        ref.xrdt_ref_find_src_nrg_range(n, ctypes.byref(a), ctypes.byref(b))
        lo[n], hi[n] = a.value, b.value
    rng = np.random.default_rng(7)
    segs = []
    for nx, ny in ((100, 100), (64, 48), (16, 16)):
        for _ in range(60):
            ang = rng.uniform(0, 2 * np.pi)
            R = rng.uniform(0.9, 3.0) * max(nx, ny)
            x1, y1 = nx / 2 + R * np.cos(ang), ny / 2 + R * np.sin(ang)
            x2, y2 = rng.integers(0, nx) + 0.5, rng.integers(0, ny) + 0.5
            segs.append((x1, y1, x2, y2, nx, ny))
    # corner and edge-grazing cases
    segs += [(-10.0, -10.0, 5.5, 5.5, 16, 16), (-10.0, 8.0, 8.5, 8.0, 16, 16),
             (8.0, -10.0, 8.0, 8.5, 16, 16), (30.0, 30.0, 15.5, 15.5, 16, 16),
             (-5.0, 0.0, 3.5, 0.5, 16, 16), (8.0, 8.0, 9.5, 9.5, 16, 16)]
    segs = np.array(segs, np.float64)
    rx = np.zeros(len(segs))
    ry = np.zeros(len(segs))
    for i, s in enumerate(segs):
        ref.xrdt_ref_get_intersection(ctypes.c_double(s[0]), ctypes.c_double(s[1]),
                                      ctypes.c_double(s[2]), ctypes.c_double(s[3]),
                                      ctypes.c_int32(int(s[4])), ctypes.c_int32(int(s[5])),
                                      ctypes.byref(qq), ctypes.byref(dd))
        rx[i], ry[i] = qq.value, dd.value
    np.savez_compressed(os.path.join(OUT, "ref_helpers.npz"), config=np.array(list(cfg), np.int32),
                        wvt_q=q, wvt_dq=dq, nrg_lo=lo, nrg_hi=hi, segs=segs, int_x=rx, int_y=ry)


def forward(nx, ny, seed, n_rays, n_amatrix, name):
    p = reference_problem(nx, ny)
    inp = make_inputs(p, seed, n_ellipses=4)
    rng = np.random.default_rng(seed + 1)
    rays = np.sort(rng.choice(p.rays, n_rays, replace=False)).astype(np.int64)
    N, C, A = po.ref_forward_rays(inp, rays)
    np.savez_compressed(
        os.path.join(OUT, name), nx=nx, ny=ny, spectrum=inp.spectrum, Ifine=inp.Ifine,
        seg=inp.seg, a1=inp.a1, a2=inp.a2, S2=inp.S2,
        tables=np.array([inp.q_min, inp.q_max, inp.a_min, inp.a_max], np.float32),
        rays=rays, N=N, C=C, A_rays=rays[:n_amatrix], A=A[:n_amatrix])


def main():
    po.build(ref=True)
    helpers()
    forward(16, 16, 1601, 48, 16, "ref_forward_16.npz")
    forward(20, 12, 2012, 24, 8, "ref_forward_20x12.npz")


if __name__ == "__main__":
    main()
