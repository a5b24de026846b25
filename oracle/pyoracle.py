"""ctypes front end of the CPU checker (test infrastructure only).

Loads oracle/liboracle.so (the FP64 restatement, xrdt_oracle.c) and, when it
was built, oracle/_ref/libxrdt_ref.so (the reference's kernel files compiled
for the host).  Only the tests, the smoke check and bench.py's CPU-baseline
leg use this module; the product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libxrdt_ref.so")
# the reference checkout beside the repository, or $XRDT_REF_SRC
REF_ROOT = os.environ.get("XRDT_REF_SRC") or os.path.abspath(os.path.join(HERE, "..", "..", "reference"))
REF_SRC = os.path.join(REF_ROOT, "Forward_projector_kernels")

_f = ctypes.POINTER(ctypes.c_float)
_d = ctypes.POINTER(ctypes.c_double)
_i32 = ctypes.POINTER(ctypes.c_int32)
_i64 = ctypes.POINTER(ctypes.c_int64)


def build(ref: bool | None = None) -> None:
    """Compiles the oracle (and the reference build when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref is None:
        ref = os.path.isdir(REF_SRC)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REF_ROOT], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(ref=False)
        _lib = ctypes.CDLL(LIB)
        _lib.xrdt_oracle_forward_rays.restype = ctypes.c_int32
        _lib.xrdt_oracle_vox_rays.restype = ctypes.c_int32
        _lib.xrdt_oracle_ct_rays.restype = ctypes.c_int32
        _lib.xrdt_oracle_decisions.restype = ctypes.c_int32
        _lib.xrdt_oracle_forward_tables.restype = ctypes.c_int32
        _lib.xrdt_oracle_attenuator.restype = ctypes.c_int64
        _lib.xrdt_oracle_get_intersection.restype = ctypes.c_int32
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref_lib():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_LIB)
        _ref.xrdt_ref_integrate_diffraction.restype = ctypes.c_int32
    return _ref


def _fp(a):
    return np.ascontiguousarray(a, np.float32).ctypes.data_as(_f)


def forward_rays(inp, rays, want_a=False, want_av=False, threads=0):
    """Oracle Nphotons, Cphotons (and Amatrix rows [n, MAT, NWT], per-voxel
    rows [n, NX*NY, NWT]) for the given linear ray indices, in FP64."""
    p = inp.problem
    rays = np.ascontiguousarray(rays, np.int64)
    n = rays.size
    N = np.zeros(n)
    C = np.zeros(n)
    A = np.zeros((n, p.n_mat, p.nwt)) if want_a else None
    Av = np.zeros((n, p.nx * p.ny, p.nwt)) if want_av else None
    keep = [np.ascontiguousarray(x, np.float32) for x in (inp.spectrum, inp.Ifine, inp.a1, inp.a2, inp.S2)]
    seg = np.ascontiguousarray(inp.seg, np.int32)
    rc = lib().xrdt_oracle_forward_rays(
        ctypes.byref(p), keep[0].ctypes.data_as(_f), keep[1].ctypes.data_as(_f),
        seg.ctypes.data_as(_i32), keep[2].ctypes.data_as(_f), keep[3].ctypes.data_as(_f),
        keep[4].ctypes.data_as(_f), ctypes.c_float(inp.q_min), ctypes.c_float(inp.q_max),
        ctypes.c_float(inp.a_min), ctypes.c_float(inp.a_max),
        rays.ctypes.data_as(_i64), ctypes.c_int64(n), N.ctypes.data_as(_d), C.ctypes.data_as(_d),
        A.ctypes.data_as(_d) if A is not None else None,
        Av.ctypes.data_as(_d) if Av is not None else None, ctypes.c_int32(threads))
    if rc != 0:
        raise ValueError("oracle rejected the input (material id above n_mat)")
    return N, C, A, Av


def forward_tables(inp, S1, rays, bilinear=False, threads=0):
    """Oracle Nphotons (coherent term from the S1 table) and Cphotons of the
    cross-section table path for the listed rays, in FP64; nearest-bin
    lookups, or bilinear ones."""
    p = inp.problem
    rays = np.ascontiguousarray(rays, np.int64)
    n = rays.size
    N = np.zeros(n)
    C = np.zeros(n)
    keep = [np.ascontiguousarray(x, np.float32) for x in (inp.spectrum, inp.a1, inp.a2, S1, inp.S2)]
    seg = np.ascontiguousarray(inp.seg, np.int32)
    rc = lib().xrdt_oracle_forward_tables(
        ctypes.byref(p), keep[0].ctypes.data_as(_f), seg.ctypes.data_as(_i32), keep[1].ctypes.data_as(_f),
        keep[2].ctypes.data_as(_f), keep[3].ctypes.data_as(_f), keep[4].ctypes.data_as(_f),
        ctypes.c_float(inp.q_min), ctypes.c_float(inp.q_max), ctypes.c_float(inp.a_min), ctypes.c_float(inp.a_max),
        ctypes.c_int32(1 if bilinear else 0), rays.ctypes.data_as(_i64), ctypes.c_int64(n),
        N.ctypes.data_as(_d), C.ctypes.data_as(_d), ctypes.c_int32(threads))
    if rc != 0:
        raise ValueError("oracle rejected the input")
    return N, C


def decisions(inp, rays, threads=0):
    """The integer decisions of the FP64 forward for the listed rays: a dict
    of win [n, 2], walk [n, nv, 4] (detector samples, detector edge, source
    samples, source edge), nq [n, nv, 2*dnrg+1], na [nv] and s2u8 [nq*na];
    non-empty voxels in the reference's loop order."""
    p = inp.problem
    rays = np.ascontiguousarray(rays, np.int64)
    n = rays.size
    seg = np.ascontiguousarray(inp.seg, np.int32)
    nv = int((seg > 0).sum())
    W = 2 * p.dnrg + 1
    out = {"win": np.zeros((n, 2), np.int32), "walk": np.zeros((n, nv, 4), np.int32),
           "nq": np.zeros((n, nv, W), np.int32), "na": np.zeros(max(nv, 1), np.int32),
           "s2u8": np.zeros(p.nq * p.na, np.uint8)}
    keep = [np.ascontiguousarray(x, np.float32) for x in (inp.spectrum, inp.Ifine, inp.a1, inp.a2, inp.S2)]
    rc = lib().xrdt_oracle_decisions(
        ctypes.byref(p), keep[0].ctypes.data_as(_f), keep[1].ctypes.data_as(_f), seg.ctypes.data_as(_i32),
        keep[2].ctypes.data_as(_f), keep[3].ctypes.data_as(_f), keep[4].ctypes.data_as(_f),
        ctypes.c_float(inp.q_min), ctypes.c_float(inp.q_max), ctypes.c_float(inp.a_min), ctypes.c_float(inp.a_max),
        rays.ctypes.data_as(_i64), ctypes.c_int64(n), out["win"].ctypes.data_as(_i32),
        out["walk"].ctypes.data_as(_i32), out["na"].ctypes.data_as(_i32), out["nq"].ctypes.data_as(_i32),
        out["s2u8"].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), ctypes.c_int32(threads))
    if rc != 0:
        raise ValueError("oracle rejected the input (material id above n_mat)")
    out["na"] = out["na"][:nv]
    return out


def vox_rays(inp, rays, x=None, w=None, threads=0):
    """The per-voxel-coefficient model of the given rays in FP64.

    x: coefficients [NY, NX, NWT] (C order; voxel index nx + ny*NX, the layout
    of the library's per-voxel operator) -> y[i] = sum Av[rays[i]] * x.
    w: weights [n_rays] -> g[NY, NX, NWT] = sum_i w[i] Av[rays[i]].
    Returns (y, g); an entry is None when its input was not given."""
    p = inp.problem
    rays = np.ascontiguousarray(rays, np.int64)
    n = rays.size
    xd = None if x is None else np.ascontiguousarray(x, np.float64).reshape(-1)
    wd = None if w is None else np.ascontiguousarray(w, np.float64).reshape(-1)
    if xd is not None and xd.size != p.nx * p.ny * p.nwt:
        raise ValueError("x must hold nx*ny*nwt coefficients")
    if wd is not None and wd.size != n:
        raise ValueError("w must hold one weight per ray")
    y = np.zeros(n) if xd is not None else None
    g = np.zeros(p.nx * p.ny * p.nwt) if wd is not None else None
    keep = [np.ascontiguousarray(a, np.float32) for a in (inp.spectrum, inp.a1, inp.a2)]
    seg = np.ascontiguousarray(inp.seg, np.int32)
    rc = lib().xrdt_oracle_vox_rays(
        ctypes.byref(p), keep[0].ctypes.data_as(_f), seg.ctypes.data_as(_i32), keep[1].ctypes.data_as(_f),
        keep[2].ctypes.data_as(_f), xd.ctypes.data_as(_d) if xd is not None else None,
        wd.ctypes.data_as(_d) if wd is not None else None, rays.ctypes.data_as(_i64), ctypes.c_int64(n),
        y.ctypes.data_as(_d) if y is not None else None, g.ctypes.data_as(_d) if g is not None else None,
        ctypes.c_int32(threads))
    if rc != 0:
        raise ValueError(f"oracle rejected the input ({rc})")
    return y, (None if g is None else g.reshape(p.ny, p.nx, p.nwt))


def ct_rays(inp, rays, threads=0):
    """(Tphotons, gain0) of the CT sinogram for the listed rays, in FP64."""
    p = inp.problem
    rays = np.ascontiguousarray(rays, np.int64)
    T = np.zeros(rays.size)
    G = np.zeros(rays.size)
    keep = [np.ascontiguousarray(a, np.float32) for a in (inp.spectrum, inp.a1, inp.a2)]
    lib().xrdt_oracle_ct_rays(ctypes.byref(p), keep[0].ctypes.data_as(_f), keep[1].ctypes.data_as(_f),
                              keep[2].ctypes.data_as(_f), rays.ctypes.data_as(_i64), ctypes.c_int64(rays.size),
                              T.ctypes.data_as(_d), G.ctypes.data_as(_d), ctypes.c_int32(threads))
    return T, G


def ref_forward_rays(inp, rays, threads=0):
    """The reference's own integrate_diffraction, compiled for the host in
    FP64, on the given rays.  Only for problems equal to the compiled
    configuration (SRC=32, COL=1024, ROW=1, NRG=64, NWT=256, NQF=768, MAT=3,
    NQ=NA=64)."""
    p = inp.problem
    cfg = (ctypes.c_int32 * 10)()
    ref_lib().xrdt_ref_config(cfg)
    want = [p.n_src, p.n_col, p.n_row, p.nrg_det, p.dnrg, p.nwt, p.nqf, p.n_mat, p.nq, p.na]
    if list(cfg) != want or p.nrg_src != p.nrg_det:
        raise ValueError(f"reference build is configured for {list(cfg)}, problem has {want}")
    rays = np.ascontiguousarray(rays, np.int64)
    n = rays.size
    N = np.zeros(n)
    C = np.zeros(n)
    A = np.zeros((n, p.n_mat, p.nwt))
    keep = [np.ascontiguousarray(x, np.float32) for x in (inp.spectrum, inp.Ifine, inp.a1, inp.a2, inp.S2)]
    seg = np.ascontiguousarray(inp.seg, np.int32)
    failed = ref_lib().xrdt_ref_integrate_diffraction(
        keep[0].ctypes.data_as(_f), keep[1].ctypes.data_as(_f), seg.ctypes.data_as(_i32),
        keep[2].ctypes.data_as(_f), keep[3].ctypes.data_as(_f), keep[4].ctypes.data_as(_f),
        ctypes.c_int32(p.nx), ctypes.c_int32(p.ny),
        ctypes.c_float(inp.q_min), ctypes.c_float(inp.q_max), ctypes.c_float(inp.a_min),
        ctypes.c_float(inp.a_max), rays.ctypes.data_as(_i64), ctypes.c_int64(n),
        N.ctypes.data_as(_d), C.ctypes.data_as(_d), A.ctypes.data_as(_d),
        ctypes.c_int32(threads or os.cpu_count()))
    if failed:
        raise RuntimeError(f"{failed} emulated blocks did not complete")
    return N, C, A


def wvt_value(p, nwt):
    q, dq = ctypes.c_double(), ctypes.c_double()
    lib().xrdt_oracle_wvt_value(ctypes.byref(p), ctypes.c_int32(nwt), ctypes.byref(q), ctypes.byref(dq))
    return q.value, dq.value


def src_nrg_range(p, nrg):
    lo, hi = ctypes.c_int32(), ctypes.c_int32()
    lib().xrdt_oracle_src_nrg_range(ctypes.byref(p), ctypes.c_int32(nrg), ctypes.byref(lo), ctypes.byref(hi))
    return lo.value, hi.value


def get_intersection(x1, y1, x2, y2, nx, ny):
    rx, ry = ctypes.c_double(), ctypes.c_double()
    lib().xrdt_oracle_get_intersection(ctypes.c_double(x1), ctypes.c_double(y1), ctypes.c_double(x2),
                                       ctypes.c_double(y2), ctypes.c_int32(nx), ctypes.c_int32(ny),
                                       ctypes.byref(rx), ctypes.byref(ry))
    return rx.value, ry.value


def attenuator(inp, ex, ey, vx, vy):
    p = inp.problem
    a1 = np.ascontiguousarray(inp.a1, np.float32)
    a2 = np.ascontiguousarray(inp.a2, np.float32)
    A1, A2 = ctypes.c_double(), ctypes.c_double()
    n = lib().xrdt_oracle_attenuator(ctypes.byref(p), a1.ctypes.data_as(_f), a2.ctypes.data_as(_f),
                                     ctypes.c_double(ex), ctypes.c_double(ey), ctypes.c_double(vx),
                                     ctypes.c_double(vy), ctypes.byref(A1), ctypes.byref(A2))
    return A1.value, A2.value, n
