"""Python front end of libxrdt.so, mirroring the reference's MEX interface.

`Forward_XRD(spectrum, Ifine, seg, a1, a2, S2, q_min, q_max, a_min, a_max)`
takes the ten arguments of the MATLAB call (main.m:56-64, Forward_XRD.cu:82-110)
and returns (Nphotons, Cphotons, Amatrix) shaped [SRC, COL, ROW, NRG] and
[NWT, MAT, SRC, COL, ROW, NRG] in column-major order, as
mxGPUCreateGPUArray lays them out (Forward_XRD.cu:143-166).

Arrays may be numpy arrays (host memory) or torch tensors on the GPU; the
library decides per pointer.  There is no CPU fallback: if libxrdt.so is
missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import weakref

import numpy as np

from .problem import Problem, reference_problem

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libxrdt.so")

FWD_PLAIN_FP64 = 0x1
FWD_NO_SYNC = 0x2
TAB_BILINEAR = 0x4
OP_PLAIN_FP64 = 0x1
(KERNEL_PREP_MAP, KERNEL_PREP_VOXELS, KERNEL_SRC_ATTEN, KERNEL_FORWARD, KERNEL_PLAIN, KERNEL_GATHER,
 KERNEL_MLEM, KERNEL_VOX_FORWARD, KERNEL_VOX_ADJOINT, KERNEL_VOX_UPDATE, KERNEL_CT, KERNEL_BASIS, KERNEL_WALK, KERNEL_SPECTRUM) = range(14)

_P = ctypes.POINTER(Problem)
_vp = ctypes.c_void_p

# name -> (restype, argtypes); must match include/xrdt.h
SIGNATURES = {
    "xrdt_abi_version": (ctypes.c_int32, []),
    "xrdt_status_string": (ctypes.c_char_p, [ctypes.c_int32]),
    "xrdt_problem_reference": (ctypes.c_int32, [_P, ctypes.c_int32, ctypes.c_int32]),
    "xrdt_problem_validate": (ctypes.c_int32, [_P]),
    "xrdt_problem_rays": (ctypes.c_int64, [_P]),
    "xrdt_problem_amatrix_elems": (ctypes.c_int64, [_P]),
    "xrdt_ctx_create": (ctypes.c_int32, [ctypes.POINTER(_vp), ctypes.c_int32, _vp]),
    "xrdt_ctx_destroy": (ctypes.c_int32, [_vp]),
    "xrdt_ctx_synchronize": (ctypes.c_int32, [_vp]),
    "xrdt_last_error": (ctypes.c_char_p, [_vp]),
    "xrdt_ctx_launch_count": (ctypes.c_int64, [_vp]),
    "xrdt_ctx_set_profiling": (ctypes.c_int32, [_vp, ctypes.c_int32]),
    "xrdt_ctx_kernel_stats": (ctypes.c_int32, [_vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64),
                                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]),
    "xrdt_forward": (ctypes.c_int32, [_vp, _P, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, ctypes.c_float, _vp, _vp, _vp, ctypes.c_uint32]),
    "xrdt_forward_tables": (ctypes.c_int32, [_vp, _P, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float,
                                             ctypes.c_float, ctypes.c_float, _vp, _vp, ctypes.c_uint32]),
    "xrdt_mlem_matrix": (ctypes.c_int32, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp, _vp, ctypes.c_int32,
                                          ctypes.c_uint32]),
    "xrdt_mlem_matrix_noalloc": (ctypes.c_int32, [_vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp, _vp, ctypes.c_int32,
                                                  _vp]),
    "xrdt_op_create": (ctypes.c_int32, [_vp, _P, _vp, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "xrdt_op_destroy": (ctypes.c_int32, [_vp]),
    "xrdt_op_voxels": (ctypes.c_int64, [_vp]),
    "xrdt_op_walk_bytes": (ctypes.c_int64, [_vp]),
    "xrdt_op_forward": (ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_uint32]),
    "xrdt_op_adjoint": (ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_uint32]),
    "xrdt_op_mlem": (ctypes.c_int32, [_vp, _vp, _vp, _vp, ctypes.c_int32, ctypes.c_uint32]),
    "xrdt_op_forward_rays": (ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_int64, _vp, ctypes.c_uint32]),
    "xrdt_basis_expand": (ctypes.c_int32, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp, ctypes.c_int32, _vp,
                                           ctypes.c_uint32]),
    "xrdt_ct_sinogram": (ctypes.c_int32, [_vp, _P, _vp, _vp, _vp, _vp, _vp, ctypes.c_uint32]),
    "xrdt_spectrum_build": (ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_int32, _vp, ctypes.c_int32, _vp, ctypes.c_int32,
                                             ctypes.c_double, ctypes.c_double, _vp, ctypes.c_uint32]),
    "xrdt_batch_create": (ctypes.c_int32, [_vp, _vp, ctypes.c_int32, ctypes.POINTER(_vp)]),
    "xrdt_batch_destroy": (ctypes.c_int32, [_vp]),
    "xrdt_batch_forward": (ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_uint32]),
    "xrdt_batch_adjoint": (ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_uint32]),
    "xrdt_batch_mlem": (ctypes.c_int32, [_vp, _vp, _vp, _vp, ctypes.c_int32, ctypes.c_uint32]),
    "xrdt_batch_tune": (ctypes.c_int32, [_vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64),
                                         ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "xrdt_op_adjoint_rays": (ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_int64, _vp, ctypes.c_uint32]),
    "xrdt_bop_create": (ctypes.c_int32, [_vp, _vp, ctypes.c_int32, ctypes.POINTER(_vp)]),
    "xrdt_bop_destroy": (ctypes.c_int32, [_vp]),
    "xrdt_bop_forward": (ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_uint32]),
    "xrdt_bop_adjoint": (ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_uint32]),
    "xrdt_bop_mlem": (ctypes.c_int32, [_vp, _vp, _vp, _vp, ctypes.c_int32, ctypes.c_uint32]),
    "xrdt_mlem_checkpoint_write": (ctypes.c_int32, [ctypes.c_char_p, _vp, ctypes.c_int64, ctypes.c_int64]),
    "xrdt_mlem_checkpoint_read": (ctypes.c_int32, [ctypes.c_char_p, _vp, ctypes.c_int64,
                                                   ctypes.POINTER(ctypes.c_int64)]),
    "xrdt_debug_decisions": (ctypes.c_int32, [_vp, _P, _vp, _vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float,
                                              ctypes.c_float, ctypes.c_float, _vp, ctypes.c_int64, _vp, _vp, _vp,
                                              _vp, _vp, ctypes.POINTER(ctypes.c_int64)]),
    "xrdt_forward_rays": (ctypes.c_int32, [_vp, _P, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_float,
                                           ctypes.c_float, ctypes.c_float, ctypes.c_float, _vp, ctypes.c_int64,
                                           _vp, _vp, _vp, ctypes.c_uint32]),
}


class XrdtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"xrdt status {status}: {msg}")
        self.status = status


_lib = None


def lib():
    """Loads libxrdt.so (building it first if the CUDA toolkit is present)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build
            build.build()
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc: int, ctx=None):
    if rc != 0:
        msg = ""
        if ctx is not None:
            msg = (lib().xrdt_last_error(ctx) or b"").decode()
        if not msg:
            msg = lib().xrdt_status_string(rc).decode()
        raise XrdtError(rc, msg)


def c_reference_problem(nx: int, ny: int | None = None) -> Problem:
    p = Problem()
    _check(lib().xrdt_problem_reference(ctypes.byref(p), nx, nx if ny is None else ny))
    return p


def validate(p: Problem) -> int:
    return lib().xrdt_problem_validate(ctypes.byref(p))


class Context:
    """An xrdt_ctx bound to one device and stream (stream=None: its own)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        h = _vp()
        _check(lib().xrdt_ctx_create(ctypes.byref(h), device, _vp(stream) if stream else None))
        self.h = h
        self._operators = weakref.WeakSet()   # destroyed before the context

    def close(self):
        if self.h:
            for op in list(self._operators):
                op.close()
            lib().xrdt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        _check(lib().xrdt_ctx_synchronize(self.h), self.h)

    @property
    def launches(self) -> int:
        return int(lib().xrdt_ctx_launch_count(self.h))

    def last_error(self) -> str:
        return (lib().xrdt_last_error(self.h) or b"").decode()

    def set_profiling(self, on: bool):
        _check(lib().xrdt_ctx_set_profiling(self.h, 1 if on else 0), self.h)

    def kernel_stats(self, kernel: int):
        """(launches, total device ms, work units) of one kernel group."""
        n, ms, w = ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64()
        _check(lib().xrdt_ctx_kernel_stats(self.h, kernel, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(w)),
               self.h)
        return n.value, ms.value, w.value


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


_TORCH_DTYPE = {np.dtype(np.float32): "torch.float32", np.dtype(np.int32): "torch.int32",
                np.dtype(np.int64): "torch.int64", np.dtype(np.float64): "torch.float64"}


def _ptr(a, dtype, n=None):
    """Device or host address of a torch tensor / numpy array (kept alive by
    caller).  A numpy array is converted to dtype; a torch tensor must have
    that element type already (the library reads the words as they are).  n:
    the number of elements the library will touch, checked when given."""
    if a is None:
        return None, None
    if hasattr(a, "data_ptr"):  # torch tensor
        if not a.is_contiguous():
            raise ValueError("tensors must be contiguous")
        want = _TORCH_DTYPE.get(np.dtype(dtype))
        if want and str(a.dtype) != want:
            raise ValueError(f"a tensor of {a.dtype} where {want} is needed")
        if n is not None and a.numel() < n:
            raise ValueError(f"a tensor of {a.numel()} elements where {n} are needed")
        return a.data_ptr(), a
    arr = np.ascontiguousarray(a, dtype=dtype)
    if n is not None and arr.size < n:
        raise ValueError(f"an array of {arr.size} elements where {n} are needed")
    return arr.ctypes.data, arr


def _numel(a) -> int:
    return int(a.numel()) if hasattr(a, "numel") else int(np.size(a))


def _estimate(x0, n, flat=True):
    """An MLEM estimate of n elements: a torch tensor (contiguous float32,
    updated in place by the library) or anything else, copied into a new
    float32 array (flattened, or in x0's shape).  Returns (x, address)."""
    if _numel(x0) != n:
        raise ValueError(f"an estimate of {_numel(x0)} elements where {n} are needed")
    if hasattr(x0, "data_ptr"):
        return x0, _ptr(x0, np.float32, n)[0]
    x = np.array(x0, dtype=np.float32, copy=True, order="C")
    if flat:
        x = x.reshape(-1)
    return x, x.ctypes.data


def forward(p: Problem, spectrum, Ifine, seg, a1, a2, S2, q_min, q_max, a_min, a_max,
            Nphotons=None, Cphotons=None, Amatrix=None, want_amatrix: bool = True,
            plain: bool = False, ctx: Context | None = None, flags: int = 0):
    """xrdt_forward.  Outputs default to new numpy arrays (host staging by
    the library); pass torch CUDA tensors to keep everything on the device.
    Returns (Nphotons, Cphotons, Amatrix-or-None) as flat arrays."""
    rays = p.rays
    if Nphotons is None:
        Nphotons = np.empty(rays, np.float32)
    if Cphotons is None:
        Cphotons = np.empty(rays, np.float32)
    if Amatrix is None and want_amatrix:
        Amatrix = np.empty(p.amatrix_elems, np.float32)
    keep = []
    ptrs = []
    nvox, ntab = p.nx * p.ny, p.nq * p.na
    for a, dt, n in ((spectrum, np.float32, p.nrg_src * p.nrg_det), (Ifine, np.float32, p.nqf * p.n_mat),
                     (seg, np.int32, nvox), (a1, np.float32, nvox), (a2, np.float32, nvox), (S2, np.float32, ntab),
                     (Nphotons, np.float32, rays), (Cphotons, np.float32, rays),
                     (Amatrix, np.float32, p.amatrix_elems)):
        pt, k = _ptr(a, dt, n)
        ptrs.append(pt)
        keep.append(k)
    fl = flags | (FWD_PLAIN_FP64 if plain else 0)
    ctx = ctx or default_context()
    rc = lib().xrdt_forward(ctx.h, ctypes.byref(p), ptrs[0], ptrs[1], ptrs[2], ptrs[3], ptrs[4], ptrs[5],
                            float(q_min), float(q_max), float(a_min), float(a_max),
                            ptrs[6], ptrs[7], ptrs[8], fl)
    _check(rc, ctx.h)
    return keep[6], keep[7], keep[8]


def forward_tables(p: Problem, spectrum, seg, a1, a2, S1, S2, q_min, q_max, a_min, a_max,
                   Nphotons=None, Cphotons=None, bilinear: bool = False, ctx: Context | None = None,
                   flags: int = 0):
    """xrdt_forward_tables: the forward model with the coherent term read
    from the cross-section table S1 [NQ*NA] (nearest bins, or both tables
    bilinearly).  Returns (Nphotons, Cphotons) as flat arrays (numpy unless
    torch CUDA tensors are passed)."""
    rays = p.rays
    if Nphotons is None:
        Nphotons = np.empty(rays, np.float32)
    if Cphotons is None:
        Cphotons = np.empty(rays, np.float32)
    keep = []
    ptrs = []
    nvox, ntab = p.nx * p.ny, p.nq * p.na
    for a, dt, n in ((spectrum, np.float32, p.nrg_src * p.nrg_det), (seg, np.int32, nvox), (a1, np.float32, nvox),
                     (a2, np.float32, nvox), (S1, np.float32, ntab), (S2, np.float32, ntab),
                     (Nphotons, np.float32, rays), (Cphotons, np.float32, rays)):
        pt, k = _ptr(a, dt, n)
        ptrs.append(pt)
        keep.append(k)
    fl = flags | (TAB_BILINEAR if bilinear else 0)
    ctx = ctx or default_context()
    rc = lib().xrdt_forward_tables(ctx.h, ctypes.byref(p), ptrs[0], ptrs[1], ptrs[2], ptrs[3], ptrs[4], ptrs[5],
                                   float(q_min), float(q_max), float(a_min), float(a_max), ptrs[6], ptrs[7], fl)
    _check(rc, ctx.h)
    return keep[6], keep[7]


def forward_rays(p: Problem, rays, spectrum, Ifine, seg, a1, a2, S2, q_min, q_max, a_min, a_max,
                 want_amatrix: bool = False, plain: bool = False, ctx: Context | None = None):
    """xrdt_forward_rays: (N[n], C[n], A_rows[n, n_mat, nwt] or None) for the
    listed linear ray indices."""
    rays = np.ascontiguousarray(rays, np.int64)
    n = rays.size
    N = np.empty(n, np.float32)
    C = np.empty(n, np.float32)
    A = np.empty((n, p.n_mat, p.nwt), np.float32) if want_amatrix else None
    keep = []
    ptrs = []
    nvox, ntab = p.nx * p.ny, p.nq * p.na
    for a, dt, m in ((spectrum, np.float32, p.nrg_src * p.nrg_det), (Ifine, np.float32, p.nqf * p.n_mat),
                     (seg, np.int32, nvox), (a1, np.float32, nvox), (a2, np.float32, nvox), (S2, np.float32, ntab)):
        pt, k = _ptr(a, dt, m)
        ptrs.append(pt)
        keep.append(k)
    ctx = ctx or default_context()
    rc = lib().xrdt_forward_rays(ctx.h, ctypes.byref(p), *ptrs, float(q_min), float(q_max), float(a_min),
                                 float(a_max), rays.ctypes.data, n, N.ctypes.data, C.ctypes.data,
                                 A.ctypes.data if A is not None else None, FWD_PLAIN_FP64 if plain else 0)
    _check(rc, ctx.h)
    return N, C, A


def debug_decisions(p: Problem, rays, spectrum, seg, a1, a2, S2, q_min, q_max, a_min, a_max,
                    ctx: Context | None = None):
    """xrdt_debug_decisions: the fast path's integer decisions for the listed
    rays, as a dict of numpy arrays: win [n, 2], walk [n, nv, 4] (detector
    samples, detector edge, source samples, source edge), nq [n, nv, W],
    na [nv], s2u8 [nq*na]; voxels in the reference's loop order."""
    ctx = ctx or default_context()
    rays = np.ascontiguousarray(rays, np.int64)
    n = rays.size
    nv_max = int((np.asarray(seg) > 0).sum())
    W = 2 * p.dnrg + 1
    win = np.zeros((n, 2), np.int32)
    walk = np.zeros((n, nv_max, 4), np.int32)
    nq = np.zeros((n, nv_max, W), np.int32)
    na = np.zeros(max(nv_max, 1), np.int32)
    s2u8 = np.zeros(p.nq * p.na, np.uint8)
    nv = ctypes.c_int64()
    keep = [np.ascontiguousarray(a, dt) for a, dt in ((spectrum, np.float32), (seg, np.int32), (a1, np.float32),
                                                      (a2, np.float32), (S2, np.float32))]
    _check(lib().xrdt_debug_decisions(ctx.h, ctypes.byref(p), *[k.ctypes.data for k in keep], float(q_min),
                                      float(q_max), float(a_min), float(a_max), rays.ctypes.data, n,
                                      win.ctypes.data, walk.ctypes.data, na.ctypes.data, nq.ctypes.data,
                                      s2u8.ctypes.data, ctypes.byref(nv)), ctx.h)
    if nv.value != nv_max:
        raise RuntimeError("voxel count mismatch")
    return {"win": win, "walk": walk, "nq": nq, "na": na[:nv_max], "s2u8": s2u8}


def basis_expand(C, B, I=None, ctx: Context | None = None):
    """xrdt_basis_expand: I = C @ B in FP32 (3xTF32 on the tensor cores).
    C [M, K] and B [K, N] row-major; returns I [M, N] (numpy unless I is a
    torch CUDA tensor)."""
    pc, kc = _ptr(C, np.float32)
    pb, kb = _ptr(B, np.float32)
    if len(kc.shape) != 2 or len(kb.shape) != 2 or int(kb.shape[0]) != int(kc.shape[1]):
        raise ValueError("C must be [M, K] and B [K, N]")
    M, K = int(kc.shape[0]), int(kc.shape[1])
    N = int(kb.shape[1])
    if I is None:
        I = np.empty((M, N), np.float32)
    pi, ki = _ptr(I, np.float32, M * N)
    ctx = ctx or default_context()
    _check(lib().xrdt_basis_expand(ctx.h, pc, M, K, pb, N, pi, 0), ctx.h)
    return ki


def spectrum_build(e_hd, n_hd, src_edges, det_edges, sigma0=0.805, sigma1=0.0125, out=None,
                   ctx: Context | None = None):
    """xrdt_spectrum_build: the spectrum-response matrix of
    spectrum_builder.m:64-95 from a fine source spectrum (bin edges e_hd
    [H+1] in keV, photons per keV n_hd [H]) on coarse source and detector
    bins.  Returns the column-major flat [NS, ND] vector that forward()
    takes as its spectrum (numpy unless out is a torch CUDA tensor)."""
    ns = _numel(src_edges) - 1
    nd = _numel(det_edges) - 1
    nh = _numel(n_hd)
    if _numel(e_hd) != nh + 1:
        raise ValueError("e_hd must hold one more edge than n_hd has bins")
    if out is None:
        out = np.empty(ns * nd, np.float32)
    ptrs = [_ptr(a, np.float32, m) for a, m in ((e_hd, nh + 1), (n_hd, nh), (src_edges, ns + 1),
                                                 (det_edges, nd + 1), (out, ns * nd))]
    ctx = ctx or default_context()
    _check(lib().xrdt_spectrum_build(ctx.h, ptrs[0][0], ptrs[1][0], nh, ptrs[2][0], ns, ptrs[3][0], nd,
                                     float(sigma0), float(sigma1), ptrs[4][0], 0), ctx.h)
    return ptrs[4][1]


def ct_sinogram(p: Problem, spectrum, a1, a2, Tphotons=None, gain0=None, ctx: Context | None = None):
    """xrdt_ct_sinogram: (Tphotons, gain0) per (source, pixel, energy bin) in
    the Nphotons layout; -log(Tphotons / gain0) is the CT sinogram."""
    if Tphotons is None:
        Tphotons = np.empty(p.rays, np.float32)
    if gain0 is None:
        gain0 = np.empty(p.rays, np.float32)
    nvox = p.nx * p.ny
    ptrs = [_ptr(a, np.float32, m) for a, m in ((spectrum, p.nrg_src * p.nrg_det), (a1, nvox), (a2, nvox),
                                                 (Tphotons, p.rays), (gain0, p.rays))]
    ctx = ctx or default_context()
    _check(lib().xrdt_ct_sinogram(ctx.h, ctypes.byref(p), *[q[0] for q in ptrs], 0), ctx.h)
    return ptrs[3][1], ptrs[4][1]


def mlem_matrix(A, y, c, x0, iters: int, K: int | None = None, ctx: Context | None = None):
    """xrdt_mlem_matrix: MLEM of main.m:154-176 on the model matrix A
    ([rays, K] rows, the Amatrix layout).  x0 is updated in place when it is a
    torch CUDA tensor; numpy inputs return a new array."""
    if K is None:
        K = _numel(x0)
    rays = _numel(y)
    pa, ka = _ptr(A, np.float32, rays * K)
    py, ky = _ptr(y, np.float32)
    pc, kc = _ptr(c, np.float32, rays)
    x, px = _estimate(x0, K, flat=False)
    ctx = ctx or default_context()
    _check(lib().xrdt_mlem_matrix(ctx.h, pa, rays, K, py, pc, px, iters, 0), ctx.h)
    return x


def mlem_checkpoint_write(path: str, x, iteration: int) -> None:
    """xrdt_mlem_checkpoint_write: the estimate x (numpy or CUDA tensor) and
    the number of iterations done, to a file."""
    px, kx = _ptr(x, np.float32)
    n = int(kx.numel() if hasattr(kx, "numel") else kx.size)
    _check(lib().xrdt_mlem_checkpoint_write(os.fsencode(path), px, n, int(iteration)))


def mlem_checkpoint_read(path: str, x):
    """xrdt_mlem_checkpoint_read into x (a float32 numpy array or CUDA
    tensor of the checkpoint's size, filled in place); returns (x, iteration)."""
    if not hasattr(x, "data_ptr"):
        if not (isinstance(x, np.ndarray) and x.dtype == np.float32 and x.flags.c_contiguous):
            raise ValueError("x must be a contiguous float32 array or tensor")
    px, kx = _ptr(x, np.float32)
    n = int(kx.numel() if hasattr(kx, "numel") else kx.size)
    it = ctypes.c_int64()
    _check(lib().xrdt_mlem_checkpoint_read(os.fsencode(path), px, n, ctypes.byref(it)))
    return x, it.value


def mlem_matrix_noalloc(A, y, c, x, iters: int, stream: int | None = None):
    """xrdt_mlem_matrix_noalloc: the same MLEM for callers that cannot
    allocate; every array must already be a torch CUDA tensor, x is updated in
    place, the library allocates nothing."""
    for t in (A, y, c, x):
        if not hasattr(t, "data_ptr") or not t.is_cuda or not t.is_contiguous():
            raise ValueError("xrdt_mlem_matrix_noalloc takes contiguous CUDA tensors only")
        if str(t.dtype) != "torch.float32":
            raise ValueError("xrdt_mlem_matrix_noalloc takes float32 tensors only")
    # the kernels read A[rays, K], y[rays] and c[rays] without host staging:
    # a short buffer would be read out of bounds on the device
    if A.numel() != y.numel() * x.numel() or c.numel() != y.numel():
        raise ValueError("need A.numel() == y.numel() * x.numel() and c.numel() == y.numel()")
    _check(lib().xrdt_mlem_matrix_noalloc(A.data_ptr(), int(y.numel()), int(x.numel()), y.data_ptr(),
                                          c.data_ptr(), x.data_ptr(), iters, _vp(stream) if stream else None))
    return x


class Operator:
    """xrdt_op: the model with one coarse-q pattern per voxel, as a
    forward/backward context (include/xrdt.h).

    Coefficients x and gradients g have NX*NY*NWT entries, voxel index
    ix + NX*iy, coarse bin fastest; ray vectors have p.rays entries in the
    Nphotons order.  Arrays may be numpy (host) or contiguous torch CUDA
    tensors; outputs default to new numpy arrays."""

    def __init__(self, p: Problem, spectrum, seg, a1, a2, ctx: Context | None = None):
        nvox = p.nx * p.ny
        keep = [_ptr(a, dt, m) for a, dt, m in ((spectrum, np.float32, p.nrg_src * p.nrg_det),
                                                (seg, np.int32, nvox), (a1, np.float32, nvox),
                                                (a2, np.float32, nvox))]
        self.ctx = ctx or default_context()
        self.p = p
        h = _vp()
        _check(lib().xrdt_op_create(self.ctx.h, ctypes.byref(p), *[k[0] for k in keep], ctypes.byref(h)),
               self.ctx.h)
        self.h = h
        self.ctx._operators.add(self)

    @property
    def voxels(self) -> int:
        return int(lib().xrdt_op_voxels(self.h))

    @property
    def unknowns(self) -> int:
        return self.p.nx * self.p.ny * self.p.nwt

    @property
    def walk_bytes(self) -> int:
        """Bytes of the kept detector-side integrals (0: walked in every call)."""
        return int(lib().xrdt_op_walk_bytes(self.h))

    def close(self):
        # an operator must not outlive its context (xrdt_op_destroy reads it)
        if getattr(self, "h", None) and self.ctx.h:
            lib().xrdt_op_destroy(self.h)
        self.h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def forward(self, x, y=None):
        """y = Av x."""
        px, kx = _ptr(x, np.float32, self.unknowns)
        if y is None:
            y = np.empty(self.p.rays, np.float32)
        py, ky = _ptr(y, np.float32, self.p.rays)
        _check(lib().xrdt_op_forward(self.h, px, py, 0), self.ctx.h)
        return ky

    def adjoint(self, w, g=None):
        """g = Av^T w."""
        pw, kw = _ptr(w, np.float32, self.p.rays)
        if g is None:
            g = np.empty(self.unknowns, np.float32)
        pg, kg = _ptr(g, np.float32, self.unknowns)
        _check(lib().xrdt_op_adjoint(self.h, pw, pg, 0), self.ctx.h)
        return kg

    def forward_rays_fp64(self, x, rays):
        """(Av x)[rays] by the FP64 kernel at the reference's launch shape."""
        rays = np.ascontiguousarray(rays, np.int64)
        px, kx = _ptr(x, np.float32, self.unknowns)
        y = np.empty(rays.size, np.float32)
        _check(lib().xrdt_op_forward_rays(self.h, px, rays.ctypes.data, rays.size, y.ctypes.data, OP_PLAIN_FP64),
               self.ctx.h)
        return y

    def adjoint_rays_fp64(self, w, rays):
        """sum_i w[i] Av[rays[i]] by the FP64 kernel at the reference's launch shape."""
        rays = np.ascontiguousarray(rays, np.int64)
        pw, kw = _ptr(w, np.float32, rays.size)
        g = np.empty(self.unknowns, np.float32)
        _check(lib().xrdt_op_adjoint_rays(self.h, pw, rays.ctypes.data, rays.size, g.ctypes.data, OP_PLAIN_FP64),
               self.ctx.h)
        return g

    def mlem(self, y, c, x0, iters: int):
        """iters MLEM updates from x0 (main.m:162-176 with per-voxel unknowns).
        A torch CUDA x0 is updated in place; numpy returns a new array."""
        py, ky = _ptr(y, np.float32, self.p.rays)
        pc, kc = _ptr(c, np.float32, self.p.rays)
        x, px = _estimate(x0, self.unknowns)
        _check(lib().xrdt_op_mlem(self.h, py, pc, px, iters, 0), self.ctx.h)
        return x


class BasisOperator:
    """xrdt_bop: an Operator whose voxels carry J coefficients of a dense q
    basis B [J, NWT] (non-negative): forward(c) = Av (c B), adjoint(w) =
    (Av^T w) B^T, MLEM on the coefficients; the expansion and contraction
    run on the tensor cores.  Coefficient arrays have NX*NY*J entries."""

    def __init__(self, op: "Operator", B):
        self.op = op
        self.ctx = op.ctx
        pb, kb = _ptr(B, np.float32)
        if len(kb.shape) != 2 or int(kb.shape[1]) != op.p.nwt:
            raise ValueError(f"the basis must be [J, NWT = {op.p.nwt}]")
        self.J = int(kb.shape[0])
        h = _vp()
        _check(lib().xrdt_bop_create(op.h, pb, self.J, ctypes.byref(h)), self.ctx.h)
        self.h = h
        self.ctx._operators.add(self)

    @property
    def unknowns(self) -> int:
        return self.op.p.nx * self.op.p.ny * self.J

    def close(self):
        if getattr(self, "h", None) and self.ctx.h:
            lib().xrdt_bop_destroy(self.h)
        self.h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def forward(self, c, y=None):
        pc, kc = _ptr(c, np.float32, self.unknowns)
        if y is None:
            y = np.empty(self.op.p.rays, np.float32)
        py, ky = _ptr(y, np.float32, self.op.p.rays)
        _check(lib().xrdt_bop_forward(self.h, pc, py, 0), self.ctx.h)
        return ky

    def adjoint(self, w, g=None):
        pw, kw = _ptr(w, np.float32, self.op.p.rays)
        if g is None:
            g = np.empty(self.unknowns, np.float32)
        pg, kg = _ptr(g, np.float32, self.unknowns)
        _check(lib().xrdt_bop_adjoint(self.h, pw, pg, 0), self.ctx.h)
        return kg

    def mlem(self, y, c, x0, iters: int):
        py, ky = _ptr(y, np.float32, self.op.p.rays)
        pc, kc = _ptr(c, np.float32, self.op.p.rays)
        x, px = _estimate(x0, self.unknowns)
        _check(lib().xrdt_bop_mlem(self.h, py, pc, px, iters, 0), self.ctx.h)
        return x


class Batch:
    """xrdt_batch: several Operators run together, one persistent launch per
    kernel and one CUDA graph per MLEM iteration.  Every array argument is a
    list of contiguous torch CUDA tensors, one per operator."""

    def __init__(self, ops, ctx: Context | None = None):
        self.ctx = ctx or ops[0].ctx
        self.ops = list(ops)
        arr = (_vp * len(self.ops))(*[op.h for op in self.ops])
        h = _vp()
        _check(lib().xrdt_batch_create(self.ctx.h, arr, len(self.ops), ctypes.byref(h)), self.ctx.h)
        self.h = h
        self.ctx._operators.add(self)

    def close(self):
        if getattr(self, "h", None) and self.ctx.h:
            lib().xrdt_batch_destroy(self.h)
        self.h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def _ptrs(self, ts, kind):
        """One array per operator: contiguous float32 CUDA tensors of the
        operator's ray count (kind "rays") or unknown count ("unknowns")."""
        if len(ts) != len(self.ops):
            raise ValueError(f"{len(ts)} arrays for {len(self.ops)} operators")
        for t, op in zip(ts, self.ops):
            if not hasattr(t, "data_ptr") or not t.is_cuda:
                raise ValueError("batch arrays must be contiguous CUDA tensors")
            _ptr(t, np.float32, op.p.rays if kind == "rays" else op.unknowns)
        return (_vp * len(ts))(*[t.data_ptr() for t in ts])

    def forward(self, xs, ys):
        _check(lib().xrdt_batch_forward(self.h, self._ptrs(xs, "unknowns"), self._ptrs(ys, "rays"), 0), self.ctx.h)
        return ys

    def adjoint(self, ws, gs):
        _check(lib().xrdt_batch_adjoint(self.h, self._ptrs(ws, "rays"), self._ptrs(gs, "unknowns"), 0), self.ctx.h)
        return gs

    def mlem(self, ys, cs, xs, iters: int):
        _check(lib().xrdt_batch_mlem(self.h, self._ptrs(ys, "rays"), self._ptrs(cs, "rays"),
                                     self._ptrs(xs, "unknowns"), iters, 0), self.ctx.h)
        return xs

    def tune(self):
        """(adjoint warps per block, adjoint tiles, forward grid, adjoint grid) chosen by the autotuner."""
        w, t, fg, ag = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
        _check(lib().xrdt_batch_tune(self.h, ctypes.byref(w), ctypes.byref(t), ctypes.byref(fg), ctypes.byref(ag)),
               self.ctx.h)
        return w.value, t.value, fg.value, ag.value


def Forward_XRD(spectrum, Ifine, segmentation, a1, a2, S2, q_min, q_max, a_min, a_max,
                problem: Problem | None = None, ctx: Context | None = None):
    """Drop-in for the MEX call of main.m:56-64.

    Without `problem`, uses the reference's compiled configuration for the
    phantom size of `segmentation` (a 2-D [NX, NY] array).  Returns numpy
    arrays shaped like the MATLAB outputs (column-major)."""
    seg = np.asarray(segmentation)
    if problem is None:
        if seg.ndim != 2:
            raise ValueError("segmentation must be a 2-D [NX, NY] array")
        problem = reference_problem(seg.shape[0], seg.shape[1])
    flat = lambda x: np.asarray(x).reshape(-1, order="F")  # noqa: E731
    N, C, A = forward(problem, flat(spectrum), flat(Ifine), flat(seg).astype(np.int32), flat(a1), flat(a2),
                      flat(S2), q_min, q_max, a_min, a_max, ctx=ctx)
    p = problem
    shp = (p.n_src, p.n_col, p.n_row, p.nrg_det)
    return (N.reshape(shp, order="F"), C.reshape(shp, order="F"),
            A.reshape((p.nwt, p.n_mat) + shp, order="F"))
