"""The C ABI library: load, exports, presets and validation (CPU only; no
compute call runs without a GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

import xrd_tomography_gb300 as xt
from xrd_tomography_gb300 import synth
from xrd_tomography_gb300.api import SIGNATURES

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "xrdt.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(xrdt_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = xt.lib()
    names = header_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(SIGNATURES), "ctypes signatures and header diverge"


def test_abi_version():
    assert xt.lib().xrdt_abi_version() == 1


def test_problem_struct_layout_matches_c():
    # the C preset and the Python preset agree byte for byte
    for nx, ny in ((100, 100), (16, 16), (20, 12)):
        assert bytes(xt.c_reference_problem(nx, ny)) == bytes(xt.reference_problem(nx, ny))


def test_problem_counts():
    p = xt.reference_problem(100)
    L = xt.lib()
    assert L.xrdt_problem_rays(ctypes.byref(p)) == 32 * 1024 * 64 == p.rays
    assert L.xrdt_problem_amatrix_elems(ctypes.byref(p)) == 256 * 3 * 32 * 1024 * 64


@pytest.mark.parametrize("index", [0, 1, 2, 4])
def test_configs_validate(index):
    assert xt.validate(synth.config_problem(index)) == 0


def test_validation_rejects_bad_problems():
    p = xt.reference_problem(16)
    assert xt.validate(p) == 0
    assert xt.validate(p.copy(nx=0)) == 2
    assert xt.validate(p.copy(nrg_src=10)) == 2          # narrower than the 11-bin window
    assert xt.validate(p.copy(reserved0=1)) == 2
    assert xt.validate(p.copy(quirks=0x80)) == 2
    assert xt.validate(p.copy(dq_step=0.0)) == 2
    assert xt.validate(p.copy(q_hi=float("nan"))) == 2
    # a source on the phantom's edge, a detector panel through the phantom
    assert xt.validate(p.copy(r_src=5.0)) == 3
    assert xt.validate(p.copy(r_det=3.0)) == 3
    assert xt.lib().xrdt_problem_validate(None) == 1


def test_status_strings():
    L = xt.lib()
    for s in range(0, 9):
        assert L.xrdt_status_string(s)


def test_null_arguments_are_reported():
    L = xt.lib()
    assert L.xrdt_ctx_create(None, 0, None) == 1
    assert L.xrdt_ctx_destroy(None) == 1
    assert L.xrdt_forward(None, None, *([None] * 6), 0.0, 0.0, 0.0, 0.0, None, None, None, 0) == 1


def test_no_silent_cpu_path_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    # without a GPU the context cannot be created: the library reports it and
    # the Python front end raises rather than computing anything on the CPU
    with pytest.raises(xt.XrdtError):
        xt.Context(0)


def test_python_boundary_checks_types_and_sizes():
    """The Python front end converts numpy arrays but never reinterprets a
    tensor of another element type, and rejects arrays shorter than the
    library will read."""
    torch = pytest.importorskip("torch")
    from xrd_tomography_gb300.api import _ptr
    p, k = _ptr(np.zeros(4, np.float64), np.float32, 4)
    assert k.dtype == np.float32 and p == k.ctypes.data
    with pytest.raises(ValueError):
        _ptr(np.zeros(3, np.float32), np.float32, 4)
    with pytest.raises(ValueError):
        _ptr(torch.zeros(4, dtype=torch.float16), np.float32)
    with pytest.raises(ValueError):
        _ptr(torch.zeros(4, dtype=torch.int64), np.int32)
    with pytest.raises(ValueError):
        _ptr(torch.zeros(3), np.float32, 4)
    assert _ptr(torch.zeros(4), np.float32, 4)[0] != 0


def test_wrappers_check_sizes_before_calling_the_library():
    """Every wrapper rejects an array shorter than the library will touch, a
    tensor of another element type or a wrong-sized estimate with ValueError,
    before it creates a context or calls the library (so this runs on CPU)."""
    torch = pytest.importorskip("torch")
    from xrd_tomography_gb300.api import Batch, BasisOperator, Operator
    inp = synth.make_inputs(synth.tiny_problem(), 3)
    p = inp.problem
    nvox = p.nx * p.ny
    f32 = lambda n: np.ones(n, np.float32)   # noqa: E731
    with pytest.raises(ValueError):          # B is [K', N] with K' != K
        xt.basis_expand(np.ones((8, 16), np.float32), np.ones((8, 16), np.float32))
    with pytest.raises(ValueError):          # I shorter than M x N
        xt.basis_expand(np.ones((8, 16), np.float32), np.ones((16, 16), np.float32), I=f32(10))
    with pytest.raises(ValueError):
        xt.spectrum_build(f32(5), f32(4), f32(3), f32(3), out=f32(3))
    with pytest.raises(ValueError):
        xt.ct_sinogram(p, inp.spectrum, f32(nvox - 1), inp.a2)
    with pytest.raises(ValueError):
        xt.forward_rays(p, [0], inp.spectrum, inp.Ifine, inp.seg, inp.a1, inp.a2, f32(3), 0.5, 4.0, 0.0, 1.0)
    rays, K = 10, 8
    with pytest.raises(ValueError):          # A shorter than rays x K
        xt.mlem_matrix(f32(rays * K - 1), f32(rays), f32(rays), f32(K), 1)
    with pytest.raises(ValueError):          # c shorter than y
        xt.mlem_matrix(f32(rays * K), f32(rays), f32(rays - 1), f32(K), 1)
    with pytest.raises(ValueError):          # estimate of another size than K
        xt.mlem_matrix(f32(rays * K), f32(rays), f32(rays), f32(K - 1), 1, K=K)
    with pytest.raises(ValueError):          # an FP64 tensor is never reinterpreted
        xt.mlem_matrix(f32(rays * K), f32(rays), f32(rays), torch.ones(K, dtype=torch.float64), 1)
    with pytest.raises(ValueError):
        Operator(p, inp.spectrum, inp.seg[:-1], inp.a1, inp.a2)
    op = Operator.__new__(Operator)          # sizes only: no handle behind it
    op.p, op.h, op.ctx = p, None, None
    n = op.unknowns
    with pytest.raises(ValueError):
        op.mlem(f32(p.rays), f32(p.rays), f32(n - 1), 1)
    with pytest.raises(ValueError):
        op.mlem(f32(p.rays - 1), f32(p.rays), f32(n), 1)
    with pytest.raises(ValueError):
        op.forward_rays_fp64(f32(n - 1), [0])
    with pytest.raises(ValueError):
        op.adjoint_rays_fp64(f32(1), [0, 1])
    with pytest.raises(ValueError):          # the basis must be [J, NWT]
        BasisOperator(op, np.ones((16, p.nwt + 1), np.float32))
    b = Batch.__new__(Batch)
    b.ops, b.h = [op], None
    with pytest.raises(ValueError):          # one array per operator
        b._ptrs([], "rays")
    with pytest.raises(ValueError):          # host tensors are not batch arrays
        b._ptrs([torch.ones(p.rays)], "rays")
