"""The MAT-file reader (xrd_tomography_gb300.matfile): the reference's data
files, version 7.3 (HDF5 behind a MATLAB header, read by the project's own
reader) and version 5 (scipy), and the fixture of measured inputs extracted
from them (tests/golden/make_real_inputs.py)."""
import glob
import os

import numpy as np
import pytest

from xrd_tomography_gb300.matfile import MatFileError, load_mat, pattern_q

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("XRDT_REF_SRC") or os.path.abspath(os.path.join(HERE, "..", "..", "reference"))
FIX = np.load(os.path.join(HERE, "golden", "real_inputs.npz"))
MATERIALS = ("cellulose", "TNT", "ammoniumnitrate", "aluminum_alloy")

needs_ref = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "open_source_data")),
                               reason="the reference's data files are not present")


@needs_ref
def test_every_data_file_of_the_reference_loads():
    files = sorted(glob.glob(os.path.join(REF, "**", "*.mat"), recursive=True))
    assert len(files) >= 11
    v73 = 0
    for f in files:
        with open(f, "rb") as fh:
            v73 += fh.read(10) == b"MATLAB 7.3"
        v = load_mat(f)
        assert v, f
    assert v73 >= 7   # the HDF5 ones go through the project's reader


@needs_ref
def test_reader_reproduces_the_fixture():
    s = load_mat(os.path.join(REF, "Spectrum_80kVp", "spectral_data_HD.mat"))["spectrum"]
    assert np.array_equal(np.asarray(s["energy"]).ravel(), FIX["spectrum_energy"])
    assert np.array_equal(np.asarray(s["counts"]).ravel(), FIX["spectrum_counts"])
    for m in MATERIALS:
        D = load_mat(os.path.join(REF, "open_source_data", m + ".mat"), names=["D"])["D"]
        assert np.array_equal(D, FIX["D_" + m])


@needs_ref
def test_struct_and_version5_files():
    phys = load_mat(os.path.join(REF, "Physics_inputs", "physical_constants.mat"))["phys"]
    assert phys.shape == (1, 1)
    h = load_mat(os.path.join(REF, "Physics_inputs", "Hubbell_data.mat"))
    assert h["Fcoh"].shape == h["Sincoh"].shape == (h["wvt_list"].shape[0], 82)
    pc = load_mat(os.path.join(REF, "Physics_inputs", "PE_and_Compton_coefs.mat"))["PE_and_Compton_coefs"]
    assert pc.shape == (2, 27) and np.all(np.isfinite(pc))


def test_fixture_shapes_and_values():
    """The 80 kVp spectrum on 1440 bins of 0.05 keV from 8 to 80 keV
    (spectrum_builder.m:26-27), and patterns with increasing 2-theta."""
    e = FIX["spectrum_energy"]
    assert e.shape == (1441,) and e[0] == 8.0 and e[-1] == 80.0
    assert np.allclose(np.diff(e), 0.05, atol=1e-9)
    assert np.all(FIX["spectrum_counts"] >= 0.0)
    for m in MATERIALS:
        D = FIX["D_" + m]
        assert D.ndim == 2 and D.shape[1] == 2 and np.all(np.isfinite(D))
        # measured scans: 2-theta rises (the aluminium alloy file repeats two
        # angles)
        assert np.mean(np.diff(D[:, 0]) > 0) > 0.98 and np.all(D[:, 0] > 0) and np.all(D[:, 0] < 180)


def test_pattern_q_conversion():
    """q = 2 E sin(theta/2) / (hbar c) with E = 8.04 keV (XRD_builder.m:10,
    :44-45); zero-count entries dropped (:39-40)."""
    D = np.array([[20.0, 5.0], [40.0, 0.0], [60.0, 2.0]])
    q, I = pattern_q(D)
    assert np.allclose(q, 2 * 8.04 * np.sin(np.radians([20.0, 60.0]) / 2) / 1.973269804, rtol=1e-15)
    assert np.array_equal(I, [5.0, 2.0])
    qt, _ = pattern_q(FIX["D_TNT"])
    assert np.all(np.diff(qt) > 0) and 0.3 < qt[0] < qt[-1] < 6.0


def _superblock(btree, heap, header=0):
    """A MATLAB 7.3 header and a version-0 HDF5 superblock (8-byte offsets
    and lengths, base address 512 as MATLAB writes it) whose root group entry
    caches the given B-tree and heap (addresses relative to the base)."""
    head = b"MATLAB 7.3 MAT-file".ljust(512, b" ")
    sb = b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + (4).to_bytes(2, "little") \
        + (16).to_bytes(2, "little") + bytes(4)
    sb += (512).to_bytes(8, "little") + (2**64 - 1).to_bytes(8, "little") * 3   # base, free space, eof, driver
    sb += bytes(8) + header.to_bytes(8, "little") + (1).to_bytes(4, "little") + bytes(4)
    sb += btree.to_bytes(8, "little") + heap.to_bytes(8, "little")
    return head + sb


def test_damaged_files_raise_matfile_error(tmp_path):
    """Damaged files end in MatFileError, not in another exception, an
    endless recursion or a loop: a root entry that points past the end, and
    a B-tree whose node is its own child."""
    p = tmp_path / "past_end.mat"
    p.write_bytes(_superblock(btree=1 << 40, heap=1 << 40))
    with pytest.raises(MatFileError):
        load_mat(str(p))

    data = bytearray(_superblock(btree=512, heap=1536).ljust(4096, b"\0"))
    # at file offset 1024 (address 512): an internal node (level 1) with one
    # key and one child, itself
    node = b"TREE" + bytes([0, 1]) + (1).to_bytes(2, "little") + bytes(16) + bytes(8) \
        + (512).to_bytes(8, "little")
    data[1024:1024 + len(node)] = node
    p = tmp_path / "cycle.mat"
    p.write_bytes(bytes(data))
    with pytest.raises(MatFileError, match="cycle"):
        load_mat(str(p))


@needs_ref
def test_truncated_reference_files_raise_matfile_error(tmp_path):
    """Every truncation of a measured pattern file either still holds the
    variable (the tail cut was unused) or raises MatFileError."""
    src = os.path.join(REF, "open_source_data", "TNT.mat")
    with open(src, "rb") as f:
        data = f.read()
    full = load_mat(src)["D"]
    for frac in (0.1, 0.3, 0.5, 0.7, 0.9, 0.99):
        p = tmp_path / f"cut{frac}.mat"
        p.write_bytes(data[:int(len(data) * frac)])
        try:
            v = load_mat(str(p))
        except MatFileError:
            continue
        assert np.array_equal(v["D"], full)


def test_not_a_mat_file(tmp_path):
    p = tmp_path / "x.mat"
    p.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes([3]) + bytes(100))
    with pytest.raises(MatFileError):
        load_mat(str(p))
