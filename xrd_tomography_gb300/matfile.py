"""Reading the reference's MATLAB data files (host side, no GPU).

The reference's inputs are MATLAB MAT-files: the materials' measured XRD
patterns (`open_source_data/*.mat`, loaded by XRD_builder.m:35-37 and its
repeats for every material), the source spectra (`Spectrum_80kVp/*.mat`,
spectrum_builder.m) and physics tables (`Physics_inputs/*.mat`).  Most are
version 7.3 files, which are HDF5 files behind a 512-byte MATLAB header; the
rest are version 5 files.  No HDF5 library is installed, so version 7.3 files
are read by the small reader below, which covers what MATLAB writes for
numeric, logical and character arrays and for structs:

* the version-0 superblock after the 512-byte user block;
* version-1 object headers (with continuation blocks) and the dataspace,
  datatype, layout, filter-pipeline, attribute and symbol-table messages;
* groups as symbol tables: a version-1 B-tree of symbol-table nodes and a
  local heap of names;
* contiguous, compact and chunked storage, the chunks indexed by a
  version-1 B-tree and compressed with deflate (zlib) and optionally
  shuffled.

MATLAB stores an array of size d1 x d2 x ... as an HDF5 dataset of
dimensions (..., d2, d1); `load_mat` returns arrays in MATLAB's shape, and
the MATLAB_class attribute decides the element type (`char` becomes a
string, `logical` a bool array).  Version-5 files go to scipy.io.loadmat.

A damaged or truncated file raises MatFileError: reads past the end of the
file, cycles of B-tree nodes or header continuations, arrays larger than
MAX_ARRAY_BYTES and undecodable chunks are all reported that way.
"""
from __future__ import annotations

import zlib

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
MAX_ARRAY_BYTES = 1 << 34    # 16 GiB: larger arrays are taken as a damaged size field
_MAX_DEPTH = 64              # B-tree levels and nested groups


class MatFileError(ValueError):
    pass


class _Hdf5:
    """The parts of the HDF5 format (version-0 superblock) that MATLAB uses."""

    def __init__(self, data: bytes):
        self.d = data
        sb = None
        for off in (0, 512, 1024, 2048):
            if data[off:off + 8] == _SIG:
                sb = off
                break
        if sb is None:
            raise MatFileError("no HDF5 superblock")
        if data[sb + 8] != 0:
            raise MatFileError(f"superblock version {data[sb + 8]} is not supported")
        self.so = data[sb + 13]   # size of offsets
        self.sl = data[sb + 14]   # size of lengths
        if self.so not in (4, 8) or self.sl not in (4, 8):
            raise MatFileError("unsupported address sizes")
        p = sb + 24
        self.base = self._u(p, self.so)
        p += 4 * self.so          # base, free-space, end-of-file, driver information
        # root group symbol table entry
        self.root = self._entry(p)

    # ---- little-endian helpers ----
    def _u(self, p, n):
        if p < 0 or p + n > len(self.d):
            raise MatFileError(f"read of {n} bytes at {p} is past the end of the file ({len(self.d)} bytes)")
        return int.from_bytes(self.d[p:p + n], "little")

    def _addr(self, p):
        a = self._u(p, self.so)
        return None if a == (1 << (8 * self.so)) - 1 else a + self.base

    def _need(self, addr, n, what):
        """An address that must hold n bytes of the file."""
        if addr is None or addr < 0 or addr + n > len(self.d):
            raise MatFileError(f"{what} at {addr} is outside the file")
        return addr

    def _nbytes(self, shape, dtype):
        n = 1
        for x in shape:
            n *= int(x)
        if n * dtype.itemsize > MAX_ARRAY_BYTES:
            raise MatFileError(f"array of shape {tuple(shape)} is larger than {MAX_ARRAY_BYTES} bytes")
        return n

    def _entry(self, p):
        name_off = self._u(p, self.so)
        header = self._addr(p + self.so)
        cache = self._u(p + 2 * self.so, 4)
        scratch = p + 2 * self.so + 8
        btree = heap = None
        if cache == 1:
            btree = self._addr(scratch)
            heap = self._addr(scratch + self.so)
        return {"name_off": name_off, "header": header, "btree": btree, "heap": heap}

    # ---- object headers ----
    def messages(self, addr):
        d = self.d
        self._need(addr, 16, "object header")
        if d[addr] != 1:
            raise MatFileError(f"object header version {d[addr]} is not supported")
        nmsg = self._u(addr + 2, 2)
        size = self._u(addr + 8, 4)
        blocks = [(addr + 16, size)]
        seen = set()
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            if start in seen:
                raise MatFileError("object header continuations form a cycle")
            seen.add(start)
            self._need(start, length, "object header block")
            p = start
            while p + 8 <= start + length and len(out) < nmsg:
                mtype = self._u(p, 2)
                msize = self._u(p + 2, 2)
                body = p + 8
                if mtype == 0x10:                       # continuation
                    blocks.append((self._addr(body), self._u(body + self.so, self.sl)))
                out.append((mtype, body, msize))
                p = body + msize
        return out

    def _dataspace(self, p):
        d = self.d
        ver, nd, flags = d[p], d[p + 1], d[p + 2]
        q = p + (8 if ver == 1 else 4)
        if ver == 2 and d[p + 3] == 0:
            return ()
        return tuple(self._u(q + i * self.sl, self.sl) for i in range(nd))

    def _datatype(self, p):
        d = self.d
        cls = d[p] & 0x0F
        bits = d[p + 1] | (d[p + 2] << 8) | (d[p + 3] << 16)
        size = self._u(p + 4, 4)
        if bits & 1:
            raise MatFileError("big-endian data is not supported")
        if cls == 0:                                    # fixed point
            return np.dtype(("i" if bits & 0x8 else "u") + str(size)).newbyteorder("<")
        if cls == 1:                                    # floating point
            return np.dtype("f" + str(size)).newbyteorder("<")
        if cls == 3:                                    # string
            return np.dtype("S" + str(size))
        if cls == 7:                                    # object reference
            return np.dtype("<u" + str(size))
        raise MatFileError(f"datatype class {cls} is not supported")

    def _attribute(self, p):
        d = self.d
        ver = d[p]
        nlen, tlen, slen = self._u(p + 2, 2), self._u(p + 4, 2), self._u(p + 6, 2)
        pad = (lambda n: (n + 7) & ~7) if ver == 1 else (lambda n: n)
        q = p + 8 + (1 if ver == 3 else 0)
        name = d[q:q + nlen].split(b"\0")[0].decode("latin-1")
        q += pad(nlen)
        dt = self._datatype(q)
        q += pad(tlen)
        shape = self._dataspace(q)
        q += pad(slen)
        n = self._nbytes(shape, dt) if shape else 1
        self._need(q, n * dt.itemsize, "attribute data")
        raw = d[q:q + n * dt.itemsize]
        return name, np.frombuffer(raw, dt, n).reshape(shape) if shape else np.frombuffer(raw, dt, 1)[0]

    def _filters(self, p):
        d = self.d
        ver, nf = d[p], d[p + 1]
        q = p + (8 if ver == 1 else 2)
        out = []
        for _ in range(nf):
            fid = self._u(q, 2)
            if ver == 1 or fid >= 256:
                nlen = self._u(q + 2, 2)
                flags, nval = self._u(q + 4, 2), self._u(q + 6, 2)
                q += 8 + ((nlen + 7) & ~7 if ver == 1 else nlen)
            else:
                nlen = 0
                flags, nval = self._u(q + 2, 2), self._u(q + 4, 2)
                q += 6
            vals = [self._u(q + 4 * i, 4) for i in range(nval)]
            q += 4 * nval + (4 if ver == 1 and nval % 2 else 0)
            out.append((fid, vals))
        return out

    # ---- groups ----
    def _heap_name(self, heap, off):
        if heap is None or self.d[heap:heap + 4] != b"HEAP":
            raise MatFileError("bad local heap")
        data = self._need(self._addr(heap + 8 + 2 * self.sl), off + 1, "local heap data")
        end = self.d.find(b"\0", data + off)
        if end < 0:
            raise MatFileError("unterminated name in a local heap")
        return self.d[data + off:end].decode("latin-1")

    def _btree_children(self, addr, key_size, depth=0, seen=None):
        d = self.d
        seen = set() if seen is None else seen
        if addr is None or d[addr:addr + 4] != b"TREE":
            raise MatFileError("bad B-tree node")
        if addr in seen or depth > _MAX_DEPTH:
            raise MatFileError("B-tree nodes form a cycle")
        seen.add(addr)
        level = self._u(addr + 5, 1)
        n = self._u(addr + 6, 2)
        p = addr + 8 + 2 * self.so
        out = []
        for _ in range(n):
            key = p
            child = self._addr(p + key_size)
            out.append((key, child))
            p += key_size + self.so
        if level > 0:
            flat = []
            for _, child in out:
                flat.extend(self._btree_children(child, key_size, depth + 1, seen))
            return flat
        return out

    def group(self, btree, heap):
        """Name -> object header address of a group's members."""
        members = {}
        for _, snod in self._btree_children(btree, self.sl):
            if snod is None or self.d[snod:snod + 4] != b"SNOD":
                raise MatFileError("bad symbol table node")
            n = self._u(snod + 6, 2)
            for i in range(n):
                e = self._entry(snod + 8 + i * (2 * self.so + 24))
                members[self._heap_name(heap, e["name_off"])] = e["header"]
        return members

    # ---- objects ----
    def read_object(self, addr):
        """('group', {name: addr}, attrs) or ('dataset', array, attrs)."""
        shape = dtype = layout = None
        filters, attrs = [], {}
        for mtype, p, _ in self.messages(addr):
            if mtype == 0x01:
                shape = self._dataspace(p)
            elif mtype == 0x03:
                dtype = self._datatype(p)
            elif mtype == 0x08:
                layout = p
            elif mtype == 0x0B:
                filters = self._filters(p)
            elif mtype == 0x0C:
                name, val = self._attribute(p)
                attrs[name] = val
            elif mtype == 0x11:
                return "group", self.group(self._addr(p), self._addr(p + self.so)), attrs
        if layout is None or dtype is None:
            raise MatFileError("object is neither a group nor a dataset")
        return "dataset", self._read_data(layout, shape or (), dtype, filters), attrs

    def _read_data(self, p, shape, dtype, filters):
        d = self.d
        ver = d[p]
        if ver != 3:
            raise MatFileError(f"layout message version {ver} is not supported")
        cls = d[p + 1]
        n = self._nbytes(shape, dtype) if shape else 1
        if cls == 0:                                    # compact
            size = self._u(p + 2, 2)
            if size < n * dtype.itemsize:
                raise MatFileError("compact data is shorter than its dataspace")
            raw = d[p + 4:p + 4 + size]
        elif cls == 1:                                  # contiguous
            a = self._addr(p + 2)
            if a is not None:
                self._need(a, n * dtype.itemsize, "contiguous data")
            raw = b"\0" * (n * dtype.itemsize) if a is None else d[a:a + n * dtype.itemsize]
        elif cls == 2:                                  # chunked
            nd = d[p + 2]
            bt = self._addr(p + 3)
            cdims = [self._u(p + 3 + self.so + 4 * i, 4) for i in range(nd)]
            return self._read_chunked(bt, shape, cdims[:-1], dtype, filters)
        else:
            raise MatFileError(f"layout class {cls} is not supported")
        arr = np.frombuffer(raw, dtype, n)
        return arr.reshape(shape) if shape else arr

    def _read_chunked(self, bt, shape, cdims, dtype, filters):
        nd = len(shape)
        if len(cdims) != nd or any(c < 1 for c in cdims):
            raise MatFileError("chunk dimensions do not match the dataspace")
        self._nbytes(shape, dtype)
        self._nbytes(cdims, dtype)
        out = np.zeros(shape, dtype)
        if bt is None:
            return out
        key_size = 8 + 8 * (nd + 1)
        for key, child in self._btree_children(bt, key_size):
            csize = self._u(key, 4)
            mask = self._u(key + 4, 4)
            offs = [self._u(key + 8 + 8 * i, 8) for i in range(nd)]
            raw = self.d[self._need(child, csize, "chunk"):child + csize]
            for k, (fid, vals) in reversed(list(enumerate(filters))):
                if mask & (1 << k):
                    continue
                if fid == 1:
                    raw = zlib.decompress(raw)
                elif fid == 2:                          # shuffle
                    es = vals[0] if vals else dtype.itemsize
                    b = np.frombuffer(raw, np.uint8)
                    raw = b.reshape(es, -1).T.tobytes()
                else:
                    raise MatFileError(f"filter {fid} is not supported")
            if len(raw) < int(np.prod(cdims)) * dtype.itemsize:
                raise MatFileError("a chunk holds fewer bytes than its dimensions")
            chunk = np.frombuffer(raw, dtype, int(np.prod(cdims))).reshape(cdims)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
            out[sl] = chunk[tuple(slice(0, x.stop - x.start) for x in sl)]
        return out


def _matlab_value(h5, kind, val, attrs, depth=0):
    cls = attrs.get("MATLAB_class")
    cls = cls.decode("latin-1") if isinstance(cls, bytes) else (str(cls) if cls is not None else None)
    if kind == "group":
        if depth > _MAX_DEPTH:
            raise MatFileError("groups nest deeper than the reader follows (a cycle?)")
        return {name: _matlab_value(h5, *h5.read_object(addr), depth=depth + 1)
                for name, addr in val.items() if not name.startswith("#")}
    if "MATLAB_empty" in attrs and int(np.asarray(attrs["MATLAB_empty"]).ravel()[0]):
        dims = tuple(int(x) for x in np.asarray(val).ravel()[::-1]) if np.size(val) else (0, 0)
        return np.zeros(dims)
    arr = np.asarray(val)
    if arr.ndim >= 1:
        arr = arr.transpose()   # HDF5 dims are MATLAB's reversed
    if cls == "char":
        return "".join(chr(c) for c in np.asarray(arr, np.int64).ravel(order="F"))
    if cls == "logical":
        return arr.astype(bool)
    return np.array(arr)


def load_mat(path: str, names=None) -> dict:
    """The variables of a MAT-file as numpy arrays in MATLAB's shapes (and
    dicts for structs, str for char arrays).  names: only these variables."""
    with open(path, "rb") as f:
        data = f.read()
    if data[512:520] != _SIG and data[:8] != _SIG:
        import scipy.io
        v = scipy.io.loadmat(path, variable_names=names)
        return {k: val for k, val in v.items() if not k.startswith("__")}
    try:
        h5 = _Hdf5(data)
        root = h5.root
        members = h5.group(root["btree"], root["heap"]) if root["btree"] is not None \
            else h5.read_object(root["header"])[1]
        out = {}
        for name, addr in members.items():
            if name.startswith("#") or (names is not None and name not in names):
                continue
            out[name] = _matlab_value(h5, *h5.read_object(addr))
        return out
    except MatFileError:
        raise
    except (IndexError, KeyError, TypeError, ValueError, OverflowError, RecursionError, zlib.error) as e:
        raise MatFileError(f"damaged or unsupported MAT-file {path}: {type(e).__name__}: {e}") from e


def pattern_q(D, e_src_kev: float = 8.04, hbarc: float = 1.973269804):
    """A measured pattern D [n, 2] (2-theta in degrees, intensity) as
    (q in 1/Angstrom, intensity) with the zero-count entries dropped, as
    XRD_builder.m:38-48 converts it (the copper K-alpha source energy and
    hbar c of :10-11)."""
    D = np.asarray(D, np.float64)
    keep = D[:, 1] > 0
    theta = D[keep, 0] / 180.0 * np.pi
    return np.sin(theta / 2.0) * (2.0 * e_src_kev) / hbarc, D[keep, 1]
