"""JLD2 solution files: the on-disk records of ``File/save.jl`` and
``File/load.jl`` (``save_project``, ``save_solution``, ``save_callback``,
``load_solution``, ``load_time_steps``, ``load_snapshots``) for the host side.

JLD2 files are HDF5 files behind a 512-byte JLD2 header: the superblock sits
at byte 512 and every address in the file is relative to it.  No HDF5
library is used: this module writes and reads the subset of the HDF5 file
format (HDF5 File Format Specification, version 3) that these records need,
in the forms JLD2 itself writes for plain bits types:

* superblock version 2; object headers version 2 ("OHDR"); the root group
  as a compact new-style group (Link Info, Group Info and one hard Link
  message per entry);
* datasets with a Dataspace (scalar, simple or null), a Datatype (IEEE
  little-endian float64 / int64 / float32 / int32, fixed-length ASCII
  string), a Fill Value (version 3) and a Data Layout message (version 3:
  compact for scalars and strings, contiguous for arrays);
* the Jenkins lookup3 checksum (``hashlittle``, initial value 0) that HDF5
  puts on the superblock and on every version-2 object header.

A Julia array ``A`` of size (n1, ..., nd) is stored by JLD2 with the HDF5
dimensions reversed, (nd, ..., n1), over the same column-major bytes; the
solver's host arrays are C-ordered numpy arrays of shape (N_e, N_c, N_p) over
the bytes of the reference's (N_p, N_c, N_e) arrays, so the numpy shape is
the HDF5 dataspace as it stands.

The reader also accepts the older layout libhdf5 writes by default
(superblock version 0, version-1 object headers with continuation blocks,
groups as symbol tables: version-1 B-tree, symbol-table nodes, local heap),
which is how it is checked against a file written by libhdf5 itself.

``project.jld2`` of the reference holds Julia structs (the conservation law,
the spatial discretisation, ...), which JLD2 serialises as committed Julia
datatypes; those cannot be produced outside Julia.  ``save_project`` writes
the same file name with the values the host side holds as plain datasets
(``tspan``, the array sizes and text descriptions), which is what
``load_snapshots`` needs.
"""
from __future__ import annotations

import os
import shutil
import struct

import numpy as np

FILE_HEADER_LENGTH = 512
JLD2_HEADER = b"HDF5-based Julia Data Format, version 0.1.1\x00 (Julia 1.10.0 64-bit little-endian)\x00"
HDF5_SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
SINGLE_OBJECT = "single_stored_object"   # JLD2's key of save_object / load_object

# header message types
MSG_DATASPACE, MSG_LINK_INFO, MSG_DATATYPE, MSG_FILL = 0x01, 0x02, 0x03, 0x05
MSG_LINK, MSG_LAYOUT, MSG_GROUP_INFO, MSG_CONTINUATION, MSG_SYMBOL_TABLE = 0x06, 0x08, 0x0A, 0x10, 0x11


# --------------------------------------------------------------------------
# Jenkins lookup3 (Bob Jenkins, public domain), byte-wise little-endian form
# --------------------------------------------------------------------------
_M32 = 0xFFFFFFFF


def _rot(x: int, k: int) -> int:
    return ((x << k) | (x >> (32 - k))) & _M32


def lookup3(data: bytes, initval: int = 0) -> int:
    """``hashlittle(data, len, initval)``: the checksum of HDF5 metadata."""
    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & _M32
    i = 0
    while n > 12:
        a = (a + int.from_bytes(data[i:i + 4], "little")) & _M32
        b = (b + int.from_bytes(data[i + 4:i + 8], "little")) & _M32
        c = (c + int.from_bytes(data[i + 8:i + 12], "little")) & _M32
        a = (a - c) & _M32; a ^= _rot(c, 4); c = (c + b) & _M32
        b = (b - a) & _M32; b ^= _rot(a, 6); a = (a + c) & _M32
        c = (c - b) & _M32; c ^= _rot(b, 8); b = (b + a) & _M32
        a = (a - c) & _M32; a ^= _rot(c, 16); c = (c + b) & _M32
        b = (b - a) & _M32; b ^= _rot(a, 19); a = (a + c) & _M32
        c = (c - b) & _M32; c ^= _rot(b, 4); b = (b + a) & _M32
        n -= 12
        i += 12
    if n == 0:
        return c
    tail = data[i:i + n] + bytes(12 - n)
    a = (a + int.from_bytes(tail[0:4], "little")) & _M32
    b = (b + int.from_bytes(tail[4:8], "little")) & _M32
    c = (c + int.from_bytes(tail[8:12], "little")) & _M32
    c ^= b; c = (c - _rot(b, 14)) & _M32
    a ^= c; a = (a - _rot(c, 11)) & _M32
    b ^= a; b = (b - _rot(a, 25)) & _M32
    c ^= b; c = (c - _rot(b, 16)) & _M32
    a ^= c; a = (a - _rot(c, 4)) & _M32
    b ^= a; b = (b - _rot(a, 14)) & _M32
    c ^= b; c = (c - _rot(b, 24)) & _M32
    return c


# --------------------------------------------------------------------------
# writing
# --------------------------------------------------------------------------
def _datatype(value) -> tuple[bytes, bytes, tuple]:
    """(Datatype message, raw bytes, dataspace dims or None for scalar)."""
    if isinstance(value, (str, bytes)):
        s = value.encode("ascii") if isinstance(value, str) else value
        # class 3 (string), version 1; null-padded ASCII
        msg = bytes([0x13, 0x01, 0, 0]) + struct.pack("<I", max(len(s), 1))
        return msg, (s if s else b"\x00"), None
    arr = np.asarray(value)
    if arr.dtype == np.bool_:
        arr = arr.astype(np.int64)
    if arr.dtype.kind == "f":
        if arr.dtype.itemsize == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            msg = bytes([0x11, 0x20, 63, 0]) + struct.pack("<I", 8) + props
        elif arr.dtype.itemsize == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            msg = bytes([0x11, 0x20, 31, 0]) + struct.pack("<I", 4) + props
        else:
            raise TypeError(f"unsupported float width {arr.dtype}")
        arr = arr.astype(arr.dtype.newbyteorder("<"), copy=False)
    elif arr.dtype.kind in "iu":
        width = arr.dtype.itemsize
        if width not in (4, 8):
            arr = arr.astype(np.int64)
            width = 8
        signed = 0x08 if arr.dtype.kind == "i" else 0x00
        msg = bytes([0x10, signed, 0, 0]) + struct.pack("<I", width) + struct.pack("<HH", 0, 8 * width)
        arr = arr.astype(arr.dtype.newbyteorder("<"), copy=False)
    else:
        raise TypeError(f"unsupported value of dtype {arr.dtype}")
    raw = np.ascontiguousarray(arr).tobytes()
    return msg, raw, (None if arr.ndim == 0 else tuple(arr.shape))


def _dataspace(dims) -> bytes:
    if dims is None:
        return bytes([2, 0, 0, 0])                       # version 2, rank 0, scalar
    # simple (an empty array too: a zero extent)
    return bytes([2, len(dims), 0, 1]) + b"".join(struct.pack("<Q", d) for d in dims)


def _message(mtype: int, data: bytes, flags: int = 0) -> bytes:
    return struct.pack("<BHB", mtype, len(data), flags) + data


def _object_header(messages: list[bytes]) -> bytes:
    body = b"".join(messages)
    n = len(body)
    if n < 256:
        code, size = 0, struct.pack("<B", n)
    elif n < 65536:
        code, size = 1, struct.pack("<H", n)
    else:
        code, size = 2, struct.pack("<I", n)
    head = b"OHDR" + bytes([2, code]) + size + body
    return head + struct.pack("<I", lookup3(head))


def _dataset_header_size(value) -> int:
    """Bytes of a dataset's object header (the layout message's address
    field has a fixed size, so the size does not depend on where the data
    lands)."""
    return len(_dataset_header(value, 0))


def _dataset_header(value, data_rel: int) -> bytes:
    dt, raw, dims = _datatype(value)
    msgs = [_message(MSG_DATASPACE, _dataspace(dims), 1), _message(MSG_DATATYPE, dt, 1),
            _message(MSG_FILL, bytes([3, 0x0A]), 1)]
    if dims is None:
        layout = bytes([3, 0]) + struct.pack("<H", len(raw)) + raw          # compact
    elif len(raw) == 0:
        layout = bytes([3, 1]) + struct.pack("<QQ", UNDEF, 0)              # contiguous, unallocated
    else:
        layout = bytes([3, 1]) + struct.pack("<QQ", data_rel, len(raw))    # contiguous
    msgs.append(_message(MSG_LAYOUT, layout))
    return _object_header(msgs)


def save(path: str, data: dict) -> None:
    """Write ``data`` (name -> float/int scalar, numpy array or string) as a
    JLD2 file: ``save(file, Dict(...))`` of JLD2/FileIO."""
    names = list(data.keys())
    for n in names:
        if not n or len(n.encode()) > 255:
            raise ValueError(f"dataset name {n!r}")
    # layout: [header 512][superblock 48][root group header][dataset headers][raw data]
    link_sizes = [len(_message(MSG_LINK, bytes([1, 0, len(n.encode())]) + n.encode() + bytes(8))) for n in names]
    root_size = len(_object_header([_message(MSG_LINK_INFO, bytes(18)), _message(MSG_GROUP_INFO, bytes(2))]
                                   + [bytes(s) for s in link_sizes]))
    rel = 48 + root_size                      # relative address of the first dataset header
    headers_rel, raws = [], []
    for n in names:
        headers_rel.append(rel)
        rel += _dataset_header_size(data[n])
    data_rel = []
    for n in names:
        _, raw, dims = _datatype(data[n])
        if dims is None or len(raw) == 0:
            data_rel.append(0)
            raws.append(b"")
            continue
        rel = (rel + 7) & ~7
        data_rel.append(rel)
        raws.append(raw)
        rel += len(raw)
    eof_abs = FILE_HEADER_LENGTH + rel
    links = [_message(MSG_LINK, bytes([1, 0, len(n.encode())]) + n.encode() + struct.pack("<Q", a))
             for n, a in zip(names, headers_rel)]
    linfo = bytes([0, 0]) + struct.pack("<QQ", UNDEF, UNDEF)
    root = _object_header([_message(MSG_LINK_INFO, linfo), _message(MSG_GROUP_INFO, bytes([0, 0]))] + links)
    assert len(root) == root_size
    sb = HDF5_SIGNATURE + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", FILE_HEADER_LENGTH, UNDEF, eof_abs, 48)
    sb += struct.pack("<I", lookup3(sb))
    out = bytearray(JLD2_HEADER.ljust(FILE_HEADER_LENGTH, b"\x00"))
    out += sb + root
    for n, a, d in zip(names, headers_rel, data_rel):
        h = _dataset_header(data[n], d)
        assert len(out) == FILE_HEADER_LENGTH + a
        out += h
    for d, raw in zip(data_rel, raws):
        if not raw:
            continue
        out += bytes(FILE_HEADER_LENGTH + d - len(out))
        out += raw
    assert len(out) == eof_abs
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        f.write(bytes(out))
    os.replace(tmp, path)


def save_object(path: str, obj) -> None:
    """JLD2's ``save_object``: one value under ``single_stored_object``."""
    save(path, {SINGLE_OBJECT: obj})


# --------------------------------------------------------------------------
# reading
# --------------------------------------------------------------------------
class FormatError(ValueError):
    pass


class _File:
    def __init__(self, buf: bytes):
        self.buf = buf
        base = None
        for off in (0, 512, 1024, 2048, 4096, 8192):
            if buf[off:off + 8] == HDF5_SIGNATURE:
                base = off
                break
        if base is None:
            raise FormatError("no HDF5 superblock at 0, 512, ..., 8192")
        self.sb = base
        ver = buf[base + 8]
        if ver in (0, 1):
            self.so, self.sl = buf[base + 13], buf[base + 14]
            if (self.so, self.sl) != (8, 8):
                raise FormatError("only 8-byte offsets and lengths are supported")
            p = base + 24 + (4 if ver == 1 else 0)
            self.base, _, self.eof, _ = struct.unpack_from("<QQQQ", buf, p)
            # root group symbol table entry: name offset, header address, cache type, scratch
            self.root = struct.unpack_from("<Q", buf, p + 40)[0]
        elif ver in (2, 3):
            self.so, self.sl = buf[base + 9], buf[base + 10]
            if (self.so, self.sl) != (8, 8):
                raise FormatError("only 8-byte offsets and lengths are supported")
            self.base, _, self.eof, self.root = struct.unpack_from("<QQQQ", buf, base + 12)
            (ck,) = struct.unpack_from("<I", buf, base + 44)
            if ck != lookup3(buf[base:base + 44]):
                raise FormatError("superblock checksum mismatch")
        else:
            raise FormatError(f"superblock version {ver}")
        if self.eof > len(buf):
            raise FormatError("file truncated: end-of-file address beyond the file")

    def at(self, rel: int) -> int:
        return self.base + rel

    # object headers ---------------------------------------------------------
    def messages(self, rel: int) -> list[tuple[int, bytes]]:
        buf, p = self.buf, self.at(rel)
        out = []
        if buf[p:p + 4] == b"OHDR":
            if buf[p + 4] != 2:
                raise FormatError("object header version")
            flags = buf[p + 5]
            q = p + 6
            if flags & 0x20:
                q += 16
            if flags & 0x10:
                q += 4
            code = flags & 3
            size = int.from_bytes(buf[q:q + (1 << code)], "little")
            q += 1 << code
            end = q + size
            if struct.unpack_from("<I", buf, end)[0] != lookup3(buf[p:end]):
                raise FormatError("object header checksum mismatch")
            chunks = [(q, end, True)]
            while chunks:
                q, end, v2 = chunks.pop(0)
                while q + 4 <= end:
                    mtype, msize, _mflags = struct.unpack_from("<BHB", buf, q)
                    q += 4
                    if flags & 0x04:
                        q += 2
                    data = buf[q:q + msize]
                    q += msize
                    if mtype == MSG_CONTINUATION:
                        addr, length = struct.unpack_from("<QQ", data)
                        c = self.at(addr)
                        if buf[c:c + 4] != b"OCHK":
                            raise FormatError("continuation chunk signature")
                        if struct.unpack_from("<I", buf, c + length - 4)[0] != lookup3(buf[c:c + length - 4]):
                            raise FormatError("continuation chunk checksum mismatch")
                        chunks.append((c + 4, c + length - 4, True))
                    else:
                        out.append((mtype, data))
            return out
        if buf[p] != 1:
            raise FormatError(f"object header version {buf[p]} at {rel}")
        nmsg, _refs, size = struct.unpack_from("<HII", buf, p + 2)
        chunks = [(p + 16, p + 16 + size)]
        seen = 0
        while chunks and seen < nmsg:
            q, end = chunks.pop(0)
            while q + 8 <= end and seen < nmsg:
                mtype, msize, _mflags = struct.unpack_from("<HHB", buf, q)
                data = buf[q + 8:q + 8 + msize]
                q += 8 + msize
                seen += 1
                if mtype == MSG_CONTINUATION:
                    addr, length = struct.unpack_from("<QQ", data)
                    chunks.append((self.at(addr), self.at(addr) + length))
                else:
                    out.append((mtype, data))
        return out

    # groups -------------------------------------------------------------
    def links(self, rel: int) -> dict[str, int]:
        msgs = self.messages(rel)
        out = {}
        for mtype, data in msgs:
            if mtype == MSG_LINK:
                out.update([self._link(data)])
            elif mtype == MSG_SYMBOL_TABLE:
                btree, heap = struct.unpack_from("<QQ", data)
                out.update(self._symbol_table(btree, heap))
            elif mtype == MSG_LINK_INFO:
                flags = data[1]
                q = 2 + (8 if flags & 1 else 0)
                fheap = struct.unpack_from("<Q", data, q)[0]
                if fheap != UNDEF:
                    raise FormatError("dense link storage (fractal heap) is not supported")
        return out

    def _link(self, data: bytes):
        if data[0] != 1:
            raise FormatError("link message version")
        flags = data[1]
        q = 2
        ltype = 0
        if flags & 0x08:
            ltype = data[q]
            q += 1
        if flags & 0x04:
            q += 8
        if flags & 0x10:
            q += 1
        w = 1 << (flags & 3)
        n = int.from_bytes(data[q:q + w], "little")
        q += w
        name = data[q:q + n].decode("utf-8")
        q += n
        if ltype != 0:
            raise FormatError(f"link {name!r}: only hard links are supported")
        return name, struct.unpack_from("<Q", data, q)[0]

    def _heap_data(self, heap_rel: int) -> int:
        p = self.at(heap_rel)
        if self.buf[p:p + 4] != b"HEAP":
            raise FormatError("local heap signature")
        return self.at(struct.unpack_from("<Q", self.buf, p + 24)[0])

    def _name(self, heap_data: int, off: int) -> str:
        end = self.buf.index(b"\x00", heap_data + off)
        return self.buf[heap_data + off:end].decode("utf-8")

    def _symbol_table(self, btree_rel: int, heap_rel: int) -> dict[str, int]:
        heap_data = self._heap_data(heap_rel)
        out = {}
        stack = [btree_rel]
        while stack:
            p = self.at(stack.pop())
            if self.buf[p:p + 4] != b"TREE" or self.buf[p + 4] != 0:
                raise FormatError("group B-tree node")
            level = self.buf[p + 5]
            used = struct.unpack_from("<H", self.buf, p + 6)[0]
            q = p + 24
            children = []
            for k in range(used):
                q += 8                                   # key k (heap offset)
                children.append(struct.unpack_from("<Q", self.buf, q)[0])
                q += 8
            if level > 0:
                stack.extend(reversed(children))
                continue
            for c in children:
                s = self.at(c)
                if self.buf[s:s + 4] != b"SNOD":
                    raise FormatError("symbol table node signature")
                nsym = struct.unpack_from("<H", self.buf, s + 6)[0]
                e = s + 8
                for _ in range(nsym):
                    name_off, header = struct.unpack_from("<QQ", self.buf, e)
                    out[self._name(heap_data, name_off)] = header
                    e += 40
        return out

    # datasets -----------------------------------------------------------
    def dataset(self, rel: int):
        dims, dtype, layout, string = None, None, None, None
        for mtype, data in self.messages(rel):
            if mtype == MSG_DATASPACE:
                dims = self._dataspace(data)
            elif mtype == MSG_DATATYPE:
                dtype, string = self._datatype(data)
            elif mtype == MSG_LAYOUT:
                layout = data
        if dims is None or dtype is None or layout is None:
            raise FormatError("not a dataset (dataspace, datatype and layout messages required)")
        raw = self._layout(layout, dims, dtype)
        if string is not None:
            return raw.split(b"\x00", 1)[0].decode("ascii" if string == 0 else "utf-8")
        if dims == "null":
            return None
        arr = np.frombuffer(raw, dtype=dtype, count=int(np.prod(dims)) if dims else 1)
        if not dims:
            return arr[0].item()
        return arr.reshape(dims).astype(dtype.newbyteorder("="))

    def _dataspace(self, data: bytes):
        ver, rank = data[0], data[1]
        if ver == 1:
            q = 8
        elif ver == 2:
            if data[3] == 2:
                return "null"
            q = 4
        else:
            raise FormatError("dataspace version")
        return tuple(struct.unpack_from(f"<{rank}Q", data, q)) if rank else ()

    def _datatype(self, data: bytes):
        cls, bits0 = data[0] & 0x0F, data[1]
        size = struct.unpack_from("<I", data, 4)[0]
        order = ">" if bits0 & 1 else "<"
        if cls == 0:
            return np.dtype(f"{order}{'i' if bits0 & 0x08 else 'u'}{size}"), None
        if cls == 1:
            return np.dtype(f"{order}f{size}"), None
        if cls == 3:
            return np.dtype(f"S{size}"), (bits0 >> 4) & 0x0F
        raise FormatError(f"datatype class {cls} is not supported")

    def _layout(self, data: bytes, dims, dtype) -> bytes:
        ver = data[0]
        n = (int(np.prod(dims)) if dims not in ((), "null") else (0 if dims == "null" else 1)) * dtype.itemsize
        if ver in (1, 2):
            # version 1/2: dimensionality, class, 5 reserved bytes, [address],
            # dimension sizes (4 bytes each), [element size], [compact data]
            rank, cls = data[1], data[2]
            q = 8
            addr = None
            if cls in (1, 2):
                addr = struct.unpack_from("<Q", data, q)[0]
                q += 8
            q += 4 * rank
            if cls == 0:
                size = struct.unpack_from("<I", data, q)[0]
                return data[q + 4:q + 4 + size]
            if cls == 1:
                if addr == UNDEF:
                    return bytes(n)
                p = self.at(addr)
                if p + n > len(self.buf):
                    raise FormatError("contiguous data beyond the end of the file")
                return self.buf[p:p + n]
            raise FormatError("chunked datasets are not supported")
        if ver not in (3, 4):
            raise FormatError(f"data layout version {ver}")
        cls = data[1]
        if cls == 0:
            size = struct.unpack_from("<H", data, 2)[0]
            return data[4:4 + size]
        if cls == 1:
            addr, size = struct.unpack_from("<QQ", data, 2)
            if addr == UNDEF:
                return bytes(n)
            p = self.at(addr)
            if p + size > len(self.buf):
                raise FormatError("contiguous data beyond the end of the file")
            return self.buf[p:p + size]
        raise FormatError("chunked datasets are not supported")


def load(path: str, names=None) -> dict:
    """Read a JLD2 (or plain HDF5) file's top-level datasets: ``load(file)``."""
    with open(path, "rb") as f:
        f_ = _File(f.read())
    links = f_.links(f_.root)
    keys = links.keys() if names is None else names
    return {k: f_.dataset(links[k]) for k in keys}


def load_object(path: str):
    """JLD2's ``load_object``."""
    return load(path, [SINGLE_OBJECT])[SINGLE_OBJECT]


# --------------------------------------------------------------------------
# File/save.jl and File/load.jl
# --------------------------------------------------------------------------
def new_path(results_path: str, overwrite: bool = False, clear: bool = False) -> str:
    """``new_path`` (File/save.jl:1-20): the results directory, with _1, _2,
    ... appended when it exists and overwrite is false."""
    if not os.path.isdir(results_path):
        path = results_path
    elif overwrite:
        if clear:
            shutil.rmtree(results_path, ignore_errors=True)
        path = results_path
    else:
        suffix = 1
        while True:
            path = results_path.rstrip("/") + f"_{suffix}/"
            if not os.path.isdir(path):
                break
            suffix += 1
    os.makedirs(path, exist_ok=True)
    return path if path.endswith("/") else path + "/"


def save_project(problem, tspan, results_path: str, overwrite: bool = False, clear: bool = False) -> str:
    """``save_project`` (File/save.jl:22-43): project.jld2 and an empty
    time_steps.jld2.  ``problem`` is the host mirror's problem (setups.Problem)
    or any object with ``host_arrays()``; its sizes and descriptions are
    stored as plain datasets."""
    results_path = new_path(results_path, overwrite, clear)
    h = problem.host_arrays() if hasattr(problem, "host_arrays") else problem
    record = {"tspan": np.asarray(tspan, dtype=np.float64),
              "N_p": np.int64(h.N_p), "N_c": np.int64(h.N_c), "N_e": np.int64(h.N_e)}
    # the reference's Julia structs, as text (setups.Problem field names)
    for key, attr in (("conservation_law", "law"), ("spatial_discretization", "sd"),
                      ("initial_data", "initial_data"), ("form", "form")):
        desc = getattr(problem, attr, None)
        if desc is not None:
            record[key] = _describe(desc)
    save(os.path.join(results_path, "project.jld2"), record)
    save_object(os.path.join(results_path, "time_steps.jld2"), np.zeros(0, dtype=np.int64))
    return results_path


def _describe(obj) -> str:
    """One line of text for a host-side object (its type and scalar fields)."""
    fields = getattr(obj, "__dict__", None)
    if not fields:
        return repr(obj)[:2000]
    parts = [f"{k}={v!r}" for k, v in fields.items() if isinstance(v, (int, float, str, bool, tuple))]
    return (type(obj).__name__ + "(" + ", ".join(parts) + ")")[:2000]


def _push_time_step(results_path: str, time_step: int) -> None:
    f = os.path.join(results_path, "time_steps.jld2")
    steps = np.asarray(load_object(f), dtype=np.int64).reshape(-1)
    save_object(f, np.append(steps, np.int64(time_step)))


def save_solution(u, t: float, results_path: str, time_step=0, du=None) -> None:
    """``save_solution`` (File/save.jl:45-81): sol_<time_step>.jld2 with u,
    t (and du, the residual at u, as the integrator form writes it); an
    integer time step is appended to time_steps.jld2."""
    rec = {"u": np.asarray(u, dtype=np.float64), "t": float(t)}
    if du is not None:
        rec["du"] = np.asarray(du, dtype=np.float64)
    save(os.path.join(results_path, f"sol_{time_step}.jld2"), rec)
    if isinstance(time_step, (int, np.integer)):
        _push_time_step(results_path, int(time_step))


def save_callback(solver, results_path: str, u0, n_steps: int, dt: float, interval: int = 1,
                  t0: float = 0.0, scheme: int = 0):
    """``save_callback`` (File/save.jl:83-93) around the device time loop.

    Runs ``n_steps`` fixed steps of the scheme on the GPU with the snapshot
    hook (``rk_steps_snapshots``: the state and its residual after every
    ``interval``-th step, copied out by the device loop) and writes
    sol_<n>.jld2 with u, t and du at step 0, at every ``interval``-th step
    and at the last step, as the reference's DiscreteCallback (condition
    ``iter % interval == 0``) and PresetTimeCallback (tspan ends) do; each
    step number is appended to time_steps.jld2.  Returns (u, t) at the end.
    ``scheme``: 0 CarpenterKennedy2N54, 1 RK4 (the library's sse_scheme)."""
    def write(u_s, t_s, step, du_s):
        # the integrator form of save_solution: skip a step already on disk,
        # log the step to screen.txt (File/save.jl:45-66)
        if os.path.exists(os.path.join(results_path, f"sol_{step}.jld2")):
            return
        with open(os.path.join(results_path, "screen.txt"), "a") as log:
            log.write(f"writing time step {step}  t = {t_s}\n")
        save_solution(u_s, t_s, results_path, step, du_s)

    u = np.array(u0, dtype=np.float64, order="C", copy=True)
    write(u, t0, 0, solver.residual(u))
    t, snaps, res = solver.rk_steps_snapshots(u, n_steps, dt, interval, scheme, with_residuals=True, t=t0)
    for k in range(len(snaps)):
        step = (k + 1) * interval
        write(snaps[k], t0 + step * dt, step, res[k])
    if n_steps % interval:
        write(u, t, n_steps, solver.residual(u))
    return u, t


def load_solution(results_path: str, time_step=0, load_du: bool = False):
    """``load_solution`` (File/load.jl:1-10): (u, t) or (u, du, t)."""
    d = load(os.path.join(results_path, f"sol_{time_step}.jld2"))
    if load_du:
        return d["u"], d["du"], d["t"]
    return d["u"], d["t"]


def load_project(results_path: str) -> dict:
    """``load_project`` (File/load.jl:12-19): the project record."""
    return load(os.path.join(results_path, "project.jld2"))


def load_time_steps(results_path: str) -> np.ndarray:
    """``load_time_steps`` (File/load.jl:29-31)."""
    return np.asarray(load_object(os.path.join(results_path, "time_steps.jld2")), dtype=np.int64).reshape(-1)


def _sizes(results_path: str):
    p = load_project(results_path)
    return int(p["N_p"]), int(p["N_c"]), int(p["N_e"])


def load_snapshots(results_path: str, time_steps):
    """``load_snapshots`` (File/load.jl:33-49): X (N_dof x N_t, each column
    a state in the reference's column-major order) and the mean time step."""
    N_p, N_c, N_e = _sizes(results_path)
    n_dof, n_t = N_p * N_c * N_e, len(time_steps)
    X = np.empty((n_dof, n_t))
    times = np.empty(n_t)
    for i, s in enumerate(time_steps):
        u, times[i] = load_solution(results_path, s)
        X[:, i] = np.asarray(u).reshape(-1)
    return X, (times[-1] - times[0]) / (n_t - 1.0)


def load_snapshots_with_derivatives(results_path: str, time_steps):
    """``load_snapshots_with_derivatives`` (File/load.jl:51-69)."""
    N_p, N_c, N_e = _sizes(results_path)
    n_dof, n_t = N_p * N_c * N_e, len(time_steps)
    U, dU = np.empty((n_dof, n_t)), np.empty((n_dof, n_t))
    times = np.empty(n_t)
    for i, s in enumerate(time_steps):
        u, du, times[i] = load_solution(results_path, s, load_du=True)
        U[:, i] = np.asarray(u).reshape(-1)
        dU[:, i] = np.asarray(du).reshape(-1)
    return U, dU, (times[-1] - times[0]) / (n_t - 1.0)
