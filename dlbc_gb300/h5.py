"""Minimal HDF5 subset reader/writer for the reference's field files.

The reference writes one dataset ``/OutArray`` per file through libhdf5
(``src/dlbc/io/hdf5.d:125-285``): global dims ``[gn0, gn1, (gn2,) (len)]``
with the vector/population component fastest (AoS) and the first lattice
axis slowest, element type native double (or native int for the mask).
Golden files were afterwards repacked with shuffle + deflate
(``tools/hdf5-repack.sh:5``).  No libhdf5 exists on this machine, so this
module implements exactly the subset those files use:

* superblock version 0 (8-byte offsets/lengths), symbol-table root group;
* version-1 object headers with continuation messages;
* dataspace (v1/v2), datatype (fixed-point / IEEE float, little endian),
  layout v3 (contiguous, chunked with a v1 B-tree), filter pipeline v1/v2
  with deflate (1) and shuffle (2);

and a writer that emits a contiguous, unfiltered ``/OutArray`` plus the
``input`` string-array attribute, readable by h5py/h5dump and by this
reader.  Everything is little-endian only (both machines this runs on are).
"""
from __future__ import annotations

import struct
import zlib
from typing import Dict, List, Optional, Tuple

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(RuntimeError):
    pass


class _Reader:
    def __init__(self, data: bytes):
        self.d = data
        if not data.startswith(_SIG):
            # the superblock may sit at 512/1024/... offsets; the reference's
            # files always start at 0
            raise H5Error("not an HDF5 file (signature missing at offset 0)")
        ver = data[8]
        if ver not in (0, 1):
            raise H5Error(f"unsupported superblock version {ver}")
        self.so = data[13]
        self.sl = data[14]
        if self.so != 8 or self.sl != 8:
            raise H5Error("only 8-byte offsets/lengths are supported")
        pos = 24 if ver == 0 else 28
        self.base, _fs, _eof, _drv = struct.unpack_from("<4Q", data, pos)
        pos += 32
        # root group symbol table entry
        _name_off, self.root_ohdr, cache_type = struct.unpack_from("<QQI", data, pos)
        self.root_btree = self.root_heap = None
        if cache_type == 1:
            self.root_btree, self.root_heap = struct.unpack_from("<QQ", data, pos + 24)

    # -- object headers ----------------------------------------------------
    def messages(self, addr: int) -> List[Tuple[int, bytes]]:
        d = self.d
        ver = d[addr]
        if ver != 1:
            raise H5Error(f"object header version {ver} unsupported")
        nmsg, _refc, hsize = struct.unpack_from("<HII", d, addr + 2)
        blocks = [(addr + 16, hsize)]
        out: List[Tuple[int, bytes]] = []
        while blocks and len(out) < nmsg:
            start, size = blocks.pop(0)
            p = start
            end = start + size
            while p + 8 <= end and len(out) < nmsg:
                mtype, msize, _flags = struct.unpack_from("<HHB", d, p)
                body = d[p + 8 : p + 8 + msize]
                p += 8 + msize
                out.append((mtype, body))
                if mtype == 0x10:
                    caddr, clen = struct.unpack_from("<QQ", body, 0)
                    blocks.append((caddr, clen))
        return out

    # -- groups --------------------------------------------------------------
    def _heap_name(self, heap_addr: int, off: int) -> str:
        d = self.d
        if d[heap_addr : heap_addr + 4] != b"HEAP":
            raise H5Error("bad local heap signature")
        data_addr = struct.unpack_from("<Q", d, heap_addr + 24)[0]
        s = data_addr + off
        e = d.index(b"\x00", s)
        return d[s:e].decode()

    def _group_links(self, btree: int, heap: int) -> Dict[str, int]:
        d = self.d
        links: Dict[str, int] = {}
        stack = [btree]
        while stack:
            node = stack.pop()
            if d[node : node + 4] != b"TREE":
                raise H5Error("bad group B-tree signature")
            ntype, level, nused = struct.unpack_from("<BBH", d, node + 4)
            if ntype != 0:
                raise H5Error("expected a group B-tree node")
            p = node + 24 + 8  # first key
            for _ in range(nused):
                child = struct.unpack_from("<Q", d, p)[0]
                p += 16
                if level > 0:
                    stack.append(child)
                    continue
                if d[child : child + 4] != b"SNOD":
                    raise H5Error("bad symbol node signature")
                nsym = struct.unpack_from("<H", d, child + 6)[0]
                q = child + 8
                for _s in range(nsym):
                    name_off, ohdr = struct.unpack_from("<QQ", d, q)
                    links[self._heap_name(heap, name_off)] = ohdr
                    q += 40
        return links

    def root_links(self) -> Dict[str, int]:
        btree, heap = self.root_btree, self.root_heap
        if btree is None:
            for mtype, body in self.messages(self.root_ohdr):
                if mtype == 0x11:
                    btree, heap = struct.unpack_from("<QQ", body, 0)
        if btree is None:
            raise H5Error("root group has no symbol table")
        return self._group_links(btree, heap)

    # -- datasets ------------------------------------------------------------
    def read_dataset(self, ohdr: int) -> np.ndarray:
        shape: Optional[Tuple[int, ...]] = None
        dtype = None
        layout = None
        filters: List[Tuple[int, Tuple[int, ...]]] = []
        for mtype, body in self.messages(ohdr):
            if mtype == 0x01:
                shape = self._dataspace(body)
            elif mtype == 0x03:
                dtype = self._datatype(body)
            elif mtype == 0x08:
                layout = body
            elif mtype == 0x0B:
                filters = self._filters(body)
        if shape is None or dtype is None or layout is None:
            raise H5Error("dataset header incomplete")
        return self._read_layout(layout, shape, dtype, filters)

    @staticmethod
    def _dataspace(b: bytes) -> Tuple[int, ...]:
        ver, rank = b[0], b[1]
        off = 8 if ver == 1 else 4
        return tuple(struct.unpack_from(f"<{rank}Q", b, off)) if rank else ()

    @staticmethod
    def _datatype(b: bytes):
        cls = b[0] & 0x0F
        bits0 = b[1]
        size = struct.unpack_from("<I", b, 4)[0]
        if bits0 & 1:
            raise H5Error("big-endian data unsupported")
        if cls == 0:
            signed = bool(bits0 & 0x08)
            return np.dtype(f"<{'i' if signed else 'u'}{size}")
        if cls == 1:
            return np.dtype(f"<f{size}")
        raise H5Error(f"datatype class {cls} unsupported")

    @staticmethod
    def _filters(b: bytes) -> List[Tuple[int, Tuple[int, ...]]]:
        ver, n = b[0], b[1]
        out = []
        p = 8 if ver == 1 else 2
        for _ in range(n):
            fid = struct.unpack_from("<H", b, p)[0]
            p += 2
            name_len = 0
            if ver == 1 or fid >= 256:
                name_len = struct.unpack_from("<H", b, p)[0]
                p += 2
            _flags, ncd = struct.unpack_from("<HH", b, p)
            p += 4
            if ver == 1:
                p += (name_len + 7) // 8 * 8
            else:
                p += name_len
            cd = struct.unpack_from(f"<{ncd}I", b, p)
            p += 4 * ncd
            if ver == 1 and ncd % 2:
                p += 4
            out.append((fid, cd))
        return out

    def _read_layout(self, b, shape, dtype, filters) -> np.ndarray:
        ver = b[0]
        if ver != 3:
            raise H5Error(f"layout message version {ver} unsupported")
        cls = b[1]
        n = int(np.prod(shape)) if shape else 1
        if cls == 1:
            addr, size = struct.unpack_from("<QQ", b, 2)
            if addr == _UNDEF:
                return np.zeros(shape, dtype)
            raw = self.d[addr : addr + n * dtype.itemsize]
            return np.frombuffer(raw, dtype).reshape(shape).copy()
        if cls == 0:
            size = struct.unpack_from("<H", b, 2)[0]
            return np.frombuffer(b[4 : 4 + size], dtype).reshape(shape).copy()
        if cls == 2:
            dimensionality = b[2]
            btree = struct.unpack_from("<Q", b, 3)[0]
            cdims = struct.unpack_from(f"<{dimensionality}I", b, 11)
            chunk = cdims[:-1]
            out = np.zeros(shape, dtype)
            self._walk_chunks(btree, dimensionality, chunk, dtype, filters, out)
            return out
        raise H5Error(f"layout class {cls} unsupported")

    def _walk_chunks(self, node, dimensionality, chunk, dtype, filters, out):
        d = self.d
        if d[node : node + 4] != b"TREE":
            raise H5Error("bad chunk B-tree signature")
        ntype, level, nused = struct.unpack_from("<BBH", d, node + 4)
        if ntype != 1:
            raise H5Error("expected a raw-data chunk B-tree node")
        keysize = 8 + 8 * dimensionality
        p = node + 24
        for _ in range(nused):
            csize, fmask = struct.unpack_from("<II", d, p)
            offs = struct.unpack_from(f"<{dimensionality}Q", d, p + 8)
            child = struct.unpack_from("<Q", d, p + keysize)[0]
            p += keysize + 8
            if level > 0:
                self._walk_chunks(child, dimensionality, chunk, dtype, filters, out)
                continue
            raw = d[child : child + csize]
            for i, (fid, cd) in reversed(list(enumerate(filters))):
                if fmask & (1 << i):
                    continue
                if fid == 1:
                    raw = zlib.decompress(raw)
                elif fid == 2:
                    es = cd[0] if cd else dtype.itemsize
                    a = np.frombuffer(raw, np.uint8)
                    nel = len(a) // es
                    raw = a[: nel * es].reshape(es, nel).T.copy().tobytes() + bytes(a[nel * es :])
                else:
                    raise H5Error(f"filter {fid} unsupported")
            block = np.frombuffer(raw, dtype)[: int(np.prod(chunk))].reshape(chunk)
            sl_out = []
            sl_in = []
            for ax, (o, c) in enumerate(zip(offs[:-1], chunk)):
                e = min(o + c, out.shape[ax])
                sl_out.append(slice(o, e))
                sl_in.append(slice(0, e - o))
            out[tuple(sl_out)] = block[tuple(sl_in)]


def read_field(path: str, name: str = "OutArray") -> np.ndarray:
    """Return dataset ``/name`` of an HDF5 file written by the reference.

    Arrays come back in the file's order: ``[x][y][z]`` (3D) or ``[x][y]``
    (2D) with an extra trailing axis for vector/population fields.
    """
    with open(path, "rb") as fh:
        data = fh.read()
    r = _Reader(data)
    links = r.root_links()
    if name not in links:
        raise H5Error(f"dataset /{name} not found in {path}")
    return r.read_dataset(links[name])


# ---------------------------------------------------------------------------
# writer
# ---------------------------------------------------------------------------

def _pad8(b: bytes) -> bytes:
    return b + b"\x00" * ((-len(b)) % 8)


def _msg(mtype: int, body: bytes, flags: int = 0) -> bytes:
    body = _pad8(body)
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _dtype_msg(dt: np.dtype) -> bytes:
    dt = np.dtype(dt)
    if dt.kind == "f":
        if dt.itemsize == 8:
            # class 1 version 1; bit fields: little endian, mantissa norm = 2 (implied msb),
            # sign bit location 63; properties: bit offset 0, precision 64, exp loc 52,
            # exp size 11, mantissa loc 0, mantissa size 52, exp bias 1023
            return struct.pack("<B3BI", 0x11, 0x20, 63, 0, 8) + struct.pack(
                "<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
        if dt.itemsize == 4:
            return struct.pack("<B3BI", 0x11, 0x20, 31, 0, 4) + struct.pack(
                "<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
        raise H5Error("unsupported float size")
    if dt.kind in "iu":
        signed = 0x08 if dt.kind == "i" else 0
        return struct.pack("<B3BI", 0x10, signed, 0, 0, dt.itemsize) + struct.pack(
            "<HH", 0, dt.itemsize * 8)
    raise H5Error(f"unsupported dtype {dt}")


def write_field(path: str, arr: np.ndarray, input_lines: Optional[List[str]] = None,
                attrs_f64: Optional[Dict[str, float]] = None,
                attrs_i32: Optional[Dict[str, int]] = None) -> None:
    """Write ``arr`` as ``/OutArray`` (contiguous, unfiltered), like
    ``dumpFieldHDF5`` (``src/dlbc/io/hdf5.d:125``).

    ``input_lines`` become the root attribute ``input`` as a 1-D array of
    fixed-length strings (the reference stores the parameter file lines
    there, ``src/dlbc/io/hdf5.d:529-548``).  ``attrs_f64``/``attrs_i32``
    add scalar root attributes (used for checkpoint globals such as the
    ``timestep``).
    """
    arr = np.ascontiguousarray(arr)
    if arr.dtype == np.float64:
        pass
    elif arr.dtype.kind in "iu":
        arr = arr.astype(np.int32)
    else:
        arr = arr.astype(np.float64)
    shape = arr.shape

    # Layout of the file we emit:
    #   superblock (96 bytes incl. root symbol table entry)
    #   root object header (symbol table message + attributes)
    #   group B-tree, local heap (+ data), symbol node
    #   dataset object header, raw data
    out = bytearray()

    def attr_msg(name: str, dt_body: bytes, ds_body: bytes, data: bytes) -> bytes:
        nm = name.encode() + b"\x00"
        body = struct.pack("<BBHHH", 1, 0, len(nm), len(dt_body), len(ds_body))
        body += _pad8(nm) + _pad8(dt_body) + _pad8(ds_body) + data
        return _msg(0x0C, body)

    def dataspace(dims) -> bytes:
        return struct.pack("<BBB5x", 1, len(dims), 0) + b"".join(struct.pack("<Q", x) for x in dims)

    root_attrs = b""
    if input_lines:
        enc = [ln.encode() for ln in input_lines]
        width = max(1, max(len(e) for e in enc) + 1)
        # string datatype: class 3, version 1, null-terminated ascii
        dt = struct.pack("<B3BI", 0x13, 0x00, 0, 0, width)
        data = b"".join(e.ljust(width, b"\x00") for e in enc)
        root_attrs += attr_msg("input", dt, dataspace([len(enc)]), data)
    for k, v in (attrs_f64 or {}).items():
        root_attrs += attr_msg(k, _dtype_msg(np.float64), dataspace([1]), struct.pack("<d", v))
    for k, v in (attrs_i32 or {}).items():
        root_attrs += attr_msg(k, _dtype_msg(np.int32), dataspace([1]), struct.pack("<i", v))

    SB = 96
    # root object header: 16-byte prefix + symbol table msg (16 body) + attrs
    root_msgs = _msg(0x11, struct.pack("<QQ", 0, 0)) + root_attrs
    root_ohdr = SB
    root_size = 16 + len(root_msgs)
    btree_addr = root_ohdr + root_size
    # group B-tree with one child (K=16 leaf -> room for 2K+1 keys, 2K children)
    K_internal = 16
    btree_size = 24 + (2 * K_internal + 1) * 8 + 2 * K_internal * 8
    heap_addr = btree_addr + btree_size
    heap_data = _pad8(b"\x00" * 8 + b"OutArray\x00")
    heap_data_addr = heap_addr + 32
    snod_addr = heap_data_addr + len(heap_data)
    K_leaf = 4
    snod_size = 8 + 2 * K_leaf * 40
    ds_ohdr = snod_addr + snod_size
    ds_msgs = _msg(0x01, dataspace(shape), 1) + _msg(0x03, _dtype_msg(arr.dtype), 1)
    ds_msgs_len_guess = len(ds_msgs) + 8 + 24  # layout message (v3 contiguous: 18 bytes -> 24)
    data_addr = ds_ohdr + 16 + ds_msgs_len_guess
    data_addr += (-data_addr) % 8
    ds_msgs += _msg(0x08, struct.pack("<BBQQ", 3, 1, data_addr, arr.nbytes))
    assert 16 + len(ds_msgs) == ds_msgs_len_guess + 16
    eof = data_addr + arr.nbytes

    # superblock v0
    out += _SIG
    out += struct.pack("<BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0)
    out += struct.pack("<HHI", K_leaf, K_internal, 0)
    out += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
    # root symbol table entry (cache type 1 -> B-tree + heap)
    out += struct.pack("<QQII", 0, root_ohdr, 1, 0) + struct.pack("<QQ", btree_addr, heap_addr)
    assert len(out) == SB
    # root object header: fix up the symbol table message body
    root_msgs = _msg(0x11, struct.pack("<QQ", btree_addr, heap_addr)) + root_attrs
    nmsgs = 1 + (1 if input_lines else 0) + len(attrs_f64 or {}) + len(attrs_i32 or {})
    out += struct.pack("<BBHII4x", 1, 0, nmsgs, 1, len(root_msgs)) + root_msgs
    assert len(out) == btree_addr
    # group B-tree node: type 0, level 0, one entry; keys are heap offsets
    bt = b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, _UNDEF, _UNDEF)
    bt += struct.pack("<Q", 0) + struct.pack("<Q", snod_addr) + struct.pack("<Q", 8)
    out += bt.ljust(btree_size, b"\x00")
    # local heap
    out += b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), _UNDEF, heap_data_addr)
    out += heap_data
    # symbol table node with one entry
    sn = b"SNOD" + struct.pack("<BBH", 1, 0, 1)
    sn += struct.pack("<QQII", 8, ds_ohdr, 0, 0) + b"\x00" * 16
    out += sn.ljust(snod_size, b"\x00")
    assert len(out) == ds_ohdr
    out += struct.pack("<BBHII4x", 1, 0, 3, 1, len(ds_msgs)) + ds_msgs
    out += b"\x00" * (data_addr - len(out))
    out += arr.tobytes()
    with open(path, "wb") as fh:
        fh.write(bytes(out))


def read_root_attr(path: str, name: str):
    """Read a scalar/1-D root attribute written by :func:`write_field`
    (numeric or fixed-length string)."""
    with open(path, "rb") as fh:
        data = fh.read()
    r = _Reader(data)
    for mtype, body in r.messages(r.root_ohdr):
        if mtype != 0x0C:
            continue
        ver, _r, nlen, dtlen, dslen = struct.unpack_from("<BBHHH", body, 0)
        p = 8
        aname = body[p : p + nlen - 1].decode()
        p += (nlen + 7) // 8 * 8
        dtb = body[p : p + dtlen]
        p += (dtlen + 7) // 8 * 8
        dsb = body[p : p + dslen]
        p += (dslen + 7) // 8 * 8
        if aname != name:
            continue
        shape = _Reader._dataspace(dsb)
        n = int(np.prod(shape)) if shape else 1
        cls = dtb[0] & 0x0F
        size = struct.unpack_from("<I", dtb, 4)[0]
        if cls == 3:
            return [body[p + i * size : p + (i + 1) * size].rstrip(b"\x00").decode() for i in range(n)]
        dt = _Reader._datatype(dtb)
        return np.frombuffer(body[p : p + n * dt.itemsize], dt).copy()
    raise H5Error(f"attribute {name} not found")
