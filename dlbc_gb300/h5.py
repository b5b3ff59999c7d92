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

attribute messages (numbers, fixed- and variable-length strings, the latter
through the global heap), and a writer that emits a contiguous, unfiltered
``/OutArray`` plus the reference's attributes: ``input`` at the root and the
``metadata`` / ``globals`` groups.  The writer follows the published HDF5
file-format specification (superblock 0); it is checked against this
reader, as no libhdf5 is installed.  Everything is little-endian only (both
machines this runs on are).
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
# attributes
# ---------------------------------------------------------------------------

def _global_heap_object(d: bytes, coll: int, index: int) -> bytes:
    """Object ``index`` of the global heap collection at ``coll``."""
    if d[coll : coll + 4] != b"GCOL":
        raise H5Error("bad global heap signature")
    size = struct.unpack_from("<Q", d, coll + 8)[0]
    p = coll + 16
    end = coll + size
    while p + 16 <= end:
        idx, _refc, _res, osize = struct.unpack_from("<HHIQ", d, p)
        if idx == 0:
            break
        if idx == index:
            return d[p + 16 : p + 16 + osize]
        p += 16 + osize + ((-osize) % 8)
    raise H5Error(f"global heap object {index} not found")


def _decode_attr(d: bytes, body: bytes):
    ver = body[0]
    if ver != 1:
        raise H5Error(f"attribute message version {ver} unsupported")
    _r, nlen, dtlen, dslen = struct.unpack_from("<BHHH", body, 1)
    p = 8
    name = body[p : p + nlen - 1].decode()
    p += (nlen + 7) // 8 * 8
    dtb = body[p : p + dtlen]
    p += (dtlen + 7) // 8 * 8
    dsb = body[p : p + dslen]
    p += (dslen + 7) // 8 * 8
    shape = _Reader._dataspace(dsb)
    n = int(np.prod(shape)) if shape else 1
    cls = dtb[0] & 0x0F
    size = struct.unpack_from("<I", dtb, 4)[0]
    if cls == 3:  # fixed-length string
        val = [body[p + i * size : p + (i + 1) * size].split(b"\x00")[0].decode() for i in range(n)]
    elif cls == 9:  # variable-length: (length, global heap collection, index) per element
        val = []
        for i in range(n):
            ln, coll, idx = struct.unpack_from("<IQI", body, p + 16 * i)
            val.append(_global_heap_object(d, coll, idx)[:ln].decode())
    else:
        dt = _Reader._datatype(dtb)
        val = np.frombuffer(body[p : p + n * dt.itemsize], dt).copy()
    return name, val


def read_attrs(path: str, group: str = "") -> Dict[str, object]:
    """All attributes of the root group (``group=""``) or of the child group
    ``/group``: numbers as 1-D arrays, strings as lists of str (fixed-length
    or variable-length, as libhdf5 writes the reference's ``input`` and
    ``metadata`` strings)."""
    with open(path, "rb") as fh:
        data = fh.read()
    r = _Reader(data)
    addr = r.root_ohdr
    if group:
        links = r.root_links()
        if group not in links:
            raise H5Error(f"group /{group} not found in {path}")
        addr = links[group]
    out: Dict[str, object] = {}
    for mtype, body in r.messages(addr):
        if mtype == 0x0C:
            name, val = _decode_attr(data, body)
            out[name] = val
    return out


def list_links(path: str) -> List[str]:
    """Names linked from the root group."""
    with open(path, "rb") as fh:
        return sorted(_Reader(fh.read()).root_links())


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
            # class 1 version 1; bit fields: little endian, mantissa normalisation 2 (implied
            # msb), sign bit at 63; properties: offset 0, precision 64, exponent at 52 (11 bits),
            # mantissa at 0 (52 bits), exponent bias 1023
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


def _dataspace(dims) -> bytes:
    # version 1, no maximum dimensions
    return struct.pack("<BBB5x", 1, len(dims), 0) + b"".join(struct.pack("<Q", x) for x in dims)


def _attr_msg(name: str, value) -> bytes:
    """Attribute message (version 1).  int -> 32-bit signed scalar [1],
    float -> double [1], str / list of str -> fixed-length null-terminated
    ASCII strings, numpy array -> its dtype and shape."""
    if isinstance(value, str):
        value = [value]
    if isinstance(value, (list, tuple)) and all(isinstance(v, str) for v in value):
        enc = [v.encode() for v in value]
        width = max(1, max(len(e) for e in enc) + 1)
        dt_body = struct.pack("<B3BI", 0x13, 0x00, 0, 0, width)
        ds_body = _dataspace([len(enc)])
        data = b"".join(e.ljust(width, b"\x00") for e in enc)
    else:
        if isinstance(value, bool):
            arr = np.array([int(value)], np.int32)
        elif isinstance(value, int):
            arr = np.array([value], np.int32)
        elif isinstance(value, float):
            arr = np.array([value], np.float64)
        else:
            arr = np.ascontiguousarray(value)
            if arr.ndim == 0:
                arr = arr.reshape(1)
        dt_body = _dtype_msg(arr.dtype)
        ds_body = _dataspace(list(arr.shape))
        data = arr.tobytes()
    nm = name.encode() + b"\x00"
    body = struct.pack("<BBHHH", 1, 0, len(nm), len(dt_body), len(ds_body))
    body += _pad8(nm) + _pad8(dt_body) + _pad8(ds_body) + data
    return _msg(0x0C, body)


# superblock parameters: group leaf node K (symbols per node / 2) and internal node K
_K_LEAF = 4
_K_INTERNAL = 16
_BTREE_SIZE = 24 + (2 * _K_INTERNAL + 1) * 8 + 2 * _K_INTERNAL * 8
_SNOD_SIZE = 8 + 2 * _K_LEAF * 40


def write_file(path: str, datasets: Dict[str, np.ndarray], root_attrs: Optional[Dict[str, object]] = None,
               groups: Optional[Dict[str, Dict[str, object]]] = None) -> None:
    """Write an HDF5 file: ``datasets`` (contiguous, unfiltered, little
    endian) and attribute-only child ``groups`` below the root group, which
    carries ``root_attrs``.

    File layout (superblock version 0, version-1 object headers, symbol-table
    groups, as libhdf5 writes with its default file-creation properties):
    superblock, then per group its object header, B-tree node, local heap and
    symbol node, then per dataset its object header and raw data.
    """
    datasets = {k: np.ascontiguousarray(v) for k, v in datasets.items()}
    groups = dict(groups or {})
    root_attrs = dict(root_attrs or {})
    if len(datasets) + len(groups) > 2 * _K_LEAF:
        raise H5Error("too many links for one symbol node")

    def heap_of(names):
        blob = bytearray(b"\x00" * 8)  # offset 0: the empty name
        offs = {}
        for nm in names:
            offs[nm] = len(blob)
            blob += _pad8(nm.encode() + b"\x00")
        return bytes(blob), offs

    # sizes first (every address is 8 bytes, so no size depends on an address)
    root_names = sorted(list(datasets) + list(groups), key=lambda s: s.encode())
    root_heap, root_offs = heap_of(root_names)
    root_attr_msgs = b"".join(_attr_msg(k, v) for k, v in root_attrs.items())
    root_msgs_len = len(_msg(0x11, b"\x00" * 16)) + len(root_attr_msgs)

    addr = 96
    root_ohdr = addr
    addr += 16 + root_msgs_len
    root_btree = addr
    addr += _BTREE_SIZE
    root_heap_hdr = addr
    addr += 32
    root_heap_data = addr
    addr += len(root_heap)
    root_snod = addr
    addr += _SNOD_SIZE

    gmeta = {}
    for g in sorted(groups, key=lambda s: s.encode()):
        msgs = b"".join(_attr_msg(k, v) for k, v in groups[g].items())
        heap, _ = heap_of([])
        ent = {"attrs": msgs, "ohdr": addr}
        addr += 16 + len(_msg(0x11, b"\x00" * 16)) + len(msgs)
        ent["btree"] = addr
        addr += _BTREE_SIZE
        ent["heap_hdr"] = addr
        addr += 32
        ent["heap_data"] = addr
        ent["heap"] = heap
        addr += len(heap)
        gmeta[g] = ent

    dmeta = {}
    for nm in sorted(datasets, key=lambda s: s.encode()):
        arr = datasets[nm]
        if arr.dtype.byteorder == ">":
            raise H5Error("big-endian arrays unsupported")
        msgs_wo_layout = _msg(0x01, _dataspace(list(arr.shape)), 1) + _msg(0x03, _dtype_msg(arr.dtype), 1)
        layout_len = len(_msg(0x08, struct.pack("<BBQQ", 3, 1, 0, 0)))
        ent = {"ohdr": addr, "msgs": msgs_wo_layout}
        addr += 16 + len(msgs_wo_layout) + layout_len
        addr += (-addr) % 8
        ent["data"] = addr
        addr += arr.nbytes
        addr += (-addr) % 8
        dmeta[nm] = ent
    eof = addr

    out = bytearray()

    def ohdr(msgs: bytes, nmsgs: int) -> bytes:
        return struct.pack("<BBHII4x", 1, 0, nmsgs, 1, len(msgs)) + msgs

    def btree(snod: Optional[int], last_key: int) -> bytes:
        if snod is None:  # empty group: a leaf with no entries
            bt = b"TREE" + struct.pack("<BBHQQ", 0, 0, 0, _UNDEF, _UNDEF) + struct.pack("<Q", 0)
        else:
            bt = b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, _UNDEF, _UNDEF)
            bt += struct.pack("<QQQ", 0, snod, last_key)
        return bt.ljust(_BTREE_SIZE, b"\x00")

    def heap_hdr(size: int, data_addr: int) -> bytes:
        return b"HEAP" + struct.pack("<B3xQQQ", 0, size, _UNDEF, data_addr)

    # superblock v0 and the root group's symbol table entry (cache type 1)
    out += _SIG
    out += struct.pack("<BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0)
    out += struct.pack("<HHI", _K_LEAF, _K_INTERNAL, 0)
    out += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
    out += struct.pack("<QQII", 0, root_ohdr, 1, 0) + struct.pack("<QQ", root_btree, root_heap_hdr)
    assert len(out) == root_ohdr
    out += ohdr(_msg(0x11, struct.pack("<QQ", root_btree, root_heap_hdr)) + root_attr_msgs, 1 + len(root_attrs))
    out += btree(root_snod if root_names else None, root_offs[root_names[-1]] if root_names else 0)
    out += heap_hdr(len(root_heap), root_heap_data) + root_heap
    sn = b"SNOD" + struct.pack("<BBH", 1, 0, len(root_names))
    for nm in root_names:
        if nm in gmeta:
            g = gmeta[nm]
            sn += struct.pack("<QQII", root_offs[nm], g["ohdr"], 1, 0) + struct.pack("<QQ", g["btree"], g["heap_hdr"])
        else:
            sn += struct.pack("<QQII", root_offs[nm], dmeta[nm]["ohdr"], 0, 0) + b"\x00" * 16
    out += sn.ljust(_SNOD_SIZE, b"\x00")
    for nm in sorted(groups, key=lambda s: s.encode()):
        g = gmeta[nm]
        assert len(out) == g["ohdr"]
        out += ohdr(_msg(0x11, struct.pack("<QQ", g["btree"], g["heap_hdr"])) + g["attrs"], 1 + len(groups[nm]))
        out += btree(None, 0)
        out += heap_hdr(len(g["heap"]), g["heap_data"]) + g["heap"]
    for nm in sorted(datasets, key=lambda s: s.encode()):
        arr, ent = datasets[nm], dmeta[nm]
        assert len(out) == ent["ohdr"]
        msgs = ent["msgs"] + _msg(0x08, struct.pack("<BBQQ", 3, 1, ent["data"], arr.nbytes))
        out += ohdr(msgs, 3)
        out += b"\x00" * (ent["data"] - len(out))
        out += arr.tobytes()
        out += b"\x00" * ((-len(out)) % 8)
    assert len(out) == eof
    with open(path, "wb") as fh:
        fh.write(bytes(out))


def write_field(path: str, arr: np.ndarray, input_lines: Optional[List[str]] = None,
                metadata: Optional[Dict[str, object]] = None,
                globals_: Optional[Dict[str, object]] = None) -> None:
    """Write ``arr`` as ``/OutArray`` the way ``dumpFieldHDF5`` lays a field
    out (``src/dlbc/io/hdf5.d:125-285``): native double (or 32-bit int for
    the mask), global dims with the vector/population component fastest.

    ``input_lines`` become the root attribute ``input`` (the parameter file
    lines, ``hdf5.d:529-548``), ``metadata`` the attributes of group
    ``/metadata`` (``hdf5.d:290-299``) and ``globals_`` those of group
    ``/globals`` (checkpoint files only, ``src/dlbc/io/checkpoint.d:248-313``,
    e.g. ``{"dlbc.lb.lb.timestep": t}``).
    """
    arr = np.ascontiguousarray(arr)
    if arr.dtype.kind in "iub":
        arr = arr.astype(np.int32)
    elif arr.dtype != np.float64:
        arr = arr.astype(np.float64)
    root = {"input": list(input_lines)} if input_lines else {}
    groups: Dict[str, Dict[str, object]] = {}
    if metadata is not None:
        groups["metadata"] = metadata
    if globals_ is not None:
        groups["globals"] = globals_
    write_file(path, {"OutArray": arr}, root, groups)


