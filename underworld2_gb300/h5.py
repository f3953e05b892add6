"""HDF5 files for checkpoints, written and read without libhdf5.

The reference saves meshes, mesh variables, swarms and swarm variables through
h5py (P/mesh/_mesh.py:495-601, P/mesh/_meshvariable.py:330-470,
P/swarm/_swarm.py:226-420, P/swarm/_swarmvariable.py:244-500): one file per
object, datasets in the root group ("vertices", "en_map", "data") and root
attributes.  Neither h5py nor libhdf5 is part of this package's environment, so
this module writes that subset of the HDF5 file format itself, following the
published format specification (version 0 superblock, version 1 object
headers, an old-style root group indexed by a version 1 B-tree, one symbol
table node and a local heap; contiguous datasets; attributes in the root
object header) -- the layout libhdf5 produces with its default "earliest"
format bounds.  The reader parses the same structures, plus what libhdf5 adds
to such files: header continuation blocks, multi-node group B-trees, version 2
dataspaces, variable-length string attributes in global heaps, and root groups
in compact new-style storage (link-info and link messages: hard, soft and
external links), which is how h5py stores a file holding an external link.
Chunked or filtered datasets and dense link storage are not supported and
raise ``NotImplementedError``.

Values are little-endian.  Python ``bool`` attributes are stored as int8 and
``str`` attributes as fixed-length null-terminated ASCII strings (h5py returns
those as ``bytes``).  External links (the reference's "mesh"/"swarm" links
from a variable's file to its mesh or swarm file) are not representable in an
old-style group; the link target is kept as a string attribute of that name.
"""
import struct

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF
_HEAP_FREE_NULL = 1          # "no free block" offset of a local heap free list
_LEAF_K = 4                  # symbol table node holds 2K entries
_INTERNAL_K = 16             # group B-tree node holds 2K children
_ENTRY = 40                  # symbol table entry size with 8-byte offsets


def _pad8(n):
    return (n + 7) & ~7


def _padded(b):
    return b + b"\0" * (_pad8(len(b)) - len(b))


# --------------------------------------------------------------------------
# datatype, dataspace and message encoders
# --------------------------------------------------------------------------
def _dtype_msg(dt):
    dt = np.dtype(dt)
    if dt.kind == "f":
        if dt.itemsize == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            sign = 63
        elif dt.itemsize == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            sign = 31
        else:
            raise TypeError("unsupported float size %d" % dt.itemsize)
        return bytes([0x10 | 1, 0x20, sign, 0]) + struct.pack("<I", dt.itemsize) + props
    if dt.kind in "iub":
        signed = 0x08 if dt.kind == "i" else 0
        return bytes([0x10 | 0, signed, 0, 0]) + struct.pack("<I", dt.itemsize) + \
            struct.pack("<HH", 0, 8 * dt.itemsize)
    if dt.kind == "S":
        return bytes([0x10 | 3, 0x00, 0, 0]) + struct.pack("<I", dt.itemsize)
    raise TypeError("unsupported dtype %s" % dt)


def _space_msg(shape):
    out = bytes([1, len(shape), 0, 0]) + b"\0" * 4
    for n in shape:
        out += struct.pack("<Q", int(n))
    return out


def _message(mtype, body, flags=0):
    body = _padded(body)
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _attr_value(v):
    """(numpy array, shape) of an attribute value as it is stored."""
    if isinstance(v, (bytes, np.bytes_)):
        b = bytes(v) + b"\0"
        return np.frombuffer(b, dtype="S%d" % len(b)), ()
    if isinstance(v, str):
        return _attr_value(v.encode("ascii", "replace"))
    if isinstance(v, (bool, np.bool_)):
        return np.array(int(v), dtype=np.int8), ()
    a = np.asarray(v)
    if a.dtype.kind == "b":
        a = a.astype(np.int8)
    elif a.dtype.kind == "U":
        a = a.astype("S")
    if a.dtype.kind == "S":
        a = a.astype("S%d" % (a.dtype.itemsize + 1))
    return np.ascontiguousarray(a.astype(a.dtype.newbyteorder("<"))), a.shape


def _attr_msg(name, value):
    a, shape = _attr_value(value)
    nm = name.encode("ascii") + b"\0"
    dt = _dtype_msg(a.dtype)
    sp = _space_msg(shape)
    body = struct.pack("<BxHHH", 1, len(nm), len(dt), len(sp)) + _padded(nm) + _padded(dt) + _padded(sp) + \
        a.tobytes()
    return _message(0x000C, body)


def _object_header(messages):
    blob = b"".join(messages)
    return struct.pack("<BxHII4x", 1, len(messages), 1, len(blob)) + blob


# --------------------------------------------------------------------------
# writer
# --------------------------------------------------------------------------
def write(path, datasets, attrs=None):
    """Write ``datasets`` (name -> array) into the root group of a new file at
    ``path``, with root attributes ``attrs`` (name -> scalar, sequence or
    string)."""
    names = sorted(datasets)
    if len(names) > 2 * _LEAF_K:
        raise ValueError("at most %d datasets per file" % (2 * _LEAF_K))
    arrays = {n: np.ascontiguousarray(np.asarray(datasets[n])) for n in names}
    for n, a in arrays.items():
        if a.dtype.byteorder == ">":
            arrays[n] = a.astype(a.dtype.newbyteorder("<"))
    # local heap: "" at offset 0, then the names
    heap = bytearray(b"\0" * 8)
    name_off = {}
    for n in names:
        name_off[n] = len(heap)
        heap += _padded(n.encode("ascii") + b"\0")
    heap_data = bytes(heap)

    root_attr_msgs = [_attr_msg(k, v) for k, v in (attrs or {}).items()]
    # sizes of the fixed structures
    sb_size = 96
    root_oh_size = 16 + len(_message(0x0011, b"\0" * 16)) + sum(len(m) for m in root_attr_msgs)
    btree_size = 24 + 2 * _INTERNAL_K * 8 + (2 * _INTERNAL_K + 1) * 8
    snod_size = 8 + 2 * _LEAF_K * _ENTRY
    heap_hdr = 32
    a_root = sb_size
    a_btree = a_root + _pad8(root_oh_size)
    a_snod = a_btree + btree_size
    a_heap = a_snod + snod_size
    a_heap_data = a_heap + heap_hdr
    pos = a_heap_data + _pad8(len(heap_data))
    # dataset object headers, then raw data
    ds_hdr_len = {}
    for n in names:
        a = arrays[n]
        msgs = [_message(0x0001, _space_msg(a.shape)), _message(0x0003, _dtype_msg(a.dtype)),
                _message(0x0005, bytes([2, 2, 2, 0])), _message(0x0008, b"\0" * 18)]
        ds_hdr_len[n] = 16 + sum(len(m) for m in msgs)
    a_ds = {}
    for n in names:
        a_ds[n] = pos
        pos += _pad8(ds_hdr_len[n])
    a_raw = {}
    for n in names:
        a_raw[n] = pos if arrays[n].nbytes else _UNDEF
        pos += _pad8(arrays[n].nbytes)
    eof = pos

    out = bytearray(eof)
    # superblock
    sb = _SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", _LEAF_K, _INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
    sb += struct.pack("<QQII", 0, a_root, 1, 0) + struct.pack("<QQ", a_btree, a_heap)
    out[0:len(sb)] = sb
    # root group object header: symbol table message + attributes
    root = _object_header([_message(0x0011, struct.pack("<QQ", a_btree, a_heap))] + root_attr_msgs)
    out[a_root:a_root + len(root)] = root
    # B-tree: one leaf child (the symbol table node)
    bt = b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", 1 if names else 0, _UNDEF, _UNDEF)
    if names:
        bt += struct.pack("<QQQ", 0, a_snod, name_off[names[-1]])
    out[a_btree:a_btree + len(bt)] = bt
    # symbol table node
    sn = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(names))
    for n in names:
        sn += struct.pack("<QQII16x", name_off[n], a_ds[n], 0, 0)
    out[a_snod:a_snod + len(sn)] = sn
    # local heap
    hp = b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", _pad8(len(heap_data)), _HEAP_FREE_NULL, a_heap_data)
    out[a_heap:a_heap + len(hp)] = hp
    out[a_heap_data:a_heap_data + len(heap_data)] = heap_data
    # datasets
    for n in names:
        a = arrays[n]
        layout = struct.pack("<BBQQ", 3, 1, a_raw[n], a.nbytes)
        msgs = [_message(0x0001, _space_msg(a.shape)), _message(0x0003, _dtype_msg(a.dtype)),
                _message(0x0005, bytes([2, 2, 2, 0])), _message(0x0008, layout)]
        oh = _object_header(msgs)
        out[a_ds[n]:a_ds[n] + len(oh)] = oh
        if a.nbytes:
            out[a_raw[n]:a_raw[n] + a.nbytes] = a.tobytes()
    with open(path, "wb") as f:
        f.write(out)


# --------------------------------------------------------------------------
# reader
# --------------------------------------------------------------------------
class _Reader:
    def __init__(self, buf):
        self.b = buf

    def u(self, fmt, off):
        return struct.unpack_from("<" + fmt, self.b, off)

    # datatype -> (numpy dtype or a tag, size)
    def dtype(self, off):
        cv, b0, b1, b2, size = self.u("BBBBI", off)
        cls = cv & 0x0F
        big = b0 & 1
        end = ">" if big else "<"
        if cls == 0:
            return np.dtype("%s%s%d" % (end, "i" if b0 & 0x08 else "u", size))
        if cls == 1:
            return np.dtype("%sf%d" % (end, size))
        if cls == 3:
            return np.dtype("S%d" % size)
        if cls == 9:
            vtype = b0 & 0x0F
            if vtype == 1:
                return "vlen_str"
            raise NotImplementedError("variable-length sequences")
        if cls == 8:   # enumeration (h5py booleans): the base type
            return self.dtype(off + 8)
        raise NotImplementedError("HDF5 datatype class %d" % cls)

    def space(self, off):
        ver, rank, flags = self.u("BBB", off)
        if ver == 1:
            p = off + 8
        elif ver == 2:
            stype = self.u("B", off + 3)[0]
            if stype == 2:
                return None
            p = off + 4
        else:
            raise NotImplementedError("dataspace version %d" % ver)
        return tuple(self.u("Q", p + 8 * i)[0] for i in range(rank))

    def messages(self, addr):
        """(type, body offset, size) of every message of the object header at addr."""
        ver = self.b[addr]
        out = []
        if ver == 1:
            nmsg, _, size = self.u("HII", addr + 2)
            blocks = [(addr + 16, size)]
            while blocks and len(out) < nmsg:
                start, length = blocks.pop(0)
                p = start
                while p + 8 <= start + length and len(out) < nmsg:
                    mtype, msize, _ = self.u("HHB", p)
                    out.append((mtype, p + 8, msize))
                    if mtype == 0x0010:
                        blocks.append(self.u("QQ", p + 8))
                    p += 8 + msize
            return out
        if self.b[addr:addr + 4] == b"OHDR":
            raise NotImplementedError("version 2 object headers")
        raise ValueError("bad object header at %d" % addr)

    def link(self, off):
        """(name, type, value) of a link message: type 0 (hard, value = object
        header address), 1 (soft, value = ("", path)) or 64 (external, value =
        (file name, object path))."""
        ver, flags = self.u("BB", off)
        if ver != 1:
            raise NotImplementedError("link message version %d" % ver)
        p = off + 2
        kind = 0
        if flags & 0x08:
            kind = self.b[p]
            p += 1
        if flags & 0x04:
            p += 8                                   # creation order
        if flags & 0x10:
            p += 1                                   # name character set
        nlen_size = 1 << (flags & 0x03)
        nlen = int.from_bytes(bytes(self.b[p:p + nlen_size]), "little")
        p += nlen_size
        name = bytes(self.b[p:p + nlen]).decode("utf-8")
        p += nlen
        if kind == 0:
            return name, 0, self.u("Q", p)[0]
        length = self.u("H", p)[0]
        body = bytes(self.b[p + 2:p + 2 + length])
        if kind == 1:
            return name, 1, ("", body.rstrip(b"\0").decode("utf-8"))
        if kind == 64:
            parts = body[1:].split(b"\0")           # version/flags byte, file name, object path
            return name, 64, (parts[0].decode("utf-8"), parts[1].decode("utf-8") if len(parts) > 1 else "/")
        raise NotImplementedError("link type %d" % kind)

    def heap_string(self, heap_addr, off):
        assert self.b[heap_addr:heap_addr + 4] == b"HEAP"
        data = self.u("Q", heap_addr + 24)[0]
        p = data + off
        e = self.b.index(b"\0", p)
        return bytes(self.b[p:e]).decode("ascii")

    def group_entries(self, btree, heap):
        sig = bytes(self.b[btree:btree + 4])
        if sig != b"TREE":
            raise ValueError("bad group B-tree")
        ntype, level, used = self.u("BBH", btree + 4)
        ents = {}
        p = btree + 24
        for i in range(used):
            child = self.u("Q", p + 8 + 16 * i)[0]
            if level > 0:
                ents.update(self.group_entries(child, heap))
                continue
            assert self.b[child:child + 4] == b"SNOD"
            nsym = self.u("H", child + 6)[0]
            for k in range(nsym):
                e = child + 8 + _ENTRY * k
                noff, oh = self.u("QQ", e)
                ents[self.heap_string(heap, noff)] = oh
        return ents

    def gheap_object(self, addr, index):
        assert self.b[addr:addr + 4] == b"GCOL"
        size = self.u("Q", addr + 8)[0]
        p = addr + 16
        while p < addr + size:
            idx, _, osize = self.u("HH4xQ", p)
            if idx == 0:
                break
            if idx == index:
                return bytes(self.b[p + 16:p + 16 + osize])
            p += 16 + _pad8(osize)
        raise KeyError("global heap object %d" % index)

    def values(self, dt, shape, off):
        n = int(np.prod(shape)) if shape else 1
        if dt == "vlen_str":
            vals = []
            for i in range(n):
                ln, addr, idx = self.u("IQI", off + 16 * i)
                vals.append(self.gheap_object(addr, idx)[:ln].decode("utf-8") if ln else "")
            return vals[0] if not shape else np.array(vals, dtype=object).reshape(shape)
        a = np.frombuffer(self.b, dtype=dt, count=n, offset=off).copy()
        if dt.kind == "S":
            a = np.array([s.rstrip(b"\0") for s in a], dtype=dt)
        return a[0] if not shape else a.reshape(shape)

    def attribute(self, off):
        ver = self.b[off]
        if ver == 1:
            nlen, dtlen, splen = self.u("HHH", off + 2)
            p = off + 8
            name = bytes(self.b[p:p + nlen - 1]).decode("ascii")
            p += _pad8(nlen)
            dt = self.dtype(p)
            p += _pad8(dtlen)
            shape = self.space(p)
            p += _pad8(splen)
        elif ver in (2, 3):
            nlen, dtlen, splen = self.u("HHH", off + 2)
            p = off + 8 + (1 if ver == 3 else 0)
            name = bytes(self.b[p:p + nlen - 1]).decode("utf-8")
            p += nlen
            dt = self.dtype(p)
            p += dtlen
            shape = self.space(p)
            p += splen
        else:
            raise NotImplementedError("attribute message version %d" % ver)
        return name, self.values(dt, shape, p)


class File:
    """Read-only view of a file: ``attrs`` (dict) and ``f[name]`` -> array for
    the datasets of the root group (``keys()`` lists them)."""

    def __init__(self, path):
        with open(path, "rb") as fh:
            self._r = _Reader(fh.read())
        r = self._r
        if bytes(r.b[0:8]) != _SIG:
            raise ValueError("'%s' is not an HDF5 file" % path)
        if r.b[8] not in (0, 1):
            raise NotImplementedError("superblock version %d" % r.b[8])
        ent = 56 if r.b[8] == 0 else 60
        root = r.u("Q", ent + 8)[0]
        self.attrs = {}
        self._entries = {}
        self.links = {}          # soft and external links: name -> (file name or "", object path)
        for mtype, off, size in r.messages(root):
            if mtype == 0x0011:
                bt, hp = r.u("QQ", off)
                self._entries = r.group_entries(bt, hp)
            elif mtype == 0x000C:
                k, v = r.attribute(off)
                self.attrs[k] = v
            elif mtype == 0x0002:
                flags = r.b[off + 1]
                heap = r.u("Q", off + 2 + (8 if flags & 1 else 0))[0]
                if heap != _UNDEF:
                    raise NotImplementedError("dense link storage (fractal heap)")
            elif mtype == 0x0006:
                name, kind, value = r.link(off)
                if kind == 0:
                    self._entries[name] = value
                else:
                    self.links[name] = value

    def keys(self):
        return list(self._entries)

    def __contains__(self, k):
        return k in self._entries

    def __getitem__(self, name):
        r = self._r
        shape = dt = addr = None
        size = 0
        for mtype, off, msize in r.messages(self._entries[name]):
            if mtype == 0x0001:
                shape = r.space(off)
            elif mtype == 0x0003:
                dt = r.dtype(off)
            elif mtype == 0x0008:
                ver, cls = r.u("BB", off)
                if ver != 3:
                    raise NotImplementedError("layout message version %d" % ver)
                if cls == 1:
                    addr, size = r.u("QQ", off + 2)
                elif cls == 0:
                    size = r.u("H", off + 2)[0]
                    addr = off + 4
                else:
                    raise NotImplementedError("chunked datasets")
            elif mtype == 0x000B:
                raise NotImplementedError("filtered datasets")
        if shape is None or dt is None:
            raise ValueError("dataset '%s' lacks a dataspace or datatype" % name)
        n = int(np.prod(shape)) if shape else 1
        if n == 0 or addr == _UNDEF:
            return np.zeros(shape, dtype=dt)
        return np.frombuffer(r.b, dtype=dt, count=n, offset=addr).copy().reshape(shape)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False
