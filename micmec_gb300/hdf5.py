"""Reading and writing HDF5 files in the classic on-disk format, without h5py.

The reference stores systems and trajectories in HDF5 through h5py
(micmec/system.py:262-370 ``from_hdf5`` / ``to_hdf5``; micmec/sampling/trajectory.py:31-85
``HDF5Writer``). h5py and the HDF5 library are not available here, so this module writes and
reads the file format itself, as published in the HDF5 File Format Specification:

* superblock version 0 (8-byte offsets and lengths, group leaf node K 4, internal node K 16);
* groups as symbol tables: a version-1 B-tree of group nodes (one level, up to 32 symbol
  table nodes of up to 8 entries each, so up to 256 members per group), symbol table nodes
  and a local heap of member names;
* version-1 object headers with dataspace (version 1), datatype (version 1: IEEE floats,
  two's-complement integers, fixed-length strings), fill value (version 2) and layout
  (version 3, contiguous) messages, and version-1 attribute messages;

which is the layout the HDF5 library itself writes by default ("earliest" file format),
so that h5py and the reference's ``System.from_hdf5`` read these files. The reader also takes
what that library writes for small files in the same format family: object-header
continuation blocks, multi-level group B-trees, version-2 dataspaces, layout messages of
versions 1 to 3 (contiguous or compact), attribute messages of versions 1 to 3, and a user
block before the superblock. Chunked or compressed datasets, variable-length types and the
newer superblock / object header versions are refused with an error.
"""

import struct

import numpy as np

__all__ = ["HGroup", "HDataset", "read", "write", "is_hdf5"]

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
_LEAF_K, _INTERNAL_K = 4, 16
_SNOD_CAP = 2 * _LEAF_K            # entries per symbol table node
_BTREE_CAP = 2 * _INTERNAL_K       # children per group B-tree node
_ENTRY = 40                        # symbol table entry
_SNOD_SIZE = 8 + _SNOD_CAP * _ENTRY
_BTREE_SIZE = 24 + (2 * _INTERNAL_K + 1) * 8 + 2 * _INTERNAL_K * 8
_HEAP_FREE_NULL = 1                # end of a local heap's free list on disk


class HDataset(object):
    """An array and its attributes."""

    def __init__(self, data, attrs=None):
        self.data = data
        self.attrs = dict(attrs or {})


class HGroup(object):
    """Members (name -> HGroup or HDataset) and attributes."""

    def __init__(self, members=None, attrs=None):
        self.members = dict(members or {})
        self.attrs = dict(attrs or {})


def _pad8(n):
    return (n + 7) & ~7


# ------------------------------------------------------------------ datatypes

def _le(a):
    a = np.asarray(a)
    if a.dtype.byteorder == ">" or (a.dtype.byteorder == "=" and not np.little_endian):
        a = a.astype(a.dtype.newbyteorder("<"))
    return a


def _storable(a):
    """The array as stored: little-endian numbers, bools as uint8, str as UTF-8 bytes."""
    a = np.asarray(a)
    if a.dtype == np.bool_:
        return a.astype(np.uint8), 0
    if a.dtype.kind == "U":
        enc = np.char.encode(a, "utf-8") if a.size else a.astype("S1")
        width = max(1, int(enc.dtype.itemsize))
        return np.asarray(enc, dtype="S%d" % width), 1
    if a.dtype.kind == "S":
        return a if a.dtype.itemsize else a.astype("S1"), 0
    if a.dtype.kind in "iuf":
        return _le(a), 0
    raise TypeError("cannot store dtype %s in HDF5" % a.dtype)


def _datatype_message(dtype, cset=0):
    size = dtype.itemsize
    if dtype.kind == "f":
        if size == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            bits = (0x20, 63, 0)
        elif size == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            bits = (0x20, 31, 0)
        else:
            raise TypeError("float size %d" % size)
        return struct.pack("<BBBBI", 0x11, *bits, size) + props
    if dtype.kind in "iu":
        signed = 0x08 if dtype.kind == "i" else 0
        return struct.pack("<BBBBI", 0x10, signed, 0, 0, size) + struct.pack("<HH", 0, 8 * size)
    if dtype.kind == "S":
        return struct.pack("<BBBBI", 0x13, 0x01 | (cset << 4), 0, 0, size)  # null-padded
    raise TypeError("cannot store dtype %s in HDF5" % dtype)


def _parse_datatype(buf, off):
    """(numpy dtype, is_utf8) of a datatype message at off."""
    cv, b0, b1, b2, size = struct.unpack_from("<BBBBI", buf, off)
    cls, ver = cv & 0x0F, cv >> 4
    if ver not in (1, 2, 3):
        raise ValueError("datatype message version %d" % ver)
    if cls == 0:
        order = ">" if b0 & 1 else "<"
        return np.dtype("%s%s%d" % (order, "i" if b0 & 0x08 else "u", size)), False
    if cls == 1:
        order = ">" if b0 & 1 else "<"
        if size not in (2, 4, 8):
            raise ValueError("float of %d bytes" % size)
        return np.dtype("%sf%d" % (order, size)), False
    if cls == 3:
        return np.dtype("S%d" % size), bool((b0 >> 4) & 0x0F)
    raise ValueError("datatype class %d is not supported" % cls)


# ------------------------------------------------------------------ dataspaces

def _dataspace_message(shape):
    rank = len(shape)
    out = struct.pack("<BBBB4x", 1, rank, 0, 0)
    for d in shape:
        out += struct.pack("<Q", d)
    return out


def _parse_dataspace(buf, off):
    ver, rank, flags = struct.unpack_from("<BBB", buf, off)
    if ver == 1:
        p = off + 8
    elif ver == 2:
        kind = buf[off + 3]
        if kind == 2:  # null dataspace
            return None
        p = off + 4
    else:
        raise ValueError("dataspace message version %d" % ver)
    return tuple(struct.unpack_from("<%dQ" % rank, buf, p)) if rank else ()


# ------------------------------------------------------------------ writer

class _Writer(object):
    def __init__(self):
        self.chunks = []   # (address, bytes)
        self.eof = 96      # after the superblock

    def alloc(self, nbytes):
        addr = self.eof
        self.eof = _pad8(self.eof + nbytes)
        return addr

    def put(self, addr, data):
        self.chunks.append((addr, bytes(data)))

    @staticmethod
    def message(mtype, data, flags=0):
        body = bytes(data)
        body += b"\0" * (_pad8(len(body)) - len(body))
        return struct.pack("<HHB3x", mtype, len(body), flags) + body

    def object_header(self, messages):
        body = b"".join(messages)
        addr = self.alloc(16 + len(body))
        self.put(addr, struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body)
        return addr

    def attribute_messages(self, attrs):
        out = []
        for name, value in attrs.items():
            a, cset = _storable(value)
            nm = name.encode("utf-8") + b"\0"
            dt = _datatype_message(a.dtype, cset)
            ds = _dataspace_message(a.shape)
            body = struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(ds))
            for part in (nm, dt, ds):
                body += part + b"\0" * (_pad8(len(part)) - len(part))
            body += a.tobytes()
            out.append(self.message(0x000C, body))
        return out

    def dataset(self, ds):
        a, cset = _storable(ds.data)
        raw = a.tobytes()
        if raw:
            addr = self.alloc(len(raw))
            self.put(addr, raw)
        else:
            addr = UNDEF
        msgs = [self.message(0x0001, _dataspace_message(a.shape)),
                self.message(0x0003, _datatype_message(a.dtype, cset), flags=1),
                # fill value: version 2, allocation late, written if set, default value defined
                self.message(0x0005, struct.pack("<BBBBI", 2, 2, 2, 1, 0), flags=1),
                # layout: version 3, contiguous
                self.message(0x0008, struct.pack("<BBQQ", 3, 1, addr, len(raw)))]
        msgs += self.attribute_messages(ds.attrs)
        return self.object_header(msgs)

    def group(self, grp):
        """Writes the group's members and tables; returns (header address, B-tree, heap)."""
        names = sorted(grp.members, key=lambda s: s.encode("utf-8"))
        if len(names) > _SNOD_CAP * _BTREE_CAP:
            raise ValueError("a group with more than %d members is not supported" % (_SNOD_CAP * _BTREE_CAP))
        entries = []
        for name in names:
            item = grp.members[name]
            if isinstance(item, HGroup):
                oh, bt, hp = self.group(item)
                entries.append((name, oh, 1, (bt, hp)))
            else:
                entries.append((name, self.dataset(item), 0, (0, 0)))
        # local heap: "" at offset 0, the names, then one free block (as the HDF5 library leaves it)
        heap = bytearray(8)
        offsets = {}
        for name in names:
            offsets[name] = len(heap)
            nm = name.encode("utf-8") + b"\0"
            heap += nm + b"\0" * (_pad8(len(nm)) - len(nm))
        free_at = len(heap)
        heap += struct.pack("<QQ", _HEAP_FREE_NULL, 16)
        heap_hdr = self.alloc(32)
        heap_data = self.alloc(len(heap))
        self.put(heap_hdr, b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), free_at, heap_data))
        self.put(heap_data, heap)
        # symbol table nodes: entries spread evenly (at least 4 per node when there are two or more)
        nnodes = max(1, -(-len(entries) // _SNOD_CAP))
        per = [len(entries) // nnodes + (1 if i < len(entries) % nnodes else 0) for i in range(nnodes)]
        snods, keys, k = [], [0], 0
        for cnt in per:
            part = entries[k:k + cnt]
            k += cnt
            body = b"SNOD" + struct.pack("<BBH", 1, 0, len(part))
            for name, oh, cache, scratch in part:
                body += struct.pack("<QQII", offsets[name], oh, cache, 0) + struct.pack("<QQ", *scratch)
            body += b"\0" * (_SNOD_SIZE - len(body))
            addr = self.alloc(_SNOD_SIZE)
            self.put(addr, body)
            snods.append(addr)
            keys.append(offsets[part[-1][0]] if part else 0)
        # group B-tree: one leaf level over the symbol table nodes
        body = b"TREE" + struct.pack("<BBHQQ", 0, 0, len(snods), UNDEF, UNDEF)
        for i, addr in enumerate(snods):
            body += struct.pack("<QQ", keys[i], addr)
        body += struct.pack("<Q", keys[len(snods)])
        body += b"\0" * (_BTREE_SIZE - len(body))
        btree = self.alloc(_BTREE_SIZE)
        self.put(btree, body)
        msgs = [self.message(0x0011, struct.pack("<QQ", btree, heap_hdr), flags=1)]
        msgs += self.attribute_messages(grp.attrs)
        return self.object_header(msgs), btree, heap_hdr


def write(filename, root):
    """Write the HGroup tree ``root`` as an HDF5 file."""
    w = _Writer()
    oh, btree, heap = w.group(root)
    sb = SIGNATURE + struct.pack("<BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0)
    sb += struct.pack("<HHI", _LEAF_K, _INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, w.eof, UNDEF)
    sb += struct.pack("<QQII", 0, oh, 1, 0) + struct.pack("<QQ", btree, heap)
    assert len(sb) == 96
    out = bytearray(w.eof)
    out[:96] = sb
    for addr, data in w.chunks:
        out[addr:addr + len(data)] = data
    with open(filename, "wb") as f:
        f.write(out)


# ------------------------------------------------------------------ reader

def _find_superblock(buf):
    off = 0
    while off + 8 <= len(buf):  # at 0, 512, 1024, 2048, ... (after a user block)
        if buf[off:off + 8] == SIGNATURE:
            return off
        off = 512 if off == 0 else 2 * off
    return -1


def is_hdf5(filename):
    with open(filename, "rb") as f:
        head = f.read(1 << 16)
    return _find_superblock(head) >= 0


class _Reader(object):
    def __init__(self, buf):
        self.buf = buf
        sb = _find_superblock(buf)
        if sb < 0:
            raise ValueError("not an HDF5 file")
        ver = buf[sb + 8]
        if ver not in (0, 1):
            raise ValueError("superblock version %d is not supported" % ver)
        if buf[sb + 13] != 8 or buf[sb + 14] != 8:
            raise ValueError("only 8-byte offsets and lengths are supported")
        p = sb + 24 + (4 if ver == 1 else 0)
        self.base = struct.unpack_from("<Q", buf, p)[0]
        self.root_entry = p + 32

    def at(self, addr):
        return self.base + addr

    def messages(self, addr):
        buf = self.buf
        p = self.at(addr)
        ver, _, nmsg, _, size = struct.unpack_from("<BBHII", buf, p)
        if ver != 1:
            raise ValueError("object header version %d is not supported" % ver)
        blocks = [(p + 16, size)]
        out = []
        while blocks:
            q, sz = blocks.pop(0)
            end = q + sz
            while q + 8 <= end:
                mtype, msize, flags = struct.unpack_from("<HHB", buf, q)
                data = q + 8
                if mtype == 0x0010:  # continuation
                    caddr, clen = struct.unpack_from("<QQ", buf, data)
                    blocks.append((self.at(caddr), clen))
                elif mtype != 0:
                    if flags & 0x02:
                        raise ValueError("shared object header messages are not supported")
                    out.append((mtype, data, flags))
                q = data + msize
        return out

    def heap_name(self, heap_addr, off):
        p = self.at(heap_addr)
        if self.buf[p:p + 4] != b"HEAP":
            raise ValueError("bad local heap")
        data = struct.unpack_from("<Q", self.buf, p + 24)[0]
        s = self.at(data) + off
        e = self.buf.index(b"\0", s)
        return self.buf[s:e].decode("utf-8")

    def btree_entries(self, btree, heap):
        buf = self.buf
        p = self.at(btree)
        if buf[p:p + 4] != b"TREE" or buf[p + 4] != 0:
            raise ValueError("bad group B-tree")
        level = buf[p + 5]
        nent = struct.unpack_from("<H", buf, p + 6)[0]
        q = p + 24
        for i in range(nent):
            child = struct.unpack_from("<Q", buf, q + 8)[0]
            q += 16
            if level > 0:
                yield from self.btree_entries(child, heap)
                continue
            s = self.at(child)
            if buf[s:s + 4] != b"SNOD":
                raise ValueError("bad symbol table node")
            nsym = struct.unpack_from("<H", buf, s + 6)[0]
            for k in range(nsym):
                e = s + 8 + _ENTRY * k
                name_off, oh = struct.unpack_from("<QQ", buf, e)
                yield self.heap_name(heap, name_off), oh

    def attribute(self, data, flags):
        buf = self.buf
        ver = buf[data]
        if ver == 1:
            nlen, tlen, slen = struct.unpack_from("<HHH", buf, data + 2)
            p = data + 8
            name = buf[p:p + nlen].split(b"\0")[0].decode("utf-8")
            p += _pad8(nlen)
            tp = p
            p += _pad8(tlen)
            sp = p
            p += _pad8(slen)
        elif ver in (2, 3):
            nlen, tlen, slen = struct.unpack_from("<HHH", buf, data + 2)
            p = data + 8 + (1 if ver == 3 else 0)
            name = buf[p:p + nlen].split(b"\0")[0].decode("utf-8")
            tp = p + nlen
            sp = tp + tlen
            p = sp + slen
        else:
            raise ValueError("attribute message version %d" % ver)
        dtype, utf8 = _parse_datatype(buf, tp)
        shape = _parse_dataspace(buf, sp)
        if shape is None:
            return name, None
        n = int(np.prod(shape)) if shape else 1
        arr = np.frombuffer(buf, dtype=dtype, count=n, offset=p).reshape(shape).copy()
        return name, _decoded(arr, utf8)

    def obj(self, addr):
        msgs = self.messages(addr)
        attrs = {}
        stab = shape = dtype = layout = None
        utf8 = False
        for mtype, data, flags in msgs:
            if mtype == 0x0011:
                stab = struct.unpack_from("<QQ", self.buf, data)
            elif mtype == 0x0001:
                shape = _parse_dataspace(self.buf, data)
            elif mtype == 0x0003:
                dtype, utf8 = _parse_datatype(self.buf, data)
            elif mtype == 0x0008:
                layout = data
            elif mtype == 0x000C:
                name, value = self.attribute(data, flags)
                attrs[name] = value
            elif flags & 0x08:
                raise ValueError("object header message type 0x%x must be understood" % mtype)
        if stab is not None:
            g = HGroup(attrs=attrs)
            for name, oh in self.btree_entries(*stab):
                g.members[name] = self.obj(oh)
            return g
        if dtype is None or layout is None:
            raise ValueError("object at %d is neither a group nor a dataset" % addr)
        return HDataset(_decoded(self.layout_data(layout, dtype, shape or ()), utf8), attrs)

    def layout_data(self, p, dtype, shape):
        buf = self.buf
        ver = buf[p]
        n = int(np.prod(shape)) if shape else 1
        if ver in (1, 2):
            rank, cls = buf[p + 1], buf[p + 2]
            q = p + 8
            if cls == 1:
                addr = struct.unpack_from("<Q", buf, q)[0]
                start = None if addr == UNDEF else self.at(addr)
            elif cls == 0:
                q += 4 * rank
                start = q + 4  # compact: size (4) then the data
            else:
                raise ValueError("chunked datasets are not supported")
        elif ver == 3:
            cls = buf[p + 1]
            if cls == 1:
                addr = struct.unpack_from("<Q", buf, p + 2)[0]
                start = None if addr == UNDEF else self.at(addr)
            elif cls == 0:
                start = p + 4
            else:
                raise ValueError("chunked datasets are not supported")
        else:
            raise ValueError("layout message version %d is not supported" % ver)
        if start is None or n == 0:
            return np.zeros(shape, dtype=dtype)
        return np.frombuffer(buf, dtype=dtype, count=n, offset=start).reshape(shape).copy()


def _decoded(arr, utf8):
    if utf8 and arr.dtype.kind == "S":
        return np.char.decode(arr, "utf-8") if arr.ndim else arr[()].decode("utf-8")
    if arr.ndim == 0:
        return arr[()]
    return arr


def read(filename):
    """The HGroup tree of an HDF5 file."""
    with open(filename, "rb") as f:
        buf = f.read()
    r = _Reader(buf)
    oh = struct.unpack_from("<Q", buf, r.root_entry + 8)[0]
    return r.obj(oh)
