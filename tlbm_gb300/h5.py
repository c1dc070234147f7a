"""The subset of the HDF5 file format that tLBM's files use, in numpy, without h5py.

``restart.h5`` (written by python/tLBM_create_restart.py, read by
TLBM_Partition::load_restart_data, src/TLBM_Partition.cpp:481-540) and ``out{n}.h5`` /
``timeAvg.h5`` (python/hdf5Helper.py:4-56) are plain h5py files: groups of contiguous,
unfiltered float32 datasets.  ``write`` produces such a file (superblock version 0, groups as
symbol tables, version-1 object headers -- HDF5's default, earliest format); ``read`` reads a
dataset from files of superblock versions 0-3, with version-1 or version-2 object headers,
groups held as symbol tables or as link messages, and contiguous or compact little-endian
float32/float64 data.  The engine's C++ reader and writer (tlbm_gb300/csrc/h5lite.cpp) are a
separate implementation of the same layouts; the tests check each against the other.
"""

import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"
LEAF_K = 8       # a symbol table node holds up to 2K entries
INTERNAL_K = 16  # a group B-tree node holds up to 2K children
FREE_NULL = 1    # end of a local heap's free list


def _pad8(n):
    return (n + 7) & ~7


# ----------------------------------------------------------------------------- writer


def _msg(mtype, body):
    body = body + b"\0" * (_pad8(len(body)) - len(body))
    return struct.pack("<HHB3x", mtype, len(body), 0) + body


def _object_header(messages):
    body = b"".join(messages)
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body


def _dataset_messages(shape, data_addr, nbytes, dtype):
    rank = len(shape)
    space = struct.pack("<BBB5x", 1, rank, 0) + b"".join(struct.pack("<Q", d) for d in shape)
    if dtype == np.float32:
        dtype_msg = struct.pack("<BBBBIHHBBBBI", 0x11, 0x20, 31, 0, 4, 0, 32, 23, 8, 0, 23, 127)
    else:
        dtype_msg = struct.pack("<BBBBIHHBBBBI", 0x11, 0x20, 63, 0, 8, 0, 64, 52, 11, 0, 52,
                                1023)
    fill = struct.pack("<BBBB", 2, 2, 2, 0)
    layout = struct.pack("<BBQQ", 3, 1, data_addr, nbytes)
    mtime = struct.pack("<B3xI", 1, 0)  # modification time (version 1)
    return [_msg(0x0001, space), _msg(0x0003, dtype_msg), _msg(0x0005, fill),
            _msg(0x0008, layout), _msg(0x0012, mtime), _msg(0x0000, b"\0" * 8)]


def write(path, datasets):
    """Write ``datasets`` (``{"group/name": array}``, nested groups allowed) to a new HDF5 file
    at ``path``; arrays keep their shape and are stored as little-endian float32 (or float64
    when given as float64)."""
    root = {}
    for name, arr in datasets.items():
        parts = [p for p in name.split("/") if p]
        node = root
        for p in parts[:-1]:
            node = node.setdefault(p, {})
            if not isinstance(node, dict):
                raise ValueError("%s is a dataset, not a group" % p)
        a = np.asarray(arr)
        a = np.ascontiguousarray(a, np.float64 if a.dtype == np.float64 else np.float32)
        node[parts[-1]] = a

    img = bytearray(96)  # superblock, filled in last

    def alloc(n):
        at = len(img)
        img.extend(b"\0" * _pad8(n))
        return at

    def put(at, b):
        img[at:at + len(b)] = b

    def group(node):
        """Write a group's children, then the group; return (header, btree, heap) addresses."""
        names = sorted(node, key=lambda s: s.encode())
        if len(names) > 2 * LEAF_K:
            raise ValueError("more than %d objects in one group" % (2 * LEAF_K))
        entries = []
        for nm in names:
            child = node[nm]
            if isinstance(child, dict):
                entries.append((nm,) + group(child))
            else:
                hdr_len = len(_object_header(_dataset_messages(child.shape, 0, 0, child.dtype)))
                hdr = alloc(hdr_len)
                data = alloc(child.nbytes)
                put(data, child.tobytes())
                put(hdr, _object_header(_dataset_messages(child.shape, data, child.nbytes,
                                                          child.dtype)))
                entries.append((nm, hdr, None, None))
        # local heap: "" at 0, the names, then one free block of 16 bytes
        seg = bytearray(8)
        offs = []
        for nm in names:
            offs.append(len(seg))
            b = nm.encode() + b"\0"
            seg += b + b"\0" * (_pad8(len(b)) - len(b))
        free_at = len(seg)
        seg += struct.pack("<QQ", FREE_NULL, 16)
        heap = alloc(32)
        seg_addr = alloc(len(seg))
        put(seg_addr, bytes(seg))
        put(heap, b"HEAP" + struct.pack("<B3xQQQ", 0, len(seg), free_at, seg_addr))
        # symbol table node
        snod = alloc(8 + 2 * LEAF_K * 40)
        b = bytearray(b"SNOD" + struct.pack("<BBH", 1, 0, len(entries)))
        for (nm, hdr, bt, hp), off in zip(entries, offs):
            if bt is None:
                b += struct.pack("<QQI4x16x", off, hdr, 0)
            else:
                b += struct.pack("<QQI4xQQ", off, hdr, 1, bt, hp)
        put(snod, bytes(b))
        # B-tree: one leaf node with the symbol table node as its only child
        btree = alloc(24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8)
        put(btree, b"TREE" + struct.pack("<BBHQQQQQ", 0, 0, 1, UNDEF, UNDEF, 0, snod,
                                         offs[-1] if offs else 0))
        hdr = alloc(len(_object_header([_msg(0x0011, struct.pack("<QQ", btree, heap))])))
        put(hdr, _object_header([_msg(0x0011, struct.pack("<QQ", btree, heap))]))
        return hdr, btree, heap

    hdr, btree, heap = group(root)
    sb = SIGNATURE + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, LEAF_K, INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, len(img), UNDEF)
    sb += struct.pack("<QQI4xQQ", 0, hdr, 1, btree, heap)
    put(0, sb)
    with open(path, "wb") as f:
        f.write(bytes(img))


# ----------------------------------------------------------------------------- reader


class _File:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        self.base = 0

    def at(self, addr, n):
        a = addr + self.base
        if addr == UNDEF or a + n > len(self.b):
            raise ValueError("address outside the file")
        return self.b[a:a + n]


def _u(b, off, n):
    return int.from_bytes(b[off:off + n], "little")


def _messages(f, addr):
    head = f.at(addr, 16)
    blocks = []
    if head[0] == 1:
        blocks.append((addr + 16, _u(head, 8, 4), False, False))
        order = False
    elif head[:4] == b"OHDR" and head[4] == 2:
        flags = head[5]
        p = 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
        w = 1 << (flags & 3)
        blocks.append((addr + p + w, _u(f.at(addr, p + w), p, w), True, False))
        order = bool(flags & 0x04)
    else:
        raise ValueError("unknown object header version")
    out = []
    i = 0
    while i < len(blocks):
        start, length, v2, cont = blocks[i]
        i += 1
        d = f.at(start, length)
        p, end = 0, length
        if v2 and cont:
            if d[:4] != b"OCHK":
                raise ValueError("bad object header continuation chunk")
            p, end = 4, length - 4
        hdr = (6 if order else 4) if v2 else 8
        while p + hdr <= end:
            if v2:
                mtype, size = d[p], _u(d, p + 1, 2)
            else:
                mtype, size = _u(d, p, 2), _u(d, p + 2, 2)
            p += hdr
            body = d[p:p + size]
            p += size
            if mtype == 0x0010:
                blocks.append((_u(body, 0, 8), _u(body, 8, 8), v2, True))
            elif mtype != 0:
                out.append((mtype, body))
    return out


def _heap_name(f, heap, off):
    h = f.at(heap, 32)
    if h[:4] != b"HEAP":
        raise ValueError("bad local heap")
    size, data = _u(h, 8, 8), _u(h, 24, 8)
    seg = f.at(data, size)
    return seg[off:seg.index(b"\0", off)].decode()


def _btree_find(f, node, heap, name, depth=0):
    if depth > 64:
        raise ValueError("group B-tree too deep")
    h = f.at(node, 24)
    if h[:4] != b"TREE" or h[4] != 0:
        raise ValueError("bad group B-tree node")
    level, n = h[5], _u(h, 6, 2)
    kc = f.at(node + 24, 16 * n + 8)
    for c in range(n):
        child = _u(kc, 8 + 16 * c, 8)
        if level > 0:
            found = _btree_find(f, child, heap, name, depth + 1)
            if found is not None:
                return found
            continue
        s = f.at(child, 8)
        if s[:4] != b"SNOD":
            raise ValueError("bad symbol table node")
        k = _u(s, 6, 2)
        e = f.at(child + 8, 40 * k)
        for j in range(k):
            if _heap_name(f, heap, _u(e, 40 * j, 8)) == name:
                return _u(e, 40 * j + 8, 8)
    return None


def _child(f, group, name):
    for mtype, d in _messages(f, group):
        if mtype == 0x0011:
            found = _btree_find(f, _u(d, 0, 8), _u(d, 8, 8), name)
            if found is not None:
                return found
        elif mtype == 0x0006:
            flags = d[1]
            p = 2
            ltype = 0
            if flags & 0x08:
                ltype = d[p]
                p += 1
            if flags & 0x04:
                p += 8
            if flags & 0x10:
                p += 1
            w = 1 << (flags & 3)
            n = _u(d, p, w)
            p += w
            if d[p:p + n].decode() == name:
                if ltype != 0:
                    raise ValueError("link %s is not a hard link" % name)
                return _u(d, p + n, 8)
        elif mtype == 0x0002:
            heap = _u(d, 10 if d[1] & 1 else 2, 8)
            if heap != UNDEF:
                raise ValueError("groups with dense link storage are not supported")
    raise KeyError(name)


def read(path, name):
    """Dataset ``name`` (``"group/name"``) of the HDF5 file at ``path`` as a numpy array of its
    stored type (float32 or float64) and shape."""
    f = _File(path)
    # the superblock sits at 0 or, after a user block, at 512, 1024, 2048, ...
    sb = 0
    while f.b[sb:sb + 8] != SIGNATURE:
        sb = 512 if sb == 0 else 2 * sb
        if sb + 8 > len(f.b):
            raise ValueError("%s is not an HDF5 file" % path)
    s = f.b[sb:sb + 100]
    ver = s[8]
    if ver in (0, 1):
        if s[13] != 8 or s[14] != 8:
            raise ValueError("only 8-byte offsets and lengths are read")
        b = 24 if ver == 0 else 28
        f.base = _u(s, b, 8)
        obj = _u(s, b + 40, 8)
    elif ver in (2, 3):
        f.base = _u(s, 12, 8)
        obj = _u(s, 36, 8)
    else:
        raise ValueError("unknown superblock version %d" % ver)
    for part in [p for p in name.split("/") if p]:
        obj = _child(f, obj, part)
    shape = elem = layout = None
    for mtype, d in _messages(f, obj):
        if mtype == 0x0001:
            rank = d[1]
            at = 8 if d[0] == 1 else 4
            shape = tuple(_u(d, at + 8 * k, 8) for k in range(rank))
        elif mtype == 0x0003:
            if d[0] & 0x0F != 1 or d[1] & 1:
                raise ValueError("only little-endian IEEE floating-point data is read")
            elem = _u(d, 4, 4)
        elif mtype == 0x0008:
            if d[0] >= 3:
                if d[1] == 1:
                    layout = ("contiguous", _u(d, 2, 8))
                elif d[1] == 0:
                    layout = ("compact", bytes(d[4:4 + _u(d, 2, 2)]))
                else:
                    raise ValueError("chunked or virtual datasets are not supported")
            elif d[2] == 1:
                layout = ("contiguous", _u(d, 8, 8))
            else:
                raise ValueError("unsupported layout")
        elif mtype == 0x000B:
            raise ValueError("filtered (compressed) datasets are not supported")
    if shape is None or elem not in (4, 8) or layout is None:
        raise ValueError("%s is not a float dataset" % name)
    count = int(np.prod(shape, dtype=np.int64)) if shape else 1
    dt = np.dtype("<f4" if elem == 4 else "<f8")
    if layout[0] == "compact":
        raw = layout[1][:count * elem]
    elif layout[1] == UNDEF:
        raw = b"\0" * (count * elem)
    else:
        raw = f.at(layout[1], count * elem)
    return np.frombuffer(raw, dt, count).reshape(shape).copy()
