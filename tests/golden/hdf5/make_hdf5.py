"""Generate the HDF5 reader fixtures tests/golden/hdf5/h5_*.h5 (+ h5_expected.npz).

The image has no libhdf5, and the one libhdf5-written file on it (scipy's
MATLAB v7.3 test file) only holds a small contiguous dataset in a version 0
file.  These fixtures encode, byte by byte from the HDF5 File Format
Specification, the other structures libhdf5 writes and the readers must
handle:

h5_v0_chunked.h5 -- superblock v0, symbol-table groups (root + nested
    "allknn"), a v1 object header continued in a second block, datasets
    "train" (f32 40x10, chunked 8x4 over a two-level v1 B-tree, shuffle +
    deflate, one chunk stored with deflate skipped by its filter mask, edge
    chunks partly outside the dataspace), "ids" (big-endian i16, contiguous),
    "half" (f16, compact), "allknn/knns" (i32) and "allknn/dists" (f64), a
    fixed-length string attribute and a variable-length one (global heap).
h5_v2_links.h5 -- superblock v2, version 2 object headers (timestamps,
    creation order, 2-byte chunk size, an OCHK continuation), compact link
    messages, dataspace v2, datatype/attribute v3, layout v4 with the single
    chunk (deflated), implicit and fixed-array chunk indexes.

Checksums of the v2 structures use Jenkins' lookup3 hashlittle (initial value
0), as the specification prescribes.  Run: python tests/golden/hdf5/make_hdf5.py
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
M32 = 0xFFFFFFFF


def lookup3(data: bytes, init: int = 0) -> int:
    """Bob Jenkins' lookup3 hashlittle (public domain, 2006)."""
    def rot(x, k):
        return ((x << k) | (x >> (32 - k))) & M32

    n = len(data)
    a = b = c = (0xDEADBEEF + n + init) & M32
    i = 0
    while n > 12:
        a = (a + int.from_bytes(data[i:i + 4], "little")) & M32
        b = (b + int.from_bytes(data[i + 4:i + 8], "little")) & M32
        c = (c + int.from_bytes(data[i + 8:i + 12], "little")) & M32
        a = (a - c) & M32; a ^= rot(c, 4); c = (c + b) & M32
        b = (b - a) & M32; b ^= rot(a, 6); a = (a + c) & M32
        c = (c - b) & M32; c ^= rot(b, 8); b = (b + a) & M32
        a = (a - c) & M32; a ^= rot(c, 16); c = (c + b) & M32
        b = (b - a) & M32; b ^= rot(a, 19); a = (a + c) & M32
        c = (c - b) & M32; c ^= rot(b, 4); b = (b + a) & M32
        i += 12
        n -= 12
    if n == 0:
        return c
    tail = data[i:i + n] + b"\0" * (12 - n)
    a = (a + int.from_bytes(tail[0:4], "little")) & M32
    b = (b + int.from_bytes(tail[4:8], "little")) & M32
    c = (c + int.from_bytes(tail[8:12], "little")) & M32
    c ^= b; c = (c - rot(b, 14)) & M32
    a ^= c; a = (a - rot(c, 11)) & M32
    b ^= a; b = (b - rot(a, 25)) & M32
    c ^= b; c = (c - rot(b, 16)) & M32
    a ^= c; a = (a - rot(c, 4)) & M32
    b ^= a; b = (b - rot(a, 14)) & M32
    c ^= b; c = (c - rot(b, 24)) & M32
    return c


class Blob:
    """A file image; alloc() hands out addresses, put() fills them."""

    def __init__(self):
        self.b = bytearray()

    def alloc(self, n, align=8):
        self.b += b"\0" * ((-len(self.b)) % align)
        at = len(self.b)
        self.b += b"\0" * n
        return at

    def put(self, at, data):
        self.b[at:at + len(data)] = data

    def add(self, data, align=8):
        at = self.alloc(len(data), align)
        self.put(at, data)
        return at


def q(v):
    return struct.pack("<Q", v)


def pad8(b):
    return b + b"\0" * ((-len(b)) % 8)


# -- message bodies ----------------------------------------------------------
def dt_int(size, signed=True, big=False):
    return bytes([0x10, (8 if signed else 0) | (1 if big else 0), 0, 0]) + struct.pack("<IHH", size, 0, 8 * size)


def dt_float(size, big=False):
    sign, eloc, esz, msz, bias = {2: (15, 10, 5, 10, 15), 4: (31, 23, 8, 23, 127), 8: (63, 52, 11, 52, 1023)}[size]
    return (bytes([0x11, 0x20 | (1 if big else 0), sign, 0]) + struct.pack("<IHH", size, 0, 8 * size) +
            bytes([eloc, esz, 0, msz]) + struct.pack("<I", bias))


def dt_str(size):
    return bytes([0x13, 0, 0, 0]) + struct.pack("<I", size)


def dt_vlen_str():
    return bytes([0x19, 0x01, 0, 0]) + struct.pack("<I", 16) + dt_int(1, signed=False)


def ds_v1(shape):
    return bytes([1, len(shape), 0, 0]) + b"\0" * 4 + b"".join(q(d) for d in shape)


def ds_v2(shape):
    return bytes([2, len(shape), 0, 1 if shape else 0]) + b"".join(q(d) for d in shape)


def attr_v1(name, dt, space, data):
    nb = name.encode() + b"\0"
    return (struct.pack("<BBHHH", 1, 0, len(nb), len(dt), len(space)) + pad8(nb) + pad8(dt) + pad8(space) + data)


def attr_v3(name, dt, space, data):
    nb = name.encode() + b"\0"
    return struct.pack("<BBHHHB", 3, 0, len(nb), len(dt), len(space), 0) + nb + dt + space + data


def ohdr_v1(msgs, total_msgs=None):
    body = b""
    for t, d, fl in msgs:
        d = pad8(d)
        body += struct.pack("<HHB3x", t, len(d), fl) + d
    return struct.pack("<BBHII4x", 1, 0, total_msgs or len(msgs), 1, len(body)) + body


def v1_msgs(msgs):
    out = b""
    for t, d, fl in msgs:
        d = pad8(d)
        out += struct.pack("<HHB3x", t, len(d), fl) + d
    return out


def ohdr_v2(msgs):
    """flags: 2-byte chunk0 size, creation order tracked, times stored."""
    body = b""
    for i, (t, d) in enumerate(msgs):
        body += struct.pack("<BHBH", t, len(d), 0, i) + d
    pre = b"OHDR" + bytes([2, 0x01 | 0x04 | 0x20]) + struct.pack("<4I", 1, 2, 3, 4) + struct.pack("<H", len(body))
    img = pre + body
    return img + struct.pack("<I", lookup3(img))


def link_msg(name, addr):
    nb = name.encode()
    return bytes([1, 0x00]) + bytes([len(nb)]) + nb + q(addr)


# -- symbol-table groups (version 0 files) -----------------------------------
def symtab_group(blob, entries):
    """entries: sorted [(name, ohdr_addr)]; returns (btree_addr, heap_addr)."""
    seg = bytearray(b"\0" * 8)
    offs = []
    for name, _ in entries:
        offs.append(len(seg))
        seg += pad8(name.encode() + b"\0")
    free = len(seg)
    seg += q(1) + q(32) + b"\0" * 16
    heap = blob.alloc(32)
    seg_at = blob.add(bytes(seg))
    blob.put(heap, b"HEAP" + bytes(4) + q(len(seg)) + q(free) + q(seg_at))
    snod = blob.alloc(8 + 8 * 40)
    img = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(entries))
    for off, (_, a) in zip(offs, entries):
        img += q(off) + q(a) + bytes(24)
    blob.put(snod, img)
    bt = blob.alloc(24 + 32 * 8 + 33 * 8)
    blob.put(bt, b"TREE" + bytes([0, 0]) + struct.pack("<H", 1) + q(UNDEF) + q(UNDEF) + q(0) + q(snod) + q(offs[-1]))
    return bt, heap


def chunk_btree(blob, leaves, rank):
    """leaves: list of lists of (size, mask, offsets, addr); a two-level tree
    when there are several leaves."""
    def node(level, ents, last_key):
        img = b"TREE" + bytes([1, level]) + struct.pack("<H", len(ents)) + q(UNDEF) + q(UNDEF)
        for size, mask, off, child in ents:
            img += struct.pack("<II", size, mask) + b"".join(q(o) for o in off) + q(0) + q(child)
        img += struct.pack("<II", 0, 0) + b"".join(q(o) for o in last_key) + q(0)
        return blob.add(img)

    ends = [(0,) * rank] * len(leaves)
    addrs = [node(0, lf, ends[i]) for i, lf in enumerate(leaves)]
    if len(addrs) == 1:
        return addrs[0]
    return node(1, [(0, 0, lf[0][2], a) for lf, a in zip(leaves, addrs)], (0,) * rank)


def chunks_of(arr, cshape):
    """Yield (offset tuple, full chunk array padded with zeros)."""
    grid = [-(-s // c) for s, c in zip(arr.shape, cshape)]
    for idx in np.ndindex(*grid):
        off = tuple(i * c for i, c in zip(idx, cshape))
        ch = np.zeros(cshape, arr.dtype)
        src = arr[tuple(slice(o, o + c) for o, c in zip(off, cshape))]
        ch[tuple(slice(0, s) for s in src.shape)] = src
        yield off, ch


def shuffle(b, w):
    n = len(b) // w
    return np.frombuffer(b[:n * w], np.uint8).reshape(n, w).T.tobytes() + b[n * w:]


def make_v0(path, rng):
    blob = Blob()
    sb = blob.alloc(96)
    train = rng.standard_normal((40, 10)).astype(np.float32)
    train[3, 7] = -0.0
    ids = (np.arange(24, dtype=np.int16) * 1000 - 5000).reshape(4, 6)
    half = (rng.standard_normal((3, 5)) * 100).astype(np.float16)
    knns = rng.integers(-(1 << 31), 1 << 31, size=(37, 5), dtype=np.int64).astype(np.int32)
    dists = rng.standard_normal((37, 5))

    cshape = (8, 4)
    leaves, cur = [], []
    for k, (off, ch) in enumerate(chunks_of(train, cshape)):
        raw = shuffle(ch.tobytes(), 4)
        mask = 0
        if k == 5:
            mask = 0b10  # deflate skipped for this chunk
        else:
            raw = zlib.compress(raw, 6)
        a = blob.add(raw)
        cur.append((len(raw), mask, off, a))
        if len(cur) == 8:
            leaves.append(cur)
            cur = []
    if cur:
        leaves.append(cur)
    tree = chunk_btree(blob, leaves, 2)
    pline = bytes([1, 2]) + bytes(6)
    pline += struct.pack("<HHHH", 2, 8, 1, 1) + pad8(b"shuffle\0") + struct.pack("<I", 4) + bytes(4)
    pline += struct.pack("<HHHH", 1, 8, 0, 1) + pad8(b"deflate\0") + struct.pack("<I", 6) + bytes(4)
    lay = bytes([3, 2, 3]) + q(tree) + struct.pack("<III", 8, 4, 4)
    h_train = blob.add(ohdr_v1([(0x01, ds_v1(train.shape), 0), (0x03, dt_float(4), 1), (0x0B, pline, 0),
                                (0x08, lay, 0)]))

    ids_at = blob.add(ids.astype(">i2").tobytes())
    h_ids = blob.add(ohdr_v1([(0x01, ds_v1(ids.shape), 0), (0x03, dt_int(2, big=True), 1),
                              (0x08, bytes([3, 1]) + q(ids_at) + q(ids.nbytes), 0)]))
    hb = half.tobytes()
    h_half = blob.add(ohdr_v1([(0x01, ds_v1(half.shape), 0), (0x03, dt_float(2), 1),
                               (0x08, bytes([3, 0]) + struct.pack("<H", len(hb)) + hb, 0)]))
    k_at = blob.add(knns.tobytes())
    d_at = blob.add(dists.tobytes())
    h_knns = blob.add(ohdr_v1([(0x01, ds_v1(knns.shape), 0), (0x03, dt_int(4), 1),
                               (0x08, bytes([3, 1]) + q(k_at) + q(knns.nbytes), 0)]))
    h_dists = blob.add(ohdr_v1([(0x01, ds_v1(dists.shape), 0), (0x03, dt_float(8), 1),
                                (0x08, bytes([3, 1]) + q(d_at) + q(dists.nbytes), 0)]))
    sub_bt, sub_heap = symtab_group(blob, [("dists", h_dists), ("knns", h_knns)])
    h_sub = blob.add(ohdr_v1([(0x11, q(sub_bt) + q(sub_heap), 1)]))

    # Global heap collection with one string object.
    vs = b"variable length value"
    gcol = blob.alloc(4096)
    obj = struct.pack("<HH4x", 1, 0) + q(len(vs)) + pad8(vs)
    blob.put(gcol, b"GCOL" + bytes([1, 0, 0, 0]) + q(4096) + obj +
             struct.pack("<HH4x", 0, 0) + q(4096 - 16 - len(obj)))

    root_bt, root_heap = symtab_group(blob, [("allknn", h_sub), ("half", h_half), ("ids", h_ids), ("train", h_train)])
    # Root header: symbol table message + a continuation to a block with the attributes.
    a1 = attr_v1("title", dt_str(12), ds_v1(()), b"knng fixture")
    a2 = attr_v1("note", dt_vlen_str(), ds_v1(()), struct.pack("<I", len(vs)) + q(gcol) + struct.pack("<I", 1))
    cont_body = v1_msgs([(0x0C, a1, 0), (0x0C, a2, 0)])
    cont = blob.add(cont_body)
    root = blob.add(ohdr_v1([(0x11, q(root_bt) + q(root_heap), 1), (0x10, q(cont) + q(len(cont_body)), 0)],
                            total_msgs=4))
    eof = len(blob.b)
    blob.put(sb, SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0) + q(0) + q(UNDEF) + q(eof) +
             q(UNDEF) + q(0) + q(root) + struct.pack("<II", 1, 0) + q(root_bt) + q(root_heap))
    with open(path, "wb") as f:
        f.write(blob.b)
    return {"train": train, "ids": ids, "half": half, "allknn/knns": knns, "allknn/dists": dists}, \
        {"title": "knng fixture", "note": vs.decode()}


def make_v2(path, rng):
    blob = Blob()
    sb = blob.alloc(48)
    train = rng.standard_normal((12, 6)).astype(np.float32)
    single = np.arange(30, dtype=np.int32).reshape(5, 6) - 7
    implicit = rng.standard_normal((9, 4)).astype(np.float32)
    fixed = (rng.standard_normal((20, 6)) * 1000).astype(np.int32)
    deep = np.arange(-8, 8, dtype=np.int8).reshape(4, 4)

    t_at = blob.add(train.tobytes())
    h_train = blob.add(ohdr_v2([(0x01, ds_v2(train.shape)), (0x03, dt_float(4)),
                                (0x08, bytes([3, 1]) + q(t_at) + q(train.nbytes))]))
    # Layout v4, single chunk index, deflated: flags bit 1 = filtered single chunk.
    zs = zlib.compress(single.tobytes())
    s_at = blob.add(zs)
    pline_v2 = bytes([2, 1]) + struct.pack("<HHH", 1, 0, 1) + struct.pack("<I", 4)
    lay = bytes([4, 2, 0x02, 3, 1]) + bytes([5, 6, 4]) + bytes([1]) + q(len(zs)) + struct.pack("<I", 0) + q(s_at)
    h_single = blob.add(ohdr_v2([(0x01, ds_v2(single.shape)), (0x03, dt_int(4)), (0x0B, pline_v2), (0x08, lay)]))
    # Implicit index: chunks 4x3 stored back to back in grid order.
    cs = (4, 3)
    chunks = b"".join(ch.tobytes() for _, ch in chunks_of(implicit, cs))
    i_at = blob.add(chunks)
    lay = bytes([4, 2, 0, 3, 1]) + bytes([4, 3, 4]) + bytes([2]) + q(i_at)
    h_impl = blob.add(ohdr_v2([(0x01, ds_v2(implicit.shape)), (0x03, dt_float(4)), (0x08, lay)]))
    # Fixed-array index over deflated 8x4 chunks (client id 1: filtered entries).
    cs = (8, 4)
    ents = []
    for off, ch in chunks_of(fixed, cs):
        z = zlib.compress(ch.tobytes())
        ents.append((blob.add(z), len(z)))
    fahd = blob.alloc(8 + 8 + 8 + 4)
    dblk_img = b"FADB" + bytes([0, 1]) + q(fahd) + b"".join(q(a) + struct.pack("<I", n)[:2] + struct.pack("<I", 0)
                                                            for a, n in ents)
    dblk = blob.add(dblk_img + struct.pack("<I", lookup3(dblk_img)))
    fahd_img = b"FAHD" + bytes([0, 1, 8 + 2 + 4, 10]) + q(len(ents)) + q(dblk)
    blob.put(fahd, fahd_img + struct.pack("<I", lookup3(fahd_img)))
    lay = bytes([4, 2, 0, 3, 1]) + bytes([8, 4, 4]) + bytes([3, 10]) + q(fahd)
    h_fixed = blob.add(ohdr_v2([(0x01, ds_v2(fixed.shape)), (0x03, dt_int(4)), (0x0B, pline_v2), (0x08, lay)]))
    # Group "sub" with a compact i8 dataset "deep".
    h_deep = blob.add(ohdr_v2([(0x01, ds_v2(deep.shape)), (0x03, dt_int(1)),
                               (0x08, bytes([3, 0]) + struct.pack("<H", deep.nbytes) + deep.tobytes())]))
    linfo = bytes([0, 0]) + q(UNDEF) + q(UNDEF)
    ginfo = bytes([0, 0])
    h_sub = blob.add(ohdr_v2([(0x02, linfo), (0x0A, ginfo), (0x06, link_msg("deep", h_deep))]))
    # Root: links in the first chunk, more in an OCHK continuation block.
    more = [(0x06, link_msg("fixed", h_fixed)), (0x06, link_msg("implicit", h_impl)),
            (0x0C, attr_v3("version", dt_float(4), ds_v2(()), struct.pack("<f", 2.5)))]
    body = b"".join(struct.pack("<BHBH", t, len(d), 0, 10 + i) + d for i, (t, d) in enumerate(more))
    ochk = b"OCHK" + body
    c_at = blob.add(ochk + struct.pack("<I", lookup3(ochk)))
    root = blob.add(ohdr_v2([(0x02, linfo), (0x0A, ginfo), (0x06, link_msg("train", h_train)),
                             (0x06, link_msg("single", h_single)), (0x06, link_msg("sub", h_sub)),
                             (0x10, q(c_at) + q(len(ochk) + 4))]))
    eof = len(blob.b)
    img = SIG + bytes([2, 8, 8, 0]) + q(0) + q(UNDEF) + q(eof) + q(root)
    blob.put(sb, img + struct.pack("<I", lookup3(img)))
    with open(path, "wb") as f:
        f.write(blob.b)
    return {"train": train, "single": single, "implicit": implicit, "fixed": fixed, "sub/deep": deep}, \
        {"version": 2.5}


def write_datasets(path, arrays, chunks=None, deflate=False):
    """Write {name: ndarray} (f32/f64/i32/i16/i8/f16, native order) into a
    version 0 file, "group/name" into one level of symbol-table groups:
    contiguous, or chunked ``chunks`` (one shape for all) over a one-level v1
    B-tree, optionally shuffled+deflated."""
    blob = Blob()
    sb = blob.alloc(96)
    entries = []
    groups = {}
    for name in sorted(arrays):
        a = np.ascontiguousarray(arrays[name])
        dt = dt_float(a.itemsize) if a.dtype.kind == "f" else dt_int(a.itemsize)
        if chunks is None:
            at = blob.add(a.tobytes())
            lay = bytes([3, 1]) + q(at) + q(a.nbytes)
            msgs = [(0x01, ds_v1(a.shape), 0), (0x03, dt, 1), (0x08, lay, 0)]
        else:
            ents = []
            for off, ch in chunks_of(a, chunks):
                raw = ch.tobytes()
                if deflate:
                    raw = zlib.compress(shuffle(raw, a.itemsize), 1)
                ents.append((len(raw), 0, off, blob.add(raw)))
            tree = chunk_btree(blob, [ents], a.ndim)
            lay = bytes([3, 2, a.ndim + 1]) + q(tree) + struct.pack(f"<{a.ndim + 1}I", *chunks, a.itemsize)
            msgs = [(0x01, ds_v1(a.shape), 0), (0x03, dt, 1), (0x08, lay, 0)]
            if deflate:
                pl = bytes([1, 2]) + bytes(6)
                pl += struct.pack("<HHHH", 2, 8, 1, 1) + pad8(b"shuffle\0") + struct.pack("<I", a.itemsize) + bytes(4)
                pl += struct.pack("<HHHH", 1, 8, 0, 1) + pad8(b"deflate\0") + struct.pack("<I", 1) + bytes(4)
                msgs.insert(2, (0x0B, pl, 0))
        hdr = blob.add(ohdr_v1(msgs))
        if "/" in name:
            g, leaf = name.split("/", 1)
            groups.setdefault(g, []).append((leaf, hdr))
        else:
            entries.append((name, hdr))
    for g in sorted(groups):
        gbt, gheap = symtab_group(blob, sorted(groups[g]))
        entries.append((g, blob.add(ohdr_v1([(0x11, q(gbt) + q(gheap), 1)]))))
    entries.sort()
    bt, heap = symtab_group(blob, entries)
    root = blob.add(ohdr_v1([(0x11, q(bt) + q(heap), 1)]))
    blob.put(sb, SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0) + q(0) + q(UNDEF) +
             q(len(blob.b)) + q(UNDEF) + q(0) + q(root) + struct.pack("<II", 1, 0) + q(bt) + q(heap))
    with open(path, "wb") as f:
        f.write(blob.b)


def main():
    rng = np.random.default_rng(20260)
    exp0, at0 = make_v0(os.path.join(HERE, "h5_v0_chunked.h5"), rng)
    exp2, at2 = make_v2(os.path.join(HERE, "h5_v2_links.h5"), rng)
    arrays = {f"v0:{k}": v for k, v in exp0.items()}
    arrays.update({f"v2:{k}": v for k, v in exp2.items()})
    np.savez(os.path.join(HERE, "h5_expected.npz"), **arrays)
    print("wrote h5_v0_chunked.h5, h5_v2_links.h5, h5_expected.npz;", at0, at2)


if __name__ == "__main__":
    main()
