"""Writer of chunked, filtered HDF5 files for the reader's tests, following
the HDF5 File Format Specification: a version-0 superblock, the root group
as a symbol table, and per dataset a version-1 object header with
dataspace, datatype, fill-value, layout (version 3, chunked) and filter
pipeline (version 1) messages, a version-1 B-tree of raw data chunks and
the filtered chunks.  This is the structure the HDF5 library writes for the
HDF5 monitor's "compressed" option (src/jams/monitors/hdf5.cc:292-323:
chunks of min(4095, rows) x 1 values, shuffle, then deflate at level 6).

No HDF5 library is available on either machine, so the files come from
this independent writer; the deflate streams come from Python's zlib.

    write(path, {"spins": Dataset(array, chunks=(4095, 1))})
"""
import struct
import zlib
from dataclasses import dataclass, field
from typing import Dict, Optional, Sequence, Set, Tuple

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SHUFFLE, DEFLATE = 2, 1


@dataclass
class Dataset:
    data: np.ndarray                       # 1-D or 2-D, float64 or float32
    chunks: Tuple[int, ...]                # chunk extents, one per dimension
    filters: Sequence[tuple] = ((SHUFFLE,), (DEFLATE, 6))   # pipeline order; (DEFLATE, level[, strategy])
    fanout: int = 64                       # chunk B-tree entries per node (smaller: more levels)
    unwritten: Set[int] = field(default_factory=set)       # chunk numbers left out (read as fill 0)
    skip_deflate: Set[int] = field(default_factory=set)    # chunks stored without deflate (filter mask bit)
    extra_filter: Optional[Tuple[int, int]] = None         # (id, flags) appended to the pipeline, masked off in every chunk


class Blob:
    def __init__(self):
        self.b = bytearray()

    def alloc(self, n):
        at = len(self.b)
        self.b.extend(bytes(n))
        return at

    def put(self, at, fmt, *v):
        struct.pack_into("<" + fmt, self.b, at, *v)


def message(mtype, body, flags=0):
    body = bytes(body) + bytes((-len(body)) % 8)
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def chunk_list(ds):
    shape = ds.data.shape
    grid = [-(-s // c) for s, c in zip(shape, ds.chunks)]
    out = []
    for idx in np.ndindex(*grid):
        out.append(tuple(i * c for i, c in zip(idx, ds.chunks)))
    return out


def encode_chunk(ds, offset, number):
    """The chunk's elements (full extents, padded with 0 past the edge),
    then the pipeline's filters in order; returns (bytes, filter mask)."""
    block = np.zeros(ds.chunks, dtype=ds.data.dtype)
    sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offset, ds.chunks, ds.data.shape))
    sub = ds.data[sl]
    block[tuple(slice(0, n) for n in sub.shape)] = sub
    raw = block.astype(block.dtype.newbyteorder("<")).tobytes()
    mask = 0
    for i, f in enumerate(ds.filters):
        if f[0] == SHUFFLE:
            es = ds.data.dtype.itemsize
            n = len(raw) // es
            a = np.frombuffer(raw[:n * es], dtype=np.uint8).reshape(n, es)
            raw = a.T.tobytes() + raw[n * es:]
        elif f[0] == DEFLATE:
            if number in ds.skip_deflate:
                mask |= 1 << i
                continue
            strategy = f[2] if len(f) > 2 else zlib.Z_DEFAULT_STRATEGY
            c = zlib.compressobj(f[1], zlib.DEFLATED, 15, 8, strategy)
            raw = c.compress(raw) + c.flush()
    if ds.extra_filter:   # an optional filter that passed over every chunk
        mask |= 1 << len(ds.filters)
    return raw, mask


def pipeline_message(ds):
    filters = list(ds.filters)
    body = bytearray()
    entries = []
    for f in filters:
        if f[0] == SHUFFLE:
            entries.append((SHUFFLE, 1, b"shuffle\0", [ds.data.dtype.itemsize]))
        else:
            entries.append((DEFLATE, 1, b"deflate\0", [f[1]]))
    if ds.extra_filter:
        entries.append((ds.extra_filter[0], ds.extra_filter[1], b"other\0\0\0", [7]))
    body += struct.pack("<BB6x", 1, len(entries))
    for fid, flags, name, cd in entries:
        body += struct.pack("<HHHH", fid, len(name), flags, len(cd)) + name
        body += struct.pack("<%dI" % len(cd), *cd)
        if len(cd) % 2:
            body += bytes(4)
    return message(0x0B, body, 1)


def write_btree(blob, ds, entries, rank):
    """Version-1 B-tree of chunks (node type 1), `fanout` entries per
    node; entries = [(offset, size, mask, address)] in offset order.
    Returns the root node's address."""
    ksz = 8 + 8 * (rank + 1)

    def key(e):
        off, size, mask, _ = e
        return struct.pack("<II", size, mask) + struct.pack("<%dQ" % (rank + 1), *(list(off) + [0]))

    level = 0
    nodes = entries
    while True:
        groups = [nodes[i:i + ds.fanout] for i in range(0, len(nodes), ds.fanout)] or [[]]
        parents = []
        for g in groups:
            at = blob.alloc(8 + 16 + len(g) * (ksz + 8) + ksz)
            blob.b[at:at + 4] = b"TREE"
            blob.put(at + 4, "BBH", 1, level, len(g))
            blob.put(at + 8, "QQ", UNDEF, UNDEF)
            p = at + 24
            for e in g:
                blob.b[p:p + ksz] = key(e)
                blob.put(p + ksz, "Q", e[3])
                p += ksz + 8
            last = g[-1] if g else ((0,) * rank, 0, 0, 0)
            upper = tuple(o + c for o, c in zip(last[0], ds.chunks))
            blob.b[p:p + ksz] = key((upper, 0, 0, 0))
            first = g[0] if g else last
            parents.append((first[0], first[1], first[2], at))
        if len(parents) == 1:
            return parents[0][3]
        nodes = parents
        level += 1


def write(path, sets: Dict[str, Dataset], layout_version=3):
    names = sorted(sets)
    blob = Blob()
    blob.alloc(96)                                     # superblock + root entry
    root = blob.alloc(16 + 24)
    heap_data = bytearray(8)
    name_off = {}
    for n in names:
        name_off[n] = len(heap_data)
        heap_data += n.encode() + b"\0"
        heap_data += bytes((-len(heap_data)) % 8)
    heap = blob.alloc(32 + len(heap_data))
    tree = blob.alloc(24 + 8 + 8 + 8)
    snod = blob.alloc(8 + 40 * len(names))
    heads = {}
    for n in names:
        ds = sets[n]
        rank = ds.data.ndim
        elements = [(off, i) for i, off in enumerate(chunk_list(ds))]
        entries = []
        for off, i in elements:
            if i in ds.unwritten:
                continue
            raw, mask = encode_chunk(ds, off, i)
            at = blob.alloc(len(raw))
            blob.b[at:at + len(raw)] = raw
            entries.append((off, len(raw), mask, at))
        bt = write_btree(blob, ds, entries, rank) if entries else UNDEF
        es = ds.data.dtype.itemsize
        msgs = bytearray()
        sp = struct.pack("<BBBB4x", 1, rank, 0, 0) + struct.pack("<%dQ" % rank, *ds.data.shape)
        msgs += message(0x01, sp)
        if es == 8:
            dt = struct.pack("<BBBBI", 0x11, 0x20, 63, 0, 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
        else:
            dt = struct.pack("<BBBBI", 0x11, 0x20, 31, 0, 4) + struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
        msgs += message(0x03, dt, 1)
        msgs += message(0x05, struct.pack("<BBBB", 2, 3, 2, 0), 1)
        if layout_version == 3:
            ly = struct.pack("<BBBQ", 3, 2, rank + 1, bt) + struct.pack("<%dI" % (rank + 1), *(list(ds.chunks) + [es]))
        else:  # version 4, single-chunk index: not read
            ly = struct.pack("<BBBBB", 4, 2, 0, rank + 1, 4) + bytes(4 * (rank + 1)) + struct.pack("<BQ", 1, bt)
        msgs += message(0x08, ly)
        msgs += pipeline_message(ds)
        oh = blob.alloc(16 + len(msgs))
        blob.put(oh, "BBHII4x", 1, 0, 5, 1, len(msgs))   # five messages
        blob.b[oh + 16:oh + 16 + len(msgs)] = msgs
        heads[n] = oh
    eof = len(blob.b)
    b = blob
    b.b[0:8] = b"\x89HDF\r\n\x1a\n"
    b.put(8, "BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0)
    b.put(16, "HHI", 4, 16, 0)
    b.put(24, "QQQQ", 0, UNDEF, eof, UNDEF)
    b.put(56, "QQII", 0, root, 1, 0)
    b.put(80, "QQ", tree, heap)
    b.put(root, "BBHII4x", 1, 0, 1, 1, 24)
    b.b[root + 16:root + 40] = message(0x11, struct.pack("<QQ", tree, heap))
    b.b[heap:heap + 4] = b"HEAP"
    b.put(heap + 8, "QQQ", len(heap_data), UNDEF, heap + 32)
    b.b[heap + 32:heap + 32 + len(heap_data)] = heap_data
    b.b[tree:tree + 4] = b"TREE"
    b.put(tree + 4, "BBH", 0, 0, 1)
    b.put(tree + 8, "QQQQQ", UNDEF, UNDEF, 0, snod, name_off[names[-1]])
    b.b[snod:snod + 4] = b"SNOD"
    b.put(snod + 4, "BBH", 1, 0, len(names))
    for i, n in enumerate(names):
        b.put(snod + 8 + 40 * i, "QQII", name_off[n], heads[n], 0, 0)
    with open(path, "wb") as f:
        f.write(bytes(b.b))
