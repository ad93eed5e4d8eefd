"""CPU tests of the array-file layer (llg_write_array_file /
llg_read_array_file): HDF5 files of the reference's spin-output layout and
the text format of load_array_from_tsv_file (src/jams/helpers/load.h)."""
import struct

import numpy as np
import pytest


def parse_h5(path):
    """Independent reading of a version-0 HDF5 file written by the library,
    following the HDF5 File Format Specification: superblock -> root symbol
    table (B-tree, local heap, symbol node) -> dataset object headers ->
    contiguous data.  Returns {name: array}."""
    b = open(path, "rb").read()
    assert b[:8] == b"\x89HDF\r\n\x1a\n"
    assert b[8] == 0 and b[13] == 8 and b[14] == 8
    leaf_k, internal_k = struct.unpack_from("<HH", b, 16)
    base, _, eof, _ = struct.unpack_from("<QQQQ", b, 24)
    assert base == 0 and eof == len(b)
    _, root_oh, cache = struct.unpack_from("<QQI", b, 56)
    btree, heap = struct.unpack_from("<QQ", b, 80)
    assert cache == 1
    # root object header: one symbol table message with the same addresses
    ver, _, nmsg, _, hsize = struct.unpack_from("<BBHII", b, root_oh)
    assert ver == 1 and nmsg == 1
    mtype, msize = struct.unpack_from("<HH", b, root_oh + 16)
    assert mtype == 0x11 and struct.unpack_from("<QQ", b, root_oh + 24) == (btree, heap)
    assert b[heap:heap + 4] == b"HEAP"
    hsz, _, hdata = struct.unpack_from("<QQQ", b, heap + 8)
    assert b[btree:btree + 4] == b"TREE"
    ntype, level, used = struct.unpack_from("<BBH", b, btree + 4)
    assert (ntype, level, used) == (0, 0, 1)
    snod = struct.unpack_from("<Q", b, btree + 24 + 8)[0]
    assert b[snod:snod + 4] == b"SNOD"
    nsym = struct.unpack_from("<H", b, snod + 6)[0]
    assert nsym <= 2 * leaf_k
    out = {}
    names = []
    for e in range(nsym):
        noff, oh = struct.unpack_from("<QQ", b, snod + 8 + 40 * e)
        name = b[hdata + noff: b.index(b"\0", hdata + noff)].decode()
        names.append(name)
        ver, _, nmsg, _, hsize = struct.unpack_from("<BBHII", b, oh)
        p, end = oh + 16, oh + 16 + hsize
        dims = dtype = addr = None
        while p + 8 <= end:
            mtype, msize = struct.unpack_from("<HH", b, p)
            d = p + 8
            if mtype == 1:
                rank = b[d + 1]
                dims = struct.unpack_from("<%dQ" % rank, b, d + 8)
            elif mtype == 3:
                assert b[d] & 0x0F == 1 and b[d + 1] & 1 == 0
                dtype = struct.unpack_from("<I", b, d + 4)[0]
                assert struct.unpack_from("<HHBBBBI", b, d + 8) == (0, 64, 52, 11, 0, 52, 1023)
            elif mtype == 8:
                assert b[d] == 3 and b[d + 1] == 1
                addr, size = struct.unpack_from("<QQ", b, d + 2)
            p = d + msize
        assert dtype == 8 and addr is not None
        n = int(np.prod(dims))
        assert size == 8 * n
        out[name] = np.frombuffer(b, dtype="<f8", count=n, offset=addr).reshape(dims)
    assert names == sorted(names)
    return out


def test_h5_round_trip_and_layout(llg, tmp_path):
    rng = np.random.default_rng(5)
    s = rng.normal(size=(1000, 3))
    path = str(tmp_path / "final.h5")
    llg.write_array_file(path, s, "/spins")
    np.testing.assert_array_equal(parse_h5(path)["spins"], s)
    np.testing.assert_array_equal(llg.read_array_file(path, "/spins"), s)
    np.testing.assert_array_equal(llg.read_array_file(path, "spins"), s)


def test_h5_one_dimensional_and_empty(llg, tmp_path):
    a = np.linspace(0.0, 1.0, 7)
    path = str(tmp_path / "alpha.h5")
    llg.write_array_file(path, a, "/alpha")
    np.testing.assert_array_equal(parse_h5(path)["alpha"].reshape(-1), a)
    np.testing.assert_array_equal(llg.read_array_file(path, "/alpha"), a)
    path = str(tmp_path / "empty.h5")
    llg.write_array_file(path, np.zeros((0, 3)), "/spins")
    assert llg.read_array_file(path, "/spins").shape == (0, 3)


def test_h5_errors(llg, tmp_path):
    path = str(tmp_path / "s.h5")
    llg.write_array_file(path, np.ones((4, 3)), "/spins")
    with pytest.raises(llg.LLGError, match="not found"):
        llg.read_array_file(path, "/mus")
    bad = tmp_path / "text.h5"
    bad.write_text("1 2 3\n")
    with pytest.raises(llg.LLGError, match="not an HDF5 file"):
        llg.read_array_file(str(bad), "/spins")
    with pytest.raises(llg.LLGError, match="LLG_ERR_IO"):
        llg.read_array_file(str(tmp_path / "missing.h5"), "/spins")


def test_text_round_trip_exact(llg, tmp_path):
    rng = np.random.default_rng(9)
    s = rng.normal(size=(50, 3)) * 10.0 ** rng.integers(-30, 30, size=(50, 3))
    path = str(tmp_path / "spins.tsv")
    llg.write_array_file(path, s)
    np.testing.assert_array_equal(llg.read_array_file(path).reshape(-1, 3), s)


def test_text_comments_and_counting_follow_the_reference(llg, tmp_path):
    """'#' and '//' lines and lines of fewer than two non-blank characters
    are comments (utils.h:115-126); a line that ends in blanks yields one
    failed extraction, counted as a 0 (load.h:22-45)."""
    path = tmp_path / "s.txt"
    path.write_text("# header\n// also a comment\n7\n1 2 3\n4.5\t5.5 6.5\n\n")
    np.testing.assert_array_equal(llg.read_array_file(str(path)), [1, 2, 3, 4.5, 5.5, 6.5])
    path.write_text("1 2 3 \n")
    np.testing.assert_array_equal(llg.read_array_file(str(path)), [1, 2, 3, 0])


def test_h5_chunked_compressed_as_the_monitor_writes(llg, tmp_path):
    """The HDF5 monitor's "compressed" option (hdf5.cc:292-323): chunks of
    min(4095, rows) x 1 values, shuffle, deflate level 6; a vector field
    and a scalar field in one file, edge chunks padded."""
    from tests import h5_chunked as H
    rng = np.random.default_rng(11)
    s = rng.normal(size=(10000, 3))
    e = rng.normal(size=5000)
    path = str(tmp_path / "compressed.h5")
    H.write(path, {"spins": H.Dataset(s, chunks=(4095, 1)), "energy": H.Dataset(e, chunks=(4095,))})
    np.testing.assert_array_equal(llg.read_array_file(path, "/spins"), s)
    np.testing.assert_array_equal(llg.read_array_file(path, "/energy"), e)
    small = rng.normal(size=(7, 3))   # fewer rows than 4095: one chunk of 7 x 1 per column
    H.write(path, {"spins": H.Dataset(small, chunks=(7, 1))})
    np.testing.assert_array_equal(llg.read_array_file(path, "/spins"), small)


@pytest.mark.parametrize("filters", [
    ((2,), (1, 0)),                      # stored deflate blocks
    ((2,), (1, 6, 4)),                   # fixed Huffman codes (Z_FIXED)
    ((1, 9),),                           # dynamic codes, no shuffle
    ((2,), (1, 6, 2)),                   # Huffman only, no matches
    ((2,), (1, 6, 3)),                   # run-length matches
    ((2,),),                             # shuffle alone
    (),                                  # chunked, no filters
])
def test_h5_chunked_filter_and_block_kinds(llg, tmp_path, filters):
    from tests import h5_chunked as H
    rng = np.random.default_rng(12)
    s = np.round(rng.normal(size=(3000, 3)), 2)   # repetitive bytes: long matches
    path = str(tmp_path / "f.h5")
    H.write(path, {"spins": H.Dataset(s, chunks=(1000, 3), filters=filters)})
    np.testing.assert_array_equal(llg.read_array_file(path, "/spins"), s)
    f32 = rng.normal(size=(900, 3)).astype(np.float32)
    H.write(path, {"spins": H.Dataset(f32, chunks=(256, 1), filters=filters)})
    np.testing.assert_array_equal(llg.read_array_file(path, "/spins"), f32.astype(np.float64))


def test_h5_chunked_deep_btree_unwritten_and_unfiltered_chunks(llg, tmp_path):
    """A chunk B-tree of several levels (two entries per node); chunks never
    written read as the fill value 0; a chunk whose filter mask skips
    deflate is only shuffled."""
    from tests import h5_chunked as H
    rng = np.random.default_rng(13)
    s = rng.normal(size=(600, 3))
    path = str(tmp_path / "deep.h5")
    ds = H.Dataset(s, chunks=(50, 1), fanout=2, unwritten={4, 17}, skip_deflate={0, 9, 35})
    H.write(path, {"spins": ds})
    want = s.copy()
    for i, off in enumerate(H.chunk_list(ds)):
        if i in ds.unwritten:
            want[off[0]:off[0] + 50, off[1]] = 0.0
    np.testing.assert_array_equal(llg.read_array_file(path, "/spins"), want)


def test_h5_chunked_errors(llg, tmp_path):
    from tests import h5_chunked as H
    rng = np.random.default_rng(14)
    s = rng.normal(size=(2000, 3))
    path = str(tmp_path / "e.h5")
    # an optional filter the writer never applied is passed over; a
    # mandatory one is refused
    H.write(path, {"spins": H.Dataset(s, chunks=(1000, 1), extra_filter=(32000, 1))})
    np.testing.assert_array_equal(llg.read_array_file(path, "/spins"), s)
    H.write(path, {"spins": H.Dataset(s, chunks=(1000, 1), extra_filter=(32000, 0))})
    with pytest.raises(llg.LLGError, match="filter 32000 is not supported"):
        llg.read_array_file(path, "/spins")
    H.write(path, {"spins": H.Dataset(s, chunks=(1000, 1))}, layout_version=4)
    with pytest.raises(llg.LLGError, match="version-4 chunk index"):
        llg.read_array_file(path, "/spins")
    # a damaged deflate stream: a flipped bit inside the first chunk
    ds = H.Dataset(s, chunks=(1000, 1))
    H.write(path, {"spins": ds})
    raw, _ = H.encode_chunk(ds, (0, 0), 0)
    b = bytearray(open(path, "rb").read())
    at = bytes(b).index(raw)
    for k in (len(raw) // 2, 3, len(raw) - 2):
        bad = bytearray(b)
        bad[at + k] ^= 0x10
        p = str(tmp_path / "bad.h5")
        open(p, "wb").write(bytes(bad))
        with pytest.raises(llg.LLGError, match="dataset /spins: (deflate chunk|chunk decodes)"):
            llg.read_array_file(p, "/spins")
