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
