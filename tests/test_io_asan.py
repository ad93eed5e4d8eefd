"""The array-file reader (jams_gb300/csrc/llg_io.cu, host C++) under
AddressSanitizer and UBSan: tests/io_fuzz_harness.cc reads 20 000 seeded
corruptions of HDF5 (contiguous, and chunked with shuffle and deflate) and
text spin files, and any read outside the file
buffer or undefined behaviour aborts it.  Every file must get a status
code, with the values matching the extents when it is accepted.  Compiled
here with g++; skipped where g++ or the sanitizer runtimes are missing."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def chunked_bases(tmp_path):
    """Chunked, filtered files (the monitor's compressed layout, fixed
    Huffman codes, a chunk B-tree of several levels) for the corpus."""
    import numpy as np
    from tests import h5_chunked as H
    rng = np.random.default_rng(21)
    s = rng.normal(size=(120, 3))
    out = []
    for name, ds in (("monitor.h5", H.Dataset(s, chunks=(50, 1))),
                     ("fixed.h5", H.Dataset(np.round(s, 1), chunks=(60, 3), filters=((2,), (1, 6, 4)))),
                     ("deep.h5", H.Dataset(s, chunks=(20, 1), fanout=2, unwritten={3}, skip_deflate={5}))):
        p = str(tmp_path / name)
        H.write(p, {"spins": ds})
        out.append(p)
    return out


def test_reader_is_clean_under_asan_on_corrupted_files(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "io_fuzz_harness")
    cmd = [gxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
           "-x", "c++", os.path.join(ROOT, "jams_gb300", "csrc", "llg_io.cu"),
           "-x", "c++", os.path.join(ROOT, "tests", "io_fuzz_harness.cc"), "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        if "asan" in res.stderr.lower() or "ubsan" in res.stderr.lower():
            pytest.skip("sanitizer runtimes not available")
        raise AssertionError(res.stderr[-3000:])
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0", UBSAN_OPTIONS="print_stacktrace=1")
    run = subprocess.run([exe, str(tmp_path), "20000", "20261204", *chunked_bases(tmp_path)], capture_output=True,
                         text=True, env=env, timeout=600)
    assert run.returncode == 0, (run.returncode, run.stdout[-1000:], run.stderr[-4000:])
    codes = dict(tuple(int(v) for v in c.split(":")) for c in run.stdout.split()[1:])
    assert sum(codes.values()) == 20000
    assert codes.get(0, 0) > 0 and codes.get(1, 0) > 0
