"""The config front end (jams_gb300/csrc/llg_config.cu, host C++) under
AddressSanitizer and UBSan: tests/config_fuzz_harness.cc sends 20 000
seeded mutations of four configs through llg_config_describe, and any
out-of-bounds access or undefined behaviour aborts it.  The number parser
once read a freed string after rejecting a malformed integer; this test
found it.  Compiled here with g++ against the CUDA headers (the
config unit includes cuda_runtime.h for its create entry point, which the
harness stubs); skipped where g++, the headers or the sanitizer runtimes
are missing."""
import os
import shutil
import subprocess

import pytest

from jams_gb300 import configs as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.exists(os.path.join(inc, "cuda_runtime.h")) else None


def test_config_parser_is_clean_under_asan_on_mutated_configs(tmp_path):
    gxx, inc = shutil.which("g++"), _cuda_include()
    if not gxx or not inc:
        pytest.skip("g++ or the CUDA headers not found")
    exe = str(tmp_path / "config_fuzz_harness")
    cmd = [gxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
           "-I" + inc, "-x", "c++", os.path.join(ROOT, "jams_gb300", "csrc", "llg_config.cu"),
           "-x", "c++", os.path.join(ROOT, "tests", "config_fuzz_harness.cc"), "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        if "asan" in res.stderr.lower() or "ubsan" in res.stderr.lower():
            pytest.skip("sanitizer runtimes not available")
        raise AssertionError(res.stderr[-3000:])
    texts = [C.sc_ferromagnet(L=6, T=10.0, steps=10), C.bcc_three_shell(L=5, T=300.0, steps=10),
             C.bcc_three_shell(L=6, T=0.0, steps=10, dipole_cutoff=2.0),
             C.triangular_dmi(L=8, T=5.0, Bz=1.0, steps=10)]
    paths = []
    for i, t in enumerate(texts):
        p = tmp_path / ("base%d.cfg" % i)
        p.write_text(t)
        paths.append(str(p))
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0", UBSAN_OPTIONS="print_stacktrace=1")
    run = subprocess.run([exe, "20000", "20261204", *paths], capture_output=True, text=True, env=env, timeout=600)
    assert run.returncode == 0, (run.returncode, run.stdout[-1000:], run.stderr[-4000:])
    codes = dict(tuple(int(v) for v in c.split(":")) for c in run.stdout.split()[1:])
    assert sum(codes.values()) == 20000
    assert codes.get(0, 0) > 0 and codes.get(-1, 0) > 0
