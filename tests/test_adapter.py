"""The JAMS solver adapter (integration/cuda_llg_fused_solver.{h,cc})
compiled against the reference's own headers (src/jams: Solver, Hamiltonian,
Monitor, Physics, globals) with the oracle's stand-in headers, linked with
the reference's Solver, Base and Physics objects (oracle/_ref, built from
the reference sources) and libjams_llg.so, then run on the CPU
(tests/adapter_check.cc): the cadence rule against the reference's driver
loop, the error convention, and a library call.  Skipped where the
reference sources are not present."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = os.environ.get("JAMS_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")
REF_OBJS = [os.path.join(ROOT, "oracle", "_ref", "core", n) for n in ("solver.o", "base.o", "physics.o")]


def _pcg_include():
    pyarrow = pytest.importorskip("pyarrow")
    return os.path.join(os.path.dirname(pyarrow.__file__), "include")


def test_adapter_builds_against_the_reference_and_keeps_its_cadence(llg, tmp_path):
    if not os.path.isdir(os.path.join(REFERENCE, "src", "jams")):
        pytest.skip("the reference sources are not present")
    if not all(os.path.exists(o) for o in REF_OBJS):
        pytest.skip("oracle/_ref was not built (oracle/Makefile.ref)")
    flags = ["-std=c++17", "-O1", "-fPIC", "-ffunction-sections", "-fdata-sections", "-w",
             "-I" + os.path.join(ROOT, "oracle", "shim"), "-I" + os.path.join(ROOT, "oracle"),
             "-I" + os.path.join(REFERENCE, "src"), "-I" + _pcg_include(), "-I" + os.path.join(ROOT, "include"),
             "-I" + os.path.join(ROOT, "integration")]
    objs = []
    for src in (os.path.join(ROOT, "integration", "cuda_llg_fused_solver.cc"),
                os.path.join(ROOT, "tests", "adapter_check.cc")):
        obj = str(tmp_path / (os.path.basename(src) + ".o"))
        r = subprocess.run(["g++", *flags, "-c", src, "-o", obj], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        objs.append(obj)
    exe = str(tmp_path / "adapter_check")
    libdir = os.path.dirname(llg.LIB_PATH)
    r = subprocess.run(["g++", "-o", exe, *objs, *REF_OBJS, "-Wl,--gc-sections", "-L" + libdir, "-ljams_llg",
                        "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "adapter checks passed" in r.stdout
