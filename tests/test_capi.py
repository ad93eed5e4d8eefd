"""CPU checks of the C ABI library: it builds for sm_103a, loads, and exports
every function include/jams_llg.h declares (no device calls)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "jams_llg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(llg_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(llg):
    lib = ctypes.CDLL(llg.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(llg.EXPORTED) == sorted(n for n in names if n in llg.EXPORTED)


def test_library_is_sm103a_only(llg):
    """Every translation unit compiles for sm_103a alone (one -gencode, no
    PTX for other targets)."""
    from jams_gb300 import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert not any("gencode" in f or "arch" in f for f in build.NVCC_FLAGS)


def test_descriptor_layout_matches_header(llg):
    """ctypes mirror of llg_desc has the field order of the header."""
    text = open(os.path.join(ROOT, "include", "jams_llg.h")).read()
    body = text[text.index("typedef struct {\n  int32_t abi_version;"):]
    body = body[: body.index("} llg_desc;")]
    fields = re.findall(r"\b([a-z_0-9]+)(?:\[\d\])?;", body)
    assert fields == [f[0] for f in llg.LlgDesc._fields_]


def test_header_is_plain_c_and_links(llg, tmp_path):
    """A C99 translation unit that includes include/jams_llg.h and takes the
    address of every declared function compiles with gcc and links against
    libjams_llg.so: the boundary is a C ABI, usable from cgo / JNI / ctypes
    stubs without C++."""
    import shutil
    import subprocess

    gcc = shutil.which("gcc")
    if gcc is None:
        import pytest

        pytest.skip("gcc not available")
    names = declared_functions()
    src = tmp_path / "consumer.c"
    src.write_text('#include "jams_llg.h"\n#include <stdio.h>\ntypedef void (*fn)(void);\nint main(void) {\n'
                   '  fn f[] = {\n' + ",\n".join("    (fn)&%s" % n for n in names) +
                   '\n  };\n  printf("%d %d\\n", (int)(sizeof f / sizeof f[0]), LLG_ABI_VERSION);\n  return 0;\n}\n')
    exe = tmp_path / "consumer"
    lib_dir = os.path.dirname(llg.LIB_PATH)
    res = subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                          str(src), "-o", str(exe), "-L", lib_dir, "-ljams_llg", "-Wl,-rpath," + lib_dir],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == [str(len(names)), str(llg.LLG_ABI_VERSION)]
