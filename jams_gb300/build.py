"""Builds libjams_llg.so (the sm_103a kernels + C ABI) in-tree with nvcc.

    python -m jams_gb300.build        # or jams_gb300.build.build()

Translation units compile in parallel to objects under jams_gb300/_build/,
then link into jams_gb300/_build/libjams_llg.so against the shared CUDA
runtime.  One -gencode: sm_103a only.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libjams_llg.so")
# the bounds-checked build (LLG_BOUNDS_CHECK): every gathered or stored index
# checked, misses reported as LLG_ERR_BOUNDS; a library of its own
OUT_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(OUT_CHECKED, "libjams_llg.so")
SOURCES = ["llg_kernels.cu", "llg_tiled.cu", "llg_tiled_dipole.cu", "llg_tiled_pair.cu", "llg_tiled_tma.cu",
           "llg_tiled_tma_pair.cu", "llg_tiled_z16.cu", "llg_fused_a.cu",
           "llg_fused_b.cu", "llg_observe.cu", "llg_host.cu", "llg_noalloc.cu", "llg_config.cu", "llg_io.cu",
           "llg_dipole.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler",
              "-fPIC,-ffp-contract=off,-Wall", "-I" + os.path.join(HERE, "..", "include")]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _compile(src: str, extra, out: str = OUT) -> str:
    obj = os.path.join(out, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), res.stdout + res.stderr))
    return obj


def _stale(objs, lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "jams_llg.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra=(), checked: bool = False) -> str:
    """Compiles libjams_llg.so (checked=True: the bounds-checked build in
    _build_checked/) and returns its path."""
    extra = list(extra) + os.environ.get("JAMS_LLG_NVCC_EXTRA", "").split()
    out, lib = (OUT_CHECKED, LIB_CHECKED) if checked else (OUT, LIB)
    if checked:
        extra.append("-DLLG_BOUNDS_CHECK")
    os.makedirs(out, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if not force and not _stale(srcs, lib):
        return lib
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra), out), srcs))
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", lib, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), res.stdout + res.stderr))
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
