"""The reference's GPU Heun path restated (refgpu.cu), for the ref-GPU column
of bench.py: build and a ctypes binding.

It takes the same llg_desc as libjams_llg.so (built by jams_gb300.llg from a
workload), runs the reference's launch structure with cuSPARSE, cuRAND and
cuBLAS in FP64, and times steps with CUDA events on its own stream.  It is a
measurement baseline, not part of the library: nothing in jams_gb300 loads it.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libjams_refgpu.so")
SRC = os.path.join(HERE, "refgpu.cu")


def build(force: bool = False) -> str:
    """Compiles libjams_refgpu.so (nvcc, sm_103a, cuSPARSE / cuBLAS / cuRAND)."""
    os.makedirs(OUT, exist_ok=True)
    hdr = os.path.join(HERE, "..", "include", "jams_llg.h")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                                                          os.path.getmtime(hdr)):
        return LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
           "-shared", "-o", LIB, SRC, "-lcusparse", "-lcublas", "-lcurand"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("refgpu build failed:\n%s\n%s" % (" ".join(cmd), res.stdout + res.stderr))
    return LIB


class RefGpu:
    """Replica 0 of a workload on the restated reference GPU path (FP64, Heun)."""

    def __init__(self, workload):
        from jams_gb300 import llg

        self.L = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        self.L.refgpu_create.argtypes = [vp, ctypes.POINTER(vp)]
        self.L.refgpu_last_error.restype = ctypes.c_char_p
        self.L.refgpu_set_state.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        self.L.refgpu_get_state.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        self.L.refgpu_run.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        self.L.refgpu_destroy.argtypes = [vp]
        self.L.refgpu_destroy.restype = None
        self.desc, self._keep = llg.build_desc(workload, llg.FP64)
        self.n = int(np.prod(workload.replicas[0].L)) * workload.model.nb
        h = vp()
        if self.L.refgpu_create(ctypes.cast(ctypes.pointer(self.desc), vp), ctypes.byref(h)) != 0:
            raise RuntimeError(self.L.refgpu_last_error().decode())
        self.h = h

    def set_state(self, s: np.ndarray) -> None:
        a = np.ascontiguousarray(s, dtype=np.float64)
        if self.L.refgpu_set_state(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) != 0:
            raise RuntimeError("refgpu_set_state failed")

    def get_state(self) -> np.ndarray:
        out = np.empty((self.n, 3))
        if self.L.refgpu_get_state(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) != 0:
            raise RuntimeError("refgpu_get_state failed")
        return out

    def run(self, nsteps: int) -> float:
        """Runs nsteps steps; returns their duration (ms, CUDA events)."""
        ms = ctypes.c_float()
        if self.L.refgpu_run(self.h, int(nsteps), ctypes.byref(ms)) != 0:
            raise RuntimeError(self.L.refgpu_last_error().decode())
        return float(ms.value)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.L.refgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
