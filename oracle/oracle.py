"""ctypes bindings for the CPU oracle (oracle/_build/liboracle.so) and, where it
was built in the development container, the reference's own CPU path
(oracle/_ref/libjams_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline leg.  The GPU library never
imports or calls anything here.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import List, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libjams_ref.so")


class OrcTerm(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("n_int", ctypes.c_int32),
        ("bi", ctypes.POINTER(ctypes.c_int32)),
        ("bj", ctypes.POINTER(ctypes.c_int32)),
        ("T", ctypes.POINTER(ctypes.c_int32)),
        ("J", ctypes.POINTER(ctypes.c_double)),
        ("K", ctypes.POINTER(ctypes.c_double)),
        ("axis", ctypes.POINTER(ctypes.c_double)),
        ("B", ctypes.c_double * 3),
        ("r_cutoff", ctypes.c_double),
        ("distance_tolerance", ctypes.c_double),
        ("lattice_parameter", ctypes.c_double),
        ("lattice_vectors", ctypes.POINTER(ctypes.c_double)),
        ("positions", ctypes.POINTER(ctypes.c_double)),
        ("pulse", ctypes.c_int32),
        ("time_center", ctypes.c_double),
        ("freq_bandwidth", ctypes.c_double),
        ("freq_center", ctypes.c_double),
        ("dc_field", ctypes.POINTER(ctypes.c_double)),
        ("ac_field", ctypes.POINTER(ctypes.c_double)),
        ("ac_frequency", ctypes.POINTER(ctypes.c_double)),
    ]


class OrcModel(ctypes.Structure):
    _fields_ = [
        ("L", ctypes.c_int32 * 3),
        ("periodic", ctypes.c_int32 * 3),
        ("nb", ctypes.c_int32),
        ("mus", ctypes.POINTER(ctypes.c_double)),
        ("gyro", ctypes.POINTER(ctypes.c_double)),
        ("alpha", ctypes.POINTER(ctypes.c_double)),
        ("n_terms", ctypes.c_int32),
        ("terms", ctypes.POINTER(OrcTerm)),
        ("dt", ctypes.c_double),
        ("temperature", ctypes.c_double),
        ("gilbert_prefactor", ctypes.c_int32),
        ("integrator", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("replica", ctypes.c_uint32),
        ("serial_noise", ctypes.c_int32),
    ]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def build(quiet: bool = True) -> None:
    """Compile liboracle.so with the Makefile beside this file."""
    out = subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile")],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_create.argtypes = [ctypes.POINTER(OrcModel), ctypes.POINTER(ctypes.c_void_p)]
        L.orc_create.restype = ctypes.c_int
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_num_spins.argtypes = [ctypes.c_void_p]
        L.orc_num_spins.restype = ctypes.c_int64
        L.orc_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int64, ctypes.c_int32]
        L.orc_fields.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                                 ctypes.POINTER(ctypes.c_double)]
        L.orc_energies.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                                   ctypes.POINTER(ctypes.c_double)]
        L.orc_magnetisation.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double)]
        L.orc_exchange_csr.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.POINTER(ctypes.c_int64)),
                                       ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)),
                                       ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
        L.orc_noise_normals.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32,
                                        ctypes.POINTER(ctypes.c_float)]
        L.orc_noise_normals.restype = None
        L.orc_sigma.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        L.orc_sigma.restype = ctypes.c_double
        L.orc_topological_charge_triangular.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int32,
                                                        ctypes.c_int32]
        L.orc_topological_charge_triangular.restype = ctypes.c_double
        L.orc_set_threads.argtypes = [ctypes.c_int32]
        L.orc_set_threads.restype = None
        _lib = L
    return _lib


class _Packed:
    """Keeps the numpy buffers behind an OrcModel alive."""

    def __init__(self, workload, replica: int, serial_noise: bool):
        m = workload.model
        rep = workload.replicas[replica]
        self.keep = []
        terms = (OrcTerm * max(len(m.terms), 1))()
        for k, t in enumerate(m.terms):
            ot = terms[k]
            ot.kind = t.kind
            ot.order = t.order
            if t.bi is not None:
                bi = np.ascontiguousarray(t.bi, dtype=np.int32)
                bj = np.ascontiguousarray(t.bj, dtype=np.int32)
                T = np.ascontiguousarray(t.T, dtype=np.int32).reshape(-1)
                J = np.ascontiguousarray(t.J, dtype=np.float64).reshape(-1)
                self.keep += [bi, bj, T, J]
                ot.n_int = len(bi)
                ot.bi, ot.bj, ot.T, ot.J = _ip(bi), _ip(bj), _ip(T), _dp(J)
            if t.K is not None:
                K = np.ascontiguousarray(t.K, dtype=np.float64)
                ax = np.ascontiguousarray(t.axis, dtype=np.float64).reshape(-1)
                self.keep += [K, ax]
                ot.K, ot.axis = _dp(K), _dp(ax)
            B = t.B
            if t.kind == 3 and rep.B is not None:
                B = rep.B
            for j in range(3):
                ot.B[j] = float(B[j])
            if t.kind == 4:   # dipole
                vec = np.ascontiguousarray(t.lattice_vectors, dtype=np.float64).reshape(-1)
                pos = np.ascontiguousarray(t.positions, dtype=np.float64).reshape(-1)
                self.keep += [vec, pos]
                ot.r_cutoff, ot.distance_tolerance = float(t.r_cutoff), float(t.distance_tolerance)
                ot.lattice_parameter = float(t.lattice_parameter)
                ot.lattice_vectors, ot.positions = _dp(vec), _dp(pos)
            ot.pulse, ot.time_center = int(t.pulse), float(t.time_center)
            ot.freq_bandwidth, ot.freq_center = float(t.freq_bandwidth), float(t.freq_center)
            for name in ("dc_field", "ac_field", "ac_frequency"):
                v = getattr(t, name)
                if v is not None:
                    a = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
                    self.keep.append(a)
                    setattr(ot, name, _dp(a))
        self.terms = terms
        mus = np.ascontiguousarray(m.mus, dtype=np.float64)
        gyro = np.ascontiguousarray(m.gyro, dtype=np.float64)
        alpha = np.ascontiguousarray(m.alpha, dtype=np.float64)
        self.keep += [mus, gyro, alpha]
        om = OrcModel()
        for j in range(3):
            om.L[j] = int(rep.L[j])
            om.periodic[j] = int(m.periodic[j])
        om.nb = m.nb
        om.mus, om.gyro, om.alpha = _dp(mus), _dp(gyro), _dp(alpha)
        om.n_terms = len(m.terms)
        om.terms = ctypes.cast(terms, ctypes.POINTER(OrcTerm))
        om.dt = m.dt
        om.temperature = float(rep.temperature)
        om.gilbert_prefactor = int(bool(m.gilbert_prefactor))
        om.integrator = int(m.integrator)
        om.seed = int(workload.seed)
        om.replica = int(replica)
        om.serial_noise = int(bool(serial_noise))
        self.model = om


class OracleSim:
    """One replica of a workload on the CPU oracle."""

    def __init__(self, workload, replica: int = 0, serial_noise: bool = False,
                 threads: Optional[int] = None):
        self.L = lib()
        if threads:
            self.L.orc_set_threads(int(threads))
        self.packed = _Packed(workload, replica, serial_noise)
        h = ctypes.c_void_p()
        if self.L.orc_create(ctypes.byref(self.packed.model), ctypes.byref(h)) != 0:
            raise RuntimeError(self.L.orc_last_error().decode())
        self.h = h
        self.n = int(self.L.orc_num_spins(h))
        self.n_terms = len(workload.model.terms)
        self.iteration = 0
        self.dt = workload.model.dt

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def run(self, spins: np.ndarray, nsteps: int, first_step: Optional[int] = None) -> np.ndarray:
        s = np.ascontiguousarray(spins, dtype=np.float64).copy()
        fs = self.iteration if first_step is None else first_step
        self.L.orc_run(self.h, _dp(s), int(fs), int(nsteps))
        self.iteration = fs + nsteps
        return s

    def time(self) -> float:
        """The solver time (ps) after the steps run so far: iteration * dt."""
        return self.iteration * self.dt

    def fields(self, spins: np.ndarray, t: Optional[float] = None) -> np.ndarray:
        s = np.ascontiguousarray(spins, dtype=np.float64)
        h = np.empty_like(s)
        self.L.orc_fields(self.h, _dp(s), self.time() if t is None else float(t), _dp(h))
        return h

    def energies(self, spins: np.ndarray, t: Optional[float] = None) -> np.ndarray:
        s = np.ascontiguousarray(spins, dtype=np.float64)
        e = np.empty(self.n_terms)
        self.L.orc_energies(self.h, _dp(s), self.time() if t is None else float(t), _dp(e))
        return e

    def magnetisation(self, spins: np.ndarray) -> np.ndarray:
        s = np.ascontiguousarray(spins, dtype=np.float64)
        m = np.empty(4)
        self.L.orc_magnetisation(self.h, _dp(s), _dp(m))
        return m

    def csr(self, term: int = 0):
        nnz = ctypes.c_int64()
        rows = ctypes.POINTER(ctypes.c_int64)()
        cols = ctypes.POINTER(ctypes.c_int32)()
        vals = ctypes.POINTER(ctypes.c_double)()
        if self.L.orc_exchange_csr(self.h, term, ctypes.byref(nnz), ctypes.byref(rows), ctypes.byref(cols),
                                   ctypes.byref(vals)) != 0:
            raise RuntimeError(self.L.orc_last_error().decode())
        k = nnz.value
        r = np.ctypeslib.as_array(rows, shape=(3 * self.n + 1,)).copy()
        c = np.ctypeslib.as_array(cols, shape=(max(k, 1),))[:k].copy()
        v = np.ctypeslib.as_array(vals, shape=(max(k, 1),))[:k].copy()
        return r, c, v

    def sigma(self, b: int) -> float:
        return float(self.L.orc_sigma(self.h, b))


def noise_normals(seed: int, replica: int, step: int, spin: int) -> np.ndarray:
    out = (ctypes.c_float * 3)()
    lib().orc_noise_normals(seed, replica, step, spin, out)
    return np.array(out[:], dtype=np.float32)


def topological_charge_triangular(spins: np.ndarray, L1: int, L2: int) -> float:
    s = np.ascontiguousarray(spins, dtype=np.float64)
    return float(lib().orc_topological_charge_triangular(_dp(s), L1, L2))


# --------------------------------------------------------------------------
# the reference itself (only where oracle/_ref was built from its sources)
# --------------------------------------------------------------------------

def reference_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


REF_OMP_LIB_PATH = os.path.join(HERE, "_ref_omp", "libjams_ref.so")
_refs = {}


def ref_lib(path: Optional[str] = None):
    """The reference build (oracle/_ref) or another build of the same
    harness, e.g. the OpenMP one in oracle/_ref_omp."""
    path = path or REF_LIB_PATH
    if path not in _refs:
        R = ctypes.CDLL(path)
        R.ref_create.argtypes = [ctypes.POINTER(OrcModel), ctypes.c_double]
        R.ref_create.restype = ctypes.c_int
        R.ref_last_error.restype = ctypes.c_char_p
        R.ref_run.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        R.ref_fields.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        R.ref_energies.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        R.ref_destroy.restype = None
        R.ref_seed.argtypes = [ctypes.c_uint64]
        R.ref_seed.restype = None
        R.ref_rk4_run.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        R.ref_term_fields.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        _refs[path] = R
    return _refs[path]


class ReferenceSim:
    """The reference's HeunLLGSolver (one global instance at a time).

    seed: seeds the reference's global pcg32 before the solver is made, so
    that its own thermal noise (pcg32_k1024 + std::normal_distribution,
    src/jams/solvers/cpu_llg_heun.cc:50-63) is reproducible.  rk4_run: the
    reference's RK4 kernels built for the host, driven as
    CudaRK4BaseSolver::run drives them (T = 0)."""

    def __init__(self, workload, replica: int = 0, seed: Optional[int] = None, lib_path: Optional[str] = None):
        self.R = ref_lib(lib_path)
        if seed is not None:
            self.R.ref_seed(int(seed))
        self.packed = _Packed(workload, replica, True)
        if self.R.ref_create(ctypes.byref(self.packed.model), float(workload.model.t_step)) != 0:
            raise RuntimeError(self.R.ref_last_error().decode())
        self.n = int(np.prod(workload.replicas[replica].L)) * workload.model.nb
        self.n_terms = len(workload.model.terms)

    def run(self, spins: np.ndarray, nsteps: int) -> np.ndarray:
        s = np.ascontiguousarray(spins, dtype=np.float64).copy()
        self.R.ref_run(_dp(s), int(nsteps))
        return s

    def rk4_run(self, spins: np.ndarray, nsteps: int) -> np.ndarray:
        s = np.ascontiguousarray(spins, dtype=np.float64).copy()
        if self.R.ref_rk4_run(_dp(s), int(nsteps)) != 0:
            raise RuntimeError(self.R.ref_last_error().decode())
        return s

    def fields(self, spins: np.ndarray) -> np.ndarray:
        s = np.ascontiguousarray(spins, dtype=np.float64)
        h = np.empty_like(s)
        self.R.ref_fields(_dp(s), _dp(h))
        return h

    def term_fields(self, spins: np.ndarray) -> np.ndarray:
        """Each term's field_ (n_terms x N x 3, meV) at the solver time."""
        s = np.ascontiguousarray(spins, dtype=np.float64)
        out = np.empty((self.n_terms,) + s.shape)
        for t in range(self.n_terms):
            if self.R.ref_term_fields(_dp(s), t, _dp(out[t])) != 0:
                raise RuntimeError("term %d" % t)
        return out

    def energies(self, spins: np.ndarray) -> np.ndarray:
        s = np.ascontiguousarray(spins, dtype=np.float64)
        e = np.empty(self.n_terms)
        self.R.ref_energies(_dp(s), _dp(e))
        return e
