"""Python binding of libjams_llg.so through its C ABI (include/jams_llg.h).

Used by the tests, the benchmark and the smoke check.  The library must have
been built (``jams_gb300.build.build()``); there is no fallback: if the shared
library is missing or no sm_103 device is present, construction raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

from . import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libjams_llg.so")

LLG_ABI_VERSION = 3
FP64 = 0
FP32C = 1
HEUN = 0
RK4 = 1

ERRORS = {
    -1: "LLG_ERR_BAD_DESC", -2: "LLG_ERR_OOM", -3: "LLG_ERR_CUDA", -4: "LLG_ERR_TIMEOUT",
    -5: "LLG_ERR_NONFINITE", -6: "LLG_ERR_NO_DEVICE", -7: "LLG_ERR_UNSUPPORTED", -8: "LLG_ERR_IO",
    -9: "LLG_ERR_BOUNDS",
}

EXPORTED = [
    "llg_create", "llg_destroy", "llg_last_error", "llg_num_spins", "llg_num_replicas",
    "llg_set_state", "llg_get_state", "llg_set_state_device", "llg_get_state_device", "llg_step",
    "llg_synchronize", "llg_iteration", "llg_set_iteration", "llg_set_temperature", "llg_set_field",
    "llg_fields", "llg_observables", "llg_topological_charge", "llg_set_stream", "llg_last_launch_count",
    "llg_profile_stages", "llg_kernel_info", "llg_set_tuning", "llg_autotune", "llg_magnetisation_noalloc",
    "llg_create_from_config", "llg_config_describe", "llg_max_steps",
    "llg_write_array_file", "llg_read_array_file", "llg_write_spins", "llg_read_spins",
    "llg_save_checkpoint", "llg_load_checkpoint", "llg_magnetisation_groups", "llg_term_fields",
    "llg_term_fields_device",
]


class LLGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s: %s" % (ERRORS.get(code, code), msg))
        self.code = code


class LlgTerm(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32), ("order", ctypes.c_int32), ("n_int", ctypes.c_int32),
        ("bi", ctypes.POINTER(ctypes.c_int32)), ("bj", ctypes.POINTER(ctypes.c_int32)),
        ("T", ctypes.POINTER(ctypes.c_int32)), ("J", ctypes.POINTER(ctypes.c_double)),
        ("K", ctypes.POINTER(ctypes.c_double)), ("axis", ctypes.POINTER(ctypes.c_double)),
        ("B", ctypes.c_double * 3),
        ("r_cutoff", ctypes.c_double), ("distance_tolerance", ctypes.c_double),
        ("lattice_parameter", ctypes.c_double), ("lattice_vectors", ctypes.POINTER(ctypes.c_double)),
        ("positions", ctypes.POINTER(ctypes.c_double)),
        ("pulse", ctypes.c_int32), ("time_center", ctypes.c_double), ("freq_bandwidth", ctypes.c_double),
        ("freq_center", ctypes.c_double), ("dc_field", ctypes.POINTER(ctypes.c_double)),
        ("ac_field", ctypes.POINTER(ctypes.c_double)), ("ac_frequency", ctypes.POINTER(ctypes.c_double)),
    ]


class LlgReplica(ctypes.Structure):
    _fields_ = [("L", ctypes.c_int32 * 3), ("temperature", ctypes.c_double), ("B", ctypes.c_double * 3),
                ("use_B", ctypes.c_int32)]


class LlgDesc(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int32), ("nb", ctypes.c_int32), ("periodic", ctypes.c_int32 * 3),
        ("mus", ctypes.POINTER(ctypes.c_double)), ("gyro", ctypes.POINTER(ctypes.c_double)),
        ("alpha", ctypes.POINTER(ctypes.c_double)), ("n_terms", ctypes.c_int32),
        ("terms", ctypes.POINTER(LlgTerm)), ("dt", ctypes.c_double), ("gilbert_prefactor", ctypes.c_int32),
        ("integrator", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("rk4_normalise_stages", ctypes.c_int32), ("seed", ctypes.c_uint64), ("n_replicas", ctypes.c_int32),
        ("replicas", ctypes.POINTER(LlgReplica)), ("device", ctypes.c_int32),
        ("steps_per_graph", ctypes.c_int32),
    ]


_libs = {}
LIB_PATH_CHECKED = os.path.join(HERE, "_build_checked", "libjams_llg.so")


def lib(checked: bool = False):
    """Loads libjams_llg.so (raises if it has not been built); checked=True:
    the bounds-checked build (jams_gb300.build.build(checked=True))."""
    path = LIB_PATH_CHECKED if checked else LIB_PATH
    if path not in _libs:
        if not os.path.exists(path):
            raise RuntimeError("libjams_llg.so is not built: run jams_gb300.build.build() (%s)" % path)
        L = ctypes.CDLL(path)
        vp, i32, i64, dp = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(ctypes.c_double)
        L.llg_create.argtypes = [ctypes.POINTER(LlgDesc), ctypes.POINTER(vp)]
        L.llg_destroy.argtypes = [vp]
        L.llg_destroy.restype = None
        L.llg_last_error.argtypes = [vp]
        L.llg_last_error.restype = ctypes.c_char_p
        L.llg_num_spins.argtypes = [vp, i32]
        L.llg_num_spins.restype = i64
        L.llg_num_replicas.argtypes = [vp]
        for f in ("llg_set_state", "llg_get_state", "llg_set_state_device", "llg_get_state_device"):
            getattr(L, f).argtypes = [vp, i32, vp]
        L.llg_step.argtypes = [vp, i32]
        L.llg_synchronize.argtypes = [vp]
        L.llg_iteration.argtypes = [vp]
        L.llg_iteration.restype = i64
        L.llg_set_iteration.argtypes = [vp, i64]
        L.llg_set_temperature.argtypes = [vp, i32, ctypes.c_double]
        L.llg_set_field.argtypes = [vp, i32, dp]
        L.llg_fields.argtypes = [vp, i32, dp]
        L.llg_term_fields.argtypes = [vp, i32, i32, dp]
        L.llg_term_fields_device.argtypes = [vp, i32, i32, vp]
        L.llg_observables.argtypes = [vp, i32, dp, dp]
        L.llg_magnetisation_groups.argtypes = [vp, i32, ctypes.POINTER(i32), i32, i32, dp]
        L.llg_topological_charge.argtypes = [vp, i32, dp]
        L.llg_set_stream.argtypes = [vp, vp]
        L.llg_last_launch_count.argtypes = [vp]
        L.llg_last_launch_count.restype = i64
        L.llg_profile_stages.argtypes = [vp, i32, dp]
        L.llg_kernel_info.argtypes = [vp, ctypes.POINTER(ctypes.c_int32)]
        L.llg_set_tuning.argtypes = [vp, i32, i32]
        L.llg_autotune.argtypes = [vp, i32, i32]
        L.llg_magnetisation_noalloc.argtypes = [vp, i64, i32, dp, vp, vp]
        L.llg_create_from_config.argtypes = [ctypes.c_char_p, ctypes.c_char_p, i32, i32, ctypes.POINTER(vp)]
        L.llg_config_describe.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, i64]
        L.llg_max_steps.argtypes = [vp]
        L.llg_max_steps.restype = i64
        cp = ctypes.c_char_p
        L.llg_write_array_file.argtypes = [cp, cp, dp, i64, i64]
        L.llg_read_array_file.argtypes = [cp, cp, dp, i64, ctypes.POINTER(i64), ctypes.POINTER(i64)]
        for f in ("llg_write_spins", "llg_read_spins"):
            getattr(L, f).argtypes = [vp, i32, cp]
        for f in ("llg_save_checkpoint", "llg_load_checkpoint"):
            getattr(L, f).argtypes = [vp, cp]
        _libs[path] = L
    return _libs[path]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def describe_config(text: str, patch: str = "") -> dict:
    """The model a JAMS config file describes (no GPU needed)."""
    import json

    L = lib()
    n = 1 << 22
    while True:
        buf = ctypes.create_string_buffer(n)
        rc = L.llg_config_describe(text.encode(), patch.encode(), buf, n)
        if rc == 0:
            return json.loads(buf.value.decode())
        msg = L.llg_last_error(None).decode()
        if "buffer too small" in msg and n < (1 << 30):
            n *= 4
            continue
        raise LLGError(rc, msg)


def write_array_file(path: str, array: np.ndarray, dataset: str = "/spins") -> None:
    """Writes a 1-D or 2-D array of doubles: HDF5 dataset `dataset` when
    `path` ends in ".h5", else text (no GPU needed)."""
    a = np.ascontiguousarray(array, dtype=np.float64)
    rows, cols = (a.shape[0], 1) if a.ndim == 1 else a.shape
    rc = lib().llg_write_array_file(os.fsencode(path), dataset.encode(), _dp(a), rows, cols)
    if rc != 0:
        raise LLGError(rc, lib().llg_last_error(None).decode())


def read_array_file(path: str, dataset: str = "/spins") -> np.ndarray:
    """Reads an array as the reference's load_array_from_file does: HDF5
    dataset (rows x cols) or every number of a text file (flat)."""
    L = lib()
    rows, cols = ctypes.c_int64(), ctypes.c_int64()
    rc = L.llg_read_array_file(os.fsencode(path), dataset.encode(), None, 0, ctypes.byref(rows), ctypes.byref(cols))
    if rc == 0:
        out = np.empty((rows.value, cols.value))
        rc = L.llg_read_array_file(os.fsencode(path), dataset.encode(), _dp(out), out.size, ctypes.byref(rows),
                                   ctypes.byref(cols))
    if rc != 0:
        raise LLGError(rc, L.llg_last_error(None).decode())
    return out if cols.value > 1 else out.reshape(-1)


def build_desc(workload: W.Workload, precision: int = FP32C, device: int = 0, steps_per_graph: int = 100,
               rk4_normalise_stages: bool = False):
    """The llg_desc of a workload and the arrays it points into (keep them
    alive while the descriptor is used)."""
    m = workload.model
    keep = []
    terms = (LlgTerm * max(len(m.terms), 1))()
    for k, t in enumerate(m.terms):
        lt = terms[k]
        lt.kind, lt.order = t.kind, t.order
        if t.bi is not None:
            arrs = [np.ascontiguousarray(t.bi, dtype=np.int32), np.ascontiguousarray(t.bj, dtype=np.int32),
                    np.ascontiguousarray(t.T, dtype=np.int32).reshape(-1),
                    np.ascontiguousarray(t.J, dtype=np.float64).reshape(-1)]
            keep += arrs
            lt.n_int = len(arrs[0])
            lt.bi, lt.bj, lt.T, lt.J = _ip(arrs[0]), _ip(arrs[1]), _ip(arrs[2]), _dp(arrs[3])
        if t.K is not None:
            K = np.ascontiguousarray(t.K, dtype=np.float64)
            ax = np.ascontiguousarray(t.axis, dtype=np.float64).reshape(-1)
            keep += [K, ax]
            lt.K, lt.axis = _dp(K), _dp(ax)
        for j in range(3):
            lt.B[j] = float(t.B[j])
        if t.kind == W.TERM_DIPOLE:
            vec = np.ascontiguousarray(t.lattice_vectors, dtype=np.float64).reshape(-1)
            pos = np.ascontiguousarray(t.positions, dtype=np.float64).reshape(-1)
            keep += [vec, pos]
            lt.r_cutoff, lt.distance_tolerance = float(t.r_cutoff), float(t.distance_tolerance)
            lt.lattice_parameter = float(t.lattice_parameter)
            lt.lattice_vectors, lt.positions = _dp(vec), _dp(pos)
        lt.pulse, lt.time_center = int(t.pulse), float(t.time_center)
        lt.freq_bandwidth, lt.freq_center = float(t.freq_bandwidth), float(t.freq_center)
        for name in ("dc_field", "ac_field", "ac_frequency"):
            v = getattr(t, name)
            if v is not None:
                a = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
                keep.append(a)
                setattr(lt, name, _dp(a))
    reps = (LlgReplica * len(workload.replicas))()
    for r, rp in enumerate(workload.replicas):
        for j in range(3):
            reps[r].L[j] = int(rp.L[j])
        reps[r].temperature = float(rp.temperature)
        if rp.B is not None:
            reps[r].use_B = 1
            for j in range(3):
                reps[r].B[j] = float(rp.B[j])
    mats = [np.ascontiguousarray(x, dtype=np.float64) for x in (m.mus, m.gyro, m.alpha)]
    keep += mats
    d = LlgDesc()
    d.abi_version = LLG_ABI_VERSION
    d.nb = m.nb
    for j in range(3):
        d.periodic[j] = int(m.periodic[j])
    d.mus, d.gyro, d.alpha = _dp(mats[0]), _dp(mats[1]), _dp(mats[2])
    d.n_terms = len(m.terms)
    d.terms = ctypes.cast(terms, ctypes.POINTER(LlgTerm))
    d.dt = m.dt
    d.gilbert_prefactor = int(bool(m.gilbert_prefactor))
    d.integrator = int(m.integrator)
    d.precision = int(precision)
    d.rk4_normalise_stages = int(bool(rk4_normalise_stages))
    d.seed = int(workload.seed if workload.noise_seed is None else workload.noise_seed)
    d.n_replicas = len(workload.replicas)
    d.replicas = ctypes.cast(reps, ctypes.POINTER(LlgReplica))
    d.device = int(device)
    d.steps_per_graph = int(steps_per_graph)
    keep += [terms, reps]
    return d, keep


class Solver:
    """A JAMS LLG solver (Heun or RK4) on one GPU for all replicas of a
    workload: the CUDAHeunLLGSolver / CUDALLGRK4Solver of the reference with
    its Hamiltonian terms fused into the stage kernels."""

    def __init__(self, workload: W.Workload, precision: int = FP32C, device: int = 0,
                 steps_per_graph: int = 100, rk4_normalise_stages: bool = False, checked: bool = False):
        self.L = lib(checked)
        self.workload = workload
        m = workload.model
        d, self._keep = build_desc(workload, precision, device, steps_per_graph, rk4_normalise_stages)
        self._desc = d
        h = ctypes.c_void_p()
        rc = self.L.llg_create(ctypes.byref(d), ctypes.byref(h))
        if rc != 0:
            raise LLGError(rc, self.L.llg_last_error(None).decode())
        self.h = h
        self.precision = precision
        self.n_terms = len(m.terms)
        self.n_replicas = len(workload.replicas)

    @classmethod
    def from_config(cls, text: str, patch: str = "", precision: int = FP32C, device: int = 0) -> "Solver":
        """A solver built from the text of a JAMS config file (and patch)."""
        self = cls.__new__(cls)
        self.L = lib()
        h = ctypes.c_void_p()
        rc = self.L.llg_create_from_config(text.encode(), patch.encode(), int(precision), int(device), ctypes.byref(h))
        if rc != 0:
            raise LLGError(rc, self.L.llg_last_error(None).decode())
        self.h = h
        d = describe_config(text, patch)
        self.workload = None
        self.precision = precision
        self.n_terms = len(d["terms"])
        self.n_replicas = 1
        self._integrator = d["integrator"]
        return self

    @property
    def max_steps(self) -> int:
        return int(self.L.llg_max_steps(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.llg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise LLGError(rc, self.L.llg_last_error(self.h).decode())

    def num_spins(self, replica: int = -1) -> int:
        return int(self.L.llg_num_spins(self.h, replica))

    def set_state(self, spins: np.ndarray, replica: int = -1) -> None:
        s = np.ascontiguousarray(spins, dtype=np.float64)
        if s.size != 3 * self.num_spins(replica):
            raise ValueError("expected %d spins" % self.num_spins(replica))
        self._check(self.L.llg_set_state(self.h, replica, s.ctypes.data))

    def get_state(self, replica: int = -1, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.num_spins(replica), 3))
        self._check(self.L.llg_get_state(self.h, replica, out.ctypes.data))
        return out

    def write_spins(self, path: str, replica: int = 0) -> None:
        """/spins (N x 3) of one replica to an HDF5 (".h5") or text file."""
        self._check(self.L.llg_write_spins(self.h, replica, os.fsencode(path)))

    def read_spins(self, path: str, replica: int = 0) -> None:
        """Sets one replica's state from /spins of an HDF5 file or a text file."""
        self._check(self.L.llg_read_spins(self.h, replica, os.fsencode(path)))

    def save_checkpoint(self, path: str) -> None:
        self._check(self.L.llg_save_checkpoint(self.h, os.fsencode(path)))

    def load_checkpoint(self, path: str) -> None:
        self._check(self.L.llg_load_checkpoint(self.h, os.fsencode(path)))

    def set_state_device(self, ptr: int, replica: int = -1) -> None:
        self._check(self.L.llg_set_state_device(self.h, replica, ptr))

    def get_state_device(self, ptr: int, replica: int = -1) -> None:
        self._check(self.L.llg_get_state_device(self.h, replica, ptr))

    def step(self, nsteps: int) -> None:
        self._check(self.L.llg_step(self.h, int(nsteps)))

    def synchronize(self) -> None:
        self._check(self.L.llg_synchronize(self.h))

    @property
    def iteration(self) -> int:
        return int(self.L.llg_iteration(self.h))

    def set_iteration(self, it: int) -> None:
        self._check(self.L.llg_set_iteration(self.h, int(it)))

    def set_temperature(self, replica: int, T: float) -> None:
        self._check(self.L.llg_set_temperature(self.h, replica, float(T)))

    def set_field(self, replica: int, B: Sequence[float]) -> None:
        b = np.ascontiguousarray(B, dtype=np.float64)
        self._check(self.L.llg_set_field(self.h, replica, _dp(b)))

    def fields(self, replica: int = 0) -> np.ndarray:
        out = np.empty((self.num_spins(replica), 3))
        self._check(self.L.llg_fields(self.h, replica, _dp(out)))
        return out

    def term_fields(self, term: int, replica: int = 0) -> np.ndarray:
        """The field (meV, N x 3) of one Hamiltonian term alone."""
        out = np.empty((self.num_spins(replica), 3))
        self._check(self.L.llg_term_fields(self.h, replica, term, _dp(out)))
        return out

    def observables(self, replica: int = 0):
        m4 = np.empty(4)
        e = np.empty(max(self.n_terms, 1))
        self._check(self.L.llg_observables(self.h, replica, _dp(m4), _dp(e)))
        return m4, e[: self.n_terms]

    def magnetisation_groups(self, group_of_basis: Sequence[int], replica: int = 0,
                             normalize: bool = True) -> np.ndarray:
        """Magnetisation by groups of basis sites (the reference monitor's
        "materials" / "positions" / "none" grouping): rows (mx, my, mz, |m|)
        per group, over sum mu_s or in Bohr magnetons (normalize=False)."""
        g = np.ascontiguousarray(group_of_basis, dtype=np.int32)
        ng = int(g.max()) + 1 if g.size else 1
        out = np.empty((ng, 4))
        self._check(self.L.llg_magnetisation_groups(self.h, replica, _ip(g), ng, int(bool(normalize)), _dp(out)))
        return out

    def topological_charge(self, replica: int = 0) -> float:
        q = np.empty(1)
        self._check(self.L.llg_topological_charge(self.h, replica, _dp(q)))
        return float(q[0])

    def set_stream(self, stream_ptr: int) -> None:
        self._check(self.L.llg_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def profile_stages(self, nsteps: int, dipole: bool = False):
        """Mean duration (ms) of each stage kernel over nsteps steps; with
        dipole=True also the dipole-field evaluation before each stage."""
        ms = np.zeros(8)
        self._check(self.L.llg_profile_stages(self.h, int(nsteps), _dp(ms)))
        integ = self.workload.model.integrator if self.workload is not None else self._integrator
        ns = 2 if integ == W.HEUN else 4
        return (ms[:ns], ms[ns:2 * ns]) if dipole else ms[:ns]

    def kernel_info(self) -> dict:
        info = (ctypes.c_int32 * 11)()
        self._check(self.L.llg_kernel_info(self.h, info))
        fam = {0: "generic", 1: "sc", 2: "bcc", 3: "bcc3", 4: "triangular", 5: "fcc", 6: "fcc2"}[info[0]]
        return {"family": fam, "planes_per_cta": info[1], "store_rhs": bool(info[2]), "tile_z": info[3],
                "tile_y": info[4], "fp64": bool(info[5]), "occupancy": info[6], "rows_per_thread": info[7],
                "fused": bool(info[8]), "tma": bool(info[9]), "stored_noise": bool(info[10])}

    def autotune(self, trial_steps: int = 20, use_cache: bool = False) -> dict:
        self._check(self.L.llg_autotune(self.h, int(trial_steps), int(bool(use_cache))))
        return self.kernel_info()

    def set_tuning(self, planes_per_cta: int, store_rhs: bool, occupancy: int = 2, narrow: bool = False,
                   pair: bool = False, fused: bool = False, tma: bool = False, noise: bool = False,
                   half_z: bool = False) -> None:
        """Tiling of the tiled FP32 kernels: planes per CTA, stored-rhs mode
        (Heun: the predictor stores the corrector's partial sum s0 + dt/2
        rhs(s0) instead of the corrector recomputing rhs(s0)), occupancy
        variant 2/3/4 (two rows per thread: 2), narrow tile (half the
        rows), two rows per thread, the fused Heun step (one kernel per
        step), planes loaded by TMA, stored noise (stored-rhs mode: the
        predictor also stores the thermal field for the corrector), the
        half-width simple-cubic tile (16 cells along z)."""
        flags = int(bool(store_rhs)) | (int(bool(narrow)) << 1) | (int(bool(pair)) << 2) | \
            (int(bool(fused)) << 3) | (int(occupancy) << 4) | (int(bool(tma)) << 8) | (int(bool(noise)) << 9) | \
            (int(bool(half_z)) << 10)
        self._check(self.L.llg_set_tuning(self.h, int(planes_per_cta), flags))

    @property
    def last_launch_count(self) -> int:
        return int(self.L.llg_last_launch_count(self.h))
