"""Lattice + Hamiltonian descriptions of the LLG workloads.

A workload is the data a JAMS config file describes for the LLG hot path:
a Bravais lattice with a basis, one material per basis site, an ordered list
of Hamiltonian terms and the solver settings.  Exchange is given as an
interaction template (basis site i, basis site j, lattice translation T, 3x3
tensor), i.e. the output of the reference's
``post_process_interactions`` (src/jams/core/interactions.cc:292-348) with
symmetry operations already applied.

Unit conventions follow the reference:
  * moments in Bohr magnetons -> mu_s = moment * kBohrMagnetonIU (meV/T),
    src/jams/containers/material.h:47
  * gyro in units of the electron gyromagnetic ratio -> gamma in rad/ps/T,
    src/jams/containers/material.h:48 and src/jams/helpers/consts.h:29-31
  * t_step in seconds -> dt = t_step / 1e-12 ps,
    src/jams/solvers/cuda_llg_heun.cu:23-29
  * energies in meV (``energy_units = "meV"``).
"""
from __future__ import annotations

import copy
import dataclasses
import itertools
import math
from typing import List, Optional, Sequence

import numpy as np

# src/jams/helpers/consts.h:15-32
K_ELECTRON_G_FACTOR = 2.0023193043625
K_HBAR_IU = 0.6582119569
K_BOHR_MAGNETON_IU = 0.0578838181
K_GYROMAGNETIC_RATIO_IU = K_ELECTRON_G_FACTOR * K_BOHR_MAGNETON_IU / K_HBAR_IU
K_BOLTZMANN_IU = 0.0861733326

TERM_EXCHANGE = 0
TERM_UNIAXIAL = 1
TERM_CUBIC = 2
TERM_APPLIED_FIELD = 3
TERM_DIPOLE = 4
TERM_ZEEMAN = 5
PULSE_STATIC, PULSE_SINC, PULSE_SINC_COS = 0, 1, 2

HEUN = 0
RK4 = 1

FP64 = 0
FP32C = 1


@dataclasses.dataclass
class Term:
    kind: int
    order: int = 0
    # exchange template
    bi: Optional[np.ndarray] = None  # int32 (n,)
    bj: Optional[np.ndarray] = None  # int32 (n,)
    T: Optional[np.ndarray] = None  # int32 (n, 3)
    J: Optional[np.ndarray] = None  # float64 (n, 3, 3) meV
    # anisotropy per basis site
    K: Optional[np.ndarray] = None  # float64 (nb,) meV
    axis: Optional[np.ndarray] = None  # float64 (nb, 3) or (nb, 3, 3)
    # applied field
    B: Sequence[float] = (0.0, 0.0, 0.0)
    # dipole: cutoff and tolerance in lattice parameters, lattice parameter (m),
    # lattice vectors (rows, lattice parameters), fractional basis positions
    r_cutoff: float = 0.0
    distance_tolerance: float = 1e-4
    lattice_parameter: float = 0.0
    lattice_vectors: Optional[np.ndarray] = None  # (3, 3)
    positions: Optional[np.ndarray] = None  # (nb, 3)
    # applied-field pulse: PULSE_*, centre time (ps), bandwidth and centre
    # frequency (THz)
    pulse: int = PULSE_STATIC
    time_center: float = 0.0
    freq_bandwidth: float = 0.0
    freq_center: float = 0.0
    # zeeman: dc and ac field per basis site (T, (nb, 3)), ac frequency (THz, (nb,))
    dc_field: Optional[np.ndarray] = None
    ac_field: Optional[np.ndarray] = None
    ac_frequency: Optional[np.ndarray] = None
    name: str = ""


@dataclasses.dataclass
class Replica:
    L: Sequence[int]
    temperature: float = 0.0
    B: Optional[Sequence[float]] = None  # overrides the applied-field term


@dataclasses.dataclass
class Model:
    nb: int
    periodic: Sequence[int]
    mus: np.ndarray
    gyro: np.ndarray
    alpha: np.ndarray
    terms: List[Term]
    t_step: float  # seconds, as in the config file
    integrator: int = HEUN
    gilbert_prefactor: bool = False
    cell: Optional[np.ndarray] = None  # 3x3, lattice vectors as columns
    basis_frac: Optional[np.ndarray] = None  # (nb, 3)

    @property
    def dt(self) -> float:
        return self.t_step / 1e-12


@dataclasses.dataclass
class Workload:
    name: str
    model: Model
    replicas: List[Replica]
    steps: int
    seed: int = 1
    start: str = "random"  # "random" or "+z"
    description: str = ""
    # a subset of a larger replica list (one rank's share): the original
    # index of each replica (its start state), and the noise key of this
    # share, distinct per share (None: the full list, keyed by seed)
    replica_ids: Optional[List[int]] = None
    noise_seed: Optional[int] = None

    @property
    def spins_per_replica(self) -> List[int]:
        return [int(np.prod(r.L)) * self.model.nb for r in self.replicas]

    @property
    def total_spins(self) -> int:
        return sum(self.spins_per_replica)


def material(moment_bohr: float, gyro: float = 1.0, alpha: float = 0.01):
    return moment_bohr * K_BOHR_MAGNETON_IU, gyro * K_GYROMAGNETIC_RATIO_IU, alpha


def isotropic(J: float) -> np.ndarray:
    return J * np.eye(3)


def exchange_term(entries, name="exchange") -> Term:
    """entries: list of (bi, bj, (T1, T2, T3), 3x3 tensor)."""
    bi = np.array([e[0] for e in entries], dtype=np.int32)
    bj = np.array([e[1] for e in entries], dtype=np.int32)
    T = np.array([e[2] for e in entries], dtype=np.int32).reshape(-1, 3)
    J = np.array([np.asarray(e[3], dtype=np.float64) for e in entries]).reshape(-1, 3, 3)
    return Term(kind=TERM_EXCHANGE, bi=bi, bj=bj, T=T, J=J, name=name)


def uniaxial_term(nb: int, K: float, axis=(0.0, 0.0, 1.0), power: int = 2) -> Term:
    ax = np.asarray(axis, dtype=np.float64)
    ax = ax / math.sqrt(float(ax @ ax))
    return Term(kind=TERM_UNIAXIAL, order=power, K=np.full(nb, K),
                axis=np.tile(ax, (nb, 1)), name="uniaxial")


def cubic_term(nb: int, K: float, order: int = 1, u=(1, 0, 0), v=(0, 1, 0), w=(0, 0, 1)) -> Term:
    ax = np.array([u, v, w], dtype=np.float64)
    ax = ax / np.sqrt((ax * ax).sum(axis=1, keepdims=True))
    return Term(kind=TERM_CUBIC, order=order, K=np.full(nb, K),
                axis=np.tile(ax, (nb, 1, 1)), name="cubic")


def field_term(B, pulse=PULSE_STATIC, time_center=0.0, freq_bandwidth=0.0, freq_center=0.0) -> Term:
    """Applied field B (T), static or times a sinc / sinc-cos pulse (centre
    time in ps, bandwidth and centre frequency in THz)."""
    return Term(kind=TERM_APPLIED_FIELD, B=tuple(float(b) for b in B), pulse=int(pulse),
                time_center=float(time_center), freq_bandwidth=float(freq_bandwidth),
                freq_center=float(freq_center), name="applied-field")


def zeeman_term(dc, ac=None, frequency=None) -> Term:
    """Zeeman term: per basis site dc field (T), optional ac field (T) and its
    frequency (THz): mu_s (B_dc + B_ac cos(2 pi f t))."""
    dc = np.ascontiguousarray(np.asarray(dc, dtype=np.float64).reshape(-1, 3))
    t = Term(kind=TERM_ZEEMAN, dc_field=dc, name="zeeman")
    if ac is not None:
        t.ac_field = np.ascontiguousarray(np.asarray(ac, dtype=np.float64).reshape(-1, 3))
        t.ac_frequency = np.ascontiguousarray(np.asarray(frequency, dtype=np.float64).reshape(-1))
    return t


def dipole_term(cell, basis_frac, r_cutoff: float, lattice_parameter: float, tolerance: float = 1e-4) -> Term:
    """Dipole-dipole interaction within r_cutoff (lattice parameters); `cell`
    holds the lattice vectors as columns (as Model.cell)."""
    return Term(kind=TERM_DIPOLE, r_cutoff=float(r_cutoff), distance_tolerance=float(tolerance),
                lattice_parameter=float(lattice_parameter),
                lattice_vectors=np.ascontiguousarray(np.asarray(cell, dtype=np.float64).T),
                positions=np.ascontiguousarray(basis_frac, dtype=np.float64).reshape(-1, 3), name="dipole")


# --------------------------------------------------------------------------
# lattices
# --------------------------------------------------------------------------

def sc_nn_entries(J: float):
    out = []
    for ax in range(3):
        for sgn in (1, -1):
            T = [0, 0, 0]
            T[ax] = sgn
            out.append((0, 0, tuple(T), isotropic(J)))
    return out


def bcc_shell_entries(J1: float, J2: float = 0.0, J3: float = 0.0):
    """bcc as a conventional cubic cell with basis (0,0,0) and (1/2,1/2,1/2).
    Shell 1: 8 neighbours at (+-1/2, +-1/2, +-1/2) a on the other sublattice;
    shell 2: 6 at <100> a; shell 3: 12 at <110> a (same sublattice)."""
    out = []
    for b in (0, 1):
        o = 1 - b
        rng = (-1, 0) if b == 0 else (0, 1)
        if J1 != 0.0:
            for t1 in rng:
                for t2 in rng:
                    for t3 in rng:
                        out.append((b, o, (t1, t2, t3), isotropic(J1)))
        if J2 != 0.0:
            for ax in range(3):
                for sgn in (1, -1):
                    T = [0, 0, 0]
                    T[ax] = sgn
                    out.append((b, b, tuple(T), isotropic(J2)))
        if J3 != 0.0:
            for a1 in range(3):
                for a2 in range(a1 + 1, 3):
                    for s1 in (1, -1):
                        for s2 in (1, -1):
                            T = [0, 0, 0]
                            T[a1] = s1
                            T[a2] = s2
                            out.append((b, b, tuple(T), isotropic(J3)))
    return out


def cross_matrix(d) -> np.ndarray:
    """[d]_x with [d]_x v = d x v."""
    return np.array([[0.0, -d[2], d[1]], [d[2], 0.0, -d[0]], [-d[1], d[0], 0.0]])


def triangular_dmi_entries(J1: float, D: float):
    """Triangular monolayer, a1 = (1,0,0), a2 = (1/2, sqrt3/2, 0).  Tensor
    J_ij = J1 I - [D_ij]_x with D_ij = D (z x r_ij), so that
    E = -1/2 sum_ij J1 S_i.S_j + sum_<ij> D_ij . (S_i x S_j)."""
    a1 = np.array([1.0, 0.0, 0.0])
    a2 = np.array([0.5, math.sqrt(3.0) / 2.0, 0.0])
    out = []
    for T in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (1, -1, 0), (-1, 1, 0)):
        r = T[0] * a1 + T[1] * a2
        r = r / math.sqrt(float(r @ r))
        d = D * np.cross(np.array([0.0, 0.0, 1.0]), r)
        out.append((0, 0, T, J1 * np.eye(3) - cross_matrix(d)))
    return out


# --------------------------------------------------------------------------
# the five workloads of the benchmark definition (sizes overridable for tests)
# --------------------------------------------------------------------------

def sc_ferromagnet(L=32, steps=1000, T=0.0, seed=1, J=1.0, dz=0.1, B=(0.0, 0.0, 1.0),
                   mu=2.0, alpha=0.1, t_step=1e-15, precision_note="", periodic=(1, 1, 1),
                   dipole_cutoff=None, lattice_parameter=3.0e-10) -> Workload:
    """Simple-cubic ferromagnet, isotropic NN exchange J (meV), uniaxial K1 = dz
    along z, Zeeman B (T), Heun, dt = 1 fs, random-sphere start; with
    dipole_cutoff (lattice parameters) also the dipole-dipole term."""
    mus, gyro, al = material(mu, 1.0, alpha)
    terms = [exchange_term(sc_nn_entries(J)), uniaxial_term(1, dz), field_term(B)]
    if dipole_cutoff:
        terms.append(dipole_term(np.eye(3), np.zeros((1, 3)), dipole_cutoff, lattice_parameter))
    model = Model(nb=1, periodic=tuple(periodic), mus=np.array([mus]), gyro=np.array([gyro]),
                  alpha=np.array([al]), terms=terms, t_step=t_step, integrator=HEUN,
                  cell=np.eye(3), basis_frac=np.zeros((1, 3)))
    Ls = (L, L, L) if np.isscalar(L) else tuple(L)
    return Workload(name=f"sc{Ls[0]}x{Ls[1]}x{Ls[2]}", model=model,
                    replicas=[Replica(L=Ls, temperature=T)], steps=steps, seed=seed,
                    start="random",
                    description="simple-cubic FM, NN J=%g meV, K1=%g meV z, B=%s T, Heun" % (J, dz, B))


def bcc_three_shell(L=64, steps=20000, T=300.0, seed=1, start="+z", t_step=0.5e-15,
                    dipole_cutoff=None, lattice_parameter=2.87e-10) -> Workload:
    """bcc, 2-site conventional basis, isotropic J1=2.0, J2=1.2, J3=-0.1 meV,
    mu_s = 2.2 muB, cubic K1 = 0.005 meV (x, y, z axes), Heun alpha = 0.05;
    with dipole_cutoff (lattice parameters) also the dipole-dipole term."""
    mus, gyro, al = material(2.2, 1.0, 0.05)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0.5]], dtype=np.float64)
    terms = [exchange_term(bcc_shell_entries(2.0, 1.2, -0.1)), cubic_term(2, 0.005)]
    desc = "bcc 2-site basis, J1=2.0 J2=1.2 J3=-0.1 meV, cubic K1=0.005 meV, Heun a=0.05 dt=0.5fs"
    if dipole_cutoff:
        terms.append(dipole_term(np.eye(3), basis, dipole_cutoff, lattice_parameter))
        desc += ", dipole r_c=%g a" % dipole_cutoff
    model = Model(nb=2, periodic=(1, 1, 1), mus=np.full(2, mus), gyro=np.full(2, gyro),
                  alpha=np.full(2, al), terms=terms, t_step=t_step, integrator=HEUN,
                  cell=np.eye(3), basis_frac=basis)
    Ls = (L, L, L) if np.isscalar(L) else tuple(L)
    return Workload(name=f"bcc{Ls[0]}_3shell" + ("_dipole" if dipole_cutoff else ""), model=model,
                    replicas=[Replica(L=Ls, temperature=T)], steps=steps, seed=seed, start=start,
                    description=desc)


def bcc_nearest_neighbour(L=256, steps=2000, T=500.0, seed=1, start="+z", t_step=0.5e-15) -> Workload:
    """bcc 2-site basis with the simple-cubic workload's Hamiltonian: NN J = 1.0
    meV (8 neighbours), uniaxial K1 = 0.1 meV z, B = (0, 0, 1) T, mu_s = 2 muB,
    alpha = 0.1, Heun dt = 0.5 fs."""
    mus, gyro, al = material(2.0, 1.0, 0.1)
    terms = [exchange_term(bcc_shell_entries(1.0)), uniaxial_term(2, 0.1), field_term((0.0, 0.0, 1.0))]
    model = Model(nb=2, periodic=(1, 1, 1), mus=np.full(2, mus), gyro=np.full(2, gyro),
                  alpha=np.full(2, al), terms=terms, t_step=t_step, integrator=HEUN,
                  cell=np.eye(3), basis_frac=np.array([[0, 0, 0], [0.5, 0.5, 0.5]]))
    Ls = (L, L, L) if np.isscalar(L) else tuple(L)
    return Workload(name=f"bcc{Ls[0]}_nn", model=model,
                    replicas=[Replica(L=Ls, temperature=T)], steps=steps, seed=seed, start=start,
                    description="bcc 2-site basis, NN J=1 meV, K1=0.1 meV z, B=1 T z, Heun a=0.1 dt=0.5fs")


def fcc_entries(J1: float, J2: Optional[float] = None):
    """Exchange template of the 4-site conventional fcc cell (sites at
    (0,0,0), (0,1/2,1/2), (1/2,0,1/2), (1/2,1/2,0)): the 12 nearest
    neighbours at a/sqrt2 and, with J2, the 6 at a."""
    f = np.array([[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]])
    out = []
    for bi in range(4):
        for bj in range(4):
            for T in itertools.product((-1, 0, 1), repeat=3):
                d = np.asarray(T) + f[bj] - f[bi]
                r2 = float(d @ d)
                if abs(r2 - 0.5) < 1e-9:
                    out.append((bi, bj, T, isotropic(J1)))
                elif J2 is not None and abs(r2 - 1.0) < 1e-9:
                    out.append((bi, bj, T, isotropic(J2)))
    return out


def fcc_ferromagnet(L=64, steps=2000, T=300.0, seed=1, J1=1.5, J2=None, start="+z", t_step=0.5e-15) -> Workload:
    """fcc, 4-site conventional basis, isotropic J1 (12 neighbours) and
    optional J2 (6), mu_s = 1.7 muB, uniaxial K1 = 0.01 meV z, B = 0.5 T z,
    Heun alpha = 0.05, dt = 0.5 fs (as the bcc configurations: the exchange
    field is ~180 T)."""
    mus, gyro, al = material(1.7, 1.0, 0.05)
    basis = np.array([[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]], dtype=np.float64)
    terms = [exchange_term(fcc_entries(J1, J2)), uniaxial_term(4, 0.01), field_term((0.0, 0.0, 0.5))]
    model = Model(nb=4, periodic=(1, 1, 1), mus=np.full(4, mus), gyro=np.full(4, gyro),
                  alpha=np.full(4, al), terms=terms, t_step=t_step, integrator=HEUN,
                  cell=np.eye(3), basis_frac=basis)
    Ls = (L, L, L) if np.isscalar(L) else tuple(L)
    shells = "J1=%g" % J1 + ("" if J2 is None else " J2=%g" % J2)
    return Workload(name=f"fcc{Ls[0]}_" + ("2shell" if J2 is not None else "nn"), model=model,
                    replicas=[Replica(L=Ls, temperature=T)], steps=steps, seed=seed, start=start,
                    description="fcc 4-site basis, %s meV, K1=0.01 meV z, B=0.5 T z, Heun a=0.05 dt=0.5fs" % shells)


def sc_temperature_sweep(n_replicas=256, L_min=16, L_max=64, T_max=1200.0, steps=10000, seed=1,
                         t_step=1e-15) -> Workload:
    """Independent simple-cubic replicas, edge length uniform in {L_min..L_max}
    (seeded), NN J = 1.0 meV, K1 = 0.05 meV z, no field, mu_s = 2 muB,
    alpha = 0.1, T linear in 0..T_max."""
    rng = np.random.default_rng(seed)
    edges = rng.integers(L_min, L_max + 1, size=n_replicas)
    mus, gyro, al = material(2.0, 1.0, 0.1)
    terms = [exchange_term(sc_nn_entries(1.0)), uniaxial_term(1, 0.05)]
    model = Model(nb=1, periodic=(1, 1, 1), mus=np.array([mus]), gyro=np.array([gyro]),
                  alpha=np.array([al]), terms=terms, t_step=t_step, integrator=HEUN,
                  cell=np.eye(3), basis_frac=np.zeros((1, 3)))
    temps = [T_max * r / max(n_replicas - 1, 1) for r in range(n_replicas)]
    reps = [Replica(L=(int(e), int(e), int(e)), temperature=t) for e, t in zip(edges, temps)]
    return Workload(name=f"sc_sweep{n_replicas}", model=model, replicas=reps, steps=steps,
                    seed=seed, start="random",
                    description="%d SC replicas L in {%d..%d}, T in 0..%g K" % (n_replicas, L_min, L_max, T_max))


def triangular_dmi_field_sweep(L=2048, n_fields=16, B_max=2.0, steps=5000, T=5.0, seed=1,
                               t_step=1e-15, dipole_cutoff=None, lattice_parameter=3.0e-10) -> Workload:
    """Triangular monolayer, tensor exchange J1 = 1.0 meV + interfacial DMI
    D = 0.3 meV, K1 = 0.2 meV z, mu_s = 2 muB, RK4 alpha = 0.3, one replica per
    field B_z in 0..B_max; with dipole_cutoff also the dipole-dipole term."""
    mus, gyro, al = material(2.0, 1.0, 0.3)
    terms = [exchange_term(triangular_dmi_entries(1.0, 0.3)), uniaxial_term(1, 0.2),
             field_term((0.0, 0.0, 0.0))]
    cell = np.array([[1.0, 0.5, 0.0], [0.0, math.sqrt(3.0) / 2.0, 0.0], [0.0, 0.0, 1.0]])
    if dipole_cutoff:
        terms.append(dipole_term(cell, np.zeros((1, 3)), dipole_cutoff, lattice_parameter))
    model = Model(nb=1, periodic=(1, 1, 0), mus=np.array([mus]), gyro=np.array([gyro]),
                  alpha=np.array([al]), terms=terms, t_step=t_step, integrator=RK4,
                  cell=cell, basis_frac=np.zeros((1, 3)))
    Ls = (L, L, 1) if np.isscalar(L) else tuple(L)
    reps = [Replica(L=Ls, temperature=T, B=(0.0, 0.0, B_max * k / max(n_fields - 1, 1)))
            for k in range(n_fields)]
    return Workload(name=f"tri{Ls[0]}_dmi_x{n_fields}", model=model, replicas=reps, steps=steps,
                    seed=seed, start="random",
                    description="triangular monolayer J1=1 D=0.3 meV, K1=0.2 meV, RK4 a=0.3, B_z sweep")


def split_exchange(w: Workload, offdiag: float = 0.0) -> Workload:
    """The same workload with its first term (an exchange template) given as
    two exchange terms of half strength each, as a config with two exchange
    modules would give it.  With offdiag != 0 the second term also carries a
    symmetric off-diagonal tensor part J_xy = J_yx = offdiag * J_xx on one
    pair: its first entry and the reverse entry (partner and site swapped,
    translation negated), so the coupling stays reciprocal.  The lattice
    families' stencils take isotropic J only (the triangular family aside),
    so the FP32C form then runs the gather kernels; without it the two terms
    are summed into one stencil."""
    w2 = copy.deepcopy(w)
    ex = w2.model.terms[0]
    assert ex.kind == TERM_EXCHANGE
    Jb = ex.J * 0.5
    if offdiag:
        Jb = Jb.copy()
        rev = [e for e in range(len(ex.bi)) if ex.bi[e] == ex.bj[0] and ex.bj[e] == ex.bi[0]
               and np.array_equal(ex.T[e], -ex.T[0])]
        for e in [0] + rev[:1]:
            Jb[e, 0, 1] += offdiag * Jb[e, 0, 0]
            Jb[e, 1, 0] += offdiag * Jb[e, 0, 0]
    w2.model.terms = [Term(kind=ex.kind, bi=ex.bi, bj=ex.bj, T=ex.T, J=ex.J * 0.5, name="exchange-a"),
                      Term(kind=ex.kind, bi=ex.bi, bj=ex.bj, T=ex.T, J=Jb, name="exchange-b")] + \
        w2.model.terms[1:]
    w2.name += "_split" if not offdiag else "_generic"
    return w2


# --------------------------------------------------------------------------
# seeded initial states
# --------------------------------------------------------------------------

def random_sphere(n: int, seed: int) -> np.ndarray:
    """Uniform unit vectors by Marsaglia's method (as uniform_random_sphere,
    src/jams/helpers/random.h:12-26), from a seeded numpy generator."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, 3))
    filled = 0
    while filled < n:
        m = max(2 * (n - filled), 16)
        v = rng.random((m, 2)) * 2.0 - 1.0
        s = (v * v).sum(axis=1)
        v = v[s <= 1.0]
        s = s[s <= 1.0]
        k = min(len(s), n - filled)
        v, s = v[:k], s[:k]
        ss = 2.0 * np.sqrt(1.0 - s)
        out[filled:filled + k, 0] = v[:, 0] * ss
        out[filled:filled + k, 1] = v[:, 1] * ss
        out[filled:filled + k, 2] = 1.0 - 2.0 * s
        filled += k
    norm = np.sqrt((out * out).sum(axis=1, keepdims=True))
    return out / norm


def initial_state(w: Workload, replica: int) -> np.ndarray:
    n = w.spins_per_replica[replica]
    if w.start == "+z":
        s = np.zeros((n, 3))
        s[:, 2] = 1.0
        return s
    rid = w.replica_ids[replica] if w.replica_ids is not None else replica
    return random_sphere(n, w.seed * 7919 + rid)
