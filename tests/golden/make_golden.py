"""Generates the golden vectors in tests/golden/ from the REFERENCE itself.

Runs the reference's own CPU Heun solver (HeunLLGSolver::run,
src/jams/solvers/cpu_llg_heun.cc:45-148), its Solver::compute_fields and its
Hamiltonian terms, compiled from the reference sources by
oracle/Makefile.ref into oracle/_ref/libjams_ref.so.  This only works where the
reference sources are present (the development container; the Makefile finds
them through $JAMS_REFERENCE_DIR or a checkout named "reference" beside
this repository):

    make -f oracle/Makefile.ref
    python tests/golden/make_golden.py [case ...]

The dipole cases run the reference's dipole-bruteforce Hamiltonian
(src/jams/hamiltonian/dipole_bruteforce.cc) compiled the same way, the pulse
cases its applied-field pulses and zeeman term (applied_field.cc, zeeman.cc);
these also hold the fields and energies after the 100 steps, at the solver
time 100 dt.

Each T = 0 fixture holds, for a small seeded case: the initial spins, the
total field, each term's field_ and the per-term energies of the reference
at those spins, and the
reference's spins after 1, 10 and 100 Heun steps.  The long cases hold the
spins after up to 1000 steps: Heun on the simple-cubic benchmark lattice
(32^3), and RK4 on a triangular DMI monolayer through the reference's RK4
kernels built for the host (oracle/ref_rk4_kernels.cc).

The thermal cases run the reference's Heun solver at T > 0 with its own
noise (pcg32_k1024 + std::normal_distribution, cpu_llg_heun.cc:50-63),
seeded through the reference's global generator so that the fixture can be
made again, once per seed (THERMAL_REF_SEEDS independent runs, in parallel
processes).  They hold each run's time averages of |M| (the magnetisation
monitor's normalisation by the summed moments) and of the energies per spin,
and their mean and standard error over the runs.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from jams_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.golden.cases import (THERMAL_REF_SEEDS, THERMAL_SEED, cases, dipole_cases, long_cases,  # noqa: E402
                                over_runs, pulse_cases, thermal_cases, thermal_summary)

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    if not O.reference_available():
        raise SystemExit("oracle/_ref/libjams_ref.so is missing: build it with oracle/Makefile.ref first")
    only = set(sys.argv[1:])
    pulsed = pulse_cases()
    for name, w in {**cases(), **dipole_cases(), **pulsed}.items():
        if only and name not in only:
            continue
        s0 = W.initial_state(w, 0)
        ref = O.ReferenceSim(w)
        out = {"s0": s0, "fields": ref.fields(s0), "energies": ref.energies(s0), "term_fields": ref.term_fields(s0)}
        s = s0
        done = 0
        for k in (1, 10, 100):
            s = ref.run(s, k - done)
            done = k
            out["s%d" % k] = s
        if name in pulsed:
            out["fields100"] = ref.fields(s)
            out["energies100"] = ref.energies(s)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, {k: v.shape for k, v in out.items()})
    for name, (w, integ, keep) in long_cases().items():
        if only and name not in only:
            continue
        s0 = W.initial_state(w, 0)
        ref = O.ReferenceSim(w)
        out = {"s0": s0} if s0.size <= 3 * 4096 else {"s0_sha256": hashlib.sha256(s0.tobytes()).hexdigest()}
        s, done = s0, 0
        for k in keep:
            s = ref.rk4_run(s, k - done) if integ == "rk4" else ref.run(s, k - done)
            done = k
            out["s%d" % k] = s
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, {k: getattr(v, "shape", v) for k, v in out.items()})
    todo = [n for n in thermal_cases() if not only or n in only]
    if todo:
        import multiprocessing as mp

        jobs = [(n, THERMAL_SEED + k) for n in todo for k in range(THERMAL_REF_SEEDS)]
        with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
            runs = pool.starmap(thermal_run, jobs)
        for name in todo:
            w, burn, every, nsamp = thermal_cases()[name]
            mine = [r for (n, _), r in zip(jobs, runs) if n == name]
            per_run = {q: [r[q + "_mean"] for r in mine] for q in ("abs_m", "e_total", "e_term0", "e_term1")}
            summ = over_runs(per_run)
            out = {"temperature": w.replicas[0].temperature, "L": np.array(w.replicas[0].L), "burn_in": burn,
                   "every": every, "samples": nsamp, "seeds": np.array([sd for (n, sd) in jobs if n == name]),
                   **{q + "_runs": np.array(v) for q, v in per_run.items()},
                   "run_nse_abs_m": np.array([r["abs_m_nse"] for r in mine]), **summ}
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
            print(name, {k: float(v) for k, v in summ.items()})


def thermal_run(name, seed):
    """One seeded thermal run of the reference (a process of its own: the
    harness holds one solver per process)."""
    w, burn, every, nsamp = thermal_cases()[name]
    ref = O.ReferenceSim(w, seed=seed)
    s = ref.run(W.initial_state(w, 0), burn)
    mus = np.tile(w.model.mus, w.spins_per_replica[0] // w.model.nb)
    abs_m, energies = [], []
    for _ in range(nsamp):
        s = ref.run(s, every)
        m = (mus[:, None] * s).sum(axis=0) / mus.sum()
        abs_m.append(float(np.linalg.norm(m)))
        energies.append(ref.energies(s))
    return thermal_summary(abs_m, energies, len(s))

if __name__ == "__main__":
    main()
