"""Generates the golden vectors in tests/golden/ from the REFERENCE itself.

Runs the reference's own CPU Heun solver (HeunLLGSolver::run,
src/jams/solvers/cpu_llg_heun.cc:45-148), its Solver::compute_fields and its
Hamiltonian terms, compiled from the reference sources by
oracle/Makefile.ref into oracle/_ref/libjams_ref.so.  This only works where the
reference sources are present (the development container):

    make -f oracle/Makefile.ref REF=/root/reference
    python tests/golden/make_golden.py

The dipole cases run the reference's dipole-bruteforce Hamiltonian
(src/jams/hamiltonian/dipole_bruteforce.cc) compiled the same way, the pulse
cases its applied-field pulses and zeeman term (applied_field.cc, zeeman.cc);
these also hold the fields and energies after the 100 steps, at the solver
time 100 dt.

Each fixture holds, for a small seeded case at T = 0: the initial spins, the
total field and per-term energies of the reference at those spins, and the
reference's spins after 1, 10 and 100 Heun steps.  The reference's thermal
noise (pcg32 + std::normal_distribution) is not reproducible elsewhere, so
fixtures are T = 0 only.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from jams_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.golden.cases import cases, dipole_cases, pulse_cases  # noqa: E402

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
        out = {"s0": s0, "fields": ref.fields(s0), "energies": ref.energies(s0)}
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


if __name__ == "__main__":
    main()
