"""Times the reference's own CPU Heun solver (HeunLLGSolver::run,
src/jams/solvers/cpu_llg_heun.cc:45-148, built from the reference sources
by oracle/Makefile.ref) against the oracle's restatement of it (the CPU
baseline of bench.py, kind "port") at the same thread count, so that the
port's numbers can stand in for the reference where its sources are absent
(the GPU machine).  Test and measurement infrastructure for the development
container:

    make -f oracle/Makefile.ref && make -f oracle/Makefile.ref OMP=1
    python oracle/time_reference_cpu.py

Pairs timed (spin-steps/s, median of three runs of a fixed step count):
  - the reference's default build (serial; JAMS_BUILD_OMP is off by default)
    against the port on 1 thread;
  - the reference's OpenMP build (oracle/_ref_omp, its sparse_interaction.cc
    serial: it does not compile with HAS_OMP) against the port on 1 thread
    and on all cores.
Workloads: the simple-cubic benchmark lattice (32^3, T = 0) and bcc 32^3 x 2
with the three-shell exchange and cubic anisotropy at 300 K (serial noise
draw in both, as the reference draws it).  Prints one JSON line per pair.
"""
from __future__ import annotations

import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _one(kind: str, name: str, threads: int, steps: int) -> float:
    sys.path.insert(0, ROOT)
    from jams_gb300 import workloads as W
    from oracle import oracle as O

    w = {"sc32": lambda: W.sc_ferromagnet(L=32), "bcc32_3shell": lambda: W.bcc_three_shell(L=32, T=300.0)}[name]()
    s = W.initial_state(w, 0)
    if kind == "port":
        sim = O.OracleSim(w, 0, serial_noise=True, threads=threads)
        s = sim.run(s, 2, first_step=0)
        t = time.perf_counter()
        sim.run(s, steps, first_step=2)
    else:
        lib = O.REF_LIB_PATH if kind == "reference" else O.REF_OMP_LIB_PATH
        sim = O.ReferenceSim(w, seed=1, lib_path=lib)
        s = sim.run(s, 2)
        t = time.perf_counter()
        sim.run(s, steps)
    dt = time.perf_counter() - t
    return sim.n * steps / dt


def measure(kind: str, name: str, threads: int, steps: int) -> float:
    """Median of three runs, each in a fresh process (OMP_NUM_THREADS set)."""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    vals = []
    for _ in range(3):
        out = subprocess.run([sys.executable, __file__, "--one", kind, name, str(threads), str(steps)], env=env,
                             capture_output=True, text=True, check=True)
        # the reference's own progress lines share stdout: take the tagged rate
        vals.append(float(next(l for l in out.stdout.splitlines() if l.startswith("rate "))[5:]))
    return statistics.median(vals)


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--one":
        print("rate %r" % _one(sys.argv[2], sys.argv[3], int(sys.argv[4]), int(sys.argv[5])), flush=True)
        return
    cores = os.cpu_count() or 1
    for name, steps in (("sc32", 200), ("bcc32_3shell", 40)):
        for ref_kind, threads in (("reference", 1), ("reference_omp", 1), ("reference_omp", cores)):
            ref = measure(ref_kind, name, threads, steps)
            port = measure("port", name, threads, steps)
            print(json.dumps({"workload": name, "threads": threads, "reference_build": ref_kind,
                              "reference_spin_steps_s": ref, "port_spin_steps_s": port, "port_over_reference": port / ref,
                              "steps": steps}), flush=True)


if __name__ == "__main__":
    main()
