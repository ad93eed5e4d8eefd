#!/usr/bin/env python3
"""LLG spin-steps/s on one GB300: the FP32C and FP64 forms and the fraction
of HBM bandwidth the dominant stage kernel reaches.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
                    [--precision fp32c|fp64] [--impl ours|reference]

A step is one stochastic-LLG time step (Heun: predictor + corrector, RK4:
four stages) over every spin of the workload.  Default workload: bcc,
2-site conventional basis, 256^3 cells (33,554,432 spins, 403 MB per FP32
state vector: larger than L2), nearest-neighbour exchange J = 1 meV,
uniaxial K1 = 0.1 meV, B = 1 T, T = 500 K thermal field, Heun dt = 0.5 fs,
FP32 spins with compensated neighbour sums (the FP32C form).  The same line
carries, each as an object of its own:
  fp64         the FP64 form on the same workload (K capped at 100 steps) and
               the FP32C / FP64 ratio;
  three_shell  the three-shell + cubic reading of the same 256^3 lattice;
  config2      bcc 64^3 x 2, three shells + cubic, 300 K (L2-resident);
  accuracy     max |dS|, d|M|, dE of FP32C against FP64 after 1000 T = 0
               steps at the workload's own size.

Timing: W untimed steps, then K timed steps (K defaults to the workload's
own run length: 2000 steps for the default), each bracketed by CUDA events
on the solver's stream with an L2 flush (a 256 MiB write) between steps, a
barrier + synchronize on both sides, max over ranks.  value = spins x K /
sum of step times.  e2e: the same steps through the C ABI with the FP64
spin state copied from pinned host memory before and back after every step.
roofline: the dominant stage kernel's algorithmic bytes per launch / its
mean CUDA-event duration, against the measured HBM copy bandwidth.
cpu_baseline / --impl reference: the oracle's restatement of the
reference's CPU Heun path (CSR SpMV, per-term field arrays, serial noise
draw as the reference does) on all host cores, a bounded number of steps
of the full lattice.

Several GPUs (torchrun, one process per GPU), no collective on the data
path.  A replica list (temperature or field sweep) is split over the ranks,
balanced by spin count; a single-replica workload runs as an independent
copy per rank (seed offset by the rank).  value = all ranks' spin-steps /
the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from jams_gb300 import workloads as W  # noqa: E402

# algorithmic bytes per spin per stage launch (state vectors that must cross
# HBM between grid-wide dependency points; stencil and noise cost 0 bytes)
STAGE_BYTES = {
    ("heun", "fp32c"): [24, 36],    # predictor: r s0, w sp; corrector: r s0, r sp, w s1
    ("heun", "fp64"): [72, 96],     # + ds written / read (the FP64 form stores it)
    ("rk4", "fp32c"): [36, 60, 60, 48],
    ("rk4", "fp64"): [72, 120, 120, 96],
}
# the metric: spin-steps/s of the FP32C and FP64 forms and the HBM
# fraction, on one GPU
METRIC = "LLG spin-steps/s on 1 GB300: FP32 vs FP64 form at \u22641e-5 max|\u0394S|; % of HBM peak"
# the default line also carries these workloads, each as an object of its own
SECONDARY = {"bcc256_nn": {"three_shell": "bcc256_3shell", "config2": "bcc64_3shell",
                           "with_dipole": "bcc256_3shell_dipole"}}
DEFAULT_WORKLOAD = "bcc256_nn"

# the fused Heun step (one kernel per step, FP32C): read s0, write s1
FUSED_STEP_BYTES = 24
STAGE_NAMES = {"heun": ["heun_predict", "heun_correct"], "rk4": ["rk4_stage1", "rk4_stage2", "rk4_stage3",
                                                                 "rk4_stage4"]}

WORKLOADS = {
    # bcc 64^3 x 2, J1..J3, cubic K, 300 K, Heun dt 0.5 fs (the benchmark's headline configuration)
    "bcc64_3shell": lambda: W.bcc_three_shell(L=64, T=300.0, start="+z"),
    # the same Hamiltonian at 128^3 x 2 (4.2 M spins): state larger than L2, for profiling
    "bcc128_3shell": lambda: W.bcc_three_shell(L=128, T=300.0, start="+z"),
    "bcc128_nn": lambda: W.bcc_nearest_neighbour(L=128, T=500.0),
    # simple-cubic 32^3, T = 0, Heun dt 1 fs (the reference's CPU-runnable case)
    "sc32": lambda: W.sc_ferromagnet(L=32, T=0.0),
    # bcc 256^3 x 2 (33.5 M spins), 500 K, both readings of its Hamiltonian
    "bcc256_nn": lambda: W.bcc_nearest_neighbour(L=256, T=500.0),
    "bcc256_3shell": lambda: W.bcc_three_shell(L=256, T=500.0),
    # 256 simple-cubic replicas, L in {16..64}, T in 0..1200 K
    "sc_sweep256": lambda: W.sc_temperature_sweep(),
    # triangular 2048^2 x 16 fields, tensor exchange + DMI, RK4, 5 K
    "tri2048_dmi_x16": lambda: W.triangular_dmi_field_sweep(),
    # fcc (4-site conventional cell), 12 + 6 neighbours, 300 K: 128^3 x 4 = 8.4 M spins
    "fcc128_2shell": lambda: W.fcc_ferromagnet(L=128, T=300.0, J2=0.2),
    # the headline and the 256^3 3-shell workloads with the dipole-dipole term
    # (FFT convolution, r_c = 8 lattice parameters)
    "bcc64_3shell_dipole": lambda: W.bcc_three_shell(L=64, T=300.0, start="+z", dipole_cutoff=8.0),
    "bcc256_3shell_dipole": lambda: W.bcc_three_shell(L=256, T=500.0, steps=2000, dipole_cutoff=8.0),
    # profiling case of the 256-point transform passes: FFT grid larger than
    # L2 (204 MB per half spectrum), about 1.5 GB on the device
    "bcc256x256x128_3shell_dipole": lambda: W.bcc_three_shell(L=(256, 256, 128), T=500.0, steps=2000,
                                                               dipole_cutoff=8.0),
    # profiling cases: state larger than L2 (129 MB) but a few GB on the device
    "bcc192_nn": lambda: W.bcc_nearest_neighbour(L=192, T=500.0),
    "bcc192_3shell": lambda: W.bcc_three_shell(L=192, T=500.0),
    "tri2048_dmi_x4": lambda: W.triangular_dmi_field_sweep(n_fields=4),
    # the headline Hamiltonian with its exchange given as two terms, one with
    # a small symmetric off-diagonal part: no stencil family applies, the
    # generic gather kernels run (the path of lattices and tensors outside
    # the compiled families)
    "bcc64_3shell_generic": lambda: split_exchange(W.bcc_three_shell(L=64, T=300.0, start="+z")),
    "bcc128_3shell_generic": lambda: split_exchange(W.bcc_three_shell(L=128, T=300.0, start="+z")),
}


def split_exchange(w):
    """The same model with the exchange as two terms, the second with a
    small symmetric off-diagonal part (J_xy = J_yx = 0.05 J_xx) on one pair
    and its reverse: no lattice family takes it, so the FP32C form runs the
    gather kernels."""
    return W.split_exchange(w, offdiag=0.05)


def kernel_name(info: dict, integ: str, stage: int, precision: str, dipole: bool = False) -> str:
    """Name of the kernel that runs stage `stage` of a step, as ncu prints it."""
    if info.get("family", "generic") != "generic" and precision == "fp32c":
        fam = {"sc": "FamSC", "bcc": "FamBCC", "bcc3": "FamBCC3", "triangular": "FamTRI", "fcc": "FamFCC",
               "fcc2": "FamFCC2"}[info["family"]]
        if info.get("fused"):
            nt = 32 * info["tile_y"] * {"fcc": 4, "fcc2": 4, "bcc": 2, "bcc3": 2}.get(info["family"], 1)
            minb = max(1, (256 * (4 if info["occupancy"] >= 4 else 2)) // nt)
            return "fused_heun<%s, %d, %d>" % (fam, info["tile_y"], minb)
        if integ == "heun":
            st = 0 if stage == 0 else (2 if info["store_rhs"] else 1)
            if info.get("stored_noise"):
                st = {0: 7, 2: 8}[st]   # stages 0 and 2 that store / load the thermal field
        else:
            st = 3 + stage
        rpt = info.get("rows_per_thread", 1) or 1
        nt = info["tile_z"] * (info["tile_y"] // rpt) * {"fcc": 4, "fcc2": 4, "bcc": 2, "bcc3": 2}.get(
            info["family"], 1)
        minb = info["occupancy"] * max(1, 256 // nt)
        tma = 1 if info.get("tma") and st != 1 else 0
        return "tiled_stage<%s, %d, %d, %d, %d, %d, %d, %d>" % (fam, info["tile_z"], info["tile_y"], rpt, st, minb,
                                                              1 if dipole else 0, tma)
    suffix = "_f32" if precision == "fp32c" else "_f64"
    if integ == "heun":
        return ("heun_predict" if stage == 0 else "heun_correct") + suffix
    return "rk4_stage%s<%d>" % (suffix, stage + 1)


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None,
                   help="timed steps (default: the workload's own run length, e.g. 20000 for bcc64_3shell)")
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    p.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"])
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-accuracy", action="store_true", help="skip the FP32C-vs-FP64 accuracy check")
    p.add_argument("--accuracy-cap", type=int, default=0,
                   help="cells per axis of the accuracy check's lattice (0: the workload's own size)")
    p.add_argument("--no-extra", action="store_true",
                   help="skip the FP64-form, three-shell and bcc 64^3 objects of the default line")
    p.add_argument("--ref-gpu", default="auto", choices=["auto", "on", "off"],
                   help="time the restated reference GPU path (baseline/refgpu.cu) on replica 0: auto = single-replica "
                        "Heun workloads whose int32 CSR fits (up to 40 M spins)")
    p.add_argument("--profile-steps", type=int, default=50)
    p.add_argument("--no-tune", action="store_true")
    p.add_argument("--tuning", default="", help="planes_per_cta,flags,occupancy instead of autotuning (flags: 1 stored rhs, 2 narrow tile, "
                        "4 two rows per thread, 8 the fused Heun step, 256 TMA plane loads, 512 stored noise, "
                        "1024 the half-width simple-cubic tile)")
    return p.parse_args(argv)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, world: int, device=None) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def init_ranks(world: int, local: int, backend: str = "nccl"):
    """One process per GPU (replicas only: no collective on the data path;
    the process group carries the barrier, the max of the timings and the
    end-of-run scalars)."""
    if world <= 1:
        return
    import torch
    import torch.distributed as dist

    if backend == "nccl":
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        dist.init_process_group(backend)


def rank_workload(name: str, rank: int, world: int = 1):
    """The workload of one rank.  A replica list (temperature or field sweep)
    is split over the ranks: rank r takes a disjoint subset, balanced by spin
    count (split_replicas), with the original replicas' starts and its own
    noise key.  A single-replica workload is not split: every
    rank integrates its own independent copy (seed offset by the rank), i.e.
    weak scaling."""
    w = WORKLOADS[name]()
    if world > 1 and len(w.replicas) > 1:
        parts = split_replicas([int(np.prod(r.L)) * w.model.nb for r in w.replicas], world)
        w.replicas = [w.replicas[i] for i in parts[rank]]
        w.replica_ids = parts[rank]          # starts of the original replicas
        w.noise_seed = w.seed * 1000003 + rank + 1   # noise streams distinct across ranks
    else:
        w.seed = w.seed + rank
    return w


def split_replicas(spins, world: int):
    """Disjoint subsets of replica indices, one per rank, that together cover
    every replica and balance the spins: largest replica first, each to the
    rank with the fewest spins so far (ties to the lower rank).  Each
    subset is returned in ascending replica order.  With at least as many
    replicas as ranks no rank is empty, and the largest rank total exceeds
    the smallest by at most one replica's spins."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(spins)), key=lambda i: (-spins[i], i))
    load = [0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += spins[i]
    return [sorted(p) for p in parts]


def job_rate(spins_all_ranks: int, steps: int, seconds: float) -> float:
    """Whole-job spin-steps/s: the spins of every rank over the slowest rank's time."""
    return spins_all_ranks * steps / seconds


def sum_over_ranks(x: float, world: int, device=None) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_scalars(values, world: int, device=None):
    """Per-rank scalar lists (e.g. |M| of every replica) gathered on every
    rank, in rank order."""
    if world <= 1:
        return [list(values)]
    import torch
    import torch.distributed as dist

    out = [None] * world
    dist.all_gather_object(out, [float(v) for v in values])   # ranks may hold different replica counts
    return out


# ------------------------------------------------------------------ clocks --

class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- CPU port --

def cpu_port_rate(w: W.Workload, seconds: float = 15.0, max_steps: int = 200, warm: int = 1):
    """Spin-steps/s of the oracle (the reference's CPU Heun/RK4 path restated
    in C, OpenMP over all host cores, serial noise draw as the reference)
    on replica 0 of the workload (replicas are independent)."""
    from oracle import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    sim = O.OracleSim(w, 0, serial_noise=True, threads=threads)
    s = W.initial_state(w, 0)
    s = sim.run(s, warm, first_step=0)
    t0 = time.perf_counter()
    s = sim.run(s, 1, first_step=warm)
    one = time.perf_counter() - t0
    n = int(max(1, min(max_steps, seconds / max(one, 1e-9))))
    t0 = time.perf_counter()
    sim.run(s, n, first_step=warm + 1)
    dt = time.perf_counter() - t0
    return sim.n * n / dt, threads, n, sim.n


def run_reference(args, rank, world):
    """--impl reference: the CPU path of the reference (restated in the
    oracle) on the host cores, K timed steps after W warm-up steps."""
    if rank != 0:
        return 0
    from oracle import oracle as O

    w = WORKLOADS[args.workload]()
    if args.steps is None:
        args.steps = w.steps
    O.build()
    threads = os.cpu_count() or 1
    sim = O.OracleSim(w, 0, serial_noise=True, threads=threads)
    s = W.initial_state(w, 0)
    s = sim.run(s, args.warmup, first_step=0)
    # bound the run to a few minutes: time one step, cap K accordingly
    t0 = time.perf_counter()
    s = sim.run(s, 1, first_step=args.warmup)
    one = time.perf_counter() - t0
    k = max(1, min(args.steps, int(120.0 / max(one, 1e-9))))
    t0 = time.perf_counter()
    sim.run(s, k, first_step=args.warmup + 1)
    dt = time.perf_counter() - t0
    value = sim.n * k / dt

    line = {
        "metric": METRIC, "value": value, "unit": "spin-steps/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": k, "warmup": args.warmup, "ms_per_step": 1e3 * dt / k,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded spins, the configuration's Hamiltonian)",
        "config": workload_config(args.workload, w, sum(w.spins_per_replica)),
        "cpu_baseline": {"value": value, "unit": "spin-steps/s", "cores": threads, "kind": "port",
                         "sample": "%d %s steps of replica 0 (%d spins, the full lattice) after %d warm-up steps, "
                                   "OpenMP on all host cores, noise drawn serially as the reference draws it"
                                   % (k, "RK4" if w.model.integrator == W.RK4 else "Heun", sim.n, args.warmup)},
        "e2e": {"value": value, "unit": "spin-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# -------------------------------------------------------------------- GPU --

def tiled_stem(name: str):
    """(family, tile z, tile y, stage) of a tiled_stage kernel name: template
    arguments <F, TZ, TY, RPT, STAGE, MINB, DIP[, TMA]>, or <F, TZ, TY, STAGE,
    MINB[, DIP]> in captures of the kernels before rows per thread existed."""
    if not name.startswith("tiled_stage<"):
        return None
    args = [a.strip() for a in name[name.index("<") + 1:name.rindex(">")].split(",")]
    return tuple(args[:3] + [args[4] if len(args) >= 7 else args[3]])


def accuracy_vs_fp64(w, steps=1000, cap=0):
    """max |dS|, d|M| and dE of the FP32C form against the FP64 form (which
    equals the oracle, and through it the reference's CPU solver, bit for
    bit) after `steps` T = 0 steps.  The workload's Hamiltonian and integrator
    on replica 0 (at most `cap` cells per axis when cap > 0, else its own
    size) with a random start."""
    import copy

    from jams_gb300 import llg

    w2 = copy.deepcopy(w)
    r0 = w2.replicas[0]
    if cap > 0:
        r0.L = tuple(min(int(l), cap) for l in r0.L)
    r0.temperature = 0.0
    w2.replicas = [r0]
    w2.start = "random"
    s0 = W.initial_state(w2, 0)
    out = {}
    for name, prec in (("fp64", llg.FP64), ("fp32c", llg.FP32C)):
        sol = llg.Solver(w2, precision=prec)
        sol.set_state(s0)
        sol.step(steps)
        m4, e = sol.observables(0)
        out[name] = (sol.get_state(0), m4[3], e)
        sol.close()
    (a, ma, ea), (b, mb, eb) = out["fp64"], out["fp32c"]
    return {"max_dS": float(np.abs(a - b).max()), "d_abs_M": float(abs(ma - mb)),
            "max_dE_rel": float(np.max(np.abs(ea - eb) / np.maximum(np.abs(ea), 1e-30))),
            "steps": steps, "T": 0.0, "spins": int(len(s0)),
            "sample": "replica 0 of the workload's model at %s cells, random start, FP32C vs FP64 (the FP64 form "
                      "equals the oracle %s)" % ("x".join(str(l) for l in r0.L),
                                                 "within FFT rounding" if any(t.kind == W.TERM_DIPOLE
                                                                              for t in w.model.terms)
                                                 else "bit for bit")}


def reference_gpu_rate(args, w):
    """The reference's GPU Heun path restated (baseline/refgpu.cu: cuSPARSE
    CSR SpMV, cuRAND, cuBLAS and its two update kernels, FP64) on replica 0 of
    the workload, on this GPU: spin-steps/s over about one second of steps."""
    supported = {W.TERM_EXCHANGE, W.TERM_UNIAXIAL, W.TERM_CUBIC, W.TERM_APPLIED_FIELD}
    n = int(np.prod(w.replicas[0].L)) * w.model.nb
    why = None
    if args.ref_gpu == "off":
        return None
    if w.model.integrator != W.HEUN:
        why = "the reference GPU path restated here is Heun"
    elif any(t.kind not in supported or t.pulse != W.PULSE_STATIC for t in w.model.terms):
        why = "terms outside the restatement (exchange, uniaxial, cubic, static field)"
    elif args.ref_gpu == "auto" and (len(w.replicas) > 1 or n > 40_000_000):
        why = "skipped by default above 40 M spins or for several replicas (--ref-gpu on)"
    elif sum(3 * len(t.bi) for t in w.model.terms if t.kind == W.TERM_EXCHANGE) * n // w.model.nb >= 2 ** 31:
        why = "the reference's CSR needs more than 2^31 stored values (int32 indices)"
    if why:
        return {"unavailable": why}
    try:
        from baseline import refgpu as R

        R.build()
        ref = R.RefGpu(w)
    except Exception as e:  # noqa: BLE001
        return {"unavailable": "ref-GPU baseline: %s" % str(e)[-200:]}
    ref.set_state(W.initial_state(w, 0))
    ref.run(5)
    probe = ref.run(10)
    k = int(min(2000, max(20, 1000.0 / max(probe / 10, 1e-3))))
    ms = ref.run(k)
    ref.close()
    return {"value": n * k / (ms * 1e-3), "unit": "spin-steps/s", "kind": "port", "precision": "fp64",
            "ms_per_step": ms / k, "steps": k, "spins": n,
            "sample": "replica 0, %d steps after 15 warm-up steps, CUDA events on the baseline's stream" % k,
            "path": "CUDAHeunLLGSolver::run restated: cuSPARSE CSR SpMV (ALG1), cuRAND normals, blocking field "
                    "copy + cuBLAS daxpy, 84x3-thread update kernels"}


def traffic_from_profiles(workload: str, kernel: str, precision: str):
    """DRAM bytes (read + write) of one launch of `kernel` on `workload`, from
    the committed ncu summary profiles/dram_traffic.json, or None."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.exists(path):
        return None
    try:
        d = json.load(open(path)).get(workload, {}).get(precision, {})
        e = d.get(kernel)
        if e is None and kernel.startswith("tiled_stage<"):
            # the same family, tile and stage compiled for another occupancy
            # or rows per thread moves the same bytes
            e = next((v for k, v in d.items() if k.startswith("tiled_stage<") and tiled_stem(k) == tiled_stem(kernel)),
                     None)
        return None if e is None else float(e["dram_bytes_per_launch"])
    except (ValueError, OSError, KeyError, TypeError):
        return None


def workload_config(name: str, w, n_spins: int) -> dict:
    """The `config` object of a bench line: the same keys and values in both
    arms (this library and --impl reference)."""
    vec_mb = n_spins * 12 / 1e6
    l2 = ("state larger than the 129 MB L2 (%.0f MB per FP32 state vector); the GPU arm also flushes L2 between "
          "timed steps (256 MiB write)" % vec_mb) if vec_mb > 129 else \
        ("state smaller than L2 (%.1f MB per FP32 state vector): the GPU arm flushes L2 between timed steps "
         "(256 MiB write)" % vec_mb)
    return {"workload": name, "description": w.description, "spins": int(n_spins), "replicas": len(w.replicas),
            "l2": l2}


def load_peak():
    """HBM copy bandwidth (GB/s) and where it came from."""
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        if peaks.get("hbm_gbs"):
            return float(peaks["hbm_gbs"]), "measured"
    except (OSError, ValueError):
        pass
    return 6800.0, "fallback"


def make_solver(llg, w, prec, local, stream, tuning_arg: str = "", tune: bool = True):
    sol = llg.Solver(w, precision=prec, device=local)
    sol.set_stream(stream.cuda_stream)
    for r in range(len(w.replicas)):
        sol.set_state(W.initial_state(w, r), r)
    if tuning_arg:
        tx, fl, oc = (int(v) for v in tuning_arg.split(","))
        sol.set_tuning(tx, bool(fl & 1), oc, bool(fl & 2), bool(fl & 4), bool(fl & 8), bool(fl & 256),
                       bool(fl & 512), bool(fl & 1024))
        tuning = sol.kernel_info()
    else:
        # the choice is cached per lattice shape ($JAMS_LLG_TUNE_CACHE), so a
        # second run of the same command launches no trial kernels
        tuning = sol.autotune(trial_steps=10, use_cache=True) if tune else sol.kernel_info()
    return sol, tuning


def timed_steps(torch, sol, steps: int, warmup: int, flush, stream, world: int, local: int, clocks=None):
    """W untimed steps, then K single steps each bracketed by CUDA events on
    the solver's stream, L2 flushed before each; barrier + synchronize on
    both sides; max over ranks.  Returns (total ms, launches, wall s)."""
    for _ in range(warmup):
        sol.step(1)
    torch.cuda.synchronize()
    if clocks is not None:
        clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    launches = 0
    t_wall = time.perf_counter()
    for k in range(steps):
        flush.fill_(float(k))
        evs[k][0].record(stream)
        sol.step(1)
        evs[k][1].record(stream)
        launches += sol.last_launch_count
    torch.cuda.synchronize()
    barrier(world)
    t_wall = time.perf_counter() - t_wall
    total_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs), world, torch.device("cuda", local))
    sol.synchronize()
    return total_ms, launches, t_wall


def stage_roofline(sol, w, name: str, precision: str, tuning: dict, flush, profile_steps: int, ms_per_step: float,
                   n_spins: int):
    """Per-stage kernel durations (CUDA events on the solver's stream, L2
    flushed before each step) and the roofline of the dominant stage kernel:
    its algorithmic bytes per launch / its mean duration, against the HBM
    copy bandwidth.  Returns (roofline, per-stage dipole ms)."""
    integ = "heun" if w.model.integrator == W.HEUN else "rk4"
    ns = len(STAGE_BYTES[(integ, precision)])
    stage_ms = np.zeros(ns)
    dip_ms = np.zeros(ns)
    for _ in range(profile_steps):
        flush.fill_(1.0)
        k_ms, d_ms = sol.profile_stages(1, dipole=True)
        stage_ms += k_ms
        dip_ms += d_ms
    stage_ms /= profile_steps
    dip_ms /= profile_steps
    dom = int(np.argmax(stage_ms))
    fused = bool(tuning.get("fused")) and precision == "fp32c"
    # the fused Heun step is one launch: it reads s0 and writes s1 (24 B per
    # spin); the two-pass form's 60 B per spin-step is kept for comparison
    step_bytes = FUSED_STEP_BYTES if fused else sum(STAGE_BYTES[(integ, precision)])
    bytes_per_launch = (FUSED_STEP_BYTES if fused else STAGE_BYTES[(integ, precision)][dom]) * n_spins
    achieved = bytes_per_launch / (stage_ms[dom] * 1e-3) / 1e9
    peak, peak_src = load_peak()
    has_dipole = any(t.kind == W.TERM_DIPOLE for t in w.model.terms)
    kname = kernel_name(tuning, integ, dom, precision, has_dipole)
    traffic = traffic_from_profiles(name, kname, precision)
    two_pass = sum(STAGE_BYTES[(integ, precision)])
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": kname, "stage": "heun_step (fused)" if fused else STAGE_NAMES[integ][dom],
                "peak_source": peak_src, "algorithmic_bytes_per_launch": int(bytes_per_launch),
                "stage_ms": [float(x) for x in stage_ms],
                "algorithmic_bytes_per_spin_step": int(step_bytes),
                "step_frac": (step_bytes * n_spins / (ms_per_step * 1e-3) / 1e9) / peak,
                "two_pass_bytes_per_spin_step": int(two_pass),
                "two_pass_equivalent_frac": (two_pass * n_spins / (ms_per_step * 1e-3) / 1e9) / peak}
    return roofline, dip_ms


def dipole_fft_bytes(w) -> int:
    """Algorithmic bytes of one FP32C dipole field evaluation, summed over
    replicas: the forward real pass reads the 3 nb spin fields (4 B per
    cell) and writes their half spectra (8 B per point); each complex pass
    reads and writes the half spectra; the k-space product reads them and
    the stored tensors (nb x 6 real + nb (nb - 1) / 2 x 6 complex per point)
    and writes the field spectra; the inverse passes mirror the forward
    ones, the inverse real pass writing the 3 nb field planes."""
    nb, per = w.model.nb, w.model.periodic
    total = 0
    for r in w.replicas:
        L = list(r.L)
        M = [L[k] if per[k] or L[k] == 1 else 2 * L[k] for k in range(3)]
        h = max([k for k in range(3) if M[k] > 1], default=0)
        cells = int(np.prod(L))
        mq = int(np.prod(M)) // M[h] * (M[h] // 2 + 1)
        f = 3 * nb
        passes = sum(1 for k in range(h) if M[k] > 1)
        spec = f * mq * 8
        real = f * cells * 4 + spec
        tensor = nb * 6 * mq * 4 + nb * (nb - 1) // 2 * 6 * mq * 8
        total += 2 * real + 2 * passes * 2 * spec + (2 * spec + tensor)
    return total


def dipole_object(w, dip_ms, stage_ms):
    """The dipole term's share of a step: per-evaluation time, and the
    transforms' algorithmic bytes over it against the measured copy peak."""
    if not any(t.kind == W.TERM_DIPOLE for t in w.model.terms):
        return None
    peak, _ = load_peak()
    ms = float(np.mean(dip_ms))
    nbytes = dipole_fft_bytes(w)
    return {"ms_per_evaluation": ms, "evaluations_per_step": int(len(dip_ms)),
            "share_of_stage_time": float(np.sum(dip_ms) / (np.sum(dip_ms) + np.sum(stage_ms))),
            "r_cutoff": next(t.r_cutoff for t in w.model.terms if t.kind == W.TERM_DIPOLE),
            "transform": "this library's register / Stockham FFT passes, scatter and gather fused",
            "bytes_per_evaluation": nbytes, "achieved_gbs": nbytes / (ms * 1e-3) / 1e9,
            "frac": nbytes / (ms * 1e-3) / 1e9 / peak if peak else None}


def secondary_form(torch, llg, args, name: str, precision: str, local: int, stream, flush, steps: int,
                   warmup: int):
    """One more workload or precision in the same line: value, ms per step,
    roofline of its dominant kernel, clocks and the kernels it ran."""
    w = WORKLOADS[name]()
    prec = llg.FP32C if precision == "fp32c" else llg.FP64
    sol, tuning = make_solver(llg, w, prec, local, stream, tune=not args.no_tune)
    n_spins = sol.num_spins(-1)
    clocks = ClockSampler(local)
    total_ms, launches, _ = timed_steps(torch, sol, steps, warmup, flush, stream, 1, local, clocks)
    clk = clocks.stop()
    ms = total_ms / steps
    roof, dip_ms = stage_roofline(sol, w, name, precision, tuning, flush, max(5, args.profile_steps // 5), ms,
                                  n_spins)
    sol.close()
    out = {"workload": name, "description": w.description, "spins": int(n_spins), "precision": precision,
           "value": n_spins * steps / (total_ms * 1e-3), "unit": "spin-steps/s", "steps": steps, "warmup": warmup,
           "ms_per_step": ms, "gpu_launches": launches, "roofline": roof, "clocks": clk, "kernels": tuning}
    dip = dipole_object(w, dip_ms, roof["stage_ms"]) if precision == "fp32c" else None
    if dip:
        out["dipole"] = dip
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch

    init_ranks(world, local)
    torch.cuda.set_device(local)
    from jams_gb300 import build as B
    from jams_gb300 import llg

    B.build()
    w = rank_workload(args.workload, rank, world)
    if args.steps is None:
        args.steps = w.steps
    prec = llg.FP32C if args.precision == "fp32c" else llg.FP64
    integ = "heun" if w.model.integrator == W.HEUN else "rk4"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)  # torch work (L2 flush, events) and the solver share one stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    sol, tuning = make_solver(llg, w, prec, local, stream, args.tuning, not args.no_tune)
    n_spins = sol.num_spins(-1)
    spins_all = int(sum_over_ranks(float(n_spins), world, torch.device("cuda", local)))

    # ---- timed region: K steps, L2 flushed between steps
    clocks = ClockSampler(local)
    total_ms, launches, t_wall = timed_steps(torch, sol, args.steps, args.warmup, flush, stream, world, local, clocks)
    clk = clocks.stop()
    ms_per_step = total_ms / args.steps
    value = job_rate(spins_all, args.steps, total_ms * 1e-3)

    # ---- per-stage kernel durations and the roofline of the dominant one
    roofline, dip_ms = stage_roofline(sol, w, args.workload, args.precision, tuning, flush, args.profile_steps,
                                      ms_per_step, n_spins)
    ns = len(STAGE_BYTES[(integ, args.precision)])

    # ---- dipole term: FFT convolution before every stage (this library's
    # transform passes with the scatter and gather fused in, and its k-space
    # product)
    dipole = dipole_object(w, dip_ms, roofline["stage_ms"]) if args.precision == "fp32c" else None

    # ---- steady state without flush: blocks of 100 steps as CUDA graphs
    blk = 100
    sol.step(blk)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nblk = max(1, min(10, args.steps // blk))
    e0.record(stream)
    for _ in range(nblk):
        sol.step(blk)
    e1.record(stream)
    torch.cuda.synchronize()
    graph_ms = e0.elapsed_time(e1) / (nblk * blk)
    steady = {"value": n_spins / (graph_ms * 1e-3), "ms_per_step": graph_ms,
              "note": "100-step CUDA-graph blocks, no L2 flush (the state stays L2-resident when it fits)"}

    # ---- e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(torch, sol, n_spins, spins_all, args.steps, world, local, ms_per_step)

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, cores, n_steps, n_rep = cpu_port_rate(w)
        cpu = {"value": rate, "unit": "spin-steps/s", "cores": cores, "kind": "port",
               "sample": "%d Heun/RK4 steps of replica 0 (%d spins, the full lattice), oracle restatement of the "
                         "reference CPU path, OpenMP on all host cores" % (n_steps, n_rep)}

    ref_gpu = None
    accuracy = None
    if rank == 0 and world == 1:
        ref_gpu = reference_gpu_rate(args, w)
        if args.precision == "fp32c" and not args.no_accuracy:
            accuracy = accuracy_vs_fp64(w, cap=args.accuracy_cap)

    # |M| of every replica of every rank at the end of the run
    mags = [float(sol.observables(r)[0][3]) for r in range(len(w.replicas))]
    mags = gather_scalars(mags, world, torch.device("cuda", local))
    sol.close()

    # ---- the rest of the metric, in the same line (rank 0, N = 1): the FP64
    # form on this workload, the three-shell reading of the 256^3 lattice and
    # the L2-resident bcc 64^3 headline configuration
    forms = {}
    if rank == 0 and world == 1 and not args.no_extra:
        ks = min(args.steps, 100)
        if args.precision == "fp32c":
            f64 = secondary_form(torch, llg, args, args.workload, "fp64", local, stream, flush, ks,
                                 min(args.warmup, 5))
            f64["fp32c_over_fp64"] = (n_spins * args.steps / (total_ms * 1e-3)) / f64["value"]
            forms["fp64"] = f64
        for key, name in SECONDARY.get(args.workload, {}).items():
            forms[key] = secondary_form(torch, llg, args, name, "fp32c", local, stream, flush, args.steps,
                                        args.warmup)

    line = {
        "metric": METRIC, "value": value, "unit": "spin-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "strong" if (world > 1 and len(WORKLOADS[args.workload]().replicas) > 1) else "weak",
        "vs_baseline": None, "dtype": "f32" if args.precision == "fp32c" else "f64",
        "data": "synthetic (seeded spins, the configuration's Hamiltonian)",
        "config": workload_config(args.workload, WORKLOADS[args.workload](), spins_all),
        "solver": {"precision": args.precision, "integrator": integ, "kernels": tuning,
                   "parallelism": ("replica list split over %d ranks" % world) if world > 1 else "single GPU"},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
        "steady_state_graph": steady, "wall_s_timed_region": t_wall,
        "final_abs_m": {"mean": float(np.mean([m for r in mags for m in r])), "ranks": len(mags)},
        "dipole": dipole, "reference_gpu": ref_gpu, "accuracy": accuracy,
    }
    line.update(forms)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def measure_e2e(torch, sol, n_spins: int, spins_all: int, steps: int, world: int, local: int, ms_per_step: float):
    """The same steps through the C ABI with host buffers: every step copies
    the FP64 state from pinned host memory, steps, and copies it back."""
    host = torch.empty((n_spins, 3), dtype=torch.float64, pin_memory=True)
    host_np = host.numpy()
    host_np[:] = sol.get_state(-1)
    ke = max(10, min(200, steps // 10))
    for _ in range(3):
        sol.set_state(host_np, -1)
        sol.step(1)
        sol.get_state(-1, out=host_np)
    torch.cuda.synchronize()
    barrier(world)
    t_set = t_step = t_get = 0.0
    t0 = time.perf_counter()
    for _ in range(ke):
        a = time.perf_counter()
        sol.set_state(host_np, -1)
        b = time.perf_counter()
        sol.step(1)
        sol.synchronize()
        c = time.perf_counter()
        sol.get_state(-1, out=host_np)
        t_set += b - a
        t_step += c - b
        t_get += time.perf_counter() - c
    dt = time.perf_counter() - t0
    dt = max_over_ranks(dt, world, torch.device("cuda", local))
    # the host link: pinned copies of the state's size, each direction
    dev = torch.empty_like(host, device="cuda")
    link = {}
    for name, dst, src in (("h2d", dev, host), ("d2h", host, dev)):
        dst.copy_(src)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(20):
            dst.copy_(src)
        torch.cuda.synchronize()
        link[name] = n_spins * 24 * 20 / (time.perf_counter() - t1) / 1e9
    # both directions at once (two streams): what each direction keeps when
    # the link is shared; the set / step / get loop cannot use it, since each
    # step's input is the previous step's result
    host2 = torch.empty_like(host, pin_memory=True)
    dev2 = torch.empty_like(dev)
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(20):
        with torch.cuda.stream(s_in):
            dev.copy_(host, non_blocking=True)
        with torch.cuda.stream(s_out):
            host2.copy_(dev2, non_blocking=True)
    torch.cuda.synchronize()
    link["duplex_each_way"] = n_spins * 24 * 20 / (time.perf_counter() - t1) / 1e9
    del host2, dev2
    floor_s = n_spins * 24 * (1.0 / link["h2d"] + 1.0 / link["d2h"]) / 1e9 + ms_per_step * 1e-3
    return {"value": job_rate(spins_all, ke, dt), "unit": "spin-steps/s", "h2d_bytes_per_step": n_spins * 24,
            "d2h_bytes_per_step": n_spins * 24, "steps": ke,
            "us_per_step": {"set_state": 1e6 * t_set / ke, "step": 1e6 * t_step / ke, "get_state": 1e6 * t_get / ke},
            "host_link_gbs": link, "link_floor_value": job_rate(spins_all, 1, floor_s)}


if __name__ == "__main__":
    sys.exit(main())
