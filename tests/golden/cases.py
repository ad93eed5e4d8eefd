"""The small seeded workloads behind the golden fixtures.

cases(): the reference's exchange, anisotropy and field terms; the FP64 form
equals these bit for bit.  dipole_cases(): with the dipole-dipole term (the
reference's dipole-bruteforce Hamiltonian); the FFT evaluation equals these
within rounding, not bit for bit.  pulse_cases(): time-dependent applied
fields (sinc and sinc-cos pulses) and zeeman dc / ac fields; their sin and cos
come from the C library, so the fixtures pin the oracle bit for bit where
they were made and the GPU form within 1e-12 elsewhere.  long_cases(): 1000
T = 0 steps, of the simple-cubic benchmark lattice at full size (Heun) and of
a triangular DMI monolayer (RK4, the reference's RK4 kernels built for the
host).  thermal_cases(): the reference's own finite-temperature Heun run,
summarised as means and numerical standard errors of |M| and the energies."""
from jams_gb300 import workloads as W


def _open_sc():
    w = W.sc_ferromagnet(L=(6, 5, 4))
    w.model.periodic = (0, 1, 1)
    return w


def _tri():
    w = W.triangular_dmi_field_sweep(L=8, n_fields=1, T=0.0)
    w.model.integrator = W.HEUN
    w.replicas[0].B = (0.0, 0.0, 0.5)
    return w


def cases():
    return {
        "sc8_nn_uniaxial_field": W.sc_ferromagnet(L=8),
        "bcc4_3shell_cubic": W.bcc_three_shell(L=4, T=0.0, start="random"),
        "bcc4_nn_uniaxial_field": W.bcc_nearest_neighbour(L=4, T=0.0, start="random"),
        "tri8_dmi_tensor": _tri(),
        "sc6x5x4_open_x": _open_sc(),
    }


def dipole_cases():
    return {
        "bcc5x6x7_3shell_dipole": W.bcc_three_shell(L=(5, 6, 7), T=0.0, start="random", dipole_cutoff=2.4),
        "sc6x5x3_film_dipole": W.sc_ferromagnet(L=(6, 5, 3), periodic=(1, 1, 0), dipole_cutoff=2.2),
    }


def _sc_pulse():
    w = W.sc_ferromagnet(L=(4, 5, 6))
    w.model.terms[2] = W.field_term((0.5, -0.3, 2.0), pulse=W.PULSE_SINC_COS, time_center=0.01,
                                    freq_bandwidth=50.0, freq_center=80.0)
    w.model.terms.append(W.zeeman_term([(0.1, 0.2, -0.3)], [(0.4, 0.0, 0.3)], [30.0]))
    return w


def _bcc_pulse():
    w = W.bcc_nearest_neighbour(L=4, T=0.0, start="random")
    w.model.terms = [t for t in w.model.terms if t.kind != W.TERM_APPLIED_FIELD]
    w.model.terms.insert(1, W.field_term((0.0, 0.0, 3.0), pulse=W.PULSE_SINC, time_center=0.02,
                                         freq_bandwidth=60.0))
    w.model.terms.append(W.zeeman_term([(0.2, 0.0, 0.0), (0.0, -0.3, 0.1)], [(0.0, 0.5, 0.0), (0.3, 0.0, 0.2)],
                                       [25.0, 40.0]))
    return w


def pulse_cases():
    return {
        "sc4x5x6_sinc_cos_zeeman_ac": _sc_pulse(),
        "bcc4_sinc_zeeman_dc_ac": _bcc_pulse(),
    }


def long_cases():
    """name -> (workload, integrator label, steps kept): T = 0, random start.
    The simple-cubic fixture keeps only the state after 1000 steps and a
    SHA-256 digest of its seeded start (W.initial_state regenerates it)."""
    tri = W.triangular_dmi_field_sweep(L=16, n_fields=1, T=0.0)
    tri.replicas[0].B = (0.0, 0.0, 0.5)
    return {
        "sc32_heun_1000": (W.sc_ferromagnet(L=32), "heun", (1000,)),
        "tri16_dmi_rk4_1000": (tri, "rk4", (1, 10, 100, 1000)),
    }


# bcc 10^3 x 2 (2000 spins) with the three-shell exchange and cubic
# anisotropy of the bcc 64^3 benchmark (mean-field ordering temperature
# about 85 K): 40 K in the ordered phase, 300 K in the paramagnetic phase.
# Start +z; burn-in steps, then samples every `every` steps.  The error of a
# mean comes from independent runs: the spectral NSE of one run of this
# length underestimates the run-to-run spread of <|M|> at 40 K several times
# (slow magnetisation modes), so the reference runs THERMAL_REF_SEEDS
# independent seeds and the GPU forms THERMAL_GPU_REPLICAS independent
# replicas, and each side's error is the standard error over its runs.
THERMAL_SEED = 20261204
THERMAL_REF_SEEDS = 8
THERMAL_GPU_REPLICAS = 16


def thermal_cases():
    """name -> (workload, burn-in steps, steps between samples, samples)."""
    return {
        "thermal_bcc10_3shell_40K": (W.bcc_three_shell(L=10, T=40.0, start="+z"), 200000, 25, 8000),
        "thermal_bcc10_3shell_300K": (W.bcc_three_shell(L=10, T=300.0, start="+z"), 20000, 25, 4000),
    }


def thermal_summary(abs_m, energies, n_spins):
    """Means and numerical standard errors (Stats::spectral_density_zero,
    src/jams/helpers/stats.cc:16-50) of |M| and of the energies per spin
    (total, then per term) of a sampled run."""
    import numpy as np

    from jams_gb300 import stats

    e = np.asarray(energies, dtype=np.float64) / n_spins
    series = {"abs_m": np.asarray(abs_m, dtype=np.float64), "e_total": e.sum(axis=1)}
    for t in range(e.shape[1]):
        series["e_term%d" % t] = e[:, t]
    out = {}
    for k, x in series.items():
        out[k + "_mean"] = float(x.mean())
        out[k + "_nse"] = stats.num_std_err(x)
        out[k + "_geweke"] = stats.geweke(x)[0]
    return out


def over_runs(per_run):
    """Mean and standard error of the mean over independent runs of per-run
    means {quantity: [value per run]}."""
    import math

    import numpy as np

    out = {}
    for k, v in per_run.items():
        v = np.asarray(v, dtype=np.float64)
        out[k + "_mean"] = float(v.mean())
        out[k + "_err"] = float(v.std(ddof=1) / math.sqrt(v.size))
    return out
