"""The small seeded workloads behind the golden fixtures (all T = 0, Heun).

cases(): the reference's exchange, anisotropy and field terms; the FP64 form
equals these bit for bit.  dipole_cases(): with the dipole-dipole term (the
reference's dipole-bruteforce Hamiltonian); the FFT evaluation equals these
within rounding, not bit for bit.  pulse_cases(): time-dependent applied
fields (sinc and sinc-cos pulses) and zeeman dc / ac fields; their sin and cos
come from the C library, so the fixtures pin the oracle bit for bit where
they were made and the GPU form within 1e-12 elsewhere."""
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
