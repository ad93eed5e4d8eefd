"""The small seeded workloads behind the golden fixtures (all T = 0, Heun)."""
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
