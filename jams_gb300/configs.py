"""JAMS config-file texts of the LLG workloads (libconfig format, as the
reference's `jams` executable reads them), for llg_create_from_config.

Each text describes the same model as the matching builder in workloads.py:
materials in Bohr magnetons, exchange with energy_units = "meV" and one
interaction per shell expanded by the crystal's symmetry operations (or an
explicit list with symops = false), t_step / t_max in seconds.
"""
from __future__ import annotations


def _header(material: str, moment: float, alpha: float, spin: str) -> str:
    return """materials = (
  { name = "%s"; moment = %r; gyro = 1.0; alpha = %r; spin = %s; }
);
""" % (material, moment, alpha, spin)


def sc_ferromagnet(L=32, T=0.0, t_step=1e-15, steps=1000, seed=1, J=1.0, dz=0.1, Bz=1.0, moment=2.0,
                   alpha=0.1, spin='"random"') -> str:
    return _header("A", moment, alpha, spin) + """
unitcell : {
  parameter = 3.0e-10;
  basis = ( [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0] );
  positions = ( ("A", [0.0, 0.0, 0.0]) );
};

lattice : { size = [%d, %d, %d]; periodic = [true, true, true]; };

hamiltonians = (
  { module = "exchange"; energy_units = "meV"; interactions = ( ("A", "A", [1.0, 0.0, 0.0], %r) ); },
  { module = "uniaxial"; energy_units = "meV"; order = "K1"; anisotropies = ( ("A", [0.0, 0.0, 1.0], %r) ); },
  { module = "applied-field"; field = [0.0, 0.0, %r]; }
);

solver : { module = "llg-heun-gpu"; t_step = %r; t_max = %r; };
physics : { temperature = %r; };
sim : { seed = %d; };
""" % (L, L, L, J, dz, Bz, t_step, t_step * steps, T, seed)


def bcc_three_shell(L=64, T=300.0, t_step=0.5e-15, steps=20000, seed=1, spin="[0.0, 0.0, 1.0]",
                    dipole_cutoff=None) -> str:
    return _header("Fe", 2.2, 0.05, spin) + """
// conventional cubic cell, two-site basis
unitcell : {
  parameter = 2.87e-10;
  basis = ( [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0] );
  positions = ( ("Fe", [0.0, 0.0, 0.0]), ("Fe", [0.5, 0.5, 0.5]) );
};

lattice : { size = [%d, %d, %d]; periodic = [true, true, true]; };

hamiltonians = (
  {
    module = "exchange";
    energy_units = "meV";
    interactions = (
      ("Fe", "Fe", [0.5, 0.5, 0.5], 2.0),    // shell 1: 8 at a<111>/2
      ("Fe", "Fe", [1.0, 0.0, 0.0], 1.2),    // shell 2: 6 at a<100>
      ("Fe", "Fe", [1.0, 1.0, 0.0], -0.1)    // shell 3: 12 at a<110>
    );
  },
  { module = "cubic"; energy_units = "meV"; K1 = ( (0.005, [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]) ); }%s
);

solver : { module = "llg-heun-gpu"; t_step = %r; t_max = %r; };
physics : { temperature = %r; };
sim : { seed = %d; };
""" % (L, L, L, (',\n  { module = "dipole-fft"; r_cutoff = %r; }' % dipole_cutoff) if dipole_cutoff else "",
       t_step, t_step * steps, T, seed)


def triangular_dmi(L=2048, T=5.0, Bz=0.0, t_step=1e-15, steps=5000, seed=1, J1=1.0, D=0.3) -> str:
    """Triangular monolayer; tensor exchange J1 I - [D_ij]x with
    D_ij = D (z x r_ij), given explicitly (symops = false): symmetry
    operations copy a tensor unchanged to every image, which is not right for
    an antisymmetric DMI tensor."""
    import math

    import numpy as np

    from . import workloads as W

    lines = []
    for (bi, bj, T_, Jm) in W.triangular_dmi_entries(J1, D):
        r = T_[0] * np.array([1.0, 0.0, 0.0]) + T_[1] * np.array([0.5, math.sqrt(3.0) / 2.0, 0.0])
        vals = ", ".join(repr(float(x)) for x in np.asarray(Jm).reshape(-1))
        lines.append('      ("A", "A", [%r, %r, 0.0], [%s])' % (float(r[0]), float(r[1]), vals))
    inter = ",\n".join(lines)
    return _header("A", 2.0, 0.3, '"random"') + """
unitcell : {
  parameter = 3.0e-10;
  basis = ( [1.0, 0.5, 0.0], [0.0, 0.8660254037844386, 0.0], [0.0, 0.0, 1.0] );
  positions = ( ("A", [0.0, 0.0, 0.0]) );
};

lattice : { size = [%d, %d, 1]; periodic = [true, true, false]; };

hamiltonians = (
  {
    module = "exchange";
    energy_units = "meV";
    symops = false;
    interactions = (
%s
    );
  },
  { module = "uniaxial"; energy_units = "meV"; order = "K1"; anisotropies = ( ("A", [0.0, 0.0, 1.0], 0.2) ); },
  { module = "applied-field"; field = [0.0, 0.0, %r]; }
);

solver : { module = "llg-rk4-gpu"; t_step = %r; t_max = %r; };
physics : { temperature = %r; };
sim : { seed = %d; };
""" % (L, L, inter, Bz, t_step, t_step * steps, T, seed)


def fcc_two_shell(L=32, T=300.0, t_step=0.5e-15, steps=2000, seed=1, J1=1.5, J2=0.2) -> str:
    """fcc conventional cell (4 sites), one interaction vector per shell
    expanded by the crystal's symmetry operations: 12 + 6 neighbours."""
    return _header("Ni", 1.7, 0.05, "[0.0, 0.0, 1.0]") + """
unitcell : {
  parameter = 3.52e-10;
  basis = ( [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0] );
  positions = ( ("Ni", [0.0, 0.0, 0.0]), ("Ni", [0.0, 0.5, 0.5]),
                ("Ni", [0.5, 0.0, 0.5]), ("Ni", [0.5, 0.5, 0.0]) );
};

lattice : { size = [%d, %d, %d]; periodic = [true, true, true]; };

hamiltonians = (
  {
    module = "exchange";
    energy_units = "meV";
    interactions = (
      ("Ni", "Ni", [0.5, 0.5, 0.0], %r),    // 12 at a<110>/2
      ("Ni", "Ni", [1.0, 0.0, 0.0], %r)     // 6 at a<100>
    );
  },
  { module = "uniaxial"; energy_units = "meV"; order = "K1"; anisotropies = ( ("Ni", [0.0, 0.0, 1.0], 0.01) ); },
  { module = "applied-field"; field = [0.0, 0.0, 0.5]; }
);

solver : { module = "llg-heun-gpu"; t_step = %r; t_max = %r; };
physics : { temperature = %r; };
sim : { seed = %d; };
""" % (L, L, L, J1, J2, t_step, t_step * steps, T, seed)
