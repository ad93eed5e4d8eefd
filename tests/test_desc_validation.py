"""CPU checks of llg_create's descriptor validation: an empty lattice, an
empty replica list, out-of-range basis indices, non-finite or unknown
parameters and a lattice too large for 32-bit spin indices are each
rejected with a status code and a message naming the field, before the
library touches a device (so these run without a GPU).

The reference rejects the same inputs while it reads its config
(jams/core/lattice.cc:688-739 for sizes and materials,
jams/core/interactions.cc:254-444 for interaction lists,
jams/hamiltonian/uniaxial_anisotropy.cc for the anisotropy order) by
throwing; the C ABI returns LLG_ERR_BAD_DESC or LLG_ERR_UNSUPPORTED with
the message in llg_last_error(NULL)."""
import ctypes
import math

import pytest

from jams_gb300 import workloads as W

BAD_DESC, UNSUPPORTED = -1, -7


def _term(d, kind):
    for t in range(d.n_terms):
        if d.terms[t].kind == kind:
            return d.terms[t]
    raise AssertionError("workload has no term of kind %d" % kind)


def _set_exchange_bj(d):
    _term(d, W.TERM_EXCHANGE).bj[0] = 7


def _set_exchange_nan(d):
    _term(d, W.TERM_EXCHANGE).J[0] = math.nan


def _set_uniaxial_order(d):
    _term(d, W.TERM_UNIAXIAL).order = 3


def _set_pulse(d):
    t = _term(d, W.TERM_APPLIED_FIELD)
    t.pulse = 9


def _set_pulse_nan(d):
    t = _term(d, W.TERM_APPLIED_FIELD)
    t.pulse = W.PULSE_SINC
    t.time_center = math.nan


def _set_L(axis, value):
    def f(d):
        d.replicas[0].L[axis] = value
    return f


def _set_mus(d):
    d.mus[0] = 0.0


CASES = [
    ("abi_version", lambda d: setattr(d, "abi_version", 2), BAD_DESC, "abi_version"),
    ("nb zero", lambda d: setattr(d, "nb", 0), BAD_DESC, "nb must be"),
    ("nb above the maximum", lambda d: setattr(d, "nb", 1000), BAD_DESC, "nb must be"),
    ("n_terms negative", lambda d: setattr(d, "n_terms", -1), BAD_DESC, "n_terms must be"),
    ("n_terms above the maximum", lambda d: setattr(d, "n_terms", 1000), BAD_DESC, "n_terms must be"),
    ("no replicas", lambda d: setattr(d, "n_replicas", 0), BAD_DESC, "at least one replica"),
    ("dt zero", lambda d: setattr(d, "dt", 0.0), BAD_DESC, "dt must be positive"),
    ("dt nan", lambda d: setattr(d, "dt", math.nan), BAD_DESC, "dt must be positive"),
    ("dt inf", lambda d: setattr(d, "dt", math.inf), BAD_DESC, "dt must be positive"),
    ("precision", lambda d: setattr(d, "precision", 5), BAD_DESC, "unknown precision"),
    ("integrator", lambda d: setattr(d, "integrator", 5), BAD_DESC, "unknown integrator"),
    ("mu_s zero", _set_mus, BAD_DESC, "mu_s of basis site 0"),
    ("empty lattice x", _set_L(0, 0), BAD_DESC, "lattice size must be positive"),
    ("empty lattice z", _set_L(2, 0), BAD_DESC, "lattice size must be positive"),
    ("negative lattice", _set_L(1, -4), BAD_DESC, "lattice size must be positive"),
    # periodic, two cells wide: the +x and -x neighbours are the same site
    ("periodic image reached twice", _set_L(0, 2), BAD_DESC, "Multiple interactions"),
    ("negative temperature", lambda d: setattr(d.replicas[0], "temperature", -1.0), BAD_DESC,
     "temperature must be >= 0"),
    ("nan temperature", lambda d: setattr(d.replicas[0], "temperature", math.nan), BAD_DESC,
     "temperature must be >= 0"),
    ("exchange basis index", _set_exchange_bj, BAD_DESC, "basis index outside"),
    ("exchange non-finite J", _set_exchange_nan, BAD_DESC, "non-finite J"),
    ("uniaxial power", _set_uniaxial_order, BAD_DESC, "uniaxial power must be 2, 4 or 6"),
    ("unknown pulse", _set_pulse, BAD_DESC, "unknown pulse type"),
    ("non-finite pulse", _set_pulse_nan, BAD_DESC, "non-finite pulse parameters"),
    ("too many spins", lambda d: [d.replicas[0].L.__setitem__(a, 2048) for a in range(3)], UNSUPPORTED,
     "too many spins"),
]


@pytest.mark.parametrize("name,mutate,code,needle", CASES, ids=[c[0] for c in CASES])
def test_bad_descriptor_is_rejected(llg, name, mutate, code, needle):
    w = W.sc_ferromagnet(L=4)
    d, keep = llg.build_desc(w, llg.FP64)
    mutate(d)
    h = ctypes.c_void_p()
    L = llg.lib()
    rc = L.llg_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == code, (name, rc, L.llg_last_error(None))
    assert not h.value
    msg = L.llg_last_error(None).decode()
    assert needle in msg, (name, msg)
    del keep


def test_null_arguments_are_rejected(llg):
    L = llg.lib()
    h = ctypes.c_void_p()
    assert L.llg_create(None, ctypes.byref(h)) == BAD_DESC
    assert "null descriptor" in L.llg_last_error(None).decode()
    d, keep = llg.build_desc(W.sc_ferromagnet(L=4), llg.FP64)
    assert L.llg_create(ctypes.byref(d), None) == BAD_DESC
    assert "out is null" in L.llg_last_error(None).decode()
    # calls on a null handle report the error instead of dereferencing it
    assert L.llg_step(None, 1) == BAD_DESC
    assert L.llg_set_iteration(None, 0) == BAD_DESC
    del keep
