"""CPU tests of the config-file front end (llg_config_describe): the model a
JAMS config describes equals the workload builders' model; parser, patch
merge, units and error reporting."""
import numpy as np
import pytest

from jams_gb300 import configs as C
from jams_gb300 import workloads as W


def template_set(term):
    out = set()
    for e in range(len(term["bi"])):
        J = tuple(round(v, 12) for v in term["J"][9 * e: 9 * e + 9])
        out.add((int(term["bi"][e]), int(term["bj"][e]), tuple(int(v) for v in term["T"][3 * e: 3 * e + 3]), J))
    return out


def workload_set(t):
    return {(int(t.bi[e]), int(t.bj[e]), tuple(int(v) for v in t.T[e]),
             tuple(round(v, 12) for v in np.asarray(t.J[e]).reshape(-1))) for e in range(len(t.bi))}


def check_model(d, w):
    m = w.model
    assert d["nb"] == m.nb
    assert d["L"] == list(w.replicas[0].L)
    np.testing.assert_array_equal(d["mus"], m.mus)
    np.testing.assert_array_equal(d["gyro"], m.gyro)
    np.testing.assert_array_equal(d["alpha"], m.alpha)
    assert d["dt"] == m.dt
    assert d["integrator"] == m.integrator
    assert len(d["terms"]) == len(m.terms)
    for td, tw in zip(d["terms"], m.terms):
        assert td["kind"] == tw.kind
        if tw.kind == W.TERM_EXCHANGE:
            assert template_set(td) == workload_set(tw)
        elif tw.kind in (W.TERM_UNIAXIAL, W.TERM_CUBIC):
            assert td["order"] == tw.order
            np.testing.assert_allclose(td["K"], tw.K, rtol=1e-15)
            np.testing.assert_allclose(td["axis"], np.asarray(tw.axis).reshape(-1), atol=1e-15)


def test_sc_config_matches_workload(llg):
    d = llg.describe_config(C.sc_ferromagnet(L=32))
    check_model(d, W.sc_ferromagnet(L=32))
    assert d["max_steps"] == 1000
    assert d["terms"][2]["B"] == [0.0, 0.0, 1.0]


def test_bcc_symmetry_expansion_gives_26_neighbours(llg):
    """One interaction vector per shell expands by the site point group to
    8 + 6 + 12 neighbours per basis site, as spglib's operations do."""
    d = llg.describe_config(C.bcc_three_shell(L=8))
    w = W.bcc_three_shell(L=8)
    check_model(d, w)
    ex = d["terms"][0]
    assert len(ex["bi"]) == 52
    assert d["max_steps"] == 20000


def test_fcc_symmetry_expansion_gives_18_neighbours(llg):
    """One vector per shell on the 4-site fcc cell expands to 12 + 6
    neighbours per site (the fcc sites' point group is the full cubic one)."""
    d = llg.describe_config(C.fcc_two_shell(L=6))
    w = W.fcc_ferromagnet(L=6, J2=0.2)
    check_model(d, w)
    assert len(d["terms"][0]["bi"]) == 4 * 18


def test_triangular_tensor_config(llg):
    d = llg.describe_config(C.triangular_dmi(L=16))
    w = W.triangular_dmi_field_sweep(L=16, n_fields=1)
    check_model(d, w)
    assert d["periodic"] == [1, 1, 0]


def test_patch_merges_over_config(llg):
    base = C.sc_ferromagnet(L=8)
    d = llg.describe_config(base, 'physics : { temperature = 100.0; }; lattice : { size = [4, 5, 6]; };')
    assert d["temperature"] == 100.0
    assert d["L"] == [4, 5, 6]
    d = llg.describe_config(base, 'hamiltonians = ( { interactions = ( ("A", "A", [1.0, 0.0, 0.0], 2.5) ); } );')
    assert set(round(v, 9) for v in d["terms"][0]["J"] if v != 0.0) == {2.5}


def test_energy_units_joules_default(llg):
    """Without energy_units the reference reads joules (kJoule2meV)."""
    cfg = C.sc_ferromagnet(L=4).replace('{ module = "exchange"; energy_units = "meV";', '{ module = "exchange";')
    cfg = cfg.replace("], 1.0) ); },", "], 1.602176634e-22) ); },")
    d = llg.describe_config(cfg)
    J = [v for v in d["terms"][0]["J"] if v != 0.0]
    np.testing.assert_allclose(J, 1.602176634e-22 * 6.24150907e21, rtol=1e-15)


def test_parser_comments_and_syntax(llg):
    cfg = C.sc_ferromagnet(L=4)
    cfg = "/* block\n comment */\n# hash comment\n" + cfg.replace("lattice : {", "lattice = { // trailing\n")
    d = llg.describe_config(cfg)
    assert d["L"] == [4, 4, 4]


@pytest.mark.parametrize("bad,msg", [
    ("lattice : { size = [4, 4, 4] ", "missing '}'"),
    ('hamiltonians = ( { module = "crystal-field"; } );', "not on the LLG hot path"),
    ('solver : { module = "monte-carlo-metropolis-cpu"; t_step = 1e-15; t_max = 1e-12; };', "unknown solver"),
])
def test_config_errors_are_reported(llg, bad, msg):
    cfg = C.sc_ferromagnet(L=4)
    if bad.startswith("lattice"):
        cfg = cfg.replace("lattice : { size = [4, 4, 4]; periodic = [true, true, true]; };", bad)
    elif bad.startswith("hamiltonians"):
        cfg = cfg[: cfg.index("hamiltonians")] + bad + cfg[cfg.index("solver"):]
    else:
        cfg = cfg[: cfg.index("solver")] + bad + cfg[cfg.index("physics"):]
    with pytest.raises(llg.LLGError, match=msg):
        llg.describe_config(cfg)


PULSE_HAMILTONIANS = """hamiltonians = (
  { module = "exchange"; energy_units = "meV"; interactions = ( ("A", "A", [1.0, 0.0, 0.0], 1.0) ); },
  { module = "applied-field"; type = "sinc-cos"; field = [0.5, -0.3, 2.0]; time_center = 1.0e-14;
    freq_bandwidth = 5.0e13; freq_center = 8.0e13; },
  { module = "zeeman"; dc_local_field = ( [0.1, 0.2, -0.3] ); ac_local_field = ( [0.4, 0.0, 0.3] );
    ac_local_frequency = ( 30.0 ); }
);
"""


def pulse_config(hamiltonians=PULSE_HAMILTONIANS):
    cfg = C.sc_ferromagnet(L=4)
    return cfg[: cfg.index("hamiltonians")] + hamiltonians + cfg[cfg.index("solver"):]


def test_time_dependent_fields_in_config(llg):
    """applied-field type sinc-cos (time_center in s, frequencies in Hz,
    converted to ps and THz as applied_field.cc:36-38,64-67) and a zeeman term
    with dc and ac fields per material (zeeman.cc:12-71)."""
    d = llg.describe_config(pulse_config())
    af, ze = d["terms"][1], d["terms"][2]
    assert af["kind"] == W.TERM_APPLIED_FIELD and ze["kind"] == W.TERM_ZEEMAN
    assert af["B"] == [0.5, -0.3, 2.0]
    assert af["pulse"] == [W.PULSE_SINC_COS, 1.0e-14 / 1e-12, 5.0e13 / 1e12, 8.0e13 / 1e12]
    assert ze["dc_field"] == [0.1, 0.2, -0.3]
    assert ze["ac_field"] == [0.4, 0.0, 0.3]
    assert ze["ac_frequency"] == [30.0]
    sinc = pulse_config(PULSE_HAMILTONIANS.replace('type = "sinc-cos"', 'type = "SINC"'))
    assert llg.describe_config(sinc)["terms"][1]["pulse"][:3] == [W.PULSE_SINC, 1.0e-14 / 1e-12, 5.0e13 / 1e12]


@pytest.mark.parametrize("change,msg", [
    (('type = "sinc-cos"', 'type = "gaussian"'), "unknown field pulse type gaussian"),
    (("ac_local_frequency = ( 30.0 );", ""), "must have a field and a frequency"),
    (("dc_local_field = ( [0.1, 0.2, -0.3] );", "dc_local_field = ( [0.1, 0.2, -0.3], [0.0, 0.0, 1.0] );"),
     "every material"),
])
def test_time_dependent_field_config_errors(llg, change, msg):
    with pytest.raises(llg.LLGError, match=msg):
        llg.describe_config(pulse_config(PULSE_HAMILTONIANS.replace(*change)))


def test_duplicate_site_pair_is_rejected_at_create(llg):
    """Reaching the same site twice is an error in the reference
    (interactions.cc:371-380); it is raised by llg_create before any device
    work, so this runs without a GPU."""
    w = W.sc_ferromagnet(L=(2, 4, 4))
    with pytest.raises(llg.LLGError, match="Multiple interactions"):
        llg.Solver(w, precision=llg.FP64)


_INLINE = '''    interactions = (
      ("Fe", "Fe", [0.5, 0.5, 0.5], 2.0),    // shell 1: 8 at a<111>/2
      ("Fe", "Fe", [1.0, 0.0, 0.0], 1.2),    // shell 2: 6 at a<100>
      ("Fe", "Fe", [1.0, 1.0, 0.0], -0.1)    // shell 3: 12 at a<110>
    );
'''


def _with_exc_file(path):
    text = C.bcc_three_shell(L=6)
    assert text.count(_INLINE) == 1
    return text.replace(_INLINE, '    exc_file = "%s";\n' % path)


def test_exc_file_jams_and_kkr_formats_equal_the_inline_list(llg, tmp_path):
    """exc_file (src/jams/core/interactions.cc:127-246): material names or
    1-based basis sites, a scalar J (6 columns) or a 3x3 tensor (14), '#',
    '//' and short lines skipped.  Both files describe the model of the
    inline list."""
    ref = llg.describe_config(C.bcc_three_shell(L=6))["terms"][0]
    jams = tmp_path / "jams.txt"
    jams.write_text("# bcc, three shells (meV)\n\nFe Fe 0.5 0.5 0.5 2.0\n  // shell 2\nFe Fe 1.0 0.0 0.0 1.2\n"
                    "x\nFe Fe 1.0 1.0 0.0 -0.1\n")
    kkr = tmp_path / "kkr.txt"
    rows = []
    for (i, j, r, J) in ((1, 2, "0.5 0.5 0.5", 2.0), (2, 1, "-0.5 -0.5 -0.5", 2.0), (1, 1, "1.0 0.0 0.0", 1.2),
                         (2, 2, "1.0 0.0 0.0", 1.2), (1, 1, "1.0 1.0 0.0", -0.1), (2, 2, "1.0 1.0 0.0", -0.1)):
        rows.append("%d %d %s %s" % (i, j, r, " ".join(repr(J if a % 4 == 0 else 0.0) for a in range(9))))
    kkr.write_text("// i j rx ry rz Jxx ... Jzz\n" + "\n".join(rows) + "\n")
    for path in (jams, kkr):
        ex = llg.describe_config(_with_exc_file(path))["terms"][0]
        got = sorted(zip(ex["bi"], ex["bj"], map(tuple, np.reshape(ex["T"], (-1, 3))),
                         map(tuple, np.reshape(ex["J"], (-1, 9)))))
        want = sorted(zip(ref["bi"], ref["bj"], map(tuple, np.reshape(ref["T"], (-1, 3))),
                          map(tuple, np.reshape(ref["J"], (-1, 9)))))
        assert got == want, path


@pytest.mark.parametrize("content,needle", [
    ("Fe Fe 0.5 0.5 0.5\n", "incorrect number of columns"),
    ("Fe 1 0.5 0.5 0.5 2.0\n", "failed to discover"),
    ("# only comments\n\n", "failed to discover"),
    ("Fe Fe 0.5 0.5 0.5 2.0\nFe Fe 1.0 0.0 zero 1.2\n", "failed to read line 2"),
    ("1 3 0.5 0.5 0.5 2.0\n", "basis index out of range"),
])
def test_exc_file_errors(llg, tmp_path, content, needle):
    p = tmp_path / "bad.txt"
    p.write_text(content)
    with pytest.raises(llg.LLGError, match=needle):
        llg.describe_config(_with_exc_file(p))


def test_exc_file_missing(llg, tmp_path):
    with pytest.raises(llg.LLGError, match="failed to open exc_file"):
        llg.describe_config(_with_exc_file(tmp_path / "absent.txt"))
