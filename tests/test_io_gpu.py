"""Spin files and checkpoints through a solver on the GPU: the spins a file
holds are the solver's state, and a checkpoint continues a trajectory bit for
bit (thermal noise included)."""
import numpy as np
import pytest

from jams_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def models():
    return {
        "sc_sweep": W.sc_temperature_sweep(n_replicas=4, L_min=5, L_max=9),
        "bcc3": W.bcc_three_shell(L=6, T=300.0, start="random"),
        "tri_rk4": W.triangular_dmi_field_sweep(L=(24, 18, 1), n_fields=2, T=5.0),
    }


def fresh(llg, w, precision):
    s = llg.Solver(w, precision=precision, steps_per_graph=4)
    for r in range(len(w.replicas)):
        s.set_state(W.initial_state(w, r), r)
    return s


@pytest.mark.parametrize("ext", ["h5", "txt"])
@pytest.mark.parametrize("prec", ["FP64", "FP32C"])
def test_spin_file_round_trip(llg, tmp_path, ext, prec):
    w = W.bcc_three_shell(L=5, T=300.0, start="random")
    a = fresh(llg, w, getattr(llg, prec))
    a.step(3)
    path = str(tmp_path / ("final." + ext))
    a.write_spins(path, 0)
    ref = a.get_state(0)
    got = llg.read_array_file(path, "/spins").reshape(-1, 3)
    np.testing.assert_array_equal(got, ref)
    b = fresh(llg, w, getattr(llg, prec))
    b.read_spins(path, 0)
    np.testing.assert_array_equal(b.get_state(0), ref)


def test_spin_file_size_is_checked(llg, tmp_path):
    w = W.sc_ferromagnet(L=4)
    s = fresh(llg, w, llg.FP64)
    path = str(tmp_path / "short.h5")
    llg.write_array_file(path, np.ones((10, 3)), "/spins")
    with pytest.raises(llg.LLGError, match="expected size: 192 actual size: 30"):
        s.read_spins(path, 0)


@pytest.mark.parametrize("name", ["sc_sweep", "bcc3", "tri_rk4"])
@pytest.mark.parametrize("prec", ["FP64", "FP32C"])
def test_checkpoint_resume_is_bit_exact(llg, tmp_path, name, prec):
    w = models()[name]
    p = getattr(llg, prec)
    a = fresh(llg, w, p)
    a.set_temperature(0, 37.0)
    a.set_field(len(w.replicas) - 1, [0.1, -0.2, 0.5])
    a.step(9)
    path = str(tmp_path / "run.ckpt")
    a.save_checkpoint(path)
    a.step(13)
    want = a.get_state(-1)
    b = llg.Solver(w, precision=p, steps_per_graph=4)   # fresh state, T, B and iteration
    b.load_checkpoint(path)
    assert b.iteration == 9
    b.step(13)
    assert b.iteration == 22
    assert np.array_equal(b.get_state(-1), want)


def test_checkpoint_rejects_other_models_and_corruption(llg, tmp_path):
    w = W.bcc_three_shell(L=5, T=300.0, start="random")
    a = fresh(llg, w, llg.FP32C)
    a.step(2)
    path = tmp_path / "run.ckpt"
    a.save_checkpoint(str(path))
    other = fresh(llg, W.bcc_three_shell(L=5, T=300.0, start="random", seed=2), llg.FP32C)
    before = other.get_state(-1)
    with pytest.raises(llg.LLGError, match="different model"):
        other.load_checkpoint(str(path))
    with pytest.raises(llg.LLGError, match="different model"):
        fresh(llg, w, llg.FP64).load_checkpoint(str(path))
    raw = bytearray(path.read_bytes())
    raw[200] ^= 1
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(bytes(raw))
    with pytest.raises(llg.LLGError, match="checksum"):
        other.load_checkpoint(str(bad))
    assert np.array_equal(other.get_state(-1), before)
    assert other.iteration == 0


def test_checkpoint_rejects_other_hamiltonian_parameters(llg, tmp_path):
    """The fingerprint covers the terms and their parameters: the same
    lattice, seed and precision with another J, K or field is refused, and
    the refused load leaves the solver untouched."""
    w = W.bcc_three_shell(L=5, T=300.0, start="random")
    a = fresh(llg, w, llg.FP32C)
    a.step(2)
    path = tmp_path / "run.ckpt"
    a.save_checkpoint(str(path))
    for change in ("J", "K", "terms"):
        w2 = W.bcc_three_shell(L=5, T=300.0, start="random")
        if change == "J":
            w2.model.terms[0].J = w2.model.terms[0].J * 1.01
        elif change == "K":
            w2.model.terms[1].K = w2.model.terms[1].K * 2.0
        else:
            w2.model.terms = w2.model.terms[:1]
        other = fresh(llg, w2, llg.FP32C)
        before = other.get_state(-1)
        with pytest.raises(llg.LLGError, match="different model"):
            other.load_checkpoint(str(path))
        assert np.array_equal(other.get_state(-1), before)
        assert other.iteration == 0
    fresh(llg, W.bcc_three_shell(L=5, T=300.0, start="random"), llg.FP32C).load_checkpoint(str(path))


def test_pinned_host_buffers_go_through_the_mapped_path(llg):
    """Pinned host buffers are read in place by the unpack kernel (results
    come back through the copy engines); the result equals the pageable
    (copied) path bit for bit, including a replica's rows in the middle of a
    pinned buffer."""
    torch = pytest.importorskip("torch")
    w = W.sc_temperature_sweep(n_replicas=3, L_min=5, L_max=8)
    sizes = [int(np.prod(r.L)) for r in w.replicas]
    n = sum(sizes)
    s = fresh(llg, w, llg.FP32C)
    s.step(3)
    want = s.get_state(-1)
    pinned = torch.empty((n, 3), dtype=torch.float64, pin_memory=True)
    got = pinned.numpy()
    s.get_state(-1, out=got)
    assert np.array_equal(got, want)
    new = W.random_sphere(n, seed=11)
    got[:] = new
    s.set_state(got)
    assert np.array_equal(s.get_state(-1), new.astype(np.float32).astype(np.float64))
    # replica 1 into / from the interior rows of the pinned buffer
    lo, hi = sizes[0], sizes[0] + sizes[1]
    got[:] = 0.0
    s.get_state(1, out=got[lo:hi])
    assert np.array_equal(got[lo:hi], s.get_state(1))
    assert not got[:lo].any() and not got[hi:].any()
    got[lo:hi] = W.random_sphere(sizes[1], seed=12)
    s.set_state(got[lo:hi], 1)
    assert np.array_equal(s.get_state(1), got[lo:hi].astype(np.float32).astype(np.float64))
