"""The allocation-free magnetisation entry point (llg_magnetisation_noalloc)
against the regular one (llg_observables) and a NumPy sum, called through
the C ABI.

It serves callers that cannot call cudaMalloc when they need the value (a
host loop that must not synchronise the device, memory owned by an external
pool), so its reduction scratch is a fixed array inside the library that
every call shares.  Two calls in a row check that the previous call's
scratch contents do not leak into the next result.  This file is collected
last: if it fails, a run that stops at the first failure has already run
every other test."""
import ctypes

import numpy as np
import pytest

from jams_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-12  # FP64 sums in a different order


def _call(L, spins, n, nb, mus, out, stream=None):
    mus = np.ascontiguousarray(mus, dtype=np.float64)
    return L.llg_magnetisation_noalloc(spins.data_ptr(), n, nb, mus.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       out.data_ptr(), stream)


@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
def test_noalloc_magnetisation_equals_observables(llg, precision):
    import torch

    w = W.bcc_three_shell(L=10, T=300.0, start="random")
    s = llg.Solver(w, precision=getattr(llg, precision))
    s.set_state(W.initial_state(w, 0))
    s.step(3)
    m_ref, _ = s.observables(0)
    spins = torch.tensor(s.get_state(0), dtype=torch.float64, device="cuda")
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    L = llg.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # the scratch keeps the previous call's contents
        rc = _call(L, spins, spins.shape[0], w.model.nb, w.model.mus, out, stream)
        assert rc == 0, L.llg_last_error(None)
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), m_ref, rtol=TOL, atol=TOL)
        out.fill_(float("nan"))


def test_noalloc_weights_each_basis_site_by_its_moment(llg):
    """Two basis sites with unequal mu_s: M = sum mu_b S_i / sum mu_b, site
    of spin i = i % nb, against NumPy; a large array first, then a small one
    (the second call reads fewer scratch slots than the first wrote)."""
    import torch

    L = llg.lib()
    mus = np.array([2.2, 0.7])
    for n in (600_002, 998):
        s = W.random_sphere(n, 7 + n)
        spins = torch.tensor(s, dtype=torch.float64, device="cuda")
        out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(L, spins, n, 2, mus, out) == 0, L.llg_last_error(None)
        torch.cuda.synchronize()
        mu = np.tile(mus, n // 2)
        m = (mu[:, None] * s).sum(axis=0) / mu.sum()
        np.testing.assert_allclose(out.cpu().numpy(), np.append(m, np.linalg.norm(m)), rtol=TOL, atol=TOL)


def test_noalloc_rejects_sizes_beyond_the_maximum(llg):
    import torch

    L = llg.lib()
    buf = torch.zeros((6, 3), dtype=torch.float64, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    for n in (0, (1 << 30) + 1):
        assert _call(L, buf, n, 1, [1.0], out) == -1
        assert b"n_spins" in L.llg_last_error(None)
    assert _call(L, buf, 5, 2, [1.0, 1.0], out) == -1        # not a multiple of nb
    assert b"multiple of nb" in L.llg_last_error(None)
    assert _call(L, buf, 5, 5, [1.0] * 5, out) == -1         # nb beyond the maximum of 4
    assert b"nb must be" in L.llg_last_error(None)
    for bad in (0.0, -1.0, float("nan"), float("inf")):
        assert _call(L, buf, 6, 2, [1.0, bad], out) == -1
        assert b"mu_s" in L.llg_last_error(None)
