"""The allocation-free magnetisation entry point (llg_magnetisation_noalloc)
against the regular one (llg_observables), called through the C ABI.

It serves callers that cannot call cudaMalloc when they need the value
(stream capture, no-sync host loops, externally pooled memory), so its
reduction scratch is a fixed array inside the library.  This file is
collected last: if it fails, a run that stops at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

from jams_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-12  # FP64 sums in a different order


@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
def test_noalloc_magnetisation_equals_observables(llg, precision):
    import torch

    w = W.bcc_three_shell(L=10, T=300.0, start="random")
    s = llg.Solver(w, precision=getattr(llg, precision))
    s.set_state(W.initial_state(w, 0))
    s.step(3)
    m_ref, _ = s.observables(0)
    spins = torch.tensor(s.get_state(0), dtype=torch.float64, device="cuda")
    mus = np.ascontiguousarray(w.model.mus, dtype=np.float64)
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    L = llg.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # the scratch keeps the previous call's contents
        rc = L.llg_magnetisation_noalloc(spins.data_ptr(), spins.shape[0], w.model.nb,
                                         mus.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.data_ptr(),
                                         stream)
        assert rc == 0, L.llg_last_error(None)
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), m_ref, rtol=TOL, atol=TOL)
        out.fill_(float("nan"))


def test_noalloc_rejects_sizes_beyond_the_maximum(llg):
    import torch

    L = llg.lib()
    buf = torch.zeros((4, 3), dtype=torch.float64, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    mus = np.ones(1)
    dp = mus.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    for n in (0, (1 << 30) + 1):
        rc = L.llg_magnetisation_noalloc(buf.data_ptr(), n, 1, dp, out.data_ptr(), None)
        assert rc == -1
        assert b"n_spins" in L.llg_last_error(None)
