"""The benchmark's byte model of one dipole field evaluation (the
algorithmic bytes its FFT roofline divides by the measured evaluation time),
counted by hand for a periodic bcc grid and an open-z simple-cubic film."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    sys.path.insert(0, ROOT)
    import bench

    return bench


def test_bcc256_dipole_bytes_per_evaluation():
    bench = _bench()
    w = bench.WORKLOADS["bcc256_3shell_dipole"]()
    cells, f = 256 ** 3, 6                       # 3 components x 2 basis sites
    mq = 256 * 256 * 129                         # half spectrum along z
    spec = f * mq * 8
    real = f * cells * 4 + spec                  # spin planes in, spectra out (and back)
    passes = 2 * 2 * spec                        # axes 0 and 1, read + write each
    conv = 2 * spec + (2 * 6 * mq * 4 + 1 * 6 * mq * 8)   # spectra in and out + the stored tensors
    want = 2 * real + 2 * passes + conv
    assert bench.dipole_fft_bytes(w) == want
    assert abs(want - 6.486e9) < 1e7


def test_open_axis_doubles_the_grid():
    bench = _bench()
    from jams_gb300 import workloads as W

    w = W.sc_ferromagnet(L=(8, 6, 3), periodic=(1, 1, 0), dipole_cutoff=2.2)
    cells, f = 8 * 6 * 3, 3
    M = (8, 6, 6)                                # open z: 2L
    mq = 8 * 6 * (6 // 2 + 1)
    spec = f * mq * 8
    want = 2 * (f * cells * 4 + spec) + 2 * (2 * 2 * spec) + (2 * spec + 1 * 6 * mq * 4)
    assert bench.dipole_fft_bytes(w) == want
    assert M[2] == 2 * 3
