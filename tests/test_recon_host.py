"""Host-side pieces of ctlib_gb300.recon that need no GPU: the seeded
Poisson log-sinogram generator of the equal-angle unrolled-reconstruction
workload."""

import numpy as np


def test_poisson_log_sinogram_seeded():
    from ctlib_gb300 import recon
    ax = np.linspace(0.0, 12.0, 4096, dtype=np.float32).reshape(1, 1, 64, 64)
    a = recon.poisson_log_sinogram(ax, 1e5, 11)
    b = recon.poisson_log_sinogram(ax, 1e5, 11)
    assert a.dtype == np.float32 and np.array_equal(a, b)
    # counts clamped >= 1: y never exceeds log(I0)
    assert a.max() <= np.log(1e5) + 1e-4
    # small line integrals: the noise is about 1/sqrt(I0) around the truth
    assert abs(float(a[0, 0, 0, :16].mean() - ax[0, 0, 0, :16].mean())) < 0.02


def test_poisson_log_sinogram_clamps_dark_readings():
    """Line integrals so large that no photon arrives give counts of 0, which
    are read as 1: y = log(I0), finite."""
    from ctlib_gb300 import recon
    y = recon.poisson_log_sinogram(np.full((1, 1, 4, 4), 40.0), 1e5, 11)
    assert np.allclose(y, np.log(1e5))
