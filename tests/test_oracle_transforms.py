"""The FFTW r2r transforms of realft (fourier.f90:16-63) restated from FFTW's
published R2HC/HC2R definitions, checked against numpy's real FFT and a direct
O(n^2) sum, plus ring_rpmd's monodromy coefficients and the ran2 stream."""
import math

import numpy as np
import pytest

from . import oracle_lib as orc


def r2hc_numpy(x):
    n = x.shape[0]
    X = np.fft.rfft(x, axis=0)
    out = np.zeros_like(x)
    out[: n // 2 + 1] = X.real
    for k in range(1, (n + 1) // 2):
        out[n - k] = X[k].imag
    return out


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 8, 12, 16, 32, 64, 7])
def test_r2hc_matches_fftw_definition(n):
    rng = np.random.default_rng(n)
    x = rng.normal(size=(n, 9))
    ref = r2hc_numpy(x) / math.sqrt(n)
    fast = orc.realft(x, +1)
    direct = orc.realft(x, +1, direct=True)
    scale = np.abs(ref).max()
    assert np.abs(fast - ref).max() <= 1e-14 * scale * max(1, n)
    assert np.abs(direct - ref).max() <= 1e-14 * scale * max(1, n)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 16, 32, 64])
def test_round_trip(n):
    rng = np.random.default_rng(100 + n)
    x = rng.normal(size=(n, 6))
    y = orc.realft(orc.realft(x, +1), -1)
    assert np.abs(y - x).max() < 1e-13


def test_ring_rpmd_free_particle_coefficients():
    import ctypes as C
    lib = orc.load()
    mass = np.array([29156.9471, 1837.1527, 1837.1527])
    nb, dt, beta = 8, 20.0, 1000.0
    monod = np.zeros(3 * 4 * nb)
    lib.orc_ring_rpmd(orc._ptr(mass), orc._ptr(monod), C.c_int(3), C.c_int(nb), C.c_double(dt), C.c_double(beta))
    m = monod.reshape(nb, 4, 3)  # [k][c][j]
    assert np.allclose(m[0, :, 0], [1.0, 0.0, dt / mass[0], 1.0])
    for k in range(1, nb):
        kk = min(k, nb - k)
        wk = 2.0 * nb / beta * math.sin(kk * math.pi / nb)
        for j in range(3):
            c, s = math.cos(wk * dt), math.sin(wk * dt)
            assert np.allclose(m[k, :, j], [c, -wk * mass[j] * s, s / (wk * mass[j]), c], rtol=1e-14)


def test_ran2_stream_reproducible_and_uniform():
    a, b = orc.Rng(4711), orc.Rng(4711)
    xa = np.array([a.ran2() for _ in range(5000)])
    xb = np.array([b.ran2() for _ in range(5000)])
    assert np.array_equal(xa, xb)
    assert 0.0 < xa.min() and xa.max() < 1.0
    assert abs(xa.mean() - 0.5) < 0.02
    g = orc.Rng(7)
    y = np.array([g.gaussian(2.0) for _ in range(20000)])
    assert abs(y.mean()) < 0.05 and abs(y.std() - 2.0) < 0.05
