"""The oracle's non-cubic Ewald sum (ewald_noncubic.f90: rwald_basic /
rwald_cell + kwald_nc), which no reference test reaches.  It is pinned to the
cubic restatement, itself pinned to the reference's golden run: on a cubic box
with the same Ewald parameters in bohr, the two give the same energy, forces
and diagonal virial (the cubic reciprocal virial's off-diagonal entries use
|k_a||k_b|, ewald_cubic.f90:488-503, the non-cubic ones k_a k_b).  On a
genuinely non-cubic 8 x 4 x 4 box: forces against central differences of the
energy, and invariance under a rigid translation."""
import numpy as np
import pytest

from . import oracle_lib as orc
from . import systems


def noncubic_params(s):
    P = orc.get_params()
    P.iamcub = 0
    orc.set_params(P)
    orc.setup_ewald(s["na"], s["box"])  # the non-cubic branch of setup_ewald (setup_options.f90:157-181)
    return orc.get_params()


def test_noncubic_equals_cubic_on_cubic_box():
    s = systems.build(ncell=(6, 6, 6), nb=1)
    r = systems.perturbed(s, seed=3)
    st, v_c, f_c, vir_c = orc.forces(r, s["box"], s["z"], 2)
    assert st == 0
    Pc = orc.get_params()
    Pn = noncubic_params(s)
    assert Pn.iamcub == 0 and Pn.kmax == Pc.kmax
    assert abs(Pn.wrcut - Pc.wrcut * s["box"][0]) < 1e-12 * Pn.wrcut
    st, v_n, f_n, vir_n = orc.forces(r, s["box"], s["z"], 2)
    assert st == 0
    assert abs(v_n - v_c) <= 1e-12 * abs(v_c)
    assert np.linalg.norm(f_n - f_c) <= 1e-12 * np.linalg.norm(f_c)
    assert np.abs(np.diag(vir_n) - np.diag(vir_c)).max() <= 1e-12 * np.abs(np.diag(vir_c)).max()


@pytest.fixture(scope="module")
def box844():
    s = systems.build(ncell=(8, 4, 4), nb=1)
    assert s["params"].iamcub == 0 and s["box"][0] > 1.9 * s["box"][1]
    return s


def test_noncubic_forces_match_energy_differences(box844):
    s = box844
    orc.set_params(s["params"])
    r = systems.perturbed(s, seed=4)
    st, v, f, vir = orc.forces(r, s["box"], s["z"], 2)
    assert st == 0
    h = 1e-5
    rng = np.random.default_rng(1)
    for _ in range(8):
        j, x = int(rng.integers(s["na"])), int(rng.integers(3))
        rp, rm = r.copy(), r.copy()
        rp[0, j, x] += h
        rm[0, j, x] -= h
        vp = orc.forces(rp, s["box"], s["z"], 2)[1]
        vm = orc.forces(rm, s["box"], s["z"], 2)[1]
        # the A&S erfc of the energy is an approximation whose derivative the force does not use
        assert abs((vp - vm) / (2 * h) - f[0, j, x]) <= 1e-5 * np.abs(f).max()


def test_noncubic_translation_invariance(box844):
    s = box844
    orc.set_params(s["params"])
    r = systems.perturbed(s, seed=5)
    st, v, f, vir = orc.forces(r, s["box"], s["z"], 2)
    st2, v2, f2, vir2 = orc.forces(r + np.array([0.31, -0.77, 1.13]), s["box"], s["z"], 2)
    assert st == 0 and st2 == 0
    assert abs(v2 - v) <= 1e-11 * abs(v)
    assert np.linalg.norm(f2 - f) <= 1e-10 * np.linalg.norm(f)
    assert np.linalg.norm(vir2 - vir) <= 1e-10 * np.linalg.norm(vir)
