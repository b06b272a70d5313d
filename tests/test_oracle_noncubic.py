"""The oracle's non-cubic Ewald sum (ewald_noncubic.f90: rwald_basic /
rwald_cell + kwald_nc), which no reference test reaches.  It is pinned to the
cubic restatement, itself pinned to the reference's golden run: on a cubic box
with the same Ewald parameters in bohr, the two give the same energy, forces
and diagonal virial (the cubic reciprocal virial's off-diagonal entries use
|k_a||k_b|, ewald_cubic.f90:488-503, the non-cubic ones k_a k_b).  On a
genuinely non-cubic 8 x 4 x 4 box: forces against central differences of the
energy, and invariance under a rigid translation.

Likewise the per-axis Berendsen barostat (beren_baro_nc, module_barostat.f90:
28-86), which no reference test reaches either: under an isotropic virial and
equal axis shares of the kinetic energy it scales every axis as the isotropic
beren_baro (pinned through the reference's NPT equilibration) does; in general
the mean of its three axis pressures is the isotropic pressure, and each water
moves by its center_water vector times its axis's scale - 1."""
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


def _baro_system(ncell):
    s = systems.build(ncell=ncell, nb=4, therm="NON", baro="BER", taufs=200.0, mts=1)
    r = systems.perturbed(s, seed=9)
    st, v, f, vir = orc.forces(r, s["box"], s["z"], 2)
    assert st == 0
    tv, tvxyz, _, _ = orc.virial_ke(r, f, np.zeros_like(f), s["beta"])
    return s, r, vir.reshape(9, order="F"), tv, tvxyz


def _driver(s, iamcub, vir, tv, tvxyz, r):
    P = orc.get_params()
    P.iamcub = iamcub
    orc.set_params(P)
    rr, box = r.copy(), s["box"].copy()
    orc.beren_driver(vir, tv, tvxyz, s["dt"], rr, box)
    return rr, box


def test_noncubic_barostat_equals_isotropic_under_isotropic_stress():
    s, r, _, tv, _ = _baro_system((4, 4, 4))
    vir = np.diag([-0.3, -0.3, -0.3]).reshape(9)  # an isotropic virial, and tvxyz = tv / 3 on every axis
    tvxyz = np.full(3, tv / 3.0)
    rc, bc = _driver(s, 1, vir, tv, tvxyz, r)
    rn, bn = _driver(s, 0, vir, tv, tvxyz, r)
    assert abs(bc[0] - s["box"][0]) > 1e-9  # the box moved
    assert np.abs(bn - bc).max() <= 1e-14 * bc[0]
    assert np.abs(rn - rc).max() <= 1e-13 * np.abs(rc).max()


def test_noncubic_barostat_axis_pressures():
    s, r, vir, tv, tvxyz = _baro_system((8, 4, 4))
    assert abs(tvxyz.sum() - tv) <= 1e-12 * abs(tv)
    rn, bn = _driver(s, 0, vir, tv, tvxyz, r)
    P = orc.get_params()
    scale = bn / s["box"]
    assert np.ptp(scale) > 1e-9  # the axes scale differently
    # pres_j = patm - (1 - scale_j) / (dt bstat) (scale_j = |1 - dt bstat (patm - pres_j)|, here near 1)
    bstat = 13531.0 / (3.0 * P.taub)
    pres = P.patm - (1.0 - scale) / (s["dt"] * bstat)
    piso = orc.pressure(vir, tv, s["na"], s["box"])
    assert abs(pres.mean() - piso) <= 1e-9 * abs(piso)
    # each water on every bead moves by its bead-averaged atom sum (center_water) times scale_j - 1
    nb, na, _ = r.shape
    rcm = r.reshape(nb, na // 3, 3, 3).sum(axis=2).mean(axis=0)  # [nm][3]
    shift = np.repeat(rcm * (scale - 1.0), 3, axis=0)
    assert np.abs(rn - r - shift[None]).max() <= 1e-12 * np.abs(r).max()
