"""Error paths of the device code, reached by host-side inputs only (no GPU
fault, trap or hang is involved): every case makes a kernel record a status
bit that the host turns into the reference's `stop` message, and the next
ordinary call works again.

* GB_E_NONFINITE: a NaN coordinate in a drop-in intramolecular force call
  (forces iopt = 4: no pair list reads the positions);
* GB_E_CONTRACT: an even contraction count (evolve_pi.f90:344-347);
* GB_E_LIST: molecules crowded into one corner of the box, so that a site has
  more partners than the list capacity sized for liquid density holds
  (neigh_list.f90:63); the build kernels write no entry past the capacity;
* GB_E_RATTLE1 / GB_E_RATTLE2: the RATTLE sweep limit lowered to 1
  (md_rattle.f90:149, 258).
"""
import ctypes as C

import numpy as np
import pytest

from rpmd_mainz_gb300 import lib
from rpmd_mainz_gb300.abi import GB_E_CONTRACT, GB_E_LIST, GB_E_NONFINITE, GB_E_RATTLE1, GB_E_RATTLE2

from . import oracle_lib as orc
from . import systems

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    yield
    lib.finalize()


def check_forces_vs_oracle(s, r, iopt):
    st, v, f, vir = orc.forces(r, s["box"], s["z"], iopt)
    assert st == 0
    vd, fd, vird = lib.forces(r, s["box"], s["z"], iopt)
    assert rel(fd, f) < TOL
    assert abs(vd - v) <= TOL * abs(v)


def test_nonfinite_force_is_reported():
    s = systems.build(param="param_qspcfw", ncell=(4, 4, 4), nb=2)
    lib.init(s["params"])
    r = systems.perturbed(s, seed=1)
    bad = r.copy()
    bad[1, 7, 2] = np.nan
    with pytest.raises(lib.GbError) as e:
        lib.forces(bad, s["box"], s["z"], 4)
    assert e.value.code == GB_E_NONFINITE
    assert "non-finite" in lib.last_error()
    check_forces_vs_oracle(s, r, 4)


def test_even_contraction_is_reported():
    s = systems.build(param="param_qspcfw", ncell=(4, 4, 4), nb=8, nbdf1=2, nbdf2=3)
    lib.init(s["params"])
    r = systems.perturbed(s, seed=2)
    with pytest.raises(lib.GbError) as e:
        lib.full_forces(r, s["box"], s["z"])
    assert e.value.code == GB_E_CONTRACT
    assert "ODD" in lib.last_error()


def test_list_overflow_is_reported():
    s = systems.build(param="param_qspcfw", ncell=(12, 12, 12), nb=1)
    lib.init(s["params"])
    r = systems.perturbed(s, seed=3, bead_spread=0.0)
    # molecules moved halfway to the box corner: eight times the density, about
    # four times the partners per site that a list sized for the liquid holds
    nm = s["nm"]
    mol = r.reshape(1, nm, 3, 3)
    shift = 0.5 * mol[:, :, :1, :]
    crowded = (mol - shift).reshape(r.shape)
    with pytest.raises(lib.GbError) as e:
        lib.forces(crowded, s["box"], s["z"], 2)
    assert e.value.code == GB_E_LIST
    # the lists are rebuilt at the next call
    check_forces_vs_oracle(s, r, 2)


def test_rattle_iteration_limit_is_reported():
    s = systems.build(param="param_tip05_rigid", ncell=(4, 4, 4), nb=1)
    lib.init(s["params"])
    lib.rattle_setup(s["nm"])
    rng = np.random.default_rng(60)
    r0 = s["r"][0].copy()
    rold = r0.copy()
    r = r0 + rng.normal(scale=0.01, size=r0.shape)
    p = rng.normal(scale=5.0, size=r0.shape)
    f = rng.normal(scale=0.01, size=r0.shape)
    dt = 20.0
    L = lib.load()
    try:
        assert L.gbrpmd_rattle_set_itmax(C.byref(C.c_int(1))) == 0
        with pytest.raises(lib.GbError) as e:
            lib.rattle_s1(r.copy(), rold, p.copy(), s["mass"], dt, f.copy())
        assert e.value.code == GB_E_RATTLE1
        with pytest.raises(lib.GbError) as e:
            lib.rattle_s2(r0.copy(), p.copy(), s["mass"], dt, f.copy())
        assert e.value.code == GB_E_RATTLE2
    finally:
        assert L.gbrpmd_rattle_set_itmax(C.byref(C.c_int(1000))) == 0
    rd, pd, fd = r.copy(), p.copy(), f.copy()
    lib.rattle_s1(rd, rold, pd, s["mass"], dt, fd)  # converges again
