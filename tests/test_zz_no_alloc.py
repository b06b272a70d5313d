"""gbrpmd_forces_ewald_static: the Ewald entry point for callers that cannot
let the library allocate device memory (a host whose device memory is handed
out by another framework's pool, or code that must not cudaMalloc/cudaFree
while its streams run).  It works in a fixed 16 MiB array reserved at load
time and always computes in FP64.  Checked against gbrpmd_forces (iopt = 2,
FP64) on two calls in a row, at the tolerance of the other device tests (1e-10
relative), on a small box and on 216 molecules at nb = 8 (about 9 MiB of the
array); sizes beyond its limit are refused before any device work, and a
crowded configuration (more partners per site than the list slots) returns
GB_E_LIST.  Collected last (file name) so that a run stopping at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from rpmd_mainz_gb300 import lib, system
from rpmd_mainz_gb300.abi import GB_E_LIST, GB_E_NOMEM

pytestmark = pytest.mark.gpu

PARAM = "tests/golden/params/param_qspcfw"
TOL = 1e-10


def static_forces(r, box, z):
    L = lib.load()
    r = np.ascontiguousarray(r, dtype=np.float64)
    nb, na, _ = r.shape
    dvdr = np.zeros_like(r)
    vir = np.zeros(9)
    v = C.c_double()
    st = L.gbrpmd_forces_ewald_static(lib._ptr(r), C.byref(v), lib._ptr(dvdr), C.byref(C.c_int(nb)),
                                      C.byref(C.c_int(na)), lib._ptr(np.ascontiguousarray(box, dtype=np.float64)),
                                      lib._ptr(np.ascontiguousarray(z, dtype=np.float64)), lib._ptr(vir))
    return st, v.value, dvdr, vir


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()


@pytest.mark.parametrize("ncell, nb", [((4, 4, 4), 4), ((6, 6, 6), 8)])
def test_static_ewald_matches_forces_twice(ncell, nb):
    s = system.water_box(PARAM, ncell=ncell, nb=nb)
    lib.init(s["params"])
    rng = np.random.default_rng(7)
    for call in range(2):
        r = s["r"] + rng.uniform(-0.1, 0.1, size=s["r"].shape)
        st, v, f, vir = static_forces(r, s["box"], s["z"])
        assert st == 0, lib.load().gbrpmd_last_error().decode()
        v0, f0, vir0 = lib.forces(r, s["box"], s["z"], 2)
        assert rel(f, f0) < TOL, call
        assert abs(v - v0) <= TOL * abs(v0), call
        assert rel(vir, vir0.reshape(-1, order="F")) < TOL, call


def test_static_ewald_refuses_oversize():
    s = system.water_box(PARAM, ncell=(6, 6, 6), nb=16)  # 648 * 16 sites > 8192
    lib.init(s["params"])
    st, _, _, _ = static_forces(s["r"], s["box"], s["z"])
    assert st == GB_E_NOMEM
    assert "8192" in lib.load().gbrpmd_last_error().decode()


def test_static_ewald_reports_crowded_lists():
    s = system.water_box(PARAM, ncell=(6, 6, 6), nb=1)
    lib.init(s["params"])
    nm = s["nm"]
    mol = s["r"].reshape(1, nm, 3, 3)
    crowded = (mol - 0.75 * mol[:, :, :1, :]).reshape(s["r"].shape)  # 64 times the density
    st, _, _, _ = static_forces(crowded, s["box"], s["z"])
    assert st == GB_E_LIST
    assert "partners" in lib.load().gbrpmd_last_error().decode()
    st, v, f, vir = static_forces(s["r"], s["box"], s["z"])  # the next call is unaffected
    assert st == 0
    v0, f0, _ = lib.forces(s["r"], s["box"], s["z"], 2)
    assert abs(v - v0) <= TOL * abs(v0)
