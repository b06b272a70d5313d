"""ctypes bindings of the oracle library (oracle/_build/liborc.so) for tests.

The oracle is the CPU FP64 restatement of the reference path; the tests use
it only as the checker.  `load()` builds the library with make if needed.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from rpmd_mainz_gb300.abi import GbParams

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liborc.so")

# globals.inc constants
TOA = 0.5291772108
TOFS = 41.341373
KBOLTZ_MAIN = 3.166829e-6  # main.f90:168 literal
TOKJMOL = 2625.49963  # globals.inc:18
TOBAR = 2.9421e+8  # globals.inc:19

_lib = None

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)


def _ptr(a, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype))


def load():
    global _lib
    if _lib is not None:
        return _lib
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    lib = C.CDLL(LIB_PATH)
    lib.orc_ran2.restype = C.c_double
    lib.orc_gaussian.restype = C.c_double
    lib.orc_bench_replicas.restype = C.c_double
    lib.orc_pressure.restype = C.c_double
    assert lib.orc_params_size() == C.sizeof(GbParams), "gb_params layout mismatch"
    _lib = lib
    return lib


def set_params(p: GbParams):
    load().orc_set_params(C.byref(p))


def get_params() -> GbParams:
    p = GbParams()
    load().orc_get_params(C.byref(p))
    return p


class Rng:
    """Saved state of ran2/gaussian (random.f90)."""

    def __init__(self, seed):
        lib = load()
        self.buf = (C.c_char * lib.orc_rng_size())()
        lib.orc_rng_reset(self.buf)
        self.irun = C.c_int(-abs(int(seed)))

    def ran2(self, rmin=0.0, rmax=1.0):
        return load().orc_ran2(self.buf, C.byref(self.irun), C.c_double(rmin), C.c_double(rmax))

    def gaussian(self, sigma=1.0):
        return load().orc_gaussian(self.buf, C.byref(self.irun), C.c_double(sigma))


def realft(data, mode, direct=False):
    """data: array (n, m) in bead-major order, i.e. Fortran data(m, n)."""
    a = np.ascontiguousarray(data, dtype=np.float64).copy()
    n, m = a.shape
    fn = load().orc_realft_direct if direct else load().orc_realft
    fn(_ptr(a), C.c_int(m), C.c_int(n), C.c_int(mode))
    return a


def setup_box_size_cub(ncell, rho, wmass):
    box = np.zeros(3)
    nc = np.array(ncell, dtype=np.int32)
    nm = load().orc_setup_box_size_cub(_ptr(nc, C.c_int), C.c_double(rho), C.c_double(wmass), _ptr(box))
    return nm, box


def cubic(nm, box, ncell):
    r = np.zeros((nm * 3, 3))
    nc = np.array(ncell, dtype=np.int32)
    st = load().orc_cubic(_ptr(r), C.c_int(nm), _ptr(np.asarray(box, float)), _ptr(nc, C.c_int))
    assert st == 0
    return r


def setup_ewald(na, box):
    load().orc_setup_ewald(C.c_int(na), _ptr(np.asarray(box, dtype=np.float64)))


def forces(r, box, z, iopt):
    """r: (nb, na, 3). Returns v, dvdr (nb, na, 3), virial (3,3) column-major -> [i, j]."""
    r = np.ascontiguousarray(r, dtype=np.float64).copy()
    nb, na, _ = r.shape
    dvdr = np.zeros_like(r)
    vir = np.zeros(9)
    v = C.c_double(0.0)
    st = load().orc_forces(_ptr(r), C.byref(v), _ptr(dvdr), C.c_int(nb), C.c_int(na),
                           _ptr(np.asarray(box, float)), _ptr(np.asarray(z, float)), _ptr(vir), C.c_int(iopt))
    return st, v.value, dvdr, vir.reshape(3, 3, order="F")


def full_forces(r, box, z):
    r = np.ascontiguousarray(r, dtype=np.float64).copy()
    nb, na, _ = r.shape
    dvdr = np.zeros_like(r)
    dvdr2 = np.zeros_like(r)
    vir = np.zeros(9)
    v, vew, voo, vint = (C.c_double(0.0) for _ in range(4))
    st = load().orc_full_forces(_ptr(r), C.c_int(na), C.c_int(nb), C.byref(v), C.byref(vew), C.byref(voo),
                                C.byref(vint), _ptr(vir), _ptr(np.asarray(z, float)),
                                _ptr(np.asarray(box, float)), _ptr(dvdr), _ptr(dvdr2))
    return dict(status=st, v=v.value, vew=vew.value, voo=voo.value, vint=vint.value, dvdr=dvdr, dvdr2=dvdr2,
                vir=vir.reshape(3, 3, order="F"), r=r)


class State:
    """Mutable trajectory state in the reference layout (nb, na, 3)."""

    def __init__(self, r, p, dvdr, dvdr2, box):
        self.r = np.ascontiguousarray(r, dtype=np.float64).copy()
        self.p = np.ascontiguousarray(p, dtype=np.float64).copy()
        self.dvdr = np.ascontiguousarray(dvdr, dtype=np.float64).copy()
        self.dvdr2 = np.ascontiguousarray(dvdr2, dtype=np.float64).copy()
        self.box = np.array(box, dtype=np.float64)
        self.vir = np.zeros(9)
        self.vir_lf = np.zeros(9)

    def copy(self):
        s = State(self.r, self.p, self.dvdr, self.dvdr2, self.box)
        s.vir = self.vir.copy()
        s.vir_lf = self.vir_lf.copy()
        return s


def evolve_pi(state: State, dt, mass, z, beta, rng: Rng, nbaro=0):
    nb, na, _ = state.r.shape
    v, vew, vlj, vint, tv = (C.c_double(0.0) for _ in range(5))
    st = load().orc_evolve_pi(_ptr(state.p), _ptr(state.r), C.byref(v), C.byref(vew), C.byref(vlj),
                              C.byref(vint), _ptr(state.dvdr), _ptr(state.dvdr2), C.c_double(dt),
                              _ptr(np.asarray(mass, float)), C.c_int(na), C.c_int(nb), _ptr(state.box),
                              _ptr(np.asarray(z, float)), C.c_double(beta), _ptr(state.vir),
                              _ptr(state.vir_lf), rng.buf, C.byref(rng.irun), C.c_int(nbaro), C.byref(tv))
    return dict(status=st, v=v.value, vew=vew.value, vlj=vlj.value, vint=vint.value, tv=tv.value)


def run_steps(state: State, dt, mass, z, beta, nsteps, thresh, rng: Rng):
    nb, na, _ = state.r.shape
    en = np.zeros((nsteps, 4))
    st = load().orc_run_steps(_ptr(state.p), _ptr(state.r), _ptr(state.dvdr), _ptr(state.dvdr2), C.c_double(dt),
                              _ptr(np.asarray(mass, float)), C.c_int(na), C.c_int(nb), _ptr(state.box),
                              _ptr(np.asarray(z, float)), C.c_double(beta), C.c_int(nsteps), C.c_double(thresh),
                              rng.buf, C.byref(rng.irun), _ptr(state.vir_lf), _ptr(en))
    return st, en


def md_eq(state: State, dt, mass, z, beta, ne, npt, rng: Rng, npre_eq=0, ttaufs=0.0):
    """md_eq's loops (orc md_eq); returns (status, pre[nq, 5], eq[ne, 12])."""
    nb, na, _ = state.r.shape
    nq = (npre_eq or min(20000, ne // 10)) if npt else 0
    pre, eq = np.zeros((max(nq, 1), 5)), np.zeros((ne, 12))
    st = load().orc_md_eq(_ptr(state.p), _ptr(state.r), _ptr(state.dvdr), _ptr(state.dvdr2), C.c_double(dt),
                          _ptr(np.asarray(mass, float)), C.c_int(na), C.c_int(nb), _ptr(state.box),
                          _ptr(np.asarray(z, float)), C.c_double(beta), C.c_int(ne), C.c_int(npre_eq),
                          C.c_int(1 if npt else 0), C.c_double(ttaufs), rng.buf, C.byref(rng.irun), _ptr(pre),
                          _ptr(eq))
    return st, pre[:nq], eq


def sample_rpmd(na, nb, mass, beta, rng: Rng):
    p = np.zeros((nb, na, 3))
    load().orc_sample_rpmd(_ptr(p), C.c_int(na), C.c_int(nb), _ptr(np.asarray(mass, float)), C.c_double(beta),
                           rng.buf, C.byref(rng.irun))
    return p


def virial_ke(r, dvdr, dvdr2, beta):
    nb, na, _ = r.shape
    tv, tq1, tq2 = C.c_double(), C.c_double(), C.c_double()
    tvxyz = np.zeros(3)
    load().orc_virial_ke(_ptr(np.ascontiguousarray(r)), _ptr(np.ascontiguousarray(dvdr)),
                         _ptr(np.ascontiguousarray(dvdr2)), C.byref(tv), _ptr(tvxyz), C.byref(tq1), C.byref(tq2),
                         C.c_double(beta), C.c_int(na), C.c_int(nb))
    return tv.value, tvxyz, tq1.value, tq2.value


def pressure(vir, tv, na, box):
    """md_pressure.f90's isotropic pressure with the LJ tail (vir column-major 3x3)."""
    return load().orc_pressure(_ptr(np.ascontiguousarray(vir, float)), C.c_double(tv), C.c_int(na),
                               _ptr(np.ascontiguousarray(box, float)))


def beren_driver(vir, tv, tvxyz, dt, r, box):
    """beren_driver (module_barostat.f90:8-26) on r [nb][na][3] and box, both in place."""
    nb, na, _ = r.shape
    load().orc_beren_driver(_ptr(np.ascontiguousarray(vir, float)), C.c_double(tv),
                            _ptr(np.ascontiguousarray(tvxyz, float)), C.c_double(dt), _ptr(r), _ptr(box),
                            C.c_int(na), C.c_int(nb))


ESTIMATORS = ("tk", "vrp", "econs", "temp", "tv", "tvx", "tvy", "tvz", "pres", "dipx", "dipy", "dipz", "dip2",
              "dipm", "den", "v")


def estimators(r, p, dvdr, dvdr2, mass, z, beta, v, vir, box):
    """md_eq's output-step estimators (orc md_eq_estimators); vir column-major 3x3."""
    nb, na, _ = r.shape
    nm = na // 3
    out, rcm, mdip = np.zeros(16), np.zeros((nm, 3)), np.zeros((nm, 3))
    load().orc_md_eq_estimators(_ptr(np.ascontiguousarray(r)), _ptr(np.ascontiguousarray(p)),
                                _ptr(np.ascontiguousarray(dvdr)), _ptr(np.ascontiguousarray(dvdr2)),
                                _ptr(np.asarray(mass, float)), _ptr(np.asarray(z, float)), C.c_int(na), C.c_int(nb),
                                C.c_double(beta), C.c_double(v), _ptr(np.asfortranarray(vir).ravel(order="F").copy()),
                                _ptr(np.asarray(box, float)), _ptr(out), _ptr(rcm), _ptr(mdip))
    d = dict(zip(ESTIMATORS, out.tolist()))
    d["rcm"], d["mdip"] = rcm, mdip
    return d


def rattle_setup(nm):
    load().orc_rattle_setup(C.c_int(nm))


def evolve_rig_pi(state: State, dt, mass, z, beta, rng: Rng, nbaro=0):
    nb, na, _ = state.r.shape
    v, v_lf, v_hf = C.c_double(), C.c_double(), C.c_double()
    st = load().orc_evolve_rig_pi(_ptr(state.p), _ptr(state.r), C.byref(v), C.byref(v_lf), C.byref(v_hf),
                                  _ptr(state.dvdr), _ptr(state.dvdr2), C.c_double(dt), _ptr(np.asarray(mass, float)),
                                  C.c_int(na), C.c_int(nb), _ptr(state.box), _ptr(np.asarray(z, float)),
                                  C.c_double(beta), _ptr(state.vir), _ptr(state.vir_lf), rng.buf,
                                  C.byref(rng.irun), C.c_int(nbaro))
    return dict(status=st, v=v.value)


def bench_replicas(nthreads, state: State, dt, mass, z, beta, nsteps):
    nb, na, _ = state.r.shape
    return load().orc_bench_replicas(C.c_int(nthreads), _ptr(state.p), _ptr(state.r), _ptr(state.dvdr),
                                     _ptr(state.dvdr2), C.c_double(dt), _ptr(np.asarray(mass, float)),
                                     C.c_int(na), C.c_int(nb), _ptr(state.box), _ptr(np.asarray(z, float)),
                                     C.c_double(beta), C.c_int(nsteps))
