"""Device parts with no counterpart in the reference, each checked against a
plain alternative of the library itself or against the host's IEEE arithmetic:

* the integer-built FP64 <-> FP32 conversions of the mixed kernels
  (gbrpmd_selftest_conversions) against numpy's conversions;
* cell-sorted skin-list rebuilds against the tiled all-pairs build
  (GBRPMD_LIST_CELLS=0) on a box large enough for cells, over steps with
  rebuilds;
* the LJ term and the k-space kernels on forked streams against the same step
  with every kernel on the step's stream (GBRPMD_BRANCHES=0).
"""
import ctypes as C
import os

import numpy as np
import pytest

from rpmd_mainz_gb300 import lib

from . import systems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    yield
    lib.finalize()


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def test_conversions_match_ieee():
    rng = np.random.default_rng(7)
    mags = 10.0 ** rng.uniform(-30, 30, size=200000)
    x = rng.normal(size=mags.size) * mags
    # differences of FP32 values: exact ties at the FP32 rounding bit are common
    a = rng.normal(size=50000).astype(np.float32).astype(np.float64)
    b = (rng.normal(size=50000) * 3).astype(np.float32).astype(np.float64)
    edge = np.array([0.0, -0.0, 1.0, -1.0, 2.0 ** -126, -(2.0 ** -126), 2.0 ** -127, 3.4e38, -3.4e38,
                     np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0)])
    x = np.concatenate([x, a - b, a + b, edge])
    n = x.size
    f32 = np.zeros(n, np.float32)
    hi = np.zeros(n, np.float32)
    lo = np.zeros(n, np.float32)
    back = np.zeros(n)
    rc = lib.load().gbrpmd_selftest_conversions(_p(x, C.c_double), n, _p(f32, C.c_float), _p(hi, C.c_float),
                                                _p(lo, C.c_float), _p(back, C.c_double))
    assert rc == 0, lib.load().gbrpmd_last_error()
    normal = (np.abs(x) >= 2.0 ** -126) & (np.abs(x) < 3.4e38)
    # round to nearest, ties to even, where the result is a normal float
    ref = x.astype(np.float32)
    ok = normal & (np.abs(ref) >= np.float32(2.0 ** -126)) & np.isfinite(ref)
    assert np.array_equal(f32[ok], ref[ok])
    # the split: hi truncated, hi + lo within 2^-46 of x (lo flushes to zero
    # below 2^-75, where the weight of its last bit leaves the FP32 range)
    assert np.all(np.abs(hi[normal].astype(np.float64)) <= np.abs(x[normal]))
    sp = normal & (np.abs(x) >= 2.0 ** -74)
    err = np.abs(hi[sp].astype(np.float64) + lo[sp].astype(np.float64) - x[sp])
    assert np.all(err <= 2.0 ** -46 * np.abs(x[sp]))
    # the widening is exact
    assert np.array_equal(back[ok], f32[ok].astype(np.float64))
    # below the normal range: signed zeros
    tiny = (np.abs(x) < 2.0 ** -126)
    assert np.all(f32[tiny & (np.abs(x) < 2.0 ** -127)] == 0.0)
    assert np.all(hi[tiny] == 0.0) and np.all(lo[tiny] == 0.0)


def _run(env, case, seed, nsteps, precision):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        s = systems.build(**case, precision=precision)
        lib.init(s["params"])
        r = systems.perturbed(s, seed=seed)
        rng = np.random.default_rng(seed + 1)
        p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] / (s["beta"] / s["nb"]))
        ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
        try:
            ctx.upload(r=r, p=p, box=s["box"])
            ctx.full_forces()
            ctx.evolve(nsteps, s["dt"], s["beta"])
            ctx.sync()
            return ctx.download(), ctx.energies(), ctx.list_rebuilds()
        finally:
            ctx.close()
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def test_cell_sorted_lists_match_all_pairs():
    # 4096 H2O, nb = 2: Ewald and LJ lists on both beads, boxes wide enough
    # for the cell grid; 2 fs steps move the atoms past the skin several times
    case = dict(param="param_qspcfw", ncell=(16, 16, 16), nb=2, mts=1, dtfs=2.0)
    (r0, p0, f0, g0), e0, n0 = _run({"GBRPMD_LIST_CELLS": "0"}, case, 150, 30, 0)
    (r1, p1, f1, g1), e1, n1 = _run({"GBRPMD_LIST_CELLS": "1"}, case, 150, 30, 0)
    assert n1[0] >= 2 and n1 == n0, (n0, n1)  # rebuilds happened, at the same steps
    assert rel(r1, r0) < 1e-12
    assert rel(p1, p0) < 1e-10
    assert rel(f1, f0) < 1e-10
    for k in ("v", "vew", "vlj", "vint"):
        assert abs(e1[k] - e0[k]) <= 1e-11 * abs(e0[k]), (k, e1[k], e0[k])


@pytest.mark.parametrize("precision", [0, 1])
def test_branches_match_one_stream(precision):
    # contracted rings: the LJ term (5 modes) and, in mixed precision, the
    # k-space kernels run on forked streams
    case = dict(param="param_qspcfw", ncell=(8, 8, 8), nb=16, mts=5, dtfs=1.25, nbdf1=1, nbdf2=5)
    (r0, p0, f0, g0), e0, _ = _run({"GBRPMD_BRANCHES": "0"}, case, 160, 10, precision)
    (r1, p1, f1, g1), e1, _ = _run({"GBRPMD_BRANCHES": "1"}, case, 160, 10, precision)
    # FP64: sums in another order only; mixed: FP32 sums over lists whose
    # order is not deterministic either way
    tol = 1e-11 if precision == 0 else 1e-6
    assert rel(r1, r0) < tol
    assert rel(p1, p0) < 10 * tol
    assert rel(f1, f0) < 10 * tol
    for k in ("v", "vew", "vlj", "vint"):
        assert abs(e1[k] - e0[k]) <= 10 * tol * abs(e0[k]) + 1e-12, (k, e1[k], e0[k])
