"""Mixed-precision device path (GB_PREC_MIXED) against the plain-FP64 device path.

The mixed path computes pair, reciprocal-space and normal-mode arithmetic in
FP32 with compensated sums and keeps energies, virials, k-space totals and the
propagator in FP64.  Bound checked here: relative RMS force error
||F_mixed - F_fp64|| / ||F_fp64|| <= 1e-5 over all beads and atoms, for the
low-frequency (Ewald + LJ) forces and for the total force; energies within
1e-5 relative, virial tensors within 1e-5 relative (Frobenius norm).  (Measured
on these snapshots: forces 2e-7 to 1e-6, energies 1e-6 to 3e-6, virials 2e-7
to 1.2e-6.)
"""
import numpy as np
import pytest

from rpmd_mainz_gb300 import lib

from . import systems

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5
ENERGY_TOL = 1e-5
VIRIAL_TOL = 1e-5


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    yield
    lib.finalize()


def both(s, fn):
    out = []
    for prec in (0, 1):
        p = s["params"]
        p.precision = prec
        lib.init(p)
        out.append(fn())
    s["params"].precision = 0
    lib.init(s["params"])
    return out


CASES = [
    # 216 H2O, nb = 8, Ewald and LJ on every bead
    dict(param="param_qspcfw", ncell=(6, 6, 6), nb=8),
    # 4096 H2O, nb = 4, Ewald on the centroid, LJ on 3 modes (centroid list)
    dict(param="param_qspcfw", ncell=(16, 16, 16), nb=4, mts=5, dtfs=1.25, nbdf1=1, nbdf2=3),
]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("seed", [1, 2])
def test_mixed_full_forces_error(case, seed):
    s = systems.build(**case)
    r = systems.perturbed(s, seed=100 + seed)
    f64, fmx = both(s, lambda: lib.full_forces(r, s["box"], s["z"]))
    e_lf = rel(fmx["dvdr"], f64["dvdr"])
    e_tot = rel(fmx["dvdr"] + fmx["dvdr2"], f64["dvdr"] + f64["dvdr2"])
    assert e_lf < FORCE_TOL, e_lf
    assert e_tot < FORCE_TOL, e_tot
    for k in ("v", "vew", "voo"):
        assert abs(fmx[k] - f64[k]) <= ENERGY_TOL * abs(f64[k]) + 1e-12, (k, fmx[k], f64[k])
    assert rel(fmx["vir"], f64["vir"]) < VIRIAL_TOL


@pytest.mark.parametrize("iopt", [0, 1, 2])
def test_mixed_forces_iopt(iopt):
    s = systems.build(param="param_qspcfw", ncell=(5, 5, 5), nb=4)
    r = systems.perturbed(s, seed=120 + iopt)
    (v64, f64, vir64), (vmx, fmx, virmx) = both(s, lambda: lib.forces(r, s["box"], s["z"], iopt))
    assert rel(fmx, f64) < FORCE_TOL
    assert abs(vmx - v64) <= ENERGY_TOL * abs(v64)
    assert rel(virmx, vir64) < VIRIAL_TOL


EVOLVE_CASES = [
    dict(param="param_qspcfw", ncell=(6, 6, 6), nb=32, mts=1, dtfs=0.5),  # every bead, fused nb = 32
    dict(param="param_qspcfw", ncell=(8, 8, 8), nb=16, mts=5, dtfs=1.25, nbdf1=1, nbdf2=5),  # contracted, MTS
]


@pytest.mark.parametrize("case", EVOLVE_CASES)
def test_mixed_evolve_tracks_fp64(case):
    """Ten evolve_pi steps in mixed precision stay within 1e-6 (positions) and
    1e-5 (momenta, forces) relative of the plain-FP64 trajectory."""
    s = systems.build(**case)
    r = systems.perturbed(s, seed=130)
    rng = np.random.default_rng(131)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] / (s["beta"] / s["nb"]))
    out = []
    for prec in (0, 1):
        prm = s["params"]
        prm.precision = prec
        lib.init(prm)
        ff = lib.full_forces(r, s["box"], s["z"])
        ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
        ctx.upload(r=r, p=p, dvdr=ff["dvdr"], dvdr2=ff["dvdr2"], box=s["box"])
        ctx.evolve(10, s["dt"], s["beta"])
        ctx.sync()
        out.append((ctx.download(), ctx.energies()))
        ctx.close()
    s["params"].precision = 0
    lib.init(s["params"])
    (r0, p0, f0, g0), e0 = out[0]
    (r1, p1, f1, g1), e1 = out[1]
    assert rel(r1, r0) < 1e-6
    assert rel(p1, p0) < 1e-5
    assert rel(f1, f0) < 1e-5
    assert rel(g1, g0) < 1e-5
    for k in ("v", "vew", "vlj", "vint", "tv"):
        assert abs(e1[k] - e0[k]) <= 1e-5 * abs(e0[k]) + 1e-9, (k, e1[k], e0[k])


def test_mixed_coordinate_just_below_box_edge():
    """A coordinate a hair below a box edge rounds to 1.0f in FP32; its hi/lo
    split must still name the same periodic point (regression case)."""
    s = systems.build(param="param_qspcfw", ncell=(6, 6, 6), nb=4)
    r = systems.perturbed(s, seed=140)
    # rigid translations (no change to the physics) that put bead 0 of three
    # oxygens at -1e-9 box lengths, one per axis
    for mol, d in ((0, 0), (5, 1), (17, 2)):
        r[:, :, d] += -1e-9 * s["box"][d] - r[0, 3 * mol, d]
    f64, fmx = both(s, lambda: lib.full_forces(r, s["box"], s["z"]))
    assert rel(fmx["dvdr"], f64["dvdr"]) < FORCE_TOL
    assert rel(fmx["dvdr"] + fmx["dvdr2"], f64["dvdr"] + f64["dvdr2"]) < FORCE_TOL


def test_mixed_structure_factors_on_tensor_cores(monkeypatch):
    """GBRPMD_SK_TC=1: the k-space structure factors as split-TF32 mma.sync
    products (k_recip_tc.cu) keep the mixed path's force and energy bounds and
    agree with the CUDA-core structure factors."""
    s = systems.build(param="param_qspcfw", ncell=(6, 6, 6), nb=8)
    r = systems.perturbed(s, seed=131)
    f64, fcc = both(s, lambda: lib.full_forces(r, s["box"], s["z"]))
    monkeypatch.setenv("GBRPMD_SK_TC", "1")
    _, ftc = both(s, lambda: lib.full_forces(r, s["box"], s["z"]))
    monkeypatch.delenv("GBRPMD_SK_TC")
    assert rel(ftc["dvdr"], f64["dvdr"]) < FORCE_TOL
    assert rel(ftc["dvdr"], fcc["dvdr"]) < FORCE_TOL
    for k in ("v", "vew"):
        assert abs(ftc[k] - f64[k]) <= ENERGY_TOL * abs(f64[k]) + 1e-12, (k, ftc[k], f64[k])
    assert rel(ftc["vir"], f64["vir"]) < VIRIAL_TOL


@pytest.mark.parametrize("case", [
    dict(param="param_qspcfw", ncell=(6, 6, 6), nb=8),
    dict(param="param_qspcfw", ncell=(8, 8, 8), nb=16, mts=1, dtfs=0.5),
])
def test_shared_centroid_list_matches_per_bead_lists(monkeypatch, case):
    """Mixed real space of several beads walks one list built on the site
    centroids (radius widened by twice the bead spread, the cut-off tested per
    bead): forces, energies and virial equal those of per-bead lists
    (GBRPMD_EW_SHARED=0) to FP32 summation order, over steps with rebuilds."""
    s = systems.build(**case)
    r = systems.perturbed(s, seed=141)
    out = []
    for shared in ("1", "0"):
        monkeypatch.setenv("GBRPMD_EW_SHARED", shared)
        p = s["params"]
        p.precision = 1
        lib.init(p)
        ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
        ctx.set_params(p)
        ctx.upload(r=r, box=s["box"])
        en = ctx.full_forces()
        f0 = ctx.download()[2]
        ctx.evolve(30, s["dt"], s["beta"])
        rr, pp, f1, f2 = ctx.download()
        out.append((en, f0, rr, pp, f1, ctx.list_rebuilds()))
        ctx.close()
    monkeypatch.delenv("GBRPMD_EW_SHARED")
    s["params"].precision = 0
    lib.init(s["params"])
    (ea, f0a, ra, pa, fa, nra), (eb, f0b, rb, pb, fb, nrb) = out
    assert rel(f0a, f0b) < 1e-6
    assert abs(ea["vew"] - eb["vew"]) <= 1e-6 * abs(eb["vew"])
    assert rel(ea["vir"], eb["vir"]) < 1e-6
    # 30 steps later: the FP32 summation-order differences, amplified by the
    # dynamics (a missed pair would show in the forces above at once)
    assert rel(ra, rb) < 1e-7 and rel(pa, pb) < 1e-4 and rel(fa, fb) < 1e-4, (rel(ra, rb), rel(pa, pb), rel(fa, fb))
    assert nra[0] >= 1  # the shared list was built (and rebuilt) on the device


@pytest.mark.parametrize("case", [
    dict(param="param_qspcfw", ncell=(6, 6, 6), nb=8),
    dict(param="param_qspcfw", ncell=(16, 16, 16), nb=4, mts=5, dtfs=1.25, nbdf1=1, nbdf2=3),
])
def test_mixed_force_pass_on_tensor_cores(monkeypatch, case):
    """The k-space force pass as split-TF32 mma.sync products (k_recip_tc.cu,
    the default) keeps the mixed path's bounds and agrees with the CUDA-core
    force pass (GBRPMD_RF_TC=0)."""
    s = systems.build(**case)
    r = systems.perturbed(s, seed=151)
    f64, ftc = both(s, lambda: lib.full_forces(r, s["box"], s["z"]))
    monkeypatch.setenv("GBRPMD_RF_TC", "0")
    _, fcc = both(s, lambda: lib.full_forces(r, s["box"], s["z"]))
    monkeypatch.delenv("GBRPMD_RF_TC")
    assert rel(ftc["dvdr"], f64["dvdr"]) < FORCE_TOL
    assert rel(ftc["dvdr"], fcc["dvdr"]) < FORCE_TOL
    for k in ("v", "vew"):
        assert abs(ftc[k] - f64[k]) <= ENERGY_TOL * abs(f64[k]) + 1e-12, (k, ftc[k], f64[k])
