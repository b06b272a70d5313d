"""md_eq's output-step estimators on the device (gbrpmd_ctx_estimators) against
the oracle's restatement (kinetic.f90, md_eq.f90:252-277, md_pressure.f90,
md_tools.f90 dipole / center_water) on the same resident state, and against the
values the reference printed for its own equilibrated restart file.

Tolerance: 1e-12 relative per estimator (FP64 sums in a different order),
1e-12 relative (L2) for the per-molecule centroid and dipole arrays.
"""
import numpy as np
import pytest

from rpmd_mainz_gb300 import lib

from . import oracle_lib as orc
from . import systems

pytestmark = pytest.mark.gpu

TOL = 1e-12
SCALARS = ("tk", "vrp", "econs", "temp", "tv", "tvx", "tvy", "tvz", "pres", "dipx", "dipy", "dipz", "dip2", "dipm",
           "den", "v")


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    yield
    lib.finalize()


def check(dev, ref, scale):
    for k in SCALARS:
        # dipole components of a near-neutral box can be small: measured against the dipole length
        den = max(abs(ref[k]), scale.get(k, 0.0), 1e-300)
        assert abs(dev[k] - ref[k]) <= TOL * den, (k, dev[k], ref[k])
    for k in ("rcm", "mdip"):
        assert np.linalg.norm(dev[k] - ref[k]) <= TOL * np.linalg.norm(ref[k]), k


def oracle_on(ctx, s, beta):
    r, p, dvdr, dvdr2 = ctx.download()
    e = ctx.energies()
    return orc.estimators(r, p, dvdr, dvdr2, s["mass"], s["z"], beta, e["v"], e["vir"], s["box"])


@pytest.mark.parametrize("case", [dict(ncell=(6, 6, 6), nb=8), dict(ncell=(4, 4, 4), nb=32, mts=5, dtfs=1.25,
                                                                     nbdf1=1, nbdf2=3)])
def test_estimators_match_oracle(case):
    s = systems.build(param="param_qspcfw", **case)
    lib.init(s["params"])
    r = systems.perturbed(s, seed=5)
    p = orc.sample_rpmd(s["na"], s["nb"], s["mass"], s["beta"], orc.Rng(77))
    ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
    try:
        ctx.upload(r=r, p=p, dvdr=np.zeros_like(r), dvdr2=np.zeros_like(r), box=s["box"])
        ctx.full_forces()
        for _ in range(2):  # after full_forces, then after evolve steps on the resident state
            dev = ctx.estimators(s["beta"], centroids=True, dipoles=True)
            ref = oracle_on(ctx, s, s["beta"])
            check(dev, ref, {k: np.sqrt(ref["dip2"]) for k in ("dipx", "dipy", "dipz")})
            ctx.evolve(4, s["dt"], s["beta"])
            ctx.sync()
    finally:
        ctx.close()


def test_estimators_at_reference_restart():
    # tests/golden/gentest_eq.npz: eq.xyz and the estimator lines the
    # reference printed for the same step (E_eq.out, V_eq.out, virial_ke_eq.out)
    from .test_oracle_golden import EQ, gentest_system

    s = gentest_system()
    lib.init(s["params"])
    r, box = EQ["r"], EQ["box"]
    na, nm, nb = s["na"], s["nm"], s["nb"]
    ctx = lib.Context(na, nb, s["mass"], s["z"])
    try:
        ctx.upload(r=r, p=np.zeros_like(r), dvdr=np.zeros_like(r), dvdr2=np.zeros_like(r), box=box)
        ctx.full_forces()
        est = ctx.estimators(s["beta"])
    finally:
        ctx.close()
    E, V, TV = EQ["E_eq"], EQ["V_eq"], EQ["virial_ke_eq"]
    assert abs(est["vrp"] / na - E[2]) <= 5e-9
    assert abs(nb * est["v"] / na - E[3]) <= 5e-9
    assert abs(est["v"] - V[1]) <= 5e-7
    assert abs(orc.TOKJMOL * est["tv"] / nm - TV[1]) <= 1e-12 * abs(TV[1])


def test_mixed_conserved_energy_tracks_fp64():
    # NVE (no thermostat), 216 H2O, nb = 8, dt 0.5 fs: the conserved RPMD
    # energy nb*v + tk + vrp of the mixed path stays with the FP64 path's over
    # 400 steps (both trajectories start from the same state); bound 2e-6 of
    # the conserved energy.  Before the normal-mode transforms of the state
    # used split twiddle tables, the FP32 round trip shrank the bead deviations
    # by a fixed ~3e-8 per step and the difference grew linearly to 2e-5.
    s = systems.build(param="param_qspcfw", ncell=(6, 6, 6), nb=8, therm="NON")
    r = systems.perturbed(s, seed=9)
    p = orc.sample_rpmd(s["na"], s["nb"], s["mass"], s["beta"], orc.Rng(21))
    series = {}
    for prec in (0, 1):
        prm = s["params"].copy()
        prm.precision = prec
        lib.init(prm)
        ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
        try:
            ctx.set_params(prm)
            ctx.upload(r=r, p=p, box=s["box"])
            ctx.full_forces()
            e = [ctx.estimators(s["beta"])["econs"]]
            for _ in range(8):
                ctx.evolve(50, s["dt"], s["beta"])
                e.append(ctx.estimators(s["beta"])["econs"])
        finally:
            ctx.close()
        series[prec] = np.array(e)
    e64, emx = series[0], series[1]
    scale = np.abs(e64).max()
    assert np.abs(emx - e64).max() <= 2e-6 * scale, (emx - e64) / scale
