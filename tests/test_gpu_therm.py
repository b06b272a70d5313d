"""The thermostat kicks and the barostat inside evolve_pi on the device,
through the drop-in C ABI, against the oracle: PRL (parinello_therm_loc) and
PRG (parinello_therm) kicks drawing the reference's random stream, and the
Berendsen barostat (nbaro = 1: beren_baro on cubic boxes, beren_baro_nc on
the others, and the barostat of evolve_rig_pi); then the reference's own gentest equilibration
(100 NVT + 1000 NPT steps, Andersen collisions, md_eq.f90) replayed on the
device from the lattice against every series the reference printed.

Tolerance: 1e-10 relative (L2) for positions, momenta and forces and for the
box after the steps, as for the other plain-FP64 parity tests.
"""
import ctypes as C

import numpy as np
import pytest

from rpmd_mainz_gb300 import lib

from . import oracle_lib as orc
from . import systems

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    yield
    lib.finalize()


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b)


def run_both(s, nsteps, nbaro=0, seed=31):
    lib.init(s["params"])
    r = systems.perturbed(s, seed=3)
    p = orc.sample_rpmd(s["na"], s["nb"], s["mass"], s["beta"], orc.Rng(11))
    ff = orc.full_forces(r, s["box"], s["z"])
    ref = orc.State(r, p, ff["dvdr"], ff["dvdr2"], s["box"].copy())
    dev = lib.State(r, p, ff["dvdr"], ff["dvdr2"], s["box"].copy())
    rng = orc.Rng(seed)
    lib.rng_reset()
    irun = C.c_int(-seed)
    for _ in range(nsteps):
        assert orc.evolve_pi(ref, s["dt"], s["mass"], s["z"], s["beta"], rng, nbaro=nbaro)["status"] == 0
        lib.evolve_pi(dev, s["dt"], s["mass"], s["z"], s["beta"], irun=irun, nbaro=nbaro)
    assert irun.value == rng.irun.value  # the same number of draws
    return ref, dev


@pytest.mark.parametrize("therm", ["PRL", "PRG"])
@pytest.mark.parametrize("case", [dict(ncell=(4, 4, 4), nb=8),
                                  dict(ncell=(4, 4, 4), nb=16, mts=5, dtfs=1.25, nbdf1=1, nbdf2=3)])
def test_thermostat_kicks_match_oracle(therm, case):
    s = systems.build(param="param_qspcfw", therm=therm, ttaufs=100.0, **case)
    ref, dev = run_both(s, 4)
    assert rel(dev.p, ref.p) < TOL
    assert rel(dev.r, ref.r) < TOL
    assert rel(dev.dvdr + dev.dvdr2, ref.dvdr + ref.dvdr2) < TOL


@pytest.mark.parametrize("case", [dict(ncell=(4, 4, 4), nb=8), dict(ncell=(5, 5, 5), nb=4, mts=5, dtfs=1.25,
                                                                     nbdf1=1, nbdf2=3)])
def test_berendsen_barostat_matches_oracle(case):
    s = systems.build(param="param_qspcfw", therm="NON", baro="BER", taufs=200.0, **case)
    ref, dev = run_both(s, 4, nbaro=1)
    assert abs(ref.box[0] - s["box"][0]) > 1e-9  # the box moved
    assert np.abs(dev.box - ref.box).max() <= TOL * ref.box[0]
    assert rel(dev.r, ref.r) < TOL
    assert rel(dev.p, ref.p) < TOL
    assert rel(dev.dvdr + dev.dvdr2, ref.dvdr + ref.dvdr2) < TOL


def test_berendsen_barostat_noncubic_matches_oracle():
    # beren_baro_nc (module_barostat.f90:28-86): one scale per axis
    s = systems.build(param="param_qspcfw", ncell=(8, 4, 4), nb=4, mts=5, dtfs=1.25, nbdf1=1, nbdf2=3,
                      therm="NON", baro="BER", taufs=200.0)
    assert s["params"].iamcub == 0
    ref, dev = run_both(s, 4, nbaro=1)
    scale = ref.box / s["box"]
    assert np.ptp(scale) > 1e-9  # the axes moved by different factors
    assert np.abs(dev.box - ref.box).max() <= TOL * ref.box.max()
    assert rel(dev.r, ref.r) < TOL
    assert rel(dev.p, ref.p) < TOL
    assert rel(dev.dvdr + dev.dvdr2, ref.dvdr + ref.dvdr2) < TOL


@pytest.mark.parametrize("ncell", [(4, 4, 4), (6, 4, 4)])
def test_rigid_barostat_matches_oracle(ncell):
    # evolve_rig_pi with nbaro = 1 (evolve_rigid.f90:203-213): virial_ke with
    # the zeroed dvdr2, then beren_driver on the bead positions; the caller's
    # vir accumulates over the calls
    s = systems.build(param="param_tip05_rigid", ncell=ncell, nb=4, therm="NON", baro="BER", taufs=100.0)
    lib.rattle_setup(s["nm"])
    lib.init(orc.get_params())
    r = s["r"].copy()
    rng = np.random.default_rng(71)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] * s["nb"] / s["beta"]) * 0.1
    st0, v0, f0, vir0 = orc.forces(r, s["box"], s["z"], 1)
    assert st0 == 0
    ref = orc.State(r, p, f0, np.zeros_like(r), s["box"].copy())
    dev = lib.State(r, p, f0, np.zeros_like(r), s["box"].copy())
    g = orc.Rng(1)
    for _ in range(3):
        eo = orc.evolve_rig_pi(ref, s["dt"], s["mass"], s["z"], s["beta"], g, nbaro=1)
        assert eo["status"] == 0
        ed = lib.evolve_rig_pi(dev, s["dt"], s["mass"], s["z"], s["beta"], nbaro=1)
    assert np.abs(ref.box - s["box"]).max() > 1e-9  # the box moved
    assert np.abs(dev.box - ref.box).max() <= TOL * ref.box.max()
    for a, b in ((dev.r, ref.r), (dev.p, ref.p), (dev.dvdr, ref.dvdr)):
        assert rel(a, b) < TOL
    assert abs(ed["v"] - eo["v"]) <= TOL * abs(eo["v"])
    assert rel(dev.vir, ref.vir) < TOL
    assert rel(dev.vir_lf, ref.vir_lf) < TOL


def test_rigid_barostat_resident_context_matches_dropin():
    # a resident context's rigid NPT steps: the virial the barostat reads
    # accumulates over its barostat steps as the drop-in caller's vir does
    s = systems.build(param="param_tip05_rigid", ncell=(6, 4, 4), nb=4, therm="NON", baro="BER", taufs=100.0)
    lib.rattle_setup(s["nm"])
    lib.init(orc.get_params())
    r = s["r"].copy()
    rng = np.random.default_rng(72)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] * s["nb"] / s["beta"]) * 0.1
    f0 = orc.forces(r, s["box"], s["z"], 1)[2]
    dev = lib.State(r, p, f0, np.zeros_like(r), s["box"].copy())
    for _ in range(3):
        lib.evolve_rig_pi(dev, s["dt"], s["mass"], s["z"], s["beta"], nbaro=1)
    ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
    try:
        ctx.upload(r=r, p=p, dvdr=f0, dvdr2=np.zeros_like(r), box=s["box"])
        ctx.set_nbaro(1)
        ctx.evolve(3, s["dt"], s["beta"])
        ctx.sync()
        rr, pp, ff, _ = ctx.download()
        box = ctx.box
    finally:
        ctx.close()
    assert np.abs(box - dev.box).max() <= 1e-12 * box.max()
    assert rel(rr, dev.r) < 1e-12 and rel(pp, dev.p) < 1e-12 and rel(ff, dev.dvdr) < 1e-12


def test_device_replays_gentest_equilibration():
    # main.f90:298-299 seeding, full_forces, sample, then md_eq (100 NVT steps,
    # then 1000 NPT steps with the Berendsen barostat), all on the device
    from .test_oracle_golden import EQ, INP, MDEQ, gentest_system

    s = gentest_system()
    lib.init(s["params"])
    na, nm, nb = s["na"], s["nm"], s["nb"]
    lib.rng_reset()
    irun = C.c_int(-INP["irun"])
    lib.gaussian(irun, 1.0)
    ctx = lib.Context(na, nb, s["mass"], s["z"])
    try:
        ctx.upload(r=s["r"], box=s["box"])
        ctx.full_forces()
        from rpmd_mainz_gb300 import system

        ctx.upload(p=system.sample_momenta(na, nb, s["mass"], s["beta"], irun))

        def md_eq_step():  # evolve, the printed estimators, then the collision test (md_eq.f90:186-315)
            ctx.evolve(1, s["dt"], s["beta"])
            ctx.sync()
            e = ctx.estimators(s["beta"])
            e["box"] = ctx.box[0]
            if lib.ran2(irun) < 0.01:  # thresh for ens = NPT
                ctx.upload(p=system.sample_momenta(na, nb, s["mass"], s["beta"], irun))
            return e

        pre = [md_eq_step() for _ in range(100)]  # NVT pre-equilibration
        ctx.set_nbaro(1)
        eq = [md_eq_step() for _ in range(INP["ne"])]
        r_end = ctx.download()[0]
    finally:
        ctx.close()
    E = np.array([[(nb * e["v"] + e["tk"] + e["vrp"]) / na, e["vrp"] / na, nb * e["v"] / na, e["tk"] / na]
                  for e in pre])
    assert np.abs(E - MDEQ["E_pre_eq"][:, 1:5]).max() <= 5.01e-9
    E = np.array([[(nb * e["v"] + e["tk"] + e["vrp"]) / na, e["vrp"] / na, nb * e["v"] / na, e["tk"] / na]
                  for e in eq])
    assert np.abs(E - MDEQ["E_eq"][:, 1:5]).max() <= 5.01e-9
    temp = np.array([e["temp"] for e in eq])
    tv = np.array([orc.TOKJMOL * e["tv"] / nm for e in eq])
    assert (np.abs(temp - MDEQ["temp_eq"][:, 1]) / MDEQ["temp_eq"][:, 1]).max() <= 1e-10
    assert (np.abs(tv - MDEQ["virial_ke_eq"][:, 1]) / np.abs(MDEQ["virial_ke_eq"][:, 1])).max() <= 1e-10
    pres = np.array([orc.TOBAR * e["pres"] for e in eq])[9::10]
    assert np.abs(pres - MDEQ["pressure_eq"][:, 1]).max() <= 1e-9 * np.abs(MDEQ["pressure_eq"][:, 1]).max()
    den = np.array([e["den"] for e in eq])[9::10]
    assert np.abs(den - MDEQ["density_eq"][:, 1]).max() <= 1e-12
    assert abs(eq[-1]["box"] - EQ["box"][0]) <= 1e-11
    assert np.abs(r_end - EQ["r"]).max() <= 1e-8


@pytest.mark.parametrize("therm", ["PRL", "PRG"])
@pytest.mark.parametrize("mode", ["device", "reference"])
def test_thermostat_reaches_temperature(therm, mode):
    # strong coupling (ttau 10 fs) from cold momenta (a tenth of the thermal
    # scale; PRG rescales, so it cannot start from zero): the kinetic
    # temperature of md_eq (md_eq.f90:272) settles at the target
    s = systems.build(param="param_qspcfw", ncell=(6, 6, 6), nb=8, temp=298.0, therm=therm, ttaufs=10.0)
    lib.init(s["params"])
    p0 = 0.1 * orc.sample_rpmd(s["na"], s["nb"], s["mass"], s["beta"], orc.Rng(8))
    ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
    try:
        ctx.set_params(s["params"])
        ctx.upload(r=s["r"], p=p0, box=s["box"])
        ctx.full_forces()
        if mode == "device":
            ctx.set_rng_mode("device", seed=123)
        else:
            ctx.set_rng(-77)
        temps = []
        for step in range(400):
            ctx.evolve(1, s["dt"], s["beta"])
            if step >= 200:
                ctx.sync()
                temps.append(ctx.estimators(s["beta"])["temp"])
    finally:
        ctx.close()
    assert abs(np.mean(temps) - 298.0) < 0.03 * 298.0, np.mean(temps)
    assert np.std(temps) < 0.1 * 298.0


def test_device_stream_replica_in_batch_equals_alone():
    s = systems.build(param="param_qspcfw", ncell=(4, 4, 4), nb=8, therm="PRL", ttaufs=50.0)
    lib.init(s["params"])
    r = systems.perturbed(s, seed=70)

    def run(batched):
        ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
        ctx.set_params(s["params"])
        ctx.upload(r=r, p=np.zeros_like(r), box=s["box"])
        ctx.full_forces()
        ctx.set_rng_mode("device", seed=9)
        if batched:
            b = lib.Batch()
            b.add(ctx, s["dt"], s["beta"])
            b.step(6)
            b.sync()
            b.close()
        else:
            ctx.evolve(6, s["dt"], s["beta"])
            ctx.sync()
        out = ctx.download()
        ctx.close()
        return out

    alone, inbatch = run(False), run(True)
    assert np.abs(alone[1]).max() > 0.0  # the kicks heated the cold start
    for a, b in zip(inbatch, alone):
        assert rel(a, b) < 1e-11
