"""Plain-FP64 device path against the oracle, through the C ABI.

Tolerance: 1e-10 relative (L2 over all beads and atoms) for forces, momenta
and positions, 1e-10 relative for energies and for the virial tensor norm.
Inputs are seeded snapshots of CUB water boxes (perturbed lattices with
spread ring polymers) and the reference's own golden frames.
"""
import json
import os

import numpy as np
import pytest

from rpmd_mainz_gb300 import lib

from . import oracle_lib as orc
from . import systems

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0)


def erel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    yield
    lib.finalize()


def setup(**kw):
    s = systems.build(**kw)
    lib.init(s["params"])
    return s


@pytest.mark.parametrize("iopt", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("nb", [2, 8])
def test_forces_iopt(iopt, nb):
    s = setup(param="param_qspcfw", ncell=(4, 4, 4), nb=nb)
    r = systems.perturbed(s, seed=10 + nb)
    st, v, f, vir = orc.forces(r, s["box"], s["z"], iopt)
    assert st == 0
    vd, fd, vird = lib.forces(r, s["box"], s["z"], iopt)
    assert rel(fd, f) < TOL
    assert erel(vd, v) < TOL
    assert rel(vird, vir) < TOL


@pytest.mark.parametrize("nb", [1, 2, 4])
def test_forces_tem_correction(nb):
    # iopt = 5 with the Scott/TIP4P-type M-site (alpha = 0.73612) and sig = 4.5 A
    s = setup(param="param_scott", ncell=(5, 5, 5), nb=nb, nbdf1=1, nbdf2=1, sig_A=4.5)
    r = systems.perturbed(s, seed=20 + nb)
    st, v, f, vir = orc.forces(r, s["box"], s["z"], 5)
    assert st == 0
    vd, fd, vird = lib.forces(r, s["box"], s["z"], 5)
    assert rel(fd, f) < TOL
    assert erel(vd, v) < TOL
    assert rel(vird, vir) < TOL


def test_ewald_large_box_cells():
    # 1728 molecules: the reference's real-space sum uses 6^3 unit-box cells
    s = setup(param="param_qspcfw", ncell=(12, 12, 12), nb=1)
    r = systems.perturbed(s, seed=5, bead_spread=0.0)
    st, v, f, vir = orc.forces(r, s["box"], s["z"], 2)
    assert st == 0
    vd, fd, vird = lib.forces(r, s["box"], s["z"], 2)
    assert rel(fd, f) < TOL
    assert erel(vd, v) < TOL
    assert rel(vird, vir) < TOL


@pytest.mark.parametrize("case", [
    dict(param="param_qspcfw", ncell=(6, 6, 6), nb=32),                              # 216 H2O, nb = 32
    dict(param="param_qspcfw", ncell=(4, 4, 4), nb=8, nbdf1=1, nbdf2=3),             # contraction
    dict(param="param_qspcfw", ncell=(4, 4, 4), nb=8, nbdf1=3, nbdf2=0),
    dict(param="param_qspcfw", ncell=(4, 4, 4), nb=8, nbdf1=0, nbdf2=5),
    dict(param="param_scott", ncell=(5, 5, 5), nb=4, nbdf1=1, nbdf2=1, sig_A=4.5),  # TEM + morse
    dict(param="param_qspcfw", ncell=(4, 4, 4), nb=6, intra_model=1),               # non power of two, spcfw
])
def test_full_forces(case):
    s = setup(**case)
    r = systems.perturbed(s, seed=30)
    ref = orc.full_forces(r, s["box"], s["z"])
    assert ref["status"] == 0
    dev = lib.full_forces(r, s["box"], s["z"])
    for k in ("dvdr", "dvdr2"):
        assert rel(dev[k], ref[k]) < TOL, k
    for k in ("v", "vew", "voo", "vint"):
        assert erel(dev[k], ref[k]) < TOL, k
    assert rel(dev["vir"], ref["vir"]) < TOL


GOLD = np.load(os.path.join(systems.GOLDEN, "gentest_frames.npz"))


def gentest():
    from rpmd_mainz_gb300 import namelist

    inp = namelist.read(os.path.join(systems.PARAMS, "gentest_input"), "input")
    return setup(param="param_scott", ncell=inp["ncellxyz"], nb=inp["nb"], temp=inp["temp"], rho=inp["rho"],
                 rcut_A=inp["rcut"], dtfs=inp["dtfs"], mts=inp["mts"], nbdf1=inp["nbdf1"], nbdf2=inp["nbdf2"],
                 sig_A=inp["sig"], therm=inp["therm"], ttaufs=inp["ttaufs"])


def frame(s, fi):
    box = GOLD["box1"][fi] / orc.TOA
    xyz = np.stack([GOLD["xyz1"][fi], GOLD["xyz2"][fi]]) / orc.TOA
    r = systems.unwrap_beads(xyz, box)
    p = np.stack([GOLD["vel1"][fi], GOLD["vel2"][fi]]) * s["mass"][None, :, None]
    return r, p, box


@pytest.mark.parametrize("fi", [0, 3])
def test_golden_frame_forces(fi):
    s = gentest()
    r, _, box = frame(s, fi)
    dev = lib.full_forces(r, box, s["z"])
    F = -(dev["dvdr"] + dev["dvdr2"])
    Fref = np.stack([GOLD["frc1"][fi], GOLD["frc2"][fi]])
    assert rel(F, Fref) < 1e-12


def test_golden_replay_evolve_pi():
    s = gentest()
    r, p, box = frame(s, 0)
    ff = lib.full_forces(r, box, s["z"])
    st = lib.State(r, p, ff["dvdr"], ff["dvdr2"], box)
    for _ in range(20):
        lib.evolve_pi(st, s["dt"], s["mass"], s["z"], s["beta"])
    r1, p1, _ = frame(s, 1)
    d = st.r - r1
    d -= box * np.round(d / box)
    assert np.abs(d).max() < 1e-11
    assert rel(st.p, p1) < 1e-11
    F = -(st.dvdr + st.dvdr2)
    assert rel(F, np.stack([GOLD["frc1"][1], GOLD["frc2"][1]])) < 1e-11


@pytest.mark.parametrize("case", [
    dict(param="param_qspcfw", ncell=(4, 4, 4), nb=8, mts=3, nbdf1=1, nbdf2=3),
    dict(param="param_qspcfw", ncell=(4, 4, 4), nb=8, mts=1),
    dict(param="param_qspcfw", ncell=(4, 4, 4), nb=16, mts=5, nbdf1=1, nbdf2=5, dtfs=1.25),
    dict(param="param_qspcfw", ncell=(3, 3, 3), nb=32, mts=2, nbdf1=1, nbdf2=3),   # fused MTS, nb = 32
    dict(param="param_qspcfw", ncell=(3, 3, 3), nb=64, mts=1),                     # fused MTS, nb = 64
    dict(param="param_qspcfw", ncell=(3, 3, 3), nb=6, mts=2, nbdf1=3, nbdf2=5),    # separate kernels
    dict(param="param_scott", ncell=(3, 3, 3), nb=4, mts=5, nbdf1=1, nbdf2=3, sig_A=4.5),  # TEM, morse
])
def test_evolve_pi_steps(case):
    s = setup(**case)
    r = systems.perturbed(s, seed=40)
    ff = orc.full_forces(r, s["box"], s["z"])
    rng = np.random.default_rng(41)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] * s["nb"] / s["beta"])
    ref = orc.State(r, p, ff["dvdr"], ff["dvdr2"], s["box"])
    dev = lib.State(r, p, ff["dvdr"], ff["dvdr2"], s["box"])
    g = orc.Rng(3)
    for _ in range(4):
        eo = orc.evolve_pi(ref, s["dt"], s["mass"], s["z"], s["beta"], g)
        ed = lib.evolve_pi(dev, s["dt"], s["mass"], s["z"], s["beta"])
        assert eo["status"] == 0
    for a, b in ((dev.r, ref.r), (dev.p, ref.p), (dev.dvdr, ref.dvdr), (dev.dvdr2, ref.dvdr2)):
        assert rel(a, b) < TOL
    for k in ("v", "vew", "vlj", "vint"):
        assert erel(ed[k], eo[k]) < TOL, k
    assert rel(dev.vir, ref.vir) < TOL
    assert rel(dev.vir_lf, ref.vir_lf) < TOL


def test_resident_context_matches_dropin():
    s = setup(param="param_qspcfw", ncell=(4, 4, 4), nb=8, mts=2, nbdf1=1, nbdf2=3)
    r = systems.perturbed(s, seed=50)
    ff = orc.full_forces(r, s["box"], s["z"])
    p = np.zeros_like(r)
    ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
    ctx.upload(r=r, p=p, dvdr=ff["dvdr"], dvdr2=ff["dvdr2"], box=s["box"])
    ctx.evolve(3, s["dt"], s["beta"])
    ctx.sync()
    rr, pp, f1, f2 = ctx.download()
    ref = orc.State(r, p, ff["dvdr"], ff["dvdr2"], s["box"])
    g = orc.Rng(1)
    for _ in range(3):
        orc.evolve_pi(ref, s["dt"], s["mass"], s["z"], s["beta"], g)
    assert rel(rr, ref.r) < TOL and rel(pp, ref.p) < TOL and rel(f1, ref.dvdr) < TOL
    ctx.close()


SKIN_CASES = [
    dict(param="param_qspcfw", ncell=(5, 5, 5), nb=8, mts=2, nbdf1=1, nbdf2=5),  # centroid LJ list
    dict(param="param_scott", ncell=(4, 4, 4), nb=2, mts=5, nbdf1=1, nbdf2=1, sig_A=4.5),  # TEM, per-bead LJ
]


@pytest.mark.parametrize("case", SKIN_CASES)
def test_skin_lists_match_oracle(case):
    """Twelve steps with reused skin lists equal the oracle, which builds every
    list from scratch; the Ewald list must have been reused at least once."""
    s = setup(**case)
    r = systems.perturbed(s, seed=70)
    ff = orc.full_forces(r, s["box"], s["z"])
    rng = np.random.default_rng(71)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] / (s["beta"] / s["nb"]))
    nsteps = 12
    ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
    ctx.set_list_skin(0.1)
    ctx.upload(r=r, p=p, dvdr=ff["dvdr"], dvdr2=ff["dvdr2"], box=s["box"])
    ctx.evolve(nsteps, s["dt"], s["beta"])
    ctx.sync()
    rr, pp, f1, f2 = ctx.download()
    rebuilds = ctx.list_rebuilds()
    ctx.close()
    ref = orc.State(r, p, ff["dvdr"], ff["dvdr2"], s["box"])
    g = orc.Rng(1)
    for _ in range(nsteps):
        orc.evolve_pi(ref, s["dt"], s["mass"], s["z"], s["beta"], g)
    assert rel(rr, ref.r) < TOL and rel(pp, ref.p) < TOL
    assert rel(f1, ref.dvdr) < TOL and rel(f2, ref.dvdr2) < TOL
    assert 1 <= rebuilds[0] < nsteps, rebuilds


@pytest.mark.parametrize("case", SKIN_CASES)
def test_skin_fraction_does_not_change_results(case):
    """No skin (full rebuild at every use), a thin skin (frequent rebuilds) and
    a thick one give the same trajectory up to summation order."""
    s = setup(**case)
    r = systems.perturbed(s, seed=72)
    ff = orc.full_forces(r, s["box"], s["z"])
    rng = np.random.default_rng(73)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] / (s["beta"] / s["nb"]))
    out = []
    for frac in (0.0, 0.003, 0.3):
        ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
        ctx.set_list_skin(frac)
        ctx.upload(r=r, p=p, dvdr=ff["dvdr"], dvdr2=ff["dvdr2"], box=s["box"])
        ctx.evolve(8, s["dt"], s["beta"])
        ctx.sync()
        out.append(ctx.download())
        ctx.close()
    for other in out[1:]:
        for a, b in zip(other, out[0]):
            assert rel(a, b) < 1e-12


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_replay_matches_plain_steps(precision):
    """Steps replayed from a captured CUDA graph, with a full_forces call in
    between (which drops the graph), equal the same steps launched one by one."""
    s = setup(param="param_qspcfw", ncell=(5, 5, 5), nb=8, mts=2, nbdf1=1, nbdf2=5)
    prm = s["params"]
    prm.precision = precision
    lib.init(prm)
    r = systems.perturbed(s, seed=80)
    ff = lib.full_forces(r, s["box"], s["z"])
    rng = np.random.default_rng(81)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] / (s["beta"] / s["nb"]))
    out = []
    for graphs in (False, True):
        ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
        ctx.set_graphs(graphs)
        ctx.upload(r=r, p=p, dvdr=ff["dvdr"], dvdr2=ff["dvdr2"], box=s["box"])
        ctx.evolve(5, s["dt"], s["beta"])
        ctx.full_forces()
        ctx.evolve(6, s["dt"], s["beta"])
        ctx.sync()
        out.append((ctx.download(), ctx.energies(), ctx.launches))
        ctx.close()
    prm.precision = 0
    lib.init(prm)
    (a, ea, la), (b, eb, lb) = out
    # FP64: only the order of atomic additions differs; mixed: the pair-list
    # order (atomic group appends) also reorders FP32 sums, at their rounding
    # level, and 11 chaotic steps grow that; the forces (differences of large
    # Coulomb terms) are compared at half the mixed path's 1e-5 force bound
    tol = 1e-12 if precision == 0 else 1e-6
    ftol = 1e-12 if precision == 0 else 5e-6
    for k, (x, y) in enumerate(zip(a, b)):
        assert rel(x, y) < (tol if k < 2 else ftol), k
    for k in ("v", "vew", "vlj", "vint", "tv"):
        assert erel(eb[k], ea[k]) < 10 * tol
    assert la == lb


def rigid_system(nb=4):
    s = setup(param="param_tip05_rigid", ncell=(4, 4, 4), nb=nb)
    lib.rattle_setup(s["nm"])
    lib.init(orc.get_params())
    return s


def test_rattle_dropin():
    s = rigid_system(nb=1)
    rng = np.random.default_rng(60)
    r0 = s["r"][0].copy()
    rold = r0.copy()
    r = r0 + rng.normal(scale=0.01, size=r0.shape)
    p = rng.normal(scale=5.0, size=r0.shape)
    f = rng.normal(scale=0.01, size=r0.shape)
    dt = 20.0
    import ctypes as C
    lorc = orc.load()
    ro, po, fo, viro = r.copy(), p.copy(), f.copy(), np.zeros(9)
    st = lorc.orc_rattle_s1(orc._ptr(ro), orc._ptr(rold), orc._ptr(po), C.c_int(s["nm"]), orc._ptr(s["mass"]),
                            C.c_double(dt), orc._ptr(fo), orc._ptr(viro), C.c_int(s["na"]))
    assert st == 0
    rd, pd, fd = r.copy(), p.copy(), f.copy()
    vird = lib.rattle_s1(rd, rold, pd, s["mass"], dt, fd)
    assert rel(rd, ro) < TOL and rel(pd, po) < TOL and rel(fd, fo) < TOL
    assert rel(vird, viro.reshape(3, 3, order="F")) < TOL
    # stage 2 on the constrained positions
    po2, fo2, viro2 = pd.copy(), fd.copy(), np.zeros(9)
    st = lorc.orc_rattle_s2(orc._ptr(ro), orc._ptr(po2), C.c_int(s["nm"]), orc._ptr(s["mass"]), C.c_double(dt),
                            orc._ptr(fo2), orc._ptr(viro2), C.c_int(s["na"]))
    assert st == 0
    pd2, fd2 = pd.copy(), fd.copy()
    vird2 = lib.rattle_s2(rd, pd2, s["mass"], dt, fd2)
    assert rel(pd2, po2) < TOL and rel(fd2, fo2) < TOL
    assert rel(vird2, viro2.reshape(3, 3, order="F")) < TOL


def test_evolve_rig_pi():
    s = rigid_system(nb=4)
    r = s["r"].copy()
    rng = np.random.default_rng(70)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] * s["nb"] / s["beta"]) * 0.1
    st0, v0, f0, vir0 = orc.forces(r, s["box"], s["z"], 1)
    ref = orc.State(r, p, f0, np.zeros_like(r), s["box"])
    dev = lib.State(r, p, f0, np.zeros_like(r), s["box"])
    g = orc.Rng(1)
    for _ in range(3):
        eo = orc.evolve_rig_pi(ref, s["dt"], s["mass"], s["z"], s["beta"], g)
        ed = lib.evolve_rig_pi(dev, s["dt"], s["mass"], s["z"], s["beta"])
        assert eo["status"] == 0
    for a, b in ((dev.r, ref.r), (dev.p, ref.p), (dev.dvdr, ref.dvdr)):
        assert rel(a, b) < TOL
    assert erel(ed["v"], eo["v"]) < TOL
    assert rel(dev.vir, ref.vir) < TOL
    assert rel(dev.vir_lf, ref.vir_lf) < TOL
