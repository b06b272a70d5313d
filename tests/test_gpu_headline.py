"""The workload the benchmark times, against the oracle.

4096 q-SPC/Fw molecules on the 16^3 CUB lattice (L = 49.71 A), nb = 32,
MTS = 5 (dt = 1.25 fs), Ewald on the centroid (nbdf1 = 1), Lennard-Jones on 5
normal modes (nbdf2 = 5): the sizes at which the device builds its real-space
superset by cell sorting (R = 3, 10 cells per axis) and the fused MTS kernel
writes both contracted rings.  The state is evolved first (a perturbed lattice
with spread ring polymers and Maxwell-Boltzmann momenta, advanced 20 steps on
the device), so the forces do not cancel by symmetry.

Tolerances: plain FP64 against the oracle 1e-10 relative (L2 over all beads and
atoms for r, p, dvdr, dvdr2; energies; virial norms); mixed precision against
the FP64 path 1e-5 relative RMS force (total and worst bead) and 1e-5 relative
energy.
"""
import numpy as np
import pytest

from rpmd_mainz_gb300 import lib

from . import oracle_lib as orc
from . import systems

pytestmark = pytest.mark.gpu

TOL = 1e-10
MIXED_TOL = 1e-5
CASE = dict(param="param_qspcfw", ncell=(16, 16, 16), nb=32, mts=5, dtfs=1.25, nbdf1=1, nbdf2=5)


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0)


def erel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(scope="module")
def evolved():
    import __graft_entry__ as g

    g.build()
    s = systems.build(**CASE)
    lib.init(s["params"])
    r0 = systems.perturbed(s, seed=4096)
    p0 = orc.sample_rpmd(s["na"], s["nb"], s["mass"], s["beta"], orc.Rng(4711))
    ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
    ctx.upload(r=r0, p=p0, box=s["box"])
    ctx.full_forces()
    ctx.evolve(20, s["dt"], s["beta"])
    state = ctx.download()
    ctx.close()
    yield s, state
    lib.finalize()


def test_headline_state_is_evolved(evolved):
    s, (r, p, f, f2) = evolved
    # beads of a ring differ, and the lattice symmetry is broken
    assert np.abs(r - r.mean(axis=0, keepdims=True)).max() > 1e-2
    assert np.linalg.norm(f + f2) > 0.0


def test_headline_full_forces(evolved):
    s, (r, _, _, _) = evolved
    lib.init(s["params"])
    ref = orc.full_forces(r, s["box"], s["z"])
    assert ref["status"] == 0
    dev = lib.full_forces(r, s["box"], s["z"])
    for k in ("dvdr", "dvdr2"):
        assert rel(dev[k], ref[k]) < TOL, k
    for k in ("v", "vew", "voo", "vint"):
        assert erel(dev[k], ref[k]) < TOL, k
    assert rel(dev["vir"], ref["vir"]) < TOL


def test_headline_evolve_pi(evolved):
    s, (r, p, f, f2) = evolved
    lib.init(s["params"])
    so = orc.State(r, p, f, f2, s["box"])
    sd = lib.State(r, p, f, f2, s["box"])
    g = orc.Rng(1)
    for step in range(2):
        eo = orc.evolve_pi(so, s["dt"], s["mass"], s["z"], s["beta"], g)
        ed = lib.evolve_pi(sd, s["dt"], s["mass"], s["z"], s["beta"])
        assert eo["status"] == 0
        for k in ("r", "p", "dvdr", "dvdr2"):
            assert rel(getattr(sd, k), getattr(so, k)) < TOL, (step, k)
        for k in ("v", "vew", "vlj", "vint"):
            assert erel(ed[k], eo[k]) < TOL, (step, k)
        assert rel(sd.vir, so.vir) < TOL, step
        assert rel(sd.vir_lf, so.vir_lf) < TOL, step


def test_headline_mixed_force_error(evolved):
    s, (r, _, _, _) = evolved
    out = []
    for prec in (0, 1):
        prm = s["params"].copy()
        prm.precision = prec
        lib.init(prm)
        out.append(lib.full_forces(r, s["box"], s["z"]))
    f64, fmx = out
    t64, tmx = f64["dvdr"] + f64["dvdr2"], fmx["dvdr"] + fmx["dvdr2"]
    assert rel(tmx, t64) < MIXED_TOL
    assert max(rel(tmx[k], t64[k]) for k in range(s["nb"])) < MIXED_TOL
    assert erel(fmx["v"], f64["v"]) < MIXED_TOL
    assert rel(fmx["vir"], f64["vir"]) < MIXED_TOL
