"""Non-cubic boxes on the device (ewald_nc: rwald_basic / rwald_cell + kwald_nc,
ewald_noncubic.f90) against the oracle, through the C ABI: forces, full_forces
with ring-polymer contraction and evolve_pi on 8 x 4 x 4 CUB lattices (128
water, the anisotropic replicas of the batch workloads), plain FP64 to 1e-10
relative; the mixed path against the FP64 path to the 1e-5 force bound; and a
non-cubic replica in a batch equal to itself alone."""
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
    n = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / (n if n > 0 else 1.0)


def setup(**kw):
    s = systems.build(**kw)
    assert s["params"].iamcub == 0
    lib.init(s["params"])
    return s


@pytest.mark.parametrize("iopt", [0, 1, 2])
@pytest.mark.parametrize("ncell,nb", [((8, 4, 4), 2), ((4, 8, 6), 4)])
def test_forces_noncubic(iopt, ncell, nb):
    s = setup(param="param_qspcfw", ncell=ncell, nb=nb)
    r = systems.perturbed(s, seed=40 + nb)
    st, v, f, vir = orc.forces(r, s["box"], s["z"], iopt)
    assert st == 0
    vd, fd, vird = lib.forces(r, s["box"], s["z"], iopt)
    assert rel(fd, f) < TOL
    assert abs(vd - v) <= TOL * abs(v)
    assert rel(vird, vir) < TOL


@pytest.mark.parametrize("case", [
    dict(param="param_qspcfw", ncell=(8, 4, 4), nb=8, nbdf1=1, nbdf2=3),
    dict(param="param_scott", ncell=(8, 4, 4), nb=4, nbdf1=1, nbdf2=1, sig_A=4.5),  # M-site and TEM
])
def test_full_forces_noncubic(case):
    s = setup(**case)
    r = systems.perturbed(s, seed=41)
    ref = orc.full_forces(r, s["box"], s["z"])
    assert ref["status"] == 0
    dev = lib.full_forces(r, s["box"], s["z"])
    for k in ("dvdr", "dvdr2"):
        assert rel(dev[k], ref[k]) < TOL, k
    for k in ("v", "vew", "voo", "vint"):
        assert abs(dev[k] - ref[k]) <= TOL * abs(ref[k]), k
    assert rel(dev["vir"], ref["vir"]) < TOL


def test_evolve_pi_noncubic():
    s = setup(param="param_qspcfw", ncell=(8, 4, 4), nb=8, mts=5, dtfs=1.25, nbdf1=1, nbdf2=3)
    r = systems.perturbed(s, seed=42)
    p = orc.sample_rpmd(s["na"], s["nb"], s["mass"], s["beta"], orc.Rng(3))
    ff = orc.full_forces(r, s["box"], s["z"])
    ref = orc.State(r, p, ff["dvdr"], ff["dvdr2"], s["box"].copy())
    dev = lib.State(r, p, ff["dvdr"], ff["dvdr2"], s["box"].copy())
    rng = orc.Rng(1)
    for _ in range(5):
        assert orc.evolve_pi(ref, s["dt"], s["mass"], s["z"], s["beta"], rng)["status"] == 0
        lib.evolve_pi(dev, s["dt"], s["mass"], s["z"], s["beta"])
    for a, b in ((dev.r, ref.r), (dev.p, ref.p), (dev.dvdr, ref.dvdr), (dev.dvdr2, ref.dvdr2)):
        assert rel(a, b) < TOL


def test_mixed_noncubic_force_error():
    s = setup(param="param_qspcfw", ncell=(8, 4, 4), nb=8)
    r = systems.perturbed(s, seed=43)
    out = []
    for prec in (0, 1):
        prm = s["params"].copy()
        prm.precision = prec
        lib.init(prm)
        out.append(lib.full_forces(r, s["box"], s["z"]))
    f64, fmx = out
    t64 = f64["dvdr"] + f64["dvdr2"]
    assert rel(fmx["dvdr"] + fmx["dvdr2"], t64) < 1e-5
    assert abs(fmx["v"] - f64["v"]) <= 1e-5 * abs(f64["v"])
    assert rel(fmx["vir"], f64["vir"]) < 1e-5


@pytest.mark.parametrize("precision", [0, 1])
def test_noncubic_replica_in_batch(precision):
    s = setup(param="param_qspcfw", ncell=(8, 4, 4), nb=8, precision=precision)
    r = systems.perturbed(s, seed=44)
    rng = np.random.default_rng(5)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] / (s["beta"] / s["nb"]))

    def fresh():
        ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
        ctx.set_params(s["params"])
        ctx.upload(r=r, p=p, box=s["box"])
        ctx.full_forces()
        return ctx

    alone = fresh()
    alone.evolve(5, s["dt"], s["beta"])
    alone.sync()
    want = alone.download()
    alone.close()
    c = fresh()
    other = systems.build(param="param_qspcfw", ncell=(4, 4, 4), nb=4, precision=precision)  # a cubic neighbour
    o = lib.Context(other["na"], other["nb"], other["mass"], other["z"])
    o.set_params(other["params"])
    o.upload(r=other["r"], box=other["box"])
    o.full_forces()
    b = lib.Batch()
    b.add(c, s["dt"], s["beta"])
    b.add(o, other["dt"], other["beta"])
    b.step(5)
    b.sync()
    got = c.download()
    tol = 1e-6 if precision else 1e-11
    for a, w in zip(got, want):
        assert rel(a, w) < tol
    b.close()
    c.close()
    o.close()
