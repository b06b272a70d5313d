"""Autotuner (gbrpmd_ctx_autotune / gbrpmd_batch_autotune): it leaves the
trajectory state as it found it, picks shapes from the candidate sets, and a
tuned context follows the same trajectory as an untuned one (1e-11 relative
FP64; mixed: 1e-5, the force-error bound -- other lane counts reorder the FP32
sums, ~1e-7 per evaluation, and six steps of a perturbed start amplify it)."""
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
    n = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / (n if n > 0 else 1.0)


def context(s, r, p):
    ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
    ctx.set_params(s["params"])
    ctx.upload(r=r, p=p, box=s["box"])
    ctx.full_forces()
    return ctx


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_keeps_state_and_trajectory(precision):
    s = systems.build(param="param_qspcfw", ncell=(6, 6, 6), nb=16, mts=5, dtfs=1.25, nbdf1=1, nbdf2=3,
                      precision=precision)
    lib.init(s["params"])
    r = systems.perturbed(s, seed=50)
    rng = np.random.default_rng(51)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] / (s["beta"] / s["nb"]))
    lib.autotune_reset()
    tuned = context(s, r, p)
    before = tuned.download()
    choice = tuned.autotune(s["dt"], s["beta"], steps=4)
    assert choice["ew_np"] in (8, 16, 32) and choice["lj_np"] in (2, 4, 8)
    assert choice["mts_mpb"] in (0, 4, 8, 14, 28) and choice["skin"] in (0.05, 0.1, 0.15, 0.2)
    assert choice["rf_g"] in (8, 16) and choice["rf_ns"] in (1, 2)
    after = tuned.download()
    for a, b in zip(after, before):
        assert np.array_equal(a, b)
    plain = context(s, r, p)
    tuned.evolve(6, s["dt"], s["beta"])
    plain.evolve(6, s["dt"], s["beta"])
    tuned.sync()
    plain.sync()
    tol = 1e-5 if precision else 1e-11
    for a, b in zip(tuned.download(), plain.download()):
        assert rel(a, b) < tol
    # a second context of the same shape takes the cached choice
    again = context(s, r, p)
    assert again.autotune(s["dt"], s["beta"], steps=4) == choice
    for c in (tuned, plain, again):
        c.close()


def test_batch_autotune():
    cases = [dict(param="param_qspcfw", ncell=(4, 4, 4), nb=8, precision=1),
             dict(param="param_qspcfw", ncell=(8, 4, 4), nb=16, precision=1),
             dict(param="param_qspcfw", ncell=(4, 4, 4), nb=8, precision=1)]
    b = lib.Batch()
    ctxs = []
    for i, case in enumerate(cases):
        s = systems.build(**case)
        lib.init(s["params"])
        r = systems.perturbed(s, seed=60 + i)
        ctx = context(s, r, np.zeros_like(r))
        b.add(ctx, s["dt"], s["beta"])
        ctxs.append(ctx)
    b.autotune(steps=3)
    b.step(4)
    b.sync()
    for ctx in ctxs:
        r, p, f, f2 = ctx.download()
        assert np.isfinite(r).all() and np.isfinite(p).all()
    b.close()
    for ctx in ctxs:
        ctx.close()
