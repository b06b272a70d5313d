"""Batched replicas (gbrpmd_batch_*): uneven replicas advanced together by one
CUDA-graph launch per step give the same trajectories as each replica alone.

Each replica has its own parameters (box, Ewald set-up, contraction, MTS,
precision), time step and temperature.  Tolerance 1e-11 relative for FP64
replicas: the only difference between a replica in the batch and alone is the
order of atomic additions (pair-list groups and FP64 sums).  For mixed-precision
replicas the same reordering changes FP32 sums at their rounding level, so
their tolerance is 1e-6.
"""
import ctypes as C

import numpy as np
import pytest

from rpmd_mainz_gb300 import lib

from . import systems

pytestmark = pytest.mark.gpu

TOL = 1e-11
MIXED_TOL = 1e-6

REPLICAS = [
    dict(param="param_qspcfw", ncell=(4, 4, 4), nb=8, mts=1, dtfs=0.5, temp=250.0),
    dict(param="param_qspcfw", ncell=(5, 5, 5), nb=4, mts=2, dtfs=1.0, temp=300.0),
    dict(param="param_qspcfw", ncell=(3, 3, 3), nb=16, mts=5, dtfs=1.25, nbdf1=1, nbdf2=5, temp=350.0),
    dict(param="param_qspcfw", ncell=(4, 4, 4), nb=32, mts=1, dtfs=0.5, temp=298.0, precision=1),
    # rigid 4-site water (evolve_rig_pi with RATTLE) beside the flexible replicas
    dict(param="param_tip05_rigid", ncell=(3, 3, 3), nb=4, mts=1, dtfs=0.5, temp=300.0),
]


def rel(a, b):
    # rigid water leaves dvdr2 zero: compare absolutely when the reference is zero
    d, n = float(np.linalg.norm(np.asarray(a) - np.asarray(b))), float(np.linalg.norm(b))
    return d / n if n > 0.0 else d


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    yield
    lib.finalize()


def make_replica(case, seed):
    s = systems.build(**case)
    lib.init(s["params"])
    # rigid water starts on its lattice, where the bond constraints hold
    r = s["r"].copy() if s["rigid"] else systems.perturbed(s, seed=seed)
    ff = lib.full_forces(r, s["box"], s["z"])
    rng = np.random.default_rng(seed + 1)
    p = rng.normal(size=r.shape) * np.sqrt(s["mass"][None, :, None] / (s["beta"] / s["nb"]))
    return s, r, p, ff


def fresh_context(s, r, p, ff):
    ctx = lib.Context(s["na"], s["nb"], s["mass"], s["z"])
    ctx.set_params(s["params"])
    ctx.upload(r=r, p=p, dvdr=ff["dvdr"], dvdr2=ff["dvdr2"], box=s["box"])
    return ctx


def test_batch_matches_replicas_alone():
    reps = [make_replica(c, 200 + 10 * i) for i, c in enumerate(REPLICAS)]
    nsteps = 6
    alone = []
    for s, r, p, ff in reps:
        ctx = fresh_context(s, r, p, ff)
        ctx.evolve(nsteps, s["dt"], s["beta"])
        ctx.sync()
        alone.append((ctx.download(), ctx.energies()))
        ctx.close()
    batch = lib.Batch()
    ctxs = [fresh_context(*rep) for rep in reps]
    for (s, *_), ctx in zip(reps, ctxs):
        batch.add(ctx, s["dt"], s["beta"])
    assert len(batch) == len(reps)
    batch.step(nsteps)
    batch.sync()
    for case, ctx, (state, e) in zip(REPLICAS, ctxs, alone):
        tol = MIXED_TOL if case.get("precision", 0) else TOL
        ctx.sync()
        got = ctx.download()
        for a, b in zip(got, state):
            assert rel(a, b) < tol
        eb = ctx.energies()
        for k in ("v", "vew", "vlj", "vint", "tv"):
            assert abs(eb[k] - e[k]) <= tol * abs(e[k]) + 1e-14, k
    batch.close()
    for ctx in ctxs:
        ctx.close()


def test_batch_membership_changes():
    """Replicas leave and join between steps (the graph is re-captured); each
    still follows its lone trajectory."""
    reps = [make_replica(c, 300 + 10 * i) for i, c in enumerate(REPLICAS[:3])]
    ref = []
    for s, r, p, ff in reps:
        ctx = fresh_context(s, r, p, ff)
        ctx.evolve(5, s["dt"], s["beta"])
        ctx.sync()
        ref.append(ctx.download())
        ctx.close()
    batch = lib.Batch()
    c0, c1, c2 = (fresh_context(*rep) for rep in reps)
    batch.add(c0, reps[0][0]["dt"], reps[0][0]["beta"])
    batch.add(c1, reps[1][0]["dt"], reps[1][0]["beta"])
    batch.step(3)                      # c0, c1: 3 steps
    batch.remove(c0)
    batch.add(c2, reps[2][0]["dt"], reps[2][0]["beta"])
    batch.step(2)                      # c1: 5, c2: 2
    batch.add(c0, reps[0][0]["dt"], reps[0][0]["beta"])
    batch.step(2)                      # c0: 5, c1: 7, c2: 4
    batch.remove(c1)
    batch.remove(c0)
    batch.step(1)                      # c2: 5
    batch.sync()
    for ctx, want in ((c0, ref[0]), (c2, ref[2])):
        got = ctx.download()
        for a, b in zip(got, want):
            assert rel(a, b) < TOL
    batch.close()
    for ctx in (c0, c1, c2):
        ctx.close()


def test_batch_andersen_matches_md_eq():
    """With thresh > 0 each replica draws its own ran2 stream exactly as the
    md_eq loop (gbrpmd_run_md_eq) does for a lone context."""
    case = dict(param="param_qspcfw", ncell=(3, 3, 3), nb=4, mts=1, dtfs=0.5)
    s, r, p, ff = make_replica(case, 400)
    thresh = 0.3
    lone = fresh_context(s, r, p, ff)
    irun = C.c_int(-977)
    lone.run_md_eq(10, s["dt"], s["beta"], thresh, irun)
    lone.sync()
    want = lone.download()
    batch = lib.Batch()
    ctx = fresh_context(s, r, p, ff)
    batch.add(ctx, s["dt"], s["beta"], thresh, -977)
    batch.step(10)
    batch.sync()
    got = ctx.download()
    for a, b in zip(got, want):
        assert rel(a, b) < TOL
    batch.close()
    ctx.close()
    lone.close()
