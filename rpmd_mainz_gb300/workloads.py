"""Synthetic multi-trajectory workloads: replica sets and request streams.

Each system is a q-SPC/Fw water box on the reference's CUB lattice at
0.997 g/cm^3 (main.f90 set-up through `system.water_box`), with momenta drawn
from the reference's ran2/gaussian stream seeded per system.  128 molecules
sit on the 8 x 4 x 4 lattice of a non-cubic box (the non-cubic Ewald sum).
"""
import ctypes as C
import os

import numpy as np

from . import system

HERE = os.path.dirname(os.path.abspath(__file__))
PARAM_QSPCFW = os.path.join(os.path.dirname(HERE), "tests", "golden", "params", "param_qspcfw")
# rigid 4-site water of the served stream: O-H 0.9572 A, HOH 104.52 deg, M-site
# 0.1546 A along the bisector, qH +0.5897 e, LJ sigma 3.1668 A, epsilon 0.21084
# kcal/mol (TIP4P/Ice charges and LJ on the TIP4P/2005 geometry)
PARAM_RIGID = os.path.join(HERE, "params", "param_tip4pice_msite01546_rigid")

# CUB lattice cells per molecule count; 128 molecules need the anisotropic
# 8 x 4 x 4 lattice (a non-cubic box, ewald_nc)
CELLS = {64: (4, 4, 4), 128: (8, 4, 4), 216: (6, 6, 6), 343: (7, 7, 7), 512: (8, 8, 8), 729: (9, 9, 9),
         1000: (10, 10, 10), 1331: (11, 11, 11), 1728: (12, 12, 12), 2048: (16, 16, 8)}


def _box(nm, nb, temp, precision, seed, dtfs=0.5, mts=1, param=PARAM_QSPCFW):
    s = system.water_box(param, ncell=CELLS[nm], nb=nb, temp=temp, dtfs=dtfs, mts=mts, precision=precision)
    irun = C.c_int(-(1 + seed))
    s["p"] = system.sample_momenta(s["na"], s["nb"], s["mass"], s["beta"], irun)
    s["seed"] = seed
    s["temp"] = temp
    return s


def replica_set(n=256, seed=2026, precision=1, sizes=(64, 128, 216, 343, 512), beads=(8, 16, 32, 64),
                temps=(250.0, 350.0)):
    """n independent NVT replicas: molecule count, bead count and temperature
    drawn uniformly per replica from a seeded generator."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nm = int(rng.choice(sizes))
        nb = int(rng.choice(beads))
        temp = float(rng.uniform(*temps))
        out.append(_box(nm, nb, temp, precision, seed=1000 * seed + i))
    return out


def request_stream(n=60, rate=50.0, seed=7, precision=1, sizes=(64, 216, 343, 512, 729, 1000, 1331, 1728, 2048),
                   beads=(4, 8, 16, 32, 64), nsteps=100, temp=298.0, rigid_fraction=0.5):
    """n trajectory requests with Poisson arrivals (mean `rate` per second):
    [(arrival_seconds, system, nsteps)], sizes and bead counts drawn per
    request; a `rigid_fraction` of them are rigid 4-site water (PARAM_RIGID,
    RATTLE, at most 1666 molecules as the reference's bond table allows), the
    rest flexible q-SPC/Fw."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        nm = int(rng.choice(sizes))
        nb = int(rng.choice(beads))
        rigid = bool(rng.random() < rigid_fraction) and nm <= 1666
        out.append((t, _box(nm, nb, temp, precision, seed=100000 + 1000 * seed + i,
                            param=PARAM_RIGID if rigid else PARAM_QSPCFW), nsteps))
    return out
