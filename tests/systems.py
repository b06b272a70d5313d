"""Water-box set-up for the tests, following main.f90's start-up order.

main.f90: namelists (137-147) -> theta, beta, dt, rcut in bohr (165-174) ->
setup_pi (sig in bohr when contraction is on, 304) -> setup_box_size + CUB
lattice (460-465) -> rattle_setup for rigid water (513-518) -> masses and
charges (526-586) -> rcut clamp to half the shortest box side (615-616) ->
setup_ewald (631).  The box, lattice and Ewald parameters come from the
oracle's restatements of those routines; everything here is test
infrastructure.
"""
import math
import os

import numpy as np

from rpmd_mainz_gb300 import namelist
from rpmd_mainz_gb300.abi import GbParams, GB_THERM_AND, GB_THERM_NONE, GB_THERM_PRG, GB_THERM_PRL

from . import oracle_lib as orc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PARAMS = os.path.join(GOLDEN, "params")

THERM = {"AND": GB_THERM_AND, "NON": GB_THERM_NONE, "PRG": GB_THERM_PRG, "PRL": GB_THERM_PRL}
BARO = {"NON": 0, "BER": 1, "MCI": 2}


def read_param(name):
    return namelist.read(os.path.join(PARAMS, name), "param")


def build(param="param_qspcfw", ncell=(6, 6, 6), nb=32, temp=298.0, rho=0.997, rcut_A=9.0, dtfs=0.5,
          mts=1, nbdf1=0, nbdf2=0, sig_A=0.0, therm="AND", ttaufs=0.0, ecut=0.0, intra_model=0,
          precision=0, baro="NON", taufs=0.0, pres_bar=1.0):
    prm = read_param(param) if isinstance(param, str) else dict(param)
    P = GbParams()
    P.oo_eps = prm["oo_eps"]
    P.oo_sig = prm["oo_sig"]
    P.oo_gam = prm.get("oo_gam", 0.0)
    P.alpha = prm["alpha"]
    P.ecut = ecut
    P.wm = prm.get("wm", 0.0)
    P.wh = prm.get("wh", 0.0)
    P.apot = prm["apot"]
    P.bpot = prm["bpot"]
    P.alp = prm.get("alp", 0.0)
    P.alpb = prm.get("alpb", 0.0)
    P.theta = prm["thetad"] * (math.acos(-1.0) / 180.0)
    P.reoh = prm["reoh"]
    P.nbdf1 = nbdf1
    P.nbdf2 = nbdf2
    P.mts = mts
    sig = sig_A
    if nb > 1 and (nbdf1 > 0 or nbdf2 > 0):
        sig = sig / orc.TOA  # setup_pi (setup_options.f90:24-26)
    P.sig = sig
    P.iamcub = 1
    P.therm = THERM[therm]
    P.ttau = 41.341373 * ttaufs
    P.intra_model = intra_model
    P.precision = precision
    # module barostat (main.f90:166, 259-270): patm = pres / tobar, taub = tofs * taufs
    P.baro = BARO[baro]
    P.taub = orc.TOFS * taufs
    P.patm = pres_bar / orc.TOBAR
    rigid = prm["apot"] == 0.0 and prm["bpot"] == 0.0
    beta = 1.0 / (orc.KBOLTZ_MAIN * temp)
    dt = orc.TOFS * dtfs
    orc.set_params(P)
    nm, box = orc.setup_box_size_cub(ncell, rho, prm["wmass"])
    r1 = orc.cubic(nm, box, ncell)
    na = 3 * nm
    r = np.repeat(r1[None, :, :], nb, axis=0)
    if rigid:
        orc.rattle_setup(nm)
        P = orc.get_params()
    else:
        P.nctot = 0
        P.nbond = 0
    mass = np.zeros(na)
    z = np.zeros(na)
    mass[0::3] = prm["omass"]
    mass[1::3] = prm["hmass"]
    mass[2::3] = prm["hmass"]
    qo = prm["qo"]
    z[0::3] = qo
    z[1::3] = -0.5 * qo
    z[2::3] = -0.5 * qo
    P.rcut = min(rcut_A / orc.TOA, 0.5 * float(min(box)))
    orc.set_params(P)
    orc.setup_ewald(na, box)
    P = orc.get_params()
    return dict(params=P, na=na, nm=nm, nb=nb, r=r, box=box, mass=mass, z=z, beta=beta, dt=dt, rigid=rigid)


def perturbed(sysd, seed, amp=0.05, bead_spread=0.1):
    """Seeded non-lattice snapshot: every atom displaced by a random vector of
    up to `amp` bohr, and each bead further by up to `bead_spread` bohr, so
    that the ring polymers have finite radius of gyration."""
    rng = np.random.default_rng(seed)
    nb, na = sysd["nb"], sysd["na"]
    r = sysd["r"].copy()
    base = rng.uniform(-amp, amp, size=(1, na, 3))
    beads = rng.uniform(-bead_spread, bead_spread, size=(nb, na, 3))
    return r + base + beads


def unwrap_beads(xyz_beads, box):
    """Undo the per-bead, per-molecule periodic wrap of print_vmd_bead
    (io.f90:549-643): shift every molecule of every bead by whole box lengths so
    that its oxygen sits at the minimum image of bead 1's oxygen."""
    out = xyz_beads.copy()
    nb, na, _ = out.shape
    for k in range(1, nb):
        o_ref = out[0, 0::3]
        o_k = out[k, 0::3]
        shift = box * np.round((o_k - o_ref) / box)
        out[k] -= np.repeat(shift, 3, axis=0)
    return out
