"""Water boxes set up the way main.f90 sets them up, through the library.

`water_box` reads a `&param` namelist file, converts the reference's input
units (main.f90:165-174: theta in degrees, rcut in Angstrom, dt in fs), builds
the CUB lattice with gbrpmd_setup_box_size / gbrpmd_cubic_lattice, fills the
Ewald parameters with gbrpmd_setup_ewald, assigns masses and charges
(main.f90:526-586), clamps rcut to half the shortest box side (main.f90:615) and
returns a GbParams ready for gbrpmd_init.
"""
import ctypes as C
import math

import numpy as np

from . import lib, namelist
from .abi import GbParams, GB_THERM_AND, GB_THERM_NONE, GB_THERM_PRG, GB_THERM_PRL

TOA = 0.5291772108      # bohr -> Angstrom (globals.inc)
TOFS = 41.341373        # fs -> atomic time units (globals.inc)
KBOLTZ = 3.166829e-6    # hartree / K (main.f90:168)
THERM = {"AND": GB_THERM_AND, "NON": GB_THERM_NONE, "PRG": GB_THERM_PRG, "PRL": GB_THERM_PRL}


def _i3(v):
    return (C.c_int * 3)(*[int(x) for x in v])


def water_box(param, ncell=(6, 6, 6), nb=32, temp=298.0, rho=0.997, rcut_A=9.0, dtfs=0.5, mts=1,
              nbdf1=0, nbdf2=0, sig_A=0.0, therm="AND", ttaufs=0.0, ecut=0.0, intra_model=0, precision=0):
    prm = namelist.read(param, "param") if isinstance(param, str) else dict(param)
    L = lib.load()
    P = GbParams()
    P.oo_eps, P.oo_sig, P.oo_gam = prm["oo_eps"], prm["oo_sig"], prm.get("oo_gam", 0.0)
    P.alpha, P.ecut, P.wm, P.wh = prm["alpha"], ecut, prm.get("wm", 0.0), prm.get("wh", 0.0)
    P.apot, P.bpot, P.alp, P.alpb = prm["apot"], prm["bpot"], prm.get("alp", 0.0), prm.get("alpb", 0.0)
    P.theta = prm["thetad"] * (math.acos(-1.0) / 180.0)
    P.reoh = prm["reoh"]
    P.nbdf1, P.nbdf2, P.mts = nbdf1, nbdf2, mts
    P.sig = sig_A / TOA if (nb > 1 and (nbdf1 > 0 or nbdf2 > 0)) else sig_A
    P.iamcub = 1
    P.therm = THERM[therm]
    P.ttau = TOFS * ttaufs
    P.intra_model, P.precision = intra_model, precision
    box = np.zeros(3)
    nm = C.c_int()
    lib._check(L.gbrpmd_setup_box_size(_i3(ncell), C.c_double(rho), C.c_double(prm["wmass"]), lib._ptr(box),
                                       C.byref(nm)))
    nm = nm.value
    na = 3 * nm
    r = np.zeros((nb, na, 3))
    lib._check(L.gbrpmd_cubic_lattice(lib._ptr(r), C.c_int(nm), C.c_int(nb), lib._ptr(box), _i3(ncell),
                                      C.c_double(P.theta), C.c_double(P.reoh)))
    rigid = prm["apot"] == 0.0 and prm["bpot"] == 0.0
    if rigid:
        P.nctot, P.nbond = 3 * nm, 3
    mass = np.zeros(na)
    z = np.zeros(na)
    mass[0::3], mass[1::3], mass[2::3] = prm["omass"], prm["hmass"], prm["hmass"]
    z[0::3], z[1::3], z[2::3] = prm["qo"], -0.5 * prm["qo"], -0.5 * prm["qo"]
    P.rcut = min(rcut_A / TOA, 0.5 * float(box.min()))
    lib._check(L.gbrpmd_setup_ewald(C.c_int(na), lib._ptr(box), C.byref(P)))
    return dict(params=P, na=na, nm=nm, nb=nb, r=r, box=box, mass=mass, z=z, beta=1.0 / (KBOLTZ * temp),
                dt=TOFS * dtfs, rigid=rigid)


def sample_momenta(na, nb, mass, beta, irun):
    """sample_rpmd + pshift from the library's ran2/gaussian stream; irun is a
    ctypes c_int seed (negative to initialise, main.f90:298)."""
    p = np.zeros((nb, na, 3))
    lib._check(lib.load().gbrpmd_sample_rpmd(lib._ptr(p), C.c_int(na), C.c_int(nb), lib._ptr(np.asarray(mass, float)),
                                             C.c_double(beta), C.byref(irun)))
    return p
