"""Pins the oracle (CPU FP64 restatement) to the reference's own regression
run, test/cmp/gentest.cmp: 125 H2O, nb = 2, Scott/TIP4P-type parameters with
M-site (alpha = 0.73612), quartic Morse stretch (intra_morse_harm), mts = 5,
ring-polymer contraction of Ewald and LJ to the centroid (nbdf1 = nbdf2 = 1)
with the TEM-switched short-range correction (sig = 4.5 A).
Fixtures: tests/golden/ (made by tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

from . import oracle_lib as orc
from . import systems
from rpmd_mainz_gb300 import namelist

GOLD = np.load(os.path.join(systems.GOLDEN, "gentest_frames.npz"))
KAT = json.load(open(os.path.join(systems.GOLDEN, "gentest_kat.json")))
INP = namelist.read(os.path.join(systems.PARAMS, "gentest_input"), "input")


def gentest_system():
    return systems.build(param="param_scott", ncell=INP["ncellxyz"], nb=INP["nb"], temp=INP["temp"],
                         rho=INP["rho"], rcut_A=INP["rcut"], dtfs=INP["dtfs"], mts=INP["mts"],
                         nbdf1=INP["nbdf1"], nbdf2=INP["nbdf2"], sig_A=INP["sig"], therm=INP["therm"],
                         ttaufs=INP["ttaufs"], baro=INP["baro"], taufs=INP["taufs"], pres_bar=INP["pres"])


def frame_state(s, fi):
    box = GOLD["box1"][fi] / orc.TOA
    xyz = np.stack([GOLD["xyz1"][fi], GOLD["xyz2"][fi]]) / orc.TOA
    r = systems.unwrap_beads(xyz, box)
    vel = np.stack([GOLD["vel1"][fi], GOLD["vel2"][fi]])
    return r, vel * s["mass"][None, :, None], box


def test_setup_known_answers():
    # output lines 44-56 (printed with f9.3 / f9.4)
    s = gentest_system()
    P, box = s["params"], s["box"]
    assert abs(box[0] - KAT["boxlx_bohr"]) < 5e-4
    assert abs(P.rcut - KAT["rcut_bohr"]) < 5e-4
    assert abs(P.wrcut * box[0] - KAT["wrcut_bohr"]) < 5e-5
    assert abs(P.walpha / box[0] - KAT["walpha_per_bohr"]) < 5e-5
    assert abs(P.rkmax / box[0] - KAT["rkmax_per_bohr"]) < 5e-5
    assert P.kmax == KAT["kmax"]
    assert abs(P.sig - KAT["sigma_bohr"]) < 5e-4


def test_cub_lattice_matches_vmd_start():
    # print_vmd_full (io.f90:310-407) wraps each centroid oxygen into [0, L)
    s = gentest_system()
    box = s["box"]
    rc = s["r"].mean(axis=0)
    for i in range(0, s["na"], 3):
        dh1, dh2 = rc[i + 1] - rc[i], rc[i + 2] - rc[i]
        rc[i] = rc[i] - box * (np.round(rc[i] / box) - 0.5)
        rc[i + 1], rc[i + 2] = dh1 + rc[i], dh2 + rc[i]
    assert np.array_equal(orc.TOA * rc, GOLD["start"])


def test_initial_energy():
    # output:70 "Initial energy =  -0.00420 E_h per atom" (f10.5)
    s = gentest_system()
    ff = orc.full_forces(s["r"], s["box"], s["z"])
    assert ff["status"] == 0
    assert abs(ff["v"] / s["na"] - KAT["initial_energy_per_atom"]) <= 5e-6


@pytest.mark.parametrize("fi", range(len(GOLD["frames"])))
def test_frame_forces(fi):
    # vmd_bead-{1,2}.frc hold -(dvdr + dvdr2) at the printed bead positions
    s = gentest_system()
    r, _, box = frame_state(s, fi)
    ff = orc.full_forces(r, box, s["z"])
    assert ff["status"] == 0
    F = -(ff["dvdr"] + ff["dvdr2"])
    Fref = np.stack([GOLD["frc1"][fi], GOLD["frc2"][fi]])
    rel = np.linalg.norm(F - Fref, axis=(1, 2)) / np.linalg.norm(Fref, axis=(1, 2))
    assert rel.max() < 1e-12, rel


@pytest.mark.parametrize("fa,fb", [(0, 1), (1, 2), (3, 4)])
def test_evolve_pi_replay(fa, fb):
    # frames fa and fb are 20 NVE steps apart in the same trajectory
    # (md_dynamics.f90:517-546, no thermostat inside evolve for therm = AND)
    s = gentest_system()
    r, p, box = frame_state(s, fa)
    ff = orc.full_forces(r, box, s["z"])
    st = orc.State(r, p, ff["dvdr"], ff["dvdr2"], box)
    rng = orc.Rng(1)
    for _ in range(20):
        assert orc.evolve_pi(st, s["dt"], s["mass"], s["z"], s["beta"], rng)["status"] == 0
    r_b, p_b, _ = frame_state(s, fb)
    d = st.r - r_b
    d -= box * np.round(d / box)
    assert np.abs(d).max() < 1e-11
    rel_p = np.linalg.norm(st.p - p_b) / np.linalg.norm(p_b)
    assert rel_p < 1e-11
    F = -(st.dvdr + st.dvdr2)
    Fref = np.stack([GOLD["frc1"][fb], GOLD["frc2"][fb]])
    assert np.linalg.norm(F - Fref) / np.linalg.norm(Fref) < 1e-11


EQ = np.load(os.path.join(systems.GOLDEN, "gentest_eq.npz"))


def test_md_eq_estimators_at_eq_restart():
    # eq.xyz is the state after md_eq's last step; E_eq.out, V_eq.out and
    # virial_ke_eq.out print that step's estimators (md_eq.f90:190-277) from
    # the positions and the forces of the same evaluation.  The momenta are not
    # in the file, so tk and the conserved energy are left out here.
    s = gentest_system()
    r, box = EQ["r"], EQ["box"]
    na, nm, nb = s["na"], s["nm"], s["nb"]
    ff = orc.full_forces(r, box, s["z"])
    assert ff["status"] == 0
    est = orc.estimators(r, np.zeros_like(r), ff["dvdr"], ff["dvdr2"], s["mass"], s["z"], s["beta"], ff["v"],
                         ff["vir"], box)
    E, V, TV = EQ["E_eq"], EQ["V_eq"], EQ["virial_ke_eq"]
    assert abs(est["vrp"] / na - E[2]) <= 5e-9                      # f13.8
    assert abs(nb * est["v"] / na - E[3]) <= 5e-9
    assert abs(est["v"] - V[1]) <= 5e-7                             # f14.6
    assert abs(orc.TOKJMOL * est["v"] / na - V[2]) <= 5e-7
    assert abs(orc.TOKJMOL * est["tv"] / nm - TV[1]) <= 1e-13 * abs(TV[1])  # list-directed, full precision


MDEQ = np.load(os.path.join(systems.GOLDEN, "gentest_md_eq.npz"))


def gentest_start():
    """main.f90's start of the gentest run: the CUB lattice, one gaussian drawn
    at the seeding (main.f90:298-299), full_forces, then sample (main.f90:785-788)."""
    s = gentest_system()
    rng = orc.Rng(INP["irun"])
    rng.gaussian(1.0)
    ff = orc.full_forces(s["r"], s["box"], s["z"])
    p = orc.sample_rpmd(s["na"], s["nb"], s["mass"], s["beta"], rng)
    return s, rng, orc.State(s["r"], p, ff["dvdr"], ff["dvdr2"], s["box"].copy())


def test_md_eq_replays_gentest_equilibration():
    # The whole equilibration of the reference's regression run, replayed from
    # the lattice with the reference's random stream: 100 NVT pre-equilibration
    # steps and 1000 NPT steps (Berendsen barostat inside evolve_pi, Andersen
    # collisions in md_eq), against every series md_eq printed and eq.xyz.
    s, rng, st = gentest_start()
    status, pre, eq = orc.md_eq(st, s["dt"], s["mass"], s["z"], s["beta"], INP["ne"], True, rng)
    assert status == 0
    assert np.abs(pre - MDEQ["E_pre_eq"]).max() <= 5.01e-9                        # f13.8
    assert np.abs(eq[:, 1:5] - MDEQ["E_eq"][:, 1:5]).max() <= 5.01e-9             # f13.8
    assert np.abs(eq[:, 7:9] - MDEQ["V_eq"][:, 1:3]).max() <= 5.01e-7             # f14.6
    for col, name in ((5, "temp_eq"), (6, "virial_ke_eq")):                       # full precision
        ref = MDEQ[name][:, 1]
        assert (np.abs(eq[:, col] - ref) / np.abs(ref)).max() <= 1e-11, name
    every10 = np.arange(9, INP["ne"], 10)
    pr = MDEQ["pressure_eq"][:, 1]
    assert np.abs(eq[every10, 9] - pr).max() <= 1e-10 * np.abs(pr).max()
    assert np.abs(eq[every10, 10] - MDEQ["density_eq"][:, 1]).max() <= 1e-13
    assert np.abs(st.box - EQ["box"]).max() <= 1e-12
    assert np.abs(st.r - EQ["r"]).max() <= 1e-9                                   # bohr
