"""The reference's on-disk formats through the C ABI (io.f90; host code, no
GPU): the restart file of print_structure read from the reference's own
eq.xyz and written back exactly, and the xyz frames of print_vmd_bead /
print_vmd_full against the frames the reference wrote in its regression run
(bead positions wrapped into the box in Angstrom, velocities) and its start
lattice."""
import os

import numpy as np
import pytest

from rpmd_mainz_gb300 import lib

from . import oracle_lib as orc
from . import systems
from .test_oracle_golden import EQ, GOLD, frame_state, gentest_system


@pytest.fixture(scope="module", autouse=True)
def built():
    from rpmd_mainz_gb300 import build

    build.build()
    lib.load()


def test_read_reference_restart_file():
    r, box = lib.read_structure(os.path.join(systems.GOLDEN, "gentest_eq.xyz"))
    assert r.shape == EQ["r"].shape
    assert np.array_equal(r, EQ["r"]) and np.array_equal(box, EQ["box"])


def test_restart_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    r = rng.normal(size=(4, 9, 3)) * np.array([1e-7, 2.5, 3e17])
    box = np.array([12.5, 0.07, 3.0e5])
    path = tmp_path / "restart.xyz"
    lib.write_structure(path, r, box)
    r2, box2 = lib.read_structure(path)
    assert np.array_equal(r2, r) and np.array_equal(box2, box)


@pytest.mark.parametrize("fi", [0, 3])
def test_vmd_bead_frames_match_reference(tmp_path, fi):
    # vmd_bead-{1,2}.{xyz,vel} of the regression run: print_vmd_bead and
    # print_vmd_bead_vels of the state; frame_state unwraps the printed beads
    s = gentest_system()
    r, p, box = frame_state(s, fi)
    # print_vmd_bead maps x to x - L (nint(x / L) - 1/2), a shift by L/2 for
    # points already in [0, L): the printed frame is the image of r - L/2
    r = r - 0.5 * box
    for bead in (1, 2):
        path = tmp_path / f"b{bead}.xyz"
        lib.write_vmd(path, "xyz", r, box, bead=bead)
        xyz, pbox = lib.read_vmd(path, s["na"])
        assert np.abs(pbox - GOLD[f"box{bead}"][fi]).max() < 1e-12
        assert np.abs(xyz - GOLD[f"xyz{bead}"][fi]).max() < 1e-10  # Angstrom
        ff = orc.full_forces(r, box, s["z"])  # print_vmd_bead_forces of the same state
        lib.write_vmd(tmp_path / "f.frc", "frc", ff["dvdr"], box, a2=ff["dvdr2"], bead=bead)
        frc, _ = lib.read_vmd(tmp_path / "f.frc", s["na"])
        ref = GOLD[f"frc{bead}"][fi]
        assert np.abs(frc - ref).max() <= 1e-11 * np.abs(ref).max()
        lib.write_vmd(tmp_path / "v.vel", "vel", p, box, mass=s["mass"], bead=bead)
        vel, _ = lib.read_vmd(tmp_path / "v.vel", s["na"])
        ref = GOLD[f"vel{bead}"][fi]
        assert np.abs(vel - ref).max() <= 1e-12 * np.abs(ref).max()


def test_vmd_centroid_frame_of_start_lattice(tmp_path):
    # vmd_start.xyz: print_vmd_full of the CUB lattice
    s = gentest_system()
    path = tmp_path / "start.xyz"
    lib.write_vmd(path, "xyz", s["r"], s["box"])
    lib.write_vmd(path, "frc", np.zeros_like(s["r"]), s["box"], a2=np.zeros_like(s["r"]), append=True)
    xyz, box = lib.read_vmd(path, s["na"], frame=0)
    assert np.abs(xyz - GOLD["start"]).max() < 1e-12
    assert np.abs(box - GOLD["start_box"]).max() < 1e-12
    frc, _ = lib.read_vmd(path, s["na"], frame=1)
    assert not frc.any()
