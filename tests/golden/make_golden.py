"""Generate the golden fixtures of tests/golden/ from the reference's own
regression run (test/cmp/gentest.cmp of DCM-UPB/RPMD_Mainz) and its param files.

Run in a checkout where the reference tree is available:

    python tests/golden/make_golden.py /path/to/RPMD_Mainz

Writes
  params/*                 the namelist files the tests use (data, unchanged)
  gentest_frames.npz       bead positions (Angstrom), forces -(dvdr+dvdr2)
                           (hartree/bohr) and velocities p/m (a.u.) of both
                           beads for a few frames of the NVE trajectories, the
                           box, and the initial CUB lattice vmd_start.xyz
  gentest_kat.json         the set-up values and initial energy printed in
                           `output`
  gentest_eq.npz           eq.xyz (print_structure restart file, io.f90:1-17:
                           the bead positions in bohr and the box after the
                           1000 NPT equilibration steps) and the last lines of
                           E_eq.out, virial_ke_eq.out and V_eq.out (md_eq.f90:
                           274-277), printed at the same step
  gentest_eq.xyz           eq.xyz itself, for the restart-file reader
  gentest_md_eq.npz        the md_eq series of the same run: E_pre_eq.out (the
                           100-step NVT pre-equilibration) and E_eq.out,
                           temp_eq.out, virial_ke_eq.out, V_eq.out,
                           pressure_eq.out, density_eq.out (1000 NPT steps)
Frames are written every pb = 20 steps of the two 2*nt = 250-step NVE
trajectories of md_dynamics.f90 (trajectory(), lines 517-546): file frames
0..11 belong to trajectory 1, 12..23 to trajectory 2.
"""
import json
import os
import re
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FRAMES = [0, 1, 2, 12, 13]


def read_xyz_frames(path):
    frames, boxes = [], []
    with open(path) as f:
        lines = f.read().splitlines()
    i = 0
    while i < len(lines):
        if not lines[i].strip():
            i += 1
            continue
        na = int(lines[i].split()[0])
        box = [float(x) for x in lines[i + 1].split()[1:4]]
        rows = []
        for ln in lines[i + 2:i + 2 + na]:
            parts = ln.split()
            rows.append([float(x) for x in parts[1:4]])
        frames.append(rows)
        boxes.append(box)
        i += 2 + na
    return np.array(frames), np.array(boxes)


def main(ref):
    cmp_dir = os.path.join(ref, "test", "cmp", "gentest.cmp")
    os.makedirs(os.path.join(HERE, "params"), exist_ok=True)
    for name in ["param_qspcfw", "param_scott", "param_tipice_rigid", "param_tip05_rigid", "param_spce_rigid"]:
        shutil.copyfile(os.path.join(ref, "params", name), os.path.join(HERE, "params", name))
    shutil.copyfile(os.path.join(cmp_dir, "input"), os.path.join(HERE, "params", "gentest_input"))

    data = {}
    for bead in (1, 2):
        for kind in ("xyz", "frc", "vel"):
            arr, box = read_xyz_frames(os.path.join(cmp_dir, f"vmd_bead-{bead}.{kind}"))
            data[f"{kind}{bead}"] = arr[FRAMES]
            if kind == "xyz":
                data[f"box{bead}"] = box[FRAMES]
    start, sbox = read_xyz_frames(os.path.join(cmp_dir, "vmd_start.xyz"))
    data["start"] = start[0]
    data["start_box"] = sbox[0]
    data["frames"] = np.array(FRAMES)
    np.savez_compressed(os.path.join(HERE, "gentest_frames.npz"), **data)

    shutil.copyfile(os.path.join(cmp_dir, "eq.xyz"), os.path.join(HERE, "gentest_eq.xyz"))  # restart file, as written
    with open(os.path.join(cmp_dir, "eq.xyz")) as f:
        tok = f.read().split()
    nm, na, nb = (int(t) for t in tok[:3])
    box = np.array([float(t) for t in tok[3:6]])
    r = np.array([float(t) for t in tok[6:6 + 3 * na * nb]]).reshape(nb, na, 3)

    def last_line(name):
        with open(os.path.join(cmp_dir, name)) as f:
            return np.array([float(t) for t in f.read().split("\n")[-2].split()])

    np.savez_compressed(os.path.join(HERE, "gentest_eq.npz"), r=r, box=box, nm=nm, na=na, nb=nb,
                        E_eq=last_line("E_eq.out"), virial_ke_eq=last_line("virial_ke_eq.out"),
                        V_eq=last_line("V_eq.out"))

    def table(name):
        with open(os.path.join(cmp_dir, name)) as f:
            return np.array([[float(t) for t in ln.split()] for ln in f if ln.strip()])

    np.savez_compressed(os.path.join(HERE, "gentest_md_eq.npz"),
                        **{n.replace(".out", ""): table(n) for n in ("E_pre_eq.out", "E_eq.out", "temp_eq.out",
                                                                      "virial_ke_eq.out", "V_eq.out",
                                                                      "pressure_eq.out", "density_eq.out")})

    out = open(os.path.join(cmp_dir, "output")).read()

    def grab(pattern):
        m = re.search(pattern, out)
        return float(m.group(1))

    kat = {
        "boxlx_bohr": grab(r"\bboxlx\s*=\s*([\d.]+)"),
        "rcut_bohr": grab(r"\brcut\s*=\s*([\d.]+)"),
        "wrcut_bohr": grab(r"\bwrcut\s*=\s*([\d.]+)"),
        "walpha_per_bohr": grab(r"\bwalpha\s*=\s*([\d.]+)"),
        "rkmax_per_bohr": grab(r"\brkmax\s*=\s*([\d.]+)"),
        "kmax": int(grab(r"\bkmax\s*=\s*(\d+)")),
        "initial_energy_per_atom": grab(r"Initial energy =\s*([-\d.]+)"),
        "sigma_bohr": grab(r"with sigma =\s*([\d.]+)"),
        "na": int(grab(r"\bna\s*=\s*(\d+)")),
    }
    with open(os.path.join(HERE, "gentest_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)
    print("wrote", sorted(data), kat)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/RPMD_Mainz")
    main(sys.argv[1])
