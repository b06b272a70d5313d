// gb_common.h -- constants shared by host and device code.
#pragma once

#include <stdint.h>

#include "../../include/gbrpmd.h"

// Accumulator slots: each slot holds [0] energy, [1..9] virial (column-major
// 3x3), [10..15] spare sums.  Raw sums over beads; the host or the finalize
// kernel divides by the bead count of the evaluation (md_forces.f90:104-105).
enum AccSlot : int {
  ACC_EW = 0,      // Ewald (real + reciprocal), unit-box energy/virial before 1/L
  ACC_LJ = 1,      // Lennard-Jones (unscaled sums; x 4 eps / 48 eps)
  ACC_INT = 2,     // intramolecular (last MTS substep for energy, sum over substeps for virial)
  ACC_TEM = 3,     // TEM short-range correction
  ACC_KE = 4,      // virial_ke partial sums: [0] tq1, [1] tq2, [2..4] tq1xyz, [5..7] tq2xyz
  ACC_EW2 = 5,     // second Ewald evaluation (contracted TEM / uncontracted Ewald)
  ACC_LJ2 = 6,
  ACC_TEM2 = 7,
  ACC_INT_V = 8,   // intramolecular energy summed over substeps (diagnostic)
  ACC_NSLOT = 9
};
#define ACC_STRIDE 16

// unit conversions of globals.inc:10-21 (CODATA values the reference uses)
#define GB_TO_K 3.157733e+5        // hartree -> kelvin
#define GB_TO_KJMOL 2625.49963     // hartree -> kJ/mol
#define GB_TO_BAR 2.9421e+8        // hartree/bohr^3 -> bar
#define GB_TO_KGCM3 6.147323129e-3 // electron masses per bohr^3 -> g/cm^3
#define GB_HBAR 1.0

// device status word bits (reported by gbrpmd_ctx_sync)
#define ST_LIST_OVERFLOW 1u
#define ST_NONFINITE 2u
#define ST_RATTLE1 4u
#define ST_RATTLE2 8u
#define ST_CUTOFF 16u

// Twiddle table layout (device global memory, built once per context by the
// host with libm):  tw[m] = cos(2 pi m / TWN), tw[TWN + m] = sin(2 pi m / TWN)
// for m = 0..TWN-1; a power-of-two length n <= TWN reads stride TWN / n.
#define TWN 256
