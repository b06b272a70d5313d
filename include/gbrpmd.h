/*
 * gbrpmd.h -- C ABI of the GB300 ring-polymer force-and-propagation library.
 *
 * The library replaces the reference's per-step RPMD path
 * (DCM-UPB/RPMD_Mainz, Fortran 90) behind the same argument lists.  Every
 * drop-in entry point takes its arguments by reference exactly like the
 * Fortran routine it replaces (double* / int*), arrays in Fortran column-major
 * order:  r(3,na,nb)  ->  r[i + 3*(j + na*k)]  (i = xyz, j = atom, k = bead).
 * Atoms are ordered O,H,H per molecule.  Units are atomic (bohr, hartree,
 * electron masses).  dvdr is +grad V per bead.
 *
 * The COMMON-block state the Fortran routines read implicitly
 * (/oo_param/, /ew_param/, /ew_setup/, /beaddiabatic/, /intra_param/,
 * /geometry/, /correct/, /multiple_ts/, /symmetry/, /constraint/ and the
 * thermostat / barostat module variables, main.f90:53-72) is passed once
 * through gbrpmd_init() so that no COMMON symbol is read from C.
 *
 * Every entry point returns an int status: GB_OK (0) or one of the GB_E*
 * codes below, which stand in for the reference's `stop` statements.
 * gbrpmd_last_error() returns the message of the last failure.
 *
 * Threading: one host thread per library instance (the reference is serial).
 * All device work runs on the library's own CUDA stream; every drop-in call
 * synchronises that stream before it returns.
 */
#ifndef GBRPMD_H
#define GBRPMD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (reference `stop` sites in comments) ------------------ */
#define GB_OK 0
#define GB_E_ARG 1           /* invalid argument / unsupported option          */
#define GB_E_NOINIT 2        /* gbrpmd_init not called                          */
#define GB_E_CUDA 3          /* CUDA runtime error or no device                 */
#define GB_E_LIST 4          /* neighbour list too small  (neigh_list.f90:63)   */
#define GB_E_RATTLE1 5       /* RATTLE stage 1 iterations (md_rattle.f90:149)   */
#define GB_E_RATTLE2 6       /* RATTLE stage 2 iterations (md_rattle.f90:258)   */
#define GB_E_CONTRACT 7      /* contraction count not odd (evolve_pi.f90:344)   */
#define GB_E_NONFINITE 8     /* non-finite force or energy                      */
#define GB_E_CUTOFF 9        /* ewc cut-off larger than half box (correct_tem)  */
#define GB_E_NOMEM 10        /* device memory exhausted / over a size limit     */
#define GB_E_UNSUPPORTED 11  /* option not implemented on the device            */

/* thermostat selector (module thermostat, `therm`, module_thermostat.f90:4) */
#define GB_THERM_NONE 0
#define GB_THERM_AND 1  /* Andersen: resampling happens in the caller (md_eq.f90:311) */
#define GB_THERM_PRG 2  /* global Parrinello kick inside evolve_pi (evolve_pi.f90:73) */
#define GB_THERM_PRL 3  /* local Langevin kick inside evolve_pi  (evolve_pi.f90:75) */

/* barostat selector (module barostat, `baro`, module_barostat.f90:5), used when
   evolve_pi is called with nbaro = 1 (md_eq.f90:55-58: ens = 'NPT') */
#define GB_BARO_NONE 0
#define GB_BARO_BER 1   /* Berendsen, beren_driver (module_barostat.f90:8-129): beren_baro on cubic
                           boxes, beren_baro_nc (one scale per axis) on the others */
#define GB_BARO_MCI 2   /* Monte Carlo volume moves (mc_baro): not on the device path  */

/* intramolecular model selector */
#define GB_INTRA_REFERENCE 0 /* potenl_opt dispatch (md_forces.f90:254-263)         */
#define GB_INTRA_SPCFW 1     /* intra_spcfw (intra_spcfw.f90), commented out in ref */

/* precision selector */
#define GB_PREC_FP64 0  /* plain FP64 everywhere                               */
#define GB_PREC_MIXED 1 /* FP32 pair / reciprocal / transform arithmetic, FP64 totals */

/* Hidden inputs of the reference path (COMMON blocks and module variables). */
typedef struct gb_params {
  /* common /oo_param/ oo_eps,oo_sig,oo_gam,rcut  (main.f90:57); rcut in bohr,
     already clamped to half the shortest box side as main.f90:615-616 does */
  double oo_eps, oo_sig, oo_gam, rcut;
  /* common /ew_param/ alpha,ecut,wm,wh  (main.f90:58) */
  double alpha, ecut, wm, wh;
  /* common /ew_setup/ wrcut,walpha,rkmax,kmax  (setup_options.f90:122) */
  double wrcut, walpha, rkmax;
  int32_t kmax;
  /* common /beaddiabatic/ nbdf1,nbdf2  (main.f90:54) */
  int32_t nbdf1, nbdf2;
  /* common /intra_param/ apot,bpot,alp,alpb  (main.f90:59) */
  double apot, bpot, alp, alpb;
  /* common /geometry/ theta,reoh  (main.f90:55); theta in radians */
  double theta, reoh;
  /* common /correct/ sig  (main.f90:60); bohr */
  double sig;
  /* common /multiple_ts/ mts  (main.f90:56) */
  int32_t mts;
  /* common /symmetry/ iamcub  (main.f90:62) */
  int32_t iamcub;
  /* common /constraint/ nctot,nbond  (main.f90:65) */
  int32_t nctot, nbond;
  /* module thermostat: therm, ttau  (module_thermostat.f90:3-4) */
  int32_t therm;
  double ttau;
  /* module barostat: taub, patm (module_barostat.f90:3-5), in atomic units
     as main.f90:166,263 converts them (taub = tofs * taufs, patm = pres / tobar) */
  double taub, patm;
  /* selectors of this library */
  int32_t intra_model; /* GB_INTRA_* */
  int32_t precision;   /* GB_PREC_*  */
  int32_t baro;        /* GB_BARO_*: module barostat's `baro` */
} gb_params;

/* ---- on-disk formats (io.f90), host only ------------------------------------ */

/* print_structure (io.f90:1-17): "nm na nb", box, r(:,:,:); append != 0 appends */
int gbrpmd_write_structure(const char *path, int append, const double *r, const double *box, int nm, int na,
                           int nb);
/* reads a print_structure restart file (list-directed: any layout); with r
   NULL only nm, na, nb and box, so that r (3 na nb doubles) can be sized */
int gbrpmd_read_structure(const char *path, int *nm, int *na, int *nb, double *box, double *r);
/* one xyz frame of print_vmd_full / _forces / _vels (bead = 0: bead average)
   or print_vmd_bead / _forces / _vels (bead = 1..nb), io.f90:310-770.
   kind 0: positions a = r (Angstrom, oxygens moved into the box unless
   reftraj != 0); 1: forces -(a + a2), a = dvdr, a2 = dvdr2; 2: velocities
   a / mass, a = p.  isotope 0 H2O, 1 D2O, 2 HDO. */
int gbrpmd_write_vmd(const char *path, int append, int kind, int bead, const double *a, const double *a2,
                     const double *mass, const double *box, int na, int nb, int isotope, int reftraj);
/* frame `frame` (0-based) of a print_vmd_* file: box and the atom lines' numbers as printed */
int gbrpmd_read_vmd(const char *path, int frame, int na, double *box, double *xyz);

/* ---- set-up --------------------------------------------------------------- */

/* Stores the hidden inputs; call once after setup_ewald (main.f90:631) and
   again whenever one of them changes.  Replaces the COMMON blocks. */
int gbrpmd_init(const gb_params *params);

/* Reads back the stored hidden inputs. */
int gbrpmd_get_params(gb_params *params);

/* Layout of gb_params as this library was compiled (no counterpart in the
   reference): returns sizeof(gb_params) and writes the byte offset of each
   field, in declaration order (oo_eps .. baro, 32 fields), into offsets[0 ..
   min(nfield, 32) - 1], so that a binding (the Fortran bind(c) type, a ctypes
   mirror) can check its own record against it. */
int gbrpmd_params_layout(int64_t *offsets, int nfield);

/* Message of the last failing call (static storage, never NULL). */
const char *gbrpmd_last_error(void);

/* Releases every device context and buffer the library holds. */
int gbrpmd_finalize(void);

/* ---- drop-in entry points ------------------------------------------------ */

/* replaces subroutine forces(r,v,dvdr,nb,na,boxlxyz,z,virial,iopt)
   (md_forces.f90:1-110).  iopt: 0 full, 1 Ewald+LJ, 2 Ewald, 3 LJ,
   4 intramolecular, 5 TEM short-range Coulomb correction.  v and virial are
   bead-averaged, dvdr is per bead.  r is not modified. */
int gbrpmd_forces(double *r, double *v, double *dvdr, const int *nb, const int *na,
                  const double *boxlxyz, const double *z, double *virial, const int *iopt);

/* No counterpart in the reference.  The FP64 results of gbrpmd_forces with
   iopt = 2 (Ewald energy, gradient and virial of nb configurations, host
   arrays in and out; always FP64, whatever gb_params.precision says), for
   callers that cannot let the library allocate device memory: hosts running
   under a device-memory budget owned by another framework's pool, or code
   that must not trigger cudaMalloc / cudaFree (and their implicit
   synchronisation) while its own streams are busy.  All device work uses one
   16 MiB array that the library reserves at load time on every GPU that loads
   it (held until exit); nothing is allocated per call.  Its device address is
   looked up on the first call made on each device, so make that first call
   before any stream capture.  The work runs on the calling thread's per-thread
   default stream (cudaStreamPerThread).  Calls share the array and the host-side
   k tables, and the array keeps the last call's contents: each call clears
   what must start at zero, and because calls in flight at the same time would
   race on both, a process-wide lock serialises them (a call returns after its
   device work is done).  Limits: na*nb <= 8192 sites, nb <= 64, at most 2048 k
   vectors, and a working set within 16 MiB, mostly the pair list (4 bytes per
   site and slot, slots for 1.1 times a uniform liquid's partners within the
   real-space cut-off plus 48): 216 water molecules at nb = 8 take about 9 MiB
   (GB_E_NOMEM beyond the limits; GB_E_LIST when a site has more partners than
   its slots). */
int gbrpmd_forces_ewald_static(double *r, double *v, double *dvdr, const int *nb, const int *na,
                               const double *boxlxyz, const double *z, double *virial);

/* replaces subroutine full_forces(r,na,nb,v,vew,voo,vint,vir,z,boxlxyz,dvdr,dvdr2)
   (md_forces.f90:305-472): low-frequency (Ewald + LJ, with ring-polymer
   contraction when nbdf1/nbdf2 > 0) into dvdr, intramolecular into dvdr2. */
int gbrpmd_full_forces(double *r, const int *na, const int *nb, double *v, double *vew,
                       double *voo, double *vint, double *vir, const double *z,
                       const double *boxlxyz, double *dvdr, double *dvdr2);

/* replaces subroutine evolve_pi(p,r,v,vew,vlj,vint,dvdr,dvdr2,dt,mass,na,nb,
   boxlxyz,z,beta,vir,vir_lf,irun,nbaro)  (evolve_pi.f90:1-322): one outer
   multiple-time-step RPMD step in the normal-mode representation, with the
   PRG / PRL thermostat kicks (drawing the process-wide random stream with irun)
   and, for nbaro = 1, the Berendsen barostat (baro = GB_BARO_BER; isotropic
   on cubic boxes, per axis on the others), which scales boxlxyz in place and
   reads vir_lf as the previous call left it. */
int gbrpmd_evolve_pi(double *p, double *r, double *v, double *vew, double *vlj,
                     double *vint, double *dvdr, double *dvdr2, const double *dt,
                     const double *mass, const int *na, const int *nb, double *boxlxyz,
                     const double *z, const double *beta, double *vir, double *vir_lf,
                     int *irun, const int *nbaro);

/* replaces subroutine rattle_setup(nm)  (md_rattle.f90:1-31); sets nctot and
   nbond of the stored parameters. */
int gbrpmd_rattle_setup(const int *nm);

/* replaces subroutine rattle_s1(r,rold,p,nm,mass,dt,dvdr,vir,na)
   (md_rattle.f90:33-162) for one bead. */
int gbrpmd_rattle_s1(double *r, const double *rold, double *p, const int *nm,
                     const double *mass, const double *dt, double *dvdr, double *vir,
                     const int *na);

/* replaces subroutine rattle_s2(r,p,nm,mass,dt,dvdr,vir,na)
   (md_rattle.f90:164-271) for one bead. */
int gbrpmd_rattle_s2(double *r, double *p, const int *nm, const double *mass,
                     const double *dt, double *dvdr, double *vir, const int *na);

/* Sweep limit of both RATTLE stages (no counterpart in the reference, whose
   md_rattle.f90 fixes it at 1000, the default here): rattle_s1 / rattle_s2 and
   evolve_rig_pi report GB_E_RATTLE1 / GB_E_RATTLE2 when the last molecule
   needed that many sweeps, as the reference stops.  Process-wide; steps
   already captured in a CUDA graph keep the limit they were captured with.
   Meant for tests of the error path (itmax >= 1). */
int gbrpmd_rattle_set_itmax(const int *itmax);

/* replaces subroutine evolve_rig_pi(p,r,v,v_lf,v_hf,dvdr,dvdr2,dt,mass,na,nb,
   boxlxyz,z,beta,vir,vir_lf,irun,nbaro)  (evolve_rigid.f90:100-224): rigid
   ring-polymer step with primitive bead springs and RATTLE, with the PRG / PRL
   thermostat kicks, and, for nbaro = 1, the Berendsen barostat on the bead
   positions after the step (evolve_rigid.f90:203-213; baro = GB_BARO_BER),
   which reads vir = vir_lf + vir_hf + the caller's vir (the value returned)
   and scales boxlxyz in place; v and vir_lf are those of the box before it. */
int gbrpmd_evolve_rig_pi(double *p, double *r, double *v, double *v_lf, double *v_hf,
                         double *dvdr, double *dvdr2, const double *dt, const double *mass,
                         const int *na, const int *nb, double *boxlxyz, const double *z,
                         const double *beta, double *vir, double *vir_lf, int *irun,
                         const int *nbaro);

/* ---- host-side set-up, in main.f90's start-up order ---------------------- */

/* replaces setup_box_size for the CUB lattice (setup_options.f90:191-270):
   box lengths from the unit-cell counts and the density (g/cm^3) */
int gbrpmd_setup_box_size(const int *ncellxyz, double rho, double wmass, double *boxlxyz,
                          int *nm);
/* replaces cubic (setup_positions.f90:94-150) and the bead copy of
   setup_positions (setup_positions.f90:78-85): r(3, 3*nm, nb) */
int gbrpmd_cubic_lattice(double *r, int nm, int nb, const double *boxlxyz, const int *ncellxyz,
                         double theta, double reoh);
/* replaces setup_ewald (setup_options.f90:104-189): fills wrcut, walpha,
   rkmax, kmax and iamcub of *params from ecut, iamcub, na and the box */
int gbrpmd_setup_ewald(int na, const double *boxlxyz, gb_params *params);
/* replaces sample_rpmd + pshift (module_thermostat.f90:199-264): momenta
   from the library's gaussian stream, centre-of-mass momentum removed */
int gbrpmd_sample_rpmd(double *p, int na, int nb, const double *mass, double beta, int *irun);

/* ---- serial random stream (random.f90:1-72) ----------------------------- */
/* The thermostat kicks inside evolve_pi draw from the reference's global
   ran2/gaussian stream.  The library owns that stream; a Fortran host routes
   its own ran2/gaussian calls here so there is exactly one stream. */

/* replaces function ran2(idum,rmin,rmax)  (random.f90:28-72) */
double gbrpmd_ran2(int *idum, const double *rmin, const double *rmax);
/* replaces function gaussian(idum,sigma)  (random.f90:1-26) */
double gbrpmd_gaussian(int *idum, const double *sigma);

/* ---- resident (device-state) interface ------------------------------------
 * A context keeps p, r, dvdr, dvdr2 of one trajectory in device memory so that
 * repeated steps need no host transfers; the drop-in calls above are built on
 * it.  Arrays passed here use the same r(3,na,nb) layout. */
typedef struct gb_context gb_context;

int gbrpmd_ctx_create(gb_context **ctx, int na, int nb, const double *mass, const double *z);
int gbrpmd_ctx_destroy(gb_context *ctx);
/* uploads r, p, dvdr, dvdr2 (any may be NULL to keep the device copy) and box */
int gbrpmd_ctx_upload(gb_context *ctx, const double *r, const double *p, const double *dvdr,
                      const double *dvdr2, const double *boxlxyz);
/* downloads the device state (any pointer may be NULL) */
int gbrpmd_ctx_download(gb_context *ctx, double *r, double *p, double *dvdr, double *dvdr2);
/* full_forces on the device state: fills dvdr and dvdr2, returns energies */
int gbrpmd_ctx_full_forces(gb_context *ctx, double *v, double *vew, double *voo,
                           double *vint, double *vir);
/* `nsteps` evolve_pi steps on the device state; energies of the last step.
   Asynchronous: results are valid after gbrpmd_ctx_sync. */
int gbrpmd_ctx_evolve(gb_context *ctx, int nsteps, double dt, double beta);
/* waits for the context's stream and reports any device-side status */
int gbrpmd_ctx_sync(gb_context *ctx);
/* energies and virials of the last step: out[0..4] = v, vew, vlj, vint, tv;
   vir[9], vir_lf[9] column-major */
int gbrpmd_ctx_energies(gb_context *ctx, double *out5, double *vir, double *vir_lf);
/* Autotuner (no counterpart in the reference): times `steps` evolve_pi steps
   of (dt, beta) on this context per candidate launch shape -- lanes per site
   of the FP32 real-space Ewald kernel, lanes per oxygen of the FP32 LJ kernel,
   warps per block and sites per lane of the FP32 k-space force kernel,
   molecules per block of
   the fused MTS kernel, pair-list skin -- one
   parameter at a time, keeps the fastest, and leaves the trajectory state as
   it found it.  Shapes are cached per (atoms, beads, precision, MTS,
   contraction, box kind, model) for the process.  Results change only by the
   order of floating-point sums.  out6 (optional): the chosen lanes (Ewald),
   lanes (LJ), molecules per MTS block (0: one wave over the SMs), skin, warps
   per k-space force block, sites per lane of the k-space force kernel.
   Rigid, barostat and PRG/PRL contexts keep the defaults. */
int gbrpmd_ctx_autotune(gb_context *ctx, double dt, double beta, int steps, double *out6);
/* forgets the cached shapes */
void gbrpmd_autotune_reset(void);
/* Random stream owned by the context (no counterpart in the reference, whose
   stream is process-wide): the PRG / PRL thermostat kicks of
   gbrpmd_ctx_evolve draw from a fresh ran2 / gaussian state seeded with idum
   (negative to initialise, as ran2 requires).  The drop-in entry points and
   gbrpmd_run_md_eq draw the process-wide stream with the caller's irun. */
int gbrpmd_ctx_set_rng(gb_context *ctx, int idum);
/* Source of the PRG / PRL kicks' random numbers on this context (no counterpart
   in the reference):
     GB_RNG_REFERENCE  the reference's ran2 / gaussian sequence, drawn on the
                       host in the reference's order (default; a 4096-water,
                       32-bead PRL step then needs ~0.8 M host draws),
     GB_RNG_DEVICE     independent N(0, 1) deviates of a counter-based
                       generator (Philox4x32-10) drawn on the device from
                       `seed` and a device kick counter: no host work, the
                       steps replay from CUDA graphs and may join batches.
   The thermostat is the same; only the numbers differ. */
#define GB_RNG_REFERENCE 0
#define GB_RNG_DEVICE 1
int gbrpmd_ctx_set_rng_mode(gb_context *ctx, int mode, uint64_t seed);
/* evolve_pi's nbaro for gbrpmd_ctx_evolve / gbrpmd_run_md_eq on this context
   (md_eq.f90:55-58: 1 when ens = 'NPT'): the Berendsen barostat scales the box
   and the water centroids inside every step (one synchronisation per step).
   Rigid water: the virial the barostat reads accumulates over the context's
   barostat steps, as the caller's vir does over evolve_rig_pi calls. */
int gbrpmd_ctx_set_nbaro(gb_context *ctx, int nbaro);
/* the context's current box (changed by the barostat) */
int gbrpmd_ctx_box(gb_context *ctx, double *box3);
/* Resets the process-wide ran2 / gaussian state (shuffle table, second
   generator, cached gaussian) to the state the reference has at program start. */
void gbrpmd_rng_reset(void);
/* The estimators md_eq prints at an output step (md_eq.f90:190-299), from the
   resident state left by the last evolve (bead representation) and the
   energies / virial of that evaluation; synchronises.  out[16]:
     0 tk     kinetic_rpmd (kinetic.f90:248-265)
     1 vrp    ring-polymer spring energy, omega_n = nb / (beta hbar) (md_eq.f90:252-270)
     2 nb*v + tk + vrp   the conserved RPMD energy (md_eq.f90:274, not divided by na)
     3 temperature in K (md_eq.f90:272)
     4 tv, 5..7 tvxyz    virial_ke (kinetic.f90:1-54)
     8 pressure in hartree/bohr^3 with the LJ tail (md_pressure.f90:1-56)
     9..11 dipx, dipy, dipz, 12 dip2, 13 dipm   dipole (md_tools.f90:75-128)
     14 density in g/cm^3 (md_eq.f90:196-198), 15 v (bead-averaged potential)
   rcm [nm][3] (optional): center_water (md_tools.f90:367-390); mdip [nm][3]
   (optional): bead-averaged molecular dipoles (m_dipole). */
int gbrpmd_ctx_estimators(gb_context *ctx, double beta, double *out16, double *rcm, double *mdip);
/* the CUDA stream (cudaStream_t) the context launches on */
void *gbrpmd_ctx_stream(gb_context *ctx);
/* number of kernel launches issued by this context since creation */
int64_t gbrpmd_ctx_launch_count(gb_context *ctx);
/* CUDA-event timing of the library's kernel regions on this context (for
   profiling and roofline reports; adds one synchronisation per pair list) */
int gbrpmd_ctx_set_profiling(gb_context *ctx, int on);
/* per region: total milliseconds, work units, launches since the last call;
   regions: 0 multiple-time-step block, 1 pair lists, 2 real-space Ewald,
   3 structure factors, 4 k-space weights, 5 k-space forces, 6 Lennard-Jones,
   7 TEM correction, 8 contraction and kicks, 9 M-site, 10 RATTLE */
int gbrpmd_ctx_region_times(gb_context *ctx, double *ms, double *units, int *counts, int nregion);
/* Measurement (no counterpart in the reference): the normal-mode transform of
   nrows rows of 32 beads (realft, fourier.f90:16-63, scaled by 1/sqrt(32)),
   timed as real FFTs in FP32 registers with split twiddles (two lanes per
   row, and four) and as a dense product on the tensor cores (mma.sync TF32,
   rows split in two terms, transform matrices in three), reps forward +
   inverse round trips per row between one load and one store.  out12: ms per
   transform (lane-pair FFT, tensor cores), round-trip relative error (pair
   FFT) and mean gain per round trip, the same for the tensor cores, forward
   relative error against an FP64 direct sum (pair FFT, tensor cores); then ms
   per transform, round-trip error, gain and forward error of the lane-quad
   FFT.  Allocates and synchronises. */
int gbrpmd_bench_nm_transform(int nrows, int reps, double *out12);
/* Watched kernel (no counterpart in the reference): a pair of timing events
   around the launch of one region's kernel (0 multiple-time-step block,
   2 real-space Ewald, 5 k-space forces, 6 Lennard-Jones; -1 stops watching),
   recorded on the stream the kernel is launched on and captured into the step
   graph with it, so that ordinary (graph-replayed, forked) steps report that
   kernel's own duration.  Setting it drops the step graph. */
int gbrpmd_ctx_watch_region(gb_context *ctx, int region);
/* milliseconds between the watch events of the last step that recorded them
   (synchronises); GB_E_ARG when none was recorded */
int gbrpmd_ctx_watch_ms(gb_context *ctx, float *ms);
/* Pair-list skin (no counterpart in the reference, which rebuilds its cell
   lists at every call): each list of the context (real-space Ewald, LJ, TEM)
   keeps a superset at cut-off * (1 + fraction), rebuilt on the device only
   when a point has moved by more than half the skin since its last rebuild, and
   filters it into the exact pair set at every use, so results do not depend on
   the fraction.  Default 0.1 (environment GBRPMD_LIST_SKIN); 0 rebuilds every
   list at every use. */
int gbrpmd_ctx_set_list_skin(gb_context *ctx, double fraction);
/* rebuilds of the three skin lists since the context was created (synchronises) */
int gbrpmd_ctx_list_rebuilds(gb_context *ctx, unsigned *counts3);
/* diagnostics (synchronises): longest list and capacity of the Ewald, LJ and
   TEM skin lists and of the exact list last built, as 4 (max, cap) pairs */
int gbrpmd_ctx_list_occupancy(gb_context *ctx, int *out8);
/* CUDA-graph replay of gbrpmd_ctx_evolve / gbrpmd_evolve_pi steps (no counterpart
   in the reference): on by default (environment GBRPMD_GRAPHS=0 turns it off);
   the second step with unchanged parameters, dt, beta and box is captured and
   later steps replay it.  Results do not depend on the setting. */
int gbrpmd_ctx_set_graphs(gb_context *ctx, int on);
/* Parameters owned by one context (instead of the set given to gbrpmd_init),
   as batch replicas of different boxes and Ewald set-ups need them. */
int gbrpmd_ctx_set_params(gb_context *ctx, const gb_params *params);

/* ---- batched replicas (no counterpart in the reference, which runs one
   trajectory per process; batch.cpp) ----
   A batch advances resident contexts of any molecule and bead counts together:
   each step is one CUDA graph with one branch per replica (captured on the
   second step after a membership change, replayed afterwards).  Every replica
   keeps its own parameters (gbrpmd_ctx_set_params), dt, beta and, with
   thresh > 0, its own Andersen test (md_eq.f90:311-315) on ran2 stream irun.
   Call gbrpmd_batch_sync before reading a replica (gbrpmd_ctx_sync,
   gbrpmd_ctx_download); queue no other work on a replica while it is in a batch. */
typedef struct gb_batch gb_batch;
int gbrpmd_batch_create(gb_batch **batch);
int gbrpmd_batch_destroy(gb_batch *batch);
int gbrpmd_batch_add(gb_batch *batch, gb_context *ctx, double dt, double beta, double thresh, int irun);
int gbrpmd_batch_remove(gb_batch *batch, gb_context *ctx);
int gbrpmd_batch_size(gb_batch *batch);
int gbrpmd_batch_step(gb_batch *batch, int nsteps);
int gbrpmd_batch_sync(gb_batch *batch);
/* gbrpmd_ctx_autotune on every replica (each distinct shape timed once) */
int gbrpmd_batch_autotune(gb_batch *batch, int steps);
void *gbrpmd_batch_stream(gb_batch *batch);

/* Device memory: what a context holds now, and what one of (na, nb) with
   these parameters will hold once it has stepped (the server's admission test). */
size_t gbrpmd_ctx_device_bytes(gb_context *ctx);
size_t gbrpmd_estimate_device_bytes(int na, int nb, const gb_params *params);

/* ---- serving loop (no counterpart in the reference; server.cpp) ----
   Continuous batching of independent trajectory requests.  A request brings
   its system (na, nb, parameters, masses, charges, box), its starting state in
   host arrays the caller keeps valid until the request is polled (final r, p,
   dvdr, dvdr2 are written back into them; dvdr/dvdr2 may both be NULL, then
   full_forces supplies the starting forces), nsteps evolve_pi steps, dt, beta
   and an optional Andersen test.  gbrpmd_server_tick admits queued requests in
   arrival order while a slot is free and the estimated device footprint fits
   the byte budget, advances all resident trajectories by up to `steps` steps
   in one batch, and retires finished ones.  gbrpmd_server_poll returns
   finished requests with status, seconds from submission to admission and to
   completion, and last-step energies (v, vew, vlj, vint, tv). */
typedef struct gb_server gb_server;
int gbrpmd_server_create(gb_server **server, size_t budget_bytes, int max_slots);
int gbrpmd_server_destroy(gb_server *server);
int gbrpmd_server_submit(gb_server *server, int na, int nb, const gb_params *params, const double *mass,
                         const double *z, const double *boxlxyz, double *r, double *p, double *dvdr,
                         double *dvdr2, int forces_given, int nsteps, double dt, double beta, double thresh,
                         int irun, int64_t *id);
int gbrpmd_server_tick(gb_server *server, int steps);
int gbrpmd_server_counts(gb_server *server, int *queued, int *active, int *finished, size_t *bytes_in_use);
int gbrpmd_server_poll(gb_server *server, int max, int64_t *ids, int *status, double *t_admit,
                       double *t_done, double *energies5, int *n);

/* the md_eq step loop (md_eq.f90:182-323) on the device state: nsteps
   evolve_pi steps, each followed by the Andersen test ran2(irun) < thresh
   that resamples all momenta (md_eq.f90:311-315) when therm is AND.
   energies (4 per step: v, vew, vlj, vint) may be NULL. */
int gbrpmd_run_md_eq(gb_context *ctx, int nsteps, double dt, double beta, double thresh,
                     int *irun, double *energies);

/* Self-check of the conversions the mixed-precision kernels build from
   integer operations instead of FP64 instructions (no counterpart in the
   reference): for n doubles in[] (host arrays), f32 = in rounded to the
   nearest FP32 (ties to even), hi + lo = in split into two FP32 (hi
   truncated to 24 bits, lo the rest rounded; lo is zero below 2^-75), back
   = f32 widened exactly.
   Outside the FP32 normal range values flush to a signed zero or saturate to
   an infinity. */
int gbrpmd_selftest_conversions(const double *in, int n, float *f32, float *hi, float *lo, double *back);

#ifdef __cplusplus
}
#endif

#endif /* GBRPMD_H */
