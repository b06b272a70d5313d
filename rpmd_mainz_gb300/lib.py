"""ctypes bindings of libgbrpmd.so with the reference's call signatures.

The functions below mirror the Fortran routines the library replaces
(md_forces.f90 `forces` / `full_forces`, evolve_pi.f90 `evolve_pi`,
md_rattle.f90 `rattle_setup` / `rattle_s1` / `rattle_s2`, evolve_rigid.f90
`evolve_rig_pi`): same arguments, same meaning, arrays shaped (nb, na, 3) in
numpy, which is the memory order of the Fortran r(3, na, nb).  A non-zero
status from the library raises GbError with the library's message, as the
reference would `stop`.

`load()` fails loudly when the library has not been built; there is no
fallback implementation.
"""
import ctypes as C
import os
import re

import numpy as np

from .abi import GbParams, STATUS_NAMES

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgbrpmd.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "gbrpmd.h")

_lib = None

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)


class GbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gbrpmd error {code} ({STATUS_NAMES.get(code, '?')}): {msg}")
        self.code = code


def header_functions():
    """Names of every function declared in include/gbrpmd.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbrpmd_\w+)\s*\(", text)))


def load(path=None):
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    lib.gbrpmd_last_error.restype = C.c_char_p
    lib.gbrpmd_ran2.restype = C.c_double
    lib.gbrpmd_ran2.argtypes = [I, D, D]
    lib.gbrpmd_gaussian.restype = C.c_double
    lib.gbrpmd_gaussian.argtypes = [I, D]
    lib.gbrpmd_ctx_stream.restype = C.c_void_p
    lib.gbrpmd_ctx_stream.argtypes = [C.c_void_p]
    lib.gbrpmd_ctx_launch_count.restype = C.c_int64
    lib.gbrpmd_ctx_launch_count.argtypes = [C.c_void_p]
    lib.gbrpmd_ctx_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, D, D]
    for name in ["gbrpmd_ctx_destroy", "gbrpmd_ctx_sync"]:
        getattr(lib, name).argtypes = [C.c_void_p]
    lib.gbrpmd_ctx_upload.argtypes = [C.c_void_p, D, D, D, D, D]
    lib.gbrpmd_ctx_download.argtypes = [C.c_void_p, D, D, D, D]
    lib.gbrpmd_ctx_full_forces.argtypes = [C.c_void_p, D, D, D, D, D]
    lib.gbrpmd_ctx_evolve.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double]
    lib.gbrpmd_ctx_energies.argtypes = [C.c_void_p, D, D, D]
    lib.gbrpmd_ctx_estimators.argtypes = [C.c_void_p, C.c_double, D, D, D]
    lib.gbrpmd_ctx_set_rng.argtypes = [C.c_void_p, C.c_int]
    lib.gbrpmd_ctx_set_rng_mode.argtypes = [C.c_void_p, C.c_int, C.c_uint64]
    lib.gbrpmd_ctx_set_nbaro.argtypes = [C.c_void_p, C.c_int]
    lib.gbrpmd_ctx_box.argtypes = [C.c_void_p, D]
    lib.gbrpmd_rng_reset.restype = None
    lib.gbrpmd_write_structure.argtypes = [C.c_char_p, C.c_int, D, D, C.c_int, C.c_int, C.c_int]
    lib.gbrpmd_read_structure.argtypes = [C.c_char_p, I, I, I, D, D]
    lib.gbrpmd_write_vmd.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, D, D, D, D, C.c_int, C.c_int, C.c_int,
                                     C.c_int]
    lib.gbrpmd_read_vmd.argtypes = [C.c_char_p, C.c_int, C.c_int, D, D]
    lib.gbrpmd_ctx_autotune.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int, D]
    lib.gbrpmd_autotune_reset.restype = None
    lib.gbrpmd_batch_autotune.argtypes = [C.c_void_p, C.c_int]
    lib.gbrpmd_ctx_set_list_skin.argtypes = [C.c_void_p, C.c_double]
    lib.gbrpmd_ctx_list_rebuilds.argtypes = [C.c_void_p, C.POINTER(C.c_uint)]
    lib.gbrpmd_ctx_set_graphs.argtypes = [C.c_void_p, C.c_int]
    lib.gbrpmd_bench_nm_transform.argtypes = [C.c_int, C.c_int, D]
    lib.gbrpmd_ctx_watch_region.argtypes = [C.c_void_p, C.c_int]
    lib.gbrpmd_ctx_watch_ms.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
    lib.gbrpmd_ctx_list_occupancy.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    lib.gbrpmd_ctx_set_params.argtypes = [C.c_void_p, C.c_void_p]
    lib.gbrpmd_run_md_eq.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_int),
                                     C.c_void_p]
    lib.gbrpmd_batch_create.argtypes = [C.POINTER(C.c_void_p)]
    lib.gbrpmd_batch_destroy.argtypes = [C.c_void_p]
    lib.gbrpmd_batch_add.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int]
    lib.gbrpmd_batch_remove.argtypes = [C.c_void_p, C.c_void_p]
    lib.gbrpmd_batch_size.argtypes = [C.c_void_p]
    lib.gbrpmd_batch_step.argtypes = [C.c_void_p, C.c_int]
    lib.gbrpmd_batch_sync.argtypes = [C.c_void_p]
    lib.gbrpmd_batch_stream.restype = C.c_void_p
    lib.gbrpmd_batch_stream.argtypes = [C.c_void_p]
    lib.gbrpmd_ctx_device_bytes.restype = C.c_size_t
    lib.gbrpmd_ctx_device_bytes.argtypes = [C.c_void_p]
    lib.gbrpmd_estimate_device_bytes.restype = C.c_size_t
    lib.gbrpmd_estimate_device_bytes.argtypes = [C.c_int, C.c_int, C.c_void_p]
    lib.gbrpmd_server_create.argtypes = [C.POINTER(C.c_void_p), C.c_size_t, C.c_int]
    lib.gbrpmd_server_destroy.argtypes = [C.c_void_p]
    lib.gbrpmd_server_submit.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, D, D, D, D, D, D, D, C.c_int,
                                         C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_int64)]
    lib.gbrpmd_server_tick.argtypes = [C.c_void_p, C.c_int]
    lib.gbrpmd_server_counts.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_size_t)]
    lib.gbrpmd_server_poll.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int), D, D, D,
                                       C.POINTER(C.c_int)]
    _lib = lib
    return lib


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(D)


def _check(st):
    if st != 0:
        raise GbError(st, load().gbrpmd_last_error().decode())


def _arr(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def init(params: GbParams):
    _check(load().gbrpmd_init(C.byref(params)))


def get_params() -> GbParams:
    p = GbParams()
    _check(load().gbrpmd_get_params(C.byref(p)))
    return p


def write_structure(path, r, box, append=False):
    """print_structure (io.f90:1-17) of r (nb, na, 3) and the box."""
    r = _arr(r)
    nb, na, _ = r.shape
    _check(load().gbrpmd_write_structure(str(path).encode(), int(append), _ptr(r), _ptr(_arr(box)), na // 3, na, nb))


def read_structure(path):
    """A print_structure restart file: (r (nb, na, 3), box)."""
    nm, na, nb = C.c_int(), C.c_int(), C.c_int()
    box = np.zeros(3)
    _check(load().gbrpmd_read_structure(str(path).encode(), C.byref(nm), C.byref(na), C.byref(nb), _ptr(box), None))
    r = np.zeros((nb.value, na.value, 3))
    _check(load().gbrpmd_read_structure(str(path).encode(), C.byref(nm), C.byref(na), C.byref(nb), _ptr(box),
                                        _ptr(r)))
    return r, box


VMD_KIND = {"xyz": 0, "frc": 1, "vel": 2}


def write_vmd(path, kind, a, box, a2=None, mass=None, bead=0, append=False, isotope=0, reftraj=False):
    """One frame of print_vmd_full* (bead 0) or print_vmd_bead* (bead 1..nb);
    kind "xyz" (a = r), "frc" (a = dvdr, a2 = dvdr2) or "vel" (a = p, with mass)."""
    a = _arr(a)
    nb, na, _ = a.shape
    _check(load().gbrpmd_write_vmd(str(path).encode(), int(append), VMD_KIND[kind], int(bead), _ptr(a),
                                   _ptr(None if a2 is None else _arr(a2)), _ptr(None if mass is None else _arr(mass)),
                                   _ptr(_arr(box)), na, nb, int(isotope), int(reftraj)))


def read_vmd(path, na, frame=0):
    """Frame `frame` of a print_vmd_* file: (numbers (na, 3) as printed, box as printed)."""
    box, xyz = np.zeros(3), np.zeros((na, 3))
    _check(load().gbrpmd_read_vmd(str(path).encode(), int(frame), int(na), _ptr(box), _ptr(xyz)))
    return xyz, box


def autotune_reset():
    """Forget the autotuner's cached shapes."""
    load().gbrpmd_autotune_reset()


def rng_reset():
    """Process-wide ran2 / gaussian state back to the reference's start-up state."""
    load().gbrpmd_rng_reset()


def last_error():
    """Message of the library's last error."""
    return load().gbrpmd_last_error().decode()


def finalize():
    _check(load().gbrpmd_finalize())


def forces(r, box, z, iopt):
    """forces(r,v,dvdr,nb,na,boxlxyz,z,virial,iopt) -> (v, dvdr, virial[3,3])."""
    r = _arr(r)
    nb, na, _ = r.shape
    dvdr = np.zeros_like(r)
    vir = np.zeros(9)
    v = C.c_double()
    _check(load().gbrpmd_forces(_ptr(r), C.byref(v), _ptr(dvdr), C.byref(C.c_int(nb)), C.byref(C.c_int(na)),
                                _ptr(_arr(box)), _ptr(_arr(z)), _ptr(vir), C.byref(C.c_int(iopt))))
    return v.value, dvdr, vir.reshape(3, 3, order="F")


def full_forces(r, box, z):
    """full_forces(r,na,nb,v,vew,voo,vint,vir,z,boxlxyz,dvdr,dvdr2)."""
    r = _arr(r)
    nb, na, _ = r.shape
    dvdr = np.zeros_like(r)
    dvdr2 = np.zeros_like(r)
    vir = np.zeros(9)
    v, vew, voo, vint = (C.c_double() for _ in range(4))
    _check(load().gbrpmd_full_forces(_ptr(r), C.byref(C.c_int(na)), C.byref(C.c_int(nb)), C.byref(v),
                                     C.byref(vew), C.byref(voo), C.byref(vint), _ptr(vir), _ptr(_arr(z)),
                                     _ptr(_arr(box)), _ptr(dvdr), _ptr(dvdr2)))
    return dict(v=v.value, vew=vew.value, voo=voo.value, vint=vint.value, dvdr=dvdr, dvdr2=dvdr2,
                vir=vir.reshape(3, 3, order="F"))


class State:
    """Trajectory arrays the caller owns, as the Fortran host owns p, r, dvdr, dvdr2."""

    def __init__(self, r, p, dvdr, dvdr2, box):
        self.r = _arr(r).copy()
        self.p = _arr(p).copy()
        self.dvdr = _arr(dvdr).copy()
        self.dvdr2 = _arr(dvdr2).copy()
        self.box = _arr(box).copy()
        self.vir = np.zeros(9)
        self.vir_lf = np.zeros(9)


def evolve_pi(state: State, dt, mass, z, beta, irun=0, nbaro=0):
    """evolve_pi(p,r,v,vew,vlj,vint,dvdr,dvdr2,dt,mass,na,nb,boxlxyz,z,beta,vir,vir_lf,irun,nbaro).
    irun: an int, or a ctypes c_int that the thermostat draws advance in place;
    state.box is scaled in place by the barostat (nbaro = 1)."""
    nb, na, _ = state.r.shape
    v, vew, vlj, vint = (C.c_double() for _ in range(4))
    idum = irun if isinstance(irun, C.c_int) else C.c_int(irun)
    _check(load().gbrpmd_evolve_pi(_ptr(state.p), _ptr(state.r), C.byref(v), C.byref(vew), C.byref(vlj),
                                   C.byref(vint), _ptr(state.dvdr), _ptr(state.dvdr2), C.byref(C.c_double(dt)),
                                   _ptr(_arr(mass)), C.byref(C.c_int(na)), C.byref(C.c_int(nb)), _ptr(state.box),
                                   _ptr(_arr(z)), C.byref(C.c_double(beta)), _ptr(state.vir), _ptr(state.vir_lf),
                                   C.byref(idum), C.byref(C.c_int(nbaro))))
    return dict(v=v.value, vew=vew.value, vlj=vlj.value, vint=vint.value)


def rattle_setup(nm):
    _check(load().gbrpmd_rattle_setup(C.byref(C.c_int(nm))))


def rattle_s1(r, rold, p, mass, dt, dvdr):
    """One bead: r, rold, p, dvdr shaped (na, 3); returns vir[3,3] (arrays updated in place)."""
    na = r.shape[0]
    vir = np.zeros(9)
    _check(load().gbrpmd_rattle_s1(_ptr(r), _ptr(_arr(rold)), _ptr(p), C.byref(C.c_int(na // 3)), _ptr(_arr(mass)),
                                   C.byref(C.c_double(dt)), _ptr(dvdr), _ptr(vir), C.byref(C.c_int(na))))
    return vir.reshape(3, 3, order="F")


def rattle_s2(r, p, mass, dt, dvdr):
    na = r.shape[0]
    vir = np.zeros(9)
    _check(load().gbrpmd_rattle_s2(_ptr(r), _ptr(p), C.byref(C.c_int(na // 3)), _ptr(_arr(mass)),
                                   C.byref(C.c_double(dt)), _ptr(dvdr), _ptr(vir), C.byref(C.c_int(na))))
    return vir.reshape(3, 3, order="F")


def evolve_rig_pi(state: State, dt, mass, z, beta, irun=0, nbaro=0):
    """evolve_rig_pi(p,r,v,v_lf,v_hf,dvdr,dvdr2,dt,mass,na,nb,boxlxyz,z,beta,vir,vir_lf,irun,nbaro);
    state.vir accumulates as the reference's caller's vir does; state.box is
    scaled in place by the barostat (nbaro = 1)."""
    nb, na, _ = state.r.shape
    v, v_lf, v_hf = C.c_double(), C.c_double(), C.c_double()
    _check(load().gbrpmd_evolve_rig_pi(_ptr(state.p), _ptr(state.r), C.byref(v), C.byref(v_lf), C.byref(v_hf),
                                       _ptr(state.dvdr), _ptr(state.dvdr2), C.byref(C.c_double(dt)),
                                       _ptr(_arr(mass)), C.byref(C.c_int(na)), C.byref(C.c_int(nb)),
                                       _ptr(state.box), _ptr(_arr(z)), C.byref(C.c_double(beta)),
                                       _ptr(state.vir), _ptr(state.vir_lf), C.byref(C.c_int(irun)),
                                       C.byref(C.c_int(nbaro))))
    return dict(v=v.value)


class Context:
    """Resident trajectory: state kept in device memory between steps."""

    def __init__(self, na, nb, mass, z):
        self.na, self.nb = na, nb
        self.h = C.c_void_p()
        _check(load().gbrpmd_ctx_create(C.byref(self.h), na, nb, _ptr(_arr(mass)), _ptr(_arr(z))))

    def close(self):
        if self.h:
            load().gbrpmd_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, r=None, p=None, dvdr=None, dvdr2=None, box=None):
        keep = [None if a is None else _arr(a) for a in (r, p, dvdr, dvdr2, box)]
        _check(load().gbrpmd_ctx_upload(self.h, *[_ptr(a) for a in keep]))
        self.sync()

    def download(self):
        shape = (self.nb, self.na, 3)
        r, p, f, f2 = (np.zeros(shape) for _ in range(4))
        _check(load().gbrpmd_ctx_download(self.h, _ptr(r), _ptr(p), _ptr(f), _ptr(f2)))
        return r, p, f, f2

    def full_forces(self):
        v, vew, voo, vint = (C.c_double() for _ in range(4))
        vir = np.zeros(9)
        _check(load().gbrpmd_ctx_full_forces(self.h, C.byref(v), C.byref(vew), C.byref(voo), C.byref(vint), _ptr(vir)))
        return dict(v=v.value, vew=vew.value, voo=voo.value, vint=vint.value, vir=vir.reshape(3, 3, order="F"))

    def evolve(self, nsteps, dt, beta):
        _check(load().gbrpmd_ctx_evolve(self.h, nsteps, dt, beta))

    def sync(self):
        _check(load().gbrpmd_ctx_sync(self.h))

    def energies(self):
        out = np.zeros(5)
        vir = np.zeros(9)
        vir_lf = np.zeros(9)
        _check(load().gbrpmd_ctx_energies(self.h, _ptr(out), _ptr(vir), _ptr(vir_lf)))
        return dict(v=out[0], vew=out[1], vlj=out[2], vint=out[3], tv=out[4], vir=vir.reshape(3, 3, order="F"),
                    vir_lf=vir_lf.reshape(3, 3, order="F"))

    def autotune(self, dt, beta, steps=10):
        """Launch shapes timed on this context (gbrpmd_ctx_autotune); returns the choice."""
        out = np.zeros(6)
        _check(load().gbrpmd_ctx_autotune(self.h, C.c_double(dt), C.c_double(beta), int(steps), _ptr(out)))
        return dict(ew_np=int(out[0]), lj_np=int(out[1]), mts_mpb=int(out[2]), skin=float(out[3]), rf_g=int(out[4]),
                    rf_ns=int(out[5]))

    def set_rng(self, idum):
        """Context-owned random stream for the PRG / PRL kicks of evolve()."""
        _check(load().gbrpmd_ctx_set_rng(self.h, int(idum)))

    def set_rng_mode(self, mode, seed=0):
        """Random numbers of the PRG / PRL kicks: "reference" (host ran2 / gaussian)
        or "device" (Philox4x32-10 on the device, seeded)."""
        _check(load().gbrpmd_ctx_set_rng_mode(self.h, {"reference": 0, "device": 1}[mode], int(seed)))

    def set_nbaro(self, nbaro):
        """evolve_pi's nbaro for evolve() / run_md_eq() (1: Berendsen barostat)."""
        _check(load().gbrpmd_ctx_set_nbaro(self.h, int(nbaro)))

    @property
    def box(self):
        b = np.zeros(3)
        _check(load().gbrpmd_ctx_box(self.h, _ptr(b)))
        return b

    ESTIMATORS = ("tk", "vrp", "econs", "temp", "tv", "tvx", "tvy", "tvz", "pres", "dipx", "dipy", "dipz", "dip2",
                  "dipm", "den", "v")

    def estimators(self, beta, centroids=False, dipoles=False):
        """md_eq's output-step estimators on the resident state (gbrpmd_ctx_estimators):
        a dict of ESTIMATORS, plus 'rcm' / 'mdip' arrays (nm, 3) when asked."""
        nm = self.na // 3
        out = np.zeros(16)
        rcm = np.zeros((nm, 3)) if centroids else None
        mdip = np.zeros((nm, 3)) if dipoles else None
        _check(load().gbrpmd_ctx_estimators(self.h, C.c_double(beta), _ptr(out), _ptr(rcm), _ptr(mdip)))
        d = dict(zip(self.ESTIMATORS, out.tolist()))
        if centroids:
            d["rcm"] = rcm
        if dipoles:
            d["mdip"] = mdip
        return d

    @property
    def stream(self):
        return load().gbrpmd_ctx_stream(self.h)

    @property
    def launches(self):
        return load().gbrpmd_ctx_launch_count(self.h)

    def set_list_skin(self, fraction):
        """Pair-list skin as a fraction of each cut-off (0: rebuild at every use)."""
        _check(load().gbrpmd_ctx_set_list_skin(self.h, C.c_double(fraction)))

    def set_params(self, params):
        """Parameters owned by this context (a batch replica needs them)."""
        _check(load().gbrpmd_ctx_set_params(self.h, C.byref(params)))

    def run_md_eq(self, nsteps, dt, beta, thresh, irun: C.c_int, energies=False):
        """md_eq step loop with the Andersen test; irun is advanced in place."""
        e = np.zeros(4 * nsteps) if energies else None
        _check(load().gbrpmd_run_md_eq(self.h, nsteps, dt, beta, thresh, C.byref(irun),
                                       None if e is None else _ptr(e)))
        return None if e is None else e.reshape(nsteps, 4)

    @property
    def device_bytes(self):
        return load().gbrpmd_ctx_device_bytes(self.h)

    def list_occupancy(self):
        """(max, cap) of the Ewald, LJ and TEM skin lists and of the exact list."""
        out = (C.c_int * 8)()
        _check(load().gbrpmd_ctx_list_occupancy(self.h, out))
        return {k: (out[2 * i], out[2 * i + 1]) for i, k in enumerate(("ewald", "lj", "tem", "exact"))}

    def set_graphs(self, on):
        """CUDA-graph replay of evolve steps (on by default)."""
        _check(load().gbrpmd_ctx_set_graphs(self.h, 1 if on else 0))

    WATCH = {"mts_block": 0, "ewald_real": 2, "recip_force": 5, "lj": 6}

    def watch(self, region):
        """Time one region's kernel inside ordinary (graph-replayed) steps:
        a region name of WATCH, or None to stop."""
        _check(load().gbrpmd_ctx_watch_region(self.h, -1 if region is None else self.WATCH[region]))

    def watch_ms(self):
        """Duration of the watched kernel in the last step (synchronises)."""
        ms = C.c_float()
        _check(load().gbrpmd_ctx_watch_ms(self.h, C.byref(ms)))
        return ms.value

    def list_rebuilds(self):
        """Rebuilds of the (Ewald, LJ, TEM) skin lists since creation."""
        out = (C.c_uint * 3)()
        _check(load().gbrpmd_ctx_list_rebuilds(self.h, out))
        return tuple(out)


def bench_nm_transform(nrows, reps=6):
    """Normal-mode transform of nrows rows of 32 beads: in-register FFT against
    the tensor-core product (gbrpmd_bench_nm_transform)."""
    out = np.zeros(12)
    _check(load().gbrpmd_bench_nm_transform(int(nrows), int(reps), _ptr(out)))
    keys = ("ms_per_transform_fft", "ms_per_transform_tensor", "roundtrip_rel_err_fft", "gain_per_roundtrip_fft",
            "roundtrip_rel_err_tensor", "gain_per_roundtrip_tensor", "forward_rel_err_fft", "forward_rel_err_tensor",
            "ms_per_transform_fft_quad", "roundtrip_rel_err_fft_quad", "gain_per_roundtrip_fft_quad",
            "forward_rel_err_fft_quad")
    return dict(zip(keys, out.tolist()))


def ran2(idum: C.c_int, rmin=0.0, rmax=1.0):
    return load().gbrpmd_ran2(C.byref(idum), C.byref(C.c_double(rmin)), C.byref(C.c_double(rmax)))


def gaussian(idum: C.c_int, sigma=1.0):
    return load().gbrpmd_gaussian(C.byref(idum), C.byref(C.c_double(sigma)))


class Batch:
    """Resident contexts advanced together, one CUDA-graph launch per step."""

    def __init__(self):
        self.h = C.c_void_p()
        self.members = []
        _check(load().gbrpmd_batch_create(C.byref(self.h)))

    def add(self, ctx, dt, beta, thresh=0.0, irun=0):
        _check(load().gbrpmd_batch_add(self.h, ctx.h, dt, beta, thresh, irun))
        self.members.append(ctx)

    def remove(self, ctx):
        _check(load().gbrpmd_batch_remove(self.h, ctx.h))
        self.members.remove(ctx)

    def autotune(self, steps=10):
        """gbrpmd_batch_autotune: launch shapes of every replica (cached per shape)."""
        _check(load().gbrpmd_batch_autotune(self.h, int(steps)))

    def step(self, nsteps=1):
        _check(load().gbrpmd_batch_step(self.h, nsteps))

    def sync(self):
        _check(load().gbrpmd_batch_sync(self.h))

    @property
    def stream(self):
        return load().gbrpmd_batch_stream(self.h)

    def __len__(self):
        return load().gbrpmd_batch_size(self.h)

    def close(self):
        if self.h:
            load().gbrpmd_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate_device_bytes(na, nb, params):
    return load().gbrpmd_estimate_device_bytes(na, nb, C.byref(params))


class Server:
    """Continuous batching of trajectory requests with resident device state."""

    def __init__(self, budget_bytes, max_slots):
        self.h = C.c_void_p()
        self.keep = {}
        _check(load().gbrpmd_server_create(C.byref(self.h), int(budget_bytes), int(max_slots)))

    def submit(self, system, r, p, nsteps, dvdr=None, dvdr2=None, thresh=0.0, irun=0, params=None,
               dt=None, beta=None):
        """Queue a trajectory.  r, p (and dvdr, dvdr2; without them the server
        computes the starting forces) are copied; poll() hands back the final state."""
        s = system
        prm = params if params is not None else s["params"]
        given = dvdr is not None
        arrs = dict(r=_arr(r).copy(), p=_arr(p).copy(), mass=_arr(s["mass"]), z=_arr(s["z"]), box=_arr(s["box"]),
                    dvdr=_arr(dvdr).copy() if given else np.zeros_like(_arr(r)),
                    dvdr2=_arr(dvdr2).copy() if given else np.zeros_like(_arr(r)), params=prm)
        rid = C.c_int64()
        _check(load().gbrpmd_server_submit(self.h, s["na"], s["nb"], C.byref(prm), _ptr(arrs["mass"]), _ptr(arrs["z"]),
                                           _ptr(arrs["box"]), _ptr(arrs["r"]), _ptr(arrs["p"]), _ptr(arrs["dvdr"]),
                                           _ptr(arrs["dvdr2"]), 1 if given else 0, int(nsteps),
                                           s["dt"] if dt is None else dt, s["beta"] if beta is None else beta,
                                           thresh, irun, C.byref(rid)))
        self.keep[rid.value] = arrs
        return rid.value

    def tick(self, steps=1):
        _check(load().gbrpmd_server_tick(self.h, int(steps)))

    def counts(self):
        q, a, f, b = C.c_int(), C.c_int(), C.c_int(), C.c_size_t()
        _check(load().gbrpmd_server_counts(self.h, C.byref(q), C.byref(a), C.byref(f), C.byref(b)))
        return dict(queued=q.value, active=a.value, finished=f.value, bytes=b.value)

    def poll(self, max_n=1024):
        ids = (C.c_int64 * max_n)()
        st = (C.c_int * max_n)()
        ta, td, en = np.zeros(max_n), np.zeros(max_n), np.zeros(5 * max_n)
        n = C.c_int()
        _check(load().gbrpmd_server_poll(self.h, max_n, ids, st, _ptr(ta), _ptr(td), _ptr(en), C.byref(n)))
        out = []
        for i in range(n.value):
            arrs = self.keep.pop(ids[i])
            out.append(dict(id=ids[i], status=st[i], t_admit=ta[i], t_done=td[i], energies=en[5 * i:5 * i + 5].copy(),
                            r=arrs["r"], p=arrs["p"], dvdr=arrs["dvdr"], dvdr2=arrs["dvdr2"]))
        return out

    def close(self):
        if self.h:
            load().gbrpmd_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
