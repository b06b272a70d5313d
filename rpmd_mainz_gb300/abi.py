"""ctypes mirror of the C ABI declared in include/gbrpmd.h.

`GbParams` has the field order and types of `struct gb_params`; ctypes lays
it out with the same natural alignment as the C compiler does.
"""
import ctypes as C

GB_OK = 0
GB_E_ARG = 1
GB_E_NOINIT = 2
GB_E_CUDA = 3
GB_E_LIST = 4
GB_E_RATTLE1 = 5
GB_E_RATTLE2 = 6
GB_E_CONTRACT = 7
GB_E_NONFINITE = 8
GB_E_CUTOFF = 9
GB_E_NOMEM = 10
GB_E_UNSUPPORTED = 11

GB_THERM_NONE = 0
GB_THERM_AND = 1
GB_THERM_PRG = 2
GB_THERM_PRL = 3

GB_BARO_NONE = 0
GB_BARO_BER = 1
GB_BARO_MCI = 2

GB_INTRA_REFERENCE = 0
GB_INTRA_SPCFW = 1

GB_PREC_FP64 = 0
GB_PREC_MIXED = 1

STATUS_NAMES = {
    GB_OK: "ok", GB_E_ARG: "invalid argument", GB_E_NOINIT: "not initialised",
    GB_E_CUDA: "CUDA error", GB_E_LIST: "neighbour list too small",
    GB_E_RATTLE1: "max iterations exceeded in rattle stage 1",
    GB_E_RATTLE2: "max iterations exceeded in rattle stage 2",
    GB_E_CONTRACT: "beadiabatic factor must be odd", GB_E_NONFINITE: "non-finite force",
    GB_E_CUTOFF: "ewc cut-off too large for box", GB_E_NOMEM: "out of device memory",
    GB_E_UNSUPPORTED: "option not supported",
}


class GbParams(C.Structure):
    _fields_ = [
        ("oo_eps", C.c_double), ("oo_sig", C.c_double), ("oo_gam", C.c_double), ("rcut", C.c_double),
        ("alpha", C.c_double), ("ecut", C.c_double), ("wm", C.c_double), ("wh", C.c_double),
        ("wrcut", C.c_double), ("walpha", C.c_double), ("rkmax", C.c_double),
        ("kmax", C.c_int32),
        ("nbdf1", C.c_int32), ("nbdf2", C.c_int32),
        ("apot", C.c_double), ("bpot", C.c_double), ("alp", C.c_double), ("alpb", C.c_double),
        ("theta", C.c_double), ("reoh", C.c_double),
        ("sig", C.c_double),
        ("mts", C.c_int32),
        ("iamcub", C.c_int32),
        ("nctot", C.c_int32), ("nbond", C.c_int32),
        ("therm", C.c_int32),
        ("ttau", C.c_double),
        ("taub", C.c_double), ("patm", C.c_double),
        ("intra_model", C.c_int32),
        ("precision", C.c_int32),
        ("baro", C.c_int32),
    ]

    def copy(self):
        out = GbParams()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(GbParams))
        return out

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}
