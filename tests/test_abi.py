"""The C ABI library loads without a GPU, exports every function that
include/gbrpmd.h declares, and its host-side pieces (parameter store, the
serial ran2/gaussian stream) behave like the reference.  No device work."""
import ctypes as C
import subprocess

import pytest

from rpmd_mainz_gb300 import lib
from rpmd_mainz_gb300.abi import GbParams

from . import oracle_lib as orc


@pytest.fixture(scope="module")
def gb():
    import __graft_entry__ as g

    from rpmd_mainz_gb300 import build

    build.build()
    return lib.load()


def test_exports_every_declared_symbol(gb):
    names = lib.header_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_params_round_trip(gb):
    p = GbParams()
    p.mts = 3
    p.walpha = 7.5
    p.nbdf1 = 1
    lib.init(p)
    q = lib.get_params()
    assert q.mts == 3 and q.walpha == 7.5 and q.nbdf1 == 1
    bad = GbParams()
    bad.mts = 0
    with pytest.raises(lib.GbError):
        lib.init(bad)


def test_ran2_gaussian_match_reference_stream(gb):
    # random.f90 ran2/gaussian, seeded as main.f90:298-299
    idum = C.c_int(-4711)
    ref = orc.Rng(4711)
    a = [lib.ran2(idum) for _ in range(200)] + [lib.gaussian(idum, 1.5) for _ in range(201)]
    b = [ref.ran2() for _ in range(200)] + [ref.gaussian(1.5) for _ in range(201)]
    assert a == b
