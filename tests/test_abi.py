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


def test_params_layout_matches_ctypes_mirror(gb):
    # sizeof(gb_params) and every field offset as the C compiler laid them out
    n = len(GbParams._fields_)
    offs = (C.c_int64 * n)()
    gb.gbrpmd_params_layout.argtypes = [C.POINTER(C.c_int64), C.c_int]
    size = gb.gbrpmd_params_layout(offs, n)
    assert size == C.sizeof(GbParams)
    for i, (name, _) in enumerate(GbParams._fields_):
        assert offs[i] == getattr(GbParams, name).offset, name


def test_fortran_binding_lists_every_field():
    # the bind(c) type of the Fortran shim in INTEGRATION.md declares the same
    # fields in the same order (and so the same layout) as struct gb_params
    import os
    import re

    text = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "INTEGRATION.md")).read()
    block = re.search(r"type, bind\(c\) :: gb_params\n(.*?)\n\s*end type", text, re.S).group(1)
    fields = []
    for line in block.splitlines():
        decl = line.split("::", 1)[1]
        fields += [f.strip() for f in decl.split(",")]
    assert fields == [name for name, _ in GbParams._fields_]
