import os

from rpmd_mainz_gb300 import namelist

from . import systems


def test_param_files():
    p = namelist.read(os.path.join(systems.PARAMS, "param_qspcfw"), "param")
    assert p["qo"] == -0.84 and p["alpha"] == 1.0 and p["thetad"] == 112.0
    assert p["oo_sig"] == 5.981913 and p["oo_eps"] == 2.47686e-4


def test_input_file():
    i = namelist.read(os.path.join(systems.PARAMS, "gentest_input"), "input")
    assert i["ncellxyz"] == [5, 5, 5] and i["nb"] == 2 and i["type"] == "RPMD"
    assert i["iamcub"] is True and i["sig"] == 4.5 and i["print"] == [1, 1, 1]


def test_comments_and_commas():
    t = "&input\n a = 1, b = 2.5d0 ! comment\n c = 'x y'\n d = .false. /\n"
    r = namelist.parse(t)
    assert r == {"a": 1, "b": 2.5, "c": "x y", "d": False}
