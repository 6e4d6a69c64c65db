"""The C ABI library without a GPU: it loads, exports every entry point that
include/ose3d.h declares, and its host-only calls agree with the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O
import ose3d

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "ose3d.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ose_[a-z_0-9]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as ge
    ge.build_library()
    return ose3d.load_library()


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    assert sorted(ose3d.EXPORTS) == syms
    for s in syms:
        assert hasattr(lib, s), s


def test_default_params_are_the_reference_main(lib):
    p = ose3d.default_params()
    assert (p.nx, p.ny, p.nz, p.bu, p.nt) == (101, 101, 101, 25, 300)
    assert abs(p.fm - 40.0) < 1e-6 and abs(p.dt - 0.001) < 1e-9 and abs(p.amp - 100.0) < 1e-6
    assert (p.sxbeg, p.sybeg, p.szbeg) == (50, 50, 0)


@pytest.mark.parametrize("dims", [(101, 101, 101, 25, 25), (20, 18, 16, 6, 5), (100, 101, 102, 25, 26),
                                  (196, 196, 196, 30, 30), (7, 1, 3, 0, 0)])
def test_padded_dims_match_oracle(lib, dims):
    nx, ny, nz, b0, b1 = dims
    p = ose3d.default_params(nx=nx, ny=ny, nz=nz, bl=b0, br=b1, bf=b0, bb=b1, bu=b0, bd=b1)
    out = [ctypes.c_int() for _ in range(3)]
    assert lib.ose_padded_dims(ctypes.byref(p), *[ctypes.byref(o) for o in out]) == 0
    d = O.derive(O.make_params(nx=nx, ny=ny, nz=nz, bl=b0, br=b1, bf=b0, bb=b1, bu=b0, bd=b1))
    assert [o.value for o in out] == [d.nxb, d.nyb, d.nzb]
    assert all(o.value % 2 == 0 for o in out)


def test_invalid_params_rejected(lib):
    p = ose3d.default_params(nx=0)
    out = [ctypes.c_int() for _ in range(3)]
    assert lib.ose_padded_dims(ctypes.byref(p), *[ctypes.byref(o) for o in out]) == 1
    assert b"nx" in lib.ose_last_error(None)


def test_null_handle_calls_are_errors(lib):
    assert lib.ose_step(None) == 1
    assert lib.ose_reset_shot(None, 0) == 1
    assert lib.ose_destroy(None) == 0
    assert lib.ose_version().startswith(b"ose3d")


def test_status_codes_mirror_the_header():
    import re
    src = open(os.path.join(ROOT, "include", "ose3d.h")).read()
    codes = {int(v): k for k, v in re.findall(r"\b(OSE_(?:OK|ERR_[A-Z]+))\s*=\s*(\d+)", src)}
    assert codes == ose3d.STATUS


def test_wait_self_test_rejects_bad_limits_before_the_device(lib):
    out = ctypes.c_int(-1)
    for bad in (0.0, -1.0, 1000.0, float("nan")):
        assert lib.ose_self_test_waits(bad, ctypes.byref(out)) == 1
    assert lib.ose_self_test_waits(5.0, None) == 1
    assert b"limit_ms" in lib.ose_last_error(None)


def test_python_class_mirrors_header_structs():
    assert ctypes.sizeof(ose3d.Params) == ctypes.sizeof(O.OseParams)
    assert [f[0] for f in ose3d.Params._fields_] == [f[0] for f in O.OseParams._fields_]
    assert [f[0] for f in ose3d.Derived._fields_] == [f[0] for f in O.OseDerived._fields_]


def test_corrector_param_count_matches_the_restatement(lib):
    import corrector_torch as CT
    assert ose3d.corrector_param_count() == CT.param_count() == 64034


def _create(lib, p, vel):
    h = ctypes.c_void_p()
    st = lib.ose_create(ctypes.byref(p), vel.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(h))
    return st, h


@pytest.mark.parametrize("case", ["axis_too_long", "receivers_below_model", "zero_velocity", "nan_velocity"])
def test_create_rejects_before_touching_the_device(lib, case):
    """ose_create validates sizes, geometry and the model on the host first,
    so these refusals need no GPU (and allocate nothing)."""
    kw = dict(nx=12, ny=10, nz=8, bu=4, bd=4, bl=4, br=4, bf=4, bb=4, nt=10, sxbeg=5, sybeg=5, szbeg=2)
    if case == "axis_too_long":
        kw.update(nx=1030 - 8)                      # padded 1030 > 1024
    if case == "receivers_below_model":
        kw.update(gzbeg=8)                          # depth index past the interior
    p = ose3d.default_params(**kw)
    vel = np.full((kw["nx"], kw["ny"], kw["nz"]), 2000.0, np.float32)
    if case == "zero_velocity":
        vel[3, 4, 5] = 0.0
    if case == "nan_velocity":
        vel[0, 0, 0] = np.nan
    st, h = _create(lib, p, vel)
    assert not h.value
    expect = {"axis_too_long": (5, b"1024"), "receivers_below_model": (1, b"gzbeg"),
              "zero_velocity": (1, b"positive"), "nan_velocity": (1, b"finite")}[case]
    assert st == expect[0]
    assert expect[1] in lib.ose_last_error(None)


def test_model_file_errors_before_the_device(lib, tmp_path):
    p = ose3d.default_params(nx=8, ny=8, nz=8, bu=4, bd=4, bl=4, br=4, bf=4, bb=4, nt=4, sxbeg=4, sybeg=4,
                             szbeg=2, gzbeg=0)
    h = ctypes.c_void_p()
    missing = str(tmp_path / "nothing.bin").encode()
    assert lib.ose_create_from_file(ctypes.byref(p), missing, ctypes.byref(h)) == 4
    assert b"cannot open" in lib.ose_last_error(None)
    short = tmp_path / "short.bin"
    np.full(8 * 8 * 8 - 1, 2000.0, np.float32).tofile(short)
    assert lib.ose_create_from_file(ctypes.byref(p), str(short).encode(), ctypes.byref(h)) == 4
    assert b"short model file" in lib.ose_last_error(None)
    assert not h.value
