"""ose_apply_operator_noalloc: the operator entry point for callers that
cannot allocate device memory (it keeps its scratch in a fixed file-scope
device array), checked against ose_apply_operator on two calls in a row and
against the FP64 oracle on grids up to its maximum size.

This file is collected last on purpose (tests/test_zz_*), so a run that
stops at the first failure has run every other test before it."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
import ose3d
from golden_util import rel_l2

KW = dict(nx=20, ny=18, nz=16, bu=6, bd=6, bl=6, br=5, bf=6, bb=6, nt=8)
ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as ge
    ge.build_library()
    return ose3d.load_library()


def test_rejects_sizes_beyond_the_maximum(lib):
    """Checked before any device work: no GPU needed."""
    dummy = (ctypes.c_float * 4)()
    p = ctypes.cast(dummy, ctypes.POINTER(ctypes.c_float))
    too_big = 2 * ose3d.NOALLOC_MAX_CELLS
    st = lib.ose_apply_operator_noalloc(128, 128, too_big // (128 * 128), 10.0, 10.0, 10.0, 1000.0,
                                        p, p, p, None)
    assert st == 5   # OSE_ERR_UNSUPPORTED
    st = lib.ose_apply_operator_noalloc(2048, 2, 2, 10.0, 10.0, 10.0, 1000.0, p, p, p, None)
    assert st == 5
    st = lib.ose_apply_operator_noalloc(33, 32, 32, 10.0, 10.0, 10.0, 1000.0, p, p, p, None)
    assert st == 1   # odd axis: OSE_ERR_INVALID


def _noalloc(torch, shape, vb, R, x, dx=10.0):
    """One call through the C ABI on torch-owned device buffers."""
    dev = torch.device("cuda", 0)
    nzb, nyb, nxb = shape
    vel_d = torch.from_numpy(np.ascontiguousarray(vb, np.float32)).to(dev)
    x_d = torch.from_numpy(np.ascontiguousarray(x, np.complex64).view(np.float32)).to(dev)
    out_d = torch.empty_like(x_d)
    torch.cuda.synchronize()
    st = ose3d.apply_operator_noalloc(nxb, nyb, nzb, dx, dx, dx, R, vel_d.data_ptr(), x_d.data_ptr(),
                                      out_d.data_ptr(), 0)
    torch.cuda.synchronize()
    assert st == 0
    return out_d.cpu().numpy().view(np.complex64).reshape(shape)


@pytest.mark.gpu
def test_noalloc_matches_apply_operator_twice(lib):
    torch = pytest.importorskip("torch")
    vel_xyz = np.random.default_rng(8).uniform(1800, 4200, (KW["nx"], KW["ny"], KW["nz"])).astype(np.float32)
    rng = np.random.default_rng(9)
    with ose3d.Modeler(ose3d.default_params(**KW), vel_xyz) as m:
        d = m.derived
        vb = m.wavefield(ose3d.FIELD_V)
        for _ in range(2):
            x = (rng.standard_normal(m.shape) + 1j * rng.standard_normal(m.shape)).astype(np.complex64)
            ref = m.apply_operator(x)
            got = _noalloc(torch, m.shape, vb, d.R, x)
            assert rel_l2(got, ref) < 1e-5


# Padded grids at the size limit: 64^3 takes the register row and column
# kernels, 32 x 32 x 256 the 256-point z-pass kernel of the plane path.
GRIDS = {"64x64x64": dict(nx=44, ny=44, nz=44, bu=10, bd=10, bl=10, br=10, bf=10, bb=10),
         "32x32x256": dict(nx=12, ny=12, nz=236, bu=10, bd=10, bl=10, br=10, bf=10, bb=10)}


def _case(name, seed):
    kw = dict(GRIDS[name], nt=8)
    p = O.make_params(**kw)
    d = O.derive(p)
    rng = np.random.default_rng(seed)
    vel = rng.uniform(1800, 4200, (kw["nx"], kw["ny"], kw["nz"])).astype(np.float32)
    vb = O.pad_model(p, vel)
    R = O.series(p, float(vb.max()))[0]
    shape = (d.nzb, d.nyb, d.nxb)
    assert d.nxb * d.nyb * d.nzb == ose3d.NOALLOC_MAX_CELLS
    return p, vb, R, shape, rng


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GRIDS))
def test_noalloc_matches_fp64_oracle_at_the_limit(lib, name):
    """Two calls in a row at OSE_NOALLOC_MAX_CELLS against the FP64 oracle;
    FP32 tolerance 2e-6 relative L2 (one application)."""
    torch = pytest.importorskip("torch")
    p, vb, R, shape, rng = _case(name, 31)
    for _ in range(2):
        x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        got = _noalloc(torch, shape, vb, R, x.astype(np.complex64))
        ref = O.apply_operator(p, vb, R, x.astype(np.complex64).astype(np.complex128))
        assert rel_l2(got, ref) < 2e-6


_FRESH = r"""
import sys
sys.path[:0] = {paths!r}
import numpy as np, torch
import ose3d
sys.path.insert(0, {tests!r})
from test_zz_no_alloc import _case, _noalloc
import oracle as O
from golden_util import rel_l2
ose3d.load_library()
p, vb, R, shape, rng = _case("64x64x64", 5)
x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
got = _noalloc(torch, shape, vb, R, x.astype(np.complex64))
ref = O.apply_operator(p, vb, R, x.astype(np.complex64).astype(np.complex128))
print("REL", rel_l2(got, ref))
"""


@pytest.mark.gpu
def test_noalloc_first_call_in_a_fresh_process(lib):
    """The entry point's own first-call set-up (symbol address, kernel
    attributes) in a process that never created a modeler handle."""
    paths = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "3d-ose_gb300"),
             os.path.join(ROOT, "tests", "golden")]
    code = _FRESH.format(paths=paths, tests=os.path.join(ROOT, "tests"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rel = float([ln for ln in r.stdout.splitlines() if ln.startswith("REL")][-1].split()[1])
    assert rel < 2e-6
