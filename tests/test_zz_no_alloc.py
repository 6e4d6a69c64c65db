"""ose_apply_operator_noalloc: the operator entry point for callers that
cannot allocate device memory (it keeps its scratch in a fixed file-scope
device array), checked against ose_apply_operator on two calls in a row.

This file is collected last on purpose (tests/test_zz_*), so a run that
stops at the first failure has run every other test before it."""
import ctypes

import numpy as np
import pytest

import ose3d
from golden_util import rel_l2

KW = dict(nx=20, ny=18, nz=16, bu=6, bd=6, bl=6, br=5, bf=6, bb=6, nt=8)


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


@pytest.mark.gpu
def test_noalloc_matches_apply_operator_twice(lib):
    torch = pytest.importorskip("torch")
    vel_xyz = np.random.default_rng(8).uniform(1800, 4200, (KW["nx"], KW["ny"], KW["nz"])).astype(np.float32)
    rng = np.random.default_rng(9)
    with ose3d.Modeler(ose3d.default_params(**KW), vel_xyz) as m:
        d = m.derived
        vb = m.wavefield(ose3d.FIELD_V)
        dev = torch.device("cuda", 0)
        vel_d = torch.from_numpy(vb.copy()).to(dev)
        for _ in range(2):
            x = (rng.standard_normal(m.shape) + 1j * rng.standard_normal(m.shape)).astype(np.complex64)
            ref = m.apply_operator(x)
            x_d = torch.from_numpy(x.view(np.float32).copy()).to(dev)
            out_d = torch.empty_like(x_d)
            torch.cuda.synchronize()
            st = ose3d.apply_operator_noalloc(d.nxb, d.nyb, d.nzb, 10.0, 10.0, 10.0, d.R,
                                              vel_d.data_ptr(), x_d.data_ptr(), out_d.data_ptr(), 0)
            torch.cuda.synchronize()
            assert st == 0
            got = out_d.cpu().numpy().view(np.complex64).reshape(m.shape)
            assert rel_l2(got, ref) < 1e-5
