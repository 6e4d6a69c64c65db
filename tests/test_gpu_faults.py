"""Device out-of-memory during ose_create, simulated on the host: with
OSE3D_FAIL_DEVICE_ALLOC=N in the environment the N-th device allocation of a
handle fails as cudaMalloc would when the device is full.  ose_create must
return OSE_ERR_NOMEM, name the allocation, free what it had allocated (the
device's free memory is unchanged) and leave the library usable: the next
create without the hook runs a step."""
import ctypes
import os

import numpy as np
import pytest

import ose3d

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as ge
    ge.build_library()
    return ose3d.load_library()


KW = dict(nx=40, ny=40, nz=40, bu=12, bd=12, bl=12, br=12, bf=12, bb=12, nt=10, fm=25.0, dt=0.002, amp=100.0,
          dx=10.0, dy=10.0, dz=10.0, sxbeg=20, sybeg=20, szbeg=3, gzbeg=0)


def _create(lib, p, vel):
    h = ctypes.c_void_p()
    st = lib.ose_create(ctypes.byref(p), vel.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(h))
    return st, h


def test_simulated_device_oom_in_create(lib):
    torch = pytest.importorskip("torch")
    p = ose3d.default_params(**KW)
    vel = np.full((KW["nx"], KW["ny"], KW["nz"]), 2500.0, np.float32)
    st, h = _create(lib, p, vel)          # warm: the context and the kernels' attributes
    assert st == 0
    lib.ose_destroy(h)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    try:
        for n in (1, 2, 5, 12):
            os.environ["OSE3D_FAIL_DEVICE_ALLOC"] = str(n)
            st, h = _create(lib, p, vel)
            assert st == 3, (n, st)
            assert not h.value
            assert b"dalloc" in lib.ose_last_error(None)
    finally:
        del os.environ["OSE3D_FAIL_DEVICE_ALLOC"]
    free1 = torch.cuda.mem_get_info()[0]
    assert abs(free1 - free0) < (4 << 20), (free0, free1)
    with ose3d.Modeler(p, vel) as m:
        m.reset_shot(0)
        m.step()
        assert np.all(np.isfinite(m.wavefield(ose3d.FIELD_Q)))
