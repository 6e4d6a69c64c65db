"""The bounded waits inside the kernels, made to run out on purpose without
faulting or hanging the GPU: ose_self_test_waits launches one single-CTA
kernel per kind whose wait nothing ever completes (the plane kernels' DSMEM
exchange mbarrier, the persistent batch's grid barrier, the MMA completion
barrier), each with a limit of a few milliseconds instead of the production
1-2 s.  Every wait must give up, record it in its error word and return, and
the context must stay usable afterwards (a time step runs and matches a run
in a fresh process bit for bit)."""
import time

import numpy as np
import pytest

import ose3d

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


KW = dict(nx=20, ny=20, nz=20, bu=6, bd=6, bl=6, br=6, bf=6, bb=6, nt=20, fm=25.0, dt=0.002, amp=100.0,
          dx=10.0, dy=10.0, dz=10.0, sxbeg=10, sybeg=10, szbeg=3, gzbeg=0)


def _steps():
    vel = np.full((KW["nx"], KW["ny"], KW["nz"]), 2500.0, np.float32)
    with ose3d.Modeler(ose3d.default_params(**KW), vel) as m:
        m.reset_shot(0)
        g = m.run(10, want_gather=True)
        return g, m.wavefield(ose3d.FIELD_Q)


def test_every_bounded_wait_runs_out_and_reports():
    g0, q0 = _steps()
    t = time.perf_counter()
    mask = ose3d.self_test_waits(5.0)
    dt = time.perf_counter() - t
    assert mask == 7, f"waits that ran out: {mask:03b}"
    assert dt < 30.0
    # the device context is intact: the same steps give the same results
    g1, q1 = _steps()
    assert np.array_equal(g0, g1) and np.array_equal(q0, q1)
