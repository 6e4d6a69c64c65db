"""Time-loop parity at the benchmark configurations' own sizes against the FP64
restatement of the same loop (oracle/oracle_torch.py: torch complex128 on the
same GPU), over a bounded prefix of each configuration's steps:

  ose142        interior 101^3 + 20-cell sponge (padded 142^3 = 2 x 71 per axis),
                layered model, 20 Hz Ricker at (50, 50, 10), receivers at z = 5,
                the reference's sponge profile;
  ose142cerjan  the same with the Cerjan sponge (factor 0.015);
  ose320x288x256  the non-power-of-two variant of the 256^3 workload.

Tolerance 1e-4 relative L2 (FP32 path vs FP64) on the receiver gather [it][ig]
and on the final P and Q; every sizeable trace also within 10x that of its
own FP64 trace, which pins the receiver order."""
import numpy as np
import pytest

import ose3d
from golden_util import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


@pytest.mark.parametrize("wl,steps", [("ose142", 300), ("ose142cerjan", 300), ("ose320x288x256", 200)])
def test_time_loop_matches_fp64_restatement(wl, steps):
    import workloads
    from oracle_torch import TorchOracle
    build, kw = workloads.CONFIGS[wl]
    vel = build()
    with ose3d.Modeler(ose3d.default_params(**kw), vel) as m:
        d = m.derived
        m.reset_shot(0)
        g = m.run_record(steps)                      # [it][ig]
        P = m.wavefield(ose3d.FIELD_P)
        Q = m.wavefield(ose3d.FIELD_Q)
    o = TorchOracle(kw, vel, "cuda")
    assert o.M == d.M
    g64 = o.run(steps)
    P64, Q64 = o.P(), o.Q()
    del o
    assert g.shape == g64.shape == (steps, kw["nx"] * kw["ny"])
    assert rel_l2(g, g64) < TOL
    assert rel_l2(P, P64) < TOL
    assert rel_l2(Q, Q64) < TOL
    tn = np.linalg.norm(g64, axis=0)
    big = tn > 1e-3 * tn.max()
    tr = np.linalg.norm(g - g64, axis=0)[big] / tn[big]
    assert np.all(tr < 10 * TOL)
