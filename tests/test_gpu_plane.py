"""The 256^3 cluster path (ose_plane.cu) against the FP64 oracle and against the
generic path.  Tolerance: 1e-4 relative L2 (FP32 vs FP64), tighter where two
FP32 implementations of the same step are compared."""
import numpy as np
import pytest

import oracle as O
import ose3d
from golden_util import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


def small_salt(seed=3):
    import workloads
    return workloads.smooth_random_salt(196, 196, 196, seed=seed)


KW = dict(nx=196, ny=196, nz=196, bu=30, bd=30, bl=30, br=30, bf=30, bb=30, nt=400, fm=25.0,
          dt=0.002, amp=100.0, dx=10.0, dy=10.0, dz=10.0, sxbeg=98, sybeg=98, szbeg=5, gzbeg=0)


@pytest.fixture(scope="module")
def model():
    return small_salt()


def test_plane_path_selected_for_256(model):
    with ose3d.Modeler(ose3d.default_params(**KW), model) as m:
        assert (m.derived.nxb, m.derived.nyb, m.derived.nzb) == (256, 256, 256)
        assert m.derived.path == ose3d.PATH_PLANE
        assert m.derived.M == 10


def test_plane_operator_matches_oracle(model):
    rng = np.random.default_rng(21)
    with ose3d.Modeler(ose3d.default_params(**KW), model) as m:
        x = (rng.standard_normal(m.shape) + 1j * rng.standard_normal(m.shape)).astype(np.complex64)
        y = m.apply_operator(x)
        vb = m.wavefield(ose3d.FIELD_V)
        R = m.derived.R
        m.select_path(ose3d.PATH_GENERIC)
        yg = m.apply_operator(x)
    ref = O.apply_operator(O.make_params(**KW), vb, R, x.astype(np.complex128))
    assert rel_l2(y, ref) < 2e-6
    assert rel_l2(yg, ref) < 2e-6


def test_plane_steps_match_oracle(model):
    with ose3d.Modeler(ose3d.default_params(**KW), model) as m:
        m.reset_shot(0)
        g = m.run(2, want_gather=True)
        Q = m.wavefield(ose3d.FIELD_Q)
        P = m.wavefield(ose3d.FIELD_P)
    og, oP, oQ = O.run(O.make_params(**KW), model, 2)
    assert rel_l2(g[:, :2], og.T) < 1e-4
    assert rel_l2(Q, oQ) < 1e-4
    assert rel_l2(P, oP) < 1e-4


def test_plane_and_generic_agree_over_300_steps(model):
    """Two different FP32 FFT factorisations of the same step stay within
    1e-4 after 300 steps (gather and final wavefield)."""
    out = {}
    for path in (ose3d.PATH_PLANE, ose3d.PATH_GENERIC):
        with ose3d.Modeler(ose3d.default_params(**KW), model) as m:
            m.select_path(path)
            m.reset_shot(0)
            g = m.run(300, want_gather=True)
            out[path] = (g, m.wavefield(ose3d.FIELD_Q), m.wavefield(ose3d.FIELD_P))
    a, b = out[ose3d.PATH_PLANE], out[ose3d.PATH_GENERIC]
    assert np.all(np.isfinite(a[1]))
    assert rel_l2(a[0], b[0]) < 1e-4
    assert rel_l2(a[1], b[1]) < 1e-4
    assert rel_l2(a[2], b[2]) < 1e-4


def test_plane_graph_replay_matches_steps(model):
    with ose3d.Modeler(ose3d.default_params(**KW), model) as m:
        m.reset_shot(0)
        for _ in range(3):
            m.step()
        q_steps = m.wavefield(ose3d.FIELD_Q)
        m.reset_shot(0)
        m.run(3)
        assert np.array_equal(q_steps, m.wavefield(ose3d.FIELD_Q))


def test_plane_path_matches_fp64_over_200_steps(model):
    """FP32 plane path vs the FP64 restatement (torch, same GPU) after 200
    steps of the 256^3 workload: gather and final wavefield within 1e-4."""
    torch = pytest.importorskip("torch")
    from oracle_torch import TorchOracle
    with ose3d.Modeler(ose3d.default_params(**KW), model) as m:
        m.reset_shot(0)
        g32 = m.run_record(200)
        P, Q = m.wavefield(ose3d.FIELD_P), m.wavefield(ose3d.FIELD_Q)
    t = TorchOracle(KW, model, "cuda")
    g64 = t.run(200)
    assert rel_l2(g32, g64) < 1e-4
    assert rel_l2(Q, t.Q()) < 1e-4
    assert rel_l2(P, t.P()) < 1e-4
    del t
    torch.cuda.empty_cache()
