"""ose_run_record (the reference's per-step receiver read, rec_slice_to_data,
ose_3d_lib.cu:876-884) enqueues steps in chunks and moves their rows through
pinned buffers while later steps run: the rows it returns, for any split of
the run into calls and across chunk boundaries, are bit for bit the gather
that ose_run leaves on the device ([ig][it] there, [it][ig] here)."""
import numpy as np
import pytest

import ose3d

pytestmark = pytest.mark.gpu

KW = dict(nx=24, ny=20, nz=18, bu=6, bd=6, bl=6, br=6, bf=6, bb=6, nt=140, fm=30.0, dt=0.0015, amp=50.0,
          sxbeg=12, sybeg=10, szbeg=4, gzbeg=2)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


@pytest.fixture(scope="module")
def vel():
    rng = np.random.default_rng(5)
    return (1800 + 1500 * rng.random((KW["nx"], KW["ny"], KW["nz"]))).astype(np.float32)


@pytest.mark.parametrize("split", [(140,), (1, 31, 32, 33, 43), (64, 65, 11)], ids=str)
def test_recorded_rows_equal_the_device_gather(vel, split):
    assert sum(split) == KW["nt"]
    with ose3d.Modeler(ose3d.default_params(**KW), vel) as m:
        m.reset_shot(0)
        ref = m.run(KW["nt"], want_gather=True)            # [ig][it]
        m.reset_shot(0)
        rows = np.concatenate([m.run_record(n) for n in split])
        assert rows.shape == (KW["nt"], KW["nx"] * KW["ny"])
        assert np.array_equal(rows, ref.T)
        with pytest.raises(ose3d.OseError):
            m.run_record(1)                                  # past nt
