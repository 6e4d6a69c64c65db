"""Batched shots (ose_batch_*) against single-shot handles on the same
windows: with the default tuning both run the same device code per block, so
gathers and wavefields agree bit for bit; after autotuning (other tiles and
radix orders) they agree within FP32 round-off."""
import numpy as np
import pytest

import ose3d
from golden_util import rel_l2

pytestmark = pytest.mark.gpu

BASE = dict(bu=6, bd=6, bl=6, br=6, bf=6, bb=6, nt=40, fm=30.0, dt=0.0015, amp=50.0,
            dx=10.0, dy=10.0, dz=10.0, gzbeg=1)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


def model(seed=4, shape=(60, 52, 40)):
    rng = np.random.default_rng(seed)
    z = np.arange(shape[2])
    v = np.where(z < 14, 1800.0, np.where(z < 28, 2600.0, 3900.0))[None, None, :]
    v = v * (1 + 0.05 * rng.standard_normal(shape))
    return np.ascontiguousarray(v, dtype=np.float32)


WINDOWS = [dict(x0=0, y0=0, z0=0, nx=20, ny=18, nz=16, sx=10, sy=9, sz=2),
           dict(x0=30, y0=20, z0=0, nx=26, ny=22, nz=24, sx=5, sy=11, sz=3),
           dict(x0=50, y0=40, z0=10, nx=16, ny=20, nz=30, sx=8, sy=10, sz=1),   # leaves the model
           dict(x0=5, y0=10, z0=4, nx=34, ny=14, nz=20, sx=17, sy=7, sz=6)]


def single(m, w):
    """A single-shot handle on the same window (cut the same way)."""
    ix = np.clip(np.arange(w["x0"], w["x0"] + w["nx"]), 0, m.shape[0] - 1)
    iy = np.clip(np.arange(w["y0"], w["y0"] + w["ny"]), 0, m.shape[1] - 1)
    iz = np.clip(np.arange(w["z0"], w["z0"] + w["nz"]), 0, m.shape[2] - 1)
    sub = m[np.ix_(ix, iy, iz)]
    p = ose3d.default_params(nx=w["nx"], ny=w["ny"], nz=w["nz"], sxbeg=w["sx"], sybeg=w["sy"],
                             szbeg=w["sz"], **BASE)
    return ose3d.Modeler(p, sub)


def test_batch_equals_single_shot_handles():
    m = model()
    p = ose3d.default_params(**BASE)
    with ose3d.Batch(p, m, WINDOWS) as b:
        Ms = {b.info(s)[0].M for s in range(b.nshots)}
        b.run(30)
        got = [(b.gather(s), b.wavefield(s, ose3d.FIELD_Q), b.wavefield(s, ose3d.FIELD_P))
               for s in range(b.nshots)]
    assert len(Ms) >= 2, "the windows should need different series orders"
    for s, w in enumerate(WINDOWS):
        with single(m, w) as h:
            h.reset_shot(0)
            h.run(30)
            assert np.array_equal(got[s][0], h.gather()), s
            assert np.array_equal(got[s][1], h.wavefield(ose3d.FIELD_Q)), s
            assert np.array_equal(got[s][2], h.wavefield(ose3d.FIELD_P)), s


def test_autotune_keeps_results_and_caches(tmp_path):
    m = model()
    p = ose3d.default_params(**BASE)
    cache = str(tmp_path / "plans.txt")
    with ose3d.Batch(p, m, WINDOWS) as b:
        b.run(20)
        ref = [b.gather(s) for s in range(b.nshots)]
        b.autotune(steps=2, cache_path=cache)
        t1 = b.tuning()
        b.run(20)
        for s in range(b.nshots):
            assert rel_l2(b.gather(s)[:, :20], ref[s][:, :20]) < 1e-5
    with ose3d.Batch(p, m, WINDOWS) as b2:
        assert b2.autotune(steps=2, cache_path=cache) < 0    # served from the cache
        assert b2.tuning() == t1


REG_WINDOWS = [dict(x0=0, y0=0, z0=0, nx=52, ny=52, nz=52, sx=20, sy=26, sz=3),     # padded 64^3 (register)
               dict(x0=8, y0=4, z0=0, nx=84, ny=52, nz=36, sx=40, sy=20, sz=2),     # 96 x 64 x 48
               dict(x0=20, y0=10, z0=2, nx=52, ny=84, nz=52, sx=30, sy=40, sz=5)]   # 64 x 96 x 64


@pytest.mark.parametrize("lanes", [0, 3])
def test_register_classes_and_lanes_match_single_shots(lanes):
    """Windows whose padded axes have register kernels (64 = 16*4, 96 = 16*6),
    batched launches (lanes 0) or per-shot launches on 3 concurrent streams:
    bit for bit the single-shot handles."""
    m = model(seed=9, shape=(100, 100, 60))
    p = ose3d.default_params(**BASE)
    with ose3d.Batch(p, m, REG_WINDOWS) as b:
        b.set_tuning(lanes=lanes)
        assert b.tuning()["lanes"] == lanes
        b.run(BASE["nt"])
        for s, w in enumerate(REG_WINDOWS):
            with single(m, w) as h:
                h.reset_shot(0)
                g = h.run(BASE["nt"], want_gather=True)
                assert np.array_equal(b.gather(s), g)
                assert np.array_equal(b.wavefield(s, ose3d.FIELD_Q), h.wavefield(ose3d.FIELD_Q))


# padded 64^3, 96 x 64 x 112 and 64 x 96 x 64: every axis 16 C with C <= 16
PERSIST_WINDOWS = [dict(x0=0, y0=0, z0=0, nx=52, ny=52, nz=52, sx=20, sy=26, sz=3),
                   dict(x0=8, y0=4, z0=0, nx=84, ny=52, nz=100, sx=40, sy=20, sz=2),
                   dict(x0=20, y0=10, z0=2, nx=52, ny=84, nz=52, sx=30, sy=40, sz=5)]


@pytest.mark.parametrize("group_mb", [0, 1])
def test_persistent_step_matches_single_shots(group_mb):
    """The whole batched step as one persistent cooperative launch (grid
    barriers between the passes), all shots in one group or one shot per
    group: bit for bit the single-shot handles."""
    m = model(seed=11, shape=(100, 100, 110))
    p = ose3d.default_params(**BASE)
    with ose3d.Batch(p, m, PERSIST_WINDOWS) as b:
        b.set_tuning(lanes=-1, group_mb=group_mb)
        assert b.tuning()["lanes"] == -1
        b.run(BASE["nt"])
        for s, w in enumerate(PERSIST_WINDOWS):
            with single(m, w) as h:
                h.reset_shot(0)
                g = h.run(BASE["nt"], want_gather=True)
                assert np.array_equal(b.gather(s), g)
                assert np.array_equal(b.wavefield(s, ose3d.FIELD_Q), h.wavefield(ose3d.FIELD_Q))
                assert np.array_equal(b.wavefield(s, ose3d.FIELD_P), h.wavefield(ose3d.FIELD_P))


def test_persistent_step_refused_where_a_length_has_no_kernel():
    m = model(seed=9, shape=(100, 100, 60))
    with ose3d.Batch(ose3d.default_params(**BASE), m, REG_WINDOWS) as b:   # a 48-long axis
        with pytest.raises(ose3d.OseError):
            b.set_tuning(lanes=-1)
        assert b.tuning()["lanes"] == 0
