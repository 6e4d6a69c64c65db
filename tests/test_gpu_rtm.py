"""Reverse-time migration (ose_rtm).

1. Time reversal: the recorded surface data of a point source at depth 30,
   propagated backwards to time 0, refocus at the source cell.
2. Imaging: a flat reflector at depth 40 cells under a 2000 m/s layer;
   reflected data (true model minus the 2000 m/s background) migrated with the
   background velocity and normalised by the source illumination image at
   depth 40 +- 3 cells below the near-surface zone (depths < 25 carry the
   usual source/receiver-side correlation artifacts)."""
import numpy as np
import pytest

import ose3d

pytestmark = pytest.mark.gpu

N = 64
KW = dict(nx=N, ny=N, nz=N, bu=20, bd=20, bl=20, br=20, bf=20, bb=20, nt=400, fm=20.0, dt=0.002,
          amp=100.0, dx=10.0, dy=10.0, dz=10.0, sxbeg=N // 2, sybeg=N // 2, szbeg=2, gzbeg=0,
          hilbert_div_nt=1)
DEPTH = 40
B = 20


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


def record(vel, kw=KW):
    with ose3d.Modeler(ose3d.default_params(**kw), vel) as m:
        m.reset_shot(0)
        return m.run_record(kw["nt"])


BACK = np.full((N, N, N), 2000.0, np.float32)


def test_backpropagated_data_refocus_at_the_source():
    kw = dict(KW, szbeg=30)
    d = record(BACK, kw)
    with ose3d.Modeler(ose3d.default_params(**kw), BACK) as m:
        m.reset_shot(0)
        m.rtm(d, every=50)
        with pytest.raises(ose3d.OseError):
            m.step()   # the state now holds the receiver wavefield
        P, Q = m.wavefield(ose3d.FIELD_P), m.wavefield(ose3d.FIELD_Q)
    E = (P.astype(np.float64) ** 2 + Q.astype(np.float64) ** 2)[B:B + N, B:B + N, B:B + N]
    z, y, x = np.unravel_index(np.argmax(E), E.shape)
    print(f"refocus at {(x, y, z)}, source at (32, 32, 30)")
    assert (x, y, z) == (32, 32, 30)
    assert E[30, 32, 32] > 100 * E[0, 32, 32]


def test_rtm_images_a_flat_reflector_at_its_depth():
    true = BACK.copy()
    true[:, :, DEPTH:] = 3000.0
    obs = record(true) - record(BACK)
    assert np.abs(obs).max() > 0
    with ose3d.Modeler(ose3d.default_params(**KW), BACK) as m:
        m.reset_shot(0)
        img, ill = m.rtm(obs, every=2)
    inner = img[B:B + N, B + 16:B + N - 16, B + 16:B + N - 16]
    il = ill[B:B + N, B + 16:B + N - 16, B + 16:B + N - 16]
    prof = np.abs(inner / (il + 1e-3 * il.max())).sum(axis=(1, 2))
    z = 25 + int(np.argmax(prof[25:60]))
    print(f"rtm: image peak at depth {z} (reflector at {DEPTH}); profile {np.round(prof[25:60] / prof[z], 2)}")
    assert abs(z - DEPTH) <= 3
    assert prof[z] > 2 * np.median(prof[25:60])
