"""Reverse-time migration (ose_rtm): a flat reflector at depth 40 cells under
a 2000 m/s layer, reflected data (true model minus the 2000 m/s background)
migrated with the background velocity, must image at depth 40 +- 4 cells
(a quarter of the 100 m wavelength at 20 Hz is 2.5 cells)."""
import numpy as np
import pytest

import ose3d

pytestmark = pytest.mark.gpu

N = 64
KW = dict(nx=N, ny=N, nz=N, bu=20, bd=20, bl=20, br=20, bf=20, bb=20, nt=400, fm=20.0, dt=0.002,
          amp=100.0, dx=10.0, dy=10.0, dz=10.0, sxbeg=N // 2, sybeg=N // 2, szbeg=2, gzbeg=0,
          hilbert_div_nt=1)
DEPTH = 40


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


def record(vel):
    with ose3d.Modeler(ose3d.default_params(**KW), vel) as m:
        m.reset_shot(0)
        return m.run_record(KW["nt"])


def test_rtm_images_a_flat_reflector_at_its_depth():
    true = np.full((N, N, N), 2000.0, np.float32)
    true[:, :, DEPTH:] = 3000.0
    back = np.full((N, N, N), 2000.0, np.float32)
    obs = record(true) - record(back)
    assert np.abs(obs).max() > 0
    with ose3d.Modeler(ose3d.default_params(**KW), back) as m:
        m.reset_shot(0)
        img = m.rtm(obs, every=2)
        with pytest.raises(ose3d.OseError):
            m.step()   # the state now holds the receiver wavefield
    b = KW["bu"]
    inner = img[b:b + N, b + 16:b + N - 16, b + 16:b + N - 16]      # interior depth, central columns
    prof = np.abs(inner).sum(axis=(1, 2))
    prof = np.convolve(prof, np.ones(3) / 3, mode="same")
    z = 15 + int(np.argmax(prof[15:60]))
    print(f"rtm: image peak at depth {z} (reflector at {DEPTH})")
    assert abs(z - DEPTH) <= 4
    assert prof[z] > 3 * np.median(prof[15:60])
