"""Receiver lists (ose_set_receivers): the reference's gxyz geometry
(sg_init_device, ose_3d_kernel.cu:202-212) honoured.  A receiver at interior
cell (x, y, z) records the same Q, bit for bit, as the receiver plane at depth
z records at (x, y); headers and reverse-time migration follow the list."""
import struct

import numpy as np
import pytest

import ose3d

pytestmark = pytest.mark.gpu

KW = dict(nx=24, ny=20, nz=18, bu=6, bd=6, bl=6, br=6, bf=6, bb=6, nt=30, fm=30.0, dt=0.0015, amp=50.0,
          sxbeg=12, sybeg=10, szbeg=4, gzbeg=0)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


@pytest.fixture(scope="module")
def vel():
    rng = np.random.default_rng(21)
    return (1800 + 1500 * rng.random((KW["nx"], KW["ny"], KW["nz"]))).astype(np.float32)


def plane_gather(vel, depth):
    with ose3d.Modeler(ose3d.default_params(**dict(KW, gzbeg=depth)), vel) as m:
        m.reset_shot(0)
        return m.run(KW["nt"], want_gather=True)


def test_list_equals_the_planes_at_its_depths(vel):
    line = ose3d.receiver_line(2, 1, 3, 3, 2, 0, 6)              # the reference's jumps, depth 3
    extra = np.array([[5, 17, 9], [20, 3, 9], [0, 0, 0]], np.int32)   # other depths
    xyz = np.concatenate([line, extra])
    with ose3d.Modeler(ose3d.default_params(**KW), vel) as m:
        m.set_receivers(xyz)
        assert m.derived.ng == len(xyz)
        m.reset_shot(0)
        g = m.run(KW["nt"], want_gather=True)
        assert g.shape == (len(xyz), KW["nt"])
    planes = {d: plane_gather(vel, d) for d in set(xyz[:, 2].tolist())}
    for i, (x, y, z) in enumerate(xyz):
        assert np.array_equal(g[i], planes[z][y * KW["nx"] + x]), (i, x, y, z)


def test_back_to_the_plane_and_bad_receivers(vel):
    with ose3d.Modeler(ose3d.default_params(**KW), vel) as m:
        m.set_receivers([[1, 1, 1]])
        with pytest.raises(ose3d.OseError):
            m.set_receivers([[KW["nx"], 0, 0]])
        m.set_receivers(None)
        assert m.derived.ng == KW["nx"] * KW["ny"]
        m.reset_shot(0)
        g = m.run(KW["nt"], want_gather=True)
    assert np.array_equal(g, plane_gather(vel, 0))


def test_su_headers_carry_the_list_coordinates(vel, tmp_path):
    xyz = np.array([[3, 4, 2], [10, 7, 5]], np.int32)
    with ose3d.Modeler(ose3d.default_params(**KW), vel) as m:
        m.set_receivers(xyz)
        m.reset_shot(0)
        m.run(KW["nt"])
        path = str(tmp_path / "list.su")
        m.write_su(path)
    raw = open(path, "rb").read()
    tr = 240 + 4 * KW["nt"]
    assert len(raw) == tr * len(xyz)
    for i, (x, y, z) in enumerate(xyz):
        h = raw[i * tr:i * tr + 240]
        gelev, = struct.unpack_from("<i", h, 40)
        gx, gy = struct.unpack_from("<ii", h, 80)
        assert (gx, gy) == (int(100 * x * 10.0), int(100 * y * 10.0))
        assert gelev == -int(100 * z * 10.0)


def test_rtm_refocuses_with_a_sparse_receiver_list():
    n = 48
    kw = dict(nx=n, ny=n, nz=n, bu=16, bd=16, bl=16, br=16, bf=16, bb=16, nt=300, fm=20.0, dt=0.002,
              amp=100.0, sxbeg=24, sybeg=24, szbeg=24, gzbeg=0, hilbert_div_nt=1)
    vel = np.full((n, n, n), 2000.0, np.float32)
    xs, ys = np.meshgrid(np.arange(0, n, 2), np.arange(0, n, 2), indexing="ij")
    xyz = np.stack([xs.ravel(), ys.ravel(), np.zeros(xs.size, int)], axis=1)
    with ose3d.Modeler(ose3d.default_params(**kw), vel) as m:
        m.set_receivers(xyz)
        m.reset_shot(0)
        d = m.run_record(kw["nt"])
        assert d.shape == (kw["nt"], len(xyz))
        m.reset_shot(0)
        m.rtm(d, every=50)
        P, Q = m.wavefield(ose3d.FIELD_P), m.wavefield(ose3d.FIELD_Q)
    b = kw["bu"]
    E = (P.astype(np.float64) ** 2 + Q.astype(np.float64) ** 2)[b:b + n, b:b + n, b:b + n]
    z, y, x = np.unravel_index(np.argmax(E), E.shape)
    print(f"sparse-list refocus at {(x, y, z)}, source at (24, 24, 24)")
    assert abs(x - 24) <= 1 and abs(y - 24) <= 1 and abs(z - 24) <= 1
