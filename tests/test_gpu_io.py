"""Checkpoint/resume, snapshots, SU/SEG-Y output and the host driver's files
against the reference's own files (goldens from tests/golden/make_golden.py)."""
import os
import subprocess

import numpy as np
import pytest

import ose3d
from golden_util import load, model_of, rel_l2

pytestmark = pytest.mark.gpu
ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


def small():
    g = load("small_judge_odd")
    kw = dict(g["params"])
    kw.pop("nsteps")
    return kw, model_of(g)


def test_checkpoint_resume_is_exact(tmp_path):
    kw, vel = small()
    p = ose3d.default_params(**kw)
    with ose3d.Modeler(p, vel) as a:
        a.reset_shot(0)
        a.run(20)
        q_ref, g_ref = a.wavefield(ose3d.FIELD_Q), a.gather()
    ck = str(tmp_path / "shot.ck")
    with ose3d.Modeler(p, vel) as b:
        b.reset_shot(0)
        b.run(8)
        b.checkpoint_save(ck)
    with ose3d.Modeler(p, vel) as c:
        c.checkpoint_load(ck)
        assert c.it == 8
        c.run(12)
        assert np.array_equal(c.wavefield(ose3d.FIELD_Q), q_ref)
        assert np.array_equal(c.gather(), g_ref)
    # a handle with other parameters refuses the file
    kw2 = dict(kw, fm=kw["fm"] + 1.0)
    with ose3d.Modeler(ose3d.default_params(**kw2), vel) as d:
        with pytest.raises(ose3d.OseError):
            d.checkpoint_load(ck)


def test_snapshots_match_stepping():
    kw, vel = small()
    p = ose3d.default_params(**kw)
    got = {}
    with ose3d.Modeler(p, vel) as a:
        a.reset_shot(0)
        a.run_snapshots(30, 7, lambda it, P, Q: got.__setitem__(it, (P, Q)), ose3d.LAYOUT_YXZ)
        assert a.it == 30
    assert sorted(got) == [6, 13, 20, 27, 29]
    with ose3d.Modeler(p, vel) as b:
        b.reset_shot(0)
        done = 0
        for it in sorted(got):
            b.run(it + 1 - done)
            done = it + 1
            assert np.array_equal(got[it][1], b.wavefield(ose3d.FIELD_Q, ose3d.LAYOUT_YXZ))
            assert np.array_equal(got[it][0], b.wavefield(ose3d.FIELD_P, ose3d.LAYOUT_YXZ))


def su_traces(path, nt, big=False):
    e = ">" if big else "<"
    dt = np.dtype([("hdr", "u1", 240), ("data", e + "f4", nt)])
    with open(path, "rb") as f:
        raw = f.read()
    off = 3600 if big else 0
    return np.frombuffer(raw[off:], dtype=dt), raw[:off]


def hdr(tr, off, fmt, big=False):
    return np.frombuffer(tr["hdr"][:, off:off + np.dtype(fmt).itemsize].tobytes(),
                         dtype=(">" if big else "<") + fmt)


@pytest.mark.parametrize("segy", [False, True])
def test_su_and_segy_traces(tmp_path, segy):
    kw, vel = small()
    kw = dict(kw, jsx=2)
    p = ose3d.default_params(**kw)
    path = str(tmp_path / ("g.sgy" if segy else "g.su"))
    with ose3d.Modeler(p, vel) as m:
        m.reset_shot(1)
        m.run(25)
        g = m.gather()
        (m.write_segy if segy else m.write_su)(path)
        ng, nt = m.derived.ng, p.nt
    tr, head = su_traces(path, nt, big=segy)
    assert len(tr) == ng
    assert np.array_equal(tr["data"].astype(np.float32), g)
    assert np.array_equal(hdr(tr, 0, "i4", segy), np.arange(1, ng + 1))      # tracl
    assert np.all(hdr(tr, 8, "i4", segy) == 2)                                # fldr = shot + 1
    assert np.all(hdr(tr, 114, "u2", segy) == nt)                             # ns
    assert np.all(hdr(tr, 116, "u2", segy) == round(p.dt * 1e6))              # dt
    assert np.all(hdr(tr, 70, "i2", segy) == -100)                            # scalco
    sx = (p.sxbeg + 1 * p.jsx) * p.dx
    assert np.all(hdr(tr, 72, "i4", segy) == round(100 * sx))
    ig = np.arange(ng)
    assert np.array_equal(hdr(tr, 80, "i4", segy), np.round(100 * (ig % p.nx) * p.dx).astype(np.int32))
    if segy:
        binh = head[3200:3600]
        assert int.from_bytes(binh[24:26], "big") == 5          # IEEE float
        assert int.from_bytes(binh[20:22], "big") == nt


def test_driver_writes_the_reference_files(tmp_path):
    """The host driver with the reference main()'s parameters and model: the
    same partest.txt bytes, the same 300-float sponge dump, the same source
    traces and (first 3 steps) the same gather as the reference's own run."""
    g = load("reference_default")
    (tmp_path / "input").mkdir()
    model_of(g).astype("<f4").tofile(tmp_path / "input" / "v3d_nx101_ny101_nz101.bin")
    exe = os.path.join(ROOT, "3d-ose_gb300", "lib", "ose_3d")
    r = subprocess.run([exe, "nsteps=3"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "output" / "partest.txt").read_bytes() == bytes(g["partest"])
    att = np.fromfile(tmp_path / "temp" / "att_x_0.bin", "<f4")
    assert att.shape == g["att_x_dump"].shape
    assert np.max(np.abs(att - g["att_x_dump"])) <= 2e-7
    rk = np.fromfile(tmp_path / "temp" / "ricker_card.bin", "<f4")
    hl = np.fromfile(tmp_path / "temp" / "hilbert_card.bin", "<f4")
    assert np.max(np.abs(rk - g["ricker"])) <= 1e-6 * np.abs(g["ricker"]).max()
    assert np.max(np.abs(hl - g["hilbert"])) <= 2e-6 * np.abs(g["hilbert"]).max()
    q = np.fromfile(tmp_path / "output" / "qshot2.bin", "<f4")
    assert q.nbytes == int(g["qshot2_bytes"])
    q = q.reshape(-1, 300)
    assert rel_l2(q[:, :3], g["gather"].T) < 1e-4
    assert np.all(q[:, 3:] == 0)
