"""Replicas on the GPU: two ranks (spawned processes, gloo rendezvous on
127.0.0.1, both on cuda:0) each run their own shot — shot index = rank, as
bench.py's replicas do — with no data-path collective between them; their
receiver gathers and final wavefields equal, bit for bit, the same two shots
run one after the other in one process.  No kernel of one rank waits on the
other's."""
import os
import socket
import sys

import numpy as np
import pytest

import ose3d

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KW = dict(nx=40, ny=36, nz=30, bu=8, bd=8, bl=8, br=8, bf=8, bb=8, nt=40, fm=30.0, dt=0.001, amp=100.0,
          sxbeg=12, sybeg=10, szbeg=4, jsx=9, jsy=7, jsz=2)
STEPS = 30


def _model():
    rng = np.random.default_rng(12)
    return (1800.0 + 1500.0 * rng.random((KW["nx"], KW["ny"], KW["nz"]))).astype(np.float32)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    for sub in ("", "3d-ose_gb300", "oracle"):
        sys.path.insert(0, os.path.join(ROOT, sub))
    import bench
    import ose3d as O3
    r, w, _ = bench.dist_env()
    d = bench.Dist(w)
    with O3.Modeler(O3.default_params(**KW), _model()) as m:
        m.reset_shot(r)
        d.barrier()
        g = m.run_record(STEPS)
        d.barrier()
        q.put((r, g, m.wavefield(O3.FIELD_Q), m.wavefield(O3.FIELD_P)))
    d.close()


def test_two_ranks_reproduce_their_shots():
    import __graft_entry__ as ge
    ge.build_library()
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {o[0]: o[1:] for o in (q.get(timeout=600) for _ in procs)}
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    ose3d.load_library()
    for shot in (0, 1):
        with ose3d.Modeler(ose3d.default_params(**KW), _model()) as m:
            m.reset_shot(shot)
            g = m.run_record(STEPS)
            ref = (g, m.wavefield(ose3d.FIELD_Q), m.wavefield(ose3d.FIELD_P))
        for a, b in zip(out[shot], ref):
            assert np.array_equal(a, b)
    assert not np.array_equal(out[0][0], out[1][0])   # two different shots
