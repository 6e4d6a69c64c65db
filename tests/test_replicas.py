"""The N-GPU forms of the bench have no data-path collective: replicas (one
independent shot per rank) for the single-shot step, and the batched form's
shots dealt round-robin to the ranks.  The ranks meet at a barrier around the
timed region and the slowest rank's time sets the whole-job rate.  World size
2 on the gloo backend (CPU), rendezvous on 127.0.0.1."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_env()
    d = bench.Dist(w)
    d.barrier()
    ms = 100.0 + 25.0 * r            # the ranks' own step times differ
    ms_max = d.max(ms)
    rate = bench.replica_rate(w, 256 ** 3, 300, ms_max)
    shots = bench.shard(range(64), r, w)    # the batched form's shots on this rank
    total = d.sum(float(len(shots)))
    d.barrier()
    d.close()
    q.put((r, w, local, ms_max, rate, shots, total))


def test_two_replicas_meet_and_take_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 and o[2] == o[0] for o in out)
    assert all(o[3] == 125.0 for o in out)                       # max over ranks, seen by both
    expect = 2 * 256 ** 3 * 300 / 0.125 / 1e9                   # whole job: both replicas' cells
    assert all(abs(o[4] - expect) < 1e-9 * expect for o in out)
    # batched shots: disjoint round-robin shares covering all 64, counted once
    assert sorted(out[0][5] + out[1][5]) == list(range(64)) and not set(out[0][5]) & set(out[1][5])
    assert all(o[6] == 64.0 for o in out)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(1)
    d.barrier()
    assert d.max(3.5) == 3.5
    assert bench.replica_rate(1, 1e9, 10, 1000.0) == pytest.approx(10.0)
