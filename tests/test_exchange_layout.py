"""The index algebra of the 256^3 plane kernels' DSMEM exchange
(3d-ose_gb300/csrc/ose_plane.cu: row_slot, col_slot, push_cols_to_rows,
push_rows_to_cols and the readers after `receive`), restated on the host: an
8-CTA cluster owns one 256 x 256 plane; CTA r holds columns x in [32r, 32r+32)
for the y transforms and rows y in [32r, 32r+32) for the x transforms.  For
both exchanges every value lands exactly once, at the receive-buffer slot the
reading thread takes for the same (y, x), and each CTA receives 7 x 8 KiB
from the others (the byte count its mbarrier is armed with)."""
import numpy as np

N, CL, SL, NS, THREADS, WARPS = 256, 8, 32, 2, 256, 8
PUSH_BYTES = (CL - 1) * SL * SL * 8


def row_slot(t, s):
    lane, warp = t & 31, t >> 5
    return (warp + WARPS * s) * 2 + (lane >> 4), lane & 15


def col_slot(t, s):
    return t & 31, (t >> 5) + WARPS * s


def _check(sent, expect):
    for d in range(CL):
        assert np.all(sent[d] >= 0), f"CTA {d}: receive slots never written"
        assert np.array_equal(sent[d], expect[d])


def test_columns_to_rows_exchange():
    # sent[d][off] = the (y, x) written there, encoded y * N + x
    sent = -np.ones((CL, SL * N), np.int64)
    remote = np.zeros(CL, np.int64)
    for r in range(CL):
        for t in range(THREADS):
            for s in range(NS):
                c, j = col_slot(t, s)
                for n1 in range(16):
                    y, x = 16 * n1 + j, SL * r + c
                    d = n1 >> 1
                    off = (16 * (n1 & 1) + j) * N + SL * r + c
                    assert sent[d, off] < 0, "slot written twice"
                    sent[d, off] = y * N + x
                    if d != r:
                        remote[d] += 8
    expect = -np.ones((CL, SL * N), np.int64)
    for d in range(CL):
        for t in range(THREADS):
            for s in range(NS):
                row, j = row_slot(t, s)
                for k2 in range(16):
                    expect[d, row * N + j + 16 * k2] = (SL * d + row) * N + (j + 16 * k2)
    _check(sent, expect)
    assert np.all(remote == PUSH_BYTES)


def test_rows_to_columns_exchange():
    sent = -np.ones((CL, N * SL), np.int64)
    remote = np.zeros(CL, np.int64)
    for r in range(CL):
        for t in range(THREADS):
            for s in range(NS):
                row, j = row_slot(t, s)
                y = SL * r + row
                for k2 in range(16):
                    x = j + 16 * k2
                    d = k2 >> 1
                    off = y * SL + j + 16 * (k2 & 1)
                    assert sent[d, off] < 0, "slot written twice"
                    sent[d, off] = y * N + x
                    if d != r:
                        remote[d] += 8
    expect = -np.ones((CL, N * SL), np.int64)
    for d in range(CL):
        for t in range(THREADS):
            for s in range(NS):
                c, j = col_slot(t, s)
                for n1 in range(16):
                    expect[d, (16 * n1 + j) * SL + c] = (16 * n1 + j) * N + (SL * d + c)
    _check(sent, expect)
    assert np.all(remote == PUSH_BYTES)


def test_receive_buffer_fits_the_transpose_buffer():
    tpad = 17
    trows = SL * 16 * tpad
    assert SL * N <= trows          # the receive buffer overlays the row transpose buffer
    assert PUSH_BYTES < (1 << 20)   # within an mbarrier's transaction count
