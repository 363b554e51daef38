"""Host-side entry points of the drop-in library on the CPU (no device work):
the TileSch FIFO (TileSch.c:10-173) and mat_prod's status and norm helpers
(mat_prod.c:15-154), against the reference's behaviour read from its
sources."""
import ctypes
import math
import os

import numpy as np
import pytest


@pytest.fixture(scope="module")
def H():
    import hybrid3_gb300 as H
    if not os.path.exists(H.LIB_PATH):
        pytest.skip("library not built")
    H.lib()
    return H


def entry(H, i, j, k, data=0):
    return H.TilSch(i, j, k, 0, data)


def test_tilsch_fifo_capacity_and_wraparound(H):
    L = H.lib()
    q = H.TilSchList()
    L.TilSch_init(ctypes.byref(q), 3)
    assert L.TilSch_empty(ctypes.byref(q)) == 1
    for n in range(3):
        assert L.TilSch_push(ctypes.byref(q), entry(H, n, n + 1, n + 2)) == 1
    assert L.TilSch_fully(ctypes.byref(q)) == 1
    assert L.TilSch_push(ctypes.byref(q), entry(H, 9, 9, 9)) == 0   # full: refused
    out = H.TilSch()
    got = []
    # interleave pops and pushes past the ring's end: order stays FIFO
    for n in range(3, 8):
        assert L.TilSch_pop(ctypes.byref(q), ctypes.byref(out)) == 1
        got.append((out.i, out.j, out.k))
        assert L.TilSch_push(ctypes.byref(q), entry(H, n, n + 1, n + 2)) == 1
    while L.TilSch_pop(ctypes.byref(q), ctypes.byref(out)):
        got.append((out.i, out.j, out.k))
    assert got == [(n, n + 1, n + 2) for n in range(8)]
    assert L.TilSch_empty(ctypes.byref(q)) == 1
    assert q.max_size == 3


def test_tilsch_depend_accumulates_bits(H):
    L = H.lib()
    MEM, LIN, YT, END = 0x1, 0x2, 0x4, 0x7
    q = H.TilSchList()
    L.TilSch_init(ctypes.byref(q), 8)
    e = entry(H, 1, 2, 3)
    # END on its own: reported ready, nothing queued
    assert L.TilSch_depend(ctypes.byref(q), e, END) == 1
    assert L.TilSch_empty(ctypes.byref(q)) == 1
    # a missing entry is appended with the given bits; later bits are OR-ed in
    assert L.TilSch_depend(ctypes.byref(q), e, MEM) == 0
    assert q.tail - q.head == 1
    assert L.TilSch_depend(ctypes.byref(q), e, LIN) == 0
    assert L.TilSch_depend(ctypes.byref(q), entry(H, 4, 5, 6), MEM) == 0
    assert L.TilSch_depend(ctypes.byref(q), e, YT) == 1   # MEM | LIN | YT == END
    assert q.tail - q.head == 2


def test_tilsch_delete_matches_the_reference_filter(H):
    L = H.lib()
    q = H.TilSchList()
    L.TilSch_init(ctypes.byref(q), 8)
    for n in range(4):
        assert L.TilSch_push(ctypes.byref(q), entry(H, n, 0, 0, 0)) == 1
    # the entry must match (i, j, k) and (data & 0x0f00) == (i & 0x0f00)
    assert L.TilSch_delete(ctypes.byref(q), entry(H, 2, 0, 0)) == 1
    assert L.TilSch_delete(ctypes.byref(q), entry(H, 2, 0, 0)) == 0
    assert L.TilSch_delete(ctypes.byref(q), entry(H, 1, 0, 1)) == 0
    out = H.TilSch()
    left = []
    while L.TilSch_pop(ctypes.byref(q), ctypes.byref(out)):
        left.append(out.i)
    assert left == [0, 1, 3]


@pytest.mark.parametrize("M,N,tm,tn,rank,procs", [(1000, 700, 128, 128, 0, 1), (1000, 700, 128, 128, 0, 2),
                                                 (1000, 700, 128, 128, 1, 2), (512, 2048, 64, 256, 2, 3)])
def test_mat_init_fields(H, M, N, tm, tn, rank, procs):
    st = H.MatStat()
    H.lib().mat_init(ctypes.byref(st), M, N, tm, tn, rank, procs)
    tiles_n = N // tn
    mine = tiles_n // procs + (1 if tiles_n % procs > rank else 0)
    assert (st.mat_M, st.mat_N) == (M, N)
    assert st.my_mat_M == M                      # not truncated, as in the reference
    assert (st.glob_tile_M, st.my_tile_M) == (M // tm, M // tm)
    assert (st.glob_tile_N, st.my_tile_N) == (tiles_n, mine)
    assert st.my_mat_N == tn * mine
    assert (st.tile_M, st.tile_N) == (tm, tn)


def test_mat_comp3_is_the_one_norm_and_propagates_nan(H):
    st = H.status(256, 128, 64)
    rng = np.random.default_rng(3)
    E = rng.standard_normal(256 * 128)
    P = ctypes.POINTER(ctypes.c_double)
    got = H.lib().mat_comp3(ctypes.byref(st), E.ctypes.data_as(P), 0, 1)
    assert got == pytest.approx(np.abs(E.reshape(128, 256)).sum(axis=1).max(), rel=1e-14)
    E[300] = np.nan
    assert math.isnan(H.lib().mat_comp3(ctypes.byref(st), E.ctypes.data_as(P), 0, 1))


def test_mat_dprint_is_tile_to_column_major(H):
    import oracle as O
    M, N, NB = 192, 128, 64
    st = H.status(M, N, NB)
    A2d = np.arange(M * N, dtype=np.float64).reshape(N, M).T   # column-major values 0..
    T = np.ascontiguousarray(O.to_tiles(A2d, NB))
    out = np.zeros(M * N)
    P = ctypes.POINTER(ctypes.c_double)
    H.lib().mat_dprint(ctypes.byref(st), out.ctypes.data_as(P), T.ctypes.data_as(P))
    assert np.array_equal(out, np.arange(M * N, dtype=np.float64))


def test_mat_remv_undoes_mat_make(H):
    st = H.status(128, 128, 32)
    A = np.zeros(128 * 128)
    P = ctypes.POINTER(ctypes.c_double)
    H.lib().mat_make(ctypes.byref(st), A.ctypes.data_as(P), 77, 0)
    assert A.min() >= 0.0 and A.max() <= 1.0 and A.std() > 0.2
    H.lib().mat_remv(ctypes.byref(st), A.ctypes.data_as(P), 77, 0)
    assert np.abs(A).max() == 0.0


def test_status_strings(H):
    L = H.lib()
    codes = [H.HQR_OK, H.HQR_ERR_INVALID, H.HQR_ERR_CUDA, H.HQR_ERR_TIMEOUT, H.HQR_ERR_NOMEM,
             H.HQR_ERR_UNSUPPORTED, H.HQR_ERR_DEVICE]
    texts = [L.hqr_status_string(c).decode() for c in codes]
    assert all(texts) and len(set(texts)) == len(texts)


def test_drop_in_rejects_bad_status_before_any_device_work(H):
    """The drop-in entry points validate mat_stat_t first (one rank, square
    tiles, whole tiles), so these calls never reach the device."""
    L = H.lib()
    L.hqr_set_error_mode(H.HQR_ERRORS_RETURN)
    P = ctypes.POINTER(ctypes.c_double)
    A = np.zeros(256 * 256)
    tau = np.zeros(128 * 128)
    bad = []
    st = H.MatStat()
    L.mat_init(ctypes.byref(st), 256, 256, 128, 128, 0, 2)      # two ranks
    bad.append((st, 0, 2))
    st = H.MatStat()
    L.mat_init(ctypes.byref(st), 256, 256, 128, 64, 0, 1)       # non-square tiles
    bad.append((st, 0, 1))
    st = H.MatStat()
    L.mat_init(ctypes.byref(st), 250, 256, 128, 128, 0, 1)      # rows not whole tiles
    bad.append((st, 0, 1))
    for st, rank, procs in bad:
        L.Hybrid_tile_QR(ctypes.byref(st), A.ctypes.data_as(P), tau.ctypes.data_as(P), rank, procs, 32)
        assert L.hqr_last_error() == H.HQR_ERR_INVALID
        L.Hybrid_make_Q(ctypes.byref(st), A.ctypes.data_as(P), A.ctypes.data_as(P), tau.ctypes.data_as(P),
                        rank, procs, 32)
        assert L.hqr_last_error() == H.HQR_ERR_INVALID
    L.Hybrid_tile_QR(None, A.ctypes.data_as(P), tau.ctypes.data_as(P), 0, 1, 32)
    assert L.hqr_last_error() == H.HQR_ERR_INVALID
