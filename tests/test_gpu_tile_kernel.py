"""GPU parity of the reference's per-tile kernels (include/tile_kernel.h) with
their own conventions (beta = +||x||, lower T), through the C ABI:

  * against the reference's own outputs (tests/golden/tile_kernels_nb32_ib8.npz,
    made by the reference's tile_kernel.c), host pointers;
  * against the oracle's restatement of tile_kernel.c on ragged shapes, leading
    dimensions larger than the row count and the quirks the reference has;
  * device pointers (used in place) give the host-pointer results.

Bar: |gpu - oracle| <= 64 n eps max(1, ||inputs||_F) elementwise (the sums run
in a different order on the GPU).
"""
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hybrid3_gb300 as H
    H.lib().hqr_set_error_mode(H.HQR_ERRORS_RETURN)
    return torch, H


def P(a):
    return a.ctypes.data


def F(a):
    return np.asfortranarray(a)


def tol(n, *arrays):
    return 64 * n * EPS * max([1.0] + [float(np.linalg.norm(a)) for a in arrays])


def ok(H):
    assert H.lib().hqr_last_error() == H.HQR_OK


def test_tile_kernels_match_the_reference_outputs(env, golden_dir):
    torch, H = env
    L = H.lib()
    g = np.load(os.path.join(golden_dir, "tile_kernels_nb32_ib8.npz"))
    NB, IB = int(g["NB"]), int(g["IB"])
    t = tol(NB, g["geqrt_A"])
    A = F(g["geqrt_A"].copy())
    TAU = np.zeros(NB)
    Y = np.zeros((NB, NB), order="F")
    T = np.zeros((NB, NB), order="F")
    L.tile_dgeqrt(NB, NB, IB, P(A), NB, P(TAU), P(Y), P(T), NB, None)
    ok(H)
    assert np.abs(A - g["geqrt_A_out"]).max() <= t
    assert np.abs(TAU[:-1] - g["geqrt_TAU"][:-1]).max() <= t   # the last TAU is never written
    assert np.abs(Y - g["geqrt_Y"]).max() <= t
    assert np.abs(T - g["geqrt_T"]).max() <= t
    T2 = np.zeros((NB, NB), order="F")
    L.tile_dlarft(NB, NB, 1, P(Y), NB, P(TAU), P(T2), NB, None)
    assert np.abs(np.tril(T2) - np.tril(g["larft_T"])).max() <= t
    C = F(g["larfb_C"].copy())
    L.tile_dlarfb(NB, NB, P(C), NB, P(Y), P(T2), NB, None)
    assert np.abs(C - g["larfb_C_out"]).max() <= t
    R = F(g["tsqrt_R"].copy())
    A2 = F(g["tsqrt_A2"].copy())
    TAU = np.zeros(NB)
    T = np.zeros((NB, NB), order="F")
    L.tile_dtsqrt(NB, NB, IB, P(R), NB, P(A2), NB, P(TAU), P(T), NB, None)
    ok(H)
    assert np.abs(R - g["tsqrt_R_out"]).max() <= t
    assert np.abs(A2 - g["tsqrt_V"]).max() <= t
    assert np.abs(TAU - g["tsqrt_TAU"]).max() <= t
    assert np.abs(T - g["tsqrt_T"]).max() <= t
    T3 = np.zeros((NB, NB), order="F")
    L.tile_dlarft(NB, NB, 1, P(A2), NB, P(TAU), P(T3), NB, None)
    assert np.abs(T3 - g["tsqrt_fullT"]).max() <= t
    A1 = F(g["ssrfb_A1"].copy())
    B2 = F(g["ssrfb_A2"].copy())
    L.tile_dssrfb(NB, NB, P(A1), P(B2), NB, P(A2), P(T3), NB, None)
    ok(H)
    assert np.abs(A1 - g["ssrfb_A1_out"]).max() <= t
    assert np.abs(B2 - g["ssrfb_A2_out"]).max() <= t


@pytest.mark.parametrize("row,col,lda", [(40, 24, 48), (32, 32, 32), (64, 16, 64), (17, 16, 20)])
def test_sub_dgeqr2_matches_oracle(env, row, col, lda):
    torch, H = env
    rng = np.random.default_rng(row * col)
    A0 = rng.uniform(-1, 1, (lda, col))
    A, Ao = F(A0.copy()), F(A0.copy())
    TAU, TAUo = np.full(col, 7.0), np.full(col, 7.0)      # sentinel: unwritten entries stay 7
    Y, Yo = np.zeros((lda, col), order="F"), np.zeros((lda, col), order="F")
    H.lib().tile_sub_dgeqr2(row, col, P(A), lda, P(TAU), P(Y), None)
    ok(H)
    O.lib().orc_tk_sub_dgeqr2(row, col, O.ptr(Ao), lda, O.ptr(TAUo), O.ptr(Yo), O.ptr(np.zeros(3 * lda * col)))
    t = tol(row, A0[:row])
    assert np.abs(A - Ao).max() <= t
    assert np.abs(TAU - TAUo).max() <= t
    assert np.abs(Y - Yo).max() <= t
    if row == col:   # quirk: the last TAU is left as it was and Y(col-1, col-1) = 0
        assert TAU[-1] == 7.0 and Y[col - 1, col - 1] == 0.0


@pytest.mark.parametrize("row,col", [(32, 32), (48, 20), (24, 8)])
def test_sub_dtsqr2_matches_oracle(env, row, col):
    torch, H = env
    rng = np.random.default_rng(100 + row)
    A1_0 = np.triu(rng.uniform(-1, 1, (col + 3, col)))
    A2_0 = rng.uniform(-1, 1, (row + 5, col))
    A1, A1o = F(A1_0.copy()), F(A1_0.copy())
    A2, A2o = F(A2_0.copy()), F(A2_0.copy())
    TAU, TAUo = np.zeros(col), np.zeros(col)
    H.lib().tile_sub_dtsqr2(row, col, P(A1), col + 3, P(A2), row + 5, P(TAU), None)
    ok(H)
    O.lib().orc_tk_sub_dtsqr2(row, col, O.ptr(A1o), col + 3, O.ptr(A2o), row + 5, O.ptr(TAUo),
                              O.ptr(np.zeros(3 * (row + col) * col)))
    t = tol(row + col, A1_0, A2_0)
    for x, y in [(A1, A1o), (A2, A2o), (TAU, TAUo)]:
        assert np.abs(x - y).max() <= t


@pytest.mark.parametrize("row,col,block", [(32, 32, 8), (40, 24, 8), (48, 40, 16), (32, 20, 8)])
def test_dgeqrt_and_dtsqrt_match_oracle(env, row, col, block):
    torch, H = env
    L, Lo = H.lib(), O.lib()
    rng = np.random.default_rng(row + col + block)
    A0 = rng.uniform(-1, 1, (row, col))
    A, Ao = F(A0.copy()), F(A0.copy())
    TAU, TAUo = np.zeros(col), np.zeros(col)
    Y, Yo = np.zeros((row, col), order="F"), np.zeros((row, col), order="F")
    T, To = np.zeros((col, col), order="F"), np.zeros((col, col), order="F")
    L.tile_dgeqrt(row, col, block, P(A), row, P(TAU), P(Y), P(T), col, None)
    ok(H)
    Lo.orc_tk_dgeqrt(row, col, block, O.ptr(Ao), row, O.ptr(TAUo), O.ptr(Yo), O.ptr(To), col,
                     O.ptr(np.zeros(3 * row * col)))
    t = tol(row, A0)
    for x, y in [(A, Ao), (Y, Yo), (T, To)]:
        assert np.abs(x - y).max() <= t
    n = col - 1 if row == col else col
    assert np.abs(TAU[:n] - TAUo[:n]).max() <= t
    # tsqrt on [R; dense]
    R0 = np.triu(rng.uniform(-1, 1, (col, col)))
    B0 = rng.uniform(-1, 1, (row, col))
    R, Ro, B, Bo = F(R0.copy()), F(R0.copy()), F(B0.copy()), F(B0.copy())
    TAU, TAUo = np.zeros(col), np.zeros(col)
    T, To = np.zeros((col, col), order="F"), np.zeros((col, col), order="F")
    L.tile_dtsqrt(row, col, block, P(R), col, P(B), row, P(TAU), P(T), col, None)
    ok(H)
    Lo.orc_tk_dtsqrt(row, col, block, O.ptr(Ro), col, O.ptr(Bo), row, O.ptr(TAUo), O.ptr(To), col,
                     O.ptr(np.zeros(3 * (row + col) * col)))
    t = tol(row + col, R0, B0)
    for x, y in [(R, Ro), (B, Bo), (TAU, TAUo), (T, To)]:
        assert np.abs(x - y).max() <= t


def test_wide_tiles_are_rejected(env):
    """row < col walks the reference's dgeqr2 loop past the last row: rejected."""
    torch, H = env
    A = np.zeros((16, 24), order="F")
    TAU, Y = np.zeros(24), np.zeros((16, 24), order="F")
    H.lib().tile_sub_dgeqr2(16, 24, P(A), 16, P(TAU), P(Y), None)
    assert H.lib().hqr_last_error() == H.HQR_ERR_INVALID
    T = np.zeros((24, 24), order="F")
    H.lib().tile_dgeqrt(16, 24, 8, P(A), 16, P(TAU), P(Y), P(T), 24, None)
    assert H.lib().hqr_last_error() == H.HQR_ERR_INVALID


def reflectors(rng, row, col):
    """Y (unit lower, zeros above the diagonal) and TAU of a real factorization
    (the oracle's tile_sub_dgeqr2 of a random row x col tile, row > col)."""
    A = F(rng.uniform(-1, 1, (row, col)))
    Y = np.zeros((row, col), order="F")
    tau = np.zeros(col)
    O.lib().orc_tk_sub_dgeqr2(row, col, O.ptr(A), row, O.ptr(tau), O.ptr(Y), O.ptr(np.zeros(3 * row * col)))
    return Y, tau


def test_sub_dlarft_and_dlarft_blocks_match_oracle(env):
    torch, H = env
    L, Lo = H.lib(), O.lib()
    rng = np.random.default_rng(5)
    row, col = 48, 32
    Y, tau = reflectors(rng, row, col)
    T = np.zeros((col, col), order="F")
    To = np.zeros((col, col), order="F")
    L.tile_sub_dlarft(row, col, P(Y), row, P(tau), P(T), col, None)
    ok(H)
    Lo.orc_tk_sub_dlarft(row, col, O.ptr(Y), row, O.ptr(tau), O.ptr(To), col, O.ptr(np.zeros(3 * row * col)))
    t = tol(row, Y, To)
    assert np.abs(T - To).max() <= t
    # block path: couples existing diagonal blocks (T starts as the block-diagonal part)
    for block in (8, 16):
        Tb = np.zeros((col, col), order="F")
        for i in range(0, col, block):
            Tb[i:i + block, i:i + block] = np.tril(To[i:i + block, i:i + block])
        Tg, Tr = F(Tb.copy()), F(Tb.copy())
        L.tile_dlarft(row, col, block, P(Y), row, P(tau), P(Tg), col, None)
        ok(H)
        Lo.orc_tk_dlarft(row, col, block, O.ptr(Y), row, O.ptr(tau), O.ptr(Tr), col,
                         O.ptr(np.zeros(3 * row * col + col * col)))
        assert np.abs(Tg - Tr).max() <= t
    # quirk: block >= col leaves T untouched
    Tu = F(rng.uniform(-1, 1, (col, col)))
    T0 = Tu.copy()
    L.tile_dlarft(row, col, col, P(Y), row, P(tau), P(Tu), col, None)
    assert np.array_equal(Tu, T0)


def test_sub_dlarfb_and_sub_dssrfb_match_oracle(env):
    torch, H = env
    L, Lo = H.lib(), O.lib()
    rng = np.random.default_rng(9)
    row, ycol, acol = 40, 24, 16
    Y, tau = reflectors(rng, row, row - 1)
    Y = F(np.hstack([Y, np.zeros((row, 1))]))
    tau = np.append(tau, 0.0)
    T = np.zeros((ycol, ycol), order="F")
    Lo.orc_tk_sub_dlarft(row, ycol, O.ptr(Y), row, O.ptr(tau), O.ptr(T), ycol, O.ptr(np.zeros(3 * row * row)))
    A0 = rng.uniform(-1, 1, (row, acol))
    A, Ao = F(A0.copy()), F(A0.copy())
    L.tile_sub_dlarfb(row, ycol, acol, P(Y), row, P(T), ycol, P(A), row, None)
    ok(H)
    Lo.orc_tk_sub_dlarfb(row, ycol, acol, O.ptr(Y), row, O.ptr(T), ycol, O.ptr(Ao), row,
                         O.ptr(np.zeros(3 * row * row)))
    assert np.abs(A - Ao).max() <= tol(row, A0, Y, T)
    # SSRFB with over_row > Y_col: rows Y_col.. of A1 are zeroed (quirk)
    over, under = 32, 40
    V = F(rng.uniform(-1, 1, (under, ycol)))
    A1_0 = rng.uniform(-1, 1, (over, acol))
    A2_0 = rng.uniform(-1, 1, (under, acol))
    A1, A1o, A2, A2o = F(A1_0.copy()), F(A1_0.copy()), F(A2_0.copy()), F(A2_0.copy())
    L.tile_sub_dssrfb(over, under, ycol, acol, P(V), under, P(T), ycol, P(A1), over, P(A2), under, None)
    ok(H)
    Lo.orc_tk_sub_dssrfb(over, under, ycol, acol, O.ptr(V), under, O.ptr(T), ycol, O.ptr(A1o), over,
                         O.ptr(A2o), under, O.ptr(np.zeros(3 * under * under)))
    t = tol(under, A1_0, A2_0, V, T)
    assert np.abs(A1 - A1o).max() <= t
    assert np.abs(A2 - A2o).max() <= t
    assert np.all(A1[ycol:] == 0.0)


def test_head_tail_and_return_variants(env):
    torch, H = env
    L, Lo = H.lib(), O.lib()
    rng = np.random.default_rng(11)
    row = col = 32
    V = F(rng.uniform(-1, 1, (row, col)))
    T = F(np.tril(rng.uniform(-1, 1, (col, col))))
    A1_0, A2_0 = rng.uniform(-1, 1, (row, col)), rng.uniform(-1, 1, (row, col))
    # tile_dssrfb == head then tail
    A1, A2 = F(A1_0.copy()), F(A2_0.copy())
    L.tile_dssrfb(row, col, P(A1), P(A2), row, P(V), P(T), col, None)
    B1, B2 = F(A1_0.copy()), F(A2_0.copy())
    U = np.zeros((row, col), order="F")
    L.tile_dssrfb_head(row, col, P(B1), P(B2), row, P(V), P(T), col, P(U))
    L.tile_dssrfb_tail(row, col, P(B2), row, P(V), P(U))
    ok(H)
    t = tol(row, A1_0, A2_0, V, T)
    assert np.abs(A1 - B1).max() <= t and np.abs(A2 - B2).max() <= t
    # return variants read T transposed: W = T^T (A1 + V^T A2)
    Tl = np.tril(T)
    W = Tl.T @ (A1_0 + V.T @ A2_0)
    C1, C2 = F(A1_0.copy()), F(A2_0.copy())
    L.tile_return_dssrfb(row, col, P(C1), P(C2), row, P(V), P(T), col, None)
    ok(H)
    assert np.abs(C1 - (A1_0 - W)).max() <= t
    assert np.abs(C2 - (A2_0 - V @ W)).max() <= t
    Yl = F(np.tril(V))
    C = F(A1_0.copy())
    L.tile_return_dlarfb(row, col, P(C), row, P(Yl), P(T), col, None)
    ok(H)
    assert np.abs(C - (A1_0 - Yl @ (Tl.T @ (Yl.T @ A1_0)))).max() <= t
    # tile_return_dlarft: tile_sub_dlarft's T stored transposed (upper)
    Y, tau = reflectors(rng, row + 8, col)
    row = row + 8
    Tlow = np.zeros((col, col), order="F")
    Lo.orc_tk_sub_dlarft(row, col, O.ptr(Y), row, O.ptr(tau), O.ptr(Tlow), col, O.ptr(np.zeros(3 * row * col)))
    Tup = np.zeros((col, col), order="F")
    L.tile_return_dlarft(row, col, P(Y), row, P(tau), P(Tup), col, None)
    ok(H)
    assert np.abs(Tup - Tlow.T).max() <= tol(row, Y, Tlow)


def test_device_pointers_are_used_in_place(env):
    torch, H = env
    L = H.lib()
    rng = np.random.default_rng(3)
    row, col, block = 48, 32, 8
    A0 = F(rng.uniform(-1, 1, (row, col)))
    hA, hTAU = A0.copy(order="F"), np.zeros(col)
    hY, hT = np.zeros((row, col), order="F"), np.zeros((col, col), order="F")
    L.tile_dgeqrt(row, col, block, P(hA), row, P(hTAU), P(hY), P(hT), col, None)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.T).copy()).cuda()   # column-major storage
    dA, dTAU = dev(A0), torch.zeros(col, dtype=torch.float64, device="cuda")
    dY = torch.zeros((col, row), dtype=torch.float64, device="cuda")
    dT = torch.zeros((col, col), dtype=torch.float64, device="cuda")
    L.tile_dgeqrt(row, col, block, dA.data_ptr(), row, dTAU.data_ptr(), dY.data_ptr(), dT.data_ptr(), col, None)
    ok(H)
    back = lambda d: d.cpu().numpy().T
    assert np.array_equal(back(dA), hA)
    assert np.array_equal(dTAU.cpu().numpy(), hTAU)
    assert np.array_equal(back(dY), hY)
    assert np.array_equal(back(dT), hT)
