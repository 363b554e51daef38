"""Batched uneven QR (hqr_batch_*) on the GPU through the C ABI: one
persistent launch factors every matrix of the batch, a second applies Q^T to
their right-hand sides.  Each matrix is checked against the oracle's
Hybrid_tile_QR / Hybrid_dormqr on the same seeded input, elementwise within
c n eps ||A|| (the single-matrix tests' bar), so the batched executor is held
to the same parity as the single-matrix one."""
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
    return H, torch


def tol(A2d):
    return 20 * max(A2d.shape) * EPS * max(1.0, np.linalg.norm(A2d))


# M, N, NB, IB: tall, square, wide, one tile, mixed tile orders in one batch
SHAPES = [(64, 32, 32, 8), (256, 128, 64, 16), (384, 384, 128, 32), (128, 128, 32, 32),
          (512, 128, 128, 32), (96, 96, 32, 16), (640, 192, 64, 32), (32, 32, 32, 8),
          (256, 512, 64, 16), (1024, 256, 128, 32), (192, 64, 64, 16), (448, 448, 64, 32),
          (288, 192, 96, 32), (384, 384, 192, 32), (192, 96, 96, 16), (512, 256, 256, 32)]


def rhs_tiles(C2d, NB):
    """M x nrhs right-hand sides as an MT x ceil(nrhs / NB) tile grid (zero-filled)."""
    M, nrhs = C2d.shape
    Cp = np.zeros((M, -(-nrhs // NB) * NB))
    Cp[:, :nrhs] = C2d
    return O.to_tiles(Cp, NB)


def make_batch(H, torch, shapes, seed0, nrhs):
    A, C, dA, dT, dC = [], [], [], [], []
    for b, (M, N, NB, IB) in enumerate(shapes):
        A2d = O.uniform_matrix(M, N, seed0 + 7 * b)
        C2d = O.uniform_matrix(M, nrhs, seed0 + 7 * b + 3)
        A.append(A2d)
        C.append(C2d)
        dA.append(torch.from_numpy(O.to_tiles(A2d, NB)).cuda())
        dC.append(torch.from_numpy(rhs_tiles(C2d, NB)).cuda())
        dT.append(torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda"))
    return A, C, dA, dT, dC


def check_against_oracle(shapes, A, C, dA, dT, dC, nrhs):
    for b, (M, N, NB, IB) in enumerate(shapes):
        At = O.to_tiles(A[b], NB)
        ra, rtau = O.tile_qr(At, M, N, NB, IB)
        t = tol(A[b])
        a = dA[b].cpu().numpy()
        assert np.abs(a - ra).max() <= t, (b, M, N, NB, IB)
        assert np.abs(dT[b].cpu().numpy() - rtau).max() <= t, (b, M, N, NB, IB)
        CT = -(-nrhs // NB)
        rc = O.from_tiles(O.dormqr(ra, rtau, rhs_tiles(C[b], NB), M, N, NB, CT), M, CT * NB, NB)[:, :nrhs]
        got = O.from_tiles(dC[b].cpu().numpy(), M, CT * NB, NB)[:, :nrhs]
        tc = 20 * M * EPS * max(1.0, np.linalg.norm(C[b]))
        assert np.abs(got - rc).max() <= tc, (b, M, N, NB, IB)


# 4: one column block of 8; 40: part of a tile (two of four blocks at NB 128);
# 100: whole tiles at NB 32 / 64, a partial one at 128; 200: several tile columns
@pytest.mark.parametrize("nrhs", [4, 40, 100, 200])
def test_batch_matches_oracle_per_matrix(env, nrhs):
    H, torch = env
    shapes = SHAPES
    A, C, dA, dT, dC = make_batch(H, torch, shapes, 500 + nrhs, nrhs)
    bt = H.Batch([s[0] for s in shapes], [s[1] for s in shapes], [s[2] for s in shapes],
                 [s[3] for s in shapes], max_nrhs=200)
    try:
        bt.geqrf([x.data_ptr() for x in dA], [x.data_ptr() for x in dT])
        st = bt.stats()
        bt.ormqr_t([x.data_ptr() for x in dA], [x.data_ptr() for x in dT], [x.data_ptr() for x in dC], nrhs)
    finally:
        bt.close()
    check_against_oracle(shapes, A, C, dA, dT, dC, nrhs)
    # the batch ran exactly the tasks of the single-matrix factorizations
    want = [0] * 6
    for b, (M, N, NB, IB) in enumerate(shapes):
        plan = H.Plan(M, N, NB, IB, H.HQR_PREC_FP64)
        try:
            x = torch.from_numpy(O.to_tiles(A[b], NB)).cuda()
            tau = torch.zeros_like(dT[b])
            H.check(H.lib().hqr_geqrf(plan.h, x.data_ptr(), tau.data_ptr(), None), "hqr_geqrf")
            c = plan.stats()["count"]
        finally:
            plan.close()
        want = [w + v for w, v in zip(want, c[:6])]
    assert st["count"][:6] == want
    assert st["count"][6] == sum(want)   # one scheduling pass per task


@pytest.mark.parametrize("ctas", [1, 2])
def test_batch_ctas_per_sm(env, ctas):
    """Small tiles run with one or two executor CTAs per SM: same results."""
    H, torch = env
    shapes = [s for s in SHAPES if s[2] <= 64 or (s[2] == 128 and s[3] == 16)] + [(512, 384, 128, 16)]
    A, C, dA, dT, dC = make_batch(H, torch, shapes, 620, 4)
    bt = H.Batch([s[0] for s in shapes], [s[1] for s in shapes], [s[2] for s in shapes],
                 [s[3] for s in shapes], max_nrhs=4, ctas_per_sm=ctas)
    try:
        assert bt.ctas_per_sm() == ctas
        bt.geqrf([x.data_ptr() for x in dA], [x.data_ptr() for x in dT])
        bt.ormqr_t([x.data_ptr() for x in dA], [x.data_ptr() for x in dT], [x.data_ptr() for x in dC], 4)
    finally:
        bt.close()
    check_against_oracle(shapes, A, C, dA, dT, dC, 4)


def test_batch_many_small_uneven(env):
    """A few hundred matrices of random uneven shapes (multiples of 32, NB 32)."""
    H, torch = env
    rng = np.random.default_rng(11)
    shapes = []
    for _ in range(300):
        m = 32 * int(rng.integers(1, 9))
        n = 32 * int(rng.integers(1, m // 32 + 1))
        shapes.append((m, n, 32, int(rng.choice([8, 16, 32]))))
    A, C, dA, dT, dC = make_batch(H, torch, shapes, 900, 4)
    bt = H.Batch([s[0] for s in shapes], [s[1] for s in shapes], [s[2] for s in shapes],
                 [s[3] for s in shapes], max_nrhs=4)
    try:
        bt.geqrf([x.data_ptr() for x in dA], [x.data_ptr() for x in dT])
        bt.ormqr_t([x.data_ptr() for x in dA], [x.data_ptr() for x in dT], [x.data_ptr() for x in dC], 4)
    finally:
        bt.close()
    idx = list(range(0, 300, 13))
    check_against_oracle([shapes[i] for i in idx], [A[i] for i in idx], [C[i] for i in idx],
                         [dA[i] for i in idx], [dT[i] for i in idx], [dC[i] for i in idx], 4)


def test_batch_zero_padding_keeps_r(env):
    """m x n matrices (multiples of 32) padded with zeros to NB = 64 / 128
    multiples: the leading n x n block of R is the unpadded matrix's R."""
    H, torch = env
    orig = [(96, 32), (160, 96), (224, 224), (352, 160)]
    shapes, padded = [], []
    for b, (m, n) in enumerate(orig):
        NB = 64 if b % 2 == 0 else 128
        Mp, Np = -(-m // NB) * NB, -(-n // NB) * NB
        A2d = np.zeros((Mp, Np))
        A2d[:m, :n] = O.uniform_matrix(m, n, 40 + b)
        shapes.append((Mp, Np, NB, 32))
        padded.append(A2d)
    dA = [torch.from_numpy(O.to_tiles(A2d, s[2])).cuda() for A2d, s in zip(padded, shapes)]
    dT = [torch.zeros((s[0] // s[2]) * (s[1] // s[2]) * s[2], dtype=torch.float64, device="cuda")
          for s in shapes]
    bt = H.Batch([s[0] for s in shapes], [s[1] for s in shapes], [s[2] for s in shapes],
                 [s[3] for s in shapes], max_nrhs=4)
    try:
        bt.geqrf([x.data_ptr() for x in dA], [x.data_ptr() for x in dT])
    finally:
        bt.close()
    for b, (m, n) in enumerate(orig):
        Mp, Np, NB, _ = shapes[b]
        R = np.triu(O.from_tiles(dA[b].cpu().numpy(), Mp, Np, NB)[:n, :n])
        ra, _ = O.tile_qr(O.to_tiles(padded[b][:m, :n], 32), m, n, 32, 32)
        Ro = np.triu(O.from_tiles(ra, m, n, 32)[:n])
        t = tol(padded[b])
        assert np.abs(np.abs(R) - np.abs(Ro)).max() <= t, b
        # the padded rows carry no reflector entries
        assert np.abs(O.from_tiles(dA[b].cpu().numpy(), Mp, Np, NB)[m:, :n]).max() == 0.0


def test_batch_in_a_cuda_graph(env):
    """geqrf + ormqr_t captured once (after a call that uploads the task tables)
    and replayed on new data in the same buffers."""
    H, torch = env
    shapes = SHAPES[:6]
    A, C, dA, dT, dC = make_batch(H, torch, shapes, 300, 4)
    pa, pt, pc = [x.data_ptr() for x in dA], [x.data_ptr() for x in dT], [x.data_ptr() for x in dC]
    bt = H.Batch([s[0] for s in shapes], [s[1] for s in shapes], [s[2] for s in shapes],
                 [s[3] for s in shapes], max_nrhs=4)
    try:
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            bt.geqrf(pa, pt, stream=s.cuda_stream)
            bt.ormqr_t(pa, pt, pc, 4, stream=s.cuda_stream)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            bt.geqrf(pa, pt, stream=s.cuda_stream, wait=False)
            bt.ormqr_t(pa, pt, pc, 4, stream=s.cuda_stream, wait=False)
        A2, C2 = [], []
        for b, (M, N, NB, IB) in enumerate(shapes):
            A2.append(O.uniform_matrix(M, N, 7000 + b))
            C2.append(O.uniform_matrix(M, 4, 7100 + b))
            dA[b].copy_(torch.from_numpy(O.to_tiles(A2[b], NB)))
            dC[b].copy_(torch.from_numpy(rhs_tiles(C2[b], NB)))
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        bt.status()
    finally:
        bt.close()
    check_against_oracle(shapes, A2, C2, dA, dT, dC, 4)


def test_batch_invalid_arguments(env):
    H, torch = env
    import ctypes
    L = H.lib()
    h = ctypes.c_void_p()
    Ls, Is = ctypes.c_long, ctypes.c_int
    # M not a multiple of NB
    assert L.hqr_batch_create(ctypes.byref(h), 1, (Ls * 1)(100), (Ls * 1)(64), (Is * 1)(64), (Is * 1)(16),
                              1, 0) == H.HQR_ERR_INVALID
    assert L.hqr_batch_create(ctypes.byref(h), 0, None, None, None, None, 1, 0) == H.HQR_ERR_INVALID
    # NB 256 tiles do not fit two executor CTAs per SM
    assert L.hqr_batch_create(ctypes.byref(h), 1, (Ls * 1)(256), (Ls * 1)(256), (Is * 1)(256), (Is * 1)(32),
                              1, 2) == H.HQR_ERR_UNSUPPORTED
    bt = H.Batch([128], [128], [64], [16], max_nrhs=4)
    dA = torch.zeros(128 * 128, dtype=torch.float64, device="cuda")
    dT = torch.zeros(2 * 2 * 64, dtype=torch.float64, device="cuda")
    try:
        P = H._ptrs
        assert L.hqr_batch_ormqr_t(bt.h, P([dA.data_ptr()]), P([dT.data_ptr()]), P([dA.data_ptr()]), 5,
                                   None) == H.HQR_ERR_INVALID   # nrhs > max_nrhs
        assert L.hqr_batch_geqrf(bt.h, P([0]), P([dT.data_ptr()]), None) == H.HQR_ERR_INVALID
    finally:
        bt.close()
