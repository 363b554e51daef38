"""GPU parity of the tiled QR path, through the C ABI, against the CPU oracle
and the reference's golden outputs.

Tolerance: |gpu - oracle| <= n * eps * ||A||_F elementwise (n = max(M, N)),
i.e. c*n*eps*||A|| with c = 1; R and V use the same Householder sign
convention (LAPACK dlarfg) and the same flat top-to-bottom TS tree as the
reference, so they agree elementwise, not only up to signs.
"""
import ctypes
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
DP = ctypes.POINTER(ctypes.c_double)


def P(a):
    return a.ctypes.data_as(DP)


@pytest.fixture(scope="module")
def H():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hybrid3_gb300 as H
    H.lib().hqr_set_error_mode(H.HQR_ERRORS_RETURN)
    return H


def tol(A2d):
    return max(A2d.shape) * EPS * np.linalg.norm(A2d)


def gpu_tile_qr(H, A, M, N, NB, IB):
    st = H.status(M, N, NB)
    a = np.ascontiguousarray(A.copy())
    tau = np.zeros(max((M // 2) * (N // 2), (M // NB) * (N // NB) * NB))
    H.lib().Hybrid_tile_QR(ctypes.byref(st), P(a), P(tau), 0, 1, IB)
    H.check(H.lib().hqr_last_error(), "Hybrid_tile_QR")
    return a, tau[: (M // NB) * (N // NB) * NB]


SHAPES = [(128, 128, 32, 8), (256, 256, 64, 16), (512, 512, 128, 32), (384, 128, 32, 8),
          (512, 256, 64, 32), (768, 768, 256, 32), (1024, 512, 256, 64), (256, 256, 32, 32)]


@pytest.mark.parametrize("M,N,NB,IB", SHAPES)
def test_tile_qr_matches_oracle(H, M, N, NB, IB):
    A2d = O.uniform_matrix(M, N, 1000 + M + N + NB)
    A = O.to_tiles(A2d, NB)
    ra, rtau = O.tile_qr(A, M, N, NB, IB)
    a, tau = gpu_tile_qr(H, A, M, N, NB, IB)
    t = tol(A2d)
    assert np.abs(a - ra).max() <= t
    assert np.abs(tau - rtau).max() <= t


@pytest.mark.parametrize("name", ["qr_uniform_n128_nb32_ib8.npz", "qr_matmake_n128_nb32_ib8.npz",
                                  "qr_uniform_n128_nb32_ib32.npz"])
def test_against_reference_golden(H, golden_dir, name):
    g = dict(np.load(os.path.join(golden_dir, name)))
    M, N, NB, IB = (int(g[k]) for k in ("M", "N", "NB", "IB"))
    t = tol(O.from_tiles(g["A"], M, N, NB))
    a, tau = gpu_tile_qr(H, g["A"], M, N, NB, IB)
    assert np.abs(a - g["A_qr"]).max() <= t
    assert np.abs(tau - g["TAU"]).max() <= t
    # Hybrid_make_Q on the reference's factorization
    st = H.status(M, N, NB)
    q = np.zeros(M * N)
    r = g["A_qr"].copy()
    H.lib().Hybrid_make_Q(ctypes.byref(st), P(q), P(r), P(g["TAU"].copy()), 0, 1, IB)
    H.check(H.lib().hqr_last_error())
    assert np.abs(q - g["Qt"]).max() <= t
    assert np.array_equal(r, g["R"])
    # Hybrid_dorgqr / Hybrid_dormqr
    q2 = np.full(M * N, 7.0)
    H.lib().Hybrid_dorgqr(ctypes.byref(st), P(q2), P(g["A_qr"].copy()), P(g["TAU"].copy()), 0, 1)
    H.check(H.lib().hqr_last_error())
    assert np.abs(q2 - g["Qt_dorgqr"]).max() <= t
    c = g["C"].copy()
    H.lib().Hybrid_dormqr(ctypes.byref(st), P(g["A_qr"].copy()), P(g["TAU"].copy()), P(c), 0, 1)
    H.check(H.lib().hqr_last_error())
    assert np.abs(c - g["QtC"]).max() <= 4 * tol(O.from_tiles(g["C"], M, N, NB))
    # Hybrid_dgemm (Q Q^T and Q R checks of main.c)
    qq = np.zeros(M * N)
    H.lib().Hybrid_dgemm(ctypes.byref(st), P(g["Qt"].copy()), P(g["Qt"].copy()), P(qq), 0, 1)
    H.check(H.lib().hqr_last_error())
    assert np.abs(qq - g["QQt"]).max() <= 1e-13
    qr = np.zeros(M * N)
    H.lib().Hybrid_dgemm(ctypes.byref(st), P(g["Qt"].copy()), P(g["R"].copy()), P(qr), 0, 1)
    assert np.abs(qr - g["QR"]).max() <= 1e-13


@pytest.mark.parametrize("M,N,NB,IB", [(256, 256, 64, 16), (512, 512, 128, 32), (512, 256, 64, 32)])
def test_make_q_matches_oracle_and_is_orthogonal(H, M, N, NB, IB):
    A2d = O.uniform_matrix(M, N, 77 + M)
    A = O.to_tiles(A2d, NB)
    a, tau = gpu_tile_qr(H, A, M, N, NB, IB)
    oq, orr = O.make_Q(a, tau, M, N, NB)
    st = H.status(M, N, NB)
    q = np.zeros(M * N)
    r = a.copy()
    H.lib().Hybrid_make_Q(ctypes.byref(st), P(q), P(r), P(tau.copy()), 0, 1, IB)
    H.check(H.lib().hqr_last_error())
    t = tol(A2d)
    assert np.abs(q - oq).max() <= t
    assert np.array_equal(r, orr)
    if M == N:
        Qt = O.from_tiles(q, M, N, NB)
        R = O.from_tiles(r, M, N, NB)
        assert np.linalg.norm(A2d - Qt.T @ R) / np.linalg.norm(A2d) < 1e-14
        assert np.linalg.norm(Qt @ Qt.T - np.eye(M)) < 1e-13


def test_make_identity_and_remv_y(H):
    M = N = 128
    NB = 32
    st = H.status(M, N, NB)
    I = np.full(M * N, 3.0)
    H.lib().Hybrid_make_I(ctypes.byref(st), P(I), 0, 1)
    H.check(H.lib().hqr_last_error())
    assert np.array_equal(O.from_tiles(I, M, N, NB), np.eye(M))
    A = O.to_tiles(O.uniform_matrix(M, N, 5), NB)
    a, tau = gpu_tile_qr(H, A, M, N, NB, 8)
    r = a.copy()
    H.lib().Hybrid_remv_Y(ctypes.byref(st), P(r), 0, 1)
    H.check(H.lib().hqr_last_error())
    R = O.from_tiles(r, M, N, NB)
    assert np.array_equal(R, np.triu(O.from_tiles(a, M, N, NB)))


def test_invalid_arguments_return_errors(H):
    L = H.lib()
    st = H.status(128, 128, 32)
    a = np.zeros(128 * 128)
    tau = np.zeros(64 * 64)
    L.Hybrid_tile_QR(ctypes.byref(st), P(a), P(tau), 0, 2, 8)     # two ranks: not supported
    assert L.hqr_last_error() == H.HQR_ERR_INVALID
    h = ctypes.c_void_p()
    assert L.hqr_plan_create(ctypes.byref(h), 100, 128, 32, 8, 0) == H.HQR_ERR_INVALID
    assert L.hqr_plan_create(ctypes.byref(h), 128, 128, 24, 8, 0) == H.HQR_ERR_UNSUPPORTED


def test_extended_api_device_pointers(H):
    torch = pytest.importorskip("torch")
    M = N = 512
    NB, IB = 128, 32
    A2d = O.uniform_matrix(M, N, 9)
    A = O.to_tiles(A2d, NB)
    plan = H.Plan(M, N, NB, IB)
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    H.check(H.lib().hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), s), "geqrf")
    ra, rtau = O.tile_qr(A, M, N, NB, IB)
    assert np.abs(dA.cpu().numpy() - ra).max() <= tol(A2d)
    st = plan.stats(s)
    MT = NT = M // NB
    NC = {128: 1}.get(NB, None)
    # GEQRT and TSQRT counts are fixed by the grid, one task per inner block
    # of w = min(IB, 32) columns
    nblk = NB // min(IB, 32)
    assert st["count"][0] == MT * nblk
    assert st["count"][1] == MT * (MT - 1) // 2 * nblk
    # make_q with the persisted T factors equals the rebuild path
    dQ = torch.zeros(M * N, dtype=torch.float64, device="cuda")
    dR = dA.clone()
    H.check(H.lib().hqr_make_q(plan.h, dQ.data_ptr(), dR.data_ptr(), dTAU.data_ptr(), 1, s), "make_q")
    oq, _ = O.make_Q(ra, rtau, M, N, NB)
    assert np.abs(dQ.cpu().numpy() - oq).max() <= tol(A2d)
    # checks on the device: ||A - Q R||_F via A^T B of the Q^T array with R
    dQR = torch.zeros_like(dQ)
    H.check(H.lib().hqr_dgemm_tn(N, NB, dQ.data_ptr(), dR.data_ptr(), dQR.data_ptr(), s))
    dA0 = torch.from_numpy(A.copy()).cuda()
    r2 = ctypes.c_double()
    H.check(H.lib().hqr_frob2(M, N, NB, dQR.data_ptr(), dA0.data_ptr(), 0.0, ctypes.byref(r2), s))
    assert np.sqrt(r2.value) / np.linalg.norm(A2d) < 1e-14
    plan.close()


def test_device_fill_matches_oracle_generator(H):
    torch = pytest.importorskip("torch")
    M, N, NB = 256, 128, 64
    d = torch.zeros(M * N, dtype=torch.float64, device="cuda")
    H.check(H.lib().hqr_fill_uniform(M, N, NB, 123, d.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), O.to_tiles(O.uniform_matrix(M, N, 123), NB))


def test_scheduler_wait_limit_returns_timeout_and_recovers(H):
    """A 1 ms wait limit is far shorter than one 256-wide panel task, so idle
    CTAs give up: the run must end with HQR_ERR_TIMEOUT (no hang, no fault)
    and the next run, with the default limit, must succeed."""
    L = H.lib()
    M = N = 1024
    NB, IB = 256, 32
    A = O.to_tiles(O.uniform_matrix(M, N, 3), NB)
    st = H.status(M, N, NB)
    a = A.copy()
    tau = np.zeros((M // 2) * (N // 2))
    L.hqr_set_timeout_ms(1)
    try:
        L.Hybrid_tile_QR(ctypes.byref(st), P(a), P(tau), 0, 1, IB)
        assert L.hqr_last_error() == H.HQR_ERR_TIMEOUT
    finally:
        L.hqr_set_timeout_ms(20000)
    a2, tau2 = gpu_tile_qr(H, A, M, N, NB, IB)
    ra, rtau = O.tile_qr(A, M, N, NB, IB)
    assert np.abs(a2 - ra).max() <= tol(O.from_tiles(A, M, N, NB))
