"""GPU parity on the workload configurations themselves, through the C ABI.

* CPU configuration: m = n = 2048, NB = 256, IB = 32, uniform[-1,1) seed
  20151130, plain FP64, through the drop-in entry points (Hybrid_tile_QR,
  Hybrid_make_Q, Hybrid_dorgqr, Hybrid_dormqr) against the oracle.
* The GPU configuration's tile orders and inner blocks, NB in {256, 512} x
  IB in {32, 64}, at n = 2048, and its tall shape scaled down to 8192 x 1024
  (32 x 4 tiles at NB = 256).
* The split precision (NB = 128) at n = 2048.
* The reference's own accuracy at n = 8192 (tests/golden/ref_norms.json,
  written by tests/golden/make_golden.py --norms from the reference's build):
  the GPU's ||A - QR||_F / ||A||_F and ||I - Q Q^T||_F must be no worse.

Elementwise bar: |gpu - oracle| <= n * eps * ||A||_F (n = max(M, N)) for R, V,
TAU and Q; 4x that of ||C||_F for Q^T C (two applications of n-long products).
Residual and orthogonality: at most 1.25x the oracle's (FP64) or 4x (split).
"""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
DP = ctypes.POINTER(ctypes.c_double)
SEED = 20151130


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


def quality(A2d, q_tiles, r_tiles, n, NB):
    Qt = O.from_tiles(q_tiles, n, n, NB)
    R = O.from_tiles(r_tiles, n, n, NB)
    return (np.linalg.norm(A2d - Qt.T @ R) / np.linalg.norm(A2d),
            np.linalg.norm(Qt @ Qt.T - np.eye(n)))


def dropin_qr_and_q(H, A, n, NB, IB, precision):
    """Hybrid_tile_QR then Hybrid_make_Q on host arrays (the reference's calls,
    main.c:148,175), with the drop-in precision set to `precision`."""
    L = H.lib()
    st = H.status(n, n, NB)
    a = np.ascontiguousarray(A.copy())
    tau = np.zeros((n // 2) * (n // 2))
    L.hqr_set_default_precision(precision)
    try:
        L.Hybrid_tile_QR(ctypes.byref(st), P(a), P(tau), 0, 1, IB)
        H.check(L.hqr_last_error(), "Hybrid_tile_QR")
        q = np.zeros(n * n)
        r = a.copy()
        L.Hybrid_make_Q(ctypes.byref(st), P(q), P(r), P(tau.copy()), 0, 1, IB)
        H.check(L.hqr_last_error(), "Hybrid_make_Q")
    finally:
        L.hqr_set_default_precision(H.HQR_PREC_FP64)
    return a, tau[: (n // NB) ** 2 * NB], q, r


def test_cpu_configuration_n2048_nb256_ib32(H):
    n, NB, IB = 2048, 256, 32
    A2d = O.uniform_matrix(n, n, SEED)
    A = O.to_tiles(A2d, NB)
    ra, rtau = O.tile_qr(A, n, n, NB, IB)
    a, tau, q, r = dropin_qr_and_q(H, A, n, NB, IB, H.HQR_PREC_FP64)
    t = tol(A2d)
    assert np.abs(a - ra).max() <= t
    assert np.abs(tau - rtau).max() <= t
    oq, orr = O.make_Q(ra, rtau, n, n, NB)
    assert np.abs(q - oq).max() <= t
    assert np.abs(r - orr).max() <= t
    res, orth = quality(A2d, q, r, n, NB)
    ref_res, ref_orth = quality(A2d, oq, orr, n, NB)
    assert res <= 1.25 * ref_res and orth <= 1.25 * ref_orth, (res, ref_res, orth, ref_orth)
    # Hybrid_dorgqr and Hybrid_dormqr on the GPU's factorization
    L = H.lib()
    st = H.status(n, n, NB)
    q2 = np.full(n * n, 3.0)
    L.Hybrid_dorgqr(ctypes.byref(st), P(q2), P(a.copy()), P(tau.copy()), 0, 1)
    H.check(L.hqr_last_error(), "Hybrid_dorgqr")
    assert np.abs(q2 - O.dorgqr(a, tau, n, n, NB)).max() <= t
    C2d = O.uniform_matrix(n, n, 4242)
    C = O.to_tiles(C2d, NB)
    c = C.copy()
    L.Hybrid_dormqr(ctypes.byref(st), P(a.copy()), P(tau.copy()), P(c), 0, 1)
    H.check(L.hqr_last_error(), "Hybrid_dormqr")
    assert np.abs(c - O.dormqr(a, tau, C, n, n, NB, n // NB)).max() <= 4 * tol(C2d)


@pytest.mark.parametrize("NB,IB", [(256, 64), (512, 32), (512, 64)])
def test_gpu_configuration_tile_orders_n2048(H, NB, IB):
    n = 2048
    A2d = O.uniform_matrix(n, n, SEED)
    A = O.to_tiles(A2d, NB)
    ra, rtau = O.tile_qr(A, n, n, NB, IB)
    a, tau, q, r = dropin_qr_and_q(H, A, n, NB, IB, H.HQR_PREC_FP64)
    t = tol(A2d)
    assert np.abs(a - ra).max() <= t
    assert np.abs(tau - rtau).max() <= t
    oq, orr = O.make_Q(ra, rtau, n, n, NB)
    assert np.abs(q - oq).max() <= t
    assert np.abs(r - orr).max() <= t
    res, orth = quality(A2d, q, r, n, NB)
    ref_res, ref_orth = quality(A2d, oq, orr, n, NB)
    assert res <= 1.25 * ref_res and orth <= 1.25 * ref_orth, (res, ref_res, orth, ref_orth)


@pytest.mark.parametrize("NB,IB", [(256, 32), (512, 64)])
def test_tall_shape_8192x1024(H, NB, IB):
    """The tall GPU configuration's aspect, scaled down; factorization and
    Q^T C through the device API (the reference driver does not finish tall
    matrices: it only terminates at a GEQRT on the last tile row)."""
    torch = pytest.importorskip("torch")
    M, N = 8192, 1024
    A2d = O.uniform_matrix(M, N, SEED)
    A = O.to_tiles(A2d, NB)
    ra, rtau = O.tile_qr(A, M, N, NB, IB)
    plan = H.Plan(M, N, NB, IB)
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    H.check(H.lib().hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "hqr_geqrf")
    t = tol(A2d)
    assert np.abs(dA.cpu().numpy() - ra).max() <= t
    assert np.abs(dTAU.cpu().numpy() - rtau).max() <= t
    C2d = O.uniform_matrix(M, NB, 4243)
    C = O.to_tiles(C2d, NB)
    dC = torch.from_numpy(C.copy()).cuda()
    H.check(H.lib().hqr_ormqr_t(plan.h, dA.data_ptr(), dTAU.data_ptr(), dC.data_ptr(), 1, 1, None),
            "hqr_ormqr_t")
    oc = O.dormqr(ra, rtau, C, M, N, NB, 1)
    assert np.abs(dC.cpu().numpy() - oc).max() <= 4 * tol(C2d)
    plan.close()


def test_split_precision_n2048(H):
    n, NB, IB = 2048, 128, 32
    A2d = O.uniform_matrix(n, n, SEED)
    A = O.to_tiles(A2d, NB)
    ra, rtau = O.tile_qr(A, n, n, NB, IB)
    a, tau, q, r = dropin_qr_and_q(H, A, n, NB, IB, H.HQR_PREC_OZAKI)
    t = tol(A2d)
    assert np.abs(a - ra).max() <= t
    assert np.abs(tau - rtau).max() <= t
    oq, orr = O.make_Q(ra, rtau, n, n, NB)
    assert np.abs(q - oq).max() <= t
    assert np.abs(r - orr).max() <= t
    res, orth = quality(A2d, q, r, n, NB)
    ref_res, ref_orth = quality(A2d, oq, orr, n, NB)
    assert res <= 4 * ref_res and orth <= 4 * ref_orth, (res, ref_res, orth, ref_orth)


def reference_norms(golden_dir, n, NB, IB):
    path = os.path.join(golden_dir, "ref_norms.json")
    for c in json.load(open(path))["cases"]:
        if c["n"] == n and c["NB"] == NB and c["IB"] == IB:
            return c
    pytest.fail(f"no reference norms for n={n} NB={NB} IB={IB} in {path}")


def device_quality(H, torch, n, NB, dA0, dR, dQ):
    """||A - Q R||_F / ||A||_F and ||I - Q Q^T||_F on the device (Hybrid_dgemm's
    A^T B on the Q^T array, main.c:201-258)."""
    L = H.lib()
    dW = torch.empty_like(dA0)
    r2, a2 = ctypes.c_double(), ctypes.c_double()
    H.check(L.hqr_dgemm_tn(n, NB, dQ.data_ptr(), dR.data_ptr(), dW.data_ptr(), None), "QR")
    H.check(L.hqr_frob2(n, n, NB, dW.data_ptr(), dA0.data_ptr(), 0.0, ctypes.byref(r2), None), "frob")
    H.check(L.hqr_frob2(n, n, NB, dA0.data_ptr(), None, 0.0, ctypes.byref(a2), None), "frob")
    res = float(np.sqrt(r2.value / a2.value))
    H.check(L.hqr_dgemm_tn(n, NB, dQ.data_ptr(), dQ.data_ptr(), dW.data_ptr(), None), "QQt")
    H.check(L.hqr_frob2(n, n, NB, dW.data_ptr(), None, 1.0, ctypes.byref(r2), None), "frob")
    return res, float(np.sqrt(r2.value))


@pytest.mark.parametrize("NB,IB,precision,factor", [(256, 32, 0, 1.25), (128, 32, 1, 1.5)])
def test_no_worse_than_the_reference_at_n8192(H, golden_dir, NB, IB, precision, factor):
    torch = pytest.importorskip("torch")
    n = 8192
    ref = reference_norms(golden_dir, n, 256, 32)
    L = H.lib()
    dA0 = torch.empty(n * n, dtype=torch.float64, device="cuda")
    H.check(L.hqr_fill_uniform(n, n, NB, SEED, dA0.data_ptr(), None), "fill")
    dA = dA0.clone()
    dTAU = torch.zeros((n // NB) ** 2 * NB, dtype=torch.float64, device="cuda")
    dQ = torch.zeros_like(dA0)
    plan = H.Plan(n, n, NB, IB, precision)
    H.check(L.hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "hqr_geqrf")
    H.check(L.hqr_make_q(plan.h, dQ.data_ptr(), dA.data_ptr(), dTAU.data_ptr(), 1, None), "hqr_make_q")
    plan.close()
    res, orth = device_quality(H, torch, n, NB, dA0, dA, dQ)
    assert res <= factor * ref["resid_fro_rel"], (res, ref)
    assert orth <= factor * ref["orth_fro"], (orth, ref)


def test_reference_nb256_fixture(H, golden_dir):
    """The reference's own outputs at NB = 256, IB = 32 (n = 512)."""
    g = dict(np.load(os.path.join(golden_dir, "qr_uniform_n512_nb256_ib32.npz")))
    M, N, NB, IB = (int(g[k]) for k in ("M", "N", "NB", "IB"))
    A2d = O.uniform_matrix(M, N, int(g["seed"]))
    A = O.to_tiles(A2d, NB)
    a, tau, q, r = dropin_qr_and_q(H, A, M, NB, IB, H.HQR_PREC_FP64)
    t = tol(A2d)
    assert np.abs(a - g["A_qr"]).max() <= t
    assert np.abs(tau - g["TAU"]).max() <= t
    assert np.abs(q - g["Qt"]).max() <= t
    C2d = O.uniform_matrix(M, N, int(g["c_seed"]))
    c = O.to_tiles(C2d, NB)
    st = H.status(M, N, NB)
    H.lib().Hybrid_dormqr(ctypes.byref(st), P(g["A_qr"].copy()), P(g["TAU"].copy()), P(c), 0, 1)
    H.check(H.lib().hqr_last_error(), "Hybrid_dormqr")
    assert np.abs(c - g["QtC"]).max() <= 4 * tol(C2d)
