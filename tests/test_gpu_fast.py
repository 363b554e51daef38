"""The reduced split precision (HQR_PREC_OZAKI_FAST) on the GPU through the C
ABI: the updates keep only the slice products of weight <= 3 (10 of 36), so
the factorization is FP32-class; least squares recovers FP64-level answers by
FP64 iterative refinement (hqr_lstsq).

Bars:
  * factorization: ||A - Q R||_F / ||A||_F <= 1e-6 and |R| elementwise within
    1e-5 ||A||_F of the FP64 oracle's (the reduced updates err by about
    2^-30 of rowmax * colmax * K per product, far inside these);
  * it is not the FP64-level path: the R error is above the split path's
    bar (10 n eps ||A||) -- the reduced products are in use;
  * least squares with 3 refinement steps (x += R^-1 (Q^T (b - A x))(1:n),
    the residual in FP64): within 4x the FP64 perturbation bound of the
    other least-squares tests (100 eps kappa (1 + kappa ||r|| / (||A||
    ||x||))) against numpy's solution at kappa 1e3 (measured 1.1x), three
    orders or more below the unrefined error.  This refinement stalls near
    kappa^2 u ||r|| / (||A|| ||x||) with u the factorization's error (about
    5e-9 here), so at kappa 1e6 with 1e-8 noise it ends near 1e-5: there the
    FP64-level split path is the one to use.
"""
import numpy as np
import pytest

import oracle as O
from ls_cases import ls_problem, ls_tol

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


@pytest.mark.parametrize("M,N", [(512, 512), (1024, 384)])
def test_fast_factorization_is_fp32_class(env, M, N):
    H, torch = env
    NB, IB = 128, 32
    A2d = O.uniform_matrix(M, N, 3100 + M + N)
    A = O.to_tiles(A2d, NB)
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    dC = torch.from_numpy(A.copy()).cuda()
    plan = H.Plan(M, N, NB, IB, H.HQR_PREC_OZAKI_FAST)
    L = H.lib()
    try:
        H.check(L.hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "hqr_geqrf")
        # Q^T A with the same reduced updates: [R; 0] up to the factorization's error
        H.check(L.hqr_ormqr_t(plan.h, dA.data_ptr(), dTAU.data_ptr(), dC.data_ptr(), N // NB, 1, None),
                "hqr_ormqr_t")
    finally:
        plan.close()
    ra, _ = O.tile_qr(A, M, N, NB, IB)
    nA = np.linalg.norm(A2d)
    R = np.triu(O.from_tiles(dA.cpu().numpy(), M, N, NB)[:N])
    Ro = np.triu(O.from_tiles(ra, M, N, NB)[:N])
    err = np.abs(R - Ro).max()
    assert err <= 1e-5 * nA
    assert err > 10 * max(M, N) * EPS * nA   # the reduced products are in use
    QtA = O.from_tiles(dC.cpu().numpy(), M, N, NB)
    assert np.linalg.norm(QtA[:N] - R) / nA <= 1e-6
    if M > N:
        assert np.linalg.norm(QtA[N:]) / nA <= 1e-6


@pytest.mark.parametrize("M,N,nrhs,kappa", [(1024, 512, 4, 1e3), (1024, 384, 16, 1e2)])
def test_fast_lstsq_refines_to_fp64(env, M, N, nrhs, kappa):
    H, torch = env
    NB, IB = 128, 32
    A, _, b = ls_problem(M, N, nrhs, kappa, 5100 + M + N)
    dA = torch.from_numpy(O.to_tiles(A, NB)).cuda()
    dB = torch.from_numpy(np.asfortranarray(b).reshape(-1, order="F").copy()).cuda()
    xn = np.linalg.lstsq(A, b, rcond=None)[0]
    t = ls_tol(A, xn, b, kappa)
    errs = []
    plan = H.Plan(M, N, NB, IB, H.HQR_PREC_OZAKI_FAST)
    try:
        for steps in (0, 3):
            dX = torch.zeros(N * nrhs, dtype=torch.float64, device="cuda")
            res = plan.lstsq(dA.data_ptr(), dB.data_ptr(), nrhs, dX.data_ptr(), refine_steps=steps)
            x = dX.cpu().numpy().reshape(N, nrhs, order="F")
            errs.append(np.linalg.norm(x - xn) / np.linalg.norm(xn))
    finally:
        plan.close()
    assert errs[1] <= 4 * t, errs
    assert errs[1] <= 1e-3 * errs[0], errs
    assert errs[1] <= errs[0], errs
    r = np.linalg.norm(b - A @ x, axis=0)
    assert np.allclose(res, r, rtol=1e-10, atol=1e-14)
