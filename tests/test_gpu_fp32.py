"""HQR_PREC_FP32 on the GPU through the C ABI: the panel blocks compute in
FP32 (values kept in FP64 arrays) and the updates keep the slice products of
weight <= 3, an FP32-class factorization -- the reference's FP32
factorization -- and least squares recovers the FP64 solution by refinement
on the augmented system (hqr_lstsq_aug).

Bars:
  * factorization: ||Q^T A - [R; 0]||_F / ||A||_F <= 1e-5 and R elementwise
    within 1e-4 ||A||_F of the FP64 oracle's (single-precision unit roundoff
    6e-8, times the growth of a few hundred columns);
  * FP32 arithmetic is in use: R differs from the oracle's by more than
    HQR_PREC_OZAKI_FAST's does on the same matrix (FP64 panels);
  * least squares: within the FP64 perturbation bound of the other
    least-squares tests (100 eps kappa (1 + kappa ||r|| / (||A|| ||x||)))
    against numpy's solution, with a large residual, at kappa 1e2 and 1e3.
"""
import numpy as np
import pytest

import oracle as O
from ls_cases import ls_problem, ls_tol

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hybrid3_gb300 as H
    H.lib().hqr_set_error_mode(H.HQR_ERRORS_RETURN)
    return H, torch


def factor(H, torch, A, M, N, NB, IB, prec):
    L = H.lib()
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    dC = torch.from_numpy(A.copy()).cuda()
    plan = H.Plan(M, N, NB, IB, prec)
    try:
        H.check(L.hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "hqr_geqrf")
        H.check(L.hqr_ormqr_t(plan.h, dA.data_ptr(), dTAU.data_ptr(), dC.data_ptr(), N // NB, 1, None),
                "hqr_ormqr_t")
    finally:
        plan.close()
    return dA.cpu().numpy(), dC.cpu().numpy()


@pytest.mark.parametrize("M,N", [(512, 512), (1024, 384)])
def test_fp32_factorization_is_fp32_class(env, M, N):
    H, torch = env
    NB, IB = 128, 32
    A2d = O.uniform_matrix(M, N, 4100 + M + N)
    A = O.to_tiles(A2d, NB)
    nA = np.linalg.norm(A2d)
    ra, _ = O.tile_qr(A, M, N, NB, IB)
    Ro = np.triu(O.from_tiles(ra, M, N, NB)[:N])
    errs = {}
    for name, prec in (("fp32", H.HQR_PREC_FP32), ("fast", H.HQR_PREC_OZAKI_FAST)):
        a, c = factor(H, torch, A, M, N, NB, IB, prec)
        R = np.triu(O.from_tiles(a, M, N, NB)[:N])
        errs[name] = np.abs(R - Ro).max()
        if name == "fp32":
            assert errs[name] <= 1e-4 * nA
            QtA = O.from_tiles(c, M, N, NB)
            assert np.linalg.norm(QtA[:N] - R) / nA <= 1e-5
            if M > N:
                assert np.linalg.norm(QtA[N:]) / nA <= 1e-5
    assert errs["fp32"] > errs["fast"], errs


@pytest.mark.parametrize("M,N,nrhs,kappa,noise,steps", [(1024, 512, 4, 1e3, 1e-2, 6),
                                                        (1024, 384, 16, 1e2, 1e-8, 4)])
def test_fp32_lstsq_refines_to_fp64_on_the_augmented_system(env, M, N, nrhs, kappa, noise, steps):
    H, torch = env
    NB, IB = 128, 32
    A, _, b = ls_problem(M, N, nrhs, kappa, 6100 + M + N, noise=noise)
    dA = torch.from_numpy(O.to_tiles(A, NB)).cuda()
    dB = torch.from_numpy(np.asfortranarray(b).reshape(-1, order="F").copy()).cuda()
    dX = torch.zeros(N * nrhs, dtype=torch.float64, device="cuda")
    xn = np.linalg.lstsq(A, b, rcond=None)[0]
    plan = H.Plan(M, N, NB, IB, H.HQR_PREC_FP32)
    try:
        res = plan.lstsq(dA.data_ptr(), dB.data_ptr(), nrhs, dX.data_ptr(), refine_steps=steps, augmented=True)
    finally:
        plan.close()
    x = dX.cpu().numpy().reshape(N, nrhs, order="F")
    assert np.linalg.norm(x - xn) / np.linalg.norm(xn) <= ls_tol(A, xn, b, kappa)
    r = np.linalg.norm(b - A @ x, axis=0)
    assert np.allclose(res, r, rtol=1e-10, atol=1e-14)
