"""GPU least squares (hqr_lstsq, through the C ABI) against the FP64 oracle:
the same algorithm restated on the CPU (oracle.lstsq) and numpy's LAPACK
least squares.

Bar: ||x - x_oracle|| / ||x_oracle|| within the perturbation bound of a
backward-stable least-squares solution, 100 eps kappa (1 + kappa ||r|| /
(||A|| ||x||)); the returned residual norms equal ||b - A x|| of the returned
x to 1e-10 and are within 1e-10 of the optimal residual.

hqr_lstsq_aug (refinement on the augmented system) is held to the same bar
from every precision of the factorization, including HQR_PREC_OZAKI_FAST on
problems with a large residual, where hqr_lstsq's refinement stalls; and
against the oracle's restatement of it (oracle.lstsq_aug).
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


def run_gpu(H, torch, A, b, NB, IB, prec, steps, augmented=False):
    M, N = A.shape
    nrhs = b.shape[1]
    dA = torch.from_numpy(O.to_tiles(A, NB)).cuda()
    dB = torch.from_numpy(np.asfortranarray(b).reshape(-1, order="F").copy()).cuda()
    dX = torch.zeros(N * nrhs, dtype=torch.float64, device="cuda")
    plan = H.Plan(M, N, NB, IB, prec)
    try:
        res = plan.lstsq(dA.data_ptr(), dB.data_ptr(), nrhs, dX.data_ptr(), refine_steps=steps,
                         augmented=augmented)
    finally:
        plan.close()
    # A is left unmodified
    assert np.array_equal(dA.cpu().numpy(), O.to_tiles(A, NB))
    return dX.cpu().numpy().reshape(N, nrhs, order="F"), np.array(res)


CASES = [  # M, N, NB, IB, precision, nrhs, kappa, refinement steps
    (512, 256, 128, 32, "fp64", 3, 1e3, 1),
    (512, 256, 64, 16, "fp64", 16, 1e6, 1),
    (512, 256, 128, 32, "split", 16, 1e6, 2),
    (1024, 384, 128, 32, "split", 5, 1e3, 0),
    (768, 768, 128, 32, "split", 130, 1e2, 1),
    (640, 640, 64, 16, "fp64", 1, 1e2, 1),
    (384, 96, 32, 8, "fp64", 7, 1e8, 2),
]


@pytest.mark.parametrize("M,N,NB,IB,prec,nrhs,kappa,steps", CASES)
def test_lstsq_matches_oracle(env, M, N, NB, IB, prec, nrhs, kappa, steps):
    H, torch = env
    A, _, b = ls_problem(M, N, nrhs, kappa, 100 + M + N + nrhs)
    p = H.HQR_PREC_OZAKI if prec == "split" else H.HQR_PREC_FP64
    x, res = run_gpu(H, torch, A, b, NB, IB, p, steps)
    xo = O.lstsq(O.to_tiles(A, NB), b, M, N, NB, IB, steps)
    xn = np.linalg.lstsq(A, b, rcond=None)[0]
    t = ls_tol(A, xn, b, kappa)
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) <= t
    assert np.linalg.norm(x - xn) / np.linalg.norm(xn) <= t
    r = np.linalg.norm(b - A @ x, axis=0)
    rn = np.linalg.norm(b - A @ xn, axis=0)
    assert np.allclose(res, r, rtol=1e-10, atol=1e-14)
    assert np.all(r <= rn * (1 + 1e-10) + 1e-14)


def test_lstsq_refinement_reduces_error(env):
    """One refinement step on the split path: the forward error against numpy's
    solution does not grow, and stays within the bound."""
    H, torch = env
    M, N, NB, IB, nrhs, kappa = 512, 256, 128, 32, 4, 1e6
    A, _, b = ls_problem(M, N, nrhs, kappa, 4242)
    xn = np.linalg.lstsq(A, b, rcond=None)[0]
    errs = []
    for steps in (0, 1):
        x, _ = run_gpu(H, torch, A, b, NB, IB, H.HQR_PREC_OZAKI, steps)
        errs.append(np.linalg.norm(x - xn) / np.linalg.norm(xn))
    assert errs[1] <= max(errs[0], 1e-12) * 1.5
    assert errs[1] <= ls_tol(A, xn, b, kappa)


def test_lstsq_rejects_bad_arguments(env):
    H, torch = env
    import ctypes
    dA = torch.zeros(256 * 512, dtype=torch.float64, device="cuda")
    dB = torch.zeros(256 * 4, dtype=torch.float64, device="cuda")
    dX = torch.zeros(512 * 4, dtype=torch.float64, device="cuda")
    wide = H.Plan(256, 512, 128, 32, H.HQR_PREC_FP64)   # M < N: no least-squares problem
    try:
        rc = H.lib().hqr_lstsq(wide.h, dA.data_ptr(), dB.data_ptr(), 256, 4, dX.data_ptr(), 512, 1,
                               None, None)
        assert rc == H.HQR_ERR_INVALID
    finally:
        wide.close()
    tall = H.Plan(512, 256, 128, 32, H.HQR_PREC_FP64)
    try:
        for nrhs, ldb, ldx in ((0, 512, 256), (4, 100, 256), (4, 512, 100)):
            rc = H.lib().hqr_lstsq(tall.h, dA.data_ptr(), dB.data_ptr(), ldb, nrhs, dX.data_ptr(), ldx, 1,
                                   None, None)
            assert rc == H.HQR_ERR_INVALID
    finally:
        tall.close()


AUG_CASES = [  # M, N, NB, IB, precision, nrhs, kappa, residual noise, refinement steps
    (512, 256, 128, 32, "fp64", 3, 1e6, 1e-8, 2),
    (768, 384, 128, 32, "fast", 5, 1e3, 1e-2, 4),
    (1024, 512, 128, 32, "fast", 17, 1e4, 1e-3, 6),
    (512, 256, 128, 32, "split", 16, 1e6, 1e-2, 3),
    (640, 640, 128, 32, "fast", 2, 1e3, 1e-8, 4),
    (384, 128, 64, 16, "fp64", 1, 1e2, 1.0, 1),
]


@pytest.mark.parametrize("M,N,NB,IB,prec,nrhs,kappa,noise,steps", AUG_CASES)
def test_lstsq_aug_reaches_the_fp64_bound(env, M, N, NB, IB, prec, nrhs, kappa, noise, steps):
    H, torch = env
    A, _, b = ls_problem(M, N, nrhs, kappa, 500 + M + N + nrhs, noise=noise)
    p = {"fp64": H.HQR_PREC_FP64, "split": H.HQR_PREC_OZAKI, "fast": H.HQR_PREC_OZAKI_FAST}[prec]
    x, res = run_gpu(H, torch, A, b, NB, IB, p, steps, augmented=True)
    xn = np.linalg.lstsq(A, b, rcond=None)[0]
    t = ls_tol(A, xn, b, kappa)
    assert np.linalg.norm(x - xn) / np.linalg.norm(xn) <= t
    if prec == "fp64":
        xo = O.lstsq_aug(O.to_tiles(A, NB), b, M, N, NB, IB, steps)
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) <= t
    r = np.linalg.norm(b - A @ x, axis=0)
    rn = np.linalg.norm(b - A @ xn, axis=0)
    assert np.allclose(res, r, rtol=1e-10, atol=1e-14)
    assert np.all(r <= rn * (1 + 1e-10) + 1e-14)


def test_lstsq_aug_beats_the_plain_refinement_with_a_large_residual(env):
    """HQR_PREC_OZAKI_FAST, kappa 1e3, residual noise 1e-2: four steps of
    hqr_lstsq's refinement stall near kappa^2 u_fast ||r|| / ||x||; the
    augmented system's reach the FP64 bound."""
    H, torch = env
    M, N, NB, IB, nrhs, kappa = 768, 384, 128, 32, 4, 1e3
    A, _, b = ls_problem(M, N, nrhs, kappa, 77, noise=1e-2)
    xn = np.linalg.lstsq(A, b, rcond=None)[0]
    xs, _ = run_gpu(H, torch, A, b, NB, IB, H.HQR_PREC_OZAKI_FAST, 4)
    xa, _ = run_gpu(H, torch, A, b, NB, IB, H.HQR_PREC_OZAKI_FAST, 4, augmented=True)
    es = np.linalg.norm(xs - xn) / np.linalg.norm(xn)
    ea = np.linalg.norm(xa - xn) / np.linalg.norm(xn)
    assert ea <= ls_tol(A, xn, b, kappa)
    assert es > 10 * ea


def test_lstsq_aug_rejects_a_tree_and_bad_arguments(env):
    H, torch = env
    dA = torch.zeros(1024 * 256, dtype=torch.float64, device="cuda")
    dB = torch.zeros(1024 * 4, dtype=torch.float64, device="cuda")
    dX = torch.zeros(256 * 4, dtype=torch.float64, device="cuda")
    plan = H.Plan(1024, 256, 128, 32, H.HQR_PREC_FP64)
    try:
        for nrhs, ldb, ldx, steps in ((0, 1024, 256, 1), (4, 100, 256, 1), (4, 1024, 100, 1), (4, 1024, 256, -1)):
            rc = H.lib().hqr_lstsq_aug(plan.h, dA.data_ptr(), dB.data_ptr(), ldb, nrhs, dX.data_ptr(), ldx,
                                       steps, None, None)
            assert rc == H.HQR_ERR_INVALID
        H.check(H.lib().hqr_plan_set_tree(plan.h, 2), "set_tree")
        rc = H.lib().hqr_lstsq_aug(plan.h, dA.data_ptr(), dB.data_ptr(), 1024, 4, dX.data_ptr(), 256, 1,
                                   None, None)
        assert rc == H.HQR_ERR_UNSUPPORTED
    finally:
        plan.close()
