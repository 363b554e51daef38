"""Domain-tree factorization (hqr_plan_set_tree) on the GPU through the C ABI.

With a tree the reflectors differ from the reference's flat tree, R does not
(up to the signs of its rows): |R_tree| is compared elementwise with |R| of the
oracle's flat tile QR within 10 n eps ||A||.  The Q^T application with the
plan's merges must give Q^T A = [R; 0] (same bar), and least squares must agree
with numpy's."""
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


CASES = [  # M, N, NB, IB, precision, domain tiles
    (1024, 256, 128, 32, "fp64", 2),
    (1024, 256, 128, 32, "split", 2),
    (1024, 256, 128, 32, "fp64", 1),
    (1280, 384, 128, 32, "split", 3),
    (768, 384, 64, 16, "fp64", 3),
    (512, 512, 128, 32, "split", 3),
    (2048, 256, 128, 32, "split", 5),
]


@pytest.mark.parametrize("M,N,NB,IB,prec,S", CASES)
def test_tree_qr_r_and_qt(env, M, N, NB, IB, prec, S):
    H, torch = env
    A2d = O.uniform_matrix(M, N, 77 + M + N + S)
    A = O.to_tiles(A2d, NB)
    p = H.HQR_PREC_OZAKI if prec == "split" else H.HQR_PREC_FP64
    plan = H.Plan(M, N, NB, IB, p)
    plan.set_tree(S)
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    L = H.lib()
    try:
        H.check(L.hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "hqr_geqrf")
        st = plan.stats()   # of the factorization
        # Q^T A through the plan's reflectors (flat part + merges)
        dC = torch.from_numpy(A.copy()).cuda()
        H.check(L.hqr_ormqr_t(plan.h, dA.data_ptr(), dTAU.data_ptr(), dC.data_ptr(), N // NB, 1, None),
                "hqr_ormqr_t")
        # without the plan's T factors the merges cannot be rebuilt
        assert L.hqr_ormqr_t(plan.h, dA.data_ptr(), dTAU.data_ptr(), dC.data_ptr(), N // NB, 0,
                             None) == H.HQR_ERR_UNSUPPORTED
    finally:
        plan.close()
    ra, _ = O.tile_qr(A, M, N, NB, IB)
    t = 10 * max(M, N) * EPS * np.linalg.norm(A2d)
    R = np.triu(O.from_tiles(dA.cpu().numpy(), M, N, NB)[:N])
    Ro = np.triu(O.from_tiles(ra, M, N, NB)[:N])
    assert np.abs(np.abs(R) - np.abs(Ro)).max() <= t
    QtA = O.from_tiles(dC.cpu().numpy(), M, N, NB)
    assert np.abs(QtA[:N] - R).max() <= t
    if M > N:
        assert np.abs(QtA[N:]).max() <= t
    # panel blocks: every panel tile and every merge, per inner block
    w = 16 if prec == "split" else min(IB, 32)
    nblk = NB // w
    MT, NT = M // NB, N // NB
    tiles = sum(MT - i for i in range(min(MT, NT)))
    merges = sum(-(-(MT - i) // S) - 1 for i in range(min(MT, NT))) if S < MT else 0
    geqrts = sum(-(-(MT - i) // S) for i in range(min(MT, NT)))
    assert st["count"][0] == geqrts * nblk
    assert st["count"][1] == (tiles - geqrts + merges) * nblk


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_tree_lstsq(env, prec):
    H, torch = env
    M, N, NB, IB, nrhs, kappa = 1024, 256, 128, 32, 6, 1e6
    A, _, b = ls_problem(M, N, nrhs, kappa, 31)
    p = H.HQR_PREC_OZAKI if prec == "split" else H.HQR_PREC_FP64
    dA = torch.from_numpy(O.to_tiles(A, NB)).cuda()
    dB = torch.from_numpy(np.asfortranarray(b).reshape(-1, order="F").copy()).cuda()
    dX = torch.zeros(N * nrhs, dtype=torch.float64, device="cuda")
    plan = H.Plan(M, N, NB, IB, p)
    plan.set_tree(2)
    try:
        plan.lstsq(dA.data_ptr(), dB.data_ptr(), nrhs, dX.data_ptr(), refine_steps=1)
    finally:
        plan.close()
    x = dX.cpu().numpy().reshape(N, nrhs, order="F")
    xn = np.linalg.lstsq(A, b, rcond=None)[0]
    assert np.linalg.norm(x - xn) / np.linalg.norm(xn) <= ls_tol(A, xn, b, kappa)


def test_tree_make_q(env):
    """Q^T from the forward application on a square plan with a tree:
    ||Q^T Q - I|| and ||Q R - A|| at FP64 level."""
    H, torch = env
    n, NB, IB = 512, 128, 32
    A2d = O.uniform_matrix(n, n, 4711)
    A = O.to_tiles(A2d, NB)
    plan = H.Plan(n, n, NB, IB, H.HQR_PREC_OZAKI)
    plan.set_tree(2)
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((n // NB) ** 2 * NB, dtype=torch.float64, device="cuda")
    dQ = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    L = H.lib()
    try:
        H.check(L.hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "hqr_geqrf")
        H.check(L.hqr_make_q(plan.h, dQ.data_ptr(), dA.data_ptr(), dTAU.data_ptr(), 1, None), "hqr_make_q")
        assert L.hqr_make_q(plan.h, dQ.data_ptr(), dA.data_ptr(), dTAU.data_ptr(), 0,
                            None) == H.HQR_ERR_UNSUPPORTED
    finally:
        plan.close()
    Qt = O.from_tiles(dQ.cpu().numpy(), n, n, NB)
    R = O.from_tiles(dA.cpu().numpy(), n, n, NB)
    assert np.allclose(R, np.triu(R))            # the reflectors were zeroed
    assert np.linalg.norm(Qt @ Qt.T - np.eye(n)) <= 100 * n * EPS
    assert np.linalg.norm(Qt.T @ R - A2d) <= 100 * n * EPS * np.linalg.norm(A2d)
