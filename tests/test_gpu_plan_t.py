"""use_plan_t of hqr_make_q / hqr_ormqr_t / hqr_ormqr_n: after hqr_geqrf on a
plan, Q^T C reuses the factorization's T factors (FP64) or prepared operands
(split precision) -- no panel task runs -- and so does Q generation in FP64.
Split Q generation and Q C apply H, not H^T: the first such call prepares the
plan's H operand set, later ones reuse it.  Results are the oracle's; once a
call has rebuilt a set from other reflectors, use_plan_t = 1 rebuilds that set
again instead of using stale operands (the other set stays valid).

Elementwise bar as in the other parity tests: n * eps * ||A||_F for Q, 4x that
of ||C||_F for Q^T C.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
GEQRT, TBUILD, OZPREP = 0, 4, 5


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hybrid3_gb300 as H
    H.lib().hqr_set_error_mode(H.HQR_ERRORS_RETURN)
    return torch, H


def tol(A2d):
    return max(A2d.shape) * EPS * np.linalg.norm(A2d)


@pytest.mark.parametrize("NB,IB,prec", [(128, 32, 1), (64, 16, 0), (128, 32, 0)])
def test_q_from_the_plans_factors(env, NB, IB, prec):
    torch, H = env
    L = H.lib()
    M = N = 768
    A2d = O.uniform_matrix(M, N, 31 + NB + prec)
    A = O.to_tiles(A2d, NB)
    plan = H.Plan(M, N, NB, IB, prec)
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    H.check(L.hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "geqrf")
    a, tau = dA.cpu().numpy(), dTAU.cpu().numpy()
    oq, _ = O.make_Q(a, tau, M, N, NB)
    C2d = O.uniform_matrix(M, N, 77)
    C = O.to_tiles(C2d, NB)
    oc = O.dormqr(a, tau, C, M, N, NB, N // NB)
    panel_slot = OZPREP if prec else TBUILD

    def make_q(use):
        dQ = torch.zeros(M * N, dtype=torch.float64, device="cuda")
        dR = dA.clone()
        H.check(L.hqr_make_q(plan.h, dQ.data_ptr(), dR.data_ptr(), dTAU.data_ptr(), use, None), "make_q")
        return dQ.cpu().numpy(), plan.stats()

    def ormqr(use):
        dC = torch.from_numpy(C.copy()).cuda()
        H.check(L.hqr_ormqr_t(plan.h, dA.data_ptr(), dTAU.data_ptr(), dC.data_ptr(), N // NB, use, None),
                "ormqr")
        return dC.cpu().numpy(), plan.stats()

    def ormqr_n(use):
        dC = torch.from_numpy(C.copy()).cuda()
        H.check(L.hqr_ormqr_n(plan.h, dA.data_ptr(), dTAU.data_ptr(), dC.data_ptr(), N // NB, use, None),
                "ormqr_n")
        return dC.cpu().numpy(), plan.stats()

    # Q C = (Q^T)^T C from the oracle's Q^T (tile layout, M = N)
    qt2d = O.from_tiles(oq, M, N, NB)
    oqc = O.to_tiles(qt2d.T @ C2d, NB)
    panels = (M // NB) * (M // NB + 1) // 2
    # reuse: no panel tasks for Q^T C; Q generation too in FP64
    c, st = ormqr(1)
    assert st["count"][panel_slot] == 0
    assert np.abs(c - oc).max() <= 4 * tol(C2d)
    q, st = make_q(1)
    assert st["count"][panel_slot] == (panels if prec else 0)
    assert np.abs(q - oq).max() <= tol(A2d)
    # the H set, once prepared, serves Q generation and Q C alike
    q, st = make_q(1)
    assert st["count"][panel_slot] == 0
    assert np.abs(q - oq).max() <= tol(A2d)
    c, st = ormqr_n(1)
    assert st["count"][panel_slot] == 0
    assert np.abs(c - oqc).max() <= 4 * tol(C2d)
    # a rebuild replaces the set it used; use_plan_t = 1 then rebuilds that set
    q, st = make_q(0)
    assert st["count"][panel_slot] == panels
    assert np.abs(q - oq).max() <= tol(A2d)
    c, st = ormqr_n(1)
    assert st["count"][panel_slot] == panels
    assert np.abs(c - oqc).max() <= 4 * tol(C2d)
    # split: the H^T set was untouched; FP64: one set, rebuilt just now
    c, st = ormqr(1)
    assert st["count"][panel_slot] == 0
    assert np.abs(c - oc).max() <= 4 * tol(C2d)
    c, st = ormqr(0)
    assert st["count"][panel_slot] == panels
    c, st = ormqr(1)
    assert st["count"][panel_slot] == panels
    assert np.abs(c - oc).max() <= 4 * tol(C2d)
    # a new factorization makes both sets reusable again (the H set after its
    # first preparation)
    dA.copy_(torch.from_numpy(A.copy()))
    H.check(L.hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "geqrf")
    c, st = ormqr(1)
    assert st["count"][panel_slot] == 0
    assert np.abs(c - oc).max() <= 4 * tol(C2d)
    c, st = ormqr_n(1)
    assert st["count"][panel_slot] == (panels if prec else 0)
    assert np.abs(c - oqc).max() <= 4 * tol(C2d)
    plan.close()
