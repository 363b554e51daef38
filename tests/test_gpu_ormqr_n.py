"""hqr_ormqr_n: C <- Q C with the Q of a tile QR (the untransposed
application, H_0 H_1 ... H_(NT-1) C, backward over the panels), in FP64 and
split precision, square and tall, for one and several tile columns of C.

Oracle: Q^T from the oracle's dormqr applied to the identity, so Q C =
(Q^T)^T C; and Q^T (Q C) = C through the oracle's dormqr.  Bars as the other
application tests: 4 n eps ||C||_F elementwise.
"""
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


@pytest.mark.parametrize("M,N,NB,IB,CT,prec", [
    (512, 512, 64, 16, 8, 0),
    (768, 384, 128, 32, 2, 0),
    (768, 384, 128, 32, 1, 1),
    (1024, 1024, 128, 32, 8, 1),
    (1024, 512, 128, 32, 3, 1),
])
def test_q_times_c_matches_oracle(env, M, N, NB, IB, CT, prec):
    torch, H = env
    L = H.lib()
    A2d = O.uniform_matrix(M, N, 900 + M + N + CT + prec)
    A = O.to_tiles(A2d, NB)
    plan = H.Plan(M, N, NB, IB, prec)
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    H.check(L.hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "geqrf")
    a, tau = dA.cpu().numpy(), dTAU.cpu().numpy()
    C2d = O.uniform_matrix(M, CT * NB, 55 + CT)
    C = O.to_tiles(C2d, NB)
    qt = O.from_tiles(O.dormqr(a, tau, O.to_tiles(np.eye(M), NB), M, N, NB, M // NB), M, M, NB)
    want = qt.T @ C2d
    for use in (0, 1):
        dC = torch.from_numpy(C.copy()).cuda()
        H.check(L.hqr_ormqr_n(plan.h, dA.data_ptr(), dTAU.data_ptr(), dC.data_ptr(), CT, use, None),
                "ormqr_n")
        got = O.from_tiles(dC.cpu().numpy(), M, CT * NB, NB)
        bar = 4 * M * EPS * np.linalg.norm(C2d)
        assert np.abs(got - want).max() <= bar
        back = O.from_tiles(O.dormqr(a, tau, O.to_tiles(got, NB), M, N, NB, CT), M, CT * NB, NB)
        assert np.abs(back - C2d).max() <= 2 * bar
    plan.close()


def test_q_times_c_is_unsupported_with_a_tree(env):
    torch, H = env
    L = H.lib()
    M, N, NB, IB = 1024, 256, 128, 32
    plan = H.Plan(M, N, NB, IB)
    H.check(L.hqr_plan_set_tree(plan.h, 2), "set_tree")
    A = O.to_tiles(O.uniform_matrix(M, N, 5), NB)
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    H.check(L.hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "geqrf")
    dC = torch.zeros(M * NB, dtype=torch.float64, device="cuda")
    assert L.hqr_ormqr_n(plan.h, dA.data_ptr(), dTAU.data_ptr(), dC.data_ptr(), 1, 1, None) == \
        H.HQR_ERR_UNSUPPORTED
    plan.close()
