"""hqr_geqrf_noalloc: the factorization for callers that cannot allocate
device memory (for instance while a CUDA graph is being captured, or when a
pool allocator owns all device memory).  It must give the same factorization
as the allocating entry point hqr_geqrf, call after call, while its scratch
is a fixed array shared by every call.

This file is collected last so that a failure here comes after every other
test has run; it also passes when run on its own in a fresh process (then its
first call performs the one-time scratch lookup).
"""
import ctypes

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


def factor_allocating(torch, H, A, M, N, NB, IB):
    plan = H.Plan(M, N, NB, IB)
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    H.check(H.lib().hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "hqr_geqrf")
    plan.close()
    return dA.cpu().numpy(), dTAU.cpu().numpy()


def factor_noalloc(torch, H, A, M, N, NB, IB):
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    H.check(H.lib().hqr_geqrf_noalloc(M, N, NB, IB, dA.data_ptr(), dTAU.data_ptr(), None),
            "hqr_geqrf_noalloc")
    return dA.cpu().numpy(), dTAU.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(env):
    torch, H = env
    # two calls in a row on different shapes: the second call reuses the
    # scratch the first one left behind
    for (M, N, NB, IB, seed) in [(1024, 1024, 256, 32, 11), (1536, 1024, 128, 32, 12)]:
        A2d = O.uniform_matrix(M, N, seed)
        A = O.to_tiles(A2d, NB)
        ref_a, ref_tau = factor_allocating(torch, H, A, M, N, NB, IB)
        a, tau = factor_noalloc(torch, H, A, M, N, NB, IB)
        tol = max(M, N) * EPS * np.linalg.norm(A2d)
        assert np.abs(a - ref_a).max() <= tol
        assert np.abs(tau - ref_tau).max() <= tol


def test_noalloc_rejects_shapes_beyond_its_scratch(env):
    torch, H = env
    dA = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = H.lib().hqr_geqrf_noalloc(8192, 8192, 256, 32, dA.data_ptr(), dA.data_ptr(), None)
    assert rc == H.HQR_ERR_UNSUPPORTED
