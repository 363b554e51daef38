"""hqr_geqrf_noalloc: the factorization for callers that cannot allocate
device memory -- a process whose device memory is owned entirely by its own
pool allocator, or a latency path that cannot take the device-wide
synchronisation an allocation may cause.  Its scratch is one fixed array that
every call shares and that keeps the previous call's contents, so each call
must give the factorization of the allocating entry point hqr_geqrf (bit for
bit: the same tasks run in the same dependency order) and the oracle's (within
n * eps * ||A||_F), whatever the previous call left behind.

The shapes below are chosen so that a call's dependency counters and ready
queues land on memory the previous call left non-zero: the first call's
tables end about 35 MiB into the array (T factors 32 MiB, then three tables of
about 1 MiB), and the second call's T factors are 34 MiB, so its counters sit
on the first call's ready queues (stale task ids).  The third call repeats the
first shape over the second call's T factors and tables.

This file is collected last so that a failure here comes after every other
test has run; it also passes when run on its own in a fresh process (then its
first call performs the one-time scratch lookup).
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
    for (M, N, NB, IB, seed) in [(2048, 2048, 32, 8, 11), (2048, 2176, 128, 32, 12),
                                 (2048, 2048, 32, 8, 13)]:
        A2d = O.uniform_matrix(M, N, seed)
        A = O.to_tiles(A2d, NB)
        a, tau = factor_noalloc(torch, H, A, M, N, NB, IB)
        ref_a, ref_tau = factor_allocating(torch, H, A, M, N, NB, IB)
        assert np.array_equal(a, ref_a)
        assert np.array_equal(tau, ref_tau)
        ora, ortau = O.tile_qr(A, M, N, NB, IB)
        tol = max(M, N) * EPS * np.linalg.norm(A2d)
        assert np.abs(a - ora).max() <= tol
        assert np.abs(tau - ortau).max() <= tol


def test_noalloc_rejects_shapes_beyond_its_scratch(env):
    torch, H = env
    dA = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = H.lib().hqr_geqrf_noalloc(8192, 8192, 256, 32, dA.data_ptr(), dA.data_ptr(), None)
    assert rc == H.HQR_ERR_UNSUPPORTED
