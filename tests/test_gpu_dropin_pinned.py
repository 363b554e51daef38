"""The drop-in entry points with page-locked host arrays (hqr_host_alloc):
their copies run as SM loads / stores through the arrays' device mappings,
and Hybrid_make_Q zeroes the reflectors of the caller's RY on the host while
the DAG runs.  The results must equal, bit for bit, those of the same calls
on pageable arrays (whose copies go through cudaMemcpyAsync), and the
oracle's within n * eps * ||A||_F.
"""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
DP = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def H():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hybrid3_gb300 as H
    H.lib().hqr_set_error_mode(H.HQR_ERRORS_RETURN)
    return H


class Pinned:
    def __init__(self, L):
        self.L, self.ptrs = L, []

    def array(self, values):
        p = ctypes.c_void_p()
        assert self.L.hqr_host_alloc(ctypes.byref(p), ctypes.c_size_t(values.size * 8)) == 0
        self.ptrs.append(p)
        a = np.ctypeslib.as_array(ctypes.cast(p, DP), shape=(values.size,))
        a[:] = values
        return a

    def free(self):
        for p in self.ptrs:
            self.L.hqr_host_free(p)


def run_calls(H, A, C, n, NB, IB, make):
    L = H.lib()
    st = H.status(n, n, NB)
    P = lambda a: a.ctypes.data_as(DP)
    a = make(A)
    tau = make(np.zeros((n // 2) * (n // 2)))
    L.Hybrid_tile_QR(ctypes.byref(st), P(a), P(tau), 0, 1, IB)
    H.check(L.hqr_last_error(), "Hybrid_tile_QR")
    q = make(np.zeros(n * n))
    r = make(a)
    L.Hybrid_make_Q(ctypes.byref(st), P(q), P(r), P(make(tau)), 0, 1, IB)
    H.check(L.hqr_last_error(), "Hybrid_make_Q")
    q2 = make(np.full(n * n, 5.0))
    L.Hybrid_dorgqr(ctypes.byref(st), P(q2), P(make(a)), P(make(tau)), 0, 1)
    H.check(L.hqr_last_error(), "Hybrid_dorgqr")
    c = make(C)
    L.Hybrid_dormqr(ctypes.byref(st), P(make(a)), P(make(tau)), P(c), 0, 1)
    H.check(L.hqr_last_error(), "Hybrid_dormqr")
    qr = make(np.zeros(n * n))
    L.Hybrid_dgemm(ctypes.byref(st), P(make(q)), P(make(r)), P(qr), 0, 1)
    H.check(L.hqr_last_error(), "Hybrid_dgemm")
    return [x.copy() for x in (a, tau, q, r, q2, c, qr)]


@pytest.mark.parametrize("M,n,NB,IB,prec", [(1024, 1024, 128, 32, 1), (768, 768, 256, 32, 0),
                                            (1024, 512, 128, 32, 0)])
def test_pinned_arrays_give_the_pageable_results(H, M, n, NB, IB, prec):
    L = H.lib()
    if M != n:
        # tall: factorization and Q^T C only (Hybrid_make_Q's driver is square)
        A2d = O.uniform_matrix(M, n, 700)
        A = O.to_tiles(A2d, NB)
        out = []
        pinned = Pinned(L)
        try:
            for make in (lambda v: np.array(v, dtype=np.float64, copy=True), pinned.array):
                st = H.status(M, n, NB)
                a = make(A)
                tau = make(np.zeros((M // 2) * (n // 2)))
                L.Hybrid_tile_QR(ctypes.byref(st), a.ctypes.data_as(DP), tau.ctypes.data_as(DP), 0, 1, IB)
                H.check(L.hqr_last_error(), "Hybrid_tile_QR")
                out.append((a.copy(), tau.copy()))
        finally:
            pinned.free()
        assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
        ra, _ = O.tile_qr(A, M, n, NB, IB)
        assert np.abs(out[0][0] - ra).max() <= max(M, n) * EPS * np.linalg.norm(A2d)
        return
    A2d = O.uniform_matrix(n, n, 600 + n)
    A = O.to_tiles(A2d, NB)
    C = O.to_tiles(O.uniform_matrix(n, n, 601), NB)
    L.hqr_set_default_precision(prec)
    pinned = Pinned(L)
    try:
        ref = run_calls(H, A, C, n, NB, IB, lambda v: np.array(v, dtype=np.float64, copy=True))
        got = run_calls(H, A, C, n, NB, IB, pinned.array)
    finally:
        L.hqr_set_default_precision(H.HQR_PREC_FP64)
        pinned.free()
    for x, y in zip(got, ref):
        assert np.array_equal(x, y)
    a, tau, q, r = ref[:4]
    ra, rtau = O.tile_qr(A, n, n, NB, IB)
    t = n * EPS * np.linalg.norm(A2d)
    assert np.abs(a - ra).max() <= t
    oq, orr = O.make_Q(ra, rtau, n, n, NB)
    assert np.abs(q - oq).max() <= t
    assert np.abs(r - orr).max() <= t
