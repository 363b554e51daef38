"""GPU parity of the split-precision path (Ozaki slices on tcgen05, FP64 panels)
against the CPU oracle.

Elementwise bar, as for the FP64 path: |gpu - oracle| <= n * eps * ||A||_F for
R, V, TAU, Q^T C and Q.  Residual and orthogonality of the generated Q are
compared with the reference's own FP64 make_Q on the same factorization (the
oracle's restatement, full-width T as in Hybrid_make_Q.c:124-130): at most 4x
its ||A - QR||_F / ||A||_F and ||I - Q Q^T||_F.  The emulated products are
individually more accurate than FP64 matrix products (see
test_split_product_is_as_accurate_as_fp64); the emulation applies each panel
tile's reflector with its full NB x NB T, like the reference's make_Q.
"""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
DP = ctypes.POINTER(ctypes.c_double)


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


def factor(torch, H, A, M, N, NB, IB, prec):
    plan = H.Plan(M, N, NB, IB, prec)
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device="cuda")
    H.check(H.lib().hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "hqr_geqrf")
    return plan, dA, dTAU


SHAPES = [(256, 256, 128, 32), (512, 512, 128, 32), (512, 256, 128, 32), (768, 512, 128, 64),
          (384, 640, 128, 16), (1024, 1024, 128, 32)]


@pytest.mark.parametrize("M,N,NB,IB", SHAPES)
def test_split_factorization_matches_oracle(env, M, N, NB, IB):
    torch, H = env
    A2d = O.uniform_matrix(M, N, 500 + M + N + NB)
    A = O.to_tiles(A2d, NB)
    plan, dA, dTAU = factor(torch, H, A, M, N, NB, IB, H.HQR_PREC_OZAKI)
    ra, rtau = O.tile_qr(A, M, N, NB, IB)
    t = tol(A2d)
    assert np.abs(dA.cpu().numpy() - ra).max() <= t
    assert np.abs(dTAU.cpu().numpy() - rtau).max() <= t
    st = plan.stats()
    MT, NT = M // NB, N // NB
    steps = min(MT, NT)
    panels = sum(MT - i for i in range(steps))
    assert st["count"][5] == panels            # one preparation per panel tile
    # panel tasks run per inner block: the split path's panels use w = 16
    nblk = NB // 16
    assert st["count"][0] == steps * nblk
    assert st["count"][1] == (panels - steps) * nblk
    plan.close()


@pytest.mark.parametrize("M,N,NB,IB", [(512, 512, 128, 32), (1024, 1024, 128, 64), (768, 512, 128, 32)])
def test_split_make_q_and_ormqr(env, M, N, NB, IB):
    torch, H = env
    A2d = O.uniform_matrix(M, N, 900 + M)
    A = O.to_tiles(A2d, NB)
    plan, dA, dTAU = factor(torch, H, A, M, N, NB, IB, H.HQR_PREC_OZAKI)
    a, tau = dA.cpu().numpy(), dTAU.cpu().numpy()
    # Q^T C on a second matrix, against the oracle's dormqr
    C = O.to_tiles(O.uniform_matrix(M, N, 77), NB)
    dC = torch.from_numpy(C.copy()).cuda()
    H.check(H.lib().hqr_ormqr_t(plan.h, dA.data_ptr(), dTAU.data_ptr(), dC.data_ptr(), N // NB, 0,
                                None), "ormqr")
    oc = O.dormqr(a, tau, C, M, N, NB, N // NB)
    assert np.abs(dC.cpu().numpy() - oc).max() <= 4 * tol(O.from_tiles(C, M, N, NB))
    # make_q (Q^T, reflectors removed)
    dQ = torch.zeros(M * N, dtype=torch.float64, device="cuda")
    dR = dA.clone()
    H.check(H.lib().hqr_make_q(plan.h, dQ.data_ptr(), dR.data_ptr(), dTAU.data_ptr(), 0, None), "make_q")
    oq, orr = O.make_Q(a, tau, M, N, NB)
    assert np.abs(dQ.cpu().numpy() - oq).max() <= tol(A2d)
    assert np.array_equal(dR.cpu().numpy(), orr)
    if M == N:
        ref_res, ref_orth = quality(A2d, oq, orr, M, N, NB)
        res, orth = quality(A2d, dQ.cpu().numpy(), dR.cpu().numpy(), M, N, NB)
        assert res <= 4 * max(ref_res, 1e-15)
        assert orth <= 4 * ref_orth
    plan.close()


def quality(A2d, q_tiles, r_tiles, M, N, NB):
    Qt = O.from_tiles(q_tiles, M, N, NB)
    R = O.from_tiles(r_tiles, M, N, NB)
    return (np.linalg.norm(A2d - Qt.T @ R) / np.linalg.norm(A2d),
            np.linalg.norm(Qt @ Qt.T - np.eye(M)))


def test_split_product_is_as_accurate_as_fp64(env):
    """The product engine alone (hqr_ozaki_product): exact on integers, and no
    worse than an FP64 matrix product against a quad-precision reference."""
    torch, H = env
    NB = 128
    rng = np.random.default_rng(NB)

    def run(X, Y):
        dX = torch.from_numpy(np.asfortranarray(X).ravel(order="F").copy()).cuda()
        dY = torch.from_numpy(np.asfortranarray(Y).ravel(order="F").copy()).cuda()
        dC = torch.zeros(NB * 64, dtype=torch.float64, device="cuda")
        H.check(H.lib().hqr_ozaki_product(NB, dX.data_ptr(), dY.data_ptr(), dC.data_ptr(), None))
        return dC.cpu().numpy().reshape(64, NB).T

    Xi = rng.integers(-1000, 1000, (NB, NB)).astype(float)
    Yi = rng.integers(-1000, 1000, (NB, 64)).astype(float)
    assert np.array_equal(run(Xi, Yi), Xi @ Yi)
    X = rng.uniform(-1, 1, (NB, NB))
    Y = rng.uniform(-1, 1, (NB, 64)) * 10.0 ** rng.integers(-6, 1, (NB, 64))
    ref = X.astype(np.longdouble) @ Y.astype(np.longdouble)
    if np.finfo(np.longdouble).eps > 1e-30:
        pytest.skip("long double is not quad precision on this host")
    e_oz = np.abs((run(X, Y) - ref).astype(float))
    e_64 = np.abs((X @ Y - ref).astype(float))
    assert e_oz.max() <= e_64.max()
    assert e_oz.mean() <= e_64.mean()


def test_split_through_drop_in_entry_points(env):
    torch, H = env
    L = H.lib()
    M = N = 512
    NB, IB = 128, 32
    A2d = O.uniform_matrix(M, N, 4)
    A = O.to_tiles(A2d, NB)
    st = H.status(M, N, NB)
    a = A.copy()
    tau = np.zeros((M // 2) * (N // 2))
    L.hqr_set_default_precision(H.HQR_PREC_OZAKI)
    try:
        L.Hybrid_tile_QR(ctypes.byref(st), a.ctypes.data_as(DP), tau.ctypes.data_as(DP), 0, 1, IB)
        H.check(L.hqr_last_error(), "Hybrid_tile_QR")
        q = np.zeros(M * N)
        L.Hybrid_make_Q(ctypes.byref(st), q.ctypes.data_as(DP), a.ctypes.data_as(DP),
                        tau.ctypes.data_as(DP), 0, 1, IB)
        H.check(L.hqr_last_error(), "Hybrid_make_Q")
    finally:
        L.hqr_set_default_precision(H.HQR_PREC_FP64)
    ra, rtau = O.tile_qr(A, M, N, NB, IB)
    oq, orr = O.make_Q(ra, rtau, M, N, NB)
    ref_res, ref_orth = quality(A2d, oq, orr, M, N, NB)
    res, orth = quality(A2d, q, a, M, N, NB)
    assert res <= 4 * max(ref_res, 1e-15)
    assert orth <= 4 * ref_orth


@pytest.mark.parametrize("NB", [64, 256])
def test_split_rejects_unsupported_tile_order(env, NB):
    torch, H = env
    h = ctypes.c_void_p()
    assert H.lib().hqr_plan_create(ctypes.byref(h), 4 * NB, 4 * NB, NB, 16, H.HQR_PREC_OZAKI) == \
        H.HQR_ERR_UNSUPPORTED
    assert H.lib().hqr_ozaki_product(NB, 1, 1, 1, None) == H.HQR_ERR_UNSUPPORTED


def graded(n, kappa, seed):
    """A = U diag(sigma) V^T, U and V Haar (QR of Gaussians, columns signed by
    diag(R), Mezzadri 2007), sigma_i = kappa^(-i/(n-1))."""
    rng = np.random.default_rng(seed)

    def haar():
        Q, R = np.linalg.qr(rng.standard_normal((n, n)))
        return Q * np.sign(np.diag(R))

    s = kappa ** (-np.arange(n) / (n - 1))
    return (haar() * s) @ haar().T


@pytest.mark.parametrize("kappa", [1e2, 1e8, 1e12])
def test_split_on_graded_condition_numbers(env, kappa):
    """Householder QR is backward stable whatever the conditioning: the split
    path's residual and orthogonality stay within 4x of the FP64 path's on the
    same matrix, and R matches the oracle elementwise (absolute errors of R are
    eps ||A||; V and TAU of the late, tiny trailing blocks are ill-determined
    for large kappa, for any two FP64 implementations alike)."""
    torch, H = env
    n, NB, IB = 512, 128, 32
    A2d = graded(n, kappa, int(np.log10(kappa)))
    A = O.to_tiles(A2d, NB)
    out = {}
    for prec in (H.HQR_PREC_OZAKI, H.HQR_PREC_FP64):
        plan, dA, dTAU = factor(torch, H, A, n, n, NB, IB, prec)
        dQ = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        a = dA.cpu().numpy()
        H.check(H.lib().hqr_make_q(plan.h, dQ.data_ptr(), dA.data_ptr(), dTAU.data_ptr(), 0, None), "make_q")
        out[prec] = (a, dTAU.cpu().numpy(), quality(A2d, dQ.cpu().numpy(), dA.cpu().numpy(), n, n, NB))
        plan.close()
    ra, rtau = O.tile_qr(A, n, n, NB, IB)
    a, tau, (res, orth) = out[H.HQR_PREC_OZAKI]
    R = np.triu(O.from_tiles(a, n, n, NB))
    assert np.abs(R - np.triu(O.from_tiles(ra, n, n, NB))).max() <= tol(A2d)
    res64, orth64 = out[H.HQR_PREC_FP64][2]
    assert res <= 4 * max(res64, 1e-16)
    assert orth <= 4 * orth64
