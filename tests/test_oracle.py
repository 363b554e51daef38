"""Pin the CPU oracle (oracle/hqr_oracle.c) before trusting it.

* against the golden fixtures produced by the reference's own sources
  (tests/golden/make_golden.py);
* against scipy's LAPACK dgeqrt / dtpqrt / dgemqrt / dtpmqrt, which implement
  the same tile kernels as the PLASMA CORE routines the reference calls;
* on the edge cases the reference's path meets (trivial reflectors, tiny
  columns, tall matrices that the reference driver cannot finish).

Tolerance for floating-point agreement: |x - y| <= n * eps * ||A||_F
elementwise (n = matrix order), i.e. the c*n*eps*||A|| bound with c = 1.
"""
import glob
import os

import numpy as np
import pytest

import oracle as O

EPS = np.finfo(np.float64).eps


def tol(A2d):
    return max(A2d.shape) * EPS * np.linalg.norm(A2d)


def load(golden_dir, name):
    return dict(np.load(os.path.join(golden_dir, name)))


QR_FIXTURES = ["qr_uniform_n128_nb32_ib8.npz", "qr_matmake_n128_nb32_ib8.npz",
               "qr_uniform_n128_nb32_ib32.npz"]


@pytest.mark.parametrize("name", QR_FIXTURES)
def test_tile_qr_matches_reference(golden_dir, name):
    g = load(golden_dir, name)
    M, N, NB, IB = (int(g[k]) for k in ("M", "N", "NB", "IB"))
    a, tau = O.tile_qr(g["A"], M, N, NB, IB)
    t = tol(O.from_tiles(g["A"], M, N, NB))
    assert np.abs(a - g["A_qr"]).max() <= t
    assert np.abs(tau - g["TAU"]).max() <= t


def test_nb256_fixture_matches_oracle(golden_dir):
    """The reference at the CPU workload's tile order (NB = 256, IB = 32),
    n = 512: factorization, Q generation and Q^T C; the inputs are regenerated
    from their seeds."""
    g = load(golden_dir, "qr_uniform_n512_nb256_ib32.npz")
    M, N, NB, IB = (int(g[k]) for k in ("M", "N", "NB", "IB"))
    A2d = O.uniform_matrix(M, N, int(g["seed"]))
    A = O.to_tiles(A2d, NB)
    C = O.to_tiles(O.uniform_matrix(M, N, int(g["c_seed"])), NB)
    t = tol(A2d)
    a, tau = O.tile_qr(A, M, N, NB, IB)
    assert np.abs(a - g["A_qr"]).max() <= t
    assert np.abs(tau - g["TAU"]).max() <= t
    q, _ = O.make_Q(g["A_qr"], g["TAU"], M, N, NB)
    assert np.abs(q - g["Qt"]).max() <= t
    c = O.dormqr(g["A_qr"], g["TAU"], C, M, N, NB, N // NB)
    assert np.abs(c - g["QtC"]).max() <= 4 * tol(O.from_tiles(C, M, N, NB))


@pytest.mark.parametrize("name", QR_FIXTURES)
def test_q_generation_matches_reference(golden_dir, name):
    g = load(golden_dir, name)
    M, N, NB = (int(g[k]) for k in ("M", "N", "NB"))
    t = tol(O.from_tiles(g["A"], M, N, NB))
    q, r = O.make_Q(g["A_qr"], g["TAU"], M, N, NB)
    assert np.abs(q - g["Qt"]).max() <= t
    assert np.abs(r - g["R"]).max() == 0.0            # R is A_qr with V zeroed
    qo = O.dorgqr(g["A_qr"], g["TAU"], M, N, NB)
    assert np.abs(qo - g["Qt_dorgqr"]).max() <= t
    c = O.dormqr(g["A_qr"], g["TAU"], g["C"], M, N, NB, N // NB)
    assert np.abs(c - g["QtC"]).max() <= tol(O.from_tiles(g["C"], M, N, NB)) * 4


@pytest.mark.parametrize("name", QR_FIXTURES)
def test_dgemm_check_matches_reference(golden_dir, name):
    g = load(golden_dir, name)
    M, N, NB = (int(g[k]) for k in ("M", "N", "NB"))
    qq = O.dgemm_tn(g["Qt"], g["Qt"], M, N, NB)
    qr = O.dgemm_tn(g["Qt"], g["R"], M, N, NB)
    assert np.abs(qq - g["QQt"]).max() <= 1e-13
    assert np.abs(qr - g["QR"]).max() <= 1e-13
    # Q R reproduces A (main.c:241-258 check)
    assert np.abs(qr - g["A"]).max() <= tol(O.from_tiles(g["A"], M, N, NB))


def test_mat_make_is_the_reference_generator(golden_dir):
    g = load(golden_dir, "qr_matmake_n128_nb32_ib8.npz")
    A = O.mat_make(128, 128, 32, 20151130)
    assert np.array_equal(A, g["A"])


def test_tile_kernels_match_reference(golden_dir):
    g = load(golden_dir, "tile_kernels_nb32_ib8.npz")
    NB, IB = int(g["NB"]), int(g["IB"])
    L = O.lib()
    work = np.zeros(3 * NB * NB)
    A = np.asfortranarray(g["geqrt_A"].copy())
    TAU = np.zeros(NB)
    Y = np.zeros((NB, NB), order="F")
    T = np.zeros((NB, NB), order="F")
    L.orc_tk_dgeqrt(NB, NB, IB, O.ptr(A), NB, O.ptr(TAU), O.ptr(Y), O.ptr(T), NB, O.ptr(work))
    t = 64 * NB * EPS * np.linalg.norm(g["geqrt_A"])
    assert np.abs(A - g["geqrt_A_out"]).max() <= t
    assert np.abs(TAU[:-1] - g["geqrt_TAU"][:-1]).max() <= t   # last TAU is never written
    assert np.abs(Y - g["geqrt_Y"]).max() <= t
    assert np.abs(T - g["geqrt_T"]).max() <= t
    T2 = np.zeros((NB, NB), order="F")
    L.orc_tk_dlarft(NB, NB, 1, O.ptr(Y), NB, O.ptr(TAU), O.ptr(T2), NB, O.ptr(work))
    assert np.abs(np.tril(T2) - np.tril(g["larft_T"])).max() <= t
    C = np.asfortranarray(g["larfb_C"].copy())
    L.orc_tk_sub_dlarfb(NB, NB, NB, O.ptr(Y), NB, O.ptr(T2), NB, O.ptr(C), NB, O.ptr(work))
    assert np.abs(C - g["larfb_C_out"]).max() <= t
    R = np.asfortranarray(g["tsqrt_R"].copy())
    A2 = np.asfortranarray(g["tsqrt_A2"].copy())
    TAU = np.zeros(NB)
    T = np.zeros((NB, NB), order="F")
    L.orc_tk_dtsqrt(NB, NB, IB, O.ptr(R), NB, O.ptr(A2), NB, O.ptr(TAU), O.ptr(T), NB, O.ptr(work))
    assert np.abs(R - g["tsqrt_R_out"]).max() <= t
    assert np.abs(A2 - g["tsqrt_V"]).max() <= t
    assert np.abs(TAU - g["tsqrt_TAU"]).max() <= t
    T3 = np.zeros((NB, NB), order="F")
    L.orc_tk_dlarft(NB, NB, 1, O.ptr(A2), NB, O.ptr(TAU), O.ptr(T3), NB, O.ptr(work))
    assert np.abs(T3 - g["tsqrt_fullT"]).max() <= t
    A1 = np.asfortranarray(g["ssrfb_A1"].copy())
    B2 = np.asfortranarray(g["ssrfb_A2"].copy())
    L.orc_tk_sub_dssrfb(NB, NB, NB, NB, O.ptr(A2), NB, O.ptr(T3), NB, O.ptr(A1), NB, O.ptr(B2),
                        NB, O.ptr(work))
    assert np.abs(A1 - g["ssrfb_A1_out"]).max() <= t
    assert np.abs(B2 - g["ssrfb_A2_out"]).max() <= t


# --------------------------------------------------------------------------
# CORE kernels against LAPACK (scipy), which restates the same routines
# --------------------------------------------------------------------------

def _scipy_lapack():
    return pytest.importorskip("scipy.linalg.lapack")


@pytest.mark.parametrize("nb,ib", [(32, 8), (64, 16), (48, 48)])
def test_core_dgeqrt_matches_lapack(nb, ib):
    lp = _scipy_lapack()
    rng = np.random.default_rng(nb + ib)
    A = np.asfortranarray(rng.uniform(-1, 1, (nb, nb)))
    a_l, t_l, info = lp.dgeqrt(ib, A.copy())
    assert info == 0
    a = A.copy(order="F")
    T = np.zeros((nb, nb), order="F")
    tau = np.zeros(nb)
    assert O.lib().orc_core_dgeqrt(nb, nb, ib, O.ptr(a), nb, O.ptr(T), nb, O.ptr(tau)) == 0
    t = tol(A)
    assert np.abs(a - a_l).max() <= t
    assert np.abs(T[:ib] - t_l).max() <= t
    for j in range(nb):
        assert tau[j] == T[j % ib, j]


@pytest.mark.parametrize("nb,ib", [(32, 8), (64, 16)])
def test_core_dtsqrt_and_dtsmqr_match_lapack(nb, ib):
    lp = _scipy_lapack()
    rng = np.random.default_rng(3 * nb + ib)
    R = np.asfortranarray(np.triu(rng.uniform(-1, 1, (nb, nb))))
    B = np.asfortranarray(rng.uniform(-1, 1, (nb, nb)))
    r_l, v_l, t_l, info = lp.dtpqrt(0, ib, R.copy(), B.copy())
    assert info == 0
    r, v = R.copy(order="F"), B.copy(order="F")
    T = np.zeros((nb, nb), order="F")
    tau = np.zeros(nb)
    O.lib().orc_core_dtsqrt(nb, nb, ib, O.ptr(r), nb, O.ptr(v), nb, O.ptr(T), nb, O.ptr(tau))
    t = tol(np.vstack([R, B]))
    assert np.abs(r - r_l).max() <= t
    assert np.abs(v - v_l).max() <= t
    assert np.abs(T[:ib] - t_l).max() <= t
    # apply the transpose of that reflector to a random pair (dtpmqrt, l = 0)
    A1 = np.asfortranarray(rng.uniform(-1, 1, (nb, nb)))
    A2 = np.asfortranarray(rng.uniform(-1, 1, (nb, nb)))
    a1_l, a2_l, info = lp.dtpmqrt(0, v_l, t_l, A1.copy(), A2.copy(), trans="T")
    assert info == 0
    a1, a2 = A1.copy(order="F"), A2.copy(order="F")
    O.lib().orc_core_dtsmqr(nb, nb, nb, nb, nb, ib, O.ptr(a1), nb, O.ptr(a2), nb, O.ptr(v), nb,
                            O.ptr(T), nb)
    assert np.abs(a1 - a1_l).max() <= t
    assert np.abs(a2 - a2_l).max() <= t


@pytest.mark.parametrize("nb,ib", [(32, 8), (64, 32)])
def test_core_dormqr_matches_lapack(nb, ib):
    lp = _scipy_lapack()
    rng = np.random.default_rng(7 * nb + ib)
    A = np.asfortranarray(rng.uniform(-1, 1, (nb, nb)))
    a_l, t_l, _ = lp.dgeqrt(ib, A.copy())
    C = np.asfortranarray(rng.uniform(-1, 1, (nb, nb)))
    c_l, info = lp.dgemqrt(a_l, t_l, C.copy(), side="L", trans="T")
    assert info == 0
    T = np.zeros((nb, nb), order="F")
    T[:ib] = t_l
    c = C.copy(order="F")
    O.lib().orc_core_dormqr(nb, nb, nb, ib, O.ptr(np.asfortranarray(a_l)), nb, O.ptr(T), nb,
                            O.ptr(c), nb)
    assert np.abs(c - c_l).max() <= tol(C)


def test_dlarfg_edge_cases():
    L = O.lib()
    import ctypes
    # zero tail -> trivial reflector (tau = 0, alpha unchanged)
    alpha = ctypes.c_double(3.0)
    x = np.zeros(5)
    tau = ctypes.c_double(-1.0)
    L.orc_dlarfg(6, ctypes.byref(alpha), O.ptr(x), 1, ctypes.byref(tau))
    assert tau.value == 0.0 and alpha.value == 3.0
    # beta = -sign(alpha) * norm
    alpha = ctypes.c_double(3.0)
    x = np.array([4.0])
    L.orc_dlarfg(2, ctypes.byref(alpha), O.ptr(x), 1, ctypes.byref(tau))
    assert alpha.value == pytest.approx(-5.0) and tau.value == pytest.approx(1.6)
    alpha = ctypes.c_double(-3.0)
    x = np.array([4.0])
    L.orc_dlarfg(2, ctypes.byref(alpha), O.ptr(x), 1, ctypes.byref(tau))
    assert alpha.value == pytest.approx(5.0)
    # tiny column: the safe-minimum rescaling keeps H orthogonal
    alpha = ctypes.c_double(1e-300)
    x = np.array([1e-300, 2e-300])
    x0 = np.concatenate([[alpha.value], x])
    L.orc_dlarfg(3, ctypes.byref(alpha), O.ptr(x), 1, ctypes.byref(tau))
    v = np.concatenate([[1.0], x])
    H = np.eye(3) - tau.value * np.outer(v, v)
    y = H @ x0
    assert abs(y[0] - alpha.value) <= 1e-14 * abs(alpha.value)
    assert np.abs(y[1:]).max() <= 1e-14 * abs(alpha.value)


def _flat_tree_scipy(A2d, NB, IB):
    """Independent flat-tree tile QR through scipy's LAPACK (dgeqrt/dtpqrt/
    dgemqrt/dtpmqrt), the kernels PLASMA's CORE routines are made of."""
    lp = _scipy_lapack()
    M, N = A2d.shape
    MT, NT = M // NB, N // NB
    A = [[np.asfortranarray(A2d[i*NB:(i+1)*NB, j*NB:(j+1)*NB]) for j in range(NT)] for i in range(MT)]
    for i in range(min(MT, NT)):
        A[i][i], t, _ = lp.dgeqrt(IB, A[i][i])
        for j in range(i + 1, NT):
            A[i][j], _ = lp.dgemqrt(A[i][i], t, A[i][j], side="L", trans="T")
        for k in range(i + 1, MT):
            r, v, t, _ = lp.dtpqrt(0, IB, A[i][i], A[k][i])
            A[i][i], A[k][i] = r, v
            for j in range(i + 1, NT):
                A[i][j], A[k][j], _ = lp.dtpmqrt(0, v, t, A[i][j], A[k][j], trans="T")
    return np.block(A)


@pytest.mark.parametrize("M,N,NB,IB", [(192, 64, 32, 8), (256, 128, 64, 16), (96, 96, 32, 32),
                                       (288, 192, 96, 32), (192, 96, 96, 16), (384, 192, 192, 32)])
def test_tall_and_square_flat_tree_against_lapack(M, N, NB, IB):
    A = O.uniform_matrix(M, N, 11)
    ref = _flat_tree_scipy(A, NB, IB)
    a, tau = O.tile_qr(O.to_tiles(A, NB), M, N, NB, IB)
    got = O.from_tiles(a, M, N, NB)
    assert np.abs(got - ref).max() <= tol(A)


def test_tall_qr_reconstructs():
    M, N, NB, IB = 256, 96, 32, 8
    A = O.uniform_matrix(M, N, 5)
    a, tau = O.tile_qr(O.to_tiles(A, NB), M, N, NB, IB)
    R = np.triu(O.from_tiles(a, M, N, NB)[:N])
    # |R| agrees with numpy's R up to row signs
    Rn = np.linalg.qr(A, mode="r")
    assert np.allclose(np.abs(R), np.abs(Rn), atol=tol(A))


def test_golden_files_present(golden_dir):
    names = {os.path.basename(p) for p in glob.glob(os.path.join(golden_dir, "*.npz"))}
    for n in QR_FIXTURES + ["tile_kernels_nb32_ib8.npz"]:
        assert n in names
