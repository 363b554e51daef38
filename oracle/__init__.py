"""CPU oracle for the tiled Householder QR path -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker.  The shipped library
never links, calls or executes anything in it.

Two CPU implementations live here:

* ``libhqr_oracle.so`` -- ``hqr_oracle.c``, a plain-C restatement of the
  reference's algorithm (the PLASMA CORE tile kernels it calls, its drivers and
  its own ``tile_kernel.c`` kernels).  Always built.
* ``_ref/libhybrid3_ref.so`` -- the reference's own C sources compiled unmodified
  against the single-rank shim headers in ``shim/`` and scipy's bundled OpenBLAS.
  Built only where the reference tree is present; it is what the restatement is
  pinned against (see ``tests/golden/make_golden.py``).

Arrays use the reference's tile layout: tile (i, j) of an MT x NT grid of
NB x NB tiles starts at element (i + j*MT)*NB*NB and is column-major inside.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhqr_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libhybrid3_ref.so")
REF_BIN_PATH = os.path.join(HERE, "_ref", "Hybrid3")

_dp = ctypes.POINTER(ctypes.c_double)
_lib = None


def build(ref_dir: str | None = None, quiet: bool = True) -> None:
    """Compile the restatement, and the reference build when ``ref_dir`` (else
    the environment variable HYBRID3_REF_DIR) names the reference's source
    tree."""
    ref_dir = ref_dir or os.environ.get("HYBRID3_REF_DIR", "")
    args = ["make", "-C", HERE, f"REF_DIR={ref_dir}"]
    out = subprocess.run(args, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        i, l, d, u = ctypes.c_int, ctypes.c_long, ctypes.c_double, ctypes.c_uint
        sig = {
            "orc_set_threads": (None, [i]),
            "orc_dlarfg": (None, [i, _dp, _dp, i, _dp]),
            "orc_core_dgeqrt": (i, [i, i, i, _dp, i, _dp, i, _dp]),
            "orc_core_dtsqrt": (i, [i, i, i, _dp, i, _dp, i, _dp, i, _dp]),
            "orc_core_dormqr": (i, [i, i, i, i, _dp, i, _dp, i, _dp, i]),
            "orc_core_dtsmqr": (i, [i, i, i, i, i, i, _dp, i, _dp, i, _dp, i, _dp, i]),
            "orc_dtsrft": (None, [i, i, i, _dp, i, _dp, _dp, i]),
            "orc_dlarft": (None, [i, i, _dp, i, _dp, _dp, i]),
            "orc_tile_qr": (i, [l, l, i, i, _dp, _dp, _dp]),
            "orc_make_Q": (None, [l, l, i, _dp, _dp, _dp]),
            "orc_make_I": (None, [l, l, i, _dp]),
            "orc_dgemm_tn": (None, [l, l, i, _dp, _dp, _dp]),
            "orc_mat_fill": (None, [l, l, i, _dp, u, i]),
            "orc_mat_comp3": (d, [l, l, _dp]),
            "orc_tile_to_colmajor": (None, [l, l, i, _dp, _dp]),
            "orc_tk_sub_dgeqr2": (None, [i, i, _dp, i, _dp, _dp, _dp]),
            "orc_tk_sub_dlarft": (None, [i, i, _dp, i, _dp, _dp, i, _dp]),
            "orc_tk_sub_dlarfb": (None, [i, i, i, _dp, i, _dp, i, _dp, i, _dp]),
            "orc_tk_sub_dssrfb": (None, [i, i, i, i, _dp, i, _dp, i, _dp, i, _dp, i, _dp]),
            "orc_tk_sub_dtsqr2": (None, [i, i, _dp, i, _dp, i, _dp, _dp]),
            "orc_tk_dgeqrt": (None, [i, i, i, _dp, i, _dp, _dp, _dp, i, _dp]),
            "orc_tk_dtsqrt": (None, [i, i, i, _dp, i, _dp, i, _dp, _dp, i, _dp]),
            "orc_tk_dlarft": (None, [i, i, i, _dp, i, _dp, _dp, i, _dp]),
            "orc_dorgqr": (None, [l, l, i, _dp, _dp, _dp]),
            "orc_dormqr": (None, [l, l, i, _dp, _dp, _dp, i]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib.orc_set_threads(os.cpu_count() or 1)
    return _lib


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and (a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"])
    return a.ctypes.data_as(_dp)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


# --------------------------------------------------------------------------
# Layout helpers (numpy, no compute beyond copies)
# --------------------------------------------------------------------------

def to_tiles(A: np.ndarray, NB: int) -> np.ndarray:
    """Column-major/2-D matrix -> flat tile-layout array."""
    M, N = A.shape
    MT, NT = M // NB, N // NB
    t = A[: MT * NB, : NT * NB].reshape(MT, NB, NT, NB)      # (ti, r, tj, c)
    t = t.transpose(2, 0, 3, 1)                               # (tj, ti, c, r)
    return np.ascontiguousarray(t).reshape(-1)


def from_tiles(T: np.ndarray, M: int, N: int, NB: int) -> np.ndarray:
    """Flat tile-layout array -> 2-D matrix."""
    MT, NT = M // NB, N // NB
    t = T.reshape(NT, MT, NB, NB).transpose(1, 3, 0, 2)      # (ti, r, tj, c)
    return np.ascontiguousarray(t).reshape(MT * NB, NT * NB)


def tau_grid(TAU: np.ndarray, M: int, N: int, NB: int) -> np.ndarray:
    """TAU array (NB per tile, tile order) -> (MT, NT, NB)."""
    MT, NT = M // NB, N // NB
    return TAU[: MT * NT * NB].reshape(NT, MT, NB).transpose(1, 0, 2)


def uniform_matrix(M: int, N: int, seed: int) -> np.ndarray:
    """Entries i.i.d. uniform[-1, 1) from a counter-based generator:
    splitmix64 of (seed, column-major index) -> top 53 bits -> [0,1) -> 2u-1.
    The CUDA library's generator produces the same values."""
    idx = np.arange(M * N, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = idx + np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return (2.0 * u - 1.0).reshape(N, M).T.copy()


# --------------------------------------------------------------------------
# The restatement (hqr_oracle.c)
# --------------------------------------------------------------------------

def tile_qr(A_tiles: np.ndarray, M: int, N: int, NB: int, IB: int, want_T: bool = False):
    """Hybrid_tile_QR restated: returns (A_out, TAU[, T]) in tile layout."""
    A = np.array(A_tiles, dtype=np.float64, copy=True)
    TAU = np.zeros((M // NB) * (N // NB) * NB)
    T = np.zeros_like(A) if want_T else None
    lib().orc_tile_qr(M, N, NB, IB, ptr(A), ptr(TAU), ptr(T) if want_T else None)
    return (A, TAU, T) if want_T else (A, TAU)


def make_Q(RY: np.ndarray, TAU: np.ndarray, M: int, N: int, NB: int):
    """Hybrid_make_Q restated: returns (Q^T array, R) in tile layout."""
    Q = np.zeros(M * N)
    R = np.array(RY, copy=True)
    lib().orc_make_Q(M, N, NB, ptr(Q), ptr(R), ptr(np.ascontiguousarray(TAU)))
    return Q, R


def dorgqr(RY: np.ndarray, TAU: np.ndarray, M: int, N: int, NB: int):
    Q = np.zeros(M * N)
    R = np.array(RY, copy=True)
    lib().orc_dorgqr(M, N, NB, ptr(Q), ptr(R), ptr(np.ascontiguousarray(TAU)))
    return Q


def dormqr(RY: np.ndarray, TAU: np.ndarray, C: np.ndarray, M: int, N: int, NB: int, CT: int):
    Cout = np.array(C, copy=True)
    R = np.ascontiguousarray(RY)
    lib().orc_dormqr(M, N, NB, ptr(R), ptr(np.ascontiguousarray(TAU)), ptr(Cout), CT)
    return Cout


def dgemm_tn(A: np.ndarray, B: np.ndarray, M: int, N: int, NB: int):
    C = np.zeros(M * N)
    lib().orc_dgemm_tn(M, N, NB, ptr(np.ascontiguousarray(A)), ptr(np.ascontiguousarray(B)), ptr(C))
    return C


def lstsq(A_tiles: np.ndarray, B: np.ndarray, M: int, N: int, NB: int, IB: int,
          refine_steps: int = 1, factor_tiles: np.ndarray | None = None) -> np.ndarray:
    """The least-squares solve of hqr_lstsq restated on the CPU: the oracle's
    tile QR of A, c = Q^T b by its dormqr, back substitution with R, then
    ``refine_steps`` FP64 refinement steps x += R^-1 (Q^T (b - A x))(1:N).
    B: (M, nrhs) array; returns x as an (N, nrhs) array.  factor_tiles: a
    perturbed A to factor instead (a stand-in for a lower-precision
    factorization); residuals always use A."""
    from scipy.linalg import solve_triangular
    B = np.asarray(B, dtype=np.float64).reshape(M, -1)
    nrhs = B.shape[1]
    A2d = from_tiles(A_tiles, M, N, NB)
    qt, R = _ls_factor(A_tiles if factor_tiles is None else factor_tiles, M, N, NB, IB, nrhs)

    def solve(rhs):
        return solve_triangular(R, qt(rhs)[:N], lower=False)

    x = solve(B)
    for _ in range(refine_steps):
        x = x + solve(B - A2d @ x)
    return x


def _ls_factor(F_tiles, M, N, NB, IB, nrhs):
    """Tile QR of F: (x -> Q^T x through the oracle's dormqr, R)."""
    CT = (nrhs + NB - 1) // NB
    RY, TAU = tile_qr(F_tiles, M, N, NB, IB)
    R = np.triu(from_tiles(RY, M, N, NB)[:N, :N])

    def qt(rhs):
        pad = np.zeros((M, CT * NB))
        pad[:, :nrhs] = rhs
        return from_tiles(dormqr(RY, TAU, to_tiles(pad, NB), M, N, NB, CT), M, CT * NB, NB)[:, :nrhs]

    return qt, R


def lstsq_aug(A_tiles: np.ndarray, B: np.ndarray, M: int, N: int, NB: int, IB: int,
              refine_steps: int = 2, factor_tiles: np.ndarray | None = None) -> np.ndarray:
    """hqr_lstsq_aug restated: x0 as in lstsq, r0 = b - A x0, then
    ``refine_steps`` steps of refinement on the augmented system
    [I A; A^T 0][r; x] = [b; 0] (Bjorck, BIT 7 (1967) 257-278): f = b - r -
    A x, g = -A^T r in FP64; h = R^-T g, d = Q^T f, x += R^-1 (d(1:N) - h),
    r += Q [h; d(N+1:M)].  Q is applied as the transpose of the oracle's
    Q^T of the identity (small cases only).  factor_tiles as in lstsq."""
    from scipy.linalg import solve_triangular
    B = np.asarray(B, dtype=np.float64).reshape(M, -1)
    nrhs = B.shape[1]
    A2d = from_tiles(A_tiles, M, N, NB)
    F = A_tiles if factor_tiles is None else factor_tiles
    qt, R = _ls_factor(F, M, N, NB, IB, nrhs)
    qt_full, _ = _ls_factor(F, M, N, NB, IB, M)
    QT = qt_full(np.eye(M))
    x = solve_triangular(R, qt(B)[:N], lower=False)
    r = B - A2d @ x
    for _ in range(refine_steps):
        f = B - r - A2d @ x
        g = -(A2d.T @ r)
        h = solve_triangular(R, g, trans="T", lower=False)
        d = qt(f)
        x = x + solve_triangular(R, d[:N] - h, lower=False)
        r = r + QT.T @ np.vstack([h, d[N:]])
    return x


def mat_make(M: int, N: int, NB: int, seed: int) -> np.ndarray:
    A = np.zeros(M * N)
    lib().orc_mat_fill(M, N, NB, ptr(A), seed, 0)
    return A


def mat_comp3(E_colmajor: np.ndarray, M: int, N: int) -> float:
    return lib().orc_mat_comp3(M, N, ptr(np.ascontiguousarray(E_colmajor)))


# --------------------------------------------------------------------------
# The shimmed reference build (_ref/), where present
# --------------------------------------------------------------------------

class MatStat(ctypes.Structure):
    """mat_stat_t (mat_prod.h:12-25)."""
    _fields_ = [("mat_M", ctypes.c_ulong), ("mat_N", ctypes.c_ulong),
                ("my_mat_M", ctypes.c_ulong), ("my_mat_N", ctypes.c_ulong),
                ("tile_M", ctypes.c_uint), ("tile_N", ctypes.c_uint),
                ("glob_tile_M", ctypes.c_uint), ("glob_tile_N", ctypes.c_uint),
                ("my_tile_M", ctypes.c_uint), ("my_tile_N", ctypes.c_uint)]


_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def ref_lib() -> ctypes.CDLL:
    """The reference's own code.  Its Hybrid_tile_QR opens two nested parallel
    regions; run it with OMP_NUM_THREADS="1,P" so that the outer region has one
    thread and the worker region P (any other setting with P > 1 does not
    terminate)."""
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_LIB_PATH)
        i, l, u = ctypes.c_int, ctypes.c_long, ctypes.c_uint
        st = ctypes.POINTER(MatStat)
        for name, args in {
            "mat_init": [st, l, l, i, i, i, i],
            "Hybrid_tile_QR": [st, _dp, _dp, i, i, i],
            "Hybrid_make_Q": [st, _dp, _dp, _dp, i, i, i],
            "Hybrid_dorgqr": [st, _dp, _dp, _dp, i, i],
            "Hybrid_dormqr": [st, _dp, _dp, _dp, i, i],
            "Hybrid_dgemm": [st, _dp, _dp, _dp, i, i],
            "Hybrid_make_I": [st, _dp, i, i],
            "mat_make": [st, _dp, u, i],
            "tile_dgeqrt": [i, i, i, _dp, i, _dp, _dp, _dp, i, _dp],
            "tile_dtsqrt": [i, i, i, _dp, i, _dp, i, _dp, _dp, i, _dp],
            "tile_dlarft": [i, i, i, _dp, i, _dp, _dp, i, _dp],
            "tile_dlarfb": [i, i, _dp, i, _dp, _dp, i, _dp],
            "tile_dssrfb": [i, i, _dp, _dp, i, _dp, _dp, i, _dp],
        }.items():
            fn = getattr(_ref, name)
            fn.restype = None
            fn.argtypes = args
    return _ref


def ref_status(M: int, N: int, NB: int) -> MatStat:
    st = MatStat()
    ref_lib().mat_init(ctypes.byref(st), M, N, NB, NB, 0, 1)
    return st


def ref_tile_qr(A_tiles: np.ndarray, M: int, N: int, NB: int, IB: int):
    st = ref_status(M, N, NB)
    A = np.array(A_tiles, copy=True)
    TAU = np.zeros((M // 2) * (N // 2) + (M // NB) * (N // NB) * NB)
    ref_lib().Hybrid_tile_QR(ctypes.byref(st), ptr(A), ptr(TAU), 0, 1, IB)
    return A, TAU[: (M // NB) * (N // NB) * NB].copy()


def ref_make_Q(RY: np.ndarray, TAU: np.ndarray, M: int, N: int, NB: int, IB: int):
    st = ref_status(M, N, NB)
    Q = np.zeros(M * N)
    R = np.array(RY, copy=True)
    ref_lib().Hybrid_make_Q(ctypes.byref(st), ptr(Q), ptr(R), ptr(np.array(TAU, copy=True)), 0, 1, IB)
    return Q, R


def ref_dorgqr(RY: np.ndarray, TAU: np.ndarray, M: int, N: int, NB: int):
    st = ref_status(M, N, NB)
    Q = np.zeros(M * N)
    R = np.array(RY, copy=True)
    ref_lib().Hybrid_dorgqr(ctypes.byref(st), ptr(Q), ptr(R), ptr(np.array(TAU, copy=True)), 0, 1)
    return Q


def ref_dormqr(RY: np.ndarray, TAU: np.ndarray, C: np.ndarray, M: int, N: int, NB: int):
    st = ref_status(M, N, NB)
    Cout = np.array(C, copy=True)
    ref_lib().Hybrid_dormqr(ctypes.byref(st), ptr(np.array(RY, copy=True)),
                            ptr(np.array(TAU, copy=True)), ptr(Cout), 0, 1)
    return Cout


def ref_dgemm(A: np.ndarray, B: np.ndarray, M: int, N: int, NB: int):
    st = ref_status(M, N, NB)
    C = np.zeros(M * N)
    ref_lib().Hybrid_dgemm(ctypes.byref(st), ptr(np.array(A, copy=True)),
                           ptr(np.array(B, copy=True)), ptr(C), 0, 1)
    return C


def ref_mat_make(M: int, N: int, NB: int, seed: int) -> np.ndarray:
    st = ref_status(M, N, NB)
    A = np.zeros(M * N)
    ref_lib().mat_make(ctypes.byref(st), ptr(A), seed, 0)
    return A
