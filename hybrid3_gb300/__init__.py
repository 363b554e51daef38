"""hybrid3_gb300 -- GB300-native tiled Householder QR behind Hybrid3's C entry
points.

The product is the shared library ``libhybrid3_gb300.so`` (C ABI declared in
``include/``).  This module only loads it with ctypes and declares the
signatures, so that Python callers (tests, benchmarks) go through exactly the
entry points a C caller links against.  There is no Python or CPU fallback:
importing the bindings fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libhybrid3_gb300.so")

HQR_OK = 0
HQR_ERR_INVALID = -1
HQR_ERR_CUDA = -2
HQR_ERR_TIMEOUT = -3
HQR_ERR_NOMEM = -4
HQR_ERR_UNSUPPORTED = -5
HQR_ERR_DEVICE = -6
HQR_PREC_FP64 = 0
HQR_PREC_OZAKI = 1
HQR_PREC_OZAKI_FAST = 2
HQR_PREC_FP32 = 3
HQR_ERRORS_ABORT = 0
HQR_ERRORS_RETURN = 1

_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class MatStat(ctypes.Structure):
    """mat_stat_t (include/mat_prod.h)."""
    _fields_ = [("mat_M", ctypes.c_ulong), ("mat_N", ctypes.c_ulong),
                ("my_mat_M", ctypes.c_ulong), ("my_mat_N", ctypes.c_ulong),
                ("tile_M", ctypes.c_uint), ("tile_N", ctypes.c_uint),
                ("glob_tile_M", ctypes.c_uint), ("glob_tile_N", ctypes.c_uint),
                ("my_tile_M", ctypes.c_uint), ("my_tile_N", ctypes.c_uint)]


class HqrStats(ctypes.Structure):
    _fields_ = [("count", ctypes.c_ulonglong * 7), ("cycles", ctypes.c_ulonglong * 7)]


class TilSch(ctypes.Structure):
    _fields_ = [("i", ctypes.c_long), ("j", ctypes.c_long), ("k", ctypes.c_long),
                ("priority", ctypes.c_uint), ("data", ctypes.c_uint)]


class TilSchList(ctypes.Structure):
    _fields_ = [("list", ctypes.POINTER(TilSch)), ("head", ctypes.c_long),
                ("tail", ctypes.c_long), ("max", ctypes.c_long), ("max_size", ctypes.c_long)]


# (name, restype, argtypes) of every exported entry point.
_I, _L, _D, _U = ctypes.c_int, ctypes.c_long, ctypes.c_double, ctypes.c_uint
_ST = ctypes.POINTER(MatStat)
SIGNATURES = {
    # include/Hybrid_tile_QR.h
    "Hybrid_dgeqrf": (None, [_ST, _dp, _dp, _I, _I]),
    "Hybrid_tile_QR": (None, [_ST, _dp, _dp, _I, _I, _I]),
    "Hybrid_make_Q": (None, [_ST, _dp, _dp, _dp, _I, _I, _I]),
    "Hybrid_make_I": (None, [_ST, _dp, _I, _I]),
    "Hybrid_remv_Y": (None, [_ST, _dp, _I, _I]),
    "Hybrid_dgemm": (None, [_ST, _dp, _dp, _dp, _I, _I]),
    "Hybrid_dorgqr": (None, [_ST, _dp, _dp, _dp, _I, _I]),
    "Hybrid_dormqr": (None, [_ST, _dp, _dp, _dp, _I, _I]),
    # include/mat_prod.h
    "mat_init": (None, [_ST, _L, _L, _I, _I, _I, _I]),
    "mat_comp": (_D, [_ST, _dp, _U, _I, _I]),
    "mat_comp2": (_D, [_ST, _dp, _dp, _I, _I]),
    "mat_comp3": (_D, [_ST, _dp, _I, _I]),
    "mat_make": (None, [_ST, _dp, _U, _I]),
    "mat_remv": (None, [_ST, _dp, _U, _I]),
    "mat_dprint": (None, [_ST, _dp, _dp]),
    "mat_print": (None, [_ST, _vp, _dp, ctypes.c_char_p]),
    "mat_print_tile": (None, [_vp, _dp, ctypes.c_char_p, _I, _I]),
    # include/TileSch.h
    "TilSch_init": (None, [ctypes.POINTER(TilSchList), _L]),
    "TilSch_pop": (_I, [ctypes.POINTER(TilSchList), ctypes.POINTER(TilSch)]),
    "TilSch_push": (_I, [ctypes.POINTER(TilSchList), TilSch]),
    "TilSch_empty": (_I, [ctypes.POINTER(TilSchList)]),
    "TilSch_fully": (_I, [ctypes.POINTER(TilSchList)]),
    "TilSch_depend": (_I, [ctypes.POINTER(TilSchList), TilSch, _U]),
    "TilSch_delete": (_I, [ctypes.POINTER(TilSchList), TilSch]),
    "TilSch_end": (None, [ctypes.POINTER(TilSchList)]),
    # include/hqr_gpu.h
    "hqr_status_string": (ctypes.c_char_p, [_I]),
    "hqr_set_error_mode": (None, [_I]),
    "hqr_set_default_precision": (None, [_I]),
    "hqr_get_default_precision": (_I, []),
    "hqr_last_error": (_I, []),
    "hqr_last_cuda_error": (ctypes.c_char_p, []),
    "hqr_set_timeout_ms": (None, [ctypes.c_longlong]),
    "hqr_plan_create": (_I, [ctypes.POINTER(_vp), _L, _L, _I, _I, _I]),
    "hqr_plan_destroy": (_I, [_vp]),
    "hqr_plan_t_factors": (_vp, [_vp]),
    "hqr_geqrf": (_I, [_vp, _vp, _vp, _vp]),
    "hqr_geqrf_async": (_I, [_vp, _vp, _vp, _vp]),
    "hqr_geqrf_noalloc": (_I, [_L, _L, _I, _I, _vp, _vp, _vp]),
    "hqr_plan_status": (_I, [_vp, _vp]),
    "hqr_plan_stats": (_I, [_vp, ctypes.POINTER(HqrStats), _vp]),
    "hqr_make_q": (_I, [_vp, _vp, _vp, _vp, _I, _vp]),
    "hqr_make_q_async": (_I, [_vp, _vp, _vp, _vp, _I, _vp]),
    "hqr_ormqr_t": (_I, [_vp, _vp, _vp, _vp, _I, _I, _vp]),
    "hqr_lstsq": (_I, [_vp, _vp, _vp, _I, _I, _vp, _I, _I, _vp, _vp]),
    "hqr_lstsq_aug": (_I, [_vp, _vp, _vp, _I, _I, _vp, _I, _I, _vp, _vp]),
    "hqr_plan_set_tree": (_I, [_vp, _I]),
    "hqr_colmajor_to_tiles_padded": (_I, [_L, _L, _L, _I, _vp, _vp, _vp]),
    "hqr_tiles_to_colmajor_padded": (_I, [_L, _L, _L, _I, _vp, _vp, _vp]),
    "hqr_batch_create": (_I, [ctypes.POINTER(_vp), _I, ctypes.POINTER(_L), ctypes.POINTER(_L),
                              ctypes.POINTER(_I), ctypes.POINTER(_I), _I, _I]),
    "hqr_batch_destroy": (_I, [_vp]),
    "hqr_batch_geqrf": (_I, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), _vp]),
    "hqr_batch_geqrf_async": (_I, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), _vp]),
    "hqr_batch_ormqr_t": (_I, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp), _I, _vp]),
    "hqr_batch_ormqr_t_async": (_I, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp), _I,
                                     _vp]),
    "hqr_batch_status": (_I, [_vp, _vp]),
    "hqr_batch_ctas_per_sm": (_I, [_vp]),
    "hqr_batch_stats": (_I, [_vp, ctypes.POINTER(HqrStats), _vp]),
    "hqr_dgemm_tn": (_I, [_L, _I, _vp, _vp, _vp, _vp]),
    "hqr_make_identity": (_I, [_L, _L, _I, _vp, _vp]),
    "hqr_fill_uniform": (_I, [_L, _L, _I, ctypes.c_uint64, _vp, _vp]),
    "hqr_frob2": (_I, [_L, _L, _I, _vp, _vp, _D, _dp, _vp]),
    "hqr_tiles_to_colmajor": (_I, [_L, _L, _I, _vp, _vp, _vp]),
    "hqr_colmajor_to_tiles": (_I, [_L, _L, _I, _vp, _vp, _vp]),
    "hqr_zero_reflectors": (_I, [_L, _L, _I, _vp, _vp]),
    "hqr_fp64_peak_tflops": (_D, [_vp]),
    "hqr_fp64_mma_peak_tflops": (_D, [_I, _vp]),
    "hqr_dropin_phase_ms": (_I, [ctypes.POINTER(ctypes.c_double)]),
    "hqr_host_alloc": (_I, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]),
    "hqr_ormqr_n": (_I, [_vp, _vp, _vp, _vp, _I, _I, _vp]),
    "hqr_ormqr_t_async": (_I, [_vp, _vp, _vp, _vp, _I, _I, _vp]),
    "hqr_ormqr_n_async": (_I, [_vp, _vp, _vp, _vp, _I, _I, _vp]),
    "hqr_host_free": (_I, [_vp]),
    "hqr_ozaki_product": (_I, [_I, _vp, _vp, _vp, _vp]),
    # include/tile_kernel.h (pointer arguments: host or device addresses)
    "tile_init": (_vp, [ctypes.c_char, _I, _I]),
    "tile_dgeqrt": (None, [_I, _I, _I, _vp, _I, _vp, _vp, _vp, _I, _vp]),
    "tile_dtsqrt": (None, [_I, _I, _I, _vp, _I, _vp, _I, _vp, _vp, _I, _vp]),
    "tile_dlarfb": (None, [_I, _I, _vp, _I, _vp, _vp, _I, _vp]),
    "tile_dssrfb": (None, [_I, _I, _vp, _vp, _I, _vp, _vp, _I, _vp]),
    "tile_sub_dgeqr2": (None, [_I, _I, _vp, _I, _vp, _vp, _vp]),
    "tile_sub_dlarft": (None, [_I, _I, _vp, _I, _vp, _vp, _I, _vp]),
    "tile_sub_dlarfb": (None, [_I, _I, _I, _vp, _I, _vp, _I, _vp, _I, _vp]),
    "tile_sub_dssrfb": (None, [_I, _I, _I, _I, _vp, _I, _vp, _I, _vp, _I, _vp, _I, _vp]),
    "tile_dlarft": (None, [_I, _I, _I, _vp, _I, _vp, _vp, _I, _vp]),
    "tile_dssrfb_head": (None, [_I, _I, _vp, _vp, _I, _vp, _vp, _I, _vp]),
    "tile_dssrfb_tail": (None, [_I, _I, _vp, _I, _vp, _vp]),
    "tile_return_dlarfb": (None, [_I, _I, _vp, _I, _vp, _vp, _I, _vp]),
    "tile_return_dssrfb": (None, [_I, _I, _vp, _vp, _I, _vp, _vp, _I, _vp]),
    "tile_return_dlarft": (None, [_I, _I, _vp, _I, _vp, _vp, _I, _vp]),
    "tile_sub_dtsqr2": (None, [_I, _I, _vp, _I, _vp, _I, _vp, _vp]),
}

_lib = None


def lib() -> ctypes.CDLL:
    """The loaded C library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m hybrid3_gb300.build` "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int, what: str = "") -> None:
    if rc != HQR_OK:
        msg = lib().hqr_status_string(rc).decode()
        if rc == HQR_ERR_CUDA:
            msg += " -- " + lib().hqr_last_cuda_error().decode()
        raise RuntimeError(f"{what}: {msg} ({rc})")


def status(M: int, N: int, NB: int) -> MatStat:
    st = MatStat()
    lib().mat_init(ctypes.byref(st), M, N, NB, NB, 0, 1)
    return st


class Plan:
    """Owns an hqr_plan_t (device T factors + scheduler workspace)."""

    def __init__(self, M: int, N: int, NB: int, IB: int, precision: int = HQR_PREC_FP64):
        h = _vp()
        check(lib().hqr_plan_create(ctypes.byref(h), M, N, NB, IB, precision), "hqr_plan_create")
        self.h = h
        self.M, self.N, self.NB, self.IB = M, N, NB, IB

    def close(self):
        if self.h:
            lib().hqr_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tree(self, domain_tiles: int):
        """Domain tree of domain_tiles tiles for the factorizations on this plan (0: flat)."""
        check(lib().hqr_plan_set_tree(self.h, domain_tiles), "hqr_plan_set_tree")

    def lstsq(self, dA, dB, nrhs, dX, refine_steps=1, ldb=None, ldx=None, stream=None, augmented=False):
        """hqr_lstsq (hqr_lstsq_aug with augmented=True) on device addresses
        (tile-layout A of this plan's shape, column-major B and X); returns
        ||b - A x||_2 per right-hand side."""
        res = (ctypes.c_double * nrhs)()
        fn = lib().hqr_lstsq_aug if augmented else lib().hqr_lstsq
        name = "hqr_lstsq_aug" if augmented else "hqr_lstsq"
        check(fn(self.h, dA, dB, ldb or self.M, nrhs, dX, ldx or self.N, refine_steps, res, stream), name)
        return list(res)

    def stats(self, stream=None):
        s = HqrStats()
        check(lib().hqr_plan_stats(self.h, ctypes.byref(s), stream), "hqr_plan_stats")
        return {"count": list(s.count), "cycles": list(s.cycles)}


def _ptrs(xs):
    return (_vp * len(xs))(*[_vp(int(x)) for x in xs])


class Batch:
    """Owns an hqr_batch_t: independent FP64 tile QRs of uneven shapes, each
    call one persistent launch over every matrix's tasks."""

    def __init__(self, M, N, NB, IB, max_nrhs: int = 1, ctas_per_sm: int = 0):
        n = len(M)
        h = _vp()
        check(lib().hqr_batch_create(ctypes.byref(h), n, (_L * n)(*M), (_L * n)(*N), (_I * n)(*NB),
                                     (_I * n)(*IB), max_nrhs, ctas_per_sm), "hqr_batch_create")
        self.h = h
        self.count = n
        self._keep = []

    def close(self):
        if self.h:
            lib().hqr_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def geqrf(self, dA, dTAU, stream=None, wait=True):
        """Factor matrix b in place at device address dA[b] (TAU to dTAU[b])."""
        a, t = _ptrs(dA), _ptrs(dTAU)
        fn = lib().hqr_batch_geqrf if wait else lib().hqr_batch_geqrf_async
        check(fn(self.h, a, t, stream), "hqr_batch_geqrf")

    def ormqr_t(self, dA, dTAU, dC, nrhs: int, stream=None, wait=True):
        """First nrhs columns of dC[b] <- Q_b^T dC[b] for the last factorization."""
        a, t, c = _ptrs(dA), _ptrs(dTAU), _ptrs(dC)
        fn = lib().hqr_batch_ormqr_t if wait else lib().hqr_batch_ormqr_t_async
        check(fn(self.h, a, t, c, nrhs, stream), "hqr_batch_ormqr_t")

    def ctas_per_sm(self) -> int:
        return lib().hqr_batch_ctas_per_sm(self.h)

    def status(self, stream=None):
        check(lib().hqr_batch_status(self.h, stream), "hqr_batch_status")

    def stats(self, stream=None):
        s = HqrStats()
        check(lib().hqr_batch_stats(self.h, ctypes.byref(s), stream), "hqr_batch_stats")
        return {"count": list(s.count), "cycles": list(s.cycles)}
