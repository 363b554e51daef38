"""The C ABI on the CPU (no device work): the library loads, and every
function declared in include/*.h is exported and has a ctypes signature."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECL = re.compile(r"\b([A-Za-z_]\w*)\s*\(([^;{}()]|\([^()]*\))*\)\s*;")
NOT_FUNCS = {"sizeof", "defined"}


def declared_functions():
    names = {}
    for path in sorted(glob.glob(os.path.join(ROOT, "include", "*.h"))):
        src = open(path).read()
        src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
        src = re.sub(r"//[^\n]*", " ", src)
        src = "\n".join(l for l in src.splitlines() if not l.lstrip().startswith("#"))
        for m in DECL.finditer(src):
            if m.group(1) not in NOT_FUNCS:
                names[m.group(1)] = os.path.basename(path)
    return names


@pytest.fixture(scope="module")
def lib():
    import hybrid3_gb300 as H
    if not os.path.exists(H.LIB_PATH):
        pytest.skip("library not built")
    return H


def test_headers_declare_the_drop_in_entry_points():
    names = declared_functions()
    for n in ["Hybrid_tile_QR", "Hybrid_make_Q", "Hybrid_dorgqr", "Hybrid_dormqr", "Hybrid_dgemm",
              "Hybrid_make_I", "Hybrid_dgeqrf", "Hybrid_remv_Y", "tile_dgeqrt", "tile_dtsqrt",
              "tile_dlarfb", "tile_dssrfb", "tile_sub_dgeqr2", "tile_sub_dlarft", "tile_sub_dlarfb",
              "tile_sub_dssrfb", "tile_dlarft", "tile_dssrfb_head", "tile_dssrfb_tail",
              "tile_return_dlarfb", "tile_return_dssrfb", "tile_return_dlarft", "tile_sub_dtsqr2",
              "tile_init", "TilSch_init", "TilSch_pop", "TilSch_push", "mat_init", "mat_comp3",
              "hqr_geqrf", "hqr_make_q", "hqr_geqrf_noalloc"]:
        assert n in names, n


def test_every_declared_function_is_exported(lib):
    so = ctypes.CDLL(lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(so, n)]
    assert not missing, missing


def test_every_declared_function_has_a_signature(lib):
    missing = [n for n in declared_functions() if n not in lib.SIGNATURES]
    assert not missing, missing
    lib.lib()   # applies every signature


def test_tile_init_allocates_three_tiles(lib):
    L = lib.lib()
    p = L.tile_init(b"d", 8, 4)
    assert p
    buf = (ctypes.c_double * 96).from_address(p)
    assert all(v == 0.0 for v in buf)
    ctypes.CDLL(None).free(ctypes.c_void_p(p))
