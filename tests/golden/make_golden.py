"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own C sources (compiled unmodified against the shim
headers by ``oracle/Makefile`` into ``oracle/_ref``) on small seeded inputs and
stores inputs and outputs as ``.npz`` files.  The tests pin the oracle
restatement and the CUDA library against these files; the reference tree is
not needed to run them.

Usage (from the repository root, where the reference tree exists):
    OMP_NUM_THREADS=1,4 python tests/golden/make_golden.py
The "1,P" thread list is required: the reference's Hybrid_tile_QR opens two
nested parallel regions (Hybrid_tile_QR.c:399-405) and only terminates when the
outer one has a single thread.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402


def qr_case(name, A_tiles, M, N, NB, IB, C_tiles, extra=None):
    a, tau = O.ref_tile_qr(A_tiles, M, N, NB, IB)
    q, r = O.ref_make_Q(a, tau, M, N, NB, IB)
    qo = O.ref_dorgqr(a, tau, M, N, NB)
    c = O.ref_dormqr(a, tau, C_tiles, M, N, NB)
    qq = O.ref_dgemm(q, q, M, N, NB)                      # Q Q^T (main.c:209)
    qr = O.ref_dgemm(q, r, M, N, NB)                      # Q R   (main.c:242)
    out = dict(M=M, N=N, NB=NB, IB=IB, A=A_tiles, A_qr=a, TAU=tau, Qt=q, R=r,
               Qt_dorgqr=qo, C=C_tiles, QtC=c, QQt=qq, QR=qr)
    if extra:
        out.update(extra)
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("wrote", name)


def tile_kernel_case(name, NB, IB, seed):
    """The reference's own tile_kernel.c entry points on random tiles."""
    rng = np.random.default_rng(seed)
    L = O.ref_lib()
    dp = O.ptr
    out = dict(NB=NB, IB=IB)
    # tile_dgeqrt
    A = np.asfortranarray(rng.uniform(-1, 1, (NB, NB)))
    out["geqrt_A"] = A.copy()
    TAU = np.zeros(NB)
    Y = np.zeros((NB, NB), order="F")
    T = np.zeros((NB, NB), order="F")
    work = np.zeros(3 * NB * NB)
    L.tile_dgeqrt(NB, NB, IB, dp(A), NB, dp(TAU), dp(Y), dp(T), NB, dp(work))
    out.update(geqrt_A_out=A.copy(), geqrt_TAU=TAU.copy(), geqrt_Y=Y.copy(), geqrt_T=T.copy())
    # tile_dlarft (block = 1 -> full lower T) on the GEQRT Y
    T2 = np.zeros((NB, NB), order="F")
    L.tile_dlarft(NB, NB, 1, dp(Y), NB, dp(TAU), dp(T2), NB, dp(work))
    out["larft_T"] = T2.copy()
    # tile_dlarfb with that (Y, T) on a random tile
    C = np.asfortranarray(rng.uniform(-1, 1, (NB, NB)))
    out["larfb_C"] = C.copy()
    L.tile_dlarfb(NB, NB, dp(C), NB, dp(Y), dp(T2), NB, dp(work))
    out["larfb_C_out"] = C.copy()
    # tile_dtsqrt on [upper(R); dense]
    R = np.asfortranarray(np.triu(rng.uniform(-1, 1, (NB, NB))))
    A2 = np.asfortranarray(rng.uniform(-1, 1, (NB, NB)))
    out.update(tsqrt_R=R.copy(), tsqrt_A2=A2.copy())
    TAU = np.zeros(NB)
    T = np.zeros((NB, NB), order="F")
    L.tile_dtsqrt(NB, NB, IB, dp(R), NB, dp(A2), NB, dp(TAU), dp(T), NB, dp(work))
    out.update(tsqrt_R_out=R.copy(), tsqrt_V=A2.copy(), tsqrt_TAU=TAU.copy(), tsqrt_T=T.copy())
    T3 = np.zeros((NB, NB), order="F")
    L.tile_dlarft(NB, NB, 1, dp(A2), NB, dp(TAU), dp(T3), NB, dp(work))
    out["tsqrt_fullT"] = T3.copy()
    # tile_dssrfb with (V, full lower T)
    A1 = np.asfortranarray(rng.uniform(-1, 1, (NB, NB)))
    B2 = np.asfortranarray(rng.uniform(-1, 1, (NB, NB)))
    out.update(ssrfb_A1=A1.copy(), ssrfb_A2=B2.copy())
    L.tile_dssrfb(NB, NB, dp(A1), dp(B2), NB, dp(A2), dp(T3), NB, dp(work))
    out.update(ssrfb_A1_out=A1.copy(), ssrfb_A2_out=B2.copy())
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("wrote", name)


def main():
    if not O.ref_available():
        O.build()
    if not O.ref_available():
        raise SystemExit("reference build not available (needs the reference tree)")
    M = N = 128
    NB, IB = 32, 8
    A = O.to_tiles(O.uniform_matrix(M, N, 20151130), NB)
    C = O.to_tiles(O.uniform_matrix(M, N, 4242), NB)
    qr_case("qr_uniform_n128_nb32_ib8.npz", A, M, N, NB, IB, C)
    # The reference's own input generator (mat_make, glibc rand, seed 20151130)
    Ar = O.ref_mat_make(M, N, NB, 20151130)
    qr_case("qr_matmake_n128_nb32_ib8.npz", Ar, M, N, NB, IB, C)
    # IB == NB (the reference's default when argv[3] is absent, main.c:87)
    qr_case("qr_uniform_n128_nb32_ib32.npz", A, M, N, NB, NB, C)
    tile_kernel_case("tile_kernels_nb32_ib8.npz", 32, 8, 7)


if __name__ == "__main__":
    main()
