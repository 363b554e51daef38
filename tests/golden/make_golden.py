"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own C sources (compiled unmodified against the shim
headers by ``oracle/Makefile`` into ``oracle/_ref``) on small seeded inputs and
stores inputs and outputs as ``.npz`` files.  The tests pin the oracle
restatement and the CUDA library against these files; the reference tree is
not needed to run them.

Usage (from the repository root, where the reference tree exists):
    OMP_NUM_THREADS=1,4 python tests/golden/make_golden.py
    OMP_NUM_THREADS=1,8 python tests/golden/make_golden.py --norms 8192 16384
The second form runs the reference's Hybrid_tile_QR + Hybrid_make_Q at the
given orders (NB = 256, IB = 32, the seeded uniform input) and records its
||A - QR||_F / ||A||_F and ||I - Q Q^T||_F in ref_norms.json: the accuracy the
GPU path is held to at sizes where an elementwise fixture would be too large.
The "1,P" thread list is required: the reference's Hybrid_tile_QR opens two
nested parallel regions (Hybrid_tile_QR.c:399-405) and only terminates when the
outer one has a single thread.
"""
import json
import os
import sys
import time

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


def slim_qr_case(name, M, N, NB, IB, seed, c_seed):
    """A larger case stored without the inputs (regenerated from their seeds by
    oracle.uniform_matrix) and without the Q Q^T / Q R products."""
    A = O.to_tiles(O.uniform_matrix(M, N, seed), NB)
    C = O.to_tiles(O.uniform_matrix(M, N, c_seed), NB)
    a, tau = O.ref_tile_qr(A, M, N, NB, IB)
    q, _ = O.ref_make_Q(a, tau, M, N, NB, IB)
    c = O.ref_dormqr(a, tau, C, M, N, NB)
    np.savez_compressed(os.path.join(HERE, name), M=M, N=N, NB=NB, IB=IB, seed=seed, c_seed=c_seed,
                        A_qr=a, TAU=tau, Qt=q, QtC=c)
    print("wrote", name)


def ref_norms(orders, NB=256, IB=32, seed=20151130):
    """The reference's own accuracy at large orders, into ref_norms.json."""
    path = os.path.join(HERE, "ref_norms.json")
    rec = json.load(open(path)) if os.path.exists(path) else {"cases": []}
    for n in orders:
        A2d = O.uniform_matrix(n, n, seed)
        A = O.to_tiles(A2d, NB)
        t0 = time.perf_counter()
        a, tau = O.ref_tile_qr(A, n, n, NB, IB)
        t1 = time.perf_counter()
        q, r = O.ref_make_Q(a, tau, n, n, NB, IB)
        t2 = time.perf_counter()
        del A, a
        Qt = O.from_tiles(q, n, n, NB)
        del q
        R = O.from_tiles(r, n, n, NB)
        del r
        E = Qt.T @ R
        E -= A2d
        resid = float(np.linalg.norm(E) / np.linalg.norm(A2d))
        del E, R, A2d
        G = Qt @ Qt.T
        G[np.diag_indices(n)] -= 1.0
        orth = float(np.linalg.norm(G))
        del G, Qt
        case = {"n": n, "NB": NB, "IB": IB, "seed": seed, "resid_fro_rel": resid, "orth_fro": orth,
                "threads": os.environ.get("OMP_NUM_THREADS", ""), "tile_qr_s": round(t1 - t0, 2),
                "make_q_s": round(t2 - t1, 2)}
        rec["cases"] = [c for c in rec["cases"] if not (c["n"] == n and c["NB"] == NB and c["IB"] == IB)]
        rec["cases"].append(case)
        rec["cases"].sort(key=lambda c: (c["n"], c["NB"], c["IB"]))
        json.dump(rec, open(path, "w"), indent=1)
        print(case, flush=True)


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
        O.build(ref_dir=os.environ.get("HYBRID3_REF_DIR", "/root/reference"))
    if not O.ref_available():
        raise SystemExit("reference build not available (needs the reference tree)")
    if "--norms" in sys.argv:
        ref_norms([int(v) for v in sys.argv[sys.argv.index("--norms") + 1:]])
        return
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
    # the tile order of the CPU workload configuration (NB = 256, IB = 32)
    slim_qr_case("qr_uniform_n512_nb256_ib32.npz", 512, 512, 256, 32, 20151130, 4242)


if __name__ == "__main__":
    main()
