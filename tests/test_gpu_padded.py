"""Column-major <-> tile layout with padded tail tiles, and QR of sizes that
are not tile multiples through zero padding, on the GPU through the C ABI.

Bar: the conversions are exact copies (bit-for-bit); the padded factorization
matches the oracle's tile QR of the same padded matrix within n eps ||A||
elementwise, and the padding stays zero (tau 0 for the padded columns)."""
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
    return H, torch


def ceil_to(x, nb):
    return -(-x // nb) * nb


@pytest.mark.parametrize("M,N,ld,NB", [(300, 200, 300, 128), (129, 1, 131, 64), (1, 257, 1, 128),
                                       (256, 256, 260, 128), (77, 45, 80, 32)])
def test_padded_round_trip(env, M, N, ld, NB):
    H, torch = env
    rng = np.random.default_rng(M * 7 + N)
    full = rng.standard_normal((ld, N))
    cm = torch.from_numpy(full.reshape(-1, order="F").copy()).cuda()
    Mp, Np = ceil_to(M, NB), ceil_to(N, NB)
    tiles = torch.full((Mp * Np,), np.nan, dtype=torch.float64, device="cuda")
    H.check(H.lib().hqr_colmajor_to_tiles_padded(M, N, ld, NB, cm.data_ptr(), tiles.data_ptr(), None))
    pad = np.zeros((Mp, Np))
    pad[:M, :N] = full[:M, :]
    assert np.array_equal(tiles.cpu().numpy(), O.to_tiles(pad, NB))
    back = torch.full((ld * N,), 7.0, dtype=torch.float64, device="cuda")
    H.check(H.lib().hqr_tiles_to_colmajor_padded(M, N, ld, NB, tiles.data_ptr(), back.data_ptr(), None))
    b = back.cpu().numpy().reshape(ld, N, order="F")
    assert np.array_equal(b[:M], full[:M])
    assert np.all(b[M:] == 7.0)   # rows beyond M of the leading dimension untouched


def test_padded_rejects_bad_arguments(env):
    H, torch = env
    d = torch.zeros(128 * 128, dtype=torch.float64, device="cuda")
    L = H.lib()
    assert L.hqr_colmajor_to_tiles_padded(10, 10, 9, 128, d.data_ptr(), d.data_ptr(), None) == H.HQR_ERR_INVALID
    assert L.hqr_tiles_to_colmajor_padded(0, 10, 10, 128, d.data_ptr(), d.data_ptr(), None) == H.HQR_ERR_INVALID


@pytest.mark.parametrize("M,N,prec", [(300, 200, "fp64"), (300, 200, "split"), (200, 200, "split"),
                                      (450, 130, "fp64")])
def test_qr_of_padded_matrix(env, M, N, prec):
    H, torch = env
    NB, IB = 128, 32
    rng = np.random.default_rng(M + N)
    A = rng.uniform(-1, 1, (M, N))
    Mp, Np = ceil_to(M, NB), ceil_to(N, NB)
    if Mp < Np:
        Mp = Np
    cm = torch.from_numpy(A.reshape(-1, order="F").copy()).cuda()
    dA = torch.empty(Mp * Np, dtype=torch.float64, device="cuda")
    H.check(H.lib().hqr_colmajor_to_tiles_padded(M, N, M, NB, cm.data_ptr(), dA.data_ptr(), None))
    pad = np.zeros((Mp, Np))
    pad[:M, :N] = A
    p = H.HQR_PREC_OZAKI if prec == "split" else H.HQR_PREC_FP64
    plan = H.Plan(Mp, Np, NB, IB, p)
    dTAU = torch.zeros((Mp // NB) * (Np // NB) * NB, dtype=torch.float64, device="cuda")
    try:
        H.check(H.lib().hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "hqr_geqrf")
    finally:
        plan.close()
    ra, rtau = O.tile_qr(O.to_tiles(pad, NB), Mp, Np, NB, IB)
    t = max(Mp, Np) * EPS * np.linalg.norm(A)
    got = dA.cpu().numpy()
    assert np.abs(got - ra).max() <= t
    assert np.abs(dTAU.cpu().numpy() - rtau).max() <= t
    R = np.triu(O.from_tiles(got, Mp, Np, NB))
    # R of the leading columns: its leading N x N block; padded columns give zero rows/columns
    assert np.all(R[:, N:] == 0.0)
    Rn = np.linalg.qr(A, mode="r")
    assert np.allclose(np.abs(R[:N, :N]), np.abs(Rn), atol=t)
