"""The oracle's least-squares restatement (tile QR, dormqr, back substitution,
FP64 refinement) against numpy's LAPACK least squares, on CPU."""
import numpy as np
import pytest

import oracle as O
from ls_cases import ls_problem, ls_tol


@pytest.mark.parametrize("M,N,NB,IB,nrhs,kappa,steps", [(256, 128, 32, 8, 3, 1e3, 1),
                                                         (384, 192, 64, 16, 5, 1e6, 2),
                                                         (192, 192, 32, 32, 2, 1e2, 0)])
def test_oracle_lstsq_matches_numpy(M, N, NB, IB, nrhs, kappa, steps):
    A, _, b = ls_problem(M, N, nrhs, kappa, 7 + M)
    x = O.lstsq(O.to_tiles(A, NB), b, M, N, NB, IB, steps)
    xn = np.linalg.lstsq(A, b, rcond=None)[0]
    err = np.linalg.norm(x - xn) / np.linalg.norm(xn)
    assert err <= ls_tol(A, xn, b, kappa)


@pytest.mark.parametrize("M,N,NB,IB,nrhs,kappa,noise", [(384, 192, 64, 16, 3, 1e3, 1e-2),
                                                         (256, 128, 32, 8, 2, 1e4, 1e-3)])
def test_oracle_augmented_refinement_reaches_the_fp64_floor(M, N, NB, IB, nrhs, kappa, noise):
    """A factorization of A rounded to FP32 (backward error about 6e-8) stands
    in for a low-precision one: refinement on the augmented system reaches
    the FP64 least-squares bound; hqr_lstsq's refinement stalls near
    kappa^2 u_32 ||r|| / ||x||, orders of magnitude above it."""
    A, _, b = ls_problem(M, N, nrhs, kappa, 31 + M, noise=noise)
    At = O.to_tiles(A, NB)
    low = O.to_tiles(A.astype(np.float32).astype(np.float64), NB)
    xn = np.linalg.lstsq(A, b, rcond=None)[0]
    bar = ls_tol(A, xn, b, kappa)
    xa = O.lstsq_aug(At, b, M, N, NB, IB, 4, factor_tiles=low)
    xs = O.lstsq(At, b, M, N, NB, IB, 4, factor_tiles=low)
    ea = np.linalg.norm(xa - xn) / np.linalg.norm(xn)
    es = np.linalg.norm(xs - xn) / np.linalg.norm(xn)
    assert ea <= bar
    assert es > 100 * ea


def test_oracle_augmented_refinement_on_an_fp64_factorization():
    M, N, NB, IB, nrhs, kappa = 256, 128, 32, 8, 4, 1e6
    A, _, b = ls_problem(M, N, nrhs, kappa, 5)
    xn = np.linalg.lstsq(A, b, rcond=None)[0]
    xa = O.lstsq_aug(O.to_tiles(A, NB), b, M, N, NB, IB, 2)
    assert np.linalg.norm(xa - xn) / np.linalg.norm(xn) <= ls_tol(A, xn, b, kappa)
