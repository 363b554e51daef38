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
