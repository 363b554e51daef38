"""Least-squares test problems shared by the oracle and GPU tests: the
least-squares workload (A = U S V^T, geometric singular values, b = A x_true
+ 1e-8 noise) at test sizes."""
import numpy as np

EPS = np.finfo(np.float64).eps


def ls_problem(M, N, nrhs, kappa, seed, noise=1e-8):
    """A = U S V^T with Haar U, V (QR of Gaussians, signs fixed by diag R) and
    singular values geometric from 1 to 1/kappa; x ~ N(0,1); b = A x + noise N(0,1)."""
    rng = np.random.default_rng(seed)

    def haar(m, n):
        q, r = np.linalg.qr(rng.standard_normal((m, n)))
        return q * np.sign(np.diag(r))

    U, V = haar(M, N), haar(N, N)
    s = kappa ** (-np.arange(N) / max(N - 1, 1))
    A = (U * s) @ V.T
    x = rng.standard_normal((N, nrhs))
    b = A @ x + noise * rng.standard_normal((M, nrhs))
    return A, x, b


def ls_tol(A, x, b, kappa):
    """Perturbation bound of a backward-stable least-squares solution (c = 100):
    100 eps kappa (1 + kappa ||r|| / (||A|| ||x||))."""
    r = b - A @ x
    return 100 * EPS * kappa * (1 + kappa * np.linalg.norm(r) / (np.linalg.norm(A, 2) * np.linalg.norm(x)))
