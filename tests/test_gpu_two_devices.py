"""The executor's per-device caches (the dynamic shared-memory opt-in of each
kernel and the SM count are per device): a factorization on device 0, then
one on device 1, each in FP64 and split precision, matches the oracle.  Runs
only where two GPUs are visible."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_factor_on_two_devices_in_turn():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available() or torch.cuda.device_count() < 2:
        pytest.skip("needs two CUDA devices")
    import hybrid3_gb300 as H
    H.lib().hqr_set_error_mode(H.HQR_ERRORS_RETURN)
    M = N = 512
    A2d = O.uniform_matrix(M, N, 77)
    nA = np.linalg.norm(A2d)
    for prec, NB, IB in ((H.HQR_PREC_FP64, 256, 32), (H.HQR_PREC_OZAKI, 128, 32)):
        A = O.to_tiles(A2d, NB)
        ra, _ = O.tile_qr(A, M, N, NB, IB)
        for dev in (0, 1):
            torch.cuda.set_device(dev)
            plan = H.Plan(M, N, NB, IB, prec)
            dA = torch.from_numpy(A.copy()).cuda(dev)
            dTAU = torch.zeros((M // NB) * (N // NB) * NB, dtype=torch.float64, device=f"cuda:{dev}")
            H.check(H.lib().hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "geqrf")
            plan.close()
            assert np.abs(dA.cpu().numpy() - ra).max() <= max(M, N) * np.finfo(float).eps * nA
    torch.cuda.set_device(0)
