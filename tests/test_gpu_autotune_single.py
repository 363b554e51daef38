"""The single-matrix autotuner on the device: every candidate that the
shape supports gets a positive measured rate, the choice is one of them, and
a plan made with the choice factors the matrix to the oracle's R."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_tune_single_measures_and_its_choice_factors():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hybrid3_gb300 as H
    from hybrid3_gb300 import autotune as AT
    H.lib().hqr_set_error_mode(H.HQR_ERRORS_RETURN)
    cands = (("split", 128, 32), ("fp64", 128, 32), ("fp64", 256, 32))
    t = AT.tune_single(H, torch, 1536, 768, want_q=True, candidates=cands, reps=1)
    rates = t["shapes"][0]["rates"]
    assert set(rates) == set(cands) and all(r > 0 for r in rates.values())
    prec, nb, ib = AT.choose_single(t, 1536, 768)
    assert (prec, nb, ib) in cands
    M, N = 1536, 768
    A2d = O.uniform_matrix(M, N, 3)
    A = O.to_tiles(A2d, nb)
    plan = H.Plan(M, N, nb, ib, {"fp64": H.HQR_PREC_FP64, "split": H.HQR_PREC_OZAKI}[prec])
    dA = torch.from_numpy(A.copy()).cuda()
    dTAU = torch.zeros((M // nb) * (N // nb) * nb, dtype=torch.float64, device="cuda")
    H.check(H.lib().hqr_geqrf(plan.h, dA.data_ptr(), dTAU.data_ptr(), None), "geqrf")
    plan.close()
    a = dA.cpu().numpy()
    ora, _ = O.tile_qr(A, M, N, nb, ib)
    R = np.triu(O.from_tiles(a, M, N, nb)[:N, :N])
    Ro = np.triu(O.from_tiles(ora, M, N, nb)[:N, :N])
    assert np.abs(R - Ro).max() <= max(M, N) * np.finfo(float).eps * np.linalg.norm(A2d)
