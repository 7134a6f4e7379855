"""The peeling variant (recon_theory_phase_space_LFM_with_filter_simple_peeling.m) against
the FP64 oracle: volume (top plane restored), peeled image and scaled top-plane projection.
Tolerance: relative L2 1e-4 in FP32, 1e-3 on the tensor cores (bf16x2)."""
import numpy as np
import pytest

from oracle import mesolf_ref as R
from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case():
    w = synth.small_config(lenslets=(6, 5), K0=61, Z=7, seed=3, n_obj=14)
    H, Ht = w.psf()
    LF = w.measured(H, w.volume())
    ref = R.recon_phase_space_peeling(LF, H, Ht, 2)
    return H, Ht, LF, ref


@pytest.mark.parametrize("prec,tol", [("fp32", 1e-4), ("bf16x2", 1e-3)])
def test_peeling_matches_oracle(cuda, case, prec, tol):
    from mesolf_gb300 import recon_theory_phase_space_LFM_with_filter_simple_peeling as peel
    H, Ht, LF, (X_ref, LF2_ref, P_ref) = case
    X, LF2, P = peel(LF, H, Ht, 2, True, 1, precision=prec)
    assert X.shape == X_ref.shape and LF2.shape == LF.shape
    assert rel_l2(P, P_ref) <= tol, rel_l2(P, P_ref)
    assert rel_l2(LF2, LF2_ref) <= tol, rel_l2(LF2, LF2_ref)
    assert rel_l2(X, X_ref) <= tol, rel_l2(X, X_ref)
    assert np.array_equal(X[:, :, 0] > 0, X_ref[:, :, 0] > 0) or rel_l2(X[:, :, 0], X_ref[:, :, 0]) <= tol


def test_peeling_variant_solve_differs_from_base(cuda, case):
    """The variant's own RL solve: floor-rounded filter bank and D + 1e-10."""
    import torch
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    from mesolf_gb300.api import _fortran
    H, Ht, LF, _ = case
    psf = PhaseSpacePSF(H, Ht)
    lf = _fortran(torch.as_tensor(np.ascontiguousarray(LF)).cuda())[0]
    got = RLSolver(psf, LF.shape, variant="peeling").run(lf, 2).cpu().numpy()
    ref = R.recon_phase_space(LF, H, Ht, 2, variant="peeling")
    assert rel_l2(got, ref) <= 1e-4, rel_l2(got, ref)
