"""Tensor-core (tcgen05, BF16 or FP16 operands, FP32 accumulation) RL path against the FP64
oracle.

Tolerances (relative L2), from the operand rounding of each mode:
  bf16x3 / fp16x3  (hi+lo split of taps and activations, 3 MMA passes)  1e-5 per projection,
                   1e-4 for a whole solve (the FP32 bar);
  bf16x2  (activations split, taps single BF16, 8 bits)     2e-3 per view step,
          1e-3 for a whole solve (the mixed-precision bar);
  fp16x2  (activations split, taps single FP16, 11 bits)    5e-4 per view step, 1e-3 per solve;
  bf16    (single BF16)                                     5e-3 per view step, 2e-3 per solve;
  fp16    (single FP16)                                     1e-3 per view step, 1e-3 per solve.
The FP16 modes scale every operand by a power of two into FP16's range (exact) and remove
the scales in the FP32 epilogues.
"""
import os

import numpy as np
import pytest

from oracle import mesolf_ref as R
from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STEP_TOL = {"bf16x3": 1e-5, "bf16x2": 2e-3, "bf16": 5e-3, "fp16x3": 1e-5, "fp16x2": 5e-4, "fp16": 1e-3}
SOLVE_TOL = {"bf16x3": 1e-4, "bf16x2": 1e-3, "bf16": 2e-3, "fp16x3": 1e-4, "fp16x2": 1e-3, "fp16": 1e-3}
PRECS = ["bf16x3", "bf16x2", "bf16", "fp16x3", "fp16x2", "fp16"]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def to_dev(x):
    import torch
    from mesolf_gb300.api import _fortran
    return _fortran(torch.as_tensor(np.ascontiguousarray(np.asarray(x, np.float32))).cuda())[0]


CASES = [((5, 4), 61, 3), ((9, 8), 91, 2), ((6, 7), 231, 2), ((3, 3), 255, 2), ((12, 11), 61, 5)]


@pytest.mark.parametrize("lenslets,K0,Z", CASES)
@pytest.mark.parametrize("prec", PRECS)
def test_tc_forward_view(cuda, lenslets, K0, Z, prec):
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    w = synth.small_config(lenslets=lenslets, K0=K0, Z=Z)
    H, Ht = w.psf()
    Xr, Xc = w.image_shape
    rng = np.random.default_rng(K0 + Z)
    vol = rng.uniform(0.2, 1.0, (Xr, Xc, Z)).astype(np.float32)
    Hn, Htn = R.normalize_psf(H, Ht)
    Hps, _ = R.gen_phasespace_psf(Hn, Htn)
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, (Xr, Xc))
    for (u, v) in [(7, 7), (0, 14), (13, 2)]:
        hx = s.forward_view(to_dev(vol), u, v, precision=prec).cpu().numpy()
        ref = R.forward_ps(Hps[:, :, u, v, :], vol.astype(np.float64), 15)
        assert rel_l2(hx, ref) <= STEP_TOL[prec], (u, v, rel_l2(hx, ref))


@pytest.mark.parametrize("lenslets,K0,Z", CASES)
@pytest.mark.parametrize("prec", PRECS)
def test_tc_view_step(cuda, lenslets, K0, Z, prec):
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    w = synth.small_config(lenslets=lenslets, K0=K0, Z=Z)
    H, Ht = w.psf()
    LF = w.measured(H, w.volume())
    Hn, Htn = R.normalize_psf(H, Ht)
    Hps, Htc = R.gen_phasespace_psf(Hn, Htn)
    rng = np.random.default_rng(1)
    X = rng.uniform(0.5, 1.5, LF.shape + (Z,)).astype(np.float32)
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, LF.shape)
    for (u, v) in [(7, 7), (0, 0), (14, 3), (2, 12)]:
        ref = R.rl_view_step(X.astype(np.float64), LF.astype(np.float64), Hps, Htc, u, v, 0.3, 15)
        got = s.view_step(to_dev(LF), to_dev(X), u, v, 0.3, precision=prec).cpu().numpy()
        assert rel_l2(got, ref) <= STEP_TOL[prec], (u, v, rel_l2(got, ref))


@pytest.mark.parametrize("prec", PRECS)
def test_tc_config1_solve_matches_golden(cuda, prec):
    """Nnum 15, 11x11 lenslets, 21 planes, K0 61, 8 RL iterations vs the FP64 oracle."""
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    g = np.load(os.path.join(GOLD, "lf165x165x21_k61.npz"))
    H, Ht = synth.config1().psf()
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, (165, 165))
    x8 = s.run(g["lf"], 8, precision=prec)
    err = rel_l2(x8, g["x8"])
    print(f"config 1, 8 iterations, {prec}: rel L2 {err:.3e}")
    assert err <= SOLVE_TOL[prec], (prec, err)


def test_tc_solve_small_uneven(cuda):
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    w = synth.small_config(lenslets=(8, 7), K0=91, Z=5, iters=2)
    H, Ht = w.psf()
    LF = w.measured(H, w.volume())
    ref = R.recon_phase_space(LF, H, Ht, 2)
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, LF.shape)
    for prec in ("bf16x3", "bf16x2", "fp16x3", "fp16x2", "fp16"):
        got = s.run(to_dev(LF), 2, precision=prec).cpu().numpy()
        assert rel_l2(got, ref) <= SOLVE_TOL[prec], (prec, rel_l2(got, ref))
    # the FP32 path on the same solver still matches after tensor-core solves
    got = s.run(to_dev(LF), 2).cpu().numpy()
    assert rel_l2(got, ref) <= 1e-4


def test_autotuned_solve_matches_heuristic_configuration(cuda, monkeypatch):
    """The autotuner (first tensor-core solve of a work set) only changes launch parameters:
    the tuned solve equals one with the built-in heuristics (MLF_TUNE=0) up to the summation
    order of the split-K partials, and the stats report the configuration."""
    import torch
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    from mesolf_gb300.api import _fortran
    w = synth.small_config(lenslets=(20, 18), K0=61, Z=5, seed=7)
    H, Ht = w.psf()
    lf = _fortran(torch.as_tensor(np.ascontiguousarray(w.measured(H, w.volume()))).cuda())[0]
    psf = PhaseSpacePSF(H, Ht)
    a = RLSolver(psf, lf.shape)
    va = a.run(lf, 2, precision="bf16x2").cpu().numpy()
    sa = a.last_stats
    assert sa["tuned"] == 1 and sa["fwd_splits"] >= 1 and 2 <= sa["fwd_stages"] <= 4 and sa["bwd_xbufs"] in (1, 2)
    monkeypatch.setenv("MLF_TUNE", "0")
    b = RLSolver(psf, lf.shape)
    vb = b.run(lf, 2, precision="bf16x2").cpu().numpy()
    assert b.last_stats["tuned"] == 0
    assert np.linalg.norm(va - vb) / np.linalg.norm(vb) <= 1e-5
