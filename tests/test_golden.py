"""Committed golden fixtures (tests/golden, made by make_golden.py from the FP64 oracle).

CPU: the oracle reproduces its own fixtures (guards against oracle / generator drift).
GPU: the CUDA path reproduces the fixtures through the C ABI within 1e-4 relative L2.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import mesolf_ref as R
from mesolf_gb300 import synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def load(name):
    return np.load(os.path.join(GOLD, name))


def test_manifest_hashes():
    man = json.load(open(os.path.join(GOLD, "manifest.json")))
    for name, digest in man.items():
        assert hashlib.sha256(open(os.path.join(GOLD, name), "rb").read()).hexdigest() == digest


def test_generator_matches_fixture():
    g = load("lf165x165x21_k61.npz")
    H, _ = synth.config1().psf()
    assert abs(H.astype(np.float64).sum() - float(g["psf_sum"])) <= 1e-9 * float(g["psf_sum"])


def test_oracle_reproduces_config1_two_iterations():
    g = load("lf165x165x21_k61.npz")
    H, Ht = synth.config1().psf()
    snaps = {}
    R.recon_phase_space(g["lf"], H, Ht, 2, callback=lambda it, X: snaps.__setitem__(it + 1, X))
    assert rel_l2(snaps[2], g["x2"]) <= 1e-6
    Hn, Htn = R.normalize_psf(H, Ht)
    Hps, _ = R.gen_phasespace_psf(Hn, Htn)
    np.testing.assert_allclose(R.view_weights(Hps), g["weights"], rtol=1e-9, atol=1e-12)


def test_oracle_reproduces_view_fixture():
    g = load("small_views.npz")
    H, Ht = synth.small_config(lenslets=(5, 4), K0=61, Z=3).psf()
    Hn, Htn = R.normalize_psf(H, Ht)
    Hps, Htc = R.gen_phasespace_psf(Hn, Htn)
    for k, (u, v) in enumerate(g["views"]):
        assert rel_l2(R.forward_ps(Hps[:, :, u, v, :], g["vol64"], 15), g["fwd"][k]) <= 1e-6
        assert rel_l2(R.backward_ps(Htc[:, :, u, v, :], g["proj64"], u, v, 15), g["bwd"][k]) <= 1e-6


@pytest.mark.gpu
def test_gpu_config1_eight_iterations_match_golden(cuda):
    """Config 'Nnum 15, 11x11 lenslets, 21 planes, K0 61', 8 FP32 RL iterations."""
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    g = load("lf165x165x21_k61.npz")
    H, Ht = synth.config1().psf()
    psf = PhaseSpacePSF(H, Ht)
    np.testing.assert_allclose(psf.weights, g["weights"], rtol=1e-9, atol=1e-12)
    s = RLSolver(psf, (165, 165))
    x8 = s.run(g["lf"], 8)
    assert x8.shape == (165, 165, 21)
    err = rel_l2(x8, g["x8"])
    assert err <= 1e-4, err
    x2 = s.run(g["lf"], 2)
    assert rel_l2(x2, g["x2"]) <= 1e-4


@pytest.mark.gpu
def test_gpu_views_match_fixture(cuda):
    import torch
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    from mesolf_gb300.api import _fortran
    g = load("small_views.npz")
    H, Ht = synth.small_config(lenslets=(5, 4), K0=61, Z=3).psf()
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, (75, 60))
    vol = _fortran(torch.as_tensor(np.ascontiguousarray(g["vol"])).cuda())[0]
    proj = _fortran(torch.as_tensor(np.ascontiguousarray(g["proj"])).cuda())[0]
    for k, (u, v) in enumerate(g["views"]):
        assert rel_l2(s.forward_view(vol, u, v).cpu().numpy(), g["fwd"][k]) <= 1e-5
        assert rel_l2(s.backward_view(proj, u, v).cpu().numpy(), g["bwd"][k]) <= 1e-5
