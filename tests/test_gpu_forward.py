"""Full light-field forward projection (forwardProjectGPU.m semantics) on the GPU against
the FP64 oracle ``forward_project_full``.

Tolerances (relative L2 against the oracle): 1e-5 for FP32 and for the tensor-core form
with both operands split (bf16x3); 2e-3 with the taps in single BF16 (bf16x2, bf16).
"""
import numpy as np
import pytest

from oracle import mesolf_ref as R
from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-5, "bf16x3": 1e-5, "bf16x2": 2e-3, "bf16": 2e-3}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def to_dev(x):
    import torch
    from mesolf_gb300.api import _fortran
    return _fortran(torch.as_tensor(np.ascontiguousarray(np.asarray(x, np.float32))).cuda())[0]


@pytest.mark.parametrize("prec", ["fp32", "bf16x3", "bf16x2", "bf16"])
@pytest.mark.parametrize("raw", [True, False])
def test_forward_project_matches_oracle(cuda, prec, raw):
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    w = synth.small_config(lenslets=(5, 4), K0=61, Z=5, seed=2)
    H, Ht = w.psf()
    vol = w.volume()
    Href = H if raw else R.normalize_psf(H, Ht)[0]
    ref = R.forward_project_full(Href, vol)
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, vol.shape[:2])
    lf = s.forward_project(to_dev(vol), raw_psf=raw, precision=prec).cpu().numpy()
    assert lf.shape == ref.shape
    assert rel_l2(lf, ref) <= TOL[prec], rel_l2(lf, ref)


def test_batch_forward_project_matches_single(cuda):
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF, RLSolver
    H, Ht = synth.make_psf(61, 15, np.arange(7) - 3, seed=4)
    psf = PhaseSpacePSF(H, Ht)
    shapes, planes = [(75, 60), (45, 105), (30, 30)], [(0, 7), (2, 3), (1, 5)]
    vols = [synth.make_volume(a, b, nz, 10, 3.0, "uniform", 0.01, seed=k)
            for k, ((a, b), (_, nz)) in enumerate(zip(shapes, planes))]
    b = BatchSolver(psf, shapes, planes)
    outs = [o.cpu().numpy() for o in b.forward_project([to_dev(v) for v in vols], precision="bf16x3")]
    for k, ((z0, nz), v) in enumerate(zip(planes, vols)):
        ref = R.forward_project_full(H[:, :, :, :, z0:z0 + nz], v)
        assert rel_l2(outs[k], ref) <= 1e-5, (k, rel_l2(outs[k], ref))


def test_forward_project_after_solve_on_same_solver(cuda):
    """The FP32 projector's staging buffer is also the filter's scratch; projecting after
    a solve on the same context must give the same image as on a fresh one."""
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    w = synth.small_config(lenslets=(5, 4), K0=61, Z=5, seed=6)
    H, Ht = w.psf()
    vol = w.volume()
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, vol.shape[:2])
    fresh = s.forward_project(to_dev(vol)).cpu().numpy()
    s.run(to_dev(w.measured(H, vol)), 1)
    again = s.forward_project(to_dev(vol)).cpu().numpy()
    hx = s.forward_view(to_dev(vol), 3, 11).cpu().numpy()
    norm = s.forward_project(to_dev(vol), raw_psf=False).cpu().numpy()
    assert np.array_equal(fresh, again)
    assert np.array_equal(hx, norm[3::15, 11::15])


def test_reference_projector_mirrors(cuda):
    """forwardProjectGPU / forwardProjectACC / forwardProjectGPU_discrete /
    forwardProjectGPU_skip_2D against their FP64 restatements (relative L2 1e-5, FP32)."""
    from mesolf_gb300 import (forwardProjectACC, forwardProjectGPU, forwardProjectGPU_discrete,
                              forwardProjectGPU_skip_2D)
    w = synth.small_config(lenslets=(5, 4), K0=61, Z=5, seed=8)
    H, _ = w.psf()
    vol = w.volume()
    assert rel_l2(forwardProjectGPU(H, vol), R.forward_project_full(H, vol)) <= 1e-5
    CA = [(31 - r, 31 + r) for r in (30, 20, 4, 6, 30)]       # centred crops (1-based), some cut the support
    got = forwardProjectACC(H, vol, CA)
    assert rel_l2(got, R.forward_project_full(H, vol, CA)) <= 1e-5
    ua = [2, 2, 3, 5, 1, 3]
    v6 = np.concatenate([vol, vol[:, :, :1] * 0.5], axis=2)
    got = forwardProjectGPU_discrete(H, v6, ua, 41)
    assert rel_l2(got, R.forward_project_discrete(H, v6, ua, 41)) <= 1e-5
    got = forwardProjectGPU_skip_2D(H, vol[:, :, 2], 3, 4)
    assert rel_l2(got, R.forward_project_skip_2d(H, vol[:, :, 2], 3, 4)) <= 1e-5
