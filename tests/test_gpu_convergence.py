"""The convergence monitor: mlf_stats.rel_change = ||X_k - X_(k-1)||_2 / ||X_k||_2 of the
last iteration, reduced in FP64 on the device, against the same norms taken on the host
from a 1-iteration and a 2-iteration solve of the same image (the first iteration of both is
the same computation).  Tolerance: 1e-6 relative (two FP64 sums of the same FP32 values in
different orders)."""
import numpy as np
import pytest

from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu


def to_dev(x):
    import torch
    from mesolf_gb300.api import _fortran
    t = torch.as_tensor(np.ascontiguousarray(np.asarray(x, dtype=np.float32)))
    return _fortran(t.cuda())[0]


@pytest.mark.parametrize("prec", ["fp32", "bf16x3", "bf16x2"])
def test_rel_change_matches_host_norms(cuda, prec):
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    w = synth.small_config(lenslets=(9, 8), K0=61, Z=7)
    H, Ht = w.psf()
    lf = to_dev(w.measured(H, w.volume()))
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, w.image_shape)
    x1 = s.run(lf, 1, precision=prec, want_stats=False).cpu().numpy().astype(np.float64)
    x2 = s.run(lf, 2, precision=prec, want_stats=True).cpu().numpy().astype(np.float64)
    got = s.last_stats["rel_change"]
    ref = float(np.linalg.norm(x2 - x1) / np.linalg.norm(x2))
    assert ref > 0.0
    assert abs(got - ref) <= 1e-6 * ref, (got, ref)
    # a second instrumented solve reuses the monitor buffers and gives the same value
    s.run(lf, 2, precision=prec, want_stats=True)
    assert s.last_stats["rel_change"] == got
    # no iteration: no change reported
    s.run(lf, 0, precision=prec, want_stats=True)
    assert s.last_stats["rel_change"] == 0.0


def test_rel_change_of_a_batch_covers_every_patch(cuda):
    import torch
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF
    w = synth.small_config(lenslets=(9, 8), K0=61, Z=7)
    H, Ht = w.psf()
    psf = PhaseSpacePSF(H, Ht)
    shapes = [(135, 120), (105, 150)]
    imgs = []
    for k, sh in enumerate(shapes):
        wk = synth.small_config(lenslets=(sh[0] // 15, sh[1] // 15), K0=61, Z=7, seed=k + 1)
        imgs.append(to_dev(wk.measured(H, wk.volume())))
    b = BatchSolver(psf, shapes)
    x1 = [o.cpu().numpy().astype(np.float64) for o in b.run(imgs, 1, precision="bf16x3", want_stats=False)]
    x2 = [o.cpu().numpy().astype(np.float64) for o in b.run(imgs, 2, precision="bf16x3", want_stats=True)]
    got = b.last_stats["rel_change"]
    d2 = sum(float(np.sum((a - c) ** 2)) for a, c in zip(x2, x1))
    n2 = sum(float(np.sum(a ** 2)) for a in x2)
    ref = (d2 / n2) ** 0.5
    assert abs(got - ref) <= 1e-6 * ref, (got, ref)
    b.close()
    torch.cuda.synchronize()
