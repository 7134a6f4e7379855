"""Race check by repetition: plain FP32 solves enqueued back to back without synchronising
(and behind a busy GPU) must be bit-identical to a synchronised solve.  The FP32 path has a
fixed summation order everywhere, so any difference is a race (this caught a missing barrier
between the first channel's tap load and the D-table row sums in the view kernel)."""
import numpy as np
import pytest

from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu


def test_async_fp32_solves_are_bit_identical(cuda):
    import torch
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    from mesolf_gb300.api import _fortran
    w = synth.small_config(lenslets=(67, 67), K0=231, Z=12, iters=2, seed=3)
    H, Ht = w.psf()
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, w.image_shape)
    lf = _fortran(torch.as_tensor(np.ascontiguousarray(w.measured(H, w.volume(), device="cuda"))).cuda())[0]
    base = s.run(lf, 2, want_stats=False).cpu().numpy()
    torch.cuda.synchronize()
    outs = [s.run(lf, 2, want_stats=False) for _ in range(8)]
    for _ in range(4):
        torch.cuda._sleep(50_000_000)        # the next solve is enqueued behind a busy GPU
        outs.append(s.run(lf, 2, want_stats=False))
    bad = [k for k, o in enumerate(outs) if not np.array_equal(o.cpu().numpy(), base)]
    assert not bad, f"solves {bad} differ from the synchronised one"
    s.close()
    psf.close()
