"""torch.ops.mesolf.* registrations: output shapes through the fake implementations (CPU),
and results equal to the Python entry points on the GPU."""
import numpy as np
import pytest
import torch

import mesolf_gb300.torch_ops  # noqa: F401  (registers the ops)
from mesolf_gb300 import synth


def test_ops_registered_with_shapes():
    from torch._subclasses.fake_tensor import FakeTensorMode
    with FakeTensorMode():
        bm = torch.empty(40, 30, 2)
        K = torch.empty(7, 7, 15, 15)
        assert torch.ops.mesolf.conv_vec(bm, K).shape == (40, 30, 2)
        lf = torch.empty(75, 60)
        H = torch.empty(61, 61, 15, 15, 5)
        assert torch.ops.mesolf.rl_solve(lf, H, H, 2, "fp32").shape == (75, 60, 5)
        outs = torch.ops.mesolf.rl_solve_batch([lf, torch.empty(45, 30)], H, H, [0, 1], [5, 3], 2, "bf16x2")
        assert [tuple(o.shape) for o in outs] == [(75, 60, 5), (45, 30, 3)]


@pytest.mark.gpu
def test_ops_match_entry_points(cuda):
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF, RLSolver, mex_lfm_convolution_vec
    rng = np.random.default_rng(1)
    bm = torch.as_tensor(rng.random((40, 33, 2), dtype=np.float32)).cuda()
    K = torch.as_tensor(rng.random((9, 9, 15, 15), dtype=np.float32)).cuda()
    assert torch.equal(torch.ops.mesolf.conv_vec(bm, K), mex_lfm_convolution_vec(bm, K).contiguous())
    w = synth.small_config(lenslets=(5, 4), K0=61, Z=5)
    H, Ht = w.psf()
    lf = torch.as_tensor(np.ascontiguousarray(w.measured(H, w.volume()))).cuda()
    Hd, Htd = torch.as_tensor(np.ascontiguousarray(H)).cuda(), torch.as_tensor(np.ascontiguousarray(Ht)).cuda()
    got = torch.ops.mesolf.rl_solve(lf, Hd, Htd, 2, "fp32")
    psf = PhaseSpacePSF(H, Ht)
    ref = RLSolver(psf, tuple(lf.shape)).run(lf, 2)
    assert torch.equal(got, ref.contiguous())
    outs = torch.ops.mesolf.rl_solve_batch([lf], Hd, Htd, [0], [5], 2, "bf16x2")
    refb = BatchSolver(psf, [tuple(lf.shape)]).run([lf], 2)
    assert torch.equal(outs[0], refb[0].contiguous())
