"""Batched tensor-core solve of independent patches (uneven lenslet counts and plane ranges of
one shared PSF) against single solves and the FP64 oracle.

A patch using planes [z0, z0+nz) of the batch PSF must reproduce a single solve with the PSF
cut to those planes: tolerance 1e-4 relative L2 between the two GPU solves at the same
precision (they differ only in FP32 summation order), and the oracle bars of the mode.
"""
import numpy as np
import pytest

from oracle import mesolf_ref as R
from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def to_dev(x):
    import torch
    from mesolf_gb300.api import _fortran
    return _fortran(torch.as_tensor(np.ascontiguousarray(np.asarray(x, np.float32))).cuda())[0]


LENS = [(5, 4), (7, 6), (3, 8)]
PLANES = [(0, 7), (2, 4), (1, 5)]


def _patches(seed=0, K0=61, Z=7):
    H, Ht = synth.make_psf(K0, 15, np.arange(Z) - Z // 2, seed=seed)
    lfs = []
    for k, ((li, lj), (z0, nz)) in enumerate(zip(LENS, PLANES)):
        w = synth.small_config(lenslets=(li, lj), K0=K0, Z=nz, seed=seed + k)
        vol = w.volume()
        lfs.append(w.measured(H[:, :, :, :, z0:z0 + nz], vol))
    return H, Ht, lfs


@pytest.mark.parametrize("prec", ["bf16x2", "bf16x3", "fp16x2"])
def test_batch_matches_single_solves(cuda, prec):
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF, RLSolver
    H, Ht, lfs = _patches()
    psf = PhaseSpacePSF(H, Ht)
    shapes = [lf.shape for lf in lfs]
    b = BatchSolver(psf, shapes, PLANES)
    outs = [o.cpu().numpy() for o in b.run([to_dev(lf) for lf in lfs], 2, precision=prec)]
    assert b.last_stats["n_views"] > 0
    for k, (lf, (z0, nz)) in enumerate(zip(lfs, PLANES)):
        sub = PhaseSpacePSF(np.asfortranarray(H[:, :, :, :, z0:z0 + nz]), np.asfortranarray(Ht[:, :, :, :, z0:z0 + nz]))
        s = RLSolver(sub, lf.shape)
        single = s.run(to_dev(lf), 2, precision=prec).cpu().numpy()
        assert outs[k].shape == single.shape == lf.shape + (nz,)
        assert rel_l2(outs[k], single) <= 1e-4, (k, rel_l2(outs[k], single))
        s.close()
        sub.close()


def test_batch_patch_matches_oracle(cuda):
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF
    H, Ht, lfs = _patches(seed=3)
    psf = PhaseSpacePSF(H, Ht)
    b = BatchSolver(psf, [lf.shape for lf in lfs], PLANES)
    outs = [o.cpu().numpy() for o in b.run([to_dev(lf) for lf in lfs], 2, precision="bf16x3")]
    for k in (1, 2):
        z0, nz = PLANES[k]
        ref = R.recon_phase_space(lfs[k], H[:, :, :, :, z0:z0 + nz], Ht[:, :, :, :, z0:z0 + nz], 2)
        assert rel_l2(outs[k], ref) <= 1e-4, (k, rel_l2(outs[k], ref))


def test_batch_order_independent_and_warm_start(cuda):
    """Each patch's result is the same alone-in-a-batch, in the mix, and in another order."""
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF
    H, Ht, lfs = _patches(seed=5)
    psf = PhaseSpacePSF(H, Ht)
    mix = BatchSolver(psf, [lf.shape for lf in lfs], PLANES)
    o_mix = [o.cpu().numpy() for o in mix.run([to_dev(lf) for lf in lfs], 2)]
    order = [2, 0, 1]
    rev = BatchSolver(psf, [lfs[k].shape for k in order], [PLANES[k] for k in order])
    o_rev = [o.cpu().numpy() for o in rev.run([to_dev(lfs[k]) for k in order], 2)]
    for j, k in enumerate(order):
        assert rel_l2(o_rev[j], o_mix[k]) <= 1e-5
        alone = BatchSolver(psf, [lfs[k].shape], [PLANES[k]])
        o_alone = alone.run([to_dev(lfs[k])], 2)[0].cpu().numpy()
        assert rel_l2(o_alone, o_mix[k]) <= 1e-5
    # warm start from the previous result: one more iteration equals continuing the solve
    o_w = [o.cpu().numpy() for o in mix.run([to_dev(lf) for lf in lfs], 1,
                                             warm=[to_dev(o) for o in o_mix])]
    assert all(np.isfinite(o).all() for o in o_w)


def test_batch_rejects_bad_arguments(cuda):
    from mesolf_gb300 import BatchSolver, MesoLFError, PhaseSpacePSF
    H, Ht, _ = _patches()
    psf = PhaseSpacePSF(H, Ht)
    with pytest.raises(MesoLFError):
        BatchSolver(psf, [(75, 60)], [(5, 4)])       # planes beyond the PSF
    with pytest.raises(MesoLFError):
        BatchSolver(psf, [(74, 60)], [(0, 7)])       # not a multiple of Nnum
    b = BatchSolver(psf, [(75, 60)], [(0, 7)])
    with pytest.raises(MesoLFError):
        b.run([to_dev(np.ones((75, 60)))], 1, precision="fp32")
