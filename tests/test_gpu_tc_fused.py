"""The fused tensor-core view step (back projection + update of view k and the forward GEMM
of view k+1 in one launch, k_tc_bwdfwd) against the two-kernel form (k_tc_bwd + k_tc_fwd,
selected with MLF_FUSED=0).  The fused kernel keeps the forward GEMM's split boundaries and
K-step order, so the solves are bit-identical; it launches one kernel fewer per view step.
The autotuner is off (MLF_TUNE=0) so that both solves use the same launch configuration;
both buffer layouts of the fused kernel are covered (MLF_FUSED_XB).
Shapes: one 128-channel tile per split (9 x 8 lenslets, 7 planes), several tiles per split
and several position tiles (20 x 18, 6 planes), and the 67 x 67 lenslet patch (3 planes)."""
import numpy as np
import pytest

from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = [((9, 8), 91, 7), ((20, 18), 61, 6), ((67, 67), 231, 3)]


def to_dev(x):
    import torch
    from mesolf_gb300.api import _fortran
    return _fortran(torch.as_tensor(np.ascontiguousarray(np.asarray(x, np.float32))).cuda())[0]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("lenslets,K0,Z", CASES)
@pytest.mark.parametrize("prec", ["bf16x2", "bf16"])
@pytest.mark.parametrize("xb", ["2", "1"])  # two X buffers and a 2-stage ring, or one and three
def test_fused_solve_equals_two_kernel_solve(cuda, monkeypatch, lenslets, K0, Z, prec, xb):
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    monkeypatch.setenv("MLF_TUNE", "0")
    monkeypatch.setenv("MLF_FUSED_XB", xb)
    w = synth.small_config(lenslets=lenslets, K0=K0, Z=Z)
    H, Ht = w.psf()
    Xr, Xc = w.image_shape
    rng = np.random.default_rng(K0 + Z)
    lf = to_dev(rng.uniform(50.0, 150.0, (Xr, Xc)).astype(np.float32))
    psf = PhaseSpacePSF(H, Ht)
    vols, launches = {}, {}
    for fused in ("1", "0"):
        monkeypatch.setenv("MLF_FUSED", fused)
        s = RLSolver(psf, (Xr, Xc))
        vols[fused] = s.run(lf, 3, precision=prec).cpu().numpy()
        launches[fused] = s.last_stats["kernel_launches"]
        s.close()
    psf.close()
    assert np.isfinite(vols["1"]).all() and vols["1"].max() > 0
    assert launches["1"] < launches["0"], launches          # the fused path ran
    assert np.array_equal(vols["1"], vols["0"]), rel_l2(vols["1"], vols["0"])


def test_fused_batch_equals_two_kernel_batch(cuda, monkeypatch):
    """Uneven patches and plane ranges in one work set: tiles of a patch outside its planes
    and splits without K-steps of a patch (zero partials) take the fused kernel's skip
    paths."""
    from mesolf_gb300 import BatchSolver, PhaseSpacePSF
    monkeypatch.setenv("MLF_TUNE", "0")
    w = synth.small_config(lenslets=(12, 10), K0=61, Z=6)
    H, Ht = w.psf()
    psf = PhaseSpacePSF(H, Ht)
    shapes = [(15 * 12, 15 * 10), (15 * 9, 15 * 11), (15 * 14, 15 * 9)]
    planes = [(0, 6), (1, 3), (2, 4)]
    rng = np.random.default_rng(5)
    lfs = [to_dev(rng.uniform(50.0, 150.0, s).astype(np.float32)) for s in shapes]
    outs = {}
    for fused in ("1", "0"):
        monkeypatch.setenv("MLF_FUSED", fused)
        b = BatchSolver(psf, shapes, planes)
        outs[fused] = [o.cpu().numpy() for o in b.run(lfs, 2, precision="bf16x2")]
        b.close()
    psf.close()
    for a, c in zip(outs["1"], outs["0"]):
        assert np.isfinite(a).all()
        assert np.array_equal(a, c), rel_l2(a, c)
