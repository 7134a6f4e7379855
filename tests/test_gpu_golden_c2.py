"""The 1005 x 1005 x 51 workload against its FP64 oracle fixture (tests/golden/
lf1005x1005x51_k231.npz, made by make_golden_c2.py): relative L2 and max-abs error of the
solve on the fixture's sample of 131072 voxels, per precision, after 3 (and 10, when the
fixture holds it) iterations.  Bars: 1e-4 for FP32, bf16x3 and fp16x3, 1e-3 for bf16x2, fp16x2 and fp16,
2e-3 for bf16 (single BF16 operands)."""
import os

import numpy as np
import pytest

from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lf1005x1005x51_k231.npz")
BARS = {"fp32": 1e-4, "bf16x3": 1e-4, "bf16x2": 1e-3, "bf16": 2e-3, "fp16x3": 1e-4, "fp16x2": 1e-3, "fp16": 1e-3}


def errors(vol, g, it):
    ref = g[f"x{it}"].astype(np.float64)
    got = np.asarray(vol, np.float64).reshape(-1, order="F")[g["idx"]]
    return (float(np.linalg.norm(got - ref) / np.linalg.norm(ref)), float(np.abs(got - ref).max()),
            float(np.abs(ref).max()))


@pytest.fixture(scope="module")
def setup(cuda):
    if not os.path.exists(FIX):
        pytest.skip("golden fixture of the 1005 x 1005 x 51 workload not generated")
    import torch
    from mesolf_gb300 import PhaseSpacePSF, RLSolver
    from mesolf_gb300.api import _fortran
    g = dict(np.load(FIX))
    H, Ht = synth.config2().psf()
    psf = PhaseSpacePSF(H, Ht)
    s = RLSolver(psf, g["lf"].shape)
    lf = _fortran(torch.as_tensor(g["lf"].astype(np.float32)).cuda())[0]
    return g, s, lf


@pytest.mark.parametrize("prec", ["fp32", "bf16x3", "bf16x2", "bf16", "fp16x3", "fp16x2", "fp16"])
def test_against_fp64_oracle(setup, prec):
    g, s, lf = setup
    for it in (3, 10):
        if f"x{it}" not in g:
            continue
        rel, mx, peak = errors(s.run(lf, it, precision=prec, want_stats=False).cpu().numpy(), g, it)
        print(f"{prec} {it} it: rel L2 {rel:.3e}  max-abs {mx:.3e} (peak {peak:.3e})")
        assert rel <= BARS[prec], (prec, it, rel)
