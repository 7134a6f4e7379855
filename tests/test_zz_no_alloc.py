"""mlf_forward_view_static: the forward projection for callers that cannot allocate device
memory (a MEX function inside MATLAB's GPU memory manager, a frame callback that must not
block on allocation).  Called through the C ABI and compared with the regular entry point
(mlf_forward_view) on two calls in a row, with different views and volumes, since every
call reuses the same static scratch array.  Kept in its own file, collected last."""
import ctypes

import numpy as np
import pytest

from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_static_forward_matches_regular_entry_point(cuda):
    import torch
    from mesolf_gb300 import PhaseSpacePSF, RLSolver, _lib
    from mesolf_gb300.api import _fortran
    lib = _lib.load()
    w = synth.small_config(lenslets=(9, 7), K0=91, Z=4)
    H, Ht = w.psf()
    Xr, Xc = w.image_shape
    psf = PhaseSpacePSF(H, Ht)
    solver = RLSolver(psf, (Xr, Xc))
    rng = np.random.default_rng(5)
    stream = torch.cuda.current_stream().cuda_stream
    for (u, v), seed in [((3, 11), 1), ((7, 7), 2)]:
        vol = rng.random((Xr, Xc, w.Z)).astype(np.float32) + seed
        vd = _fortran(torch.as_tensor(np.ascontiguousarray(vol)).cuda())[0]
        ref = solver.forward_view(vd, u, v).cpu().numpy()
        hx = torch.full((Xc // 15, Xr // 15), float("nan"), dtype=torch.float32, device="cuda").t()
        st = lib.mlf_forward_view_static(psf.handle, ctypes.c_void_p(vd.data_ptr()), Xr, Xc, u, v,
                                         ctypes.c_void_p(hx.data_ptr()), ctypes.c_void_p(stream))
        _lib.check(st)
        torch.cuda.synchronize()
        got = hx.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_l2(got, ref) <= 1e-5, (u, v, rel_l2(got, ref))
    solver.close()
    psf.close()


def test_static_forward_rejects_bad_arguments(cuda):
    import torch
    from mesolf_gb300 import PhaseSpacePSF, _lib
    lib = _lib.load()
    H, Ht = synth.small_config(lenslets=(3, 3), K0=61, Z=2).psf()
    psf = PhaseSpacePSF(H, Ht)
    buf = torch.zeros(45 * 45 * 2, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    assert lib.mlf_forward_view_static(psf.handle, p, 44, 45, 0, 0, p, None) == _lib.MLF_ERR_INVALID
    assert lib.mlf_forward_view_static(psf.handle, p, 45, 45, 15, 0, p, None) == _lib.MLF_ERR_INVALID
    host = np.zeros(4, np.float32)
    assert lib.mlf_forward_view_static(psf.handle, host.ctypes.data, 45, 45, 0, 0, p, None) == _lib.MLF_ERR_INVALID
    psf.close()
