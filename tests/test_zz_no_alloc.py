"""mlf_forward_view_static: the forward projection for callers that cannot allocate device
memory (a MEX function inside MATLAB's GPU memory manager, a frame callback that must not
block on allocation).  Called through the C ABI on two calls in a row, with different views
and volumes, since every call reuses the same static scratch array, and compared with the
regular entry point (mlf_forward_view) and with the FP64 oracle's forward_ps, for tap counts
T = 3, 5, 9 and 15 (the 1005 x 1005 px image of 67 x 67 lenslets).  The device's free memory
is the same before and after a call.  Kept in its own file, collected last."""
import ctypes

import numpy as np
import pytest

from mesolf_gb300 import synth
from oracle import mesolf_ref as R

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


CASES = [  # lenslets, K0 (-> T = S/15), Z
    ((9, 7), 91, 4), ((5, 6), 61, 3), ((8, 8), 151, 2), ((67, 67), 231, 2)]


@pytest.mark.parametrize("lenslets,K0,Z", CASES)
def test_static_forward_matches_regular_entry_point_and_oracle(cuda, lenslets, K0, Z):
    import torch
    from mesolf_gb300 import PhaseSpacePSF, RLSolver, _lib
    from mesolf_gb300.api import _fortran
    lib = _lib.load()
    w = synth.small_config(lenslets=lenslets, K0=K0, Z=Z)
    H, Ht = w.psf()
    Xr, Xc = w.image_shape
    psf = PhaseSpacePSF(H, Ht)
    solver = RLSolver(psf, (Xr, Xc))
    rng = np.random.default_rng(K0 + Z)
    stream = torch.cuda.current_stream().cuda_stream
    for k, ((u, v), seed) in enumerate([((3, 11), 1), ((7, 7), 2)]):
        vol = rng.random((Xr, Xc, Z)).astype(np.float32) + seed
        vd = _fortran(torch.as_tensor(np.ascontiguousarray(vol)).cuda())[0]
        ref = solver.forward_view(vd, u, v).cpu().numpy()
        hx = torch.full((Xc // 15, Xr // 15), float("nan"), dtype=torch.float32, device="cuda").t()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = lib.mlf_forward_view_static(psf.handle, ctypes.c_void_p(vd.data_ptr()), Xr, Xc, u, v,
                                         ctypes.c_void_p(hx.data_ptr()), ctypes.c_void_p(stream))
        _lib.check(st)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        got = hx.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_l2(got, ref) <= 1e-5, (u, v, rel_l2(got, ref))
        h_uv, _ = R.phasespace_view(H, Ht, u, v)
        oracle = R.forward_ps(h_uv, vol, 15)
        assert rel_l2(got, oracle) <= 1e-5, (u, v, rel_l2(got, oracle))
        if k > 0:   # the first call may load the library's device code
            assert free_after == free_before
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
    # the per-CTA tile limit, ceil(Li/4) * ceil(Lj/8) <= 256, is checked before any access:
    # 64 x 128 lenslets need 16 * 16 = 256 tiles (the most allowed), 65 x 128 need 17 * 16
    assert lib.mlf_forward_view_static(psf.handle, p, 133 * 15, 133 * 15, 0, 0, p, None) == _lib.MLF_ERR_UNSUPPORTED
    assert lib.mlf_forward_view_static(psf.handle, p, 65 * 15, 128 * 15, 0, 0, p, None) == _lib.MLF_ERR_UNSUPPORTED
    psf.close()
