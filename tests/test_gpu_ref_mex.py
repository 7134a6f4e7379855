"""The MEX projector against the reference's OWN kernel.

``oracle/refbuild.py`` compiles the reference file ``src/cuda/mex_lfm_convolution_vec.cu``
unchanged (its legacy texture fetches stood in for by plain loads) into a cubin, and
``oracle/ref_mex/ref_mex_launch.cu`` launches its ``lfm_convolution_kernel_vec`` with the
reference's launch geometry.  These tests run that kernel and this library's
``mlf_conv_vec`` on the same device inputs:

* on the reference's own MEX test input (``src/cuda/vols_slice.mat``: 376 x 376 x 77,
  extracted into ``tests/golden/vols_slice_sparse.npz``) with 241-wide PSF-like kernels,
  both routes of ``mlf_conv_vec`` equal the reference kernel to 1e-5 relative L2;
* with kernels whose first columns are not zero, outputs at ``x mod 15`` outside 1..4 equal
  the reference kernel (1e-5); at ``x mod 15`` in 1..4 the reference kernel's shared-memory
  fill overlaps itself (``oracle.mesolf_ref.mex_slot_overlap_kernels``), and its output lies
  within the bound that overlap allows around the ideal correlation this library computes.

The CPU tests pin the fixture to the statistics of the reference file and check the overlap
model.  The GPU tests skip when the cubin was not built (no reference tree where the build
ran).
"""
import os

import numpy as np
import pytest

from oracle import mesolf_ref as R

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURE = os.path.join(ROOT, "tests", "golden", "vols_slice_sparse.npz")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def load_fixture():
    d = np.load(FIXTURE)
    shape = tuple(int(s) for s in d["shape"])
    flat = np.zeros(int(np.prod(shape)), np.float32)
    flat[d["index"]] = d["value"]
    return flat.reshape(shape, order="F")


def psf_like_kernels(kw, seed, border):
    """15 x 15 Gaussian discs of radius < kw/2 - border, shifted per phase: zero in the
    first and last `border` columns and rows, as a cropped PSF is."""
    rng = np.random.default_rng(seed)
    c = (kw - 1) / 2.0
    x = np.arange(kw, dtype=np.float64)
    K = np.zeros((kw, kw, 15, 15), np.float64)
    rad = c - border - 8
    for a in range(15):
        for b in range(15):
            cx, cy = c + 0.4 * (a - 7), c + 0.4 * (b - 7)
            r2 = (x[:, None] - cx) ** 2 + (x[None, :] - cy) ** 2
            g = np.exp(-r2 / (2 * (rad / 2.5) ** 2)) * (r2 <= rad * rad)
            K[:, :, a, b] = g / g.sum() * rng.uniform(0.9, 1.1)
    assert not K[:border].any() and not K[-border:].any()
    return np.asfortranarray(K.astype(np.float32))


# ------------------------------------------------------------------------------ CPU
def test_fixture_matches_the_reference_file_statistics():
    """nnz, sum and max of src/cuda/vols_slice.mat as read from the reference tree."""
    v = load_fixture()
    assert v.shape == (376, 376, 77) and v.dtype == np.float32
    assert np.count_nonzero(v) == 72050
    assert abs(float(v.sum(dtype=np.float64)) - 3570.6109531892444) < 1e-9
    assert float(v.max()) == np.float32(1.0858954191207886)


def test_slot_overlap_model():
    rng = np.random.default_rng(3)
    K = rng.random((67, 67, 15, 15)).astype(np.float32)
    np.testing.assert_array_equal(R.mex_slot_overlap_kernels(K), K)    # kw < 68: no overlap
    K = rng.random((137, 137, 15, 15)).astype(np.float32)             # kw // 68 = 2 columns
    K2 = R.mex_slot_overlap_kernels(K)
    changed = np.argwhere(K2 != K)
    assert set(changed[:, 0]) <= {0, 1} and set(changed[:, 2]) <= {1, 2, 3, 4}
    assert K2[1, 5, 3, 7] == K[1, 6, 2, 7]                             # next row of the previous phase
    assert K2[0, 136, 2, 9] == K[0, 0, 2, 9]                           # last row: next kernel's first row
    np.testing.assert_array_equal(K2[2:], K[2:])


# ------------------------------------------------------------------------------ GPU
@pytest.fixture(scope="module")
def refmex(cuda):
    from oracle import refbuild
    try:
        return refbuild.ReferenceMex()
    except FileNotFoundError as e:
        pytest.skip(f"reference kernel not available: {e}")


def _dev(x):
    import torch
    from mesolf_gb300.api import _fortran
    return _fortran(torch.as_tensor(np.ascontiguousarray(np.asarray(x, np.float32))).cuda())[0]


def _run_ref(refmex, bm_dev, K_dev):
    import torch
    W, H = bm_dev.shape[0], bm_dev.shape[1]
    n = bm_dev.shape[2] if bm_dev.dim() == 3 else 1
    out = torch.empty_like(bm_dev)
    ms = refmex.run(bm_dev.data_ptr(), W, H, n, K_dev.data_ptr(), K_dev.shape[0], out.data_ptr())
    return out, ms


@pytest.mark.gpu
def test_reference_kernel_on_the_reference_fixture(refmex):
    """The reference's MEX input, 241-wide PSF-like kernels: the reference kernel, the direct
    route and the tensor-core route agree to 1e-5 relative L2 (and 1e-5 of the peak)."""
    import time
    import torch
    from mesolf_gb300 import mex_lfm_convolution_vec
    bm = _dev(load_fixture())
    K = _dev(psf_like_kernels(241, 0, border=8))
    ref, ref_ms = _run_ref(refmex, bm, K)
    ref = ref.cpu().numpy()
    peak = float(np.abs(ref).max())
    assert peak > 0
    for method in ("direct", "tensor", "auto"):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        got = mex_lfm_convolution_vec(bm, K, method=method)
        torch.cuda.synchronize()
        ms = 1e3 * (time.perf_counter() - t0)
        got = got.cpu().numpy()
        e = rel_l2(got, ref)
        m = float(np.abs(got - ref).max()) / peak
        print(f"vols_slice 376x376x77 kw241: {method} rel L2 {e:.2e} max {m:.2e} ({ms:.1f} ms; "
              f"reference kernel {ref_ms:.1f} ms)")
        assert e <= 1e-5 and m <= 1e-5, (method, e, m)


OVERLAP_CASES = [  # W, H, n, kw: fixture width; W > 1024 (two blocks per row); odd/even kw; kw < 68
    (376, 48, 2, 241), (1100, 40, 2, 241), (200, 90, 2, 137), (150, 100, 2, 240), (120, 80, 2, 61),
    (90, 61, 1, 341)]


@pytest.mark.gpu
@pytest.mark.parametrize("W,H,n,kw", OVERLAP_CASES)
def test_reference_kernel_slot_overlap(refmex, W, H, n, kw):
    """Dense non-negative kernels (non-zero first columns).  Outputs at x mod 15 not in 1..4
    equal the reference kernel (1e-5 relative L2 and of the peak).  At x mod 15 in 1..4 the
    reference uses, row by row, either the proper first kw//68 taps or the overlapping fill's
    (its output is deterministic only if the race always goes one way): |reference - ideal|
    stays within conv(bitmap, |K_overlap - K|), the most the overlap can move it."""
    from mesolf_gb300 import mex_lfm_convolution_vec
    rng = np.random.default_rng(W + kw)
    bm_h = rng.random((W, H, n)).astype(np.float32)
    K_h = rng.random((kw, kw, 15, 15)).astype(np.float32)
    K_alt_h = R.mex_slot_overlap_kernels(K_h)
    bm, K = _dev(bm_h), _dev(K_h)
    ref1, _ = _run_ref(refmex, bm, K)
    ref2, _ = _run_ref(refmex, bm, K)
    ref, ref2 = ref1.cpu().numpy(), ref2.cpu().numpy()
    ideal = mex_lfm_convolution_vec(bm, K, method="direct").cpu().numpy()
    alt = mex_lfm_convolution_vec(bm, _dev(K_alt_h), method="direct").cpu().numpy()
    bound = mex_lfm_convolution_vec(bm, _dev(np.abs(K_alt_h - K_h)), method="direct").cpu().numpy()
    peak = float(np.abs(ideal).max())
    aff = np.zeros((W, 1, 1), bool)
    aff[np.isin(np.arange(W) % 15, [1, 2, 3, 4])] = True
    aff = np.broadcast_to(aff, ref.shape)
    un = ~aff if kw >= 68 else np.ones_like(aff)
    e_un = rel_l2(ref[un], ideal[un])
    m_un = float(np.abs(ref[un] - ideal[un]).max()) / peak
    assert e_un <= 1e-5 and m_un <= 1e-5, (e_un, m_un)
    if kw < 68:
        return
    d = ref[aff].astype(np.float64) - ideal[aff]
    tol = 1e-5 * peak
    assert np.all(np.abs(d) <= bound[aff] * (1 + 1e-4) + tol)
    near_ideal = float(np.mean(np.abs(d) <= tol))
    near_alt = float(np.mean(np.abs(ref[aff].astype(np.float64) - alt[aff]) <= tol))
    print(f"slot overlap W{W} H{H} n{n} kw{kw}: unaffected rel L2 {e_un:.2e}; affected pixels: "
          f"{near_ideal:.3f} equal the ideal, {near_alt:.3f} equal the overlap outcome, max |ref-ideal| "
          f"{float(np.abs(d).max()) / peak:.2e} of the peak, rel L2 {rel_l2(ref[aff], ideal[aff]):.2e}; "
          f"repeat bit-identical: {bool(np.array_equal(ref, ref2))}")
