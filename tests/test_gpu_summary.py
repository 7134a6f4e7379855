"""Summary image (summary_image_generation_module.m) on the GPU against the FP64 oracle
``summary_image``.

Tolerances (relative L2 against the oracle): summary image 1e-4 (FP32 movie, sliding window
sums with a compensated window-1 sum); rank-1 backgrounds 1e-5.
"""
import numpy as np
import pytest

from oracle import mesolf_ref as R
from mesolf_gb300 import synth

pytestmark = pytest.mark.gpu

TOL_IMG, TOL_BG = 1e-4, 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("P,T,w1,w2,poly,it", [
    (4096, 500, 100, 20, 3, 5),     # reference defaults; float4 paths
    (1001, 333, 100, 20, 3, 2),     # P % 4 != 0: scalar paths
    (640, 97, 150, 40, 2, 1),       # windows longer than the movie
    (512, 64, 300, 5, 3, 3),        # window 1 of more than 2T frames: the global mean
    (300, 50, 3, 1, 1, 1),          # unit window 2, power 1
    (256, 41, 4, 6, 3, 2),          # even windows
    (96, 1, 100, 20, 3, 1),         # one frame
    (2048, 700, 60, 10, 4, 2),      # power 4 (runtime power), bulk steps
    (1500, 1000, 33, 7, 2, 1),      # odd windows, power 2
    (1000, 400, 500, 100, 3, 1),    # long windows: 64 pixels per block
    (500, 600, 1000, 200, 3, 1),    # longer windows: 32 pixels per block, one per thread
    (700, 90, 30, 8, 0, 1),         # power 0: a constant series, zero image
])
def test_pixelwise_matches_oracle(cuda, P, T, w1, w2, poly, it):
    from mesolf_gb300.api import summary_image
    Y = synth.sensor_movie(P, T, seed=P + T)
    img, s, t = summary_image(Y, "pixelwise", it, w1, w2, poly)
    ri, rs, rt = R.summary_image(Y, "pixelwise", it, w1, w2, poly)
    if np.isfinite(ri).all():
        assert rel_l2(img, ri) <= TOL_IMG
    else:  # one frame or power 0: a zero image, 0/0 as in MATLAB
        assert np.isnan(img).all()
    assert rel_l2(s, rs) <= TOL_BG
    assert rel_l2(t, rt) <= TOL_BG


@pytest.mark.parametrize("P,T,it", [(4096, 300, 5), (999, 120, 1)])
def test_global_matches_oracle(cuda, P, T, it):
    from mesolf_gb300.api import summary_image
    Y = synth.sensor_movie(P, T, seed=7)
    img, s, t = summary_image(Y, "global", it)
    ri, rs, rt = R.summary_image(Y, "global", it)
    assert rel_l2(img, ri) <= TOL_IMG
    assert rel_l2(s, rs) <= TOL_BG
    assert rel_l2(t, rt) <= TOL_BG


def test_module_signature_and_device_inputs(cuda):
    """The reference-named module on a (h, w, T) movie, host and device, same results."""
    import torch
    from mesolf_gb300.api import summary_image_generation_module
    h, w, T = 48, 40, 200
    Y = synth.sensor_movie(h * w, T, seed=3)
    mov3 = np.asfortranarray(Y.reshape((h, w, T), order="F"))
    SI = {"detrend_mode": "pixelwise", "bg_iter": 3, "pixelwise_window_1": 50}
    img, bs, bt = summary_image_generation_module(mov3, {"size": (h, w)}, SI)
    assert img.shape == (h, w) and bs.shape == (h, w) and bt.shape == (1, T)
    ri, rs, rt = R.summary_image(Y, "pixelwise", 3, 50, 20, 3)
    assert rel_l2(img.reshape(-1, order="F"), ri) <= TOL_IMG
    assert rel_l2(bs.reshape(-1, order="F"), rs) <= TOL_BG
    d = torch.as_tensor(np.ascontiguousarray(mov3.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
    dimg, dbs, dbt = summary_image_generation_module(d, {"size": (h, w)}, SI)
    assert dimg.is_cuda and tuple(dimg.shape) == (h, w)
    assert np.array_equal(dimg.cpu().numpy(), img)
    assert np.array_equal(dbs.cpu().numpy(), bs) and np.array_equal(dbt.cpu().numpy().reshape(1, T), bt)


def test_full_size_properties(cuda):
    """A 1005 x 1005-pixel, 400-frame movie built on the device: the temporal background has
    unit norm, the summary image lies in [0, 1] with maximum 1, results repeat bit for bit,
    and a pixel sample matches the oracle run on those pixels' series alone (the pixelwise
    image before normalisation depends only on the pixel's own series and the movie max)."""
    import torch
    from mesolf_gb300.api import summary_image
    P, T = 1005 * 1005, 400
    Y = synth.sensor_movie(P, T, seed=11, device="cuda")
    img, s, t = summary_image(Y, "pixelwise", 5, 100, 20, 3)
    img2, s2, t2 = summary_image(Y, "pixelwise", 5, 100, 20, 3)
    assert torch.equal(img, img2) and torch.equal(s, s2) and torch.equal(t, t2)
    assert abs(float(torch.linalg.vector_norm(t.double())) - 1.0) < 1e-6
    assert float(img.min()) >= 0.0 and float(img.max()) == 1.0
    idx = torch.arange(0, P, 9973, device="cuda")
    Ys = Y[idx].cpu().numpy().astype(np.float64)
    M = float(Y.max())
    y = Ys / M
    z = R.movmean(y - R.movmean(y, 100, axis=1), 20, axis=1) ** 3
    ref = R.compute_std_image(z)
    got = img[idx].double().cpu().numpy()
    scale = float(np.dot(got, ref) / np.dot(ref, ref))  # the image max comes from other pixels
    assert rel_l2(got / scale, ref) <= TOL_IMG
