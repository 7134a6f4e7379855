"""Frame rectification (image_load_module_aug.m) on the GPU against the FP64 oracle
``image_load``.  Tolerance: relative L2 1e-6 and max-abs 1e-5 on the normalised movie
(FP32 bilinear weights and sums of integer frames)."""
import numpy as np
import pytest

from oracle import mesolf_ref as R
from mesolf_gb300 import rectify as RC

pytestmark = pytest.mark.gpu

SI0 = dict(Nnum=15, frames_dx=15.27, frames_x_offset=512.3, frames_y_offset=498.6,
           frames_crop_border_microlenses=[1, 1, 1, 1], patch_mode="carpet", n_patches=2)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def frames_u16(shape, n, seed):
    rng = np.random.default_rng(seed)
    base = rng.random(shape) * 3000
    return np.stack([(base + 500 * rng.random(shape)).astype(np.uint16) for _ in range(n)], axis=2)


@pytest.mark.parametrize("sel", [
    dict(),                                                   # defaults: every frame
    dict(frames_start=2, frames_step=3, frames_end=11),       # groups of 3, last group short
    dict(frames_start=1, frames_step=2, frames_average=False),
])
@pytest.mark.parametrize("dtype", ["u16", "f32"])
@pytest.mark.parametrize("shape", [(1024, 1040), (1023, 1041)])  # frames 16-byte aligned, or not
def test_image_load_matches_oracle(cuda, sel, dtype, shape):
    SI = dict(SI0, **sel)
    frames = frames_u16(shape, 12, seed=3)
    if dtype == "f32":
        frames = frames.astype(np.float32) * np.float32(0.37)
    infos = RC.determine_patch_info_aug(SI, frames.shape[:2])
    for info in infos[:2]:
        got = RC.image_load_module_aug(info, SI, frames)
        ref = R.image_load(frames, info, SI)
        assert got.shape == ref.shape
        assert rel_l2(got, ref) <= 1e-6 and np.abs(got - ref).max() <= 1e-5


def test_device_frames_and_rectify_mod(cuda):
    import torch
    frames = frames_u16((700, 650), 5, seed=4).astype(np.float32)
    info = RC.determine_patch_info_aug(dict(SI0, frames_x_offset=300.7, frames_y_offset=333.1), frames.shape[:2])[0]
    host = RC.image_load_module_aug(info, SI0, frames)
    dev_frames = torch.as_tensor(np.ascontiguousarray(frames.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
    dev = RC.image_load_module_aug(info, SI0, dev_frames)
    assert dev.is_cuda and np.array_equal(dev.cpu().numpy(), host)
    img = frames[:, :, 0].astype(np.float64)
    got = RC.img_rectify_mod(img, 7.3, 6.9, 15, 15.27)
    ref = R.img_rectify_mod(img, 7.3, 6.9, 15, 15.27)
    assert got.shape == ref.shape and rel_l2(got, ref) <= 1e-6


def test_shape_mismatch_raises(cuda):
    from mesolf_gb300._lib import MesoLFError
    frames = frames_u16((600, 600), 2, seed=5)
    info = RC.determine_patch_info_aug(dict(SI0, frames_x_offset=300.0, frames_y_offset=300.0), (600, 600))[0]
    bad = dict(info, size=(info["size"][0] + 15, info["size"][1]))
    with pytest.raises(MesoLFError, match="shape is different"):
        RC.image_load_module_aug(bad, SI0, frames)


def test_rectified_movie_feeds_summary_image(cuda):
    """The unnormalised movie gives the same summary image as the normalised one (the summary
    divides by the movie maximum itself)."""
    import torch
    from mesolf_gb300.api import summary_image
    rng = np.random.default_rng(6)
    frames = (rng.random((500, 520, 64)) * 2000).astype(np.uint16)
    info = RC.determine_patch_info_aug(dict(SI0, frames_x_offset=250.2, frames_y_offset=240.8), (500, 520))[0]
    dev = torch.as_tensor(np.ascontiguousarray(frames.transpose(2, 1, 0)).astype(np.float32)).cuda().permute(2, 1, 0)
    a = RC.image_load_module_aug(info, SI0, dev)
    b = RC.image_load_module_aug(info, SI0, dev, normalize=False)
    ia, _, _ = summary_image(a, "pixelwise", 2, 20, 5, 3)
    ib, _, _ = summary_image(b, "pixelwise", 2, 20, 5, 3)
    assert rel_l2(ia.cpu().numpy(), ib.cpu().numpy()) <= 1e-5
