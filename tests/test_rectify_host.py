"""Rectification host logic and its oracle (CPU): the bilinear / linear-extrapolation
interpolant against scipy's RegularGridInterpolator, MATLAB colon counts, and the product's
patch layout (``determine_patch_info_aug``) against the oracle's restatement."""
import numpy as np
import pytest

from oracle import mesolf_ref as R
from mesolf_gb300 import rectify as RC

CONFIGS = [
    dict(Nnum=15, frames_dx=15.27, frames_x_offset=1012.3, frames_y_offset=998.6,
         frames_crop_border_microlenses=[1, 1, 1, 1], patch_mode="carpet", n_patches=2),
    dict(Nnum=15, frames_dx=15.0, frames_x_offset=700.0, frames_y_offset=650.5,
         frames_crop_border_microlenses=[1, 1, 1, 1], patch_mode="carpet", n_patches=[2, 3]),
    dict(Nnum=15, frames_dx=14.62, frames_x_offset=33.2, frames_y_offset=40.9,
         frames_crop_border_microlenses=[2, 1, 1, 3], patch_mode="carpet", n_patches=3),
    dict(Nnum=11, frames_dx=11.4, frames_x_offset=500.0, frames_y_offset=501.0,
         frames_crop_border_microlenses=[1, 1, 1, 1], patch_mode="roi",
         ROI_list=[[1, 1, 400, 300], [200, 350, 700, 900]], ROI_patch_size=230),
]
SHAPES = [(2048, 2048), (1400, 1500), (900, 1000), (1100, 1100)]


def test_interp2_matches_scipy_linear_extrapolation():
    from scipy.interpolate import RegularGridInterpolator
    rng = np.random.default_rng(0)
    img = rng.random((40, 37))
    yq = np.linspace(-0.7, 41.3, 53)
    xq = np.linspace(-1.1, 38.9, 61)
    gi = RegularGridInterpolator((np.arange(1, 41.0), np.arange(1, 38.0)), img, method="linear",
                                 bounds_error=False, fill_value=None)
    Yq, Xq = np.meshgrid(yq, xq, indexing="ij")
    assert np.abs(R.interp2_linear(img, yq, xq) - gi(np.stack([Yq, Xq], -1))).max() < 1e-12


def test_matlab_colon_counts():
    assert np.allclose(R.matlab_colon(1, 0.5, 3), [1, 1.5, 2, 2.5, 3])
    assert np.allclose(R.matlab_colon(5, -1, 1), [5, 4, 3, 2, 1])
    assert len(R.matlab_colon(0, 0.1, 0.3)) == 4           # (0.3-0)/0.1 = 2.9999999999999996
    assert len(R.matlab_colon(3, 1, 2)) == 0
    for a, d, b in [(0, 0.1, 0.3), (7.5, -1.018, -1.018), (12.3, 1.018, 2048.9)]:
        assert np.array_equal(RC._colon(a, d, b), R.matlab_colon(a, d, b))


@pytest.mark.parametrize("k", range(len(CONFIGS)))
def test_patch_info_matches_oracle(k):
    SI, shape = CONFIGS[k], SHAPES[k]
    got = RC.determine_patch_info_aug(SI, shape)
    ref = R.determine_patch_info(SI, shape)
    assert len(got) == len(ref) > 0
    for g, r in zip(got, ref):
        assert np.array_equal(g["location"], r["location"]) and tuple(g["size"]) == tuple(r["size"])
        assert np.array_equal(g["raw_cut"], r["raw_cut"])
        assert g["raw_cut_xCenter"] == r["raw_cut_xCenter"] and g["raw_cut_yCenter"] == r["raw_cut_yCenter"]
        assert g["size"][0] % SI["Nnum"] == 0 and g["size"][1] % SI["Nnum"] == 0
        # the raw cut rectifies to exactly the patch size (the reference errors otherwise)
        rc = g["raw_cut"]
        shp = (rc[0, 1] - rc[0, 0] + 1, rc[1, 1] - rc[1, 0] + 1)
        assert RC.rectified_size(shp, g["raw_cut_xCenter"], g["raw_cut_yCenter"], SI["Nnum"],
                                 SI["frames_dx"]) == tuple(g["size"])


def test_patch_info_errors_and_discards():
    SI = dict(CONFIGS[0], frames_crop_border_microlenses=[70, 70, 0, 0])
    with pytest.raises(ValueError, match="X-cut range"):
        RC.determine_patch_info_aug(SI, (2048, 2048))
    with pytest.raises(ValueError, match="X-cut range"):
        R.determine_patch_info(SI, (2048, 2048))
    # without a border crop the safety margin of the first patch runs off the grid: both raise
    SI = dict(CONFIGS[0], frames_crop_border_microlenses=[0, 0, 0, 0], frames_x_offset=8.1)
    with pytest.raises(IndexError):
        RC.determine_patch_info_aug(SI, (2048, 2048))
    with pytest.raises(IndexError):
        R.determine_patch_info(SI, (2048, 2048))
    # 50 x 50 carpet: patches under 50 px are discarded
    SI = dict(CONFIGS[0], n_patches=50)
    assert RC.determine_patch_info_aug(SI, (2048, 2048)) == [] == R.determine_patch_info(SI, (2048, 2048))


def test_image_load_oracle_mean_then_rectify():
    """Averaging groups and the frame selection of image_load_module_aug.m:44-105."""
    SI = dict(CONFIGS[1], frames_start=2, frames_step=3, frames_end=11, frames_average=True)
    info = R.determine_patch_info(SI, SHAPES[1])[0]
    rng = np.random.default_rng(1)
    frames = (rng.random(SHAPES[1] + (12,)) * 4000).astype(np.uint16)
    mov = R.image_load(frames, info, SI)
    assert mov.shape == (info["size"][0] * info["size"][1], 4) and mov.max() == 1.0
    (y0, y1), (x0, x1) = info["raw_cut"]
    grp = frames[y0 - 1:y1, x0 - 1:x1, 10:11].astype(np.float64).mean(axis=2)   # last group: frame 11 only
    last = R.img_rectify_mod(grp, info["raw_cut_xCenter"], info["raw_cut_yCenter"], 15, SI["frames_dx"])
    full = R.image_load(frames, info, dict(SI, frames_average=False, frames_step=1, frames_start=11))
    assert np.allclose(last.reshape(-1, order="F") / last.max(), full[:, 0] / full[:, 0].max())
