"""Frame rectification and patch layout: the steps that turn raw sensor frames into the
per-patch sensor movie (the input of the summary image and of the reconstruction).

* :func:`determine_patch_info_aug` -- ``src/module/determine_patch_info_aug.m:1-290`` (no
  plot): patch locations in the rectified frame and their raw cuts, host logic.
* :func:`img_rectify_mod` -- ``src/module/image_load_module_aug.m:126-164`` on one frame.
* :func:`image_load_module_aug` -- ``src/module/image_load_module_aug.m:1-123`` on frames in
  memory: frame selection / averaging, cut, rectification and max normalisation on the GPU
  (``mlf_rectify_frames``).  Reading the TIFF files stays with the caller.

Frames are MATLAB-ordered (rows, cols, frame) arrays: numpy (host) or torch CUDA tensors.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import check


def _colon(a, d, b):
    """MATLAB ``a:d:b`` (d != 0) with a 1e-10 relative tolerance on the element count."""
    q = (b - a) / d
    tol = 1e-10 * max(1.0, abs(q))
    n = 0 if q < -tol else int(math.floor(q + tol)) + 1
    return a + d * np.arange(n, dtype=np.float64)


def rectification_axis(center, lo, hi, M, dx):
    """``[fliplr(center:-dx/M:lo), center+dx/M:dx/M:hi]`` with the 1-based index of ``center``
    in it and the left cut ``mod(index - floor(M/2), M)`` that aligns the first lenslet.
    Returns (grid, center_index, left_cut)."""
    s = dx / M
    grid = np.concatenate([_colon(center, -s, lo)[::-1], _colon(center + s, s, hi)])
    ci = int(np.searchsorted(grid, center)) + 1          # the grid is increasing; center is in it
    c0 = ci - M // 2
    return grid, ci, c0 % M


def rectified_size(shape, x_center, y_center, M, dx):
    """(rows, cols) that :func:`img_rectify_mod` gives for a raw patch of ``shape``."""
    out = []
    for n, c in ((shape[0], y_center), (shape[1], x_center)):
        g, _, q = rectification_axis(c, -dx / M, n + 0.9, M, dx)
        out.append(M * ((len(g) - q) // M))
    return tuple(out)


def determine_patch_info_aug(SI, frame_shape):
    """Patch list of ``determine_patch_info_aug(SI)``: ``frame_shape`` = (rows, cols) of the
    first frame (the reference reads it from the first TIFF).  SI keys: Nnum, frames_dx,
    frames_x_offset, frames_y_offset, frames_crop_border_microlenses, patch_mode ('carpet' with
    n_patches, or 'roi' with ROI_list and ROI_patch_size).  Each entry: location ([top, left],
    [bottom, right], 1-based, rectified frame), size, raw_cut ([y0, y1], [x0, x1], 1-based raw
    frame), raw_cut_xCenter, raw_cut_yCenter."""
    rows, cols = (int(v) for v in frame_shape)
    M, dx = int(SI["Nnum"]), float(SI["frames_dx"])
    xl, xr, yu, yd = (int(v) for v in SI.get("frames_crop_border_microlenses", (0, 0, 0, 0)))
    gx, cx0, qx = rectification_axis(float(SI["frames_x_offset"]), 1.0, float(cols), M, dx)
    gy, cy0, qy = rectification_axis(float(SI["frames_y_offset"]), 1.0, float(rows), M, dx)
    nlx, nly = (len(gx) - qx) // M, (len(gy) - qy) // M       # whole lenslets after the left cut
    if xl + xr >= nlx:
        raise ValueError("X-cut range is larger than the x-size of image")
    if yu + yd >= nly:
        raise ValueError("Y-cut range is larger than the y-size of image")
    gh, gw = (nly - yu - yd) * M, (nlx - xl - xr) * M          # cropped rectified frame

    def tiles(org, extent, step, count):
        # 1-based [first, last] of tile k of a run of `extent` starting at `org`, tiles of `step`
        return [(org + k * step, org + min((k + 1) * step, extent) - 1) for k in range(count)]

    boxes = []
    mode = SI.get("patch_mode", "carpet")
    if mode == "carpet":
        n = SI.get("n_patches", 1)
        nh, nw = (n, n) if np.isscalar(n) else (int(n[0]), int(n[1]))
        sh, sw = -(-(gh // nh) // M) * M, -(-(gw // nw) // M) * M
        th, tw = tiles(1, gh, sh, nh), tiles(1, gw, sw, nw)
        boxes = [(th[k % nh], tw[k // nh]) for k in range(nh * nw)]
    elif mode == "roi":
        rps = int(SI["ROI_patch_size"])
        rps -= rps % M
        for roi in np.atleast_2d(np.asarray(SI["ROI_list"], dtype=np.int64)):
            ext = (int(roi[2] - roi[0] + 1), int(roi[3] - roi[1] + 1))
            step = [e if e < rps else rps for e in ext]
            cnt = [1 if e < rps else -(-e // rps) for e in ext]
            th, tw = tiles(int(roi[0]), ext[0], step[0], cnt[0]), tiles(int(roi[1]), ext[1], step[1], cnt[1])
            boxes += [(th[k % cnt[0]], tw[k // cnt[0]]) for k in range(cnt[0] * cnt[1])]
    else:
        raise ValueError("patch_mode should be either 'carpet' or 'roi'")
    top0, left0 = yu * M + 1, xl * M + 1
    margin = -(-M // 2) - 2
    half = -(-M // 2)
    out = []
    for (t, b), (l, r) in boxes:
        ph, pw = (b - t + 1) - (b - t + 1) % M, (r - l + 1) - (r - l + 1) % M
        if ph < 50 or pw < 50:
            continue
        b, r = t + ph - 1, l + pw - 1
        # grid indices (1-based) of the patch with its safety margin
        gt, gb = t + top0 + qy - 2 - margin, b + top0 + qy - 2 + margin - 1
        gl, gr = l + left0 + qx - 2 - margin, r + left0 + qx - 2 + margin - 1
        if min(gt, gl) < 1 or gb > len(gy) or gr > len(gx):
            raise IndexError("Index exceeds the number of array elements")
        cy = int(math.floor((gt + gb) / 2 + 0.5))
        cx = int(math.floor((gl + gr) / 2 + 0.5))
        my, mx = (cy0 - cy) % M, (cx0 - cx) % M
        yc = gy[cy - (M - my) - 1] if my >= half else gy[cy + my - 1]
        xc = gx[cx - (M - mx) - 1] if mx >= half else gx[cx + mx - 1]
        out.append({"location": np.array([[t, l], [b, r]]), "size": (ph, pw),
                    "raw_cut": np.array([[max(math.floor(gy[gt - 1]), 1), min(math.ceil(gy[gb - 1]), rows)],
                                         [max(math.floor(gx[gl - 1]), 1), min(math.ceil(gx[gr - 1]), cols)]]),
                    "raw_cut_yCenter": float(yc - gy[gt - 1]), "raw_cut_xCenter": float(xc - gx[gl - 1])})
    return out


def _frames_arg(frames):
    if type(frames).__module__.startswith("torch"):
        import torch
        if getattr(torch, "uint16", None) is not None and frames.dtype == torch.uint16:
            dt = _lib.MLF_DTYPE_U16
        elif frames.dtype == torch.float32:
            dt = _lib.MLF_DTYPE_F32
        else:
            frames = frames.to(torch.float32)
            dt = _lib.MLF_DTYPE_F32
        t = frames if frames.dim() == 3 else frames[:, :, None]
        rev = (2, 1, 0)
        t = t.permute(rev).contiguous().permute(rev)            # column-major
        return t, t.data_ptr(), tuple(t.shape), dt
    a = np.asarray(frames)
    if a.ndim == 2:
        a = a[:, :, None]
    if a.dtype == np.uint16:
        dt = _lib.MLF_DTYPE_U16
    else:
        a = a.astype(np.float32, copy=False)
        dt = _lib.MLF_DTYPE_F32
    a = np.asfortranarray(a)
    return a, a.ctypes.data, a.shape, dt


def image_load_module_aug(patch_info, SI, frames, normalize=True, stream=None, out_device=None):
    """``sensor_movie = image_load_module_aug(patch_info, SI)`` on frames in memory: ``frames``
    (rows, cols, n_files) uint16 or float32, the files in ``dir`` order.  SI keys: Nnum,
    frames_dx, frames_start (1), frames_step (1), frames_end (inf), frames_average (True).
    Returns the (size_h*size_w, n_frames) float32 movie (host array, or CUDA tensor for CUDA
    frames), divided by its maximum unless ``normalize`` is False (the summary image divides by
    the maximum itself).  ``out_device``: a CUDA device for the movie when the frames are on the
    host (frames from a camera buffer, movie kept in HBM for the next step)."""
    lib = _lib.load()
    keep, ptr, shape, dt = _frames_arg(frames)
    H, W, n = shape
    end = SI.get("frames_end", math.inf)
    end = -1 if end is None or not math.isfinite(end) else int(end)
    start, step = int(SI.get("frames_start", 1)), int(SI.get("frames_step", 1))
    last = n if end < 0 else min(n, end)
    if last < start:
        raise _lib.MesoLFError(_lib.MLF_ERR_INVALID, "no frame selected")
    n_final = (last - start) // step + 1
    h, w = (int(v) for v in patch_info["size"])
    rc = np.ascontiguousarray(np.asarray(patch_info["raw_cut"], dtype=np.int64).reshape(-1))
    on_dev = type(frames).__module__.startswith("torch") and frames.is_cuda
    if on_dev or out_device is not None:
        import torch
        dev = frames.device if on_dev else torch.device(out_device)
        out = torch.empty((n_final, h * w), dtype=torch.float32, device=dev).T
        optr = out.data_ptr()
        sp = ctypes.c_void_p(int(stream) if stream is not None else torch.cuda.current_stream(dev).cuda_stream)
    else:
        out = np.empty((h * w, n_final), dtype=np.float32, order="F")
        optr = out.ctypes.data
        sp = ctypes.c_void_p(int(stream) if stream is not None else 0)
    nout = ctypes.c_int64(0)
    check(lib.mlf_rectify_frames(ptr, dt, H, W, n, rc.ctypes.data, float(patch_info["raw_cut_xCenter"]),
                                 float(patch_info["raw_cut_yCenter"]), int(SI["Nnum"]), float(SI["frames_dx"]),
                                 h, w, start, step, end, int(bool(SI.get("frames_average", True))),
                                 int(bool(normalize)), optr, ctypes.byref(nout), sp))
    del keep
    return out


def img_rectify_mod(IMG_BW, xCenter, yCenter, M, dx):
    """``IMG_RESAMPLE = img_rectify_mod(IMG_BW, xCenter, yCenter, M, dx)`` on the GPU: one raw
    patch (rows, cols) resampled onto the lenslet grid; returns (rows', cols') float32."""
    a = np.asarray(IMG_BW) if not type(IMG_BW).__module__.startswith("torch") else IMG_BW
    H, W = a.shape[:2]
    h, w = rectified_size((H, W), float(xCenter), float(yCenter), int(M), float(dx))
    info = {"size": (h, w), "raw_cut": [[1, H], [1, W]], "raw_cut_xCenter": xCenter, "raw_cut_yCenter": yCenter}
    mov = image_load_module_aug(info, {"Nnum": M, "frames_dx": dx}, a, normalize=False)
    return mov.reshape((h, w), order="F") if isinstance(mov, np.ndarray) else mov.T.reshape(w, h).T
