"""Host-side mirror of the reference's call interface for the projector / RL path.

* :func:`mex_lfm_convolution_vec` -- ``out = mex_lfm_convolution_vec(bitmap, kernels)``
  (``src/cuda/mex_lfm_convolution_vec.cu:276-421``).
* :func:`recon_theory_phase_space_LFM_with_filter` --
  ``Xguess = recon_theory_phase_space_LFM_with_filter(LFIMG, H, Ht, maxIter, gpuFlag, gpu_id)``
  (``src/recon/recon_theory_phase_space_LFM_with_filter.m:10``).
* :func:`determine_patch_info_aug`, :func:`image_load_module_aug`, :func:`img_rectify_mod`
  -- raw frames to the per-patch sensor movie (``mesolf_gb300/rectify.py``).
* :func:`summary_image_generation_module` -- the step that produces ``LFIMG``
  (``src/module/summary_image_generation_module.m:1-133``).
* :class:`PhaseSpacePSF` / :class:`RLSolver` -- the same solve split into a resident PSF
  and a reusable per-image-size context (what a serving loop keeps in HBM).

Arrays are indexed in MATLAB order (``bitmap[x, y, i]``, ``H[x, y, a, b, z]``,
``vol[r, c, z]``).  numpy arrays are host memory; torch CUDA tensors are device memory
(any strides; they are made column-major).  Every call goes through libmesolf_lf.so:
there is no CPU fallback, and a missing library raises.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import MLFStats, check
from .rectify import determine_patch_info_aug, image_load_module_aug, img_rectify_mod  # noqa: F401

PRECISIONS = {"fp32": _lib.MLF_PREC_FP32, "bf16x3": _lib.MLF_PREC_BF16X3, "bf16": _lib.MLF_PREC_BF16,
              "bf16x2": _lib.MLF_PREC_BF16X2, "fp16": _lib.MLF_PREC_FP16, "fp16x2": _lib.MLF_PREC_FP16X2,
              "fp16x3": _lib.MLF_PREC_FP16X3}


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _fortran(x):
    """(keepalive, pointer) of x as float32 column-major memory."""
    if _is_torch(x):
        import torch
        t = x.to(torch.float32)
        rev = tuple(range(t.dim() - 1, -1, -1))
        want = []
        s = 1
        for d in t.shape:
            want.append(s)
            s *= d
        if list(t.stride()) != want:
            t = t.permute(rev).contiguous().permute(rev)
        return t, t.data_ptr()
    a = np.asfortranarray(np.asarray(x, dtype=np.float32))
    return a, a.ctypes.data


def _empty_like_kind(ref, shape):
    if _is_torch(ref):
        import torch
        rev = tuple(range(len(shape) - 1, -1, -1))
        t = torch.empty(tuple(reversed(shape)), dtype=torch.float32, device=ref.device).permute(rev)
        return t, t.data_ptr()
    a = np.empty(shape, dtype=np.float32, order="F")
    return a, a.ctypes.data


def _stream_of(x, stream):
    if stream is not None:
        return ctypes.c_void_p(int(stream))
    if _is_torch(x) and x.is_cuda:
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
    return ctypes.c_void_p(0)


CONV_METHODS = {"auto": 0, "direct": 1, "tensor": 2}


def mex_lfm_convolution_vec(bitmap, kernels, stream=None, method="auto"):
    """Drop-in for the MEX projector.

    bitmap: (W, H) or (W, H, n) float32; kernels: (kw, kw, 15, 15) float32.  Returns an
    array of the bitmap's shape, in the bitmap's memory kind.  Input checks follow
    ``mex_lfm_convolution_vec.cu:305-355`` and raise ``MesoLFError`` like its
    ``mexErrMsgIdAndTxt``.  ``method``: "direct" (CUDA-core FP32), "tensor" (the tensor-core
    route, FP32-class accuracy), "auto" (tensor cores for large calls when they apply).
    """
    lib = _lib.load()
    shp = tuple(bitmap.shape)
    if len(shp) not in (2, 3):
        raise _lib.MesoLFError(_lib.MLF_ERR_INVALID, "Invalid input to mex_lfm_convolution_vec()")
    if len(kernels.shape) != 4:
        raise _lib.MesoLFError(_lib.MLF_ERR_INVALID, "Invalid input to mex_lfm_convolution_vec()")
    W, Hh = shp[0], shp[1]
    n = shp[2] if len(shp) == 3 else 1
    kw = kernels.shape[0]
    b_keep, bp = _fortran(bitmap)
    k_keep, kp = _fortran(kernels)
    out, op = _empty_like_kind(bitmap, shp)
    check(lib.mlf_conv_vec_ex(bp, W, Hh, n, kp, kw, int(kernels.shape[2]), op, CONV_METHODS[method],
                              _stream_of(bitmap, stream)))
    del b_keep, k_keep
    return out


def mex_lfm_convolution_vec_accumulate(bitmaps, plane, slot, n_out, kernels, stream=None):
    """``out[:, :, o] = sum over j with slot[j] == o of mex_lfm_convolution_vec(bitmaps[:, :, j],
    kernels[:, :, :, :, plane[j]])`` in one pass (``mlf_conv_vec_accumulate``).  bitmaps
    (W, H, n), kernels (kw, kw, 15, 15, Z); plane and slot 0-based integer sequences of n."""
    lib = _lib.load()
    W, Hh, n = bitmaps.shape
    kw, Z = kernels.shape[0], kernels.shape[4]
    pl = np.ascontiguousarray(np.asarray(plane, dtype=np.int32))
    sl = np.ascontiguousarray(np.asarray(slot, dtype=np.int32))
    if pl.size != n or sl.size != n:
        raise _lib.MesoLFError(_lib.MLF_ERR_INVALID, "plane and slot must have one entry per slice")
    bk, bp = _fortran(bitmaps)
    kk, kp = _fortran(kernels)
    out, op = _empty_like_kind(bitmaps, (W, Hh, int(n_out)))
    check(lib.mlf_conv_vec_accumulate(bp, W, Hh, n, pl.ctypes.data, sl.ctypes.data, int(n_out), kp, kw,
                                      int(kernels.shape[2]), Z, op, _stream_of(bitmaps, stream)))
    del bk, kk
    return out


DETREND_MODES = {"pixelwise": _lib.MLF_DETREND_PIXELWISE, "global": _lib.MLF_DETREND_GLOBAL}

#: Defaults of the summary-image parameters (``src/mesolf_set_params.m:114-132``).
SUMMARY_DEFAULTS = {"detrend_mode": "pixelwise", "bg_iter": 5, "pixelwise_window_1": 100,
                    "pixelwise_window_2": 20, "pixelwise_poly_index": 3}


def summary_image(movie, detrend_mode="pixelwise", bg_iter=5, window_1=100, window_2=20, poly_index=3,
                  stream=None, pass_ms=None):
    """Summary image of a (pixels, frames) movie (``mlf_summary_image``): returns
    ``(summary, bg_spatial, bg_temporal)`` with shapes (P,), (P,), (T,), host arrays for a host
    movie and CUDA tensors for a CUDA tensor.  ``pass_ms``: an optional float64 array of 5
    that receives the device time of the passes (``mlf_summary_image_ex``)."""
    lib = _lib.load()
    if detrend_mode not in DETREND_MODES:
        raise _lib.MesoLFError(_lib.MLF_ERR_INVALID, 'Invalid value for param "detrend_mode"')
    shape = tuple(movie.shape)
    if len(shape) != 2:
        raise _lib.MesoLFError(_lib.MLF_ERR_INVALID, "the movie must be (pixels, frames)")
    P, T = shape
    keep, mp = _fortran(movie)
    img, ip = _empty_like_kind(movie, (P,))
    bs, sp = _empty_like_kind(movie, (P,))
    bt, tp = _empty_like_kind(movie, (T,))
    pm = None
    if pass_ms is not None:
        if not (isinstance(pass_ms, np.ndarray) and pass_ms.dtype == np.float64 and pass_ms.size >= 5):
            raise _lib.MesoLFError(_lib.MLF_ERR_INVALID, "pass_ms must be a float64 array of 5")
        pm = pass_ms.ctypes.data
    check(lib.mlf_summary_image_ex(mp, P, T, DETREND_MODES[detrend_mode], int(bg_iter), int(window_1),
                                   int(window_2), int(poly_index), ip, sp, tp, pm, _stream_of(movie, stream)))
    del keep
    return img, bs, bt


def summary_image_generation_module(sensor_movie, patch_info, SI):
    """``[summary_image, bg_spatial_init, bg_temporal_init] =
    summary_image_generation_module(sensor_movie, patch_info, SI)``
    (``src/module/summary_image_generation_module.m:1-133``).  sensor_movie is
    (size_h * size_w, frames) or (size_h, size_w, frames); patch_info["size"] gives
    (size_h, size_w); SI is a dict with the keys of :data:`SUMMARY_DEFAULTS` (missing keys take
    those defaults).  Returns the (size_h, size_w) summary image normalised to its maximum,
    the (size_h, size_w) rank-1 spatial background and the (1, frames) temporal background.
    The reference's TIFF/PNG outputs and trend plot are not produced."""
    prm = dict(SUMMARY_DEFAULTS)
    prm.update({k: v for k, v in dict(SI).items() if k in SUMMARY_DEFAULTS})
    h, w = (int(v) for v in patch_info["size"][:2])
    T = sensor_movie.shape[-1]
    mov = sensor_movie.reshape((h * w, T), order="F") if not _is_torch(sensor_movie) else \
        sensor_movie.permute(*reversed(range(sensor_movie.dim()))).reshape(T, h * w).T
    img, bs, bt = summary_image(mov, prm["detrend_mode"], prm["bg_iter"], prm["pixelwise_window_1"],
                                prm["pixelwise_window_2"], prm["pixelwise_poly_index"])
    if _is_torch(img):
        return (img.reshape(w, h).T, bs.reshape(w, h).T, bt.reshape(1, T))
    return img.reshape((h, w), order="F"), bs.reshape((h, w), order="F"), bt.reshape(1, T)


def seed_library_projections(Ht, sample, sample_mask, ring, ring_mask, unique_arrays):
    """The "collect and forward-project" section of
    ``src/gen_seed_library_local_with_ring_bg_same_size.m:257-318``: for every depth z, the
    slices of every segment at that depth (``find(unique_array == z)``) are projected with
    ``Ht(:,:,:,:,z)`` through ``mex_lfm_convolution_vec`` and added to the segment's
    accumulator, for the sample, its mask (binarised, ``> 0``), the ring and its mask.

    Segment i's volumes are (W, H, d_i) arrays, ``unique_arrays[i]`` the 1-based PSF plane
    of each of its d_i slices.  Returns ``(m_spatial_init_ext, m_seg_mask_ext,
    m_ring_init_ext, m_ring_mask_ext)``, each (W, H, N_seg), as host float32 arrays (the
    reference gathers them).  One batched pass on the GPU instead of 4 MEX calls per depth."""
    nseg = len(unique_arrays)
    kinds = [sample, sample_mask, ring, ring_mask]
    depth = [np.asarray(v).shape[2] if np.asarray(v).ndim == 3 else 1 for v in sample]
    W, Hh = np.asarray(sample[0]).shape[:2]
    n = 4 * sum(depth)
    bm = np.empty((W, Hh, n), dtype=np.float32, order="F")   # every slice copied once, in place
    plane, slot = np.empty(n, np.int32), np.empty(n, np.int32)
    j = 0
    for k, vols in enumerate(kinds):
        for i in range(nseg):
            v = np.asarray(vols[i])
            if v.ndim == 2:
                v = v[:, :, None]
            d = v.shape[2]
            if k in (1, 3):
                np.greater(v, 0, out=bm[:, :, j:j + d], casting="unsafe")
            else:
                bm[:, :, j:j + d] = v
            plane[j:j + d] = np.ravel(unique_arrays[i])[:d].astype(np.int32) - 1
            slot[j:j + d] = k * nseg + i
            j += d
    out = mex_lfm_convolution_vec_accumulate(bm, plane, slot, 4 * nseg, np.asfortranarray(Ht, dtype=np.float32))
    out = np.asarray(out)
    return tuple(np.asfortranarray(out[:, :, k * nseg:(k + 1) * nseg]) for k in range(4))


class PhaseSpacePSF:
    """Normalised phase-space PSF resident in HBM (``…_with_filter.m:13-40``)."""

    def __init__(self, H, Ht, stream=None):
        lib = _lib.load()
        if tuple(H.shape) != tuple(Ht.shape) or len(H.shape) != 5:
            raise _lib.MesoLFError(_lib.MLF_ERR_INVALID, "H and Ht must both be K0 x K0 x N x N x Z")
        K0, _, N, _, Z = H.shape
        hk, hp = _fortran(H)
        tk, tp = _fortran(Ht)
        h = ctypes.c_void_p()
        check(lib.mlf_psf_create(hp, tp, K0, N, Z, ctypes.byref(h), _stream_of(H, stream)))
        self._h = h
        self.K0, self.N, self.Z = int(K0), int(N), int(Z)
        n = ctypes.c_int32()
        z = ctypes.c_int64()
        s = ctypes.c_int64()
        check(lib.mlf_psf_info(h, ctypes.byref(n), ctypes.byref(z), ctypes.byref(s)))
        self.S = int(s.value)
        w = np.zeros((N, N), dtype=np.float64, order="F")
        check(lib.mlf_psf_weights(h, w.ctypes.data))
        self.weights = w
        del hk, tk

    @property
    def handle(self):
        return self._h

    @property
    def device_bytes(self):
        return int(_lib.load().mlf_psf_device_bytes(self._h))

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().mlf_psf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RLSolver:
    """Solve context for one image size (scratch volume, sub-aperture images, graphs)."""

    VARIANTS = {"base": 0, "peeling": 1}

    def __init__(self, psf: PhaseSpacePSF, image_shape, variant="base"):
        lib = _lib.load()
        self.psf = psf
        self.Xr, self.Xc = int(image_shape[0]), int(image_shape[1])
        self.variant = variant
        h = ctypes.c_void_p()
        check(lib.mlf_solver_create_variant(psf.handle, self.Xr, self.Xc, self.VARIANTS[variant], ctypes.byref(h)))
        self._h = h
        self.last_stats = None

    @property
    def device_bytes(self):
        return int(_lib.load().mlf_solver_device_bytes(self._h))

    def run(self, lfimg, max_iter, precision="fp32", warm_start=None, out=None, stream=None,
            want_stats=True):
        """Run ``max_iter`` RL iterations; returns the (Xr, Xc, Z) volume."""
        lib = _lib.load()
        lk, lp = _fortran(lfimg)
        wk, wp = (None, None) if warm_start is None else _fortran(warm_start)
        shape = (self.Xr, self.Xc, self.psf.Z)
        if out is None:
            out, op = _empty_like_kind(lfimg, shape)
        else:
            op = out.data_ptr() if _is_torch(out) else out.ctypes.data
        st = MLFStats()
        check(lib.mlf_solver_run(self._h, lp, int(max_iter), PRECISIONS[precision], wp, op,
                                 ctypes.byref(st) if want_stats else None, _stream_of(lfimg, stream)))
        self.last_stats = st.as_dict() if want_stats else None
        del lk, wk
        return out

    def run_peeling(self, lfimg, max_iter, precision="fp32", stream=None, want_stats=True):
        """The peeling solve (``…_with_filter_simple_peeling.m:13-266``) on a device image;
        needs ``variant="peeling"``.  Returns (volume, peeled image, proj_sensor) on the device."""
        lk, lp = _fortran(lfimg)
        vol, vp = _empty_like_kind(lfimg, (self.Xr, self.Xc, self.psf.Z))
        lf2, l2p = _empty_like_kind(lfimg, (self.Xr, self.Xc))
        proj, pp = _empty_like_kind(lfimg, (self.Xr, self.Xc))
        st = MLFStats()
        check(_lib.load().mlf_solver_run_peeling(self._h, lp, int(max_iter), PRECISIONS[precision], vp, l2p, pp,
                                                 ctypes.byref(st) if want_stats else None,
                                                 _stream_of(lfimg, stream)))
        self.last_stats = st.as_dict() if want_stats else None
        del lk
        return vol, lf2, proj

    def forward_view(self, vol, u, v, stream=None, precision="fp32"):
        """HX of view (u, v) (0-based) for a device volume -> (Xr/N, Xc/N) device array."""
        import torch
        vk, vp = _fortran(vol)
        hx = torch.empty((self.Xc // self.psf.N, self.Xr // self.psf.N), dtype=torch.float32,
                         device=vol.device).t()
        if precision == "fp32":
            check(_lib.load().mlf_forward_view(self._h, vp, int(u), int(v), hx.data_ptr(),
                                               _stream_of(vol, stream)))
        else:
            check(_lib.load().mlf_forward_view_prec(self._h, vp, int(u), int(v), PRECISIONS[precision],
                                                    hx.data_ptr(), _stream_of(vol, stream)))
        del vk
        return hx

    def backward_view(self, proj, u, v, stream=None):
        """Back projection of a (Xr/N, Xc/N) device array for view (u, v) -> (Xr, Xc, Z)."""
        pk, pp = _fortran(proj)
        out, op = _empty_like_kind(proj, (self.Xr, self.Xc, self.psf.Z))
        check(_lib.load().mlf_backward_view(self._h, pp, int(u), int(v), op, _stream_of(proj, stream)))
        del pk
        return out

    def view_step(self, lfimg, vol, u, v, w, stream=None, precision="fp32"):
        """One RL view update of a device volume in place (``…_with_filter.m:109-137``)."""
        lk, lp = _fortran(lfimg)
        check(_lib.load().mlf_rl_view_step_prec(self._h, lp, vol.data_ptr(), int(u), int(v), float(w),
                                                PRECISIONS[precision], _stream_of(vol, stream)))
        del lk
        return vol

    def forward_project(self, vol, raw_psf=True, precision="fp32", stream=None):
        """Full light-field image (Xr, Xc) of a device (Xr, Xc, Z) volume, the reference's
        ``forwardProjectGPU(H, vol)`` (``src/recon/forwardProjectGPU.m:1-20``).  ``raw_psf``
        projects with H as given (True) or with the per-plane normalised H of the solve."""
        vk, vp = _fortran(vol)
        lf, lp = _empty_like_kind(vol, (self.Xr, self.Xc))
        check(_lib.load().mlf_forward_project(self._h, vp, lp, 1 if raw_psf else 0, PRECISIONS[precision],
                                              _stream_of(vol, stream)))
        del vk
        return lf

    def sample_filter(self, vol, stream=None):
        """The per-iteration flux-preserving low-pass on a device volume, in place."""
        check(_lib.load().mlf_sample_filter(self._h, vol.data_ptr(), _stream_of(vol, stream)))
        return vol

    def cancel(self):
        """Ask the solve in progress (from another thread) to stop between view steps; its
        output is left unwritten and a synchronous run raises MesoLFError (MLF_ERR_CANCELLED)."""
        check(_lib.load().mlf_solver_cancel(self._h))

    @property
    def cancelled(self):
        """True if the last solve stopped early (read after its stream was synchronised)."""
        return bool(_lib.load().mlf_solver_cancelled(self._h))

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().mlf_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchSolver:
    """Independent patches solved together on the tensor cores (one launch per view step
    for all of them).  ``shapes`` = [(Xr, Xc), ...]; ``planes`` = [(z0, nz), ...] plane
    ranges of the shared PSF (default: all planes)."""

    def __init__(self, psf: PhaseSpacePSF, shapes, planes=None):
        lib = _lib.load()
        self.psf = psf
        self.shapes = [(int(a), int(b)) for a, b in shapes]
        P = len(self.shapes)
        if planes is None:
            planes = [(0, psf.Z)] * P
        self.planes = [(int(a), int(b)) for a, b in planes]
        xr = (ctypes.c_int64 * P)(*[a for a, _ in self.shapes])
        xc = (ctypes.c_int64 * P)(*[b for _, b in self.shapes])
        z0 = (ctypes.c_int32 * P)(*[a for a, _ in self.planes])
        nz = (ctypes.c_int32 * P)(*[b for _, b in self.planes])
        h = ctypes.c_void_p()
        check(lib.mlf_batch_create(psf.handle, P, xr, xc, z0, nz, ctypes.byref(h)))
        self._h = h
        self.last_stats = None

    @property
    def device_bytes(self):
        return int(_lib.load().mlf_batch_device_bytes(self._h))

    @staticmethod
    def plan_bytes(psf: PhaseSpacePSF, shapes, planes=None):
        """Device bytes a BatchSolver for these patches would allocate (upper bound; no
        allocation), for admission by free HBM."""
        P = len(shapes)
        if planes is None:
            planes = [(0, psf.Z)] * P
        xr = (ctypes.c_int64 * P)(*[int(a) for a, _ in shapes])
        xc = (ctypes.c_int64 * P)(*[int(b) for _, b in shapes])
        z0 = (ctypes.c_int32 * P)(*[int(a) for a, _ in planes])
        nz = (ctypes.c_int32 * P)(*[int(b) for _, b in planes])
        out = ctypes.c_int64()
        check(_lib.load().mlf_batch_plan_bytes(psf.handle, P, xr, xc, z0, nz, ctypes.byref(out)))
        return int(out.value)

    def run(self, lfimgs, max_iter, precision="bf16x2", warm=None, outs=None, stream=None, want_stats=True):
        """Device (torch CUDA) images in, list of (Xr, Xc, nz) device volumes out.  A None
        image leaves that patch out of this run (its output entry is returned as given, or
        None); at least one patch needs an image."""
        import torch
        lib = _lib.load()
        P = len(self.shapes)
        keep = []
        lp = (ctypes.c_void_p * P)()
        first = next((im for im in lfimgs if im is not None), None)
        if first is None:
            raise ValueError("BatchSolver.run: no patch has an image")
        for k, im in enumerate(lfimgs):
            if im is None:
                continue
            t, ptr = _fortran(im)
            keep.append(t)
            lp[k] = ptr
        wp = None
        if warm is not None:
            wp = (ctypes.c_void_p * P)()
            for k, x in enumerate(warm):
                if x is not None:
                    t, ptr = _fortran(x)
                    keep.append(t)
                    wp[k] = ptr
        if outs is None:
            outs = [None if lfimgs[k] is None else
                    _empty_like_kind(lfimgs[k], (self.shapes[k][0], self.shapes[k][1], self.planes[k][1]))[0]
                    for k in range(P)]
        op = (ctypes.c_void_p * P)(*[(o.data_ptr() if (o is not None and lfimgs[k] is not None) else None)
                                     for k, o in enumerate(outs)])
        st = MLFStats()
        check(lib.mlf_batch_run(self._h, lp, int(max_iter), PRECISIONS[precision], wp, op,
                                ctypes.byref(st) if want_stats else None, _stream_of(first, stream)))
        self.last_stats = st.as_dict() if want_stats else None
        del keep
        return outs

    def cancel(self):
        """Ask the run in progress on this work set (from another thread) to stop between
        view steps; its outputs are left unwritten (see mlf_batch_cancel)."""
        check(_lib.load().mlf_batch_cancel(self._h))

    @property
    def cancelled(self):
        """True if the last run stopped early (read after its stream was synchronised)."""
        return bool(_lib.load().mlf_batch_cancelled(self._h))

    def forward_project(self, vols, raw_psf=True, precision="bf16x3", stream=None):
        """Full light-field images of device volumes (patch k: (Xr, Xc, nz) with the PSF
        planes of its range) on the tensor cores; returns a list of (Xr, Xc) device arrays."""
        P = len(self.shapes)
        keep = []
        vp = (ctypes.c_void_p * P)()
        for k, v in enumerate(vols):
            t, ptr = _fortran(v)
            keep.append(t)
            vp[k] = ptr
        outs = [_empty_like_kind(vols[k], self.shapes[k])[0] for k in range(P)]
        op = (ctypes.c_void_p * P)(*[o.data_ptr() for o in outs])
        check(_lib.load().mlf_batch_forward_project(self._h, vp, op, 1 if raw_psf else 0, PRECISIONS[precision],
                                                    _stream_of(vols[0], stream)))
        del keep
        return outs

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().mlf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def recon_theory_phase_space_LFM_with_filter(LFIMG, H, Ht, maxIter, gpuFlag=True, gpu_id=1,
                                             precision="fp32"):
    """Same arguments as the reference solver; returns the volume as a host float64
    array (the reference returns ``gather(Xguess)`` in double).  ``gpuFlag`` must be
    true: this library has no CPU branch."""
    if not gpuFlag:
        raise _lib.MesoLFError(_lib.MLF_ERR_UNSUPPORTED,
                               "gpuFlag=false: libmesolf_lf.so implements only the GPU path")
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.set_device(int(gpu_id) - 1)
    except ImportError:
        pass
    psf = PhaseSpacePSF(H, Ht)
    try:
        solver = RLSolver(psf, LFIMG.shape)
        try:
            vol = solver.run(np.asarray(LFIMG), maxIter, precision=precision)
        finally:
            solver.close()
    finally:
        psf.close()
    return np.asarray(vol, dtype=np.float64)


def recon_theory_phase_space_LFM_with_filter_simple_peeling(LFIMG, H_origin, Ht_origin, maxIter, gpuFlag=True,
                                                            gpu_id=1, precision="fp32"):
    """``[Xguess, LFIMG, proj_sensor] = recon_theory_phase_space_LFM_with_filter_simple_peeling(
    LFIMG, H_origin, Ht_origin, maxIter, gpuFlag, gpu_id)`` (``…_simple_peeling.m:13``): host
    float64 arrays out, as the reference gathers them.  ``gpuFlag`` must be true."""
    if not gpuFlag:
        raise _lib.MesoLFError(_lib.MLF_ERR_UNSUPPORTED,
                               "gpuFlag=false: libmesolf_lf.so implements only the GPU path")
    import torch
    torch.cuda.set_device(int(gpu_id) - 1)
    psf = PhaseSpacePSF(H_origin, Ht_origin)
    try:
        solver = RLSolver(psf, np.shape(LFIMG), variant="peeling")
        try:
            lf = _fortran(torch.as_tensor(np.ascontiguousarray(np.asarray(LFIMG, np.float32))).cuda())[0]
            vol, lf2, proj = solver.run_peeling(lf, maxIter, precision=precision)
            out = tuple(x.double().cpu().numpy() for x in (vol, lf2, proj))
        finally:
            solver.close()
    finally:
        psf.close()
    return out


# ----------------------------------------------------------------------------- full forward projectors
def phase_space_kept_mask(K0, N):
    """(K0, K0, N, N) bool: the PSF pixels that the phase-space realignment keeps
    (``gen_phasespace_PSF_theory.m:8-27``: crop to S = K0 - mod(K0 - N, 2N) starting at
    i1 = round(K0/2) - fix(S/2), then shift slice (a, b) by (a - h, b - h), h = (N-1)/2, with
    zero fill).  Projections through the phase-space operator equal the reference's
    full-resolution sums exactly when every PSF pixel outside this mask is zero."""
    S = K0 - (K0 - N) % (2 * N)
    i1 = int(np.floor(K0 / 2 + 0.5)) - S // 2 - 1
    h = (N - 1) // 2
    idx = np.arange(K0)
    rows = np.zeros((K0, N), bool)
    for a in range(N):
        lo = i1 + max(0, h - a)
        hi = i1 + S - 1 - max(0, a - h)
        rows[:, a] = (idx >= lo) & (idx <= hi)
    return rows[:, None, :, None] & rows[None, :, None, :]


def _project_full(H, vol, precision):
    import warnings

    import torch
    H = np.asfortranarray(np.asarray(H, np.float32))
    K0, N = H.shape[0], H.shape[2]
    keep = phase_space_kept_mask(K0, N)
    if np.any(H[~keep[..., None].repeat(H.shape[4], axis=4)] != 0):
        warnings.warn("PSF has support outside the phase-space crop; those pixels are not projected",
                      RuntimeWarning, stacklevel=3)
    psf = PhaseSpacePSF(H, np.asfortranarray(H[::-1, ::-1]))
    try:
        s = RLSolver(psf, vol.shape[:2])
        try:
            v = _fortran(torch.as_tensor(np.ascontiguousarray(np.asarray(vol, np.float32))).cuda())[0]
            lf = s.forward_project(v, raw_psf=True, precision=precision)
            return lf.double().cpu().numpy()
        finally:
            s.close()
    finally:
        psf.close()


def forwardProjectGPU(H, realspace, precision="fp32"):
    """``TOTALprojection = forwardProjectGPU(H, realspace, ...)`` (``src/recon/forwardProjectGPU.m:1-20``):
    ``sum_{a,b,z} conv2(realspace_z .* [phase (a, b)], H(:,:,a,b,z), 'same')``, host float64 out."""
    return _project_full(H, realspace, precision)


def forwardProjectACC(H, realspace, CAindex, precision="fp32"):
    """``forwardProjectACC(H, realspace, CAindex)`` (``src/recon/forwardProjectACC.m:1-18``): the
    PSF of plane z cropped to rows / columns ``CAindex(z,1):CAindex(z,2)`` (1-based) before the
    'same' convolution.  The crop must be centred on the PSF (the 'same' centre of the
    cropped kernel is then the PSF centre), which is how MesoLF builds CAindex."""
    H = np.asarray(H, np.float32)
    K0 = H.shape[0]
    Hc = np.zeros_like(H, order="F")
    for z in range(H.shape[4]):
        lo, hi = int(CAindex[z][0]) - 1, int(CAindex[z][1])
        if (lo + (hi - lo) // 2) != K0 // 2:
            raise ValueError(f"CAindex row {z}: crop [{lo + 1}, {hi}] is not centred on the {K0}-px PSF")
        Hc[lo:hi, lo:hi, :, :, z] = H[lo:hi, lo:hi, :, :, z]
    return _project_full(Hc, realspace, precision)


def forwardProjectGPU_discrete(H, realspace, unique_array, max_PSF_size, precision="fp32"):
    """``forwardProjectGPU_discrete(H, realspace, ..., unique_array, max_PSF_size)``
    (``src/recon/forwardProjectGPU_discrete.m:1-20``): volume plane cc is projected with PSF
    plane ``unique_array(cc)`` (1-based) cropped to the central ``2*floor(max_PSF_size/2)+1``
    pixels.  Planes sharing a PSF plane are summed first (the projection is linear)."""
    H = np.asarray(H, np.float32)
    K0 = H.shape[0]
    half = int(max_PSF_size) // 2
    c = int(np.ceil(K0 / 2)) - 1
    zs = sorted(set(int(u) - 1 for u in np.ravel(unique_array)))
    Hc = np.zeros(H.shape[:4] + (len(zs),), np.float32, order="F")
    lo, hi = max(0, c - half), min(K0, c + half + 1)
    vol = np.asarray(realspace, np.float64)
    v2 = np.zeros(vol.shape[:2] + (len(zs),))
    for k, z in enumerate(zs):
        Hc[lo:hi, lo:hi, :, :, k] = H[lo:hi, lo:hi, :, :, z]
    for cc, u in enumerate(np.ravel(unique_array)):
        v2[:, :, zs.index(int(u) - 1)] += vol[:, :, cc]
    return _project_full(Hc, v2, precision)


def forwardProjectGPU_skip_2D(H, realspace, step, cc, precision="fp32"):
    """``forwardProjectGPU_skip_2D(H, realspace, ..., step, cc)``
    (``src/recon/forwardProjectGPU_skip_2D.m:1-16``): a 2-D image projected with PSF plane
    ``cc`` (1-based), only the pixels whose lenslet phase (a, b) has ``a, b = 1, 1+step, ...``."""
    H = np.asarray(H, np.float32)
    N = H.shape[2]
    img = np.asarray(realspace, np.float64)
    keep = np.zeros(img.shape, bool)
    for a in range(0, N, int(step)):
        for b in range(0, N, int(step)):
            keep[a::N, b::N] = True
    Hz = np.asfortranarray(H[:, :, :, :, int(cc) - 1:int(cc)])
    return _project_full(Hz, np.where(keep, img, 0.0)[:, :, None], precision)
