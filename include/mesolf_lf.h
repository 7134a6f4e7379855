/*
 * mesolf_lf.h -- C ABI of libmesolf_lf.so, the GB300 (sm_103a) light-field projector and
 * phase-space Richardson-Lucy deconvolver.
 *
 * Conventions
 *   - Every entry point returns an int status (MLF_OK == 0) and never aborts the
 *     process; mlf_last_error() returns the calling thread's last message.
 *   - Arrays use MATLAB's column-major layout and dimension order, so a MEX shim passes
 *     mxGetData()/mxGPUGetData() pointers straight through.
 *   - "dev" pointers must be device memory of the current CUDA device; "any" pointers may
 *     be device or host memory (detected with cudaPointerGetAttributes; host buffers are
 *     staged through the library's own device buffers).
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).  Calls are
 *     stream-ordered; functions documented "synchronous" synchronise the stream before
 *     returning, as the reference MEX does.
 *   - An mlf_psf may be shared read-only by many solvers; an mlf_solver is used by one
 *     host thread / stream at a time.
 */
#ifndef MESOLF_LF_H
#define MESOLF_LF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MLF_ABI_VERSION 3

enum mlf_status_code {
  MLF_OK = 0,
  MLF_ERR_INVALID = 1,     /* bad argument: shape, size, null pointer, unsupported Nnum */
  MLF_ERR_CUDA = 2,        /* a CUDA runtime call failed (message holds cudaGetErrorString) */
  MLF_ERR_NOMEM = 3,       /* device allocation failed / admission refused for lack of HBM */
  MLF_ERR_UNSUPPORTED = 4, /* valid input outside what this build implements */
  MLF_ERR_TIMEOUT = 5,     /* a bounded wait expired (device status flag) */
  MLF_ERR_CANCELLED = 6    /* request cancelled by the caller */
};

enum mlf_precision {
  MLF_PREC_FP32 = 0,       /* plain FP32 FMA projector (the drop-in path) */
  MLF_PREC_BF16X3 = 1,     /* tensor cores: taps and activations split hi+lo BF16 (3 passes) */
  MLF_PREC_BF16 = 2,       /* tensor cores: single BF16 operands (1 pass) */
  MLF_PREC_BF16X2 = 3,     /* tensor cores: activations split hi+lo, taps single BF16 (2 passes) */
  MLF_PREC_FP16 = 4,       /* tensor cores: single FP16 operands (1 pass) */
  MLF_PREC_FP16X2 = 5,     /* tensor cores: activations split hi+lo FP16, taps single FP16 (2 passes) */
  MLF_PREC_FP16X3 = 6      /* tensor cores: taps and activations split hi+lo FP16 (3 passes) */
  /* all tensor-core modes accumulate in FP32; ratio, update, filter and sums stay FP32.
   * FP16 operands carry power-of-two scales so that FP16's range (6.1e-5 .. 65504) holds
   * them: each back-projection tap row (view, channel) and each forward tap column (view,
   * tap) is scaled to a maximum in [2^14, 2^15) on the device when the FP16 tables are
   * built; the ratio image by its per-view maximum; the volume by a running maximum kept
   * on the device (every back projection raises it).  Powers of two are exact, and the
   * FP32 epilogues remove them (the tap-row scale cancels in C/D). */
};

typedef struct mlf_psf mlf_psf;       /* phase-space PSF resident in HBM */
typedef struct mlf_solver mlf_solver; /* per-image-size solve context (scratch in HBM) */
typedef struct mlf_batch mlf_batch;   /* many patches solved together on the tensor cores */

typedef struct mlf_stats {
  int32_t n_views;              /* active views per iteration (weight != 0) */
  int32_t iterations;           /* iterations run */
  double gpu_ms;                /* device time of the solve (CUDA events) */
  double view_ms;               /* gpu_ms / (iterations * n_views) */
  double view_kernel_ms;        /* summed device time of the projector (view) kernel launches */
  int64_t view_kernel_launches; /* number of projector kernel launches timed */
  int64_t kernel_launches;      /* kernels launched by the solve */
  /* tensor-core solves: the launch configuration in use, chosen by the autotuner on the
   * first solve of the work set at this precision (timing candidates on one view step)
   * unless the environment sets MLF_TUNE=0; 0 for FP32 solves */
  int32_t fwd_splits;           /* split-K count of the forward GEMM over the channels */
  int32_t fwd_stages;           /* shared-memory ring depth of the forward GEMM */
  int32_t bwd_xbufs;            /* X-tile buffers per half in the back projection (1 or 2) */
  int32_t tuned;                /* 1 if chosen by timing, 0 if the built-in heuristics */
  /* convergence monitor (ABI 3): ||X_k - X_(k-1)||_2 / ||X_k||_2 of the last iteration k,
   * both sums in FP64 on the device (over all patches of a batch); 0 when no iteration ran */
  double rel_change;
} mlf_stats;

/* Library / ABI version (MLF_ABI_VERSION). */
int mlf_version(void);

/* Device characterisation: runs a register-only FP32 FMA kernel on the current device
 * for about `ms` milliseconds and returns the achieved FP32 rate in TFLOP/s (the
 * denominator the plain FP32 projector is judged against).  No counterpart in the
 * reference. */
int mlf_probe_fp32_peak(double ms, double* tflops, void* stream);

/* Failure-detection check: one thread waits, with the bounded mbarrier wait every
 * tensor-core kernel uses, on a barrier that nothing arrives at, for `limit` polls
 * (1..2^20, ~64 ns apart).  The wait gives up, the kernel records the timeout and returns,
 * and this returns MLF_ERR_TIMEOUT with the context still usable.  No counterpart in the
 * reference. */
int mlf_probe_wait_timeout(uint32_t limit, void* stream);

/* Copy the calling thread's last error message into buf (always NUL-terminated).
 * Returns the status code of that error. */
int mlf_last_error(char* buf, size_t len);

/* ---------------------------------------------------------------------------------
 * MEX projector.  Replaces mexFunction of src/cuda/mex_lfm_convolution_vec.cu:276-421
 * (kernel semantics :43-266):
 *   out(x,y,i) = sum_{kx,ky < kw} bitmap(x+kx-kw/2, y+ky-kw/2, i) * kernels(kx,ky,x%nnum,y%nnum)
 * zero outside the bitmap (the reference's edge clipping, :55-78).
 *   bitmap  : any, float32, W x H x n (column-major; W = MATLAB dims[0])
 *   kernels : any, float32, kw x kw x nnum x nnum
 *   out     : any, float32, W x H x n (fully written; the reference zero-initialises it)
 * Limits as the reference: 1 <= kw <= 341 (:41,344), n >= 1 (:332), nnum == 15 (:35).
 * Synchronous (the reference calls cudaDeviceSynchronize, :406). */
int mlf_conv_vec(const float* bitmap, int64_t W, int64_t H, int64_t n,
                 const float* kernels, int64_t kw, int32_t nnum, float* out, void* stream);
/* The same projector with a choice of method: MLF_CONV_DIRECT (CUDA-core FP32 correlation),
 * MLF_CONV_TENSOR (the correlation recast as the full forward projection of re-indexed
 * kernels, batched over the slices on the tensor cores with both operands split,
 * FP32-class accuracy; kernels up to 241 wide with a finite non-zero sum), MLF_CONV_AUTO
 * (the tensor cores from 1e11 flop when they apply, else direct; what mlf_conv_vec does). */
enum mlf_conv_method { MLF_CONV_AUTO = 0, MLF_CONV_DIRECT = 1, MLF_CONV_TENSOR = 2 };
int mlf_conv_vec_ex(const float* bitmap, int64_t W, int64_t H, int64_t n, const float* kernels, int64_t kw,
                    int32_t nnum, float* out, int32_t method, void* stream);
/* Sum of MEX projections in one pass, the "collect and forward-project" section of
 * src/gen_seed_library_local_with_ring_bg_same_size.m:257-318 (per depth z: the slices of
 * every segment at that depth projected with Ht(:,:,:,:,z), added to that segment's
 * accumulator; four kinds of slices).  out[:,:,o] = sum over the input slices j with
 * slot[j] = o of mex_lfm_convolution_vec(bitmaps[:,:,j], kernels[:,:,:,:,plane[j]]).
 * bitmaps W x H x n, kernels kw x kw x 15 x 15 x Z, out W x H x n_out (host or device);
 * plane[], slot[] host arrays of n.  On the tensor cores (one batched forward projection of
 * the re-indexed kernels, FP32-class accuracy) when kw <= 241 and every plane's kernel sum is
 * finite and non-zero; otherwise slice by slice with the direct kernel.  Synchronous. */
int mlf_conv_vec_accumulate(const float* bitmaps, int64_t W, int64_t H, int64_t n, const int32_t* plane,
                            const int32_t* slot, int64_t n_out, const float* kernels, int64_t kw, int32_t nnum,
                            int64_t Z, float* out, void* stream);

/* ---------------------------------------------------------------------------------
 * Summary image, the step that produces LFIMG.  Replaces
 * summary_image_generation_module(sensor_movie, patch_info, SI)
 * (src/module/summary_image_generation_module.m:43-133, with src/rank_1_factorization.m and
 * src/compute_std_image.m): rank-1 background by bg_iter alternating iterations, then
 *   MLF_DETREND_PIXELWISE: per pixel y = movie/max, y - movmean(y, window_1), movmean(., window_2),
 *                          .^poly_index, population std over the frames;
 *   MLF_DETREND_GLOBAL:    compute_std_image(movie/max, bg_spatial, bg_temporal) as written;
 * summary = image / max(image).  movie: P pixels x T frames, column-major (frame-contiguous),
 * host or device.  Outputs (host or device): summary P, bg_spatial P (Y t / max, not normalised
 * in the last iteration), bg_temporal T (unit norm); bg_spatial / bg_temporal may be NULL.
 * A negative std radicand (possible through compute_std_image's expansion) gives 0 where
 * MATLAB gives a complex value.  The global mode's Savitzky-Golay baseline is only plotted by
 * the reference and is not computed.  Synchronous. */
enum mlf_detrend_mode { MLF_DETREND_PIXELWISE = 0, MLF_DETREND_GLOBAL = 1 };
int mlf_summary_image(const float* movie, int64_t P, int64_t T, int32_t mode, int32_t bg_iter, int32_t window_1,
                      int32_t window_2, int32_t poly_index, float* summary_out, float* bg_spatial_out,
                      float* bg_temporal_out, void* stream);
/* The same, with the device time of each pass (CUDA events on `stream`) in pass_ms[5]:
 * first column pass (with the max), mean later column pass, mean row pass, last pass (the
 * image), finalisation (image max and scale); pass_ms may be NULL. */
int mlf_summary_image_ex(const float* movie, int64_t P, int64_t T, int32_t mode, int32_t bg_iter,
                         int32_t window_1, int32_t window_2, int32_t poly_index, float* summary_out,
                         float* bg_spatial_out, float* bg_temporal_out, double* pass_ms, void* stream);

/* ---------------------------------------------------------------------------------
 * Frame rectification, the step that produces the sensor movie.  Replaces the per-patch
 * part of image_load_module_aug(patch_info, SI) (src/module/image_load_module_aug.m:19-164)
 * on frames already in memory (reading the TIFF files stays with the caller):
 *   output frames i = 0 .. n_final-1, n_final = numel(frames_start:frames_step:min(n_frames, frames_end));
 *   frames_average != 0: output i is the mean of input frames
 *       frames_start + i*frames_step + j, j < frames_step (stopping at the last frame);
 *   otherwise output i is input frame frames_start + i*frames_step (frame numbers 1-based);
 *   each cut to raw_cut = {y0, y1, x0, x1} (1-based, inclusive; rows y, columns x) and
 *   rectified by img_rectify_mod (:126-164: griddedInterpolant bilinear with linear
 *   extrapolation onto the dx/Nnum grid anchored at (raw_cut_yCenter, raw_cut_xCenter),
 *   first lenslet aligned, cut to whole lenslets), which must give size_h x size_w
 *   (MLF_ERR_INVALID with the reference's message otherwise);
 *   normalize != 0: the movie is divided by its maximum (as the reference does).
 * frames: H x W x n_frames, column-major, MLF_DTYPE_U16 or MLF_DTYPE_F32, host or device
 * (from host memory only the cut region of the frames used is copied).  frames_end < 0 means
 * no end.  movie_out: (size_h*size_w) x n_final floats, column-major, host or device;
 * *n_out receives n_final (may be NULL).  Synchronous. */
enum mlf_dtype { MLF_DTYPE_F32 = 0, MLF_DTYPE_U16 = 1 };
int mlf_rectify_frames(const void* frames, int32_t dtype, int64_t H, int64_t W, int64_t n_frames,
                       const int64_t* raw_cut, double raw_cut_xCenter, double raw_cut_yCenter, int32_t Nnum,
                       double frames_dx, int64_t size_h, int64_t size_w, int64_t frames_start, int64_t frames_step,
                       int64_t frames_end, int32_t frames_average, int32_t normalize, float* movie_out,
                       int64_t* n_out, void* stream);

/* ---------------------------------------------------------------------------------
 * Phase-space PSF.  Replaces recon_theory_phase_space_LFM_with_filter.m:13-40 and
 * gen_phasespace_PSF_theory.m:1-31: per-depth FP64 normalisation of H and Ht, the
 * phase-space realignment of H, the crop of Ht, and the view weights (weight_cut 0.2,
 * scale 0.3).  H, Ht: any, float32, K0 x K0 x N x N x Z (MATLAB layout); K0 odd.
 * The result owns its HBM (per-view projector taps for every view). */
int mlf_psf_create(const float* H, const float* Ht, int64_t K0, int32_t N, int64_t Z,
                   mlf_psf** out, void* stream);
int mlf_psf_destroy(mlf_psf* psf);
/* Shape queries: N, Z, phase-space PSF side S. */
int mlf_psf_info(const mlf_psf* psf, int32_t* N, int64_t* Z, int64_t* S);
/* View weights (N x N, column-major, FP64) exactly as the solver uses them. */
int mlf_psf_weights(const mlf_psf* psf, double* w_host);
/* Bytes of HBM the PSF holds. */
int64_t mlf_psf_device_bytes(const mlf_psf* psf);

/* ---------------------------------------------------------------------------------
 * RL solve.  Replaces recon_theory_phase_space_LFM_with_filter(LFIMG, H, Ht, maxIter,
 * gpuFlag, gpu_id) (recon_theory_phase_space_LFM_with_filter.m:10-151): flat initial
 * guess sum(LFIMG)/numel, views in spiral order skipping zero weights, per view
 * forward projection -> ratio -> back projection -> multiplicative update -> blend,
 * and the flux-preserving NIP low-pass (sample_filter) after each iteration.
 *
 * mlf_solver_create sizes a context for Xr x Xc images (Xr, Xc multiples of N).
 *   lfimg      : any, float32, Xr x Xc
 *   warm_start : any or NULL, float32, Xr x Xc x Z (replaces the flat initial guess)
 *   vol_out    : any, float32, Xr x Xc x Z
 *   precision  : enum mlf_precision
 *   stats      : host, may be NULL
 * Synchronous when any pointer is host memory or stats != NULL. */
int mlf_solver_create(mlf_psf* psf, int64_t Xr, int64_t Xc, mlf_solver** out);
int mlf_solver_destroy(mlf_solver* s);
/* Solver variants.  MLF_VARIANT_PEELING is the solve inside
 * recon_theory_phase_space_LFM_with_filter_simple_peeling.m: filter bank of floor(Z/3)
 * rounded down to even (:55-58) and the update X .* C ./ (D + 1e-10) (:149). */
enum mlf_variant { MLF_VARIANT_BASE = 0, MLF_VARIANT_PEELING = 1 };
int mlf_solver_create_variant(mlf_psf* psf, int64_t Xr, int64_t Xc, int32_t variant, mlf_solver** out);
/* [Xguess, LFIMG, proj_sensor] = recon_theory_phase_space_LFM_with_filter_simple_peeling(
 *     LFIMG, H, Ht, maxIter, gpuFlag, gpu_id)  (…_simple_peeling.m:13-266), on a solver made
 * with MLF_VARIANT_PEELING: RL solve; forward-project the top plane and its >10 %-of-max
 * mask with the normalised H (all N*N views); scale the projection to the image over the
 * mask, subtract 0.9 of it from the image (clamped at 0); solve again from the flat guess;
 * put the first solve's top plane back.  lfimg, vol_out (Xr x Xc x Z) and the optional
 * lf_peeled_out / proj_sensor_out (Xr x Xc) are device pointers.  The top-plane
 * projections run in FP32 for MLF_PREC_FP32 and on the tensor cores with both operands
 * split (MLF_PREC_BF16X3) otherwise.  Stream-ordered; synchronous when stats != NULL. */
int mlf_solver_run_peeling(mlf_solver* s, const float* lfimg, int32_t max_iter, int32_t precision,
                           float* vol_out, float* lf_peeled_out, float* proj_sensor_out, mlf_stats* stats,
                           void* stream);
int64_t mlf_solver_device_bytes(const mlf_solver* s);
int mlf_solver_run(mlf_solver* s, const float* lfimg, int32_t max_iter, int32_t precision,
                   const float* warm_start, float* vol_out, mlf_stats* stats, void* stream);

/* ---------------------------------------------------------------------------------
 * Batched solve of independent patches (the reference solves patches one MATLAB process
 * at a time: mesolf.m:55-98 with SI.worker_ix).  All patches share one PSF; patch k has
 * Xr[k] x Xc[k] pixels (multiples of N, uneven sizes allowed) and uses the PSF planes
 * [z0[k], z0[k] + nz[k]) -- its result equals a solve with the PSF cut to those planes
 * (per-depth normalisation makes a plane range a PSF of its own; the view weights are
 * recomputed for the range).  Each view step of all patches is one launch of the
 * tensor-core GEMMs over the concatenated lenslet positions; precision must be one of the
 * tensor-core modes (MLF_PREC_BF16*, MLF_PREC_FP16*).  lfimg[k], warm[k] (warm may be NULL or hold NULLs) and vol_out[k]
 * (Xr[k] x Xc[k] x nz[k]) are device pointers.  Synchronous when stats != NULL. */
int mlf_batch_create(mlf_psf* psf, int32_t npatch, const int64_t* Xr, const int64_t* Xc, const int32_t* z0,
                     const int32_t* nz, mlf_batch** out);
int mlf_batch_destroy(mlf_batch* b);
/* Device bytes mlf_batch_create would allocate for these patches (an upper bound, for
 * admission by free HBM before creating the work set; it includes the convergence-monitor
 * volume that the first solve with stats allocates).  No allocation. */
int mlf_batch_plan_bytes(const mlf_psf* psf, int32_t npatch, const int64_t* Xr, const int64_t* Xc,
                         const int32_t* z0, const int32_t* nz, int64_t* bytes);
int64_t mlf_batch_device_bytes(const mlf_batch* b);
/* A run may leave patches out: lfimg[k] == NULL means patch k sits this run out (its
 * weights are 0 for every view, so its tiles are skipped; warm[k] and vol_out[k] are not
 * touched and may be NULL).  A serving loop sizes one work set for all its patches once and
 * runs any subset of them, so no work set is created on the request path.  At least one
 * patch must have an image. */
int mlf_batch_run(mlf_batch* b, const float* const* lfimg, int32_t max_iter, int32_t precision,
                  const float* const* warm, float* const* vol_out, mlf_stats* stats, void* stream);

/* Cancellation (failure handling of a serving loop: a request withdrawn while its solve
 * runs).  mlf_batch_cancel / mlf_solver_cancel may be called from any host thread while a
 * run of that work set is in progress: they set a word in mapped pinned host memory that
 * the first CTA of every view-step kernel reads; from the next view step on, every kernel
 * of the run returns at entry (before any barrier or TMEM allocation), and the run's output
 * volumes are left unwritten (a warm-start volume passed as both warm and output keeps the
 * previous frame).  A run with stats (synchronous) then returns MLF_ERR_CANCELLED; for a
 * stream-ordered run, mlf_batch_cancelled / mlf_solver_cancelled tell, once the stream has
 * been synchronised, whether the last run stopped early.  The next run clears the request
 * when it starts.  No counterpart in the reference (its MATLAB loop has none; the peeling
 * variant's retry loop, …_simple_peeling.m:122-178, restarts a failed solve instead). */
int mlf_batch_cancel(mlf_batch* b);
int mlf_batch_cancelled(const mlf_batch* b);
int mlf_solver_cancel(mlf_solver* s);
int mlf_solver_cancelled(const mlf_solver* s);

/* One-shot form with the reference's argument order (H, Ht raw PSFs).  Builds the PSF
 * and a solver, runs, frees.  Synchronous. */
int mlf_rl_solve(const float* lfimg, int64_t Xr, int64_t Xc, const float* H, const float* Ht,
                 int64_t K0, int32_t N, int64_t Z, int32_t max_iter, int32_t precision,
                 float* vol_out, mlf_stats* stats, void* stream);

/* ---------------------------------------------------------------------------------
 * Building blocks of one RL view, exposed for parity tests and for callers that drive
 * the view loop themselves.  (u, v) are 0-based view indices; volumes are Xr x Xc x Z
 * float32 device arrays in MATLAB layout.
 *
 * Forward projection of one view: recon_…_with_filter.m:243-249
 *   hx (dev, Xr/N x Xc/N) = (sum_z conv2(vol_z, Hps(:,:,u,v,z), 'same'))((N+1)/2:N:end, ...) */
int mlf_forward_view(mlf_solver* s, const float* vol, int32_t u, int32_t v, float* hx, void* stream);
/* Back projection of one view: recon_…_with_filter.m:211-220
 *   out (dev, Xr x Xc x Z): out_z = conv2(B, Ht(:,:,u,v,z), 'same'), B(u:N:end, v:N:end) = proj */
int mlf_backward_view(mlf_solver* s, const float* proj, int32_t u, int32_t v, float* out, void* stream);

/* One view of the RL inner loop, recon_…_with_filter.m:109-137: forward projection of
 * view (u, v), ratio with LFIMG(u:N:end, v:N:end), back projection, update with weight w.
 *   lfimg (dev, Xr x Xc); vol (dev, Xr x Xc x Z) updated in place.
 * Uses the solver's volume buffer as scratch. */
int mlf_rl_view_step(mlf_solver* s, const float* lfimg, float* vol, int32_t u, int32_t v, double w,
                     void* stream);
/* The same view step and forward projection at a given enum mlf_precision (the
 * tensor-core forms for MLF_PREC_BF16* and MLF_PREC_FP16*). */
int mlf_rl_view_step_prec(mlf_solver* s, const float* lfimg, float* vol, int32_t u, int32_t v, double w,
                          int32_t precision, void* stream);
int mlf_forward_view_prec(mlf_solver* s, const float* vol, int32_t u, int32_t v, int32_t precision,
                          float* hx, void* stream);
/* Full light-field forward projection of a volume, the reference's forwardProjectGPU
 * (src/recon/forwardProjectGPU.m:1-20; CPU twin forwardProjectACC.m:1-18 without the
 * CAindex crop): LF = sum_{a,b,z} conv2(vol_z .* [phase (a,b)], H(:,:,a,b,z), 'same').
 * Evaluated through the phase-space operator: pixel (u + N*i, v + N*j) of the LF image is
 * view (u, v)'s forward projection at lenslet (i, j), for all N*N views.  This equals the
 * reference's sum wherever each H(:,:,a,b,z) lies inside the phase-space crop of side
 * S = K0 - mod(K0 - N, 2N) (gen_phasespace_PSF_theory.m:8-9).  raw_psf = 1 projects with H
 * as given; raw_psf = 0 with the per-plane normalised H (the operator the RL solve uses).
 * vol (dev, Xr x Xc x Z) and lf_out (dev, Xr x Xc).  Stream-ordered. */
int mlf_forward_project(mlf_solver* s, const float* vol, float* lf_out, int32_t raw_psf, int32_t precision,
                        void* stream);
/* The same for every patch of a batch (vols[k]: Xr[k] x Xc[k] x nz[k], projected with
 * the PSF planes [z0[k], z0[k] + nz[k])), on the tensor cores (MLF_PREC_BF16*, MLF_PREC_FP16*). */
int mlf_batch_forward_project(mlf_batch* b, const float* const* vols, float* const* lf_out, int32_t raw_psf,
                              int32_t precision, void* stream);
/* The per-iteration flux-preserving NIP low-pass, sample_filter (recon_…_with_filter.m:222-240,
 * filter bank :44-61), applied in place to vol (dev, Xr x Xc x Z). */
int mlf_sample_filter(mlf_solver* s, float* vol, void* stream);

/* Forward projection of one view that allocates no device memory (no counterpart in the
 * reference; the regular form is mlf_forward_view).  For callers that cannot call
 * cudaMalloc/cudaFree: a MEX function working inside MATLAB's GPU memory manager, or a
 * frame callback of the acquisition loop that must not block on the device-wide
 * synchronisation allocation can cause.  Same result as mlf_forward_view(u, v):
 *   hx (dev, Xr/N x Xc/N) = (sum_z conv2(vol_z, Hps(:,:,u,v,z), 'same'))((N+1)/2:N:end, ...)
 * for vol (dev, Xr x Xc x Z, MATLAB layout), with the PSF's resident taps.
 * Scratch: a static device array of 2 Mi floats (8 MiB) that every GPU loading the
 * library holds until exit.  Limit: one CTA covers the whole lenslet grid in 4 x 8 tiles,
 * so ceil((Xr/N)/4) * ceil((Xc/N)/8) must not exceed 256 (e.g. 67 x 67 lenslets: 17 * 9 =
 * 153; 64 x 128 at most) -- MLF_ERR_UNSUPPORTED otherwise.  The array's address is looked
 * up on every call with the caller's device current (a reset device may place it
 * elsewhere); the first call on a device, and the first after a cudaDeviceReset, loads the
 * library's device code: make it before any stream capture.  Calls share the array, so
 * calls whose kernels overlap on the GPU (other streams or threads) race and must be
 * serialised by the caller. */
int mlf_forward_view_static(const mlf_psf* psf, const float* vol, int64_t Xr, int64_t Xc, int32_t u,
                            int32_t v, float* hx, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MESOLF_LF_H */
