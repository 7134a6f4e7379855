// Internal structures shared by the translation units of libmesolf_lf.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "mesolf_lf.h"

namespace mlf {

// ------------------------------------------------------------------ error plumbing
int fail(int code, const std::string& msg);  // records the message, returns code
void clear_error();

#define MLF_CUDA(call)                                                              \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return ::mlf::fail(MLF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// after a kernel launch: report the launch site with the error
#define MLF_LAUNCHED()                                                                           \
  do {                                                                                           \
    cudaError_t e_ = cudaGetLastError();                                                         \
    if (e_ != cudaSuccess)                                                                       \
      return ::mlf::fail(MLF_ERR_CUDA, std::string(__FILE__).substr(std::string(__FILE__).rfind('/') + 1) + \
                                           ":" + std::to_string(__LINE__) + ": kernel launch: " + \
                                           cudaGetErrorString(e_));                              \
  } while (0)

// precision modes (enum mlf_precision)
inline bool prec_valid(int p) { return p >= MLF_PREC_FP32 && p <= MLF_PREC_FP16X3; }
inline bool prec_tensor(int p) { return prec_valid(p) && p != MLF_PREC_FP32; }
inline bool prec_f16(int p) { return p >= MLF_PREC_FP16 && p <= MLF_PREC_FP16X3; }
constexpr int kPrecModes = MLF_PREC_FP16X3 + 1;

#define MLF_TRY(call)             \
  do {                            \
    int st_ = (call);             \
    if (st_ != MLF_OK) return st_; \
  } while (0)

// Device allocation owned by a host object.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  int alloc(size_t n, const char* what);
  void release();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// Cancellation of a run in progress (mlf_solver_cancel / mlf_batch_cancel).  `req` is a
// word of mapped pinned host memory that the host sets; thread 0 of the first CTA of every
// view-step kernel (k_view, k_tc_bwd) reads it and, when set, raises `stop` (device memory,
// which every CTA of every later kernel checks at entry before any barrier, so the rest of
// the run's view steps return at once) and `stopped_host` (mapped, read by the host after
// the stream is synchronised).  The kernels that write a run's outputs skip them when `stop`
// is set, so a cancelled run leaves its outputs (e.g. a warm-start volume) as they were.
// begin() clears the request on the host and both stop words in stream order.
struct CancelState {
  int* host = nullptr;      // [0] request (host writes), [1] stopped (device writes), mapped
  int* req_dev = nullptr;   // device addresses of host[0] and host[1]
  int* stopped_dev = nullptr;
  DevBuf stop;              // int on the device: the kernels' entry check
  CancelState() = default;
  CancelState(const CancelState&) = delete;
  CancelState& operator=(const CancelState&) = delete;
  ~CancelState();
  int init();                 // allocates: outside any stream capture
  int begin(cudaStream_t st);
  void request() const;       // any thread
  bool stopped() const;       // after the run's stream has been synchronised
};
// the kernels' view of a CancelState (all null: not cancellable)
struct CancelRef {
  const int* req;
  int* stopped_host;
  int* stop;
};
inline CancelRef cancel_ref(const CancelState& c) { return CancelRef{c.req_dev, c.stopped_dev, c.stop.as<int>()}; }

// Serialises CUDA graph captures against device memory allocation and release in this
// library (cudaFree synchronises the device, which would invalidate a capture running
// on another thread).  Recursive: releases can nest inside locked regions.
std::recursive_mutex& device_mutex();

// true if ptr is device (or managed) memory usable by kernels on the current device
bool is_device_ptr(const void* ptr);

// Allow `func` the device's whole opt-in dynamic shared memory (minus its static usage).
// The attribute is global to the function, so it is never lowered for one caller's size.
int allow_max_dyn_smem(const void* func);

struct TcPsfState;     // tensor-core operands of a PSF (mlf_tc.cu)
struct TcSolverState;  // tensor-core work set of one or more patches (mlf_tc.cu)
void tc_psf_free(TcPsfState* t);
void tc_solver_free(TcSolverState* t);

// Where a patch's volume lives in a phase-major buffer: channel
// ch = (beta*N + alpha)*Zch + z0 + z (z < Z planes of the patch), or, plane-major (pm = 1),
// ch = (z0 + z)*N*N + beta*N + alpha; position b*Pa + a inside a plane of `plane` floats.
// The plain FP32 solver uses Zch = Z, z0 = 0, Pa padded to 4, channel-major order; the
// tensor-core work set uses Pa = Li, one plane spanning all its patches, and the plane-major
// order, so that a patch's plane range is one contiguous channel range.
struct PatchGeo {
  int N, Z, Zch, z0, Li, Lj, Pa;
  int64_t plane, Xr, Xc;
  int pm;
};
__host__ __device__ inline int64_t geo_channel(const PatchGeo& g, int alpha, int beta, int z) {
  return g.pm ? (int64_t)(g.z0 + z) * g.N * g.N + beta * g.N + alpha
              : ((int64_t)beta * g.N + alpha) * g.Zch + g.z0 + z;
}
// plane of channel ch relative to z0 (outside [0, Z) for the other planes)
__host__ __device__ inline int geo_plane(const PatchGeo& g, int64_t ch) {
  return (g.pm ? (int)(ch / ((int64_t)g.N * g.N)) : (int)(ch % g.Zch)) - g.z0;
}

// ------------------------------------------------------------------ PSF
// Per-view projector taps in phase-major ("polyphase") form.  For view (u, v) (0-based,
// view = u + N*v) and volume channel ch = (beta*N + alpha)*Z + z the forward taps are
//   wf[view][ch][db*T + da] = Hps_z[N(2q-da) + N-1-alpha, N(2q-db) + N-1-beta]
// and the backward taps
//   wb[view][ch][dj*T + di] = Htc_z[N(2q-di) + f_alpha, N(2q-dj) + f_beta],
//   f_alpha = (alpha - u + h) mod N,  h = (N-1)/2,  T = 2q+1 = S/N.
struct Psf {
  int device = 0;
  int N = 0, Z = 0, K0 = 0, S = 0, q = 0, T = 0;
  int64_t nch = 0;           // N*N*Z volume channels
  int64_t taps_per_view = 0; // nch * T * T
  DevBuf wf, wb;             // float [N*N][nch][T*T]
  std::vector<double> weights;  // N*N, index u + N*v (MATLAB weight(u+1, v+1))
  std::vector<double> wsum_vz;  // [N*N][Z] FP64 sums of Hps(:,:,u,v,z) (weights of plane ranges)
  std::vector<double> hsum_z;   // [Z] FP64 sums of the raw H(:,:,:,:,z)
  DevBuf hsum_dev;              // float [Z], the same on the device
  std::vector<int> view_order;  // active views in spiral order (view = u + N*v)
  std::vector<int> spiral;      // all N*N views in spiral order
  TcPsfState* tc = nullptr;     // built on the first tensor-core solve
  ~Psf() { tc_psf_free(tc); }
  size_t bytes() const;
};

// ------------------------------------------------------------------ solver
struct FilterPlan {
  // sample_filter as separable circular convolutions.  For bank entry e the 1-D kernels
  // are cx_e (length Xr) and cy_e (length Xc) with half-widths Wx_e / Wy_e.
  int n_entries = 0;
  std::vector<int> plane_entry;  // per plane: bank entry or -1 (pass-through)
  std::vector<int> wx, wy;       // per entry half-width
  DevBuf cx, cy;                 // float [n_entries][Xr] / [n_entries][Xc], index = offset d mod len
  DevBuf plane_entry_dev;        // int [Z]
  DevBuf wx_dev, wy_dev;         // int [n_entries]
  DevBuf sums;                   // double [2][Z][max_blocks] partial flux sums
  int max_blocks = 0;
};

struct Solver {
  Psf* psf = nullptr;
  int device = 0;
  int variant = MLF_VARIANT_BASE;  // MLF_VARIANT_PEELING: floor-rounded filter bank, D + 1e-10
  int64_t Xr = 0, Xc = 0;
  int N = 0, Z = 0, Li = 0, Lj = 0, q = 0, T = 0;
  int Pa = 0;          // row pitch (floats) of a phase-major plane (FP32 kernels)
  int64_t plane = 0;   // floats per plane (Lj * Pa)
  int64_t nch = 0;
  // view-kernel geometry
  int tilesA = 0, tilesB = 0, tps = 0, slots = 0, tstride = 0, threads = 0, grid = 0;
  int RP = 0, RProws = 0, XP = 0, XProws = 0, maxc = 0;
  size_t smem = 0;
  int ncA[3] = {0, 0, 0}, ncB[3] = {0, 0, 0};
  DevBuf X;          // float [nch][plane]      phase-major volume
  DevBuf Xtmp;       // float [nch][plane]      scratch volume (back-projection output, filter)
  DevBuf lfs;        // float [N*N][Lj*Li]      sub-aperture images
  DevBuf rpad;       // float [RProws][RP]      halo-padded ratio image
  DevBuf part;       // float [grid*slots][tilesB*VW_TY][tilesA*VW_TX] per-slot forward partials
  DevBuf hx;         // float [Lj*Li]           last forward projection
  DevBuf cls;        // int tables: clsA[3][Li], clsB[3][Lj], rngA[3][maxc][2], rngB[3][maxc][2]
  DevBuf red;        // double scratch for reductions
  DevBuf stage_in, stage_out;  // device staging for host arrays
  DevBuf Xprev;      // float [nch][plane]      volume at the start of the iteration (stats only)
  DevBuf relbuf;     // double: block partials and the relative change of the last iteration
  FilterPlan filt;
  // optional per-launch timing of the projector kernels (enabled when stats are requested)
  std::vector<cudaEvent_t> tev;
  int tev_used = 0;
  bool timing = false;
  bool lite = false;            // batch member: geometry, filter plan and filter scratch only
  bool lite_ready = false;      // ... the latter two built by lite_prepare on the first solve
  int z0 = 0;                   // first PSF plane of this patch (batch members)
  CancelState cancel;           // cancellation of the solver's plain FP32 runs
  bool last_run_tc = false;     // the last run took the tensor-core path (its work set's CancelState)
  TcSolverState* tc = nullptr;  // built on the first tensor-core solve
  ~Solver();
  size_t bytes() const;
};

// ------------------------------------------------------------------ entry points used across TUs
int psf_build(Psf* psf, const float* dH, const float* dHt, cudaStream_t st);
int solver_init(Solver* s);
int solver_run(Solver* s, const float* d_lf, int max_iter, int precision, const float* d_warm,
               float* d_out, mlf_stats* stats, cudaStream_t st);
int forward_view(Solver* s, const float* d_vol, int u, int v, float* d_hx, cudaStream_t st);
int backward_view(Solver* s, const float* d_proj, int u, int v, float* d_out, cudaStream_t st);
int rl_view_step(Solver* s, const float* d_lf, float* d_vol, int u, int v, double w, int precision,
                 cudaStream_t st);
// layout kernels on an arbitrary PatchGeo (mlf_rl.cu)
int launch_extract_views(const float* d_lf, const PatchGeo& g, float* lfs, int64_t view_stride, int64_t off,
                         cudaStream_t st);
int launch_to_phase(const float* d_vol, const PatchGeo& g, float* X, cudaStream_t st,
                    const float* zscale = nullptr);
int launch_scatter_views(const float* lfs, const PatchGeo& g, float* d_lf, int64_t view_stride, int64_t off,
                         cudaStream_t st);
int forward_project(Solver* s, const float* d_vol, float* d_lf, const float* d_zscale, int precision,
                    cudaStream_t st);
// the peeling variant's two solves and top-plane peel (…_simple_peeling.m:13-266)
int peel_solve(Solver* s, const float* d_lf, int max_iter, int precision, float* d_out, float* d_lf_peeled,
               float* d_proj, mlf_stats* stats, cudaStream_t st);
inline float solver_d_eps(const Solver* s) { return s->variant == MLF_VARIANT_PEELING ? 1e-10f : 0.f; }
// skip (nullable): a device word; the copy is skipped when it is non-zero (a cancelled run)
int launch_from_phase(const float* X, const PatchGeo& g, float* d_vol, cudaStream_t st, const int* skip = nullptr);
// flat initial guess sum(lf)/(Xr*Xc*Z) on the patch's planes, 0 on the other channels
int launch_init_flat(const float* d_lf, const PatchGeo& g, float* X, double* scratch, cudaStream_t st);
// Convergence monitor: rel = ||X - Xprev||_2 / ||X||_2 over n floats, both sums in FP64
// (fixed-order reductions), then Xprev <- X.  `buf` holds kRelChangeBufDoubles doubles; the
// result is buf[0].  rel_change_prepare allocates Xprev / buf (not during a graph capture).
constexpr int kRelChangeBlocks = 512;
constexpr int kRelChangeBufDoubles = 2 * kRelChangeBlocks + 8;
int launch_rel_change(const float* X, float* Xprev, int64_t n, double* buf, cudaStream_t st);
int rel_change_read(const double* buf, double* out);
int filter_run_geo(Solver* s, const PatchGeo& g, float* X, cudaStream_t st);
PatchGeo solver_geo(const Solver* s);
std::vector<double> psf_range_weights(const Psf* p, int z0, int nz);
int rl_iteration_count_views(const std::vector<std::vector<double>>& w);
int forward_view_prec(Solver* s, const float* d_vol, int u, int v, int precision, float* d_hx, cudaStream_t st);
int sample_filter(Solver* s, float* d_vol, cudaStream_t st);
int filter_init(Solver* s);
// a batch member's filter plan and scratch, on first use (allocates: outside any capture)
int lite_prepare(Solver* s);
int timing_mark(Solver* s, cudaStream_t st);
// tensor-core path (mlf_tc.cu).  A work set covers P patches (P = 1 for a single solver);
// `members[p]` supplies each patch's geometry, filter plan and filter scratch.
int tc_psf_prepare(Psf* p, cudaStream_t st);
int tc_work_create(Psf* psf, const std::vector<Solver*>& members, TcSolverState** out, cudaStream_t st);
int tc_solver_prepare(Solver* s, cudaStream_t st);
// full solve: lf[p], warm[p] (nullable), out[p] device pointers in MATLAB layout
int tc_run(TcSolverState* w, const std::vector<Solver*>& members, const std::vector<const float*>& lf,
           const std::vector<const float*>& warm, const std::vector<float*>& out, int max_iter, int precision,
           mlf_stats* stats, Solver* timing_owner, cudaStream_t st);
int tc_forward_view(Solver* s, int precision, const float* d_vol, int view, float* hx_out, cudaStream_t st);
// full LF images of vols[p] (all N*N views), zscale as in forward_project
int tc_forward_project(TcSolverState* w, const std::vector<Solver*>& members, const std::vector<const float*>& vols,
                       const std::vector<float*>& lf_out, int precision, const float* zscale, cudaStream_t st);
int tc_view_step(Solver* s, int precision, const float* d_lf, float* d_vol, int view, float w, cudaStream_t st);
int tc_check_error(TcSolverState* w);
// the work set's cancellation state (created with the work set)
CancelState& tc_cancel_state(TcSolverState* w);
size_t tc_psf_bytes(const Psf* p);
size_t tc_solver_bytes(const Solver* s);
size_t tc_work_bytes(const TcSolverState* w);
// device bytes tc_work_create would allocate for patches of Li[p] x Lj[p] lenslets (upper bound)
size_t tc_work_plan_bytes(const Psf* psf, const std::vector<int>& Li, const std::vector<int>& Lj, int nsm);
int filter_run(Solver* s, cudaStream_t st);
int conv_vec_run(const float* d_bitmap, int64_t W, int64_t H, int64_t n, const float* d_kernels,
                 int64_t kw, int nnum, float* d_out, cudaStream_t st);
// pieces of the tensor-core route of the MEX projector (mlf_conv_vec.cu)
int summary_run(const float* dY, int64_t P, int64_t T, int mode, int bg_iter, int w1, int w2, int poly,
                float* d_img, float* d_s, float* d_t, double* pass_ms, cudaStream_t st);
int rectify_run(const void* d_raw, int dtype, int64_t total, int64_t fstride, int64_t cstride, int64_t row0, int64_t col0,
                int64_t h, int64_t w, double xc, double yc, int M, double dx, int64_t out_h, int64_t out_w,
                int64_t f0, int64_t fstep, int navg, int64_t flast, int64_t n_out, float* d_out, bool normalize,
                cudaStream_t st);
int launch_mex_reindex(const float* K, int kw, int K0, int nn, float* Hp, cudaStream_t st);
int launch_mex_pad(const float* bm, int64_t W, int64_t H, int64_t n, int64_t Wp, int64_t Hq, bool zero_last,
                   float* dst, cudaStream_t st);
int launch_mex_pad_add(const float* src, int64_t W, int64_t H, int64_t Wp, int64_t Hq, bool zero_last, float* dst,
                       cudaStream_t st);
int launch_mex_crop(const float* src, int64_t Wp, int64_t Hq, int64_t W, int64_t H, int64_t n, float* out,
                    cudaStream_t st);

// Entry check of the cancellable kernels, by thread 0 (the caller broadcasts the result to
// its CTA before any barrier): CTA 0 turns a host request into the stop words; every CTA
// then returns when the device stop word is set.
#ifdef __CUDACC__
__device__ __forceinline__ int cancel_entry(const CancelRef& c) {
  if (!c.stop) return 0;
  if (blockIdx.x == 0 && blockIdx.y == 0 && c.req && *reinterpret_cast<const volatile int*>(c.req) != 0) {
    *reinterpret_cast<volatile int*>(c.stop) = 1;
    *reinterpret_cast<volatile int*>(c.stopped_host) = 1;
  }
  return *reinterpret_cast<const volatile int*>(c.stop);
}
#endif

// view kernels (instantiated per tap count T in mlf_view_T*.cu)
struct ViewArgs {
  float* X;            // phase-major volume (read; written when updating)
  float* Cout;         // MODE_BWDC: phase-major back projection output
  const float* rpad;   // halo-padded ratio image
  const float* wb;     // backward taps of the current view [nch][T*T]
  const float* wf;     // forward taps of the view being projected [nch][T*T]
  float* part;         // [gridDim.x * slots][tilesB*VW_TY][tilesA*VW_TX] forward partials
  const int* clsA;     // [3][Li]
  const int* clsB;     // [3][Lj]
  const int* rngA;     // [3][maxc][2]
  const int* rngB;     // [3][maxc][2]
  float w;             // view weight
  float d_eps;         // added to D in the update (1e-10 in the peeling variant, else 0)
  int u, v;            // current view (backward / update)
  int do_fwd;          // MODE_STEP: also project with wf
  int N, Z, Li, Lj, Pa, q;
  int64_t plane, nch;
  int tilesA, tilesB, tps, slots, tstride;  // tstride: threads per slot (>= tps)
  int RP, RProws, XP, XProws, maxc, slot_floats;
  CancelRef cancel;    // all null: not cancellable
};
enum ViewMode { MODE_FWD = 0, MODE_STEP = 1, MODE_BWDC = 2 };

// View-kernel geometry shared by host and device (the tiles: VW_TY x VW_TX below for
// k_view, VT_TY x VT_TX in mlf_view.cuh for the allocation-free forward projection).
// Tap-row pitch of the view kernels' shared tap buffers:
constexpr int view_tap_pitch(int T) { return (T + 3) & ~3; }
// view_qpad(q) = round_up(q, 4) (16-byte aligned for cp.async), so the window offset of the
// forward correlation is view_qpad(q) - q; the back projection's is s_alpha + 1 in {0,1,2}.
constexpr int view_qpad(int q) { return (q + 3) & ~3; }
constexpr int view_offmax(int q) { return (view_qpad(q) - q) > 2 ? (view_qpad(q) - q) : 2; }
// float4 loads per window row: 4 outputs + T - 1 taps + the largest offset
constexpr int view_nw(int T) { return (4 + T - 1 + view_offmax((T - 1) / 2) + 3) / 4; }
// The view kernel's own tile (conv_rows in mlf_view.cuh): 4 b x 8 a, and its float4 loads
// per window row (8 outputs + T - 1 taps + the largest offset).  The tile of conv_tile
// above (8 b x 4 a) is the allocation-free forward projection's.
constexpr int VW_TY = 4;
constexpr int VW_TX = 8;
// threads per view-kernel CTA at most (two slots of up to 160 tiles)
constexpr int kViewMaxThreads = 320;
// Staged planes of the view kernel (ratio image, forward input) are stored with their
// 16-byte column chunks swizzled: in every other 32-float block the chunks of each pair
// trade places (column c lives at c ^ 4 when bit 5 of c is set), except a last chunk whose
// partner lies past the row.  With a row pitch of 4 mod 8 floats and the lane order of the
// view kernel, the 16-byte window loads of a warp meet 1.3 distinct rows per bank on
// average (2.6 unswizzled) at the 67 x 67 lenslet patch.
__host__ __device__ inline int view_pcol(int c, int pitch) {
  return ((c & 32) && (c | 4) < pitch) ? (c ^ 4) : c;
}
// Smallest pitch >= need (floats) that is 4 mod 8.
__host__ __device__ constexpr int view_plane_pitch(int need) { return ((need + 3) & ~7) + 4; }
constexpr int view_nw8(int T) { return (VW_TX + T - 1 + view_offmax((T - 1) / 2) + 3) / 4; }
int prepare_view_kernels(int T, size_t smem);
int occupancy_view_kernel(int T, int threads, size_t smem, int* blocks);
int launch_view_kernel(int T, int mode, const ViewArgs& a, int grid, int threads, size_t smem,
                       cudaStream_t st);
bool view_taps_supported(int T);

}  // namespace mlf
