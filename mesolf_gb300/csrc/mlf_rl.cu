// Phase-space Richardson-Lucy solve on one GPU (host orchestration + small kernels).
//
// recon_theory_phase_space_LFM_with_filter.m:72-146: flat initial guess, iterations of
// the spiral view loop (forward projection, ratio, back projection, update, blend) and
// the per-iteration sample_filter.  Each view step is one launch of the fused view
// kernel (back projection + D + update of view k, forward projection of view k+1) plus
// one launch of the partial-sum reduction that forms the next ratio image.  The
// mixed-precision (tensor-core) forms are in mlf_tc.cu; this file keeps the layout
// kernels, which take a PatchGeo so they also serve the patches of a batch.
#include <nvtx3/nvToolsExt.h>
#include <algorithm>
#include <cmath>
#include <map>
#include <utility>
#include <vector>

#include "mlf_internal.h"

namespace mlf {

namespace {

__device__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Sum of n floats into part[blockIdx.x] (FP64); fixed per-block order.
__global__ void k_sum_partial(const float* __restrict__ a, int64_t n, double* part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s += (double)a[i];
  s = warp_sum_d(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
    part[blockIdx.x] = r;
  }
}

// Flat initial guess, recon_…_with_filter.m:72-73: ones/sum(ones)*sum(LFIMG) on the
// patch's planes (channels whose z is outside [z0, z0+Z) get 0).  Only the valid
// positions of each plane are written (row padding stays as it is).
__global__ void k_init_flat(float* X, PatchGeo g, const double* part, int nparts, double inv_count) {
  __shared__ float val;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < nparts; ++i) s += part[i];
    val = (float)(inv_count * s);
  }
  __syncthreads();
  const int64_t LL = (int64_t)g.Li * g.Lj;
  const int64_t n = (int64_t)g.N * g.N * g.Zch * LL;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ch = i / LL;
    const int rem = (int)(i - ch * LL);
    const int z = geo_plane(g, ch);
    X[ch * g.plane + (int64_t)(rem / g.Li) * g.Pa + rem % g.Li] = (z >= 0 && z < g.Z) ? val : 0.f;
  }
}

__device__ __forceinline__ int64_t phase_index(const PatchGeo& g, int64_t e) {
  const int64_t r = e % g.Xr;
  const int64_t c = (e / g.Xr) % g.Xc;
  const int z = (int)(e / (g.Xr * g.Xc));
  const int alpha = (int)(r % g.N), a = (int)(r / g.N);
  const int beta = (int)(c % g.N), b = (int)(c / g.N);
  const int64_t ch = geo_channel(g, alpha, beta, z);
  return ch * g.plane + (int64_t)b * g.Pa + a;
}

// MATLAB (Xr, Xc, Z) volume -> phase-major planes; one thread per voxel of the input.
// zscale (nullable): per-plane factor applied on the way in.
__global__ void k_to_phase(const float* __restrict__ vol, PatchGeo g, float* __restrict__ X,
                           const float* __restrict__ zscale) {
  const int64_t n = g.Xr * g.Xc * g.Z;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    X[phase_index(g, e)] = zscale ? vol[e] * zscale[e / (g.Xr * g.Xc)] : vol[e];
}

__global__ void k_from_phase(const float* __restrict__ X, PatchGeo g, float* __restrict__ vol,
                             const int* __restrict__ skip) {
  if (skip && *reinterpret_cast<const volatile int*>(skip)) return;  // cancelled run: leave vol as it is
  const int64_t n = g.Xr * g.Xc * g.Z;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    vol[e] = X[phase_index(g, e)];
}

// Sub-aperture images, LFIMG(u:N:end, v:N:end) for every view u + N*v:
// lfs[view * view_stride + off + b*Li + a].
__global__ void k_extract_views(const float* __restrict__ lf, PatchGeo g, float* __restrict__ lfs,
                                int64_t view_stride, int64_t off) {
  const int64_t n = g.Xr * g.Xc;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e % g.Xr, c = e / g.Xr;
    const int u = (int)(r % g.N), a = (int)(r / g.N);
    const int v = (int)(c % g.N), b = (int)(c / g.N);
    lfs[(int64_t)(u + g.N * v) * view_stride + off + (int64_t)b * g.Li + a] = lf[e];
  }
}

// ---- top-plane peeling (…_simple_peeling.m:183-205)
constexpr int kPeelBlocks = 256;

__global__ void k_max_partial(const float* __restrict__ a, int64_t n, float* part) {
  __shared__ float sh[32];
  float m = -INFINITY;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, a[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) m = fmaxf(m, sh[i]);
    part[blockIdx.x] = fmaxf(m, sh[0]);
  }
}

// sum(m .* a) and sum(m .* b) per block (FP64), into part[blockIdx] and part[gridDim + blockIdx]
__global__ void k_dot2_partial(const float* __restrict__ m, const float* __restrict__ a,
                               const float* __restrict__ b, int64_t n, double* part) {
  __shared__ double sh[2][32];
  double sa = 0.0, sb = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    sa += (double)m[i] * a[i];
    sb += (double)m[i] * b[i];
  }
  sa = warp_sum_d(sa);
  sb = warp_sum_d(sb);
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = sa;
    sh[1][threadIdx.x >> 5] = sb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ra = 0.0, rb = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      ra += sh[0][i];
      rb += sh[1][i];
    }
    part[blockIdx.x] = ra;
    part[gridDim.x + blockIdx.x] = rb;
  }
}

// plane 0 of the mask volume: top > 0.1 * max(top)   (:190)
__global__ void k_peel_mask(const float* __restrict__ top, int64_t n, const float* maxpart, int nb,
                            float* __restrict__ vol) {
  __shared__ float thr;
  if (threadIdx.x == 0) {
    float m = -INFINITY;
    for (int i = 0; i < nb; ++i) m = fmaxf(m, maxpart[i]);
    thr = (float)((double)m * 0.1);
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    vol[i] = top[i] > thr ? 1.f : 0.f;
}

// proj *= sum(pm .* LF) / sum(pm .* proj) with pm = projm / sum(projm)  (:195-199);
// LF2 = max(LF - 0.9 * proj, 0)  (:202-203)
__global__ void k_peel_apply(const float* __restrict__ lf, const float* __restrict__ proj, int64_t n,
                             const double* sum_m, const double* dots, int nb, float* __restrict__ lf2,
                             float* __restrict__ proj_out) {
  __shared__ float scale;
  if (threadIdx.x == 0) {
    double sm = 0.0, a = 0.0, b = 0.0;
    for (int i = 0; i < nb; ++i) {
      sm += sum_m[i];
      a += dots[i];
      b += dots[nb + i];
    }
    scale = (float)((a / sm) / (b / sm));
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float p = proj[i] * scale;
    proj_out[i] = p;
    const float r = lf[i] - p * 0.9f;
    lf2[i] = r < 0.f ? 0.f : r;
  }
}

// Inverse of k_extract_views: LF(u + N*a, v + N*b) = lfs[(u + N*v) * view_stride + off + b*Li + a].
__global__ void k_scatter_views(const float* __restrict__ lfs, PatchGeo g, float* __restrict__ lf,
                                int64_t view_stride, int64_t off) {
  const int64_t n = g.Xr * g.Xc;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e % g.Xr, c = e / g.Xr;
    const int u = (int)(r % g.N), a = (int)(r / g.N);
    const int v = (int)(c % g.N), b = (int)(c / g.N);
    lf[e] = lfs[(int64_t)(u + g.N * v) * view_stride + off + (int64_t)b * g.Li + a];
  }
}

// HX = sum of the per-slot forward partials (fixed order).  Optionally writes HX and the
// ratio image R = LF_sub ./ HX with non-finite -> 0 (recon_…_with_filter.m:116-117) into
// the halo-padded buffer read by the next view kernel.  A partial plane holds row b of the
// lenslet grid at b * HP (HP >= Li, the view kernel's tile-padded width), planes PPL floats
// apart.  One block covers 32 positions (lanes); its 8 warps take the partials k = w, w+8,
// ... with four accumulators each, and the warps' sums are added in a fixed order
// (deterministic).
constexpr int kReduceGroups = 8;
__global__ void __launch_bounds__(32 * kReduceGroups)
k_reduce_ratio(const float* __restrict__ part, int nparts, int Li, int Lj, int HP, int64_t PPL,
               const float* __restrict__ lfsub, float* __restrict__ hx_out,
               float* __restrict__ rpad, int RP, int off) {
  __shared__ float sh[kReduceGroups][32];
  const int LL = Li * Lj;
  const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  const int a = i % Li, b = i / Li;
  const float* pp = part + (int64_t)b * HP + a;
  float s = 0.f;
  if (i < LL) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int k = grp;
    for (; k + 3 * kReduceGroups < nparts; k += 4 * kReduceGroups) {
      s0 += pp[k * PPL];
      s1 += pp[(k + kReduceGroups) * PPL];
      s2 += pp[(k + 2 * kReduceGroups) * PPL];
      s3 += pp[(k + 3 * kReduceGroups) * PPL];
    }
    for (; k < nparts; k += kReduceGroups) s0 += pp[k * PPL];
    s = (s0 + s1) + (s2 + s3);
  }
  sh[grp][lane] = s;
  __syncthreads();
  if (grp != 0 || i >= LL) return;
  float hx = 0.f;
#pragma unroll
  for (int g = 0; g < kReduceGroups; ++g) hx += sh[g][lane];
  if (hx_out) hx_out[i] = hx;
  if (rpad) {
    float r = lfsub[i] / hx;
    if (!isfinite(r)) r = 0.f;
    rpad[(b + off) * RP + view_pcol(a + off, RP)] = r;  // swizzled plane columns
  }
}

// proj (Li x Lj, MATLAB layout) into the interior of the halo-padded ratio buffer.
__global__ void k_fill_rpad(const float* __restrict__ proj, int Li, int Lj, float* rpad, int RP,
                            int off) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Li * Lj) return;
  const int a = i % Li, b = i / Li;
  rpad[(b + off) * RP + view_pcol(a + off, RP)] = proj[i];  // swizzled plane columns
}

inline int ceil_div(int a, int b) { return (a + b - 1) / b; }
inline int round_up(int a, int b) { return ceil_div(a, b) * b; }

int grid_for(int64_t n, int threads = 256) {
  int64_t g = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 16));
}


ViewArgs view_args(Solver* s) {
  ViewArgs a{};
  const int* cls = s->cls.as<int>();
  a.X = s->X.as<float>();
  a.Cout = nullptr;
  a.rpad = s->rpad.as<float>();
  a.part = s->part.as<float>();
  a.clsA = cls;
  a.clsB = cls + 3 * s->Li;
  a.rngA = cls + 3 * s->Li + 3 * s->Lj;
  a.rngB = a.rngA + 3 * s->maxc * 2;
  a.d_eps = solver_d_eps(s);
  a.N = s->N; a.Z = s->Z; a.Li = s->Li; a.Lj = s->Lj; a.Pa = s->Pa; a.q = s->q;
  a.plane = s->plane; a.nch = s->nch;
  a.tilesA = s->tilesA; a.tilesB = s->tilesB; a.tps = s->tps; a.slots = s->slots; a.tstride = s->tstride;
  a.RP = s->RP; a.RProws = s->RProws; a.XP = s->XP; a.XProws = s->XProws; a.maxc = s->maxc;
  a.cancel = CancelRef{nullptr, nullptr, nullptr};  // solves set it (enqueue_iteration)
  a.slot_floats = round_up(s->XProws * s->XP + 4 * s->T * view_tap_pitch(s->T) + s->maxc * s->maxc + s->T * s->maxc, 4);
  return a;
}

const float* wf_of(const Solver* s, int view) {
  return s->psf->wf.as<float>() + (int64_t)view * s->psf->taps_per_view;
}
const float* wb_of(const Solver* s, int view) {
  return s->psf->wb.as<float>() + (int64_t)view * s->psf->taps_per_view;
}

// D-table classes: for output coarse index a and channel shift s in {-1,0,1}, the valid
// taps are di in [max(0, q-s-a), min(2q, L-1-a-s+q)].  Identical (lo, hi) pairs share a
// class.
void build_classes(int L, int q, std::vector<int>& cls, std::vector<std::pair<int, int>> rng[3],
                   int nc[3]) {
  cls.assign(3 * L, 0);
  for (int s = -1; s <= 1; ++s) {
    std::map<std::pair<int, int>, int> id;
    rng[s + 1].clear();
    for (int a = 0; a < L; ++a) {
      int lo = std::max(0, q - s - a);
      int hi = std::min(2 * q, L - 1 - a - s + q);
      if (lo > hi) { lo = 1; hi = 0; }
      auto key = std::make_pair(lo, hi);
      auto it = id.find(key);
      int c;
      if (it == id.end()) {
        c = (int)rng[s + 1].size();
        id[key] = c;
        rng[s + 1].push_back(key);
      } else {
        c = it->second;
      }
      cls[(s + 1) * L + a] = c;
    }
    nc[s + 1] = (int)rng[s + 1].size();
  }
}

}  // namespace

int timing_mark(Solver* s, cudaStream_t st) {
  if (!s->timing) return MLF_OK;
  if (s->tev_used >= (int)s->tev.size()) {
    const size_t grow = std::max<size_t>(256, s->tev.size());
    for (size_t k = 0; k < grow; ++k) {
      cudaEvent_t e;
      MLF_CUDA(cudaEventCreate(&e));
      s->tev.push_back(e);
    }
  }
  // Inside a stream capture the record must become a graph node of its own.
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  MLF_CUDA(cudaStreamIsCapturing(st, &cs));
  MLF_CUDA(cudaEventRecordWithFlags(s->tev[s->tev_used++], st,
                                    cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal
                                                                        : cudaEventRecordDefault));
  return MLF_OK;
}

namespace {

int run_view(Solver* s, int mode, int view_cur, int view_next, float w, bool do_fwd,
             cudaStream_t st, bool cancellable = false) {
  MLF_TRY(timing_mark(s, st));
  ViewArgs a = view_args(s);
  if (cancellable) a.cancel = cancel_ref(s->cancel);
  const int N = s->N;
  a.u = view_cur % N;
  a.v = view_cur / N;
  a.w = w;
  a.do_fwd = do_fwd ? 1 : 0;
  a.wb = wb_of(s, view_cur);
  a.wf = wf_of(s, view_next >= 0 ? view_next : view_cur);
  MLF_TRY(launch_view_kernel(s->T, mode, a, s->grid, s->threads, s->smem, st));
  return timing_mark(s, st);
}

int run_reduce(Solver* s, int view, float* hx_out, bool ratio, cudaStream_t st) {
  const int LL = s->Li * s->Lj;
  const float* lfsub = s->lfs.as<float>() + (int64_t)view * LL;
  const int HP = s->tilesA * VW_TX;
  k_reduce_ratio<<<ceil_div(LL, 32), 32 * kReduceGroups, 0, st>>>(
      s->part.as<float>(), s->grid * s->slots, s->Li, s->Lj, HP, (int64_t)s->tilesB * VW_TY * HP, lfsub, hx_out,
      ratio ? s->rpad.as<float>() : nullptr, s->RP, s->q + 1);
  MLF_LAUNCHED();
  return MLF_OK;
}

// One RL iteration of the plain FP32 path (recon_…_with_filter.m:100-142), stream-ordered.
int enqueue_iteration(Solver* s, int64_t* launches, cudaStream_t st) {
  const std::vector<int>& views = s->psf->view_order;
  const int V = (int)views.size();
  int64_t n = 0;
  if (V > 0) {
    MLF_TRY(run_view(s, MODE_FWD, views[0], views[0], 0.f, true, st, true));
    MLF_TRY(run_reduce(s, views[0], nullptr, true, st));
    n += 2;
    for (int k = 0; k < V; ++k) {
      const int cur = views[k];
      const bool more = k + 1 < V;
      const float w = (float)s->psf->weights[cur];
      MLF_TRY(run_view(s, MODE_STEP, cur, more ? views[k + 1] : -1, w, more, st, true));
      ++n;
      if (more) {
        MLF_TRY(run_reduce(s, views[k + 1], nullptr, true, st));
        ++n;
      }
    }
  }
  MLF_TRY(filter_run_geo(s, solver_geo(s), s->X.as<float>(), st));
  n += 5;
  if (launches) *launches += n;
  return MLF_OK;
}

}  // namespace

// ------------------------------------------------------------------ cancellation
namespace {
__global__ void k_cancel_begin(int* stop, int* stopped_host) {
  *stop = 0;
  *reinterpret_cast<volatile int*>(stopped_host) = 0;
}
}  // namespace

CancelState::~CancelState() {
  if (host) cudaFreeHost(host);
}
int CancelState::init() {
  if (host) return MLF_OK;
  MLF_CUDA(cudaHostAlloc((void**)&host, 64, cudaHostAllocMapped));
  host[0] = host[1] = 0;
  int* d = nullptr;
  MLF_CUDA(cudaHostGetDevicePointer((void**)&d, host, 0));
  req_dev = d;
  stopped_dev = d + 1;
  MLF_TRY(stop.alloc(sizeof(int), "cancellation word"));
  MLF_CUDA(cudaMemset(stop.p, 0, sizeof(int)));
  return MLF_OK;
}
int CancelState::begin(cudaStream_t st) {
  MLF_TRY(init());
  reinterpret_cast<volatile int*>(host)[0] = 0;
  k_cancel_begin<<<1, 1, 0, st>>>(stop.as<int>(), stopped_dev);
  MLF_LAUNCHED();
  return MLF_OK;
}
void CancelState::request() const {
  if (host) reinterpret_cast<volatile int*>(host)[0] = 1;
}
bool CancelState::stopped() const { return host && reinterpret_cast<const volatile int*>(host)[1] != 0; }

Solver::~Solver() {
  for (cudaEvent_t e : tev) cudaEventDestroy(e);
  tc_solver_free(tc);
}

size_t Solver::bytes() const {
  return X.bytes + Xtmp.bytes + lfs.bytes + rpad.bytes + part.bytes + hx.bytes + cls.bytes +
         red.bytes + stage_in.bytes + stage_out.bytes + Xprev.bytes + relbuf.bytes + filt.cx.bytes +
         filt.cy.bytes + filt.sums.bytes + tc_solver_bytes(this);
}

size_t Psf::bytes() const { return wf.bytes + wb.bytes + tc_psf_bytes(this); }

bool view_taps_supported(int T) { return T >= 3 && T <= 17 && (T % 2) == 1; }

PatchGeo solver_geo(const Solver* s) {
  return PatchGeo{s->N, s->Z, s->Z, 0, s->Li, s->Lj, s->Pa, s->plane, s->Xr, s->Xc};
}

int launch_extract_views(const float* d_lf, const PatchGeo& g, float* lfs, int64_t view_stride, int64_t off,
                         cudaStream_t st) {
  k_extract_views<<<grid_for(g.Xr * g.Xc), 256, 0, st>>>(d_lf, g, lfs, view_stride, off);
  MLF_LAUNCHED();
  return MLF_OK;
}
int launch_to_phase(const float* d_vol, const PatchGeo& g, float* X, cudaStream_t st, const float* zscale) {
  k_to_phase<<<grid_for(g.Xr * g.Xc * g.Z), 256, 0, st>>>(d_vol, g, X, zscale);
  MLF_LAUNCHED();
  return MLF_OK;
}
int launch_scatter_views(const float* lfs, const PatchGeo& g, float* d_lf, int64_t view_stride, int64_t off,
                         cudaStream_t st) {
  k_scatter_views<<<grid_for(g.Xr * g.Xc), 256, 0, st>>>(lfs, g, d_lf, view_stride, off);
  MLF_LAUNCHED();
  return MLF_OK;
}
int launch_from_phase(const float* X, const PatchGeo& g, float* d_vol, cudaStream_t st, const int* skip) {
  k_from_phase<<<grid_for(g.Xr * g.Xc * g.Z), 256, 0, st>>>(X, g, d_vol, skip);
  MLF_LAUNCHED();
  return MLF_OK;
}
// ------------------------------------------------------------------ convergence monitor
// Block b of kRelChangeBlocks takes the float4 groups b*256 + tid, + grid*256, ... (a fixed
// partition), sums (x - xp)^2 and x^2 in FP64 in a fixed order, and copies X into Xprev.
__global__ void __launch_bounds__(256) k_rel_change_partial(const float* __restrict__ X,
                                                           float* __restrict__ Xprev, int64_t n,
                                                           double* __restrict__ part) {
  __shared__ double sh[2][8];
  double d2 = 0.0, x2 = 0.0;
  const int64_t n4 = n / 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const float4* x4 = reinterpret_cast<const float4*>(X);
  float4* p4 = reinterpret_cast<float4*>(Xprev);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
    const float4 x = x4[i], xp = p4[i];
    const double a = (double)x.x - xp.x, b = (double)x.y - xp.y, c = (double)x.z - xp.z,
                 d = (double)x.w - xp.w;
    d2 += a * a + b * b + c * c + d * d;
    x2 += (double)x.x * x.x + (double)x.y * x.y + (double)x.z * x.z + (double)x.w * x.w;
    p4[i] = x;
  }
  for (int64_t i = 4 * n4 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double a = (double)X[i] - Xprev[i];
    d2 += a * a;
    x2 += (double)X[i] * X[i];
    Xprev[i] = X[i];
  }
  for (int o = 16; o > 0; o >>= 1) {
    d2 += __shfl_down_sync(0xffffffffu, d2, o);
    x2 += __shfl_down_sync(0xffffffffu, x2, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[0][w] = d2;
    sh[1][w] = x2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      a += sh[0][k];
      b += sh[1][k];
    }
    part[2 + 2 * blockIdx.x] = a;
    part[3 + 2 * blockIdx.x] = b;
  }
}

__global__ void k_rel_change_final(double* buf, int nb) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a = 0.0, b = 0.0;
  for (int k = 0; k < nb; ++k) {
    a += buf[2 + 2 * k];
    b += buf[3 + 2 * k];
  }
  buf[0] = b > 0.0 ? sqrt(a / b) : 0.0;
}

int launch_rel_change(const float* X, float* Xprev, int64_t n, double* buf, cudaStream_t st) {
  if (reinterpret_cast<uintptr_t>(X) % 16 != 0 || reinterpret_cast<uintptr_t>(Xprev) % 16 != 0)
    return fail(MLF_ERR_INVALID, "relative change: volume buffers must be 16-byte aligned");
  k_rel_change_partial<<<kRelChangeBlocks, 256, 0, st>>>(X, Xprev, n, buf);
  k_rel_change_final<<<1, 32, 0, st>>>(buf, kRelChangeBlocks);
  MLF_LAUNCHED();
  return MLF_OK;
}

int rel_change_read(const double* buf, double* out) {
  MLF_CUDA(cudaMemcpy(out, buf, sizeof(double), cudaMemcpyDeviceToHost));
  return MLF_OK;
}

int launch_init_flat(const float* d_lf, const PatchGeo& g, float* X, double* scratch, cudaStream_t st) {
  const int nb = 256;
  k_sum_partial<<<nb, 256, 0, st>>>(d_lf, g.Xr * g.Xc, scratch);
  k_init_flat<<<grid_for((int64_t)g.N * g.N * g.Zch * g.Li * g.Lj), 256, 0, st>>>(
      X, g, scratch, nb, 1.0 / ((double)g.Xr * g.Xc * g.Z));
  MLF_LAUNCHED();
  return MLF_OK;
}

// Weights of a plane range [z0, z0+nz) of the PSF: recon_…_with_filter.m:30-38 applied to
// sum over those planes of Hps(:,:,u,v,z) (per-plane normalisation makes a plane subset
// of the PSF a PSF of its own).
std::vector<double> psf_range_weights(const Psf* p, int z0, int nz) {
  const int V = p->N * p->N;
  std::vector<double> w(V, 0.0);
  for (int v = 0; v < V; ++v)
    for (int z = z0; z < z0 + nz; ++z) w[v] += p->wsum_vz[(size_t)v * p->Z + z];
  for (double& x : w)
    if (std::isnan(x)) x = 0.0;
  double tot = 0.0;
  for (double x : w) tot += x;
  for (double& x : w) x = x / tot;
  double mn = w[0];
  for (double x : w) mn = (x < mn || std::isnan(mn)) ? x : mn;
  for (double& x : w) x = x - mn;
  double mx = w[0];
  for (double x : w) mx = (x > mx || std::isnan(mx)) ? x : mx;
  for (double& x : w) x = x / mx;
  for (double& x : w)
    if (x < 0.2) x = 0.0;
  for (double& x : w) x = x * 0.3;
  return w;
}

int solver_init(Solver* s) {
  Psf* p = s->psf;
  s->N = p->N;
  if (!s->lite) s->Z = p->Z;
  s->q = p->q;
  s->T = p->T;
  s->nch = p->nch;
  s->Li = (int)(s->Xr / s->N);
  s->Lj = (int)(s->Xc / s->N);
  if (!view_taps_supported(s->T))
    return fail(MLF_ERR_UNSUPPORTED, "phase-space PSF side S/N = " + std::to_string(s->T) +
                                         " not in {3,5,...,17} (K0 up to 255 at N = 15)");
  s->Pa = round_up(s->Li, 4);
  s->plane = (int64_t)s->Lj * s->Pa;
  // the view kernel indexes channels and per-channel tap blocks in 32 bits
  if (s->nch * (int64_t)s->T * s->T >= (int64_t)INT32_MAX)
    return fail(MLF_ERR_UNSUPPORTED, "too many depth planes for the view kernel's 32-bit channel indices");
  if (s->lite) return MLF_OK;  // batch member: geometry now, filter plan and scratch on first solve
  s->tilesA = ceil_div(s->Li, VW_TX);
  s->tilesB = ceil_div(s->Lj, VW_TY);
  s->tps = s->tilesA * s->tilesB;
  if (s->tps > 256)
    return fail(MLF_ERR_UNSUPPORTED, "patch of " + std::to_string(s->Li) + " x " +
                                         std::to_string(s->Lj) +
                                         " lenslets exceeds the 128 x 64 per-solve limit; tile the field of view");
  const int NW = view_nw8(s->T);
  s->RP = view_plane_pitch(VW_TX * (s->tilesA - 1) + 4 * NW);
  s->RProws = s->tilesB * VW_TY + s->T + 1;
  s->XP = s->RP;
  s->XProws = s->tilesB * VW_TY + s->T - 1;

  std::vector<int> clsA, clsB;
  std::vector<std::pair<int, int>> rngA[3], rngB[3];
  build_classes(s->Li, s->q, clsA, rngA, s->ncA);
  build_classes(s->Lj, s->q, clsB, rngB, s->ncB);
  s->maxc = 1;
  for (int k = 0; k < 3; ++k) s->maxc = std::max({s->maxc, s->ncA[k], s->ncB[k]});
  std::vector<int> tab;
  tab.insert(tab.end(), clsA.begin(), clsA.end());
  tab.insert(tab.end(), clsB.begin(), clsB.end());
  for (auto* rng : {rngA, rngB})
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < s->maxc; ++c) {
        if (c < (int)rng[k].size()) {
          tab.push_back(rng[k][c].first);
          tab.push_back(rng[k][c].second);
        } else {
          tab.push_back(1);
          tab.push_back(0);
        }
      }
  MLF_TRY(s->cls.alloc(tab.size() * sizeof(int), "class tables"));
  MLF_CUDA(cudaMemcpy(s->cls.p, tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice));

  const int slot_floats = round_up(s->XProws * s->XP + 4 * s->T * view_tap_pitch(s->T) + s->maxc * s->maxc + s->T * s->maxc, 4);
  int dev_smem = 0, nsm = 0;
  MLF_CUDA(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device));
  MLF_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, s->device));
  // Channel slots per CTA (they share the staged ratio image).  Small patches: as many as
  // the shared memory holds, up to 192 threads.  Patches of 128..160 tiles: two slots when
  // two such CTAs fit an SM's shared memory (20 warps per SM instead of 15); larger: one.
  const int64_t R_floats = (int64_t)s->RProws * s->RP;
  const int64_t fit = ((int64_t)dev_smem / (int64_t)sizeof(float) - R_floats) / slot_floats;
  int sm_per_sm = 0;
  MLF_CUDA(cudaDeviceGetAttribute(&sm_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, s->device));
  const int64_t two_slot_bytes = (int64_t)sizeof(float) * (R_floats + 2 * (int64_t)slot_floats);
  if (s->tps < 128)
    s->slots = std::max(1, std::min({32, 192 / s->tps, (int)std::max<int64_t>(1, fit)}));
  else
    s->slots = (2 * s->tps <= kViewMaxThreads && 2 * (two_slot_bytes + 1024) <= sm_per_sm) ? 2 : 1;
  // several slots: each starts on a warp boundary when that costs no extra warp
  s->tstride = (s->slots > 1 && round_up(s->slots * round_up(s->tps, 32), 32) == round_up(s->slots * s->tps, 32))
                   ? round_up(s->tps, 32) : s->tps;
  s->threads = round_up(s->slots * s->tstride, 32);
  s->smem = sizeof(float) * ((size_t)s->RProws * s->RP + (size_t)s->slots * slot_floats);
  if ((int)s->smem > dev_smem) return fail(MLF_ERR_UNSUPPORTED, "view kernel shared memory exceeds the device limit");
  MLF_TRY(prepare_view_kernels(s->T, s->smem));
  int per_sm = 1;
  MLF_TRY(occupancy_view_kernel(s->T, s->threads, s->smem, &per_sm));
  per_sm = std::max(1, per_sm);
  const int64_t max_blocks = (s->nch + s->slots - 1) / s->slots;
  s->grid = (int)std::min<int64_t>(max_blocks, (int64_t)nsm * per_sm);

  const int64_t vol = s->nch * s->plane;
  const int64_t LL = (int64_t)s->Li * s->Lj;
  MLF_TRY(s->X.alloc(vol * sizeof(float), "volume"));
  MLF_TRY(s->Xtmp.alloc(vol * sizeof(float), "scratch volume"));
  MLF_TRY(s->lfs.alloc((size_t)s->N * s->N * LL * sizeof(float), "sub-aperture images"));
  MLF_TRY(s->rpad.alloc((size_t)s->RProws * s->RP * sizeof(float), "ratio image"));
  MLF_TRY(s->part.alloc((size_t)s->grid * s->slots * (s->tilesB * VW_TY) * (s->tilesA * VW_TX) * sizeof(float),
                        "forward partials"));
  MLF_TRY(s->hx.alloc(LL * sizeof(float), "forward projection"));
  MLF_TRY(s->red.alloc(4096 * sizeof(double), "reduction scratch"));
  MLF_CUDA(cudaMemset(s->X.p, 0, s->X.bytes));
  MLF_CUDA(cudaMemset(s->Xtmp.p, 0, s->Xtmp.bytes));
  MLF_CUDA(cudaMemset(s->rpad.p, 0, s->rpad.bytes));
  MLF_TRY(filter_init(s));
  return MLF_OK;
}

int lite_prepare(Solver* s) {
  if (!s->lite || s->lite_ready) return MLF_OK;
  MLF_TRY(s->Xtmp.alloc((size_t)s->Xr * s->Xc * s->Z * sizeof(float), "filter scratch"));
  MLF_TRY(s->red.alloc(4096 * sizeof(double), "reduction scratch"));
  MLF_TRY(filter_init(s));
  s->lite_ready = true;
  return MLF_OK;
}

int solver_run(Solver* s, const float* d_lf, int max_iter, int precision, const float* d_warm,
               float* d_out, mlf_stats* stats, cudaStream_t st) {
  if (precision != MLF_PREC_FP32) {
    MLF_TRY(tc_solver_prepare(s, st));
    s->last_run_tc = true;
    return tc_run(s->tc, {s}, {d_lf}, {d_warm}, {d_out}, max_iter, precision, stats, s, st);
  }
  s->last_run_tc = false;
  const PatchGeo g = solver_geo(s);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (stats) {
    MLF_CUDA(cudaEventCreate(&e0));
    MLF_CUDA(cudaEventCreate(&e1));
    MLF_CUDA(cudaEventRecord(e0, st));
  }
  int64_t launches = 0;
  s->timing = stats != nullptr;
  s->tev_used = 0;
  MLF_TRY(s->cancel.begin(st));
  ++launches;
  MLF_TRY(launch_extract_views(d_lf, g, s->lfs.as<float>(), (int64_t)s->Li * s->Lj, 0, st));
  ++launches;
  if (d_warm) {
    MLF_TRY(launch_to_phase(d_warm, g, s->X.as<float>(), st));
    ++launches;
  } else {
    MLF_TRY(launch_init_flat(d_lf, g, s->X.as<float>(), s->red.as<double>(), st));
    launches += 2;
  }
  const bool monitor = stats != nullptr && max_iter > 0;
  if (monitor) {
    if (!s->Xprev.p) MLF_TRY(s->Xprev.alloc(s->X.bytes, "convergence monitor volume"));
    if (!s->relbuf.p) MLF_TRY(s->relbuf.alloc(kRelChangeBufDoubles * sizeof(double), "convergence monitor sums"));
    MLF_CUDA(cudaMemcpyAsync(s->Xprev.p, s->X.p, s->X.bytes, cudaMemcpyDeviceToDevice, st));
  }
  for (int it = 0; it < max_iter; ++it) {
    nvtxRangePushA("RL iteration (enqueue)");
    const int rc_it = enqueue_iteration(s, &launches, st);
    nvtxRangePop();
    MLF_TRY(rc_it);
    if (monitor) {
      MLF_TRY(launch_rel_change(s->X.as<float>(), s->Xprev.as<float>(), (int64_t)(s->X.bytes / sizeof(float)),
                                s->relbuf.as<double>(), st));
      launches += 2;
    }
  }
  MLF_TRY(launch_from_phase(s->X.as<float>(), g, d_out, st, s->cancel.stop.as<int>()));
  ++launches;
  if (stats) {
    MLF_CUDA(cudaEventRecord(e1, st));
    MLF_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    MLF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    stats->n_views = (int)s->psf->view_order.size();
    stats->iterations = max_iter;
    stats->gpu_ms = ms;
    stats->view_ms = (max_iter > 0 && stats->n_views > 0) ? ms / (max_iter * stats->n_views) : 0.0;
    double vk = 0.0;
    for (int k = 0; k + 1 < s->tev_used; k += 2) {
      float t = 0.f;
      MLF_CUDA(cudaEventElapsedTime(&t, s->tev[k], s->tev[k + 1]));
      vk += t;
    }
    stats->view_kernel_ms = vk;
    stats->view_kernel_launches = s->tev_used / 2;
    stats->kernel_launches = launches;
    stats->fwd_splits = stats->fwd_stages = stats->bwd_xbufs = stats->tuned = 0;
    stats->rel_change = 0.0;
    if (monitor) MLF_TRY(rel_change_read(s->relbuf.as<double>(), &stats->rel_change));
    if (s->cancel.stopped()) {
      s->timing = false;
      s->tev_used = 0;
      return fail(MLF_ERR_CANCELLED, "solve cancelled between view steps; outputs left unwritten");
    }
  }
  s->timing = false;
  s->tev_used = 0;
  return MLF_OK;
}

int forward_view(Solver* s, const float* d_vol, int u, int v, float* d_hx, cudaStream_t st) {
  MLF_CUDA(cudaMemsetAsync(s->Xtmp.p, 0, s->Xtmp.bytes, st));  // zero row padding (see forward_project)
  MLF_TRY(launch_to_phase(d_vol, solver_geo(s), s->Xtmp.as<float>(), st));
  ViewArgs a = view_args(s);
  a.X = s->Xtmp.as<float>();
  a.u = u; a.v = v; a.w = 0.f; a.do_fwd = 1;
  a.wb = wb_of(s, u + s->N * v);
  a.wf = wf_of(s, u + s->N * v);
  MLF_TRY(launch_view_kernel(s->T, MODE_FWD, a, s->grid, s->threads, s->smem, st));
  return run_reduce(s, u + s->N * v, d_hx, false, st);
}

// Full light-field image of a volume: the forward projections of all N*N views
// interleaved, LF(u + N*a, v + N*b) = HX_{u,v}(a, b).  `zscale` (nullable, device, Z
// floats) multiplies each plane first; with the plane sums of the raw H it turns the
// solver's per-plane normalised PSF back into H.
int forward_project(Solver* s, const float* d_vol, float* d_lf, const float* d_zscale, int precision,
                    cudaStream_t st) {
  if (precision != MLF_PREC_FP32) {
    MLF_TRY(tc_solver_prepare(s, st));
    return tc_forward_project(s->tc, {s}, {d_vol}, {d_lf}, precision, d_zscale, st);
  }
  if (s->lite) return fail(MLF_ERR_INVALID, "forward projection needs a full solver context");
  const PatchGeo g = solver_geo(s);
  const int N = s->N;
  const int64_t LL = (int64_t)s->Li * s->Lj;
  // the scratch's row padding must be zero (the filter also uses it, in another layout)
  MLF_CUDA(cudaMemsetAsync(s->Xtmp.p, 0, s->Xtmp.bytes, st));
  MLF_TRY(launch_to_phase(d_vol, g, s->Xtmp.as<float>(), st, d_zscale));
  for (int view = 0; view < N * N; ++view) {
    ViewArgs a = view_args(s);
    a.X = s->Xtmp.as<float>();
    a.u = view % N; a.v = view / N; a.w = 0.f; a.do_fwd = 1;
    a.wb = wb_of(s, view);
    a.wf = wf_of(s, view);
    MLF_TRY(launch_view_kernel(s->T, MODE_FWD, a, s->grid, s->threads, s->smem, st));
    MLF_TRY(run_reduce(s, view, s->lfs.as<float>() + view * LL, false, st));
  }
  return launch_scatter_views(s->lfs.as<float>(), g, d_lf, LL, 0, st);
}

int peel_solve(Solver* s, const float* d_lf, int max_iter, int precision, float* d_out, float* d_lf_peeled,
               float* d_proj, mlf_stats* stats, cudaStream_t st) {
  if (s->variant != MLF_VARIANT_PEELING)
    return fail(MLF_ERR_INVALID, "peeling solve needs a solver created with MLF_VARIANT_PEELING");
  const int64_t n_img = s->Xr * s->Xc, n_vol = n_img * s->Z;
  DevBuf top, vol, proj, projm, lf2, proj_out, part;
  MLF_TRY(top.alloc(n_img * 4, "peeling top plane"));
  MLF_TRY(vol.alloc(n_vol * 4, "peeling volume"));
  MLF_TRY(proj.alloc(n_img * 4, "peeling projection"));
  MLF_TRY(projm.alloc(n_img * 4, "peeling projection"));
  MLF_TRY(lf2.alloc(n_img * 4, "peeled image"));
  MLF_TRY(proj_out.alloc(n_img * 4, "peeling projection"));
  MLF_TRY(part.alloc(sizeof(double) * 3 * kPeelBlocks + sizeof(float) * kPeelBlocks, "peeling sums"));
  double* sum_m = part.as<double>();
  double* dots = sum_m + kPeelBlocks;
  float* maxp = reinterpret_cast<float*>(dots + 2 * kPeelBlocks);
  const int fprec = precision == MLF_PREC_FP32 ? MLF_PREC_FP32 : MLF_PREC_BF16X3;

  mlf_stats s1{};
  MLF_TRY(solver_run(s, d_lf, max_iter, precision, nullptr, d_out, stats ? &s1 : nullptr, st));  // :118-172
  MLF_CUDA(cudaMemcpyAsync(top.p, d_out, n_img * 4, cudaMemcpyDeviceToDevice, st));              // :183
  MLF_CUDA(cudaMemsetAsync(vol.p, 0, n_vol * 4, st));
  MLF_CUDA(cudaMemcpyAsync(vol.p, top.p, n_img * 4, cudaMemcpyDeviceToDevice, st));              // :184-185
  MLF_TRY(forward_project(s, vol.as<float>(), proj.as<float>(), nullptr, fprec, st));            // :191
  k_max_partial<<<kPeelBlocks, 256, 0, st>>>(top.as<float>(), n_img, maxp);
  k_peel_mask<<<grid_for(n_img), 256, 0, st>>>(top.as<float>(), n_img, maxp, kPeelBlocks, vol.as<float>());
  MLF_LAUNCHED();
  MLF_TRY(forward_project(s, vol.as<float>(), projm.as<float>(), nullptr, fprec, st));           // :193
  k_sum_partial<<<kPeelBlocks, 256, 0, st>>>(projm.as<float>(), n_img, sum_m);
  k_dot2_partial<<<kPeelBlocks, 256, 0, st>>>(projm.as<float>(), d_lf, proj.as<float>(), n_img, dots);
  k_peel_apply<<<grid_for(n_img), 256, 0, st>>>(d_lf, proj.as<float>(), n_img, sum_m, dots, kPeelBlocks,
                                               lf2.as<float>(), proj_out.as<float>());
  MLF_LAUNCHED();
  MLF_TRY(solver_run(s, lf2.as<float>(), max_iter, precision, nullptr, d_out, stats, st));       // :208-257
  MLF_CUDA(cudaMemcpyAsync(d_out, top.p, n_img * 4, cudaMemcpyDeviceToDevice, st));              // :262
  if (d_lf_peeled) MLF_CUDA(cudaMemcpyAsync(d_lf_peeled, lf2.p, n_img * 4, cudaMemcpyDeviceToDevice, st));
  if (d_proj) MLF_CUDA(cudaMemcpyAsync(d_proj, proj_out.p, n_img * 4, cudaMemcpyDeviceToDevice, st));
  if (stats) {
    stats->gpu_ms += s1.gpu_ms;
    stats->iterations += s1.iterations;
    stats->view_kernel_ms += s1.view_kernel_ms;
    stats->view_kernel_launches += s1.view_kernel_launches;
    stats->kernel_launches += s1.kernel_launches + 9 + 2 * (int64_t)s->N * s->N * 2;
  }
  // the scratch buffers are released on return: wait for the work that reads them
  MLF_CUDA(cudaStreamSynchronize(st));
  return MLF_OK;
}

int forward_view_prec(Solver* s, const float* d_vol, int u, int v, int precision, float* d_hx, cudaStream_t st) {
  if (precision == MLF_PREC_FP32) return forward_view(s, d_vol, u, v, d_hx, st);
  MLF_TRY(tc_solver_prepare(s, st));
  return tc_forward_view(s, precision, d_vol, u + s->N * v, d_hx, st);
}

int backward_view(Solver* s, const float* d_proj, int u, int v, float* d_out, cudaStream_t st) {
  const int LL = s->Li * s->Lj;
  MLF_CUDA(cudaMemsetAsync(s->rpad.p, 0, s->rpad.bytes, st));
  k_fill_rpad<<<ceil_div(LL, 256), 256, 0, st>>>(d_proj, s->Li, s->Lj, s->rpad.as<float>(), s->RP, s->q + 1);
  MLF_LAUNCHED();
  ViewArgs a = view_args(s);
  a.Cout = s->Xtmp.as<float>();
  a.u = u; a.v = v; a.w = 0.f; a.do_fwd = 0;
  a.wb = wb_of(s, u + s->N * v);
  a.wf = wf_of(s, u + s->N * v);
  MLF_TRY(launch_view_kernel(s->T, MODE_BWDC, a, s->grid, s->threads, s->smem, st));
  return launch_from_phase(s->Xtmp.as<float>(), solver_geo(s), d_out, st);
}

int rl_view_step(Solver* s, const float* d_lf, float* d_vol, int u, int v, double w, int precision,
                 cudaStream_t st) {
  const int view = u + s->N * v;
  if (precision != MLF_PREC_FP32) {
    MLF_TRY(tc_solver_prepare(s, st));
    return tc_view_step(s, precision, d_lf, d_vol, view, (float)w, st);
  }
  const PatchGeo g = solver_geo(s);
  MLF_TRY(launch_extract_views(d_lf, g, s->lfs.as<float>(), (int64_t)s->Li * s->Lj, 0, st));
  MLF_TRY(launch_to_phase(d_vol, g, s->X.as<float>(), st));
  MLF_TRY(run_view(s, MODE_FWD, view, view, 0.f, true, st));
  MLF_TRY(run_reduce(s, view, nullptr, true, st));
  MLF_TRY(run_view(s, MODE_STEP, view, -1, (float)w, false, st));
  return launch_from_phase(s->X.as<float>(), g, d_vol, st);
}

int sample_filter(Solver* s, float* d_vol, cudaStream_t st) {
  const PatchGeo g = solver_geo(s);
  MLF_TRY(launch_to_phase(d_vol, g, s->X.as<float>(), st));
  MLF_TRY(filter_run_geo(s, g, s->X.as<float>(), st));
  return launch_from_phase(s->X.as<float>(), g, d_vol, st);
}

// ---------------------------------------------------------------- dispatch per T
#define MLF_DECL_T(T)                                                                     \
  int prepare_view_T##T(size_t smem);                                                    \
  int occupancy_view_T##T(int threads, size_t smem, int* blocks);                        \
  int launch_view_T##T(int mode, const ViewArgs& a, int grid, int threads, size_t smem, \
                       cudaStream_t st);
MLF_DECL_T(3) MLF_DECL_T(5) MLF_DECL_T(7) MLF_DECL_T(9) MLF_DECL_T(11) MLF_DECL_T(13) MLF_DECL_T(15) MLF_DECL_T(17)
#undef MLF_DECL_T

#define MLF_CASES(EXPR) \
  switch (T) {          \
    case 3: return EXPR(3);   \
    case 5: return EXPR(5);   \
    case 7: return EXPR(7);   \
    case 9: return EXPR(9);   \
    case 11: return EXPR(11); \
    case 13: return EXPR(13); \
    case 15: return EXPR(15); \
    case 17: return EXPR(17); \
    default: return fail(MLF_ERR_UNSUPPORTED, "unsupported tap count"); \
  }

int prepare_view_kernels(int T, size_t smem) {
#define E(t) prepare_view_T##t(smem)
  MLF_CASES(E)
#undef E
}
int occupancy_view_kernel(int T, int threads, size_t smem, int* blocks) {
#define E(t) occupancy_view_T##t(threads, smem, blocks)
  MLF_CASES(E)
#undef E
}
int launch_view_kernel(int T, int mode, const ViewArgs& a, int grid, int threads, size_t smem,
                       cudaStream_t st) {
#define E(t) launch_view_T##t(mode, a, grid, threads, smem, st)
  MLF_CASES(E)
#undef E
}

}  // namespace mlf
