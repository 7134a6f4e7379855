// Phase-space PSF construction on the GPU.
//
// Follows recon_theory_phase_space_LFM_with_filter.m:13-40 and
// gen_phasespace_PSF_theory.m:1-31:
//   * per-depth normalisation H(:,:,:,:,z) /= sum(H(:,:,:,:,z)) (FP64 sums),
//   * the phase-space realignment of H (crop to S = K0 - mod(K0-N, 2N), integer shift of
//     each source position, lenslet-phase regrouping, flip of the source index), whose
//     closed form is
//       Hps[p, q', u, v, z] = H[i1+p+u-h, i1+q'+v-h, N-1-(p mod N), N-1-(q' mod N), z]
//     (zero when p+u-h or q'+v-h leaves [0, S)),
//   * the crop Htc = Ht[i1:i1+S, i1:i1+S],
//   * view weights w(u,v) = sum_{x,y,z} Hps(x,y,u,v,z), NaN -> 0, /sum, -min, /max,
//     < 0.2 -> 0, * 0.3.
// The realigned PSFs are never materialised: the kernel writes the per-channel
// polyphase taps that the view kernels consume (layout documented in mlf_internal.h).
#include <cmath>
#include <vector>

#include "mlf_internal.h"

namespace mlf {

namespace {

constexpr int kSumBlocks = 64;   // blocks per depth in the FP64 sums
constexpr int kSumThreads = 256;

__device__ double block_sum_d(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
  __syncthreads();
  return r;
}

// part[z * kSumBlocks + blk] = sum of a contiguous chunk of depth slice z
__global__ void k_slice_sums(const float* __restrict__ A, int64_t slice, double* part) {
  __shared__ double sh[32];
  const int z = blockIdx.y;
  const float* p = A + (int64_t)z * slice;
  const int64_t chunk = (slice + gridDim.x - 1) / gridDim.x;
  const int64_t lo = (int64_t)blockIdx.x * chunk;
  const int64_t hi = min(slice, lo + chunk);
  double s = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += (double)p[i];
  s = block_sum_d(s, sh);
  if (threadIdx.x == 0) part[z * gridDim.x + blockIdx.x] = s;
}

// inv[z] = 1 / sum_z  (fixed summation order)
__global__ void k_inv_sums(const double* part, int nblk, int Z, double* inv) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z >= Z) return;
  double s = 0.0;
  for (int i = 0; i < nblk; ++i) s += part[z * nblk + i];
  inv[z] = 1.0 / s;
}

struct TapGeom {
  int N, Z, K0, S, q, T, i1, h;
  int64_t nch, tpv;  // channels, taps per view
};

__device__ __forceinline__ double hps_value(const float* __restrict__ H, const double* __restrict__ invH,
                                            const TapGeom& g, int u, int v, int p, int pq, int z) {
  // Hps[p, pq, u, v, z] (normalised, FP64)
  const int rp = p + u - g.h, rq = pq + v - g.h;
  if (rp < 0 || rp >= g.S || rq < 0 || rq >= g.S) return 0.0;
  const int a = g.N - 1 - (p % g.N), b = g.N - 1 - (pq % g.N);
  const int64_t K0 = g.K0;
  const int64_t idx = (int64_t)(g.i1 + rp) + K0 * (g.i1 + rq) +
                      K0 * K0 * (a + (int64_t)g.N * (b + (int64_t)g.N * z));
  return (double)H[idx] * invH[z];
}

// One thread per (view, channel, tap) element of wf and wb.
__global__ void k_build_taps(const float* __restrict__ H, const float* __restrict__ Ht,
                             const double* __restrict__ invH, const double* __restrict__ invHt,
                             TapGeom g, float* __restrict__ wf, float* __restrict__ wb) {
  const int64_t total = (int64_t)g.N * g.N * g.tpv;
  const int TT = g.T * g.T;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t view = e / g.tpv;
    const int64_t rem = e - view * g.tpv;
    const int64_t ch = rem / TT;
    const int t = (int)(rem - ch * TT);
    const int u = (int)(view % g.N), v = (int)(view / g.N);
    const int z = (int)(ch % g.Z);
    const int alpha = (int)((ch / g.Z) % g.N);
    const int beta = (int)(ch / ((int64_t)g.Z * g.N));
    const int dy = t / g.T, dx = t - dy * g.T;
    // forward: wf[db][da] = Hps_z[N(2q-da) + N-1-alpha, N(2q-db) + N-1-beta]
    {
      const int p = g.N * (2 * g.q - dx) + g.N - 1 - alpha;
      const int pq = g.N * (2 * g.q - dy) + g.N - 1 - beta;
      wf[e] = (float)hps_value(H, invH, g, u, v, p, pq, z);
    }
    // backward: wb[dj][di] = Htc_z[N(2q-di) + f_alpha, N(2q-dj) + f_beta]
    {
      const int fa = ((alpha - u + g.h) % g.N + g.N) % g.N;
      const int fb = ((beta - v + g.h) % g.N + g.N) % g.N;
      const int p = g.N * (2 * g.q - dx) + fa;
      const int pq = g.N * (2 * g.q - dy) + fb;
      const int64_t K0 = g.K0;
      const int64_t idx = (int64_t)(g.i1 + p) + K0 * (g.i1 + pq) +
                          K0 * K0 * (u + (int64_t)g.N * (v + (int64_t)g.N * z));
      wb[e] = (float)((double)Ht[idx] * invHt[z]);
    }
  }
}

// wsum[view][z] = sum over x, y of Hps(:, :, u, v, z) in FP64 (one block per (view, z),
// fixed order).
__global__ void k_view_sums(const float* __restrict__ H, const double* __restrict__ invH, TapGeom g,
                            double* wsum) {
  __shared__ double sh[32];
  const int view = blockIdx.x, z = blockIdx.y;
  const int u = view % g.N, v = view / g.N;
  const int64_t n = (int64_t)g.S * g.S;
  double s = 0.0;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const int p = (int)(e % g.S);
    const int pq = (int)(e / g.S);
    s += hps_value(H, invH, g, u, v, p, pq, z);
  }
  s = block_sum_d(s, sh);
  if (threadIdx.x == 0) wsum[(int64_t)view * g.Z + z] = s;
}

// gen_spiral, recon_theory_phase_space_LFM_with_filter.m:156-188 (1-based outputs).
void gen_spiral(int Nnum, std::vector<int>& ii, std::vector<int>& jj) {
  const int loop_n = (Nnum + 1) / 2;  // mode(Nnum) is Nnum itself, never 0
  ii.assign(Nnum * Nnum, 0);
  jj.assign(Nnum * Nnum, 0);
  int start = 0;
  for (int k = 1; k <= loop_n; ++k) {
    const int cs = Nnum - 2 * (k - 1);
    const int bias = k - 1;
    if (cs > 1) {
      std::vector<int> in, jn;
      for (int t = 1; t <= cs; ++t) { in.push_back(t); jn.push_back(1); }
      for (int t = 0; t < cs - 1; ++t) { in.push_back(cs); jn.push_back(2 + t); }
      for (int t = cs - 1; t >= 1; --t) { in.push_back(t); jn.push_back(cs); }
      for (int t = 0; t < cs - 2; ++t) { in.push_back(1); jn.push_back(cs - 1 - t); }
      for (size_t t = 0; t < in.size(); ++t) {
        ii[start + t] = in[t] + bias;
        jj[start + t] = jn[t] + bias;
      }
      start += 4 * (cs - 1);
    } else {
      ii[start] = 1 + bias;
      jj[start] = 1 + bias;
    }
  }
}

}  // namespace

int psf_build(Psf* psf, const float* dH, const float* dHt, cudaStream_t st) {
  const int N = psf->N, Z = psf->Z, K0 = psf->K0;
  const int S = K0 - ((K0 - N) % (2 * N));
  // i1 = round(K0/2) - fix(S/2), 1-based, MATLAB round half away from zero
  const int i1 = (int)std::floor(K0 / 2.0 + 0.5) - S / 2 - 1;
  psf->S = S;
  psf->T = S / N;
  psf->q = (psf->T - 1) / 2;
  psf->nch = (int64_t)N * N * Z;
  psf->taps_per_view = psf->nch * psf->T * psf->T;
  TapGeom g{N, Z, K0, S, psf->q, psf->T, i1, (N - 1) / 2, psf->nch, psf->taps_per_view};

  const int64_t slice = (int64_t)K0 * K0 * N * N;
  DevBuf part, inv, wsum;
  MLF_TRY(part.alloc(sizeof(double) * Z * kSumBlocks * 2, "psf sums"));
  MLF_TRY(inv.alloc(sizeof(double) * Z * 2, "psf sums"));
  MLF_TRY(wsum.alloc(sizeof(double) * N * N * Z, "psf weights"));
  double* partH = part.as<double>();
  double* partHt = partH + (int64_t)Z * kSumBlocks;
  double* invH = inv.as<double>();
  double* invHt = invH + Z;
  k_slice_sums<<<dim3(kSumBlocks, Z), kSumThreads, 0, st>>>(dH, slice, partH);
  k_slice_sums<<<dim3(kSumBlocks, Z), kSumThreads, 0, st>>>(dHt, slice, partHt);
  k_inv_sums<<<(Z + 127) / 128, 128, 0, st>>>(partH, kSumBlocks, Z, invH);
  k_inv_sums<<<(Z + 127) / 128, 128, 0, st>>>(partHt, kSumBlocks, Z, invHt);
  MLF_LAUNCHED();

  const size_t nt = (size_t)N * N * psf->taps_per_view;
  MLF_TRY(psf->wf.alloc(nt * sizeof(float), "psf forward taps"));
  MLF_TRY(psf->wb.alloc(nt * sizeof(float), "psf backward taps"));
  k_build_taps<<<2048, 256, 0, st>>>(dH, dHt, invH, invHt, g, psf->wf.as<float>(),
                                     psf->wb.as<float>());
  k_view_sums<<<dim3(N * N, Z), 256, 0, st>>>(dH, invH, g, wsum.as<double>());
  MLF_LAUNCHED();

  psf->wsum_vz.assign((size_t)N * N * Z, 0.0);
  MLF_CUDA(cudaMemcpyAsync(psf->wsum_vz.data(), wsum.p, sizeof(double) * N * N * Z, cudaMemcpyDeviceToHost, st));
  std::vector<double> inv_h(Z);
  MLF_CUDA(cudaMemcpyAsync(inv_h.data(), invH, sizeof(double) * Z, cudaMemcpyDeviceToHost, st));
  MLF_CUDA(cudaStreamSynchronize(st));
  psf->hsum_z.resize(Z);
  std::vector<float> hs(Z);
  for (int z = 0; z < Z; ++z) {
    psf->hsum_z[z] = 1.0 / inv_h[z];
    hs[z] = (float)psf->hsum_z[z];
  }
  MLF_TRY(psf->hsum_dev.alloc(sizeof(float) * Z, "psf plane sums"));
  MLF_CUDA(cudaMemcpy(psf->hsum_dev.p, hs.data(), sizeof(float) * Z, cudaMemcpyHostToDevice));
  std::vector<double> w(N * N, 0.0);
  for (int v = 0; v < N * N; ++v)
    for (int z = 0; z < Z; ++z) w[v] += psf->wsum_vz[(size_t)v * Z + z];

  // weights (recon_…_with_filter.m:30-38), FP64 on the host, IEEE NaN semantics kept
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
  psf->weights = w;

  // active views in spiral order (recon_…_with_filter.m:95,100-106)
  std::vector<int> ii, jj;
  gen_spiral(N, ii, jj);
  psf->view_order.clear();
  psf->spiral.clear();
  for (int k = 0; k < N * N; ++k) {
    const int u = ii[k] - 1, v = jj[k] - 1;
    psf->spiral.push_back(u + N * v);
    if (w[u + N * v] == 0.0) continue;
    psf->view_order.push_back(u + N * v);
  }
  return MLF_OK;
}

}  // namespace mlf
