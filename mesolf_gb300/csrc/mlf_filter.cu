// Flux-preserving NIP low-pass applied after every RL iteration.
//
// recon_theory_phase_space_LFM_with_filter.m:44-61 builds, per bank entry i, the filter
//   F_i = |fftshift(fft2(g_i))| / max,  g_i(x, y) = exp(-((x/w_i)^2 + (y/w_i)^2))
// and sample_filter (:222-240) applies  real(ifft2(ifftshift(fftshift(fft2(X_z)) .* F)))
// to the planes inside the bank's range, then rescales to the plane's original sum.
// Because ifftshift(fftshift(A) .* F) = A .* ifftshift(F) and g is separable,
//   ifftshift(F_i) = ax_i (x) ay_i,   ax_i = |fft(gx_i)| / max|fft(gx_i)|,
// so the filter is a separable CIRCULAR convolution with the real, even kernels
// cx_i = ifft(ax_i) and cy_i = ifft(ay_i).  The kernels are computed here in FP64 and
// truncated where the remaining tail mass is below 1e-12 of the total (the Gaussian
// widths used give compact kernels; a wide kernel falls back to the full circulant).
// The plane sums before and after filtering are accumulated in FP64.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mlf_internal.h"

namespace mlf {

namespace {

constexpr int kLines = 32;      // lines per CTA (one per lane)
constexpr int kPad = 33;        // shared-memory row stride (bank-conflict free)
constexpr int kChunk = 8;       // consecutive outputs per thread
constexpr int kFiltThreads = 512;
constexpr int kLoadUnroll = 8;   // loads in flight per thread while staging lines
constexpr int kRephaseLines = 4; // lines per block of k_rephase

struct FGeo {
  int64_t Xr, Xc;
  int Z;
};

// Offset in the phase-major volume X of the source of line (c, z) of the MATLAB layout
// (length Xr = N*Li), element i enumerated as i = alpha*Li + a: that element is
// line[N*a + alpha] = X[ch(alpha, beta, z)][b][a], beta = c mod N, b = c / N, so that
// consecutive i read consecutive floats of one channel row.
__device__ __forceinline__ int64_t line_src(const PatchGeo& g, int c, int z, int i) {
  const int alpha = i / g.Li, a = i - alpha * g.Li;
  return geo_channel(g, alpha, c % g.N, z) * g.plane + (int64_t)(c / g.N) * g.Pa + a;
}

// MATLAB layout -> phase-major for the filtered planes, scaling each plane by scale[z]: one
// block per kRephaseLines lines (c, zlist[blockIdx.y]); the lines are staged in shared
// memory so that both the read of V and the write of X's channel rows are coalesced.
__global__ void k_rephase(const float* __restrict__ V, const double* __restrict__ scale,
                          const int* __restrict__ zlist, PatchGeo g, float* __restrict__ X) {
  extern __shared__ float lines[];  // [kRephaseLines][Xr]
  const int c0 = blockIdx.x * kRephaseLines, z = zlist[blockIdx.y];
  const int Xr = (int)g.Xr;
  const int nl = (int)(g.Xc - c0 < kRephaseLines ? g.Xc - c0 : kRephaseLines);
  const int total = nl * Xr;
  const float* src = V + ((int64_t)z * g.Xc + c0) * g.Xr;  // nl consecutive lines
  for (int e0 = threadIdx.x; e0 < total; e0 += kLoadUnroll * blockDim.x) {
    float v[kLoadUnroll];
#pragma unroll
    for (int u = 0; u < kLoadUnroll; ++u) {
      const int e = e0 + u * blockDim.x;
      v[u] = e < total ? src[e] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kLoadUnroll; ++u) {
      const int e = e0 + u * blockDim.x;
      if (e < total) lines[e] = v[u];
    }
  }
  __syncthreads();
  const double sc = scale[z];
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int l = e / Xr, i = e - l * Xr;
    const int alpha = i / g.Li, a = i - alpha * g.Li;
    X[line_src(g, c0 + l, z, i)] = (float)((double)lines[l * Xr + g.N * a + alpha] * sc);
  }
}

// Circular 1-D filtering of kLines lines of length L held in shared memory as
// buf[i * kPad + line].  taps[k] = c[(k - wlo) mod L] for k < nt, zero for nt <= k < ntp
// (ntp a multiple of 8, taps in shared memory, 16-byte aligned):
//   y[i] = sum_k taps[k] * x[(i + wlo - k) mod L]
// Each thread produces kChunk = 8 consecutive outputs of one line (lane = line) and walks the
// taps in groups of 8 over a 16-value register window, so one group costs 8 window loads
// and 2 tap loads for 64 FMAs.  Every output adds its products in the order k = 0, 1, ...
// (the zero taps add exactly nothing).
// `emit(line, i, value)` stores an output; returns the thread's FP64 sum of outputs.
template <class Emit>
__device__ double filter_lines(const float* __restrict__ buf, int L, const float* __restrict__ taps,
                               int ntp, int wlo, int nlines, Emit emit) {
  static_assert(kChunk == 8, "the register window assumes 8 outputs per thread");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  double s = 0.0;
  const int nchunks = (L + kChunk - 1) / kChunk;
  for (int chk = warp; chk < nchunks; chk += nwarps) {
    if (lane >= nlines) continue;
    const int i0 = chk * kChunk;
    const int j = (i0 + wlo) % L;  // index of x for output i0 at k = 0
    float w[16];                    // w[m] = x[(j - k0 - 8 + m) mod L] within the group at k0
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      int jt = j + t;
      if (jt >= L) jt -= L;
      w[8 + t] = buf[jt * kPad + lane];
    }
    int jb = j - 8;
    while (jb < 0) jb += L;
    float acc[kChunk];
#pragma unroll
    for (int t = 0; t < kChunk; ++t) acc[t] = 0.f;
    for (int k0 = 0; k0 < ntp; k0 += 8) {
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        int jm = jb + m;
        if (jm >= L) jm -= L;
        w[m] = buf[jm * kPad + lane];
      }
      const float4 c0 = *reinterpret_cast<const float4*>(taps + k0);
      const float4 c1 = *reinterpret_cast<const float4*>(taps + k0 + 4);
      const float c[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
#pragma unroll
      for (int sk = 0; sk < 8; ++sk)
#pragma unroll
        for (int t = 0; t < kChunk; ++t) acc[t] = fmaf(c[sk], w[8 + t - sk], acc[t]);
#pragma unroll
      for (int m = 0; m < 8; ++m) w[8 + m] = w[m];
      jb -= 8;
      while (jb < 0) jb += L;
    }
#pragma unroll
    for (int t = 0; t < kChunk; ++t) {
      const int i = i0 + t;
      if (i < L) {
        emit(lane, i, acc[t]);
        s += (double)acc[t];
      }
    }
  }
  return s;
}

// Stage the taps of bank entry e in shared memory, zero-padded to a multiple of 8.
__device__ __forceinline__ int stage_taps(float* tsm, const float* __restrict__ taps, int nt) {
  const int ntp = (nt + 7) & ~7;
  for (int k = threadIdx.x; k < ntp; k += blockDim.x) tsm[k] = k < nt ? taps[k] : 0.f;
  return ntp;
}

// shared-memory offset (floats) of the staged taps, after a line buffer of L lines
__host__ __device__ constexpr int taps_offset(int L) { return (L * kPad + 3) & ~3; }

__device__ void block_reduce_store(double s, double* out) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
    *out = r;
  }
}

// Pass along r: grid (ceil(Xc / kLines), Zf).  Lines = columns c of plane z, gathered
// straight from the phase-major volume X (line_src); the row-filtered lines are written to
// V in MATLAB layout.  Also accumulates the plane's input sum (sum_before).
__global__ void k_filter_r(const float* __restrict__ X, PatchGeo pg, float* __restrict__ V, FGeo g,
                           const int* __restrict__ zlist, const int* __restrict__ plane_entry,
                           const float* __restrict__ cx, const int* __restrict__ wlo_e,
                           const int* __restrict__ nt_e, int tap_stride, double* sums_in) {
  extern __shared__ __align__(16) float buf[];  // [Xr][kPad], then the taps
  const int z = zlist[blockIdx.y];
  const int e = plane_entry[z];
  const int c0 = blockIdx.x * kLines;
  const int nlines = (int)(g.Xc - c0 < kLines ? g.Xc - c0 : kLines);
  float* plane = V + (int64_t)z * g.Xr * g.Xc;
  const int L = (int)g.Xr;
  float* tsm = buf + taps_offset(L);
  const int ntp = stage_taps(tsm, cx + (int64_t)e * tap_stride, nt_e[e]);
  // element e = l * L + i of the block's lines; 8 loads in flight per thread
  double sin = 0.0;
  const int total = nlines * L;
  for (int e0 = threadIdx.x; e0 < total; e0 += kLoadUnroll * blockDim.x) {
    float v[kLoadUnroll];
#pragma unroll
    for (int u = 0; u < kLoadUnroll; ++u) {
      const int e = e0 + u * blockDim.x;
      v[u] = 0.f;
      if (e < total) {
        const int l = e / L;
        v[u] = X[line_src(pg, c0 + l, z, e - l * L)];
      }
    }
#pragma unroll
    for (int u = 0; u < kLoadUnroll; ++u) {
      const int e = e0 + u * blockDim.x;
      if (e < total) {
        const int l = e / L, i = e - l * L;
        const int alpha = i / pg.Li, a = i - alpha * pg.Li;
        buf[(pg.N * a + alpha) * kPad + l] = v[u];
        sin += (double)v[u];
      }
    }
  }
  __syncthreads();
  double sout = filter_lines(buf, L, tsm, ntp, wlo_e[e], nlines,
                             [&](int l, int i, float y) { plane[(int64_t)(c0 + l) * g.Xr + i] = y; });
  (void)sout;
  block_reduce_store(sin, sums_in + (int64_t)blockIdx.y * gridDim.x + blockIdx.x);
}

// Pass along c (stride Xr): grid (ceil(Xr / kLines), Zf).  Lines = rows r of plane z.
// Accumulates the plane's filtered sum.
__global__ void k_filter_c(float* __restrict__ V, FGeo g, const int* __restrict__ zlist,
                           const int* __restrict__ plane_entry, const float* __restrict__ cy,
                           const int* __restrict__ wlo_e, const int* __restrict__ nt_e, int tap_stride,
                           double* sums_out) {
  extern __shared__ __align__(16) float buf[];  // [Xc][kPad], then the taps
  const int z = zlist[blockIdx.y];
  const int e = plane_entry[z];
  const int64_t r0 = (int64_t)blockIdx.x * kLines;
  float* tsm = buf + taps_offset((int)g.Xc);
  const int ntp = stage_taps(tsm, cy + (int64_t)e * tap_stride, nt_e[e]);
  const int nlines = (int)(g.Xr - r0 < kLines ? g.Xr - r0 : kLines);
  float* plane = V + (int64_t)z * g.Xr * g.Xc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  // 8 column loads in flight per thread
  for (int c0 = warp; c0 < (int)g.Xc; c0 += kLoadUnroll * nwarps) {
    float v[kLoadUnroll];
#pragma unroll
    for (int u = 0; u < kLoadUnroll; ++u) {
      const int c = c0 + u * nwarps;
      v[u] = (c < g.Xc && lane < nlines) ? plane[(int64_t)c * g.Xr + r0 + lane] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kLoadUnroll; ++u) {
      const int c = c0 + u * nwarps;
      if (c < g.Xc && lane < nlines) buf[c * kPad + lane] = v[u];
    }
  }
  __syncthreads();
  const int L = (int)g.Xc;
  double s = filter_lines(buf, L, tsm, ntp, wlo_e[e], nlines,
                          [&](int l, int i, float y) { plane[(int64_t)i * g.Xr + r0 + l] = y; });
  block_reduce_store(s, sums_out + (int64_t)blockIdx.y * gridDim.x + blockIdx.x);
}

// scale[z] = sum_before / sum_after for filtered planes (fixed-order sums), 1 otherwise.
__global__ void k_filter_scale(const double* sin, int nin, const double* sout, int nout,
                               const int* zlist, int nzf, int Z, double* scale) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z >= Z) return;
  int k = -1;
  for (int t = 0; t < nzf; ++t)
    if (zlist[t] == z) k = t;
  if (k < 0) {
    scale[z] = 1.0;
    return;
  }
  double a = 0.0, b = 0.0;
  for (int i = 0; i < nin; ++i) a += sin[(int64_t)k * nin + i];
  for (int i = 0; i < nout; ++i) b += sout[(int64_t)k * nout + i];
  // An all-zero plane (flux underflowed to 0) stays zero.  The reference's
  // sum_before * buf / sum(buf) would give 0/0 = NaN there (…_with_filter.m:233), which the
  // next update's blend (1-w)*X would carry forward; FP32 planes reach exact zero long
  // before FP64 ones do.
  scale[z] = (b != 0.0) ? a / b : 0.0;
}

// |fft(g)|, g[n] = exp(-((n + 1 - L/2) / w)^2), by direct DFT in FP64.
std::vector<double> axis_mag(int L, double w) {
  std::vector<double> g(L), c(L), s(L), out(L);
  for (int n = 0; n < L; ++n) {
    const double x = (n + 1) - L / 2.0;
    g[n] = std::exp(-(x / w) * (x / w));
    c[n] = std::cos(2.0 * M_PI * n / L);
    s[n] = std::sin(2.0 * M_PI * n / L);
  }
  for (int k = 0; k < L; ++k) {
    double re = 0.0, im = 0.0;
    int64_t idx = 0;
    for (int n = 0; n < L; ++n) {
      re += g[n] * c[idx];
      im -= g[n] * s[idx];
      idx += k;
      if (idx >= L) idx -= L;
    }
    out[k] = std::sqrt(re * re + im * im);
  }
  return out;
}

// Circular kernel c = ifft(a / max a) (real and even), FP64.
std::vector<double> circ_kernel(const std::vector<double>& a) {
  const int L = (int)a.size();
  double mx = 0.0;
  for (double v : a) mx = std::max(mx, v);
  std::vector<double> cs(L), out(L);
  for (int n = 0; n < L; ++n) cs[n] = std::cos(2.0 * M_PI * n / L);
  for (int d = 0; d < L; ++d) {
    double acc = 0.0;
    int64_t idx = 0;
    for (int k = 0; k < L; ++k) {
      acc += (a[k] / mx) * cs[idx];
      idx += d;
      if (idx >= L) idx -= L;
    }
    out[d] = acc / L;
  }
  return out;
}

// Half-width beyond which the kernel's tail mass is < 1e-12 of its total; wlo/nt taps.
void truncate_kernel(const std::vector<double>& c, int* wlo, int* nt) {
  const int L = (int)c.size();
  double tot = 0.0;
  for (double v : c) tot += std::fabs(v);
  int W = (L - 1) / 2;
  for (int w = 0; 2 * w + 1 < L; ++w) {
    double tail = 0.0;
    for (int d = 0; d < L; ++d) {
      const int dist = std::min(d, L - d);
      if (dist > w) tail += std::fabs(c[d]);
    }
    if (tail <= 1e-12 * tot) { W = w; break; }
  }
  if (2 * W + 1 >= L) {
    *wlo = (L - 1) / 2;
    *nt = L;
  } else {
    *wlo = W;
    *nt = 2 * W + 1;
  }
}

}  // namespace

int filter_init(Solver* s) {
  FilterPlan& f = s->filt;
  const int Z = s->Z, N = s->N;
  // omega_NIP_array and the plane -> bank-entry map, recon_…_with_filter.m:21-26,54-56,224-231
  // base: ceil(Z/3) rounded up to even; peeling variant (…_simple_peeling.m:55-58): floor(Z/3)
  // rounded down to even
  int R = (int)std::ceil(Z / 3.0);
  if (R % 2 == 1) R += 1;
  if (s->variant == MLF_VARIANT_PEELING) {
    R = Z / 3;
    if (R % 2 == 1) R -= 1;
  }
  const int nb = 3 * R;
  std::vector<double> om(nb);
  for (int i = 0; i < nb; ++i) {
    const double axis = (i + 1) - nb / 2.0;
    const double t = axis / 100.0 * 2.0 * std::sqrt(std::log(2.0));
    om[i] = (N - 7) * std::exp(-t * t);
    if (om[i] < 0.2) om[i] = 0.2;
  }
  const int half_z = (int)std::floor(Z / 2.0 + 0.5);
  f.plane_entry.assign(Z, -1);
  std::vector<int> used(nb, -1), entries;
  for (int z1 = 1; z1 <= Z; ++z1) {
    if (z1 >= half_z - nb / 2.0 + 1 && z1 <= half_z + nb / 2.0) {
      const int bank = (int)(z1 - half_z + nb / 2.0) - 1;
      if (used[bank] < 0) {
        used[bank] = (int)entries.size();
        entries.push_back(bank);
      }
      f.plane_entry[z1 - 1] = used[bank];
    }
  }
  f.n_entries = (int)entries.size();
  const int Lr = (int)s->Xr, Lc = (int)s->Xc;
  std::vector<float> cx((size_t)std::max(1, f.n_entries) * Lr, 0.f), cy((size_t)std::max(1, f.n_entries) * Lc, 0.f);
  std::vector<int> wlo_x(std::max(1, f.n_entries), 0), nt_x(std::max(1, f.n_entries), 1);
  std::vector<int> wlo_y(std::max(1, f.n_entries), 0), nt_y(std::max(1, f.n_entries), 1);
  for (int e = 0; e < f.n_entries; ++e) {
    const double w = om[entries[e]];
    const std::vector<double> kx = circ_kernel(axis_mag(Lr, w));
    const std::vector<double> ky = (Lc == Lr) ? kx : circ_kernel(axis_mag(Lc, w));
    truncate_kernel(kx, &wlo_x[e], &nt_x[e]);
    truncate_kernel(ky, &wlo_y[e], &nt_y[e]);
    for (int k = 0; k < nt_x[e]; ++k) cx[(size_t)e * Lr + k] = (float)kx[((k - wlo_x[e]) % Lr + Lr) % Lr];
    for (int k = 0; k < nt_y[e]; ++k) cy[(size_t)e * Lc + k] = (float)ky[((k - wlo_y[e]) % Lc + Lc) % Lc];
  }
  f.wx = nt_x;
  f.wy = nt_y;
  std::vector<int> zlist;
  for (int z = 0; z < Z; ++z)
    if (f.plane_entry[z] >= 0) zlist.push_back(z);
  const int nzf = (int)zlist.size();
  // int table: plane_entry[Z] | zlist[Z] | wlo_x | nt_x | wlo_y | nt_y
  std::vector<int> itab;
  itab.insert(itab.end(), f.plane_entry.begin(), f.plane_entry.end());
  itab.insert(itab.end(), zlist.begin(), zlist.end());
  itab.resize(2 * Z, 0);
  itab.insert(itab.end(), wlo_x.begin(), wlo_x.end());
  itab.insert(itab.end(), nt_x.begin(), nt_x.end());
  itab.insert(itab.end(), wlo_y.begin(), wlo_y.end());
  itab.insert(itab.end(), nt_y.begin(), nt_y.end());
  MLF_TRY(f.cx.alloc(cx.size() * sizeof(float), "filter kernels"));
  MLF_TRY(f.cy.alloc(cy.size() * sizeof(float), "filter kernels"));
  MLF_TRY(f.plane_entry_dev.alloc(itab.size() * sizeof(int), "filter tables"));
  MLF_CUDA(cudaMemcpy(f.cx.p, cx.data(), cx.size() * sizeof(float), cudaMemcpyHostToDevice));
  MLF_CUDA(cudaMemcpy(f.cy.p, cy.data(), cy.size() * sizeof(float), cudaMemcpyHostToDevice));
  MLF_CUDA(cudaMemcpy(f.plane_entry_dev.p, itab.data(), itab.size() * sizeof(int), cudaMemcpyHostToDevice));
  const int gr = (int)((s->Xc + kLines - 1) / kLines), gc = (int)((s->Xr + kLines - 1) / kLines);
  f.max_blocks = std::max(gr, gc);
  MLF_TRY(f.sums.alloc(sizeof(double) * (2 * (size_t)std::max(1, nzf) * f.max_blocks + Z), "filter sums"));
  const size_t smem_r = sizeof(float) * ((size_t)taps_offset(Lr) + ((Lr + 7) & ~7));
  const size_t smem_c = sizeof(float) * ((size_t)taps_offset(Lc) + ((Lc + 7) & ~7));
  int dev_smem = 0;
  MLF_CUDA(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device));
  if ((int)std::max(smem_r, smem_c) > dev_smem)
    return fail(MLF_ERR_UNSUPPORTED, "image side too large for the sample filter's line buffers");
  MLF_TRY(allow_max_dyn_smem((const void*)k_filter_r));
  MLF_TRY(allow_max_dyn_smem((const void*)k_filter_c));
  return MLF_OK;
}

// The filter of one patch whose volume lives in X with layout g (g.Z planes, the plan's).
int filter_run_geo(Solver* s, const PatchGeo& g, float* X, cudaStream_t st) {
  FilterPlan& f = s->filt;
  const int Z = s->Z;
  int nzf = 0;
  for (int z = 0; z < Z; ++z) nzf += f.plane_entry[z] >= 0;
  if (nzf == 0) return MLF_OK;
  const int* itab = f.plane_entry_dev.as<int>();
  const int* pe = itab;
  const int* zl = itab + Z;
  const int ne = std::max(1, f.n_entries);
  const int* wlo_x = itab + 2 * Z;
  const int* nt_x = wlo_x + ne;
  const int* wlo_y = nt_x + ne;
  const int* nt_y = wlo_y + ne;
  const FGeo fg{s->Xr, s->Xc, Z};
  float* V = s->Xtmp.as<float>();
  const int gr = (int)((s->Xc + kLines - 1) / kLines), gc = (int)((s->Xr + kLines - 1) / kLines);
  double* sin = f.sums.as<double>();
  double* sout = sin + (size_t)nzf * f.max_blocks;
  double* scale = sout + (size_t)nzf * f.max_blocks;
  const int Lr = (int)s->Xr, Lc = (int)s->Xc;
  k_filter_r<<<dim3(gr, nzf), kFiltThreads, sizeof(float) * ((size_t)taps_offset(Lr) + ((Lr + 7) & ~7)), st>>>(
      X, g, V, fg, zl, pe, f.cx.as<float>(), wlo_x, nt_x, Lr, sin);
  k_filter_c<<<dim3(gc, nzf), kFiltThreads, sizeof(float) * ((size_t)taps_offset(Lc) + ((Lc + 7) & ~7)), st>>>(
      V, fg, zl, pe, f.cy.as<float>(), wlo_y, nt_y, Lc, sout);
  k_filter_scale<<<(Z + 255) / 256, 256, 0, st>>>(sin, gr, sout, gc, zl, nzf, Z, scale);
  k_rephase<<<dim3((Lc + kRephaseLines - 1) / kRephaseLines, nzf), 256, sizeof(float) * kRephaseLines * Lr, st>>>(
      V, scale, zl, g, X);
  MLF_LAUNCHED();
  return MLF_OK;
}

}  // namespace mlf
