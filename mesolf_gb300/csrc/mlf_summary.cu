// Summary image of a sensor movie: the input LFIMG of the reconstruction.  Follows
// src/module/summary_image_generation_module.m:43-133 with src/rank_1_factorization.m:32-45
// and src/compute_std_image.m:22-26.  The movie is P pixels x T frames, column-major (one
// frame = P contiguous floats), as the reference's sensor_movie.
//
//   rank-1 background (both modes; mathematically s = Y t / M, t normalised):
//     t = colsum(Y);  repeat bg_iter times { t = t / |t|;  s = Y t / M;  t = s' Y }
//   The reference normalises s between iterations; that scale cancels in the next t, so it
//   is not applied (s stays below sqrt(T) in magnitude).  M = max(Y).
//   'pixelwise':  y = Y / M;  z = y - movmean(y, w1);  m = movmean(z, w2);  x = m.^poly;
//                 img = sqrt(sum(x.^2)/T - mean(x)^2)
//   'global':     y = Y / M;  img = sqrt((sum(y.^2) - s.^2)/T - B.^2 + 2 B s C - s.^2 C^2),
//                 B = mean(y), C = mean(t) (compute_std_image as written)
//   summary = img / max(img).
//
// Passes over the movie (HBM-bound streams): one column pass per iteration (the first also
// takes the max), one row pass per iteration but the last, and a last row pass that also
// computes the image.  bg_iter = 5 reads the movie 2 * bg_iter times.
//
// Column passes: one block per 4 frames x pixel split; each float4 of s is loaded once for
// the 4 frames; partial sums per split are reduced in a fixed order (deterministic).  Row
// passes: one thread per pixel (per 4 pixels in the plain row pass), frames streamed with a
// register prefetch of the next group of frames.  The moving means run as sliding window
// sums over ring buffers in shared memory (one ring column per thread, conflict-free); the
// window-1 sum carries a TwoSum compensation term so that its error does not grow with T.
#include "mlf_internal.h"

namespace mlf {

namespace {

constexpr int SI_COL_THREADS = 512;
constexpr int SI_FPB = 4;           // frames per column-pass block
constexpr int SI_ROW_THREADS = 256;
constexpr int SI_ROW_U = 8;         // float4 frames prefetched per plain row-pass group
constexpr int SI_PIX_U = 32;        // frames prefetched per pixelwise group
constexpr int SI_RED_THREADS = 1024;

// scal[]: 0 M, 1 1/M, 2 mean(t), 3 max(img)
enum { SC_M = 0, SC_INVM = 1, SC_TMEAN = 2, SC_IMGMAX = 3, SC_N = 4 };

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

template <class T>
__device__ __forceinline__ T block_sum(T v, T* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  T r = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
  return r;  // valid in thread 0
}

__device__ __forceinline__ float block_max(float v, float* sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  float r = -INFINITY;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r = fmaxf(r, sh[i]);
  return r;  // valid in thread 0
}

// t_part[ps*T + j] = sum_{p in split ps} w[p] * Y[p, j] (w = 1 when null), for the
// SI_FPB frames of block x; WITH_MAX: max_part[block] = max of Y over the block's elements.
// VEC: P % 4 == 0, Y and w 16-byte aligned, chunk % 4 == 0.
template <bool VEC, bool WITH_MAX>
__global__ void __launch_bounds__(SI_COL_THREADS)
k_si_coldot(const float* __restrict__ Y, int64_t P, int64_t T, const float* __restrict__ w, int64_t chunk,
            float* __restrict__ t_part, float* __restrict__ max_part) {
  __shared__ float sh[32];
  const int64_t j0 = (int64_t)blockIdx.x * SI_FPB;
  const int nf = (int)(T - j0 < SI_FPB ? T - j0 : SI_FPB);
  const int64_t p0 = (int64_t)blockIdx.y * chunk, p1 = P < p0 + chunk ? P : p0 + chunk;
  float acc[SI_FPB];
#pragma unroll
  for (int f = 0; f < SI_FPB; ++f) acc[f] = 0.f;
  float m = -INFINITY;
  if (VEC) {
    for (int64_t p = p0 + 4 * (int64_t)threadIdx.x; p < p1; p += 4 * SI_COL_THREADS) {
      const float4 wv = w ? __ldg(reinterpret_cast<const float4*>(w + p)) : make_float4(1.f, 1.f, 1.f, 1.f);
#pragma unroll
      for (int f = 0; f < SI_FPB; ++f) {
        if (f < nf) {
          const float4 y = __ldcs(reinterpret_cast<const float4*>(Y + (j0 + f) * P + p));
          acc[f] = fmaf(wv.x, y.x, fmaf(wv.y, y.y, fmaf(wv.z, y.z, fmaf(wv.w, y.w, acc[f]))));
          if (WITH_MAX) m = fmaxf(m, fmaxf(fmaxf(y.x, y.y), fmaxf(y.z, y.w)));
        }
      }
    }
  } else {
    for (int64_t p = p0 + threadIdx.x; p < p1; p += SI_COL_THREADS) {
      const float wv = w ? __ldg(w + p) : 1.f;
#pragma unroll
      for (int f = 0; f < SI_FPB; ++f) {
        if (f < nf) {
          const float y = __ldcs(Y + (j0 + f) * P + p);
          acc[f] = fmaf(wv, y, acc[f]);
          if (WITH_MAX) m = fmaxf(m, y);
        }
      }
    }
  }
#pragma unroll
  for (int f = 0; f < SI_FPB; ++f) {
    const float r = block_sum(acc[f], sh);
    if (threadIdx.x == 0 && f < nf) t_part[(int64_t)blockIdx.y * T + j0 + f] = r;
  }
  if (WITH_MAX) {
    const float r = block_max(m, sh);
    if (threadIdx.x == 0) max_part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = r;
  }
}

// One block: t = sum over splits of t_part (fixed order), t /= |t| (FP64 norm), mean(t);
// nmax > 0: M = max(max_part[0..nmax)).
__global__ void __launch_bounds__(SI_RED_THREADS)
k_si_tnorm(const float* __restrict__ t_part, int ps, int64_t T, const float* __restrict__ max_part, int64_t nmax,
           float* __restrict__ t, float* __restrict__ scal) {
  __shared__ double shd[32];
  __shared__ float shf[32];
  __shared__ double bc[2];
  double ss = 0.0;
  for (int64_t j = threadIdx.x; j < T; j += SI_RED_THREADS) {
    float v = 0.f;
    for (int s = 0; s < ps; ++s) v += t_part[(int64_t)s * T + j];
    t[j] = v;
    ss += (double)v * v;
  }
  ss = block_sum(ss, shd);
  if (threadIdx.x == 0) bc[0] = sqrt(ss);
  __syncthreads();
  const double nrm = bc[0];
  double st = 0.0;
  for (int64_t j = threadIdx.x; j < T; j += SI_RED_THREADS) {
    const float v = (float)((double)t[j] / nrm);
    t[j] = v;
    st += v;
  }
  st = block_sum(st, shd);
  if (threadIdx.x == 0) scal[SC_TMEAN] = (float)(st / (double)T);
  if (nmax > 0) {
    float m = -INFINITY;
    for (int64_t i = threadIdx.x; i < nmax; i += SI_RED_THREADS) m = fmaxf(m, max_part[i]);
    m = block_max(m, shf);
    if (threadIdx.x == 0) {
      scal[SC_M] = m;
      scal[SC_INVM] = 1.f / m;
    }
  }
}

// s[p] = sum_j Y[p, j] t[j] / M, four pixels per thread (P % 4 == 0, Y 16-byte aligned).
__global__ void __launch_bounds__(SI_ROW_THREADS)
k_si_rowdot4(const float* __restrict__ Y, int64_t P, int64_t T, const float* __restrict__ t,
             const float* __restrict__ scal, float* __restrict__ s) {
  const int64_t p = 4 * ((int64_t)blockIdx.x * SI_ROW_THREADS + threadIdx.x);
  if (p >= P) return;
  const float* y = Y + p;
  float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
  int64_t j = 0;
  for (; j + SI_ROW_U <= T; j += SI_ROW_U) {
    float4 v[SI_ROW_U];
#pragma unroll
    for (int u = 0; u < SI_ROW_U; ++u) v[u] = __ldcs(reinterpret_cast<const float4*>(y + (j + u) * P));
#pragma unroll
    for (int u = 0; u < SI_ROW_U; u += 2) {
      const float t0 = __ldg(t + j + u), t1 = __ldg(t + j + u + 1);
      a.x = fmaf(v[u].x, t0, a.x); a.y = fmaf(v[u].y, t0, a.y);
      a.z = fmaf(v[u].z, t0, a.z); a.w = fmaf(v[u].w, t0, a.w);
      b.x = fmaf(v[u + 1].x, t1, b.x); b.y = fmaf(v[u + 1].y, t1, b.y);
      b.z = fmaf(v[u + 1].z, t1, b.z); b.w = fmaf(v[u + 1].w, t1, b.w);
    }
  }
  for (; j < T; ++j) {
    const float4 v = __ldcs(reinterpret_cast<const float4*>(y + j * P));
    const float tj = __ldg(t + j);
    a.x = fmaf(v.x, tj, a.x); a.y = fmaf(v.y, tj, a.y);
    a.z = fmaf(v.z, tj, a.z); a.w = fmaf(v.w, tj, a.w);
  }
  const float im = scal[SC_INVM];
  *reinterpret_cast<float4*>(s + p) = make_float4((a.x + b.x) * im, (a.y + b.y) * im, (a.z + b.z) * im, (a.w + b.w) * im);
}

// The same, one pixel per thread (any P or alignment).
__global__ void __launch_bounds__(SI_ROW_THREADS)
k_si_rowdot1(const float* __restrict__ Y, int64_t P, int64_t T, const float* __restrict__ t,
             const float* __restrict__ scal, float* __restrict__ s) {
  const int64_t p = (int64_t)blockIdx.x * SI_ROW_THREADS + threadIdx.x;
  if (p >= P) return;
  const float* y = Y + p;
  float a = 0.f, b = 0.f;
  int64_t j = 0;
  for (; j + 2 * SI_ROW_U <= T; j += 2 * SI_ROW_U) {
    float v[2 * SI_ROW_U];
#pragma unroll
    for (int u = 0; u < 2 * SI_ROW_U; ++u) v[u] = __ldcs(y + (j + u) * P);
#pragma unroll
    for (int u = 0; u < 2 * SI_ROW_U; u += 2) {
      a = fmaf(v[u], __ldg(t + j + u), a);
      b = fmaf(v[u + 1], __ldg(t + j + u + 1), b);
    }
  }
  for (; j < T; ++j) a = fmaf(__ldcs(y + j * P), __ldg(t + j), a);
  s[p] = (a + b) * scal[SC_INVM];
}

template <int POLY>
__device__ __forceinline__ float powi(float m, int poly) {
  if (POLY >= 0) {
    if (POLY == 0) return 1.f;
    float x = m;
#pragma unroll
    for (int q = 1; q < POLY; ++q) x *= m;
    return x;
  }
  float x = 1.f;
  for (int q = 0; q < poly; ++q) x *= m;
  return x;
}

// Last pass, 'pixelwise': s (as k_si_rowdot1) and the detrended std image of each pixel.
// Shared memory: ring1[R1][blockDim] (last raw values), ring2[R2][blockDim] (last z values),
// R = min(window, T).  Unified step k = 0 .. T-1+a1+a2: Y[k] enters window 1 (k < T),
// Y[k-w1] leaves it; z[i1] (i1 = k - a1) enters window 2, z[i1-w2] leaves it; the mean of
// window 2 around i2 = i1 - a2 gives x[i2].  Window of element i: [i-b, i+a] clipped to
// [0, T-1], b = floor(w/2), a = w-1-b (MATLAB movmean / smoothdata 'movmean').  The rings
// hold raw movie values; 1/M is applied to the window-2 mean (the detrend is linear).
// Steps k in [max(w1, a1 + w2), T) have full windows on both sides and every add and drop:
// they run a branch-free form (R1 = w1, R2 = w2 there, so drop slot = write slot) that adds
// (new - dropped) to the window-1 sum with one TwoSum.  POLY >= 0 fixes the power at compile
// time; -1 takes it from `poly`.
template <int POLY>
__global__ void __launch_bounds__(128)
k_si_pixelwise(const float* __restrict__ Y, int64_t P, int T, const float* __restrict__ t,
               const float* __restrict__ scal, int w1, int w2, int R1, int R2, int poly,
               float* __restrict__ s_out, float* __restrict__ img, float* __restrict__ img_max_part) {
  extern __shared__ float ring[];
  __shared__ float sh[32];
  const int nt = blockDim.x;
  float* ring1 = ring + threadIdx.x;
  float* ring2 = ring + (int64_t)R1 * nt + threadIdx.x;
  const int64_t p = (int64_t)blockIdx.x * nt + threadIdx.x;
  float v_img = -INFINITY;
  if (p < P) {
    const float invM = scal[SC_INVM];
    const int b1 = w1 / 2, a1 = w1 - 1 - b1, b2 = w2 / 2, a2 = w2 - 1 - b2;
    const float rw1 = 1.f / (float)w1, rw2i = invM / (float)w2;
    const int R1n = R1 * nt, R2n = R2 * nt;
    const float* y = Y + p;
    float S1 = 0.f, L1 = 0.f, S2 = 0.f, sx = 0.f, sxx = 0.f, sa = 0.f, sb = 0.f;
    // ring offsets (slot * nt): in1 = k % R1, dr1 = (k - w1) % R1, c1 = (k - a1) % R1,
    //                           in2 = i1 % R2, dr2 = (i1 - w2) % R2
    int in1 = 0, dr1 = 0, c1 = 0, in2 = 0, dr2 = 0;
    auto adv = [](int& o, int nt_, int Rn) {
      o += nt_;
      if (o == Rn) o = 0;
    };
    const int K = T + a1 + a2;
    auto step = [&](int k, float raw) {
      // window 1
      if (k < T) {
        if (k >= w1) {  // R1 == w1 here: the dropped value sits in the slot being written
          float s, e;
          two_sum(S1, -ring1[in1], s, e);
          S1 = s;
          L1 += e;
        }
        ring1[in1] = raw;
        float s, e;
        two_sum(S1, raw, s, e);
        S1 = s;
        L1 += e;
        adv(in1, nt, R1n);
      } else if (k >= w1 && k - w1 < T) {
        float s, e;
        two_sum(S1, -ring1[dr1], s, e);
        S1 = s;
        L1 += e;
      }
      if (k >= w1) adv(dr1, nt, R1n);
      const int i1 = k - a1;
      if (i1 < 0) return;
      // z[i1], window 2
      if (i1 < T) {
        const int cnt = min(i1 + a1, T - 1) - max(i1 - b1, 0) + 1;
        const float rc = cnt == w1 ? rw1 : 1.f / (float)cnt;
        const float z = fmaf(-(S1 + L1), rc, ring1[c1]);
        adv(c1, nt, R1n);
        float zd = 0.f;
        if (i1 >= w2) zd = ring2[in2];  // R2 == w2 here
        ring2[in2] = z;
        S2 += z - zd;
        adv(in2, nt, R2n);
      } else if (i1 >= w2 && i1 - w2 < T) {
        S2 -= ring2[dr2];
      }
      if (i1 >= w2) adv(dr2, nt, R2n);
      const int i2 = i1 - a2;
      if (i2 < 0 || i2 >= T) return;
      const int cnt = min(i2 + a2, T - 1) - max(i2 - b2, 0) + 1;
      const float m = S2 * (cnt == w2 ? rw2i : invM / (float)cnt);
      const float x = powi<POLY>(m, poly);
      sx += x;
      sxx = fmaf(x, x, sxx);
    };
    const int k_bulk = max(w1, a1 + w2);
    float cur[SI_PIX_U];
#pragma unroll
    for (int u = 0; u < SI_PIX_U; ++u) cur[u] = u < T ? __ldcs(y + (int64_t)u * P) : 0.f;
    int k = 0;
    for (; k < T; k += SI_PIX_U) {
      float nxt[SI_PIX_U];
      if (k + 2 * SI_PIX_U <= T) {
#pragma unroll
        for (int u = 0; u < SI_PIX_U; ++u) nxt[u] = __ldcs(y + (int64_t)(k + SI_PIX_U + u) * P);
      } else {
#pragma unroll
        for (int u = 0; u < SI_PIX_U; ++u) {
          const int kk = k + SI_PIX_U + u;
          nxt[u] = kk < T ? __ldcs(y + (int64_t)kk * P) : 0.f;
        }
      }
      if (k >= k_bulk && k + SI_PIX_U <= T) {
        // bulk: both windows full, every add and drop present
        float4 tq[SI_PIX_U / 4];
#pragma unroll
        for (int q = 0; q < SI_PIX_U / 4; ++q) tq[q] = __ldg(reinterpret_cast<const float4*>(t + k) + q);
#pragma unroll
        for (int u = 0; u < SI_PIX_U; ++u) {
          const float raw = cur[u];
          const float4 tv = tq[u / 4];
          const float tj = (u & 3) == 0 ? tv.x : (u & 3) == 1 ? tv.y : (u & 3) == 2 ? tv.z : tv.w;
          if (u & 1)
            sb = fmaf(raw, tj, sb);
          else
            sa = fmaf(raw, tj, sa);
          const float d = ring1[in1];
          ring1[in1] = raw;
          float s1, e1;
          two_sum(S1, raw - d, s1, e1);  // (raw - d) rounds relative to the values, not to S1
          S1 = s1;
          L1 += e1;
          adv(in1, nt, R1n);
          const float z = fmaf(-(S1 + L1), rw1, ring1[c1]);
          adv(c1, nt, R1n);
          const float zd = ring2[in2];
          ring2[in2] = z;
          S2 += z - zd;
          adv(in2, nt, R2n);
          const float x = powi<POLY>(S2 * rw2i, poly);
          sx += x;
          sxx = fmaf(x, x, sxx);
        }
        dr1 = in1;  // R1 == w1, R2 == w2: the drop slots follow the write slots
        dr2 = in2;
      } else {
#pragma unroll
        for (int u = 0; u < SI_PIX_U; ++u) {
          const int kk = k + u;
          if (kk < T) {
            const float tj = __ldg(t + kk);
            if (u & 1)
              sb = fmaf(cur[u], tj, sb);
            else
              sa = fmaf(cur[u], tj, sa);
            step(kk, cur[u]);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < SI_PIX_U; ++u) cur[u] = nxt[u];
    }
    for (k = T; k < K; ++k) step(k, 0.f);
    s_out[p] = (sa + sb) * invM;
    const float mx = sx / (float)T;
    const float v = sxx / (float)T - mx * mx;
    v_img = sqrtf(fmaxf(v, 0.f));
    img[p] = v_img;
  }
  const float r = block_max(v_img, sh);
  if (threadIdx.x == 0) img_max_part[blockIdx.x] = r;
}

// Last pass, 'global': s and compute_std_image(Y/M, s, t) as written in the reference.  The
// expansion cancels terms of the size of mean(y)^2 against each other, so sum(y^2), sum(y)
// and s carry TwoSum compensation (s also the exact product error) and the formula runs in
// FP64 per pixel.
__global__ void __launch_bounds__(SI_ROW_THREADS)
k_si_global(const float* __restrict__ Y, int64_t P, int64_t T, const float* __restrict__ t,
            const float* __restrict__ scal, float* __restrict__ s_out, float* __restrict__ img,
            float* __restrict__ img_max_part) {
  __shared__ float sh[32];
  const int64_t p = (int64_t)blockIdx.x * SI_ROW_THREADS + threadIdx.x;
  float v_img = -INFINITY;
  if (p < P) {
    const float invM = scal[SC_INVM];
    const float* y = Y + p;
    float S = 0.f, LS = 0.f, A = 0.f, LA = 0.f, B = 0.f, LB = 0.f;
    auto acc = [&](float raw, float tj) {
      const float yv = raw * invM;
      const float pr = yv * tj;
      const float ep = fmaf(yv, tj, -pr);
      float s, e;
      two_sum(S, pr, s, e);
      S = s;
      LS += e + ep;
      const float sq = yv * yv;
      const float eq = fmaf(yv, yv, -sq);
      two_sum(A, sq, s, e);
      A = s;
      LA += e + eq;
      two_sum(B, yv, s, e);
      B = s;
      LB += e;
    };
    int64_t j = 0;
    for (; j + 2 * SI_ROW_U <= T; j += 2 * SI_ROW_U) {
      float v[2 * SI_ROW_U];
#pragma unroll
      for (int u = 0; u < 2 * SI_ROW_U; ++u) v[u] = __ldcs(y + (j + u) * P);
#pragma unroll
      for (int u = 0; u < 2 * SI_ROW_U; ++u) acc(v[u], __ldg(t + j + u));
    }
    for (; j < T; ++j) acc(__ldcs(y + j * P), __ldg(t + j));
    const double sd = (double)S + (double)LS;  // Y/M already applied: s = (Y/M) t
    s_out[p] = (float)sd;
    const double Tn = (double)T, C = (double)scal[SC_TMEAN];
    const double Ad = (double)A + (double)LA, Bm = ((double)B + (double)LB) / Tn;
    const double v = (Ad - sd * sd) / Tn - Bm * Bm + 2.0 * Bm * sd * C - sd * sd * C * C;
    v_img = (float)sqrt(fmax(v, 0.0));
    img[p] = v_img;
  }
  const float r = block_max(v_img, sh);
  if (threadIdx.x == 0) img_max_part[blockIdx.x] = r;
}

__global__ void __launch_bounds__(SI_RED_THREADS)
k_si_imgmax(const float* __restrict__ part, int64_t n, float* __restrict__ scal) {
  __shared__ float sh[32];
  float m = -INFINITY;
  for (int64_t i = threadIdx.x; i < n; i += SI_RED_THREADS) m = fmaxf(m, part[i]);
  m = block_max(m, sh);
  if (threadIdx.x == 0) scal[SC_IMGMAX] = m;
}

__global__ void k_si_scale(float* __restrict__ img, int64_t P, const float* __restrict__ scal) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < P) img[p] = img[p] / scal[SC_IMGMAX];
}

int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace

// Threads per block of the pixelwise pass (128, or fewer for long windows) so that the rings
// fit the device's shared memory; 0 if even 32 do not fit.
int summary_block(int64_t T, int w1, int w2, size_t smem_max, size_t* smem) {
  const int64_t per = 4 * (std::min<int64_t>(w1, T) + std::min<int64_t>(w2, T));
  for (int nt = 128; nt >= 32; nt /= 2)
    if ((size_t)(per * nt) <= smem_max) {
      *smem = (size_t)(per * nt);
      return nt;
    }
  return 0;
}

namespace {
// CUDA events around each pass when pass times are wanted (none otherwise)
struct PassClock {
  std::vector<cudaEvent_t> ev;
  bool on;
  explicit PassClock(bool want) : on(want) {}
  ~PassClock() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  }
  int mark(cudaStream_t st) {
    if (!on) return MLF_OK;
    cudaEvent_t e;
    MLF_CUDA(cudaEventCreate(&e));
    ev.push_back(e);
    MLF_CUDA(cudaEventRecord(e, st));
    return MLF_OK;
  }
  float ms(size_t i) const {
    float v = 0.f;
    cudaEventElapsedTime(&v, ev[i], ev[i + 1]);
    return v;
  }
};
}  // namespace

int summary_run(const float* dY, int64_t P, int64_t T, int mode, int bg_iter, int w1, int w2, int poly,
                float* d_img, float* d_s, float* d_t, double* pass_ms, cudaStream_t st) {
  PassClock clk(pass_ms != nullptr);
  // a window of 2T or more covers the whole series for every element: same result as 2T
  w1 = (int)std::min<int64_t>(w1, 2 * T);
  w2 = (int)std::min<int64_t>(w2, 2 * T);
  int dev = 0, optin = 0;
  MLF_CUDA(cudaGetDevice(&dev));
  MLF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  size_t smem = 0;
  const int nt = mode == MLF_DETREND_PIXELWISE ? summary_block(T, w1, w2, (size_t)optin - 256, &smem) : 128;
  if (nt == 0)
    return fail(MLF_ERR_UNSUPPORTED, "mlf_summary_image: moving-mean windows of " + std::to_string(w1) + " and " +
                                         std::to_string(w2) + " frames exceed the shared-memory rings");
  const bool vec = P % 4 == 0 && reinterpret_cast<uintptr_t>(dY) % 16 == 0;
  const int64_t ngrp = cdiv(T, SI_FPB);
  // pixel splits: about 16 column blocks per SM in total, splits of >= 16K pixels
  int64_t ps = std::max<int64_t>(1, std::min<int64_t>(cdiv(2432, ngrp), P / 16384));
  int64_t chunk = (cdiv(P, ps) + 3) / 4 * 4;
  ps = cdiv(P, chunk);
  const int64_t nrow = cdiv(P, nt);
  DevBuf tpart, maxpart, scal, imgpart, sbuf, tbuf;
  MLF_TRY(tbuf.alloc(sizeof(float) * (T + 4), "summary: temporal background"));  // 16-byte aligned
  float* tb = tbuf.as<float>();
  MLF_TRY(tpart.alloc(sizeof(float) * ps * T, "summary: column partial sums"));
  MLF_TRY(maxpart.alloc(sizeof(float) * ps * ngrp, "summary: max partials"));
  MLF_TRY(scal.alloc(sizeof(float) * SC_N, "summary: scalars"));
  MLF_TRY(imgpart.alloc(sizeof(float) * std::max(nrow, cdiv(P, SI_ROW_THREADS)), "summary: image max partials"));
  MLF_TRY(sbuf.alloc(sizeof(float) * P, "summary: spatial background"));
  float* sc = scal.as<float>();
  const dim3 cgrid((unsigned)ngrp, (unsigned)ps);
  float* s_tmp = sbuf.as<float>();
  const bool s_aligned = reinterpret_cast<uintptr_t>(s_tmp) % 16 == 0;
  MLF_TRY(clk.mark(st));
  for (int it = 0; it < bg_iter; ++it) {
    if (it == 0) {
      if (vec)
        k_si_coldot<true, true><<<cgrid, SI_COL_THREADS, 0, st>>>(dY, P, T, nullptr, chunk, tpart.as<float>(),
                                                                  maxpart.as<float>());
      else
        k_si_coldot<false, true><<<cgrid, SI_COL_THREADS, 0, st>>>(dY, P, T, nullptr, chunk, tpart.as<float>(),
                                                                   maxpart.as<float>());
    } else {
      if (vec && s_aligned)
        k_si_coldot<true, false><<<cgrid, SI_COL_THREADS, 0, st>>>(dY, P, T, s_tmp, chunk, tpart.as<float>(), nullptr);
      else
        k_si_coldot<false, false><<<cgrid, SI_COL_THREADS, 0, st>>>(dY, P, T, s_tmp, chunk, tpart.as<float>(), nullptr);
    }
    MLF_LAUNCHED();
    k_si_tnorm<<<1, SI_RED_THREADS, 0, st>>>(tpart.as<float>(), (int)ps, T, maxpart.as<float>(),
                                             it == 0 ? ps * ngrp : 0, tb, sc);
    MLF_LAUNCHED();
    MLF_TRY(clk.mark(st));
    if (it + 1 < bg_iter) {
      if (vec)
        k_si_rowdot4<<<(unsigned)cdiv(P / 4, SI_ROW_THREADS), SI_ROW_THREADS, 0, st>>>(dY, P, T, tb, sc, s_tmp);
      else
        k_si_rowdot1<<<(unsigned)cdiv(P, SI_ROW_THREADS), SI_ROW_THREADS, 0, st>>>(dY, P, T, tb, sc, s_tmp);
      MLF_LAUNCHED();
      MLF_TRY(clk.mark(st));
    }
  }
  int64_t nparts;
  if (mode == MLF_DETREND_PIXELWISE) {
    const int R1 = (int)std::min<int64_t>(w1, T), R2 = (int)std::min<int64_t>(w2, T);
    auto kp = poly == 1 ? k_si_pixelwise<1> : poly == 2 ? k_si_pixelwise<2> : poly == 3 ? k_si_pixelwise<3>
                                                                                      : k_si_pixelwise<-1>;
    MLF_TRY(allow_max_dyn_smem((const void*)kp));
    kp<<<(unsigned)nrow, nt, smem, st>>>(dY, P, (int)T, tb, sc, w1, w2, R1, R2, poly, d_s, d_img, imgpart.as<float>());
    nparts = nrow;
  } else {
    nparts = cdiv(P, SI_ROW_THREADS);
    k_si_global<<<(unsigned)nparts, SI_ROW_THREADS, 0, st>>>(dY, P, T, tb, sc, d_s, d_img, imgpart.as<float>());
  }
  MLF_LAUNCHED();
  MLF_TRY(clk.mark(st));
  k_si_imgmax<<<1, SI_RED_THREADS, 0, st>>>(imgpart.as<float>(), nparts, sc);
  k_si_scale<<<(unsigned)cdiv(P, 256), 256, 0, st>>>(d_img, P, sc);
  MLF_LAUNCHED();
  MLF_TRY(clk.mark(st));
  MLF_CUDA(cudaMemcpyAsync(d_t, tb, sizeof(float) * T, cudaMemcpyDeviceToDevice, st));
  MLF_CUDA(cudaStreamSynchronize(st));  // the scratch above is released on return
  if (pass_ms) {
    // marks: start, then per iteration: after column pass (+ t normalisation), after row pass
    // (all but the last iteration); after the last pass; after the finalisation
    double col0 = 0, col = 0, row = 0;
    size_t m = 0;
    for (int it = 0; it < bg_iter; ++it) {
      (it == 0 ? col0 : col) += clk.ms(m++);
      if (it + 1 < bg_iter) row += clk.ms(m++);
    }
    pass_ms[0] = col0;
    pass_ms[1] = bg_iter > 1 ? col / (bg_iter - 1) : 0.0;
    pass_ms[2] = bg_iter > 1 ? row / (bg_iter - 1) : 0.0;
    pass_ms[3] = clk.ms(m++);
    pass_ms[4] = clk.ms(m);
  }
  return MLF_OK;
}

}  // namespace mlf
