// Mixed-precision phase-space RL view step on the 5th-generation tensor cores (tcgen05).
//
// The per-view operators of recon_theory_phase_space_LFM_with_filter.m:109-137 are cast
// as two GEMMs over the lenslet grid (positions p = b*Li + a), the volume channels
// (plane-major, ch = z*N*N + beta*N + alpha, so a patch's plane range is one contiguous
// channel range and tiles outside it are skipped) and the projector taps:
//
//   back projection   C[p, ch] = sum_t' AR[p, t'] * Wb'[ch, t']        (t' in a (T+2)^2 window)
//   D = bwd(ones)     D[p, ch] = sum_t' A1[p, t'] * Wb'[ch, t']
//   update            X[ch][p] <- w*clean(X*C/D) + (1-w)*X              (FP32, epilogue)
//   forward (next v)  Y[p, t]  = sum_ch Xb[p, ch] * Wf[ch, t]           (split over ch)
//                     HX[j][i] = sum_t Y[(j+db-q)*Li + (i+da-q), t=(db,da)]  (col2im)
//
// AR = im2col of the ratio image R (rows p, columns the 17x17 window around the lenslet,
// absorbing the per-channel phase shift s_alpha, s_beta into zero-padded taps), A1 = the
// same im2col of the all-ones image (0/1, exact in BF16).  Operands are BF16, optionally
// split hi + lo (x = hi + lo, both BF16) with the products accumulated in FP32 in TMEM:
//   MLF_PREC_BF16    C = ARh Wbh                   Y = Xh Wfh
//   MLF_PREC_BF16X2  C = (ARh + ARl) Wbh           Y = (Xh + Xl) Wfh      (activations split)
//   MLF_PREC_BF16X3  C = ARh Wbh + ARh Wbl + ARl Wbh, Y likewise          (both split)
// D uses exactly the tap values C uses (Wbh, or Wbh + Wbl when the taps are split), so C/D
// is a weighted mean of R with consistent weights.  Splitting the activations (X, R) rather
// than the taps is the more accurate two-pass form: the tap rounding cancels in C/D.  The ratio, the update, the depth sums (inside C, D, Y) and the sample filter
// stay in FP32.
//
// Both GEMM kernels are warp-specialised: one thread issues TMA tile loads (128-byte
// swizzle) into a shared-memory ring, one thread issues tcgen05.mma into TMEM accumulators,
// one warp owns the TMEM allocation, and the remaining warps run the epilogue (tcgen05.ld,
// 32 TMEM lanes per warp).  The volume X stays FP32 in HBM: the back projection updates it
// through TMA tiles, and the forward GEMM splits each FP32 tile into its BF16 operand in
// shared memory, so no BF16 copy of the volume is ever written.  Every wait is bounded; a
// timeout sets a device error flag, drains in-flight copies and MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <type_traits>
#include <vector>

#include "mlf_internal.h"
#include "mlf_tc.cuh"

namespace mlf {

namespace {

using bf16 = __nv_bfloat16;

constexpr int BM = 128;           // positions per tile (TMEM lanes)
constexpr int BK = 64;            // K per stage (one 128-byte swizzle row of BF16)
constexpr int STAGES = 2;
constexpr int TILE_A = BM * BK * 2;  // 16 KB
constexpr uint32_t WAIT_LIMIT = 1u << 22;  // polls; ~0.3-1 s with the back-off sleep

// Device status word values (tc_check_error turns any of them into MLF_ERR_TIMEOUT).
// TC_ERR_TIMEOUT_DRAIN: a wait for copies or MMAs already issued gave up while the CTA was
// finishing.  The CTA still frees its TMEM: an MMA completes within microseconds, so a
// commit that has not arrived after the wait limit (about a second) means the barrier
// itself failed, and a CTA that exits holding TMEM would block the allocation of every
// later CTA on its SM.
enum TcErr { TC_ERR_TIMEOUT_PRODUCER = 1, TC_ERR_TIMEOUT_MMA = 2, TC_ERR_TIMEOUT_EPILOGUE = 3,
             TC_ERR_TIMEOUT_DRAIN = 4 };

// shared abort flag written by one role and polled by the others
__device__ __forceinline__ bool aborted(const int* f) { return *reinterpret_cast<const volatile int*>(f) != 0; }
__device__ __forceinline__ void set_abort(int* f) { *reinterpret_cast<volatile int*>(f) = 1; }

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

__device__ __forceinline__ void split_bf16(float x, bf16& hi, bf16& lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

// FP16 operands (MLF_PREC_FP16*): the same hi + lo split in FP16, applied to values that
// carry a power-of-two scale putting their largest magnitude in [2^14, 2^15).
using f16 = __half;
__device__ __forceinline__ void split_f16(float x, f16& hi, f16& lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(x - __half2float(hi));
}
__device__ __forceinline__ void split2(float x, bf16& hi, bf16& lo) { split_bf16(x, hi, lo); }
__device__ __forceinline__ void split2(float x, f16& hi, f16& lo) { split_f16(x, hi, lo); }
__device__ __forceinline__ float to_f32(bf16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float to_f32(f16 v) { return __half2float(v); }

// 2^k with m * 2^k in [2^14, 2^15) -- the scale that puts an FP16 operand's largest
// magnitude m just below FP16's maximum (65504) -- or 1 for m = 0 or a non-finite m.
__host__ __device__ inline float f16_scale(float m) {
  if (!(m > 0.f) || !(m <= 3.0e38f)) return 1.f;
  int e = 0;
  frexpf(m, &e);  // m = f * 2^e, f in [0.5, 1)
  int k = 15 - e;
  k = k < -126 ? -126 : (k > 126 ? 126 : k);
  return ldexpf(1.f, k);
}
// maximum of non-negative floats through their bit patterns (which order like unsigned ints)
__device__ __forceinline__ void atomic_max_nonneg(float* addr, float v) {
  atomicMax(reinterpret_cast<unsigned*>(addr), __float_as_uint(v));
}

// ------------------------------------------------------------------ back projection + update
struct TcBwdArgs {
  int* err;
  const int* tile_patch;  // patch of each position tile
  const int* pinfo;       // per patch: Li, Lj, LL, pos0, z0, nz, -, -
  const float* wrow;      // per patch: weight of the current view (0: view inactive for it)
  int CHP, nch, KB, brow0, NN;   // brow0 = view * CHP (row of this view in Wb'); NN = N*N channels per plane
  int use_alo;                      // add ARl * Wbh to C (activation split)
  int use_blo;                      // add ARh * Wbl to C and A1 * Wbl to D (tap split)
  float d_eps;                      // added to D (peeling variant)
  const float* dtab;                // D from class tables of the current view: [ncls][ncls][CHP]
  int q, ncls;                      // (T-1)/2 and 2q+3 classes per axis
  // FP16 modes only (null otherwise)
  const float* rmax;    // |R| maximum of this view: AR carries f16_scale(rmax), removed here
  float* rmax_next;     // the next view's slot, reset to 0 here for its col2im
  float* xmax;          // running maximum of X (the forward GEMM's scale), raised by the update
  const float* bscale;  // scale of each tap row of this view [CHP] (to scale d_eps with D)
  CancelRef cancel;     // solves: stop between view steps when cancelled (null otherwise)
};

constexpr int BWD_BN = 128;                            // channels per tile
constexpr int BWD_EPI_WARPS = 16;                      // 4 per TMEM lane quadrant
constexpr int BWD_IO_WARP = 2 + BWD_EPI_WARPS;          // X-tile stores and loads
constexpr int BWD_THREADS = 32 * (3 + BWD_EPI_WARPS);  // producer, MMA, epilogue, X I/O
constexpr int XTILE = BM * BWD_BN * 4;                 // FP32 X tile, 64 KB (two 32 KB halves)
constexpr int XHALF = XTILE / 2;

// Stage layout for a precision mode: Ah | [Al] | [A1] | Bh | [Bl]  (A1 only when D is a GEMM)
struct BwdLayout {
  int offAl, offA1, offBh, offBl, stage;
};
__host__ __device__ inline BwdLayout bwd_layout(int use_alo, int use_blo, bool d_gemm) {
  BwdLayout L;
  int o = TILE_A;
  L.offAl = use_alo ? o : 0;
  if (use_alo) o += TILE_A;
  L.offA1 = o;
  if (d_gemm) o += TILE_A;
  L.offBh = o;
  o += TILE_A;
  L.offBl = use_blo ? o : 0;
  if (use_blo) o += TILE_A;
  L.stage = o;
  return L;
}
inline size_t bwd_smem_bytes(int use_alo, int use_blo, bool d_gemm, int xbufs) {
  return (size_t)STAGES * bwd_layout(use_alo, use_blo, d_gemm).stage + (size_t)xbufs * XTILE + 1024;
}

// D from class tables.  On each axis a position's back-projection window (T+2 taps around
// the lenslet, the channel's phase shift absorbed into zero taps) loses its first k
// columns when the position is k-1 lenslets from the low edge (class k = 1..q+1) or its
// last k columns near the high edge (class q+1+k), else nothing (class 0); this needs at
// least 2q+2 lenslets per side.  dtab[cb][ca][ch] = the sum of the channel's window taps over
// the rows of class cb and the columns of class ca: exactly the tap values C is built from
// (hi, or hi + lo when the taps are split), so C / D keeps cancelling their rounding.
// Class-major, so an epilogue thread's 16 channels are contiguous.
__device__ __forceinline__ void dtab_range(int c, int q, int T2, int* lo, int* hi) {
  if (c == 0) {
    *lo = 0;
    *hi = T2 - 1;
  } else if (c <= q + 1) {
    *lo = c;
    *hi = T2 - 1;
  } else {
    *lo = 0;
    *hi = T2 - 1 - (c - q - 1);
  }
}
__device__ __forceinline__ void load_dtab16(const float* p, float (&v)[16]) {
  const float4* p4 = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float4 t = __ldg(p4 + k);
    v[4 * k + 0] = t.x;
    v[4 * k + 1] = t.y;
    v[4 * k + 2] = t.z;
    v[4 * k + 3] = t.w;
  }
}
__device__ __forceinline__ int dtab_class(int i, int L, int q) {
  if (i <= q) return q + 1 - i;
  if (i >= L - q - 1) return (q + 1) + (q + 2 - L + i);
  return 0;
}

// Tables of all views, built once per PSF and tap split: block = (32 channels, view), 128
// threads.  The 32 channels' windows go to shared memory, then row sums per (channel, row,
// class), then the table entries per (channel, class pair), written channel-contiguous.
constexpr int DTAB_THREADS = 128;
__host__ __device__ inline int dtab_ch_words(int T) { return ((T + 2) * (T + 2)) | 1; }
template <typename E>
__global__ void __launch_bounds__(DTAB_THREADS) k_tc_dtab(const E* __restrict__ hi, const E* __restrict__ lo,
                                                          int CHP, int KB, int T, float* __restrict__ dtab) {
  extern __shared__ float dsh[];
  const int T2 = T + 2, q = (T - 1) / 2, nc = 2 * q + 3;
  const int c0 = blockIdx.x * 32, view = blockIdx.y;
  const int stride = dtab_ch_words(T);
  float* W = dsh;                 // [32][stride]
  float* rs = dsh + 32 * stride;  // [32][stride]: row sums at wy * nc + class
  const int64_t row0 = (int64_t)view * CHP + c0;
  for (int e = threadIdx.x; e < 32 * T2 * T2; e += DTAB_THREADS) {
    const int c = e / (T2 * T2), k = e - c * (T2 * T2);
    const int64_t r = (row0 + c) * (int64_t)KB + k;
    W[c * stride + k] = to_f32(hi[r]) + (lo ? to_f32(lo[r]) : 0.f);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * T2 * nc; e += DTAB_THREADS) {
    const int c = e & 31, rest = e >> 5;
    const int wy = rest / nc, cl = rest - wy * nc;
    int l, h;
    dtab_range(cl, q, T2, &l, &h);
    float sum = 0.f;
    for (int wx = l; wx <= h; ++wx) sum += W[c * stride + wy * T2 + wx];
    rs[c * stride + rest] = sum;
  }
  __syncthreads();
  float* out = dtab + (int64_t)view * nc * nc * CHP + c0;
  for (int e = threadIdx.x; e < 32 * nc * nc; e += DTAB_THREADS) {
    const int c = e & 31, cls = e >> 5;
    const int cb = cls / nc, ca = cls - cb * nc;
    int l, h;
    dtab_range(cb, q, T2, &l, &h);
    float sum = 0.f;
    for (int wy = l; wy <= h; ++wy) sum += rs[c * stride + wy * nc + ca];
    out[(int64_t)cls * CHP + c] = sum;
  }
}

// Tiles whose patch has weight 0 for this view, or whose channels lie outside the patch's
// planes, are skipped: the update would leave X bit for bit as it is.  Every role walks the
// same sequence.
__device__ __forceinline__ bool bwd_skip(const TcBwdArgs& a, int t, int mtiles) {
  const int pp = __ldg(a.tile_patch + (t % mtiles));
  if (__ldg(a.wrow + pp) == 0.f) return true;
  // channels are plane-major: skip channel tiles outside the patch's planes
  const int n0 = (t / mtiles) * BWD_BN;
  const int c0 = __ldg(a.pinfo + 8 * pp + 4) * a.NN, c1 = c0 + __ldg(a.pinfo + 8 * pp + 5) * a.NN;
  return n0 + BWD_BN <= c0 || n0 >= c1;
}
__device__ __forceinline__ int bwd_next(const TcBwdArgs& a, int t, int total, int mtiles) {
  while (t < total && bwd_skip(a, t, mtiles)) t += gridDim.x;
  return t;
}

// Persistent over (position tile, channel tile) pairs.  Warp 0: TMA producer of the
// operand ring; warp 1: TMEM owner and MMA issuer; warps 2..17: epilogue; warp 18: X-tile
// stores and loads (so no epilogue warp ever waits on a copy).  The accumulators
// are double buffered in TMEM (2 x 256 columns) so the epilogue of one tile overlaps the
// MMAs of the next.  D is a second GEMM on the im2col of ones (DGEMM) or comes from the
// per-view class tables.  The X tile (128 positions x 128 channels, FP32) moves HBM -> shared
// memory -> HBM by TMA in two 64-channel halves, each with its own barriers; with XB = 2
// buffers per half the I/O warp requests tile i+2 as soon as tile i is stored, so the load
// of the next tile is in flight while the current one is computed.
// Epilogue warp e (warp e+2) covers TMEM lanes 32*((e+2)%4).., channel half e/8 and the
// 32-channel quarter ((e%8)/4).
template <bool DGEMM, int XB, bool F16>
__global__ void __launch_bounds__(BWD_THREADS, 1)
k_tc_bwd(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
         const __grid_constant__ CUtensorMap mA1, const __grid_constant__ CUtensorMap mBh,
         const __grid_constant__ CUtensorMap mBl, const __grid_constant__ CUtensorMap mX, TcBwdArgs a,
         int mtiles, int ntiles) {
  {  // a cancelled solve: the rest of its view steps return at once (CTA-uniform, before TMEM)
    __shared__ int s_stop;
    if (threadIdx.x == 0) s_stop = cancel_entry(a.cancel);
    __syncthreads();
    if (s_stop) return;
  }
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], tfull[2], tempty[2], xfull[XB][2], hdone[2][2], mdone;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int KS = a.KB / BK;
  const int total = mtiles * ntiles;
  const bool need_blo = a.use_blo != 0, need_alo = a.use_alo != 0;
  const BwdLayout L = bwd_layout(a.use_alo, a.use_blo, DGEMM);
  float* xs = reinterpret_cast<float*>(smem + STAGES * L.stage);  // [XB][2 halves][64 ch][128 pos]
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&tfull[b], 1);
      tc::mbar_init(&tempty[b], BWD_EPI_WARPS);
      tc::mbar_init(&hdone[b][0], BWD_EPI_WARPS / 2);  // [tile parity][half]
      tc::mbar_init(&hdone[b][1], BWD_EPI_WARPS / 2);
    }
    for (int b = 0; b < XB; ++b) {
      tc::mbar_init(&xfull[b][0], 1);
      tc::mbar_init(&xfull[b][1], 1);
    }
    tc::mbar_init(&mdone, 1);
    tc::fence_mbar_init();
    abort_flag = 0;
    tc::tma_prefetch_desc(&mAh);
    if (DGEMM) tc::tma_prefetch_desc(&mA1);
    tc::tma_prefetch_desc(&mBh);
    tc::tma_prefetch_desc(&mX);
    if (F16 && blockIdx.x == 0) *a.rmax_next = 0.f;
  }
  if (warp == 1) tc::tmem_alloc(&tmem_base, 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer (continuous ring over all tiles of this CTA)
      const uint32_t bytes = (DGEMM ? 3 : 2) * TILE_A + (need_alo ? TILE_A : 0) + (need_blo ? TILE_A : 0);
      int it = 0;
      for (int t = bwd_next(a, blockIdx.x, total, mtiles); t < total && !aborted(&abort_flag);
           t = bwd_next(a, t + gridDim.x, total, mtiles)) {
        const int m0 = (t % mtiles) * BM, n0 = (t / mtiles) * BWD_BN;
        for (int ks = 0; ks < KS; ++ks, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!tc::mbar_wait(&empty[s], ph ^ 1, WAIT_LIMIT)) {
            set_abort(&abort_flag);
            atomicExch(a.err, TC_ERR_TIMEOUT_PRODUCER);
            break;
          }
          uint8_t* st = smem + s * L.stage;
          tc::mbar_arrive_expect_tx(&full[s], bytes);
          tc::tma_load_2d(st, &mAh, &full[s], ks * BK, m0);
          if (need_alo) tc::tma_load_2d(st + L.offAl, &mAl, &full[s], ks * BK, m0);
          if (DGEMM) tc::tma_load_2d(st + L.offA1, &mA1, &full[s], ks * BK, m0);
          tc::tma_load_2d(st + L.offBh, &mBh, &full[s], ks * BK, a.brow0 + n0);
          if (need_blo) tc::tma_load_2d(st + L.offBl, &mBl, &full[s], ks * BK, a.brow0 + n0);
        }
      }
      // drain: every issued copy must have landed before the CTA can exit
      for (int i = std::max(0, it - STAGES); i < it; ++i)
        if (!tc::mbar_wait(&full[i % STAGES], (i / STAGES) & 1, WAIT_LIMIT)) atomicExch(a.err, TC_ERR_TIMEOUT_DRAIN);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer
      const uint32_t idesc = F16 ? tc::idesc_f16_f32(BM, BWD_BN) : tc::idesc_bf16_f32(BM, BWD_BN);
      int it = 0, ti = 0;
      for (int t = bwd_next(a, blockIdx.x, total, mtiles); t < total && !aborted(&abort_flag);
           t = bwd_next(a, t + gridDim.x, total, mtiles), ++ti) {
        const int buf = ti & 1;
        const uint32_t tph = (ti >> 1) & 1;
        if (!tc::mbar_wait(&tempty[buf], tph ^ 1, WAIT_LIMIT)) {
          set_abort(&abort_flag);
          atomicExch(a.err, TC_ERR_TIMEOUT_MMA);
          break;
        }
        tc::tc_fence_after();
        const uint32_t tC = tmem_base + buf * 256, tD = tC + 128;
        bool ok = true;
        for (int ks = 0; ks < KS; ++ks, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!tc::mbar_wait(&full[s], ph, WAIT_LIMIT)) {
            set_abort(&abort_flag);
            atomicExch(a.err, TC_ERR_TIMEOUT_MMA);
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t st = tc::smem_u32(smem + s * L.stage);
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            const uint32_t acc = (ks > 0 || k > 0) ? 1u : 0u;
            const uint64_t dah = tc::desc_kmajor_sw128(st + 32 * k);
            const uint64_t dbh = tc::desc_kmajor_sw128(st + L.offBh + 32 * k);
            tc::mma_bf16(tC, dah, dbh, idesc, acc);
            if (DGEMM) tc::mma_bf16(tD, tc::desc_kmajor_sw128(st + L.offA1 + 32 * k), dbh, idesc, acc);
            if (need_blo) {
              const uint64_t dbl = tc::desc_kmajor_sw128(st + L.offBl + 32 * k);
              tc::mma_bf16(tC, dah, dbl, idesc, 1u);
              if (DGEMM) tc::mma_bf16(tD, tc::desc_kmajor_sw128(st + L.offA1 + 32 * k), dbl, idesc, 1u);
            }
            if (need_alo) {
              const uint64_t dal = tc::desc_kmajor_sw128(st + L.offAl + 32 * k);
              tc::mma_bf16(tC, dal, dbh, idesc, 1u);
            }
          }
          tc::mma_commit(&empty[s]);
        }
        if (!ok) break;
        tc::mma_commit(&tfull[buf]);
      }
      // every issued MMA must have completed before TMEM is released
      tc::mma_commit(&mdone);
      if (!tc::mbar_wait(&mdone, 0, WAIT_LIMIT)) atomicExch(a.err, TC_ERR_TIMEOUT_DRAIN);
    }
    // ---------------- epilogue: update X in shared memory
  } else if (warp < BWD_IO_WARP) {
    const int e = warp - 2;
    const int half = e >> 3;                   // channels 64*half .. 64*half+63
    const int sub = (e & 7) >> 2;              // 32-channel quarter inside the half
    const int quad = warp & 3;                 // TMEM lanes 32*quad .. 32*quad+31
    const int row = quad * 32 + lane;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    // FP16: C carries the ratio image's scale; 1/scale is a power of two (exact)
    const float rinv = F16 ? 1.f / f16_scale(*a.rmax) : 1.f;
    float xm = 0.f;  // FP16: largest updated value (for the running maximum of X)
    int ti = 0;
    for (int t = bwd_next(a, blockIdx.x, total, mtiles); t < total; t = bwd_next(a, t + gridDim.x, total, mtiles), ++ti) {
      const int buf = ti & 1;
      const uint32_t tph = (ti >> 1) & 1;
      const int xb = ti % XB;
      float* xh = xs + (xb * 2 + half) * (XHALF / 4);   // [64 ch][128 pos]
      const int m0 = (t % mtiles) * BM, n0 = (t / mtiles) * BWD_BN;
      const int pp = __ldg(a.tile_patch + (t % mtiles));
      const int* pi = a.pinfo + 8 * pp;
      const int local = m0 + row - __ldg(pi + 3);
      const bool pos_ok = local < __ldg(pi + 2);
      // D of this thread's first 16 channels, requested before the waits
      float dpre[16];
      int cls = 0;
      if (!DGEMM) {
        const int Li = __ldg(pi + 0), Lj = __ldg(pi + 1);
        const int jj = local / Li, ii = local - jj * Li;
        if (pos_ok) cls = dtab_class(jj, Lj, a.q) * a.ncls + dtab_class(ii, Li, a.q);
        load_dtab16(a.dtab + (int64_t)cls * a.CHP + n0 + (half * 4 + sub * 2) * 16, dpre);
      }
      bool ok = !aborted(&abort_flag) && tc::mbar_wait(&tfull[buf], tph, WAIT_LIMIT);
      tc::tc_fence_after();
      ok = ok && tc::mbar_wait(&xfull[xb][half], (ti / XB) & 1, WAIT_LIMIT);
      if (!ok) {
        if (lane == 0) atomicExch(a.err, TC_ERR_TIMEOUT_EPILOGUE);
        set_abort(&abort_flag);
        break;
      }
      // channels are plane-major (ch = z*NN + ...): the patch's planes [z0, z0+nz) are the
      // channel range [z0*NN, (z0+nz)*NN), cut at the real channel count
      const int ch_lo = __ldg(pi + 4) * a.NN;
      const unsigned ch_n = (unsigned)(min(a.nch, (__ldg(pi + 4) + __ldg(pi + 5)) * a.NN) - ch_lo);
      const float wv = __ldg(a.wrow + pp);
      const float wc = wv * rinv;  // weight of the X .* C ./ D term (== wv outside FP16 modes)
      const uint32_t tC = tmem_base + buf * 256 + lane_off, tD = tC + 128;
#pragma unroll
      for (int cc = 0; cc < 2; ++cc) {
        const int c = half * 4 + sub * 2 + cc;  // 16-channel chunk of the tile
        const int chb = n0 + c * 16;
        float cv[16], dv[16];
        if (DGEMM) {
          tc::tmem_ld16x2(tC + c * 16, tD + c * 16, cv, dv);
        } else {
          if (cc == 0) {
#pragma unroll
            for (int j = 0; j < 16; ++j) dv[j] = dpre[j];
          } else {
            load_dtab16(a.dtab + (int64_t)cls * a.CHP + chb, dv);
          }
          tc::tmem_ld16(tC + c * 16, cv);
        }
        // D of the FP16 modes carries the tap row's scale: d_eps is scaled with it
        if (F16 && a.d_eps != 0.f) {
#pragma unroll
          for (int j = 0; j < 16; ++j) dv[j] += a.d_eps * __ldg(a.bscale + chb + j);
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          float* xp = xh + ((sub * 2 + cc) * 16 + j) * BM + row;
          if (pos_ok && (unsigned)(chb + j - ch_lo) < ch_n) {
            const float xo = *xp;
            float xc = __fdividef(xo * cv[j], F16 ? dv[j] : dv[j] + a.d_eps);   // :130  X .* C ./ D
            if (!(xc >= 0.f) || isinf(xc)) xc = 0.f;       // :132-134
            float xn = __fmaf_rn(xc, wc, __fmul_rn(1.f - wv, xo));  // :136
            if (xn < 0.f) xn = 0.f;                        // :137
            *xp = xn;
            if (F16) xm = fmaxf(xm, xn);
          }
        }
      }
      // TMEM buffer free for the MMA warp; this warp's part of the half written
      tc::tc_fence_before();
      tc::fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) {
        tc::mbar_arrive(&tempty[buf]);
        tc::mbar_arrive(&hdone[buf][half]);
      }
    }
    if (F16) {
      const unsigned active = __activemask();
      const unsigned m = __reduce_max_sync(active, __float_as_uint(xm));
      if (lane == __ffs(active) - 1 && m != 0u) atomicMax(reinterpret_cast<unsigned*>(a.xmax), m);
    }
  } else if (warp == BWD_IO_WARP) {
    if (lane == 0) {
      // ---------------- X I/O: first XB tiles in, then per tile: store both halves once
      // their epilogue warps are done, and refill the buffer with tile i + XB
      int issued = 0, ti = 0;
      int tl = bwd_next(a, blockIdx.x, total, mtiles);
      for (int b = 0; b < XB && tl < total; ++b, ++issued) {
        for (int h = 0; h < 2; ++h) {
          tc::mbar_arrive_expect_tx(&xfull[b][h], XHALF);
          tc::tma_load_2d(xs + (b * 2 + h) * (XHALF / 4), &mX, &xfull[b][h], (tl % mtiles) * BM,
                          (tl / mtiles) * BWD_BN + 64 * h);
        }
        tl = bwd_next(a, tl + gridDim.x, total, mtiles);
      }
      for (int t = bwd_next(a, blockIdx.x, total, mtiles); t < total; t = bwd_next(a, t + gridDim.x, total, mtiles), ++ti) {
        const int xb = ti % XB;
        const int m0 = (t % mtiles) * BM, n0 = (t / mtiles) * BWD_BN;
        bool ok = true;
        for (int h = 0; h < 2 && ok; ++h) {
          // one barrier per tile parity: it cannot run two phases ahead, since tile i+2's
          // X is only loaded after tile i is stored
          if (aborted(&abort_flag) || !tc::mbar_wait(&hdone[ti & 1][h], (ti >> 1) & 1, WAIT_LIMIT)) {
            ok = false;
            break;
          }
          tc::tma_store_2d(&mX, xs + (xb * 2 + h) * (XHALF / 4), m0, n0 + 64 * h);
          tc::bulk_commit();
        }
        if (!ok) {
          if (!aborted(&abort_flag)) atomicExch(a.err, TC_ERR_TIMEOUT_EPILOGUE);
          set_abort(&abort_flag);
          break;
        }
        tc::bulk_wait_read0();
        int tn = bwd_next(a, t + gridDim.x, total, mtiles);
        if (XB == 2 && tn < total) tn = bwd_next(a, tn + gridDim.x, total, mtiles);
        if (tn < total) {
          for (int h = 0; h < 2; ++h) {
            tc::mbar_arrive_expect_tx(&xfull[xb][h], XHALF);
            tc::tma_load_2d(xs + (xb * 2 + h) * (XHALF / 4), &mX, &xfull[xb][h], (tn % mtiles) * BM,
                            (tn / mtiles) * BWD_BN + 64 * h);
          }
          ++issued;
        }
      }
      tc::bulk_wait0();
      // loads not consumed (after an abort) must land before the CTA exits; a tile whose
      // stores were issued had its loads consumed
      for (int k = ti; k < issued; ++k)
        for (int h = 0; h < 2; ++h)
          if (!tc::mbar_wait(&xfull[k % XB][h], (k / XB) & 1, WAIT_LIMIT)) atomicExch(a.err, TC_ERR_TIMEOUT_DRAIN);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) tc::tmem_dealloc(tmem_base, 512);
}

// ------------------------------------------------------------------ forward projection
constexpr int FWD_MAX_STAGES = 4;
struct TcFwdArgs {
  float* ypart;  // [split][NB][MP] (tap-major: col2im reads it coalesced)
  int* err;
  int stages;    // shared-memory ring depth (2..FWD_MAX_STAGES)
  int MP, NB, NH, nparts, ks_per_split, KS, frow0;  // frow0 = view * NB
  int use_alo, use_blo;                             // activation / tap hi+lo splits
  const float* wview;      // per patch weight of the projected view (nullable: project all)
  const int* tile_patch;   // patch of each position tile
  const int* pinfo;        // per patch: Li, Lj, LL, pos0, z0, nz, -, -
  int NN;                  // N*N channels per plane (plane-major channels)
  // FP16 modes only (null otherwise)
  const float* xmax;       // running maximum of X: the operand is X * f16_scale(xmax)
  const float* fsinv;      // inverse scales of the view's tap columns [NB]
  CancelRef cancel;        // solves: stop between view steps when cancelled (null otherwise)
};

// The forward GEMM reads the FP32 volume directly: each stage's 32 KB region receives the
// X tile [64 channels][128 positions] by TMA; four converter warps (one position row per
// thread) take their 64 values into registers, meet on an mbarrier (bounded wait), and
// write the BF16 hi / lo operand back into the same region in the K-major 128-byte-swizzled
// layout a TMA load would have produced (16-byte chunk c of row p at chunk c ^ (p & 7)).
// The MMA warp waits for the converters.  Warp 0: TMA producer; warp 1: MMA issuer;
// warp 2: TMEM owner; warps 4..7: converters, then the epilogue (TMEM quadrant = warp % 4).
constexpr int FWD_THREADS = 256;
constexpr int FWD_XTILE = BM * BK * 4;  // 32 KB: FP32 X tile, then A hi | A lo (16 KB each)

template <bool F16>
__global__ void __launch_bounds__(FWD_THREADS, 1)
k_tc_fwd(const __grid_constant__ CUtensorMap mX, const __grid_constant__ CUtensorMap mBh,
         const __grid_constant__ CUtensorMap mBl, TcFwdArgs a) {
  // a patch that does not use this view needs no projection for it (whole CTA, before any
  // barrier or TMEM allocation)
  if (a.wview && __ldg(a.wview + __ldg(a.tile_patch + blockIdx.x)) == 0.f) return;
  {  // a cancelled solve: the rest of its view steps return at once (CTA-uniform, before TMEM)
    __shared__ int s_stop;
    if (threadIdx.x == 0) s_stop = cancel_entry(a.cancel);
    __syncthreads();
    if (s_stop) return;
  }
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  __shared__ __align__(8) uint64_t full[FWD_MAX_STAGES], rdone[FWD_MAX_STAGES], conv[FWD_MAX_STAGES],
      empty[FWD_MAX_STAGES], accb;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM;
  const int split = blockIdx.y;
  // this split's channel blocks, clipped to the patch's planes (an empty range writes zeros)
  const int* pq = a.pinfo + 8 * __ldg(a.tile_patch + blockIdx.x);
  const int klo = __ldg(pq + 4) * a.NN / BK;
  const int khi = ((__ldg(pq + 4) + __ldg(pq + 5)) * a.NN + BK - 1) / BK;
  const int ks0 = max(split * a.ks_per_split, klo);
  const int ks1 = min(min(a.KS, split * a.ks_per_split + a.ks_per_split), khi);
  const int tileB = a.NB * 128;  // NB rows x 128 bytes
  const int S = a.stages;
  const int offAl = TILE_A, offBh = FWD_XTILE, offBl = offBh + tileB;
  const int stage_bytes = offBh + tileB * (a.use_blo ? 2 : 1);
  const uint32_t tcols = a.NB > 256 ? 512u : 256u;
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&rdone[s], 4);
      tc::mbar_init(&conv[s], 4);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&accb, 1);
    tc::fence_mbar_init();
    abort_flag = 0;
    tc::tma_prefetch_desc(&mX);
    tc::tma_prefetch_desc(&mBh);
  }
  if (warp == 2) tc::tmem_alloc(&tmem_base, tcols);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tY = tmem_base;

  if (warp == 0 && lane == 0) {
    const uint32_t bytes = FWD_XTILE + tileB * (a.use_blo ? 2 : 1);
    int issued = 0;
    for (int ks = ks0; ks < ks1; ++ks) {
      const int i = ks - ks0, s = i % S;
      const uint32_t ph = (i / S) & 1;
      if (!tc::mbar_wait(&empty[s], ph ^ 1, WAIT_LIMIT)) {
        set_abort(&abort_flag);
        atomicExch(a.err, TC_ERR_TIMEOUT_PRODUCER);
        break;
      }
      uint8_t* st = smem + s * stage_bytes;
      tc::mbar_arrive_expect_tx(&full[s], bytes);
      tc::tma_load_2d(st, &mX, &full[s], m0, ks * BK);
      for (int p = 0; p < a.nparts; ++p) {
        tc::tma_load_2d(st + offBh + p * a.NH * 128, &mBh, &full[s], ks * BK, a.frow0 + p * a.NH);
        if (a.use_blo)
          tc::tma_load_2d(st + offBl + p * a.NH * 128, &mBl, &full[s], ks * BK, a.frow0 + p * a.NH);
      }
      ++issued;
    }
    for (int i = std::max(0, issued - S); i < issued; ++i)
      if (!tc::mbar_wait(&full[i % S], (i / S) & 1, WAIT_LIMIT)) atomicExch(a.err, TC_ERR_TIMEOUT_DRAIN);
  } else if (warp == 1 && lane == 0) {
    const uint32_t idesc = F16 ? tc::idesc_f16_f32(BM, a.NH) : tc::idesc_bf16_f32(BM, a.NH);
    for (int ks = ks0; ks < ks1; ++ks) {
      const int i = ks - ks0, s = i % S;
      const uint32_t ph = (i / S) & 1;
      if (aborted(&abort_flag) || !tc::mbar_wait(&full[s], ph, WAIT_LIMIT) ||
          !tc::mbar_wait(&conv[s], ph, WAIT_LIMIT)) {
        set_abort(&abort_flag);
        atomicExch(a.err, TC_ERR_TIMEOUT_MMA);
        break;
      }
      tc::tc_fence_after();
      const uint32_t st = tc::smem_u32(smem + s * stage_bytes);
#pragma unroll
      for (int k = 0; k < BK / 16; ++k) {
        const uint32_t acc = (i > 0 || k > 0) ? 1u : 0u;
        const uint64_t dah = tc::desc_kmajor_sw128(st + 32 * k);
        for (int p = 0; p < a.nparts; ++p) {
          const uint32_t dcol = tY + p * a.NH;
          const uint64_t dbh = tc::desc_kmajor_sw128(st + offBh + p * a.NH * 128 + 32 * k);
          tc::mma_bf16(dcol, dah, dbh, idesc, acc);
          if (a.use_blo) {
            const uint64_t dbl = tc::desc_kmajor_sw128(st + offBl + p * a.NH * 128 + 32 * k);
            tc::mma_bf16(dcol, dah, dbl, idesc, 1u);
          }
          if (a.use_alo) {
            const uint64_t dal = tc::desc_kmajor_sw128(st + offAl + 32 * k);
            tc::mma_bf16(dcol, dal, dbh, idesc, 1u);
          }
        }
      }
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(&accb);
  } else if (warp >= 4) {
    // converters: FP32 X tile -> BF16 (FP16: scaled) hi / lo operand, in place
    const int p = threadIdx.x - 128;  // position row of the tile
    const float sx = F16 ? f16_scale(*a.xmax) : 1.f;
    for (int ks = ks0; ks < ks1; ++ks) {
      const int i = ks - ks0, s = i % S;
      const uint32_t ph = (i / S) & 1;
      if (aborted(&abort_flag) || !tc::mbar_wait(&full[s], ph, WAIT_LIMIT)) {
        set_abort(&abort_flag);
        if (lane == 0) atomicExch(a.err, TC_ERR_TIMEOUT_EPILOGUE);
        break;
      }
      uint8_t* st = smem + s * stage_bytes;
      const float* xf = reinterpret_cast<const float*>(st);  // [64 ch][128 pos]
      float x[BK];
#pragma unroll
      for (int c = 0; c < BK; ++c) x[c] = xf[c * BM + p];
      // every converter has its values before the region is overwritten (bounded wait)
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&rdone[s]);
      if (!tc::mbar_wait(&rdone[s], ph, WAIT_LIMIT)) {
        set_abort(&abort_flag);
        if (lane == 0) atomicExch(a.err, TC_ERR_TIMEOUT_EPILOGUE);
        break;
      }
#pragma unroll
      for (int c8 = 0; c8 < BK / 8; ++c8) {
        using E = typename std::conditional<F16, f16, bf16>::type;
        __align__(16) E hi[8];
        __align__(16) E lo[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) split2(F16 ? x[c8 * 8 + j] * sx : x[c8 * 8 + j], hi[j], lo[j]);
        const int off = p * 128 + ((c8 ^ (p & 7)) << 4);
        *reinterpret_cast<uint4*>(st + off) = *reinterpret_cast<const uint4*>(hi);
        if (a.use_alo) *reinterpret_cast<uint4*>(st + offAl + off) = *reinterpret_cast<const uint4*>(lo);
      }
      tc::fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&conv[s]);
    }
  }
  if (warp >= 4) {
    __syncwarp();
    const bool ok = tc::mbar_wait(&accb, 0, WAIT_LIMIT);
    tc::tc_fence_after();
    if (!ok && lane == 0) atomicExch(a.err, TC_ERR_TIMEOUT_EPILOGUE);
    const int quad = warp & 3;
    const int row = quad * 32 + lane;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    float* out = a.ypart + (int64_t)split * a.NB * a.MP + m0 + row;  // + t * MP
    const bool empty_split = ks1 <= ks0;
    // FP16: remove the volume's and the tap column's scales (powers of two: exact)
    const float xinv = F16 ? 1.f / f16_scale(*a.xmax) : 1.f;
    if (ok) {
      for (int c = 0; c < (a.nparts * a.NH) / 16; ++c) {
        float v[16];
        tc::tmem_ld16(tY + lane_off + c * 16, v);
        if (aborted(&abort_flag)) continue;
        if (F16) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] *= xinv * __ldg(a.fsinv + c * 16 + j);
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) out[(int64_t)(c * 16 + j) * a.MP] = empty_split ? 0.f : v[j];
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 2) tc::tmem_dealloc(tmem_base, tcols);
}

// ------------------------------------------------------------------ fused back projection + next forward
// One launch per view step for the BF16 modes (bf16, bf16x2) when D comes from the class
// tables and the forward taps fit one MMA (N <= 256): back projection + update of view k as
// in k_tc_bwd, and the forward GEMM of view k+1 on each updated X tile while it is still in
// shared memory, so the volume is read and written once per view (k_tc_fwd re-reads it).
// Work items are (position tile m, split s): the channel tiles of split s -- the split
// boundaries of k_tc_fwd, so Y accumulates over the same K-steps in the same order (the
// results are bit for bit those of k_tc_bwd + k_tc_fwd).  Per tile:
//   producer:  the 5 AR / Wb stages of tile i, then the 1-2 Wf half stages of tile i-1
//   MMA:       back projection of tile i into C[i & 1], then the forward of tile i-1 into Y
//   epilogue:  update of tile i (as k_tc_bwd); after the I/O warp has stored the FP32 half
//              (its TMA store has read the buffer), every warp of the half reads its values,
//              meets the others on an mbarrier, and writes the BF16 hi / lo operand back into
//              the same 32 KB in the K-major 128-byte-swizzled layout; after the item's last
//              forward MMA it drains Y (TMEM) into the split's partials
//   X I/O:     loads, stores, and reloads a buffer only after the forward MMAs that read it
// TMEM: C buffers at columns 0 and 128, Y at 256 (NB <= 256 columns).  XB X buffers per
// half and an NS-stage operand ring: (2, 2) or (1, 3) fit the shared memory.  Every wait is
// bounded; a timeout sets the device status word and the abort flag.
struct TcFusedArgs {
  TcBwdArgs b;
  float* ypart;        // [splits][NB][MP]
  const float* wview;  // per patch weight of the projected (next) view
  int MP, NB, splits, ks_per_split, KS, frow0, ntiles;
};

struct FusedItem {
  int m, s, n_lo, n_hi, ks0, ks1, c0, c1;
  bool wcur, wnext;
};
__device__ __forceinline__ FusedItem fused_item(const TcFusedArgs& a, int item) {
  FusedItem f;
  f.m = item / a.splits;
  f.s = item - f.m * a.splits;
  const int pp = __ldg(a.b.tile_patch + f.m);
  const int* pi = a.b.pinfo + 8 * pp;
  const int z0 = __ldg(pi + 4), nz = __ldg(pi + 5);
  f.c0 = z0 * a.b.NN;                 // channel range of the patch (as bwd_skip)
  f.c1 = f.c0 + nz * a.b.NN;
  const int klo = z0 * a.b.NN / BK;   // K-steps of the forward (as k_tc_fwd)
  const int khi = ((z0 + nz) * a.b.NN + BK - 1) / BK;
  f.ks0 = max(f.s * a.ks_per_split, klo);
  f.ks1 = min(min(a.KS, f.s * a.ks_per_split + a.ks_per_split), khi);
  f.n_lo = f.s * (a.ks_per_split / 2);
  f.n_hi = min(a.ntiles, (f.s + 1) * (a.ks_per_split / 2));
  f.wcur = __ldg(a.b.wrow + pp) != 0.f;
  f.wnext = a.wview ? __ldg(a.wview + pp) != 0.f : true;
  return f;
}
// flags of channel tile n of an item: bit 0 back projection, bits 1-2 forward halves
__device__ __forceinline__ int fused_tile(const FusedItem& f, int n) {
  const int n0 = n * BWD_BN;
  const bool b = f.wcur && !(n0 + BWD_BN <= f.c0 || n0 >= f.c1);
  const bool h0 = f.wnext && 2 * n >= f.ks0 && 2 * n < f.ks1;
  const bool h1 = f.wnext && 2 * n + 1 >= f.ks0 && 2 * n + 1 < f.ks1;
  return (b ? 1 : 0) | (h0 ? 2 : 0) | (h1 ? 4 : 0);
}
__device__ __forceinline__ int fused_nfwd(const FusedItem& f) {
  int c = 0;
  for (int n = f.n_lo; n < f.n_hi; ++n) {
    const int fl = fused_tile(f, n);
    c += ((fl >> 1) & 1) + ((fl >> 2) & 1);
  }
  return c;
}

template <int XB, int NS>
__global__ void __launch_bounds__(BWD_THREADS, 1)
k_tc_bwdfwd(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
            const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mX,
            const __grid_constant__ CUtensorMap mF, TcFusedArgs a, int nitems) {
  {  // a cancelled solve: the rest of its view steps return at once (CTA-uniform, before TMEM)
    __shared__ int s_stop;
    if (threadIdx.x == 0) s_stop = cancel_entry(a.b.cancel);
    __syncthreads();
    if (s_stop) return;
  }
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  __shared__ __align__(8) uint64_t full[NS], empty[NS], tfull[2], tempty[2], xfull[XB][2], hdone[2][2],
      xstored[XB][2], rdone[XB][2], aready[XB][2], afree[XB][2], yfull, ydone, mdone;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int KS = a.b.KB / BK;
  const bool need_alo = a.b.use_alo != 0;
  const BwdLayout L = bwd_layout(a.b.use_alo, 0, false);
  float* xs = reinterpret_cast<float*>(smem + NS * L.stage);  // [XB][2 halves][64 ch][128 pos]
  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&tfull[b], 1);
      tc::mbar_init(&tempty[b], BWD_EPI_WARPS);
      tc::mbar_init(&hdone[b][0], BWD_EPI_WARPS / 2);
      tc::mbar_init(&hdone[b][1], BWD_EPI_WARPS / 2);
    }
    for (int b = 0; b < XB; ++b)
      for (int h = 0; h < 2; ++h) {
        tc::mbar_init(&xfull[b][h], 1);
        tc::mbar_init(&xstored[b][h], 1);
        tc::mbar_init(&rdone[b][h], BWD_EPI_WARPS / 2);
        tc::mbar_init(&aready[b][h], BWD_EPI_WARPS / 2);
        tc::mbar_init(&afree[b][h], 1);
      }
    tc::mbar_init(&yfull, 1);
    tc::mbar_init(&ydone, BWD_EPI_WARPS);
    tc::mbar_init(&mdone, 1);
    tc::fence_mbar_init();
    abort_flag = 0;
    tc::tma_prefetch_desc(&mAh);
    tc::tma_prefetch_desc(&mBh);
    tc::tma_prefetch_desc(&mX);
    tc::tma_prefetch_desc(&mF);
  }
  if (warp == 1) tc::tmem_alloc(&tmem_base, 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer: bwd stages of tile i, then the Wf halves of tile i-1
      const uint32_t bbytes = 2 * TILE_A + (need_alo ? TILE_A : 0);
      const uint32_t fbytes = (uint32_t)a.NB * 128;
      int it = 0;
      bool ok = true;
      int pn = -1, pfl = 0;  // previous active tile
      auto stage = [&](bool fwd, int ks, int m0, int n0) {
        const int s = it % NS;
        const uint32_t ph = (it / NS) & 1;
        if (!tc::mbar_wait(&empty[s], ph ^ 1, WAIT_LIMIT)) {
          set_abort(&abort_flag);
          atomicExch(a.b.err, TC_ERR_TIMEOUT_PRODUCER);
          ok = false;
          return;
        }
        uint8_t* st = smem + s * L.stage;
        if (fwd) {
          tc::mbar_arrive_expect_tx(&full[s], fbytes);
          tc::tma_load_2d(st, &mF, &full[s], ks * BK, a.frow0);
        } else {
          tc::mbar_arrive_expect_tx(&full[s], bbytes);
          tc::tma_load_2d(st, &mAh, &full[s], ks * BK, m0);
          if (need_alo) tc::tma_load_2d(st + L.offAl, &mAl, &full[s], ks * BK, m0);
          tc::tma_load_2d(st + L.offBh, &mBh, &full[s], ks * BK, a.b.brow0 + n0);
        }
        ++it;
      };
      for (int item = blockIdx.x; item < nitems && ok && !aborted(&abort_flag); item += gridDim.x) {
        const FusedItem f = fused_item(a, item);
        for (int n = f.n_lo; n < f.n_hi && ok; ++n) {
          const int fl = fused_tile(f, n);
          if (!fl) continue;
          if (fl & 1)
            for (int ks = 0; ks < KS && ok; ++ks) stage(false, ks, f.m * BM, n * BWD_BN);
          if (pn >= 0)
            for (int h = 0; h < 2 && ok; ++h)
              if (pfl & (2 << h)) stage(true, 2 * pn + h, 0, 0);
          pn = n;
          pfl = fl;
        }
      }
      if (pn >= 0 && ok)
        for (int h = 0; h < 2 && ok; ++h)
          if (pfl & (2 << h)) stage(true, 2 * pn + h, 0, 0);
      // drain: every issued copy must have landed before the CTA can exit
      for (int i = std::max(0, it - NS); i < it; ++i)
        if (!tc::mbar_wait(&full[i % NS], (i / NS) & 1, WAIT_LIMIT)) atomicExch(a.b.err, TC_ERR_TIMEOUT_DRAIN);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer
      const uint32_t bdesc_i = tc::idesc_bf16_f32(BM, BWD_BN);
      const uint32_t fdesc_i = tc::idesc_bf16_f32(BM, a.NB);
      const uint32_t tY = tmem_base + 256;
      int it = 0, bt = 0, ti = 0, yitems = 0;
      int cnt_ready[XB][2] = {};  // forward uses of each buffer half (aready phases)
      bool ok = true;
      int pn = -1, pfl = 0, pxb = 0;  // previous active tile and its X buffer
      int pleft = 0;                  // forward halves of the previous tile's item still to issue
      bool pfirst = false;            // the previous tile's item has issued no forward MMA yet
      int cur_left = 0;
      bool cur_first = false;
      auto wait_stage = [&]() -> uint32_t {
        const int s = it % NS;
        const uint32_t ph = (it / NS) & 1;
        if (!tc::mbar_wait(&full[s], ph, WAIT_LIMIT)) {
          set_abort(&abort_flag);
          atomicExch(a.b.err, TC_ERR_TIMEOUT_MMA);
          ok = false;
        }
        tc::tc_fence_after();
        return tc::smem_u32(smem + s * L.stage);
      };
      // forward halves of a tile whose update has been converted into its X buffer
      auto forward = [&](int fl, int xb, int& left, bool& first) {
        for (int h = 0; h < 2 && ok; ++h) {
          if (!(fl & (2 << h))) continue;
          if (first && yitems > 0 && !tc::mbar_wait(&ydone, (yitems - 1) & 1, WAIT_LIMIT)) {
            set_abort(&abort_flag);
            atomicExch(a.b.err, TC_ERR_TIMEOUT_MMA);
            ok = false;
            break;
          }
          if (!tc::mbar_wait(&aready[xb][h], cnt_ready[xb][h] & 1, WAIT_LIMIT)) {
            set_abort(&abort_flag);
            atomicExch(a.b.err, TC_ERR_TIMEOUT_MMA);
            ok = false;
            break;
          }
          ++cnt_ready[xb][h];
          const uint32_t st = wait_stage();
          if (!ok) break;
          const uint32_t xa = tc::smem_u32(xs + (xb * 2 + h) * (XHALF / 4));
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            const uint32_t acc = (first && k == 0) ? 0u : 1u;
            const uint64_t dah = tc::desc_kmajor_sw128(xa + 32 * k);
            const uint64_t dbh = tc::desc_kmajor_sw128(st + 32 * k);
            tc::mma_bf16(tY, dah, dbh, fdesc_i, acc);
            if (need_alo) tc::mma_bf16(tY, tc::desc_kmajor_sw128(xa + TILE_A + 32 * k), dbh, fdesc_i, 1u);
          }
          first = false;
          tc::mma_commit(&empty[it % NS]);
          tc::mma_commit(&afree[xb][h]);
          ++it;
          if (--left == 0) {
            tc::mma_commit(&yfull);
            ++yitems;
          }
        }
      };
      for (int item = blockIdx.x; item < nitems && ok && !aborted(&abort_flag); item += gridDim.x) {
        const FusedItem f = fused_item(a, item);
        cur_left = fused_nfwd(f);
        cur_first = true;
        for (int n = f.n_lo; n < f.n_hi && ok; ++n) {
          const int fl = fused_tile(f, n);
          if (!fl) continue;
          if (fl & 1) {
            const int buf = bt & 1;
            if (!tc::mbar_wait(&tempty[buf], ((bt >> 1) & 1) ^ 1, WAIT_LIMIT)) {
              set_abort(&abort_flag);
              atomicExch(a.b.err, TC_ERR_TIMEOUT_MMA);
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint32_t tC = tmem_base + buf * 128;
            for (int ks = 0; ks < KS && ok; ++ks) {
              const uint32_t st = wait_stage();
              if (!ok) break;
#pragma unroll
              for (int k = 0; k < BK / 16; ++k) {
                const uint32_t acc = (ks > 0 || k > 0) ? 1u : 0u;
                const uint64_t dah = tc::desc_kmajor_sw128(st + 32 * k);
                const uint64_t dbh = tc::desc_kmajor_sw128(st + L.offBh + 32 * k);
                tc::mma_bf16(tC, dah, dbh, bdesc_i, acc);
                if (need_alo) tc::mma_bf16(tC, tc::desc_kmajor_sw128(st + L.offAl + 32 * k), dbh, bdesc_i, 1u);
              }
              tc::mma_commit(&empty[it % NS]);
              ++it;
            }
            if (!ok) break;
            tc::mma_commit(&tfull[buf]);
            ++bt;
          }
          if (pn >= 0) forward(pfl, pxb, pleft, pfirst);
          if (!ok) break;
          // this tile becomes the previous one: its forward runs after the next tile's back
          // projection, with its item's count of forward halves still to issue (pleft) and
          // whether it opens the item's Y accumulation (pfirst)
          pn = n;
          pfl = fl;
          pxb = ti % XB;
          pleft = cur_left;
          pfirst = cur_first;
          cur_left -= ((fl >> 1) & 1) + ((fl >> 2) & 1);
          if (((fl >> 1) & 1) + ((fl >> 2) & 1)) cur_first = false;
          ++ti;
        }
      }
      if (pn >= 0 && ok) forward(pfl, pxb, pleft, pfirst);
      // every issued MMA must have completed before TMEM is released
      tc::mma_commit(&mdone);
      if (!tc::mbar_wait(&mdone, 0, WAIT_LIMIT)) atomicExch(a.b.err, TC_ERR_TIMEOUT_DRAIN);
    }
  } else if (warp < BWD_IO_WARP) {
    // ---------------- epilogue: update X (as k_tc_bwd), then the forward operand, then Y
    const int e = warp - 2;
    const int half = e >> 3;
    const int sub = (e & 7) >> 2;
    const int quad = warp & 3;
    const int row = quad * 32 + lane;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    int bt = 0, ti = 0, yitems = 0;
    int cnt_use[XB] = {};  // loads into each buffer
    int cnt_fwd[XB] = {};  // forward uses of this warp's half of each buffer
    bool ok = true;
    for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
      const FusedItem f = fused_item(a, item);
      const int pp = __ldg(a.b.tile_patch + f.m);
      const int* pi = a.b.pinfo + 8 * pp;
      const int m0 = f.m * BM;
      const int local = m0 + row - __ldg(pi + 3);
      const bool pos_ok = local < __ldg(pi + 2);
      int cls = 0;
      {
        const int Li = __ldg(pi + 0), Lj = __ldg(pi + 1);
        const int jj = local / Li, ii = local - jj * Li;
        if (pos_ok) cls = dtab_class(jj, Lj, a.b.q) * a.b.ncls + dtab_class(ii, Li, a.b.q);
      }
      const int ch_lo = __ldg(pi + 4) * a.b.NN;
      const unsigned ch_n = (unsigned)(min(a.b.nch, (__ldg(pi + 4) + __ldg(pi + 5)) * a.b.NN) - ch_lo);
      const float wv = __ldg(a.b.wrow + pp);
      const int nf = fused_nfwd(f);
      for (int n = f.n_lo; n < f.n_hi && ok; ++n) {
        const int fl = fused_tile(f, n);
        if (!fl) continue;
        const int xb = ti % XB, use = cnt_use[xb]++;
        float* xh = xs + (xb * 2 + half) * (XHALF / 4);  // [64 ch][128 pos]
        const int n0 = n * BWD_BN;
        if (aborted(&abort_flag) || !tc::mbar_wait(&xfull[xb][half], use & 1, WAIT_LIMIT)) {
          ok = false;
          break;
        }
        if (fl & 1) {
          const int buf = bt & 1;
          float dpre[16];
          load_dtab16(a.b.dtab + (int64_t)cls * a.b.CHP + n0 + (half * 4 + sub * 2) * 16, dpre);
          if (!tc::mbar_wait(&tfull[buf], (bt >> 1) & 1, WAIT_LIMIT)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t tC = tmem_base + buf * 128 + lane_off;
#pragma unroll
          for (int cc = 0; cc < 2; ++cc) {
            const int c = half * 4 + sub * 2 + cc;
            const int chb = n0 + c * 16;
            float cv[16], dv[16];
            if (cc == 0) {
#pragma unroll
              for (int j = 0; j < 16; ++j) dv[j] = dpre[j];
            } else {
              load_dtab16(a.b.dtab + (int64_t)cls * a.b.CHP + chb, dv);
            }
            tc::tmem_ld16(tC + c * 16, cv);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              float* xp = xh + ((sub * 2 + cc) * 16 + j) * BM + row;
              if (pos_ok && (unsigned)(chb + j - ch_lo) < ch_n) {
                const float xo = *xp;
                float xc = __fdividef(xo * cv[j], dv[j] + a.b.d_eps);  // :130  X .* C ./ D
                if (!(xc >= 0.f) || isinf(xc)) xc = 0.f;               // :132-134
                float xn = __fmaf_rn(xc, wv, __fmul_rn(1.f - wv, xo));  // :136
                if (xn < 0.f) xn = 0.f;                                // :137
                *xp = xn;
              }
            }
          }
          tc::tc_fence_before();
          ++bt;
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(&tempty[buf]);
        }
        // this warp's part of the half written (or read only): the I/O warp may store it
        tc::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&hdone[ti & 1][half]);
        if (fl & (2 << half)) {
          // the stored FP32 half -> BF16 hi / lo forward operand, in place
          if (!tc::mbar_wait(&xstored[xb][half], use & 1, WAIT_LIMIT)) {
            ok = false;
            break;
          }
          float x[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) x[j] = xh[(sub * 32 + j) * BM + row];
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(&rdone[xb][half]);
          if (!tc::mbar_wait(&rdone[xb][half], cnt_fwd[xb]++ & 1, WAIT_LIMIT)) {
            ok = false;
            break;
          }
          uint8_t* xb8 = reinterpret_cast<uint8_t*>(xh);
#pragma unroll
          for (int q8 = 0; q8 < 4; ++q8) {
            const int c8 = sub * 4 + q8;
            __align__(16) bf16 hi[8];
            __align__(16) bf16 lo[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) split_bf16(x[q8 * 8 + j], hi[j], lo[j]);
            const int off = row * 128 + ((c8 ^ (row & 7)) << 4);
            *reinterpret_cast<uint4*>(xb8 + off) = *reinterpret_cast<const uint4*>(hi);
            if (need_alo) *reinterpret_cast<uint4*>(xb8 + TILE_A + off) = *reinterpret_cast<const uint4*>(lo);
          }
          tc::fence_proxy_async_smem();
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(&aready[xb][half]);
        }
        ++ti;
      }
      if (!ok || !f.wnext) continue;
      // the split's partial Y of this position tile: 15 16-column chunks over the 4 warps of
      // this TMEM quadrant (an item without forward K-steps writes zeros, as k_tc_fwd does)
      float* out = a.ypart + (int64_t)f.s * a.NB * a.MP + m0 + row;
      const int wq = e >> 2;  // 0..3: warp within the quadrant
      if (nf > 0) {
        if (!tc::mbar_wait(&yfull, yitems & 1, WAIT_LIMIT)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        for (int c = wq; c < a.NB / 16; c += 4) {
          float v[16];
          tc::tmem_ld16(tmem_base + 256 + lane_off + c * 16, v);
#pragma unroll
          for (int j = 0; j < 16; ++j) out[(int64_t)(c * 16 + j) * a.MP] = v[j];
        }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&ydone);
        ++yitems;
      } else {
        for (int c = wq; c < a.NB / 16; c += 4)
#pragma unroll
          for (int j = 0; j < 16; ++j) out[(int64_t)(c * 16 + j) * a.MP] = 0.f;
      }
    }
    if (!ok) {
      // a wait of this warp gave up (or another role aborted first: keep its status)
      if (lane == 0 && !aborted(&abort_flag)) atomicExch(a.b.err, TC_ERR_TIMEOUT_EPILOGUE);
      set_abort(&abort_flag);
    }
  } else if (warp == BWD_IO_WARP) {
    if (lane == 0) {
      // ---------------- X I/O: first XB active tiles in; per tile store the updated halves,
      // tell the epilogue they are stored, and refill the buffer once the forward MMAs of
      // both halves have read it
      int ti = 0, loaded = 0;
      int cnt_free[XB][2] = {};
      bool ok = true;
      // the active tiles of this CTA in order; next_tile yields the next one not yet loaded
      int li_item = blockIdx.x, li_n = -1;
      FusedItem li_f;
      bool li_valid = false;
      auto next_tile = [&](int& m_out, int& n_out) -> bool {
        while (li_item < nitems) {
          if (!li_valid) {
            li_f = fused_item(a, li_item);
            li_n = li_f.n_lo - 1;
            li_valid = true;
          }
          for (++li_n; li_n < li_f.n_hi; ++li_n)
            if (fused_tile(li_f, li_n)) {
              m_out = li_f.m;
              n_out = li_n;
              return true;
            }
          li_item += gridDim.x;
          li_valid = false;
        }
        return false;
      };
      auto load = [&](int xb, int m, int n) {
        for (int h = 0; h < 2; ++h) {
          tc::mbar_arrive_expect_tx(&xfull[xb][h], XHALF);
          tc::tma_load_2d(xs + (xb * 2 + h) * (XHALF / 4), &mX, &xfull[xb][h], m * BM, n * BWD_BN + 64 * h);
        }
        ++loaded;
      };
      for (int b = 0; b < XB; ++b) {
        int m, n;
        if (!next_tile(m, n)) break;
        load(b, m, n);
      }
      for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
        const FusedItem f = fused_item(a, item);
        for (int n = f.n_lo; n < f.n_hi && ok; ++n) {
          const int fl = fused_tile(f, n);
          if (!fl) continue;
          const int xb = ti % XB;
          for (int h = 0; h < 2 && ok; ++h) {
            if (aborted(&abort_flag) || !tc::mbar_wait(&hdone[ti & 1][h], (ti >> 1) & 1, WAIT_LIMIT)) {
              ok = false;
              break;
            }
            if (fl & 1) {
              tc::tma_store_2d(&mX, xs + (xb * 2 + h) * (XHALF / 4), f.m * BM, n * BWD_BN + 64 * h);
              tc::bulk_commit();
            }
          }
          if (!ok) break;
          tc::bulk_wait_read0();
          for (int h = 0; h < 2; ++h) tc::mbar_arrive(&xstored[xb][h]);
          int m2, n2;
          if (next_tile(m2, n2)) {  // tile ti + XB, into this buffer
            // the buffer is free once the forward MMAs that read its halves are done
            for (int h = 0; h < 2 && ok; ++h) {
              if (!(fl & (2 << h))) continue;
              if (!tc::mbar_wait(&afree[xb][h], cnt_free[xb][h] & 1, WAIT_LIMIT)) ok = false;
              ++cnt_free[xb][h];
            }
            if (!ok) break;
            load(xb, m2, n2);
          } else {
            for (int h = 0; h < 2; ++h)
              if (fl & (2 << h)) ++cnt_free[xb][h];
          }
          ++ti;
        }
      }
      if (!ok) {
        if (!aborted(&abort_flag)) atomicExch(a.b.err, TC_ERR_TIMEOUT_EPILOGUE);
        set_abort(&abort_flag);
      }
      tc::bulk_wait0();
      // loads not consumed (after an abort) must land before the CTA exits
      for (int k = ti; k < loaded; ++k)
        for (int h = 0; h < 2; ++h)
          if (!tc::mbar_wait(&xfull[k % XB][h], (k / XB) & 1, WAIT_LIMIT)) atomicExch(a.b.err, TC_ERR_TIMEOUT_DRAIN);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) tc::tmem_dealloc(tmem_base, 512);
}

// ------------------------------------------------------------------ small kernels
// Tensor-core channels are plane-major (ch = z*N*N + beta*N + alpha); the FP32 tap tables
// are indexed by the channel-major (beta*N + alpha)*Z + z.
__device__ __forceinline__ int64_t tc_to_fp32_channel(int64_t ch, int N, int Z, int* alpha, int* beta) {
  *alpha = (int)(ch % N);
  *beta = (int)((ch / N) % N);
  const int z = (int)(ch / ((int64_t)N * N));
  return ((int64_t)*beta * N + *alpha) * Z + z;
}

// Extended back-projection taps, BF16 hi/lo:  Wb'[view][ch][t'] for the (T+2)^2 window,
// t' = dj'*(T+2) + di', holding wb[view][ch][(dj'-sb-1)*T + (di'-sa-1)] (0 elsewhere).
// FP16 tables: each row scaled by rowscale[view * CHP + ch] (nullable: unscaled).
template <typename E>
__global__ void k_tc_build_wbx(const float* __restrict__ wb, int N, int Z, int T, int64_t nch, int CHP, int KB,
                               const float* __restrict__ rowscale, E* __restrict__ hi, E* __restrict__ lo) {
  const int T2 = T + 2, h = (N - 1) / 2;
  const int64_t total = (int64_t)N * N * CHP * KB;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % KB);
    const int64_t r = e / KB;
    const int64_t ch = r % CHP;
    const int view = (int)(r / CHP);
    float val = 0.f;
    if (ch < nch && k < T2 * T2) {
      const int u = view % N, v = view / N;
      int alpha, beta;
      const int64_t chf = tc_to_fp32_channel(ch, N, Z, &alpha, &beta);
      const int sa = (alpha - u + h + N) / N - 1, sb = (beta - v + h + N) / N - 1;  // floor division
      const int dj = k / T2 - sb - 1, di = k % T2 - sa - 1;
      if (dj >= 0 && dj < T && di >= 0 && di < T)
        val = wb[((int64_t)view * nch + chf) * T * T + dj * T + di];
      if (rowscale) val *= rowscale[r];
    }
    E h16, l16;
    split2(val, h16, l16);
    hi[e] = h16;
    lo[e] = l16;
  }
}

// Forward taps transposed, BF16 hi/lo: Wf'[view][t][ch] = wf[view][ch][t] (t < T^2).
// FP16 tables: each tap column t of a view scaled by 1 / colscale_inv[view * NB + t]
// (nullable: unscaled).
template <typename E>
__global__ void k_tc_build_wft(const float* __restrict__ wf, int N, int Z, int T, int64_t nch, int CHP, int NB,
                               const float* __restrict__ colscale_inv, E* __restrict__ hi, E* __restrict__ lo) {
  const int64_t total = (int64_t)N * N * NB * CHP;
  const int TT = T * T;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ch = e % CHP;
    const int64_t r = e / CHP;
    const int t = (int)(r % NB);
    const int view = (int)(r / NB);
    float val = 0.f;
    if (ch < nch && t < TT) {
      int alpha, beta;
      val = wf[((int64_t)view * nch + tc_to_fp32_channel(ch, N, Z, &alpha, &beta)) * TT + t];
      if (colscale_inv) val *= 1.f / colscale_inv[r];
    }
    E h16, l16;
    split2(val, h16, l16);
    hi[e] = h16;
    lo[e] = l16;
  }
}

// Scales of the FP16 tap tables, one warp per row or column: bscale[view][ch] =
// f16_scale(max_t |wb[view][ch][t]|) for the back-projection rows (it cancels in C / D);
// fsinv[view][t] = 1 / f16_scale(max_ch |wf[view][ch][t]|) for the forward GEMM's columns
// (the forward epilogue multiplies by it).
__global__ void k_tc_f16_scales(const float* __restrict__ wb, const float* __restrict__ wf, int N, int Z, int T,
                                int64_t nch, int CHP, int NB, float* __restrict__ bscale, float* __restrict__ fsinv) {
  const int TT = T * T;
  const int64_t nbr = (int64_t)N * N * CHP, nfr = (int64_t)N * N * NB;
  const int lane = threadIdx.x & 31;
  const int64_t wstride = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nbr + nfr; r += wstride) {
    float m = 0.f;
    int alpha, beta;
    if (r < nbr) {
      const int view = (int)(r / CHP);
      const int64_t ch = r % CHP;
      if (ch < nch) {
        const float* row = wb + ((int64_t)view * nch + tc_to_fp32_channel(ch, N, Z, &alpha, &beta)) * TT;
        for (int t = lane; t < TT; t += 32) m = fmaxf(m, fabsf(row[t]));
      }
    } else {
      const int view = (int)((r - nbr) / NB), t = (int)((r - nbr) % NB);
      if (t < TT)
        for (int64_t ch = lane; ch < nch; ch += 32)
          m = fmaxf(m, fabsf(wf[((int64_t)view * nch + tc_to_fp32_channel(ch, N, Z, &alpha, &beta)) * TT + t]));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) {
      if (r < nbr)
        bscale[r] = f16_scale(m);
      else
        fsinv[r - nbr] = 1.f / f16_scale(m);
    }
  }
}

// *amax = max(*amax, max |x[i]|) over n floats (amax holds a non-negative float).
__global__ void k_tc_absmax(const float* __restrict__ x, int64_t n, float* amax) {
  float m = 0.f;
  const int64_t n4 = n / 4;
  const float4* x4 = reinterpret_cast<const float4*>(x);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 v = __ldg(x4 + i);
    m = fmaxf(fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y))), fmaxf(fabsf(v.z), fabsf(v.w)));
  }
  for (int64_t i = 4 * n4 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[i]));
  const unsigned w = __reduce_max_sync(0xffffffffu, __float_as_uint(m));
  if ((threadIdx.x & 31) == 0 && w != 0u) atomicMax(reinterpret_cast<unsigned*>(amax), w);
}

// im2col of the ratio images (or of ones when R == nullptr) over the (T+2)^2 window, for
// all patches: row = global position, R indexed by global position.  One warp per row; the
// lanes walk the row's KB columns (columns past (T+2)^2 and rows past a patch's positions
// are zero).
// FP16 (rmax non-null): values scaled by f16_scale(*rmax), the ratio image's maximum.
constexpr int IM2COL_WARPS = 8;
template <typename E>
__global__ void __launch_bounds__(32 * IM2COL_WARPS)
k_tc_im2col(const float* __restrict__ R, const int* __restrict__ tile_patch, const int* __restrict__ pinfo,
            int MP, int T, int KB, const float* __restrict__ rmax, E* __restrict__ hi, E* __restrict__ lo) {
  const int T2 = T + 2, q = (T - 1) / 2, KK = T2 * T2;
  const int lane = threadIdx.x & 31;
  const float sc = rmax ? f16_scale(*rmax) : 1.f;
  for (int pos = blockIdx.x * IM2COL_WARPS + (threadIdx.x >> 5); pos < MP; pos += gridDim.x * IM2COL_WARPS) {
    const int* pi = pinfo + 8 * tile_patch[pos / BM];
    const int Li = pi[0], Lj = pi[1], pos0 = pi[3];
    const int local = pos - pos0;
    const bool row_ok = local < pi[2];
    const int b = row_ok ? local / Li : 0;
    const int a = local - b * Li;
    E* hrow = hi + (int64_t)pos * KB;
    E* lrow = lo ? lo + (int64_t)pos * KB : nullptr;
    for (int k = lane; k < KB; k += 32) {
      float val = 0.f;
      if (row_ok && k < KK) {
        const int dj = k / T2;
        const int j = b + dj - q - 1, i = a + (k - dj * T2) - q - 1;
        if (j >= 0 && j < Lj && i >= 0 && i < Li) val = R ? __ldg(R + pos0 + j * Li + i) * sc : 1.f;
      }
      E h16, l16;
      split2(val, h16, l16);
      hrow[k] = h16;
      if (lrow) lrow[k] = l16;
    }
  }
}

// HX[j][i] = sum_{db,da} sum_split Y[split][t = db*T+da][(j+db-q)*Li + (i+da-q)] for every valid
// position of every patch; ratio R = LF_sub ./ HX (non-finite -> 0).  A block covers 32
// consecutive positions (lanes); warp w takes the tap rows db = w, w+16, ..., so each load of
// a warp is 32 consecutive floats of one tap's row.  Four split partials are loaded before
// they are added, so every thread keeps several loads in flight; the warps' sums are added
// in a fixed order (deterministic).  rmax (nullable, FP16 modes) receives max |R|.
constexpr int COL2IM_WARPS = 16;
__global__ void __launch_bounds__(32 * COL2IM_WARPS)
k_tc_col2im_ratio(const float* __restrict__ ypart, int splits, int MP, int NB, int T,
                  const int* __restrict__ tile_patch, const int* __restrict__ pinfo,
                  const float* __restrict__ lfsub, float* __restrict__ hx_out, float* __restrict__ rimg,
                  float* __restrict__ rmax) {
  __shared__ float part[COL2IM_WARPS][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pos = blockIdx.x * 32 + lane;
  float s = 0.f;
  bool valid = pos < MP;
  int pos0 = 0, Li = 1, Lj = 0, j = 0, i = 0;
  if (valid) {
    const int* pi = pinfo + 8 * tile_patch[pos / BM];
    Li = pi[0];
    Lj = pi[1];
    pos0 = pi[3];
    const int local = pos - pos0;
    valid = local < pi[2];
    j = local / Li;
    i = local - j * Li;
  }
  if (valid) {
    const int q = (T - 1) / 2;
    const int64_t sstride = (int64_t)NB * MP;
    const int da_lo = max(0, q - i), da_hi = min(T - 1, Li - 1 - i + q);  // 0 <= i + da - q < Li
    for (int db = w; db < T; db += COL2IM_WARPS) {
      const int b = j + db - q;
      if (b < 0 || b >= Lj) continue;
      // element (db, da): (db*T + da)*MP + pos0 + b*Li + i + da - q
      const float* yrow = ypart + (int64_t)(db * T) * MP + pos0 + (int64_t)b * Li + (i - q);
#pragma unroll 2
      for (int da = da_lo; da <= da_hi; ++da) {
        const float* y = yrow + (int64_t)da * (MP + 1);
        int sp = 0;
        for (; sp + 4 <= splits; sp += 4) {
          const float v0 = __ldg(y + sp * sstride), v1 = __ldg(y + (sp + 1) * sstride);
          const float v2 = __ldg(y + (sp + 2) * sstride), v3 = __ldg(y + (sp + 3) * sstride);
          s += (v0 + v1) + (v2 + v3);
        }
        for (; sp < splits; ++sp) s += __ldg(y + sp * sstride);
      }
    }
  }
  part[w][lane] = s;
  __syncthreads();
  float rabs = 0.f;
  if (w == 0 && valid) {
    float h = 0.f;
#pragma unroll
    for (int k = 0; k < COL2IM_WARPS; ++k) h += part[k][lane];
    if (hx_out) hx_out[pos] = h;
    if (rimg) {
      float r = lfsub[pos] / h;
      if (!isfinite(r)) r = 0.f;
      rimg[pos] = r;
      rabs = fabsf(r);
    }
  }
  if (rmax && w == 0) {
    const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(rabs));
    if (lane == 0 && m != 0u) atomicMax(reinterpret_cast<unsigned*>(rmax), m);
  }
}

// ------------------------------------------------------------------ host side
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int get_encoder() {
  if (g_encode) return MLF_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  MLF_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
  if (q != cudaDriverEntryPointSuccess || !fn)
    return fail(MLF_ERR_CUDA, "cuTensorMapEncodeTiled not available from the driver");
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return MLF_OK;
}

// 2-D BF16 (or FP16) matrix [rows][cols] (cols contiguous, multiple of 64), box 64 x box_rows, SW128.
int make_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols, uint32_t box_rows, bool fp16 = false) {
  MLF_TRY(get_encoder());
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = g_encode(m, fp16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                        const_cast<void*>(base), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MLF_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return MLF_OK;
}

inline int rup(int a, int b) { return (a + b - 1) / b * b; }

}  // namespace

struct TcPsfState {
  int KB = 0, NB = 0, NH = 0, nparts = 1, CHP = 0;
  int fwd_dyn_max = 0;  // dynamic shared memory available to the forward GEMM
  int bwd_dyn_max = 0;  // ... and to the back projection (smallest of its instantiations)
  int fused_dyn_max = 0;  // ... and to the fused back projection + forward
  DevBuf dtab[2];       // D class tables of every view, [view][ncls][ncls][CHP]; taps hi / hi + lo
  DevBuf wbx_hi, wbx_lo, wft_hi, wft_lo;
  CUtensorMap mBh, mBl, mFh, mFl;
  // FP16 forms, built on the first use of an MLF_PREC_FP16* mode: the scaled tap tables,
  // the back-projection row scales [view][CHP], the forward columns' inverse scales
  // [view][NB] and their D class tables
  bool f16_ready = false;
  DevBuf wbx16_hi, wbx16_lo, wft16_hi, wft16_lo, bscale, fsinv, dtab16[2];
  CUtensorMap mBh16, mBl16, mFh16, mFl16;
};

// Work set of P patches sharing one PSF: positions of all patches concatenated (each
// patch padded to whole 128-position tiles), the FP32 volume X[ch][position] of every
// patch, the BF16 operand buffers, the union view order and per-patch view weights.
struct TcSolverState {
  int P = 0, MP = 0, Zch = 0, splits = 1, ks_per_split = 0, KSF = 0, nsm = 0;
  float d_eps = 0.f;  // the members' variant (all the same)
  // launch configuration per precision: split-K count of the forward GEMM (the partials
  // buffer holds splits_max), its ring depth, the back projection's X buffers per half
  struct Tune {
    int done = 0, tuned = 0, splits = 0, ksp = 0, fwd_stages = 0, xbufs = 0;
  };
  Tune tune[kPrecModes];
  int splits_max = 1, splits_def = 1, ksp_def = 0;
  int fwd_stages = 0, xbufs = 0;  // in use (0: derive from shared memory)
  bool dtab_ok = false;  // every patch has >= 2q+2 lenslets per side: D from class tables
  std::vector<int> pos0, Li, Lj, LL, z0, nz;
  std::vector<int> views;   // union of the patches' active views, spiral order
  std::vector<float> wtab;  // [views][P]
  DevBuf X, lfs, rimg, tile_patch, pinfo, wtab_dev, wscratch, ar_hi, ar_lo, a1, ypart, err;
  DevBuf Xprev, relbuf;  // convergence monitor (solves with stats only)
  // FP16 modes: the im2col of ones in FP16, and the operand scales' state: [0] running
  // maximum of X, [1], [2] max |R| of the even / odd view steps of an iteration
  DevBuf a1h, f16s;
  CancelState cancel;       // cancellation of the work set's solves
  // patches taking part in the weights now on the device (a run may leave patches out)
  std::vector<char> active_dev;
  std::vector<float> wtab_cur;  // the uploaded weights ([views][P], left-out patches 0)
  CUtensorMap mARh, mARl, mA1, mA1h, mXv;
  // One RL iteration (view loop + filters of every patch) as an instantiated CUDA graph,
  // per precision and with / without per-view timing nodes.  All buffers above are fixed
  // for the life of the work set, so a captured iteration stays valid.
  struct Iteration {
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;  // kernel nodes
    int tev_used = 0;      // timing events recorded by one replay
  };
  Iteration iter[kPrecModes][2];
  // Captures run on this private stream (the legacy default stream cannot be captured);
  // the instantiated graph is then launched on the caller's stream.
  cudaStream_t capture_stream = nullptr;
  ~TcSolverState() {
    for (auto& row : iter)
      for (auto& g : row)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (capture_stream) cudaStreamDestroy(capture_stream);
  }
};

void tc_psf_free(TcPsfState* t) { delete t; }
void tc_solver_free(TcSolverState* t) { delete t; }

int tc_psf_prepare(Psf* p, cudaStream_t st) {
  if (p->tc) return MLF_OK;
  if (p->T > 17) return fail(MLF_ERR_UNSUPPORTED, "tensor-core path: tap count above 17");
  std::unique_ptr<TcPsfState> t(new TcPsfState());
  t->KB = rup((p->T + 2) * (p->T + 2), BK);
  const int TT = p->T * p->T;
  t->NB = rup(TT, 16);
  if (t->NB > 256) {
    t->NB = rup(TT, 32);
    t->NH = t->NB / 2;
    t->nparts = 2;
  } else {
    t->NH = t->NB;
    t->nparts = 1;
  }
  t->CHP = rup((int)p->nch, 128);
  const int V = p->N * p->N;
  const size_t nb = (size_t)V * t->CHP * t->KB, nf = (size_t)V * t->NB * t->CHP;
  MLF_TRY(t->wbx_hi.alloc(nb * 2, "tc back-projection taps"));
  MLF_TRY(t->wbx_lo.alloc(nb * 2, "tc back-projection taps"));
  MLF_TRY(t->wft_hi.alloc(nf * 2, "tc forward taps"));
  MLF_TRY(t->wft_lo.alloc(nf * 2, "tc forward taps"));
  k_tc_build_wbx<bf16><<<4096, 256, 0, st>>>(p->wb.as<float>(), p->N, p->Z, p->T, p->nch, t->CHP, t->KB,
                                             nullptr, t->wbx_hi.as<bf16>(), t->wbx_lo.as<bf16>());
  k_tc_build_wft<bf16><<<4096, 256, 0, st>>>(p->wf.as<float>(), p->N, p->Z, p->T, p->nch, t->CHP, t->NB,
                                             nullptr, t->wft_hi.as<bf16>(), t->wft_lo.as<bf16>());
  MLF_LAUNCHED();
  MLF_TRY(make_map(&t->mBh, t->wbx_hi.p, (uint64_t)V * t->CHP, t->KB, BWD_BN));
  MLF_TRY(make_map(&t->mBl, t->wbx_lo.p, (uint64_t)V * t->CHP, t->KB, BWD_BN));
  MLF_TRY(make_map(&t->mFh, t->wft_hi.p, (uint64_t)V * t->NB, t->CHP, t->NH));
  MLF_TRY(make_map(&t->mFl, t->wft_lo.p, (uint64_t)V * t->NB, t->CHP, t->NH));
  {
    int optin = 0, dev = 0;
    MLF_CUDA(cudaGetDevice(&dev));
    MLF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fb, ff;
    int bmax = optin, fstat = 0;
    for (const void* f : {(const void*)k_tc_bwd<true, 1, false>, (const void*)k_tc_bwd<false, 1, false>,
                          (const void*)k_tc_bwd<false, 2, false>, (const void*)k_tc_bwd<true, 1, true>,
                          (const void*)k_tc_bwd<false, 1, true>, (const void*)k_tc_bwd<false, 2, true>}) {
      MLF_CUDA(cudaFuncGetAttributes(&fb, f));
      MLF_TRY(allow_max_dyn_smem(f));
      bmax = std::min(bmax, optin - (int)fb.sharedSizeBytes);
    }
    MLF_TRY(allow_max_dyn_smem((const void*)k_tc_dtab<bf16>));
    MLF_TRY(allow_max_dyn_smem((const void*)k_tc_dtab<f16>));
    t->bwd_dyn_max = bmax;
    int fmx = optin;
    for (const void* f : {(const void*)k_tc_bwdfwd<1, 3>, (const void*)k_tc_bwdfwd<2, 2>}) {
      MLF_CUDA(cudaFuncGetAttributes(&fb, f));
      MLF_TRY(allow_max_dyn_smem(f));
      fmx = std::min(fmx, optin - (int)fb.sharedSizeBytes);
    }
    t->fused_dyn_max = fmx;
    if (bwd_smem_bytes(1, 1, true, 1) > (size_t)bmax)
      return fail(MLF_ERR_UNSUPPORTED, "tensor-core back projection needs more shared memory than the device offers");
    for (const void* f : {(const void*)k_tc_fwd<false>, (const void*)k_tc_fwd<true>}) {
      MLF_CUDA(cudaFuncGetAttributes(&ff, f));
      fstat = std::max(fstat, (int)ff.sharedSizeBytes);
    }
    t->fwd_dyn_max = optin - fstat;
    MLF_CUDA(cudaFuncSetAttribute(k_tc_fwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, t->fwd_dyn_max));
    MLF_CUDA(cudaFuncSetAttribute(k_tc_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, t->fwd_dyn_max));
  }
  p->tc = t.release();
  return MLF_OK;
}

// The FP16 tap tables (scaled, see k_tc_f16_scales), built once per PSF on first use.
int tc_f16_prepare(const Psf* p, cudaStream_t st) {
  TcPsfState* t = p->tc;
  if (t->f16_ready) return MLF_OK;
  const int V = p->N * p->N;
  const size_t nb = (size_t)V * t->CHP * t->KB, nf = (size_t)V * t->NB * t->CHP;
  MLF_TRY(t->wbx16_hi.alloc(nb * 2, "tc FP16 back-projection taps"));
  MLF_TRY(t->wbx16_lo.alloc(nb * 2, "tc FP16 back-projection taps"));
  MLF_TRY(t->wft16_hi.alloc(nf * 2, "tc FP16 forward taps"));
  MLF_TRY(t->wft16_lo.alloc(nf * 2, "tc FP16 forward taps"));
  MLF_TRY(t->bscale.alloc((size_t)V * t->CHP * 4, "tc FP16 tap scales"));
  MLF_TRY(t->fsinv.alloc((size_t)V * t->NB * 4, "tc FP16 tap scales"));
  k_tc_f16_scales<<<2048, 256, 0, st>>>(p->wb.as<float>(), p->wf.as<float>(), p->N, p->Z, p->T, p->nch, t->CHP,
                                        t->NB, t->bscale.as<float>(), t->fsinv.as<float>());
  k_tc_build_wbx<f16><<<4096, 256, 0, st>>>(p->wb.as<float>(), p->N, p->Z, p->T, p->nch, t->CHP, t->KB,
                                            t->bscale.as<float>(), t->wbx16_hi.as<f16>(), t->wbx16_lo.as<f16>());
  k_tc_build_wft<f16><<<4096, 256, 0, st>>>(p->wf.as<float>(), p->N, p->Z, p->T, p->nch, t->CHP, t->NB,
                                            t->fsinv.as<float>(), t->wft16_hi.as<f16>(), t->wft16_lo.as<f16>());
  MLF_LAUNCHED();
  MLF_TRY(make_map(&t->mBh16, t->wbx16_hi.p, (uint64_t)V * t->CHP, t->KB, BWD_BN, true));
  MLF_TRY(make_map(&t->mBl16, t->wbx16_lo.p, (uint64_t)V * t->CHP, t->KB, BWD_BN, true));
  MLF_TRY(make_map(&t->mFh16, t->wft16_hi.p, (uint64_t)V * t->NB, t->CHP, t->NH, true));
  MLF_TRY(make_map(&t->mFl16, t->wft16_lo.p, (uint64_t)V * t->NB, t->CHP, t->NH, true));
  t->f16_ready = true;
  return MLF_OK;
}

size_t tc_psf_bytes(const Psf* p) {
  if (!p->tc) return 0;
  const TcPsfState* t = p->tc;
  return t->wbx_hi.bytes + t->wbx_lo.bytes + t->wft_hi.bytes + t->wft_lo.bytes + t->dtab[0].bytes +
         t->dtab[1].bytes + t->wbx16_hi.bytes + t->wbx16_lo.bytes + t->wft16_hi.bytes + t->wft16_lo.bytes +
         t->bscale.bytes + t->fsinv.bytes + t->dtab16[0].bytes + t->dtab16[1].bytes;
}

size_t tc_work_bytes(const TcSolverState* t) {
  if (!t) return 0;
  return t->X.bytes + t->lfs.bytes + t->rimg.bytes + t->tile_patch.bytes + t->pinfo.bytes + t->wtab_dev.bytes +
         t->wscratch.bytes + t->ar_hi.bytes + t->ar_lo.bytes + t->a1.bytes +
         t->ypart.bytes + t->err.bytes + t->Xprev.bytes + t->relbuf.bytes + t->a1h.bytes + t->f16s.bytes;
}

size_t tc_solver_bytes(const Solver* s) { return tc_work_bytes(s->tc); }

size_t tc_work_plan_bytes(const Psf* psf, const std::vector<int>& Li, const std::vector<int>& Lj, int nsm) {
  const int KB = rup((psf->T + 2) * (psf->T + 2), BK);
  const int TT = psf->T * psf->T;
  const int NB = rup(TT, 16) > 256 ? rup(TT, 32) : rup(TT, 16);
  const int64_t CHP = rup((int)psf->nch, 128);
  int64_t MP = 0, tiles = 0;
  for (size_t p = 0; p < Li.size(); ++p) {
    MP += rup(Li[p] * Lj[p], BM);
    tiles += rup(Li[p] * Lj[p], BM) / BM;
  }
  const int KSF = (int)(CHP / BK);
  const int mt = (int)(MP / BM);
  int splits = std::max(1, std::min(KSF, nsm / std::max(1, mt)));
  const int ksp = (KSF + splits - 1) / splits;
  splits = (KSF + ksp - 1) / ksp;
  const int64_t P = (int64_t)Li.size();
  return (size_t)(psf->nch * MP * 4 + (int64_t)psf->N * psf->N * MP * 4 + MP * 4 + tiles * 4 + 8 * P * 4 +
                  (int64_t)psf->N * psf->N * P * 4 + P * 4 + 4 * MP * KB * 2 + 16 +
                  (int64_t)splits * MP * NB * 4 + 4 +
                  // convergence monitor, allocated by the first solve that asks for stats
                  psf->nch * MP * 4 + (int64_t)kRelChangeBufDoubles * 8);
}

int tc_work_create(Psf* psf, const std::vector<Solver*>& members, TcSolverState** out, cudaStream_t st) {
  MLF_TRY(tc_psf_prepare(psf, st));
  const TcPsfState* tp = psf->tc;
  std::unique_ptr<TcSolverState> t(new TcSolverState());
  t->P = (int)members.size();
  t->Zch = psf->Z;
  t->d_eps = solver_d_eps(members[0]);
  int off = 0;
  std::vector<int> info(8 * t->P, 0), tiles;
  for (int p = 0; p < t->P; ++p) {
    const Solver* m = members[p];
    t->pos0.push_back(off);
    t->Li.push_back(m->Li);
    t->Lj.push_back(m->Lj);
    t->LL.push_back(m->Li * m->Lj);
    t->z0.push_back(m->z0);
    t->nz.push_back(m->Z);
    const int* v = &info[8 * p];
    (void)v;
    info[8 * p + 0] = m->Li;
    info[8 * p + 1] = m->Lj;
    info[8 * p + 2] = m->Li * m->Lj;
    info[8 * p + 3] = off;
    info[8 * p + 4] = m->z0;
    info[8 * p + 5] = m->Z;
    const int padded = rup(m->Li * m->Lj, BM);
    for (int k = 0; k < padded / BM; ++k) tiles.push_back(p);
    off += padded;
  }
  t->MP = off;
  // union view order and per-patch weights (plane ranges give per-patch weights)
  std::vector<std::vector<double>> w(t->P);
  for (int p = 0; p < t->P; ++p) w[p] = psf_range_weights(psf, t->z0[p], t->nz[p]);
  for (int view : psf->spiral) {
    bool any = false;
    for (int p = 0; p < t->P; ++p) any = any || w[p][view] != 0.0;
    if (!any) continue;
    t->views.push_back(view);
    for (int p = 0; p < t->P; ++p) t->wtab.push_back((float)w[p][view]);
  }
  t->KSF = tp->CHP / BK;
  MLF_CUDA(cudaDeviceGetAttribute(&t->nsm, cudaDevAttrMultiProcessorCount, members[0]->device));
  const int mt = t->MP / BM;
  t->splits = std::max(1, std::min(t->KSF, t->nsm / std::max(1, mt)));
  // even K-steps per split: a split then covers whole 128-channel tiles (the fused kernel's
  // work items keep the forward GEMM's split boundaries)
  t->ks_per_split = (((t->KSF + t->splits - 1) / t->splits) + 1) & ~1;
  t->splits = (t->KSF + t->ks_per_split - 1) / t->ks_per_split;
  t->splits_def = t->splits;
  t->ksp_def = t->ks_per_split;
  t->splits_max = std::min(t->KSF, 2 * t->splits);
  const int64_t nch = psf->nch;
  MLF_TRY(t->X.alloc((size_t)nch * t->MP * 4, "tc volume (FP32)"));
  MLF_TRY(t->lfs.alloc((size_t)psf->N * psf->N * t->MP * 4, "tc sub-aperture images"));
  MLF_TRY(t->rimg.alloc((size_t)t->MP * 4, "tc ratio image"));
  MLF_TRY(t->tile_patch.alloc(tiles.size() * sizeof(int), "tc tables"));
  MLF_TRY(t->pinfo.alloc(info.size() * sizeof(int), "tc tables"));
  MLF_TRY(t->wtab_dev.alloc(std::max<size_t>(1, t->wtab.size()) * sizeof(float), "tc weights"));
  MLF_TRY(t->wscratch.alloc(std::max(1, t->P) * sizeof(float), "tc weights"));
  MLF_TRY(t->ar_hi.alloc((size_t)t->MP * tp->KB * 2, "tc im2col"));
  MLF_TRY(t->ar_lo.alloc((size_t)t->MP * tp->KB * 2, "tc im2col"));
  MLF_TRY(t->a1.alloc((size_t)t->MP * tp->KB * 2, "tc im2col"));
  MLF_TRY(t->a1h.alloc((size_t)t->MP * tp->KB * 2, "tc im2col"));
  MLF_TRY(t->f16s.alloc(4 * sizeof(float), "tc FP16 operand scales"));
  MLF_TRY(t->cancel.init());
  t->active_dev.assign(t->P, 1);
  MLF_TRY(t->ypart.alloc((size_t)t->splits_max * t->MP * tp->NB * 4, "tc forward partials"));
  MLF_TRY(t->err.alloc(sizeof(int), "tc error flag"));
  t->dtab_ok = true;
  for (int p = 0; p < t->P; ++p)
    t->dtab_ok = t->dtab_ok && t->Li[p] >= 2 * psf->q + 2 && t->Lj[p] >= 2 * psf->q + 2;
  MLF_CUDA(cudaMemcpy(t->tile_patch.p, tiles.data(), tiles.size() * sizeof(int), cudaMemcpyHostToDevice));
  MLF_CUDA(cudaMemcpy(t->pinfo.p, info.data(), info.size() * sizeof(int), cudaMemcpyHostToDevice));
  if (!t->wtab.empty())
    MLF_CUDA(cudaMemcpy(t->wtab_dev.p, t->wtab.data(), t->wtab.size() * sizeof(float), cudaMemcpyHostToDevice));
  MLF_CUDA(cudaMemsetAsync(t->X.p, 0, t->X.bytes, st));
  MLF_CUDA(cudaMemsetAsync(t->lfs.p, 0, t->lfs.bytes, st));
  MLF_CUDA(cudaMemsetAsync(t->err.p, 0, sizeof(int), st));
  MLF_CUDA(cudaMemsetAsync(t->f16s.p, 0, t->f16s.bytes, st));
  k_tc_im2col<bf16><<<(t->MP + IM2COL_WARPS - 1) / IM2COL_WARPS, 32 * IM2COL_WARPS, 0, st>>>(
      nullptr, t->tile_patch.as<int>(), t->pinfo.as<int>(), t->MP, psf->T, tp->KB, nullptr, t->a1.as<bf16>(),
      (bf16*)nullptr);
  k_tc_im2col<f16><<<(t->MP + IM2COL_WARPS - 1) / IM2COL_WARPS, 32 * IM2COL_WARPS, 0, st>>>(
      nullptr, t->tile_patch.as<int>(), t->pinfo.as<int>(), t->MP, psf->T, tp->KB, nullptr, t->a1h.as<f16>(),
      (f16*)nullptr);
  MLF_LAUNCHED();
  // the im2col buffers hold BF16 or FP16 values by mode: the maps only move 2-byte elements
  MLF_TRY(make_map(&t->mARh, t->ar_hi.p, t->MP, tp->KB, BM));
  MLF_TRY(make_map(&t->mARl, t->ar_lo.p, t->MP, tp->KB, BM));
  MLF_TRY(make_map(&t->mA1, t->a1.p, t->MP, tp->KB, BM));
  MLF_TRY(make_map(&t->mA1h, t->a1h.p, t->MP, tp->KB, BM, true));
  {
    MLF_TRY(get_encoder());
    cuuint64_t dims[2] = {(cuuint64_t)t->MP, (cuuint64_t)nch};
    cuuint64_t strides[1] = {(cuuint64_t)t->MP * 4};
    cuuint32_t box[2] = {BM, BWD_BN / 2};
    cuuint32_t es[2] = {1, 1};
    CUresult r = g_encode(&t->mXv, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, t->X.p, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(MLF_ERR_CUDA, "cuTensorMapEncodeTiled (volume) failed: " + std::to_string((int)r));
  }
  *out = t.release();
  return MLF_OK;
}

int tc_solver_prepare(Solver* s, cudaStream_t st) {
  if (s->tc) return MLF_OK;
  return tc_work_create(s->psf, {s}, &s->tc, st);
}

namespace {

// (activation split, tap split) per precision mode
void splits_of(int precision, int* alo, int* blo) {
  *alo = (precision == MLF_PREC_BF16X2 || precision == MLF_PREC_BF16X3 || precision == MLF_PREC_FP16X2 ||
          precision == MLF_PREC_FP16X3) ? 1 : 0;
  *blo = (precision == MLF_PREC_BF16X3 || precision == MLF_PREC_FP16X3) ? 1 : 0;
}
bool act_split(int precision) {
  int alo, blo;
  splits_of(precision, &alo, &blo);
  return alo != 0;
}

// FP16 modes: reset the operand scales' state and take the running maximum of X from the
// whole work-set volume (the start of an iteration, or of a stand-alone projection).
int tc_f16_begin(TcSolverState* t, int precision, cudaStream_t st, int64_t* launches = nullptr) {
  if (!prec_f16(precision)) return MLF_OK;
  MLF_CUDA(cudaMemsetAsync(t->f16s.p, 0, t->f16s.bytes, st));
  k_tc_absmax<<<2 * t->nsm, 512, 0, st>>>(t->X.as<float>(), (int64_t)(t->X.bytes / sizeof(float)), t->f16s.as<float>());
  MLF_LAUNCHED();
  if (launches) ++*launches;
  return MLF_OK;
}

PatchGeo work_geo(const TcSolverState* t, const Solver* m, int p) {
  return PatchGeo{m->N, t->nz[p], t->Zch, t->z0[p], t->Li[p], t->Lj[p], t->Li[p], (int64_t)t->MP, m->Xr, m->Xc, 1};
}

// wview (nullable): per-patch weights of `view`; patches with weight 0 are not projected.
int tc_fwd_launch(const Psf* psf, TcSolverState* t, int precision, int view, cudaStream_t st,
                  const float* wview = nullptr, bool cancellable = false) {
  const TcPsfState* tp = psf->tc;
  int alo, blo;
  splits_of(precision, &alo, &blo);
  TcFwdArgs a{};
  a.ypart = t->ypart.as<float>();
  a.err = t->err.as<int>();
  a.MP = t->MP;
  a.NB = tp->NB;
  a.NH = tp->NH;
  a.nparts = tp->nparts;
  a.ks_per_split = t->ks_per_split;
  a.KS = t->KSF;
  a.frow0 = view * tp->NB;
  a.use_alo = alo;
  a.use_blo = blo;
  a.wview = wview;
  a.tile_patch = t->tile_patch.as<int>();
  a.pinfo = t->pinfo.as<int>();
  a.NN = psf->N * psf->N;
  if (cancellable) a.cancel = cancel_ref(t->cancel);
  const bool use16 = prec_f16(precision);
  if (use16) {
    a.xmax = t->f16s.as<float>();
    a.fsinv = tp->fsinv.as<float>() + (int64_t)view * tp->NB;
  }
  const size_t stage = (size_t)FWD_XTILE + (size_t)tp->NB * 128 * (blo ? 2 : 1);
  a.stages = (int)std::max<size_t>(2, std::min<size_t>(FWD_MAX_STAGES, (size_t)(tp->fwd_dyn_max - 1024) / stage));
  if (t->fwd_stages > 0 && (size_t)t->fwd_stages * stage + 1024 <= (size_t)tp->fwd_dyn_max) a.stages = t->fwd_stages;
  const size_t fsmem = (size_t)a.stages * stage + 1024;
  if (fsmem > (size_t)tp->fwd_dyn_max)
    return fail(MLF_ERR_UNSUPPORTED, "tensor-core forward projection: taps tile exceeds shared memory");
  if (use16)
    k_tc_fwd<true><<<dim3(t->MP / BM, t->splits), FWD_THREADS, fsmem, st>>>(t->mXv, tp->mFh16, tp->mFl16, a);
  else
    k_tc_fwd<false><<<dim3(t->MP / BM, t->splits), FWD_THREADS, fsmem, st>>>(t->mXv, tp->mFh, tp->mFl, a);
  MLF_LAUNCHED();
  return MLF_OK;
}

// slot (FP16 modes): the max |R| slot of this view step (its parity within the iteration)
int tc_col2im(const Psf* psf, TcSolverState* t, int view, bool ratio, float* hx_out, cudaStream_t st,
              int precision = MLF_PREC_BF16X2, int slot = 0) {
  float* rmax = (ratio && prec_f16(precision)) ? t->f16s.as<float>() + 1 + slot : nullptr;
  k_tc_col2im_ratio<<<(t->MP + 31) / 32, 32 * COL2IM_WARPS, 0, st>>>(
      t->ypart.as<float>(), t->splits, t->MP, psf->tc->NB, psf->T, t->tile_patch.as<int>(), t->pinfo.as<int>(),
      t->lfs.as<float>() + (int64_t)view * t->MP, hx_out, ratio ? t->rimg.as<float>() : nullptr, rmax);
  MLF_LAUNCHED();
  return MLF_OK;
}

int tc_im2col_ratio(const Psf* psf, TcSolverState* t, int precision, cudaStream_t st, int slot = 0) {
  const dim3 grid((t->MP + IM2COL_WARPS - 1) / IM2COL_WARPS), block(32 * IM2COL_WARPS);
  if (prec_f16(precision))
    k_tc_im2col<f16><<<grid, block, 0, st>>>(t->rimg.as<float>(), t->tile_patch.as<int>(), t->pinfo.as<int>(), t->MP,
                                             psf->T, psf->tc->KB, t->f16s.as<float>() + 1 + slot,
                                             t->ar_hi.as<f16>(), act_split(precision) ? t->ar_lo.as<f16>() : nullptr);
  else
    k_tc_im2col<bf16><<<grid, block, 0, st>>>(t->rimg.as<float>(), t->tile_patch.as<int>(), t->pinfo.as<int>(),
                                              t->MP, psf->T, psf->tc->KB, nullptr, t->ar_hi.as<bf16>(),
                                              act_split(precision) ? t->ar_lo.as<bf16>() : nullptr);
  MLF_LAUNCHED();
  return MLF_OK;
}

// D class tables of every view for one tap split, built on first use (outside any graph
// capture: it allocates) and kept with the PSF.
int tc_dtab_prepare(const Psf* psf, int precision, cudaStream_t st) {
  int alo, blo;
  splits_of(precision, &alo, &blo);
  TcPsfState* tp = psf->tc;
  const bool use16 = prec_f16(precision);
  DevBuf& dt = use16 ? tp->dtab16[blo] : tp->dtab[blo];
  if (dt.p) return MLF_OK;
  const int nc = 2 * psf->q + 3, V = psf->N * psf->N;
  MLF_TRY(dt.alloc((size_t)V * nc * nc * tp->CHP * sizeof(float), "tc D class tables"));
  const size_t dsm = sizeof(float) * 64 * (size_t)dtab_ch_words(psf->T);
  if (use16)
    k_tc_dtab<f16><<<dim3(tp->CHP / 32, V), DTAB_THREADS, dsm, st>>>(
        tp->wbx16_hi.as<f16>(), blo ? tp->wbx16_lo.as<f16>() : nullptr, tp->CHP, tp->KB, psf->T, dt.as<float>());
  else
    k_tc_dtab<bf16><<<dim3(tp->CHP / 32, V), DTAB_THREADS, dsm, st>>>(
        tp->wbx_hi.as<bf16>(), blo ? tp->wbx_lo.as<bf16>() : nullptr, tp->CHP, tp->KB, psf->T, dt.as<float>());
  MLF_LAUNCHED();
  return MLF_OK;
}

int tc_bwd_launch(const Psf* psf, TcSolverState* t, int precision, int view, const float* wrow, cudaStream_t st,
                  int slot = 0, bool cancellable = false) {
  const TcPsfState* tp = psf->tc;
  int alo, blo;
  splits_of(precision, &alo, &blo);
  const bool dgemm = !t->dtab_ok;
  const bool use16 = prec_f16(precision);
  const int q = psf->q, nc = 2 * q + 3;
  const DevBuf& dt = use16 ? tp->dtab16[blo] : tp->dtab[blo];
  if (!dgemm && !dt.p) return fail(MLF_ERR_INVALID, "tensor-core D class tables not prepared");
  TcBwdArgs a{};
  a.err = t->err.as<int>();
  a.tile_patch = t->tile_patch.as<int>();
  a.pinfo = t->pinfo.as<int>();
  a.wrow = wrow;
  a.CHP = tp->CHP; a.nch = (int)psf->nch; a.KB = tp->KB; a.brow0 = view * tp->CHP; a.NN = psf->N * psf->N;
  a.use_alo = alo;
  a.use_blo = blo;
  a.d_eps = t->d_eps;
  a.dtab = dgemm ? nullptr : dt.as<float>() + (int64_t)view * nc * nc * tp->CHP;
  a.q = q;
  a.ncls = nc;
  if (cancellable) a.cancel = cancel_ref(t->cancel);
  if (use16) {
    a.rmax = t->f16s.as<float>() + 1 + slot;
    a.rmax_next = t->f16s.as<float>() + 1 + (slot ^ 1);
    a.xmax = t->f16s.as<float>();
    a.bscale = tp->bscale.as<float>() + (int64_t)view * tp->CHP;
  }
  const int mt = t->MP / BM, nt = tp->CHP / BWD_BN;
  const int grid = std::min(mt * nt, t->nsm);
  // two X buffers when they fit (D from tables frees the A1 operand's ring slots)
  int xbufs = (!dgemm && bwd_smem_bytes(alo, blo, false, 2) <= (size_t)tp->bwd_dyn_max) ? 2 : 1;
  if (t->xbufs == 1) xbufs = 1;
  const size_t smem = bwd_smem_bytes(alo, blo, dgemm, xbufs);
  if (use16) {
    const CUtensorMap &mBh = tp->mBh16, &mBl = tp->mBl16;
    if (dgemm)
      k_tc_bwd<true, 1, true><<<grid, BWD_THREADS, smem, st>>>(t->mARh, t->mARl, t->mA1h, mBh, mBl, t->mXv, a, mt, nt);
    else if (xbufs == 2)
      k_tc_bwd<false, 2, true><<<grid, BWD_THREADS, smem, st>>>(t->mARh, t->mARl, t->mA1h, mBh, mBl, t->mXv, a, mt, nt);
    else
      k_tc_bwd<false, 1, true><<<grid, BWD_THREADS, smem, st>>>(t->mARh, t->mARl, t->mA1h, mBh, mBl, t->mXv, a, mt, nt);
  } else {
    if (dgemm)
      k_tc_bwd<true, 1, false><<<grid, BWD_THREADS, smem, st>>>(t->mARh, t->mARl, t->mA1, tp->mBh, tp->mBl, t->mXv, a,
                                                                mt, nt);
    else if (xbufs == 2)
      k_tc_bwd<false, 2, false><<<grid, BWD_THREADS, smem, st>>>(t->mARh, t->mARl, t->mA1, tp->mBh, tp->mBl, t->mXv, a,
                                                                 mt, nt);
    else
      k_tc_bwd<false, 1, false><<<grid, BWD_THREADS, smem, st>>>(t->mARh, t->mARl, t->mA1, tp->mBh, tp->mBl, t->mXv, a,
                                                                 mt, nt);
  }
  MLF_LAUNCHED();
  return MLF_OK;
}


// The fused back projection + next forward applies to the BF16 modes with D from the class
// tables, a forward taps tile of one MMA (N <= 256) and even split sizes; MLF_FUSED=0 keeps
// the two kernels.
bool tc_fused_ok(const Psf* psf, const TcSolverState* t, int precision) {
  if (precision != MLF_PREC_BF16 && precision != MLF_PREC_BF16X2) return false;
  const TcPsfState* tp = psf->tc;
  if (!t->dtab_ok || tp->nparts != 1 || tp->NB > 256 || t->ks_per_split % 2 != 0) return false;
  const char* env = std::getenv("MLF_FUSED");
  if (env && std::strcmp(env, "0") == 0) return false;
  int alo, blo;
  splits_of(precision, &alo, &blo);
  return !blo && 3 * (size_t)bwd_layout(alo, 0, false).stage + XTILE + 1024 <= (size_t)tp->fused_dyn_max;
}

int tc_bwdfwd_launch(const Psf* psf, TcSolverState* t, int precision, int view, int view_next, const float* wrow,
                     const float* wnext, cudaStream_t st, bool cancellable = false) {
  const TcPsfState* tp = psf->tc;
  int alo, blo;
  splits_of(precision, &alo, &blo);
  const int q = psf->q, nc = 2 * q + 3;
  const DevBuf& dt = tp->dtab[0];
  if (!dt.p) return fail(MLF_ERR_INVALID, "tensor-core D class tables not prepared");
  TcFusedArgs a{};
  a.b.err = t->err.as<int>();
  a.b.tile_patch = t->tile_patch.as<int>();
  a.b.pinfo = t->pinfo.as<int>();
  a.b.wrow = wrow;
  a.b.CHP = tp->CHP; a.b.nch = (int)psf->nch; a.b.KB = tp->KB; a.b.brow0 = view * tp->CHP; a.b.NN = psf->N * psf->N;
  a.b.use_alo = alo;
  a.b.use_blo = 0;
  a.b.d_eps = t->d_eps;
  a.b.dtab = dt.as<float>() + (int64_t)view * nc * nc * tp->CHP;
  a.b.q = q;
  a.b.ncls = nc;
  if (cancellable) a.b.cancel = cancel_ref(t->cancel);
  a.ypart = t->ypart.as<float>();
  a.wview = wnext;
  a.MP = t->MP;
  a.NB = tp->NB;
  a.splits = t->splits;
  a.ks_per_split = t->ks_per_split;
  a.KS = t->KSF;
  a.frow0 = view_next * tp->NB;
  a.ntiles = tp->CHP / BWD_BN;
  const int nitems = (t->MP / BM) * t->splits;
  const int grid = std::min(nitems, t->nsm);
  // (X buffers, ring stages): (2, 2), or (1, 3) where two X buffers do not fit or the
  // environment sets MLF_FUSED_XB=1 (slower on the 1005 x 1005 x 51 workload: 0.218 vs
  // 0.189 ms per view, the single X buffer serialises the tiles)
  const size_t stage = (size_t)bwd_layout(alo, 0, false).stage;
  const size_t smem22 = 2 * stage + 2 * (size_t)XTILE + 1024, smem13 = 3 * stage + (size_t)XTILE + 1024;
  const char* env = std::getenv("MLF_FUSED_XB");
  bool one = env && std::strcmp(env, "1") == 0;
  if (smem22 > (size_t)tp->fused_dyn_max) one = true;
  if (one && smem13 > (size_t)tp->fused_dyn_max) return fail(MLF_ERR_UNSUPPORTED, "fused view step: shared memory");
  if (one)
    k_tc_bwdfwd<1, 3><<<grid, BWD_THREADS, smem13, st>>>(t->mARh, t->mARl, tp->mBh, t->mXv, tp->mFh, a, nitems);
  else
    k_tc_bwdfwd<2, 2><<<grid, BWD_THREADS, smem22, st>>>(t->mARh, t->mARl, tp->mBh, t->mXv, tp->mFh, a, nitems);
  MLF_LAUNCHED();
  return MLF_OK;
}

// The view loop of one iteration over all patches of the work set.
int tc_enqueue_views(const Psf* psf, TcSolverState* t, int precision, Solver* timer, int64_t* launches,
                     cudaStream_t st) {
  const int V = (int)t->views.size();
  if (V == 0) return MLF_OK;
  int64_t n = 0;
  MLF_TRY(tc_f16_begin(t, precision, st, &n));
  MLF_TRY(timing_mark(timer, st));
  MLF_TRY(tc_fwd_launch(psf, t, precision, t->views[0], st, t->wtab_dev.as<float>(), true));
  MLF_TRY(timing_mark(timer, st));
  MLF_TRY(tc_col2im(psf, t, t->views[0], true, nullptr, st, precision, 0));
  MLF_TRY(tc_im2col_ratio(psf, t, precision, st, 0));
  n += 3;
  const bool fused = tc_fused_ok(psf, t, precision);
  for (int k = 0; k < V; ++k) {
    MLF_TRY(timing_mark(timer, st));
    if (fused && k + 1 < V) {
      // back projection of view k and forward projection of view k+1 in one launch
      MLF_TRY(tc_bwdfwd_launch(psf, t, precision, t->views[k], t->views[k + 1],
                               t->wtab_dev.as<float>() + (size_t)k * t->P,
                               t->wtab_dev.as<float>() + (size_t)(k + 1) * t->P, st, true));
      MLF_TRY(timing_mark(timer, st));
      MLF_TRY(tc_col2im(psf, t, t->views[k + 1], true, nullptr, st, precision, (k + 1) & 1));
      MLF_TRY(tc_im2col_ratio(psf, t, precision, st, (k + 1) & 1));
      n += 3;
      continue;
    }
    MLF_TRY(tc_bwd_launch(psf, t, precision, t->views[k], t->wtab_dev.as<float>() + (size_t)k * t->P, st, k & 1, true));
    ++n;
    if (k + 1 < V) {
      MLF_TRY(tc_fwd_launch(psf, t, precision, t->views[k + 1], st, t->wtab_dev.as<float>() + (size_t)(k + 1) * t->P,
                            true));
      MLF_TRY(timing_mark(timer, st));
      MLF_TRY(tc_col2im(psf, t, t->views[k + 1], true, nullptr, st, precision, (k + 1) & 1));
      MLF_TRY(tc_im2col_ratio(psf, t, precision, st, (k + 1) & 1));
      n += 3;
    } else {
      MLF_TRY(timing_mark(timer, st));
    }
  }
  if (launches) *launches += n;
  return MLF_OK;
}

// Capture one RL iteration over the work set into an executable graph.
int capture_iteration(const Psf* psf, TcSolverState* t, const std::vector<Solver*>& members, int precision,
                      Solver* timer, TcSolverState::Iteration* out) {
  if (!t->capture_stream) MLF_CUDA(cudaStreamCreateWithFlags(&t->capture_stream, cudaStreamNonBlocking));
  cudaStream_t st = t->capture_stream;
  std::lock_guard<std::recursive_mutex> lk(device_mutex());
  MLF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  int64_t launches = 0;
  int rc = tc_enqueue_views(psf, t, precision, timer, &launches, st);
  for (int p = 0; rc == MLF_OK && p < t->P; ++p) {
    rc = filter_run_geo(members[p], work_geo(t, members[p], p), t->X.as<float>() + t->pos0[p], st);
    launches += 5;
  }
  // the instrumented variant (stats requested) also measures the iteration's relative change
  if (rc == MLF_OK && timer->timing && t->Xprev.p) {
    rc = launch_rel_change(t->X.as<float>(), t->Xprev.as<float>(), (int64_t)(t->X.bytes / sizeof(float)),
                           t->relbuf.as<double>(), st);
    launches += 2;
  }
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &g);
  if (rc != MLF_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(MLF_ERR_CUDA, std::string("capture of the RL iteration: ") + cudaGetErrorString(ce));
  }
  const cudaError_t ie = cudaGraphInstantiateWithFlags(&out->exec, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) {
    out->exec = nullptr;
    return fail(MLF_ERR_CUDA, std::string("instantiate the RL iteration graph: ") + cudaGetErrorString(ie));
  }
  out->launches = launches;
  out->tev_used = timer->tev_used;
  return MLF_OK;
}

}  // namespace

// The launch configuration of this precision (tuned, or the heuristics) into effect.
void tc_apply_tune(TcSolverState* t, int precision) {
  const TcSolverState::Tune& g = t->tune[precision];
  if (g.done) {
    t->splits = g.splits;
    t->ks_per_split = g.ksp;
    t->fwd_stages = g.fwd_stages;
    t->xbufs = g.xbufs;
  } else {
    t->splits = t->splits_def;
    t->ks_per_split = t->ksp_def;
    t->fwd_stages = 0;
    t->xbufs = 0;
  }
}

// Autotuner: time the candidate launch configurations on the first view step of the work
// set (forward GEMM: split-K count in {s/2, s, 2s} x ring depth in {2, 3, 4}; back
// projection: one or two X buffers per half) and keep the fastest.  X is saved before and
// restored after, so the solve is unaffected.  Runs once per work set and precision, before
// the iteration is captured; MLF_TUNE=0 keeps the heuristics.
int tc_autotune(const Psf* psf, TcSolverState* t, int precision, cudaStream_t st) {
  TcSolverState::Tune& g = t->tune[precision];
  if (g.done) return MLF_OK;
  g.done = 1;
  g.splits = t->splits_def;
  g.ksp = t->ksp_def;
  const char* env = std::getenv("MLF_TUNE");
  if ((env && std::strcmp(env, "0") == 0) || t->views.empty()) return MLF_OK;
  DevBuf xsave;
  MLF_TRY(xsave.alloc(t->X.bytes, "autotune volume copy"));
  MLF_CUDA(cudaMemcpyAsync(xsave.p, t->X.p, t->X.bytes, cudaMemcpyDeviceToDevice, st));
  MLF_TRY(tc_f16_begin(t, precision, st));
  cudaEvent_t e0, e1;
  MLF_CUDA(cudaEventCreate(&e0));
  MLF_CUDA(cudaEventCreate(&e1));
  auto timed = [&](auto&& launch, float* ms) -> int {
    MLF_TRY(launch());  // warm
    MLF_CUDA(cudaEventRecord(e0, st));
    for (int r = 0; r < 2; ++r) MLF_TRY(launch());
    MLF_CUDA(cudaEventRecord(e1, st));
    MLF_CUDA(cudaEventSynchronize(e1));
    MLF_CUDA(cudaEventElapsedTime(ms, e0, e1));
    return MLF_OK;
  };
  const int v0 = t->views[0];
  const float* w0 = t->wtab_dev.as<float>();
  float best = 1e30f;
  for (int s : {std::max(1, t->splits_def / 2), t->splits_def, t->splits_max}) {
    const int ksp = (((t->KSF + s - 1) / s) + 1) & ~1;
    const int sp = (t->KSF + ksp - 1) / ksp;
    if (sp > t->splits_max) continue;
    for (int stg = 2; stg <= FWD_MAX_STAGES; ++stg) {
      t->splits = sp;
      t->ks_per_split = ksp;
      t->fwd_stages = stg;
      float ms = 0.f;
      MLF_TRY(timed([&] { return tc_fwd_launch(psf, t, precision, v0, st, w0); }, &ms));
      if (ms < best) {
        best = ms;
        g.splits = sp;
        g.ksp = ksp;
        g.fwd_stages = stg;
      }
    }
  }
  // the back projection needs the ratio image of view 0 under the chosen forward
  t->splits = g.splits;
  t->ks_per_split = g.ksp;
  t->fwd_stages = g.fwd_stages;
  MLF_TRY(tc_fwd_launch(psf, t, precision, v0, st, w0));
  MLF_TRY(tc_col2im(psf, t, v0, true, nullptr, st, precision, 0));
  MLF_TRY(tc_im2col_ratio(psf, t, precision, st, 0));
  if (t->dtab_ok) {
    best = 1e30f;
    for (int xb = 1; xb <= 2; ++xb) {
      t->xbufs = xb;
      float ms = 0.f;
      MLF_TRY(timed([&] {
        MLF_CUDA(cudaMemcpyAsync(t->X.p, xsave.p, t->X.bytes, cudaMemcpyDeviceToDevice, st));
        return tc_bwd_launch(psf, t, precision, v0, w0, st);
      }, &ms));
      if (ms < best) {
        best = ms;
        g.xbufs = xb;
      }
    }
  }
  MLF_CUDA(cudaMemcpyAsync(t->X.p, xsave.p, t->X.bytes, cudaMemcpyDeviceToDevice, st));
  MLF_CUDA(cudaStreamSynchronize(st));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  g.tuned = 1;
  return MLF_OK;
}

int tc_run(TcSolverState* t, const std::vector<Solver*>& members, const std::vector<const float*>& lf,
           const std::vector<const float*>& warm, const std::vector<float*>& out, int max_iter, int precision,
           mlf_stats* stats, Solver* timer, cudaStream_t st) {
  const Psf* psf = members[0]->psf;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (stats) {
    MLF_CUDA(cudaEventCreate(&e0));
    MLF_CUDA(cudaEventCreate(&e1));
    MLF_CUDA(cudaEventRecord(e0, st));
  }
  for (Solver* m : members) MLF_TRY(lite_prepare(m));  // filter plans of batch members (allocates)
  timer->timing = stats != nullptr;
  timer->tev_used = 0;
  int64_t launches = 0;
  // patches without an image sit this run out: their weights are 0 for every view (their
  // tiles are skipped, their X left as it is) and nothing of theirs is read or written
  {
    std::vector<char> active(t->P);
    for (int p = 0; p < t->P; ++p) active[p] = lf[p] != nullptr;
    if (active != t->active_dev) {
      const size_t V = t->views.size();
      t->wtab_cur.assign(t->wtab.begin(), t->wtab.end());
      for (size_t k = 0; k < V; ++k)
        for (int p = 0; p < t->P; ++p)
          if (!active[p]) t->wtab_cur[k * t->P + p] = 0.f;
      if (!t->wtab_cur.empty())
        MLF_CUDA(cudaMemcpyAsync(t->wtab_dev.p, t->wtab_cur.data(), t->wtab_cur.size() * sizeof(float),
                                 cudaMemcpyHostToDevice, st));
      t->active_dev = active;
    }
  }
  MLF_TRY(t->cancel.begin(st));
  ++launches;
  if (prec_f16(precision)) MLF_TRY(tc_f16_prepare(psf, st));
  if (t->dtab_ok) MLF_TRY(tc_dtab_prepare(psf, precision, st));
  for (int p = 0; p < t->P; ++p) {
    if (!lf[p]) continue;
    const PatchGeo g = work_geo(t, members[p], p);
    float* Xp = t->X.as<float>() + t->pos0[p];
    MLF_TRY(launch_extract_views(lf[p], g, t->lfs.as<float>(), t->MP, t->pos0[p], st));
    if (warm[p]) {
      MLF_TRY(launch_to_phase(warm[p], g, Xp, st));
      launches += 2;
    } else {
      MLF_TRY(launch_init_flat(lf[p], g, Xp, members[p]->red.as<double>(), st));
      launches += 3;
    }
  }
  const bool monitor = stats != nullptr && max_iter > 0;
  if (monitor) {  // before any capture: these allocate
    if (!t->Xprev.p) MLF_TRY(t->Xprev.alloc(t->X.bytes, "convergence monitor volume"));
    if (!t->relbuf.p) MLF_TRY(t->relbuf.alloc(kRelChangeBufDoubles * sizeof(double), "convergence monitor sums"));
  }
  if (max_iter > 0) {
    MLF_TRY(tc_autotune(psf, t, precision, st));  // first solve at this precision only
    tc_apply_tune(t, precision);
    if (monitor) MLF_CUDA(cudaMemcpyAsync(t->Xprev.p, t->X.p, t->X.bytes, cudaMemcpyDeviceToDevice, st));
    TcSolverState::Iteration& g = t->iter[precision][timer->timing ? 1 : 0];
    if (!g.exec) {
      timer->tev_used = 0;
      MLF_TRY(capture_iteration(psf, t, members, precision, timer, &g));
    }
    // The timing events of the graph are re-recorded by every replay; the per-view kernel
    // time reported is that of the last iteration, times the iteration count.
    timer->tev_used = g.tev_used;
    for (int it = 0; it < max_iter; ++it) MLF_CUDA(cudaGraphLaunch(g.exec, st));
    launches += g.launches * max_iter;
  }
  for (int p = 0; p < t->P; ++p) {
    if (!lf[p]) continue;
    MLF_TRY(launch_from_phase(t->X.as<float>() + t->pos0[p], work_geo(t, members[p], p), out[p], st,
                              t->cancel.stop.as<int>()));
    ++launches;
  }
  if (stats) {
    MLF_CUDA(cudaEventRecord(e1, st));
    MLF_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    MLF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    stats->n_views = (int)t->views.size();
    stats->iterations = max_iter;
    stats->gpu_ms = ms;
    stats->view_ms = (max_iter > 0 && stats->n_views > 0) ? ms / (max_iter * stats->n_views) : 0.0;
    double vk = 0.0;
    for (int k = 0; k + 1 < timer->tev_used; k += 2) {
      float tt = 0.f;
      MLF_CUDA(cudaEventElapsedTime(&tt, timer->tev[k], timer->tev[k + 1]));
      vk += tt;
    }
    stats->view_kernel_ms = vk * max_iter;
    stats->view_kernel_launches = (int64_t)(timer->tev_used / 2) * max_iter;
    stats->kernel_launches = launches;
    stats->fwd_splits = t->splits;
    stats->fwd_stages = t->fwd_stages;
    stats->bwd_xbufs = t->xbufs ? t->xbufs : (t->dtab_ok ? 2 : 1);
    stats->tuned = t->tune[precision].tuned;
    stats->rel_change = 0.0;
    if (monitor) MLF_TRY(rel_change_read(t->relbuf.as<double>(), &stats->rel_change));
    MLF_TRY(tc_check_error(t));
    if (t->cancel.stopped()) {
      timer->timing = false;
      timer->tev_used = 0;
      return fail(MLF_ERR_CANCELLED, "solve cancelled between view steps; outputs left unwritten");
    }
  }
  timer->timing = false;
  timer->tev_used = 0;
  return MLF_OK;
}

CancelState& tc_cancel_state(TcSolverState* t) { return t->cancel; }

// Forward projection of one view with the tensor cores (parity tests), single solver.
int tc_forward_view(Solver* s, int precision, const float* d_vol, int view, float* hx_out, cudaStream_t st) {
  TcSolverState* t = s->tc;
  tc_apply_tune(t, precision);
  if (prec_f16(precision)) MLF_TRY(tc_f16_prepare(s->psf, st));
  MLF_TRY(launch_to_phase(d_vol, work_geo(t, s, 0), t->X.as<float>(), st));
  MLF_TRY(tc_f16_begin(t, precision, st));
  MLF_TRY(tc_fwd_launch(s->psf, t, precision, view, st));
  return tc_col2im(s->psf, t, view, false, hx_out, st);
}

int tc_forward_project(TcSolverState* t, const std::vector<Solver*>& members, const std::vector<const float*>& vols,
                       const std::vector<float*>& lf_out, int precision, const float* zscale, cudaStream_t st) {
  const Psf* psf = members[0]->psf;
  const int N = psf->N;
  tc_apply_tune(t, precision);
  if (prec_f16(precision)) MLF_TRY(tc_f16_prepare(psf, st));
  for (int p = 0; p < t->P; ++p)
    MLF_TRY(launch_to_phase(vols[p], work_geo(t, members[p], p), t->X.as<float>() + t->pos0[p], st,
                            zscale ? zscale + t->z0[p] : nullptr));
  MLF_TRY(tc_f16_begin(t, precision, st));
  for (int view = 0; view < N * N; ++view) {
    MLF_TRY(tc_fwd_launch(psf, t, precision, view, st));
    MLF_TRY(tc_col2im(psf, t, view, false, t->lfs.as<float>() + (int64_t)view * t->MP, st));
  }
  for (int p = 0; p < t->P; ++p)
    MLF_TRY(launch_scatter_views(t->lfs.as<float>(), work_geo(t, members[p], p), lf_out[p], t->MP, t->pos0[p], st));
  return MLF_OK;
}

// One RL view step on the tensor cores (parity tests), single solver.
int tc_view_step(Solver* s, int precision, const float* d_lf, float* d_vol, int view, float w, cudaStream_t st) {
  TcSolverState* t = s->tc;
  tc_apply_tune(t, precision);
  const PatchGeo g = work_geo(t, s, 0);
  MLF_TRY(launch_extract_views(d_lf, g, t->lfs.as<float>(), t->MP, 0, st));
  MLF_TRY(launch_to_phase(d_vol, g, t->X.as<float>(), st));
  MLF_CUDA(cudaMemcpyAsync(t->wscratch.p, &w, sizeof(float), cudaMemcpyHostToDevice, st));
  if (prec_f16(precision)) MLF_TRY(tc_f16_prepare(s->psf, st));
  if (t->dtab_ok) MLF_TRY(tc_dtab_prepare(s->psf, precision, st));
  MLF_TRY(tc_f16_begin(t, precision, st));
  MLF_TRY(tc_fwd_launch(s->psf, t, precision, view, st));
  MLF_TRY(tc_col2im(s->psf, t, view, true, nullptr, st, precision, 0));
  MLF_TRY(tc_im2col_ratio(s->psf, t, precision, st, 0));
  MLF_TRY(tc_bwd_launch(s->psf, t, precision, view, t->wscratch.as<float>(), st, 0));
  MLF_TRY(launch_from_phase(t->X.as<float>(), g, d_vol, st));
  MLF_CUDA(cudaStreamSynchronize(st));
  return MLF_OK;
}

int tc_check_error(TcSolverState* t) {
  if (!t) return MLF_OK;
  int e = 0;
  MLF_CUDA(cudaMemcpy(&e, t->err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (e != 0) {
    cudaMemset(t->err.p, 0, sizeof(int));
    return fail(MLF_ERR_TIMEOUT, "tensor-core kernel wait timed out (code " + std::to_string(e) + ")");
  }
  return MLF_OK;
}

}  // namespace mlf
