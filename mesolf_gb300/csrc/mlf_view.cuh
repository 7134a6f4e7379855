// Per-view phase-space RL kernel (plain FP32 path).
//
// The volume lives in phase-major layout: channel ch = (beta*N + alpha)*Z + z holds the
// coarse plane P_ch[b][a] = X(N*a + alpha, N*b + beta, z) (row pitch Pa).  In that layout
// the reference's per-view operators (recon_theory_phase_space_LFM_with_filter.m:211-249)
// become, per channel, small dense correlations on the lenslet grid:
//
//   forward  (:243-249)  HX[j][i]  += sum_{db,da} P_ch[j+db-q][i+da-q] * wf_ch[db][da]
//   backward (:211-220)  C_ch[b][a] = sum_{dj,di} R[b+sb-q+dj][a+sa-q+di] * wb_ch[dj][di]
//   D        (:123)      D_ch[b][a] = the same sum over the taps that land inside R
//   update   (:130-137)  X <- w*clean(X*C/D) + (1-w)*X, clamped at 0
//
// with sa = floor((alpha-u+h)/N), sb = floor((beta-v+h)/N).  One CTA owns one or more
// channel slots (two for the 67 x 67 lenslet patch, sharing one staged ratio image); each
// thread of a slot owns a 4 (b) x 8 (a) output tile.  Inputs are staged in shared memory
// with zero halos, so the tap loops need no bounds checks; the sliding windows are read
// with aligned 128-bit shared loads, each input row once per tile (conv_rows).  The X tile
// of a channel is copied with cp.async straight into the forward-input plane and updated
// there in place.  Each slot adds its channels' forward projections into its own partial
// plane in global memory (L2-resident, tile rows 32-byte aligned), in channel order; a
// second kernel reduces the planes in a fixed order.  Keeping those sums out of registers
// leaves each thread under 96 registers, so two CTAs of two slots (20 warps) fit an SM.
// A channel needs two CTA barriers: after the update (the forward projection reads the
// neighbouring tiles' updated X) and at its end (the next channel's X overwrites the
// plane).  The next channel's D table is built between them: its row sums read the taps
// from global memory while the back projection runs, its table after the first barrier.
#pragma once

#include <cuda_runtime.h>

#include "mlf_internal.h"

namespace mlf {

// Tile of conv_tile (8 b x 4 a), used by the allocation-free forward projection
// (mlf_noalloc.cu).
constexpr int VT_TY = 8;  // tile rows (b direction)
constexpr int VT_TX = 4;  // tile cols (a direction)

// acc[ty][tx] += sum_{dy<T, dx<T} in[(ty+dy)*pitch + OFF + tx + dx] * w[dy*WP+dx]
// `in` must be 16-byte aligned and pitch a multiple of 4.  Tap rows are WP floats apart;
// when WP is a multiple of 4 a row is read with 16-byte loads (the padding is not used).
// For a fixed output the products are added in the order dy, then dx.
template <int T, int OFF, int WP = T>
__device__ __forceinline__ void conv_tile(const float* __restrict__ in, int pitch,
                                          const float* __restrict__ w,
                                          float (&acc)[VT_TY][VT_TX]) {
  constexpr int NW = view_nw(T);
  static_assert(OFF + VT_TX + T - 1 <= 4 * NW, "window too short");
#pragma unroll 1
  for (int dy = 0; dy < T; ++dy) {
    float wr[T];
    if constexpr (WP % 4 == 0) {
      const float4* w4 = reinterpret_cast<const float4*>(w + dy * WP);
#pragma unroll
      for (int k = 0; k < (T + 3) / 4; ++k) {
        const float4 t4 = w4[k];
        wr[4 * k] = t4.x;
        if (4 * k + 1 < T) wr[4 * k + 1] = t4.y;
        if (4 * k + 2 < T) wr[4 * k + 2] = t4.z;
        if (4 * k + 3 < T) wr[4 * k + 3] = t4.w;
      }
    } else {
#pragma unroll
      for (int dx = 0; dx < T; ++dx) wr[dx] = w[dy * WP + dx];
    }
    const float* rowp = in + dy * pitch;
#pragma unroll
    for (int ty = 0; ty < VT_TY; ++ty) {
      float win[4 * NW];
      const float4* r4 = reinterpret_cast<const float4*>(rowp + ty * pitch);
#pragma unroll
      for (int k = 0; k < NW; ++k) {
        float4 t4 = r4[k];
        win[4 * k + 0] = t4.x;
        win[4 * k + 1] = t4.y;
        win[4 * k + 2] = t4.z;
        win[4 * k + 3] = t4.w;
      }
#pragma unroll
      for (int dx = 0; dx < T; ++dx)
#pragma unroll
        for (int tx = 0; tx < VT_TX; ++tx)
          acc[ty][tx] = fmaf(win[OFF + tx + dx], wr[dx], acc[ty][tx]);
    }
  }
}

// acc[ty][tx] += sum_{dy<T, dx<T} in[(ty+dy)*pitch + col(OFF + tx + dx)] * w[dy*WP+dx]
// for the 4 x 8 tile of the view kernel, on a plane whose columns are swizzled in 16-byte
// chunks: chunk k of this thread's window (columns a0 + 4k .. a0 + 4k + 3) starts at column
// view_pcol(a0 + 4k, pitch) of a row.  Walks the VW_TY + T - 1 input rows once: row r is loaded
// into registers once and serves every output row ty with a tap row dy = r - ty (tap rows
// come from shared memory as broadcast 16-byte loads), so the input window is read once
// per tile instead of once per tap row.  Per output the products are added in the order
// dy, then dx -- the order of conv_tile -- so the results are the same bit for bit.
// `in` 16-byte aligned, a0 and pitch multiples of 4, WP a multiple of 4.
template <int T, int OFF, int WP>
__device__ __forceinline__ void conv_rows(const float* __restrict__ in, int pitch, int a0,
                                          const float* __restrict__ w, float (&acc)[VW_TY][VW_TX]) {
  constexpr int NW = view_nw8(T);
  static_assert(OFF + VW_TX + T - 1 <= 4 * NW, "window too short");
  static_assert(WP % 4 == 0, "tap rows must be 16-byte aligned");
  int off[NW];
#pragma unroll
  for (int k = 0; k < NW; ++k) off[k] = view_pcol(a0 + 4 * k, pitch);
#pragma unroll 1
  for (int r = 0; r < VW_TY + T - 1; ++r) {
    float win[4 * NW];
    const float* row = in + r * pitch;
#pragma unroll
    for (int k = 0; k < NW; ++k) {
      const float4 t4 = *reinterpret_cast<const float4*>(row + off[k]);
      win[4 * k + 0] = t4.x;
      win[4 * k + 1] = t4.y;
      win[4 * k + 2] = t4.z;
      win[4 * k + 3] = t4.w;
    }
#pragma unroll
    for (int ty = 0; ty < VW_TY; ++ty) {
      const int dy = r - ty;
      if (dy < 0 || dy >= T) continue;
      float wr[T];
      const float4* w4 = reinterpret_cast<const float4*>(w + dy * WP);
#pragma unroll
      for (int k = 0; k < (T + 3) / 4; ++k) {
        const float4 t4 = w4[k];
        wr[4 * k] = t4.x;
        if (4 * k + 1 < T) wr[4 * k + 1] = t4.y;
        if (4 * k + 2 < T) wr[4 * k + 2] = t4.z;
        if (4 * k + 3 < T) wr[4 * k + 3] = t4.w;
      }
#pragma unroll
      for (int dx = 0; dx < T; ++dx)
#pragma unroll
        for (int tx = 0; tx < VW_TX; ++tx) acc[ty][tx] = fmaf(win[OFF + tx + dx], wr[dx], acc[ty][tx]);
    }
  }
}

__device__ __forceinline__ int floor_div(int a, int b) {
  int q = a / b;
  return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

__device__ __forceinline__ void cp_async16(float* smem, const float* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// D table of channel ch, in two steps separated by a CTA barrier (lt = thread within the
// slot, tps = threads per slot).  Row sums, read from the channel's taps in global memory:
//   rowp[dj][ca] = sum_{di in rngA[sa][ca]} wb[ch][dj][di]
// then the table:
//   dtab[cb][ca] = sum_{dj in rngB[sb][cb]} rowp[dj][ca]
// Both add in index order, so the values do not depend on the launch shape.
template <int T>
__device__ __forceinline__ void view_d_rows(const ViewArgs& A, int ch, int lt, float* rowp) {
  const int h = (A.N - 1) / 2;
  const int alpha = (int)((ch / A.Z) % A.N);
  const int sa = floor_div(alpha - A.u + h, A.N);
  const int* rA = A.rngA + (sa + 1) * A.maxc * 2;
  const float* w = A.wb + ch * (T * T);
  for (int i = lt; i < T * A.maxc; i += A.tps) {
    const int dj = i / A.maxc, ca = i - dj * A.maxc;
    const int lo = __ldg(rA + 2 * ca), hi = __ldg(rA + 2 * ca + 1);
    float v[T];  // the whole tap row in flight at once; the sum takes [lo, hi] in order
#pragma unroll
    for (int di = 0; di < T; ++di) v[di] = __ldg(w + dj * T + di);
    float s = 0.f;
#pragma unroll
    for (int di = 0; di < T; ++di)
      if (di >= lo && di <= hi) s += v[di];
    rowp[i] = s;
  }
}
template <int T>
__device__ __forceinline__ void view_d_table(const ViewArgs& A, int ch, int lt, const float* rowp,
                                             float* dtab) {
  const int h = (A.N - 1) / 2;
  const int beta = ch / (A.Z * A.N);
  const int sb = floor_div(beta - A.v + h, A.N);
  const int* rB = A.rngB + (sb + 1) * A.maxc * 2;
  for (int i = lt; i < A.maxc * A.maxc; i += A.tps) {
    const int cb = i / A.maxc, ca = i - cb * A.maxc;
    const int lo = __ldg(rB + 2 * cb), hi = __ldg(rB + 2 * cb + 1);
    float v[T];
#pragma unroll
    for (int dj = 0; dj < T; ++dj) v[dj] = rowp[dj * A.maxc + ca];
    float s = 0.f;
#pragma unroll
    for (int dj = 0; dj < T; ++dj)
      if (dj >= lo && dj <= hi) s += v[dj];
    dtab[i] = s;
  }
}

// At most kViewMaxThreads threads and two CTAs per SM: 96 registers per thread.
template <int T, int MODE>
__global__ void __launch_bounds__(kViewMaxThreads, 2) k_view(ViewArgs A) {
  extern __shared__ __align__(16) float sm[];
  constexpr int TT = T * T;
  constexpr int TW = view_tap_pitch(T);  // tap-row pitch in shared memory
  constexpr int TTW = T * TW;
  constexpr int Q = (T - 1) / 2;
  constexpr int QP = view_qpad(Q);      // column of the forward-input interior
  constexpr bool BWD = (MODE != MODE_FWD);
  constexpr bool XIN = (MODE != MODE_BWDC);
  const int tid = threadIdx.x;
  const int slot = tid / A.tstride;          // slots start at multiples of tstride >= tps
  const int lt = tid - slot * A.tstride;     // thread index within slot
  const bool slot_ok = slot < A.slots && lt < A.tps;
  // tile of this thread: with more than 8 tile columns, lanes 8k .. 8k+7 take columns 0..7
  // of one tile row (a 64-float span, so a warp's window loads spread over all banks) and
  // the remaining columns follow; fewer columns: row-major
  int ta, tb;
  if (A.tilesA > 8 && lt >= 8 * A.tilesB) {
    const int w2 = A.tilesA - 8, l2 = lt - 8 * A.tilesB;
    ta = 8 + l2 % w2;
    tb = l2 / w2;
  } else if (A.tilesA > 8) {
    ta = lt & 7;
    tb = lt >> 3;
  } else {
    ta = lt % A.tilesA;
    tb = lt / A.tilesA;
  }
  const int a0 = ta * VW_TX, b0 = tb * VW_TY;
  // swizzled columns of this tile's two X chunks in the forward-input plane
  const int xc0 = view_pcol(a0 + QP, A.XP), xc1 = view_pcol(a0 + QP + 4, A.XP);

  // ---- a cancelled solve: the rest of its view steps return at once (CTA-uniform)
  {
    __shared__ int s_stop;
    if (tid == 0) s_stop = cancel_entry(A.cancel);
    __syncthreads();
    if (s_stop) return;
  }

  // ---- shared memory carve-up
  float* rs = sm;                                              // [RProws][RP] (BWD only)
  float* slot_base = rs + (BWD ? A.RProws * A.RP : 0);
  float* xin = slot_base + (slot_ok ? slot : 0) * A.slot_floats;  // [XProws][XP]
  float* taps = xin + A.XProws * A.XP;                         // [2 buffers][wb | wf]
  float* dtab = taps + 4 * TTW;                                // [maxc][maxc]
  float* rowp = dtab + A.maxc * A.maxc;                        // [T][maxc]

  // ---- zero the slots (halos must be zero), stage R
  {
    const int total = A.slots * A.slot_floats;
    for (int i = tid; i < total; i += blockDim.x) slot_base[i] = 0.f;
    if (BWD) {
      const int nr = A.RProws * A.RP;
      const float4* src = reinterpret_cast<const float4*>(A.rpad);
      float4* dst = reinterpret_cast<float4*>(rs);
      for (int i = tid; i < nr / 4; i += blockDim.x) dst[i] = src[i];
    }
  }

  constexpr bool DT = (MODE == MODE_STEP);  // the update needs D
  const int h = (A.N - 1) / 2;
  // channel indices and tap offsets (nch * T * T) fit in 32 bits: checked by the solver
  const int nch = (int)A.nch;
  const int step = (int)gridDim.x * A.slots;
  const int first = (int)blockIdx.x * A.slots + slot;
  // this thread's tile in its slot's forward partial plane [tilesB*VW_TY][tilesA*VW_TX]
  // (tile rows 32-byte aligned); recomputed where used rather than held across the loop
  auto hx_tile = [&]() {
    const int HP = A.tilesA * VW_TX;
    return A.part + ((int64_t)blockIdx.x * A.slots + (slot_ok ? slot : 0)) * ((int64_t)A.tilesB * VW_TY * HP) +
           (int64_t)b0 * HP + a0;
  };
  bool hx_written = false;

  // taps of the first channel into buffer 0, its D row sums; the table after the barrier
  // (the row sums come from other threads)
  if (slot_ok && first < nch) {
    for (int i = lt; i < TT; i += A.tps) {
      const int j = (i / T) * TW + i % T;
      if (BWD) taps[j] = __ldg(A.wb + first * TT + i);
      if (XIN) taps[TTW + j] = __ldg(A.wf + first * TT + i);
    }
    if (DT) view_d_rows<T>(A, first, lt, rowp);
  }
  __syncthreads();
  if (DT && slot_ok && first < nch) view_d_table<T>(A, first, lt, rowp, dtab);
  __syncthreads();

  int buf = 0;
  for (int base = (int)blockIdx.x * A.slots; base < nch; base += step, buf ^= 1) {
    const int ch = base + slot;
    const int nxt = ch + step;
    const bool active = slot_ok && ch < nch;
    const bool more = slot_ok && nxt < nch;
    const int alpha = active ? (int)((ch / A.Z) % A.N) : 0;
    const int beta = active ? ch / (A.Z * A.N) : 0;
    const int sa = floor_div(alpha - A.u + h, A.N);
    const int sb = floor_div(beta - A.v + h, A.N);
    const float* wbs = taps + buf * 2 * TTW;
    const float* wfs = wbs + TTW;

    // ---- X tile -> forward-input plane (interior at rows +Q, cols +QP), asynchronously.
    // A plane row has Pa (a multiple of 4) floats: the second 16-byte half of the last tile
    // may lie past it and is then not copied (its shared-memory cells stay zero).
    if (XIN && active) {
      const float* Xch = A.X + ch * A.plane;
#pragma unroll
      for (int y = 0; y < VW_TY; ++y) {
        const int b = b0 + y;
        if (b >= A.Lj) continue;
        cp_async16(xin + (b + Q) * A.XP + xc0, Xch + (int64_t)b * A.Pa + a0);
        if (a0 + 4 < A.Pa) cp_async16(xin + (b + Q) * A.XP + xc1, Xch + (int64_t)b * A.Pa + a0 + 4);
      }
    }

    // One correlation call site for both phases (back projection of view k, forward
    // projection of view k+1), so that a single unrolled body per window offset is hot.
#pragma unroll 1
    for (int ph = 0; ph < 2; ++ph) {
      if (ph == 1 && !(XIN && (MODE == MODE_FWD || A.do_fwd))) break;
      if (active && ph == 0 && !BWD) {
        cp_async_wait_all();  // forward only: this thread's X tile has landed in xin
      } else if (active) {
        float acc[VW_TY][VW_TX];
#pragma unroll
        for (int y = 0; y < VW_TY; ++y)
#pragma unroll
          for (int x = 0; x < VW_TX; ++x) acc[y][x] = 0.f;
        if (ph == 1 && hx_written) {  // this tile's forward partials into L1 for the add below
          const float* hxp = hx_tile();
#pragma unroll
          for (int y = 0; y < VW_TY; ++y)
            asm volatile("prefetch.global.L1 [%0];" ::"l"(hxp + y * A.tilesA * VW_TX));
        }
        const float* in = ph == 0 ? rs + (b0 + sb + 1) * A.RP : xin + b0 * A.XP;
        const int pitch = ph == 0 ? A.RP : A.XP;
        const float* wsel = ph == 0 ? wbs : wfs;
        switch (ph == 0 ? sa + 1 : QP - Q) {
          case 0: conv_rows<T, 0, TW>(in, pitch, a0, wsel, acc); break;
          case 1: conv_rows<T, 1, TW>(in, pitch, a0, wsel, acc); break;
          case 2: conv_rows<T, 2, TW>(in, pitch, a0, wsel, acc); break;
          default:
            if constexpr (QP - Q == 3) conv_rows<T, 3, TW>(in, pitch, a0, wsel, acc);
            break;
        }
        if (ph == 0) {
          if (MODE == MODE_BWDC) {
#pragma unroll
            for (int y = 0; y < VW_TY; ++y) {
              const int b = b0 + y;
              if (b >= A.Lj) continue;
#pragma unroll
              for (int x = 0; x < VW_TX; ++x)
                if (a0 + x < A.Li) A.Cout[(int64_t)ch * A.plane + (int64_t)b * A.Pa + a0 + x] = acc[y][x];
            }
          } else {
            cp_async_wait_all();  // this thread's X tile has landed in xin
            const int* cA = A.clsA + (sa + 1) * A.Li;
            const int* cB = A.clsB + (sb + 1) * A.Lj;
            float* Xch = A.X + ch * A.plane;
#pragma unroll
            for (int y = 0; y < VW_TY; ++y) {
              const int b = b0 + y;
              if (b >= A.Lj) continue;
              const int cb = __ldg(cB + b);
              float* xrow = xin + (b + Q) * A.XP;
              const float4 x0 = *reinterpret_cast<const float4*>(xrow + xc0);
              const float4 x1 = *reinterpret_cast<const float4*>(xrow + xc1);
              const float xo8[VW_TX] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
              float xn8[VW_TX];
#pragma unroll
              for (int x = 0; x < VW_TX; ++x) {
                const int a = a0 + x;
                const float xo = xo8[x];
                xn8[x] = xo;  // columns past the patch keep their (zero) value
                if (a >= A.Li) continue;
                const float c = acc[y][x];
                const float d = dtab[cb * A.maxc + __ldg(cA + a)];
                float xc = xo * c / (d + A.d_eps);           // :130  X .* C ./ D
                if (!(xc >= 0.f) || isinf(xc)) xc = 0.f;     // :132-134 NaN, Inf, < 0
                float xn = __fmaf_rn(xc, A.w, __fmul_rn(1.f - A.w, xo));  // :136
                if (xn < 0.f) xn = 0.f;                      // :137
                xn8[x] = xn;
              }
              const float4 n0 = make_float4(xn8[0], xn8[1], xn8[2], xn8[3]);
              const float4 n1 = make_float4(xn8[4], xn8[5], xn8[6], xn8[7]);
              *reinterpret_cast<float4*>(xrow + xc0) = n0;
              *reinterpret_cast<float4*>(xrow + xc1) = n1;
              // the plane row has Pa (a multiple of 4) floats: its padding columns get back
              // their own values; a second half past the row is not written
              float4* g = reinterpret_cast<float4*>(Xch + (int64_t)b * A.Pa + a0);
              g[0] = n0;
              if (a0 + 4 < A.Pa) g[1] = n1;
            }
          }
        } else {
          // forward partials: plane += this channel's projection (tile rows are 32 bytes)
          float* hxp = hx_tile();
          const int HP = A.tilesA * VW_TX;
#pragma unroll
          for (int y = 0; y < VW_TY; ++y) {
            float4* p4 = reinterpret_cast<float4*>(hxp + y * HP);
            float4 lo = make_float4(acc[y][0], acc[y][1], acc[y][2], acc[y][3]);
            float4 hi = make_float4(acc[y][4], acc[y][5], acc[y][6], acc[y][7]);
            if (hx_written) {
              const float4 o0 = p4[0], o1 = p4[1];
              lo.x = o0.x + lo.x; lo.y = o0.y + lo.y; lo.z = o0.z + lo.z; lo.w = o0.w + lo.w;
              hi.x = o1.x + hi.x; hi.y = o1.y + hi.y; hi.z = o1.z + hi.z; hi.w = o1.w + hi.w;
            }
            p4[0] = lo;
            p4[1] = hi;
          }
          hx_written = true;
        }
      }
      if (ph == 0) {
        // the next channel's D row sums (global taps) while other warps still correlate;
        // the table below reads them after the barrier, once dtab has been read
        if (DT && more) view_d_rows<T>(A, nxt, lt, rowp);
        __syncthreads();
      }
    }
    // the next channel: its D table and its taps (into the other buffer)
    if (more) {
      if (DT) view_d_table<T>(A, nxt, lt, rowp, dtab);
      float* nb = taps + (buf ^ 1) * 2 * TTW;
      for (int i = lt; i < TT; i += A.tps) {
        const int j = (i / T) * TW + i % T;
        if (BWD) nb[j] = __ldg(A.wb + nxt * TT + i);
        if (XIN) nb[TTW + j] = __ldg(A.wf + nxt * TT + i);
      }
    }
    __syncthreads();
  }

  // a slot that projected no channel still owes the reduction a zero plane
  if ((MODE == MODE_FWD || (MODE == MODE_STEP && A.do_fwd)) && slot_ok && !hx_written) {
    float* hxp = hx_tile();
    const int HP = A.tilesA * VW_TX;
#pragma unroll
    for (int y = 0; y < VW_TY; ++y) {
      float4* p4 = reinterpret_cast<float4*>(hxp + y * HP);
      p4[0] = make_float4(0.f, 0.f, 0.f, 0.f);
      p4[1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

#define MLF_INSTANTIATE_VIEW(T)                                                                  \
  int prepare_view_T##T(size_t smem) {                                                          \
    (void)smem;                                                                                 \
    MLF_TRY(allow_max_dyn_smem((const void*)k_view<T, MODE_FWD>));                              \
    MLF_TRY(allow_max_dyn_smem((const void*)k_view<T, MODE_STEP>));                             \
    return allow_max_dyn_smem((const void*)k_view<T, MODE_BWDC>);                               \
  }                                                                                             \
  int occupancy_view_T##T(int threads, size_t smem, int* blocks) {                              \
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_view<T, MODE_STEP>, \
                                                                  threads, smem);               \
    if (e != cudaSuccess)                                                                       \
      return fail(MLF_ERR_CUDA, std::string("occupancy: ") + cudaGetErrorString(e));            \
    return MLF_OK;                                                                              \
  }                                                                                             \
  int launch_view_T##T(int mode, const ViewArgs& a, int grid, int threads, size_t smem,         \
                       cudaStream_t st) {                                                       \
    switch (mode) {                                                                             \
      case MODE_FWD: k_view<T, MODE_FWD><<<grid, threads, smem, st>>>(a); break;                \
      case MODE_STEP: k_view<T, MODE_STEP><<<grid, threads, smem, st>>>(a); break;              \
      default: k_view<T, MODE_BWDC><<<grid, threads, smem, st>>>(a); break;                     \
    }                                                                                           \
    cudaError_t e = cudaGetLastError();                                                         \
    if (e != cudaSuccess)                                                                       \
      return fail(MLF_ERR_CUDA, std::string("view kernel launch: ") + cudaGetErrorString(e));   \
    return MLF_OK;                                                                              \
  }

}  // namespace mlf
