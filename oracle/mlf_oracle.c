/*
 * mlf_oracle.c -- C/OpenMP restatement (FP64) of one view of the reference's phase-space
 * RL loop, used ONLY as test infrastructure and as the timed CPU baseline (never by the
 * product library).  Same formulation as oracle/mesolf_ref.py:
 *
 *   forward   recon_theory_phase_space_LFM_with_filter.m:243-249 (CPU twin :191-198)
 *             HX = (sum_z conv2(X_z, h_z, 'same'))((N+1)/2:N:end, (N+1)/2:N:end),
 *             evaluated only at the sampled outputs, each by a direct dot product;
 *   backward  :211-220 (CPU twin :201-208): C_z = conv2(B, t_z, 'same') with B non-zero
 *             only on the lattice (u + N i, v + N j), evaluated as a scatter of kernel copies;
 *   update    :116-117 ratio, :123 D = bwd(ones), :130-137 update / blend / clamps.
 *
 * Arrays are MATLAB column-major: X(r, c, z) at X[r + Xr*(c + Xc*z)], h(p, q, z) at
 * h[p + S*(q + S*z)].  u, v are 0-based.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int mlf_oracle_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* HX(i, j), i < Li = Xr/N, j < Lj = Xc/N. */
void mlf_oracle_forward(const double* h, int64_t S, const double* X, int64_t Xr, int64_t Xc, int64_t Z,
                        int64_t N, double* HX) {
  const int64_t Li = Xr / N, Lj = Xc / N, m = S / 2, c0 = (N - 1) / 2;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t j = 0; j < Lj; ++j)
    for (int64_t i = 0; i < Li; ++i) {
      const int64_t r = c0 + N * i, c = c0 + N * j;
      double s = 0.0;
      for (int64_t z = 0; z < Z; ++z) {
        const double* hz = h + S * S * z;
        const double* Xz = X + Xr * Xc * z;
        /* conv2 'same': P(r, c) = sum_{k,l} X(k, l) h(r - k + m, c - l + m) */
        for (int64_t q = 0; q < S; ++q) {
          const int64_t l = c - q + m;
          if (l < 0 || l >= Xc) continue;
          const double* hq = hz + S * q;
          const double* Xl = Xz + Xr * l;
          int64_t plo = r + m - (Xr - 1), phi = r + m;
          if (plo < 0) plo = 0;
          if (phi > S - 1) phi = S - 1;
          for (int64_t p = plo; p <= phi; ++p) s += Xl[r - p + m] * hq[p];
        }
      }
      HX[i + Li * j] = s;
    }
}

/* C(r, c, z) = sum_{i,j} R(i, j) t(r - (u + N i) + m, c - (v + N j) + m, z). */
void mlf_oracle_backward(const double* t, int64_t S, const double* R, int64_t Li, int64_t Lj, int64_t u,
                         int64_t v, int64_t N, int64_t Z, double* C) {
  const int64_t Xr = Li * N, Xc = Lj * N, m = S / 2;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t z = 0; z < Z; ++z) {
    double* Cz = C + Xr * Xc * z;
    const double* tz = t + S * S * z;
    memset(Cz, 0, sizeof(double) * Xr * Xc);
    for (int64_t j = 0; j < Lj; ++j)
      for (int64_t i = 0; i < Li; ++i) {
        const double val = R[i + Li * j];
        if (val == 0.0) continue;
        const int64_t r0 = u + N * i - m, cc0 = v + N * j - m; /* output (r, c) uses t(r - r0, c - cc0) */
        for (int64_t q = 0; q < S; ++q) {
          const int64_t c = cc0 + q;
          if (c < 0 || c >= Xc) continue;
          double* Cc = Cz + Xr * c;
          const double* tq = tz + S * q;
          for (int64_t p = 0; p < S; ++p) {
            const int64_t r = r0 + p;
            if (r >= 0 && r < Xr) Cc[r] += val * tq[p];
          }
        }
      }
  }
}

/* One view of the RL loop, X updated in place; scratch: 2 volumes + 2 lenslet images. */
int mlf_oracle_view_step(const double* h, const double* t, int64_t S, const double* LF, double* X, int64_t Xr,
                         int64_t Xc, int64_t Z, int64_t N, int64_t u, int64_t v, double w) {
  const int64_t Li = Xr / N, Lj = Xc / N, nv = Xr * Xc * Z;
  double* HX = (double*)malloc(sizeof(double) * Li * Lj);
  double* ones = (double*)malloc(sizeof(double) * Li * Lj);
  double* C = (double*)malloc(sizeof(double) * nv);
  double* D = (double*)malloc(sizeof(double) * nv);
  if (!HX || !ones || !C || !D) {
    free(HX); free(ones); free(C); free(D);
    return 1;
  }
  mlf_oracle_forward(h, S, X, Xr, Xc, Z, N, HX);
  for (int64_t j = 0; j < Lj; ++j)
    for (int64_t i = 0; i < Li; ++i) {
      double r = LF[(u + N * i) + Xr * (v + N * j)] / HX[i + Li * j];
      HX[i + Li * j] = isfinite(r) ? r : 0.0;
      ones[i + Li * j] = 1.0;
    }
  mlf_oracle_backward(t, S, HX, Li, Lj, u, v, N, Z, C);
  mlf_oracle_backward(t, S, ones, Li, Lj, u, v, N, Z, D);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < nv; ++k) {
    double xc = X[k] * C[k] / D[k];
    if (isnan(xc) || isinf(xc) || xc < 0) xc = 0.0;
    double xn = xc * w + (1.0 - w) * X[k];
    X[k] = xn < 0 ? 0.0 : xn;
  }
  free(HX); free(ones); free(C); free(D);
  return 0;
}
