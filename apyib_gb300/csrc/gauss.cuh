// Gaussian-integral building blocks shared by the AO integral kernels (ints.cu)
// and their nuclear-derivative kernels (ints_deriv.cu): the Boys function,
// McMurchie-Davidson Hermite coefficients and Hermite integrals, one-dimensional
// Obara-Saika overlap tables, and the description of one Cartesian function.
#pragma once
#include <math.h>

#include "common.cuh"

namespace agbg {

constexpr int kLMax = 3;                   // f shells
constexpr double kPi = 3.14159265358979323846;
// Per-thread table sizes for shells up to angular momentum LM (the kernels are
// instantiated for LM = 1, 2, 3 so that s/p and d bases keep small local arrays).
__host__ __device__ constexpr int rsize(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
__host__ __device__ constexpr int emax(int LM) { return 2 * LM + 3; }   // Hermite / OS extent (+2: kinetic)

__device__ __forceinline__ void cart_pow(int l, int k, int& x, int& y, int& z) {
  int i = 0;
  while ((i + 1) * (i + 2) / 2 <= k) ++i;
  const int j = k - i * (i + 1) / 2;
  x = l - i;
  y = i - j;
  z = j;
}

// Boys function F_n(T) = int_0^1 t^(2n) exp(-T t^2) dt, n = 0..nmax.
// T < 30: the series F_m = e^-T sum_k (2T)^k / ((2m+1)(2m+3)...(2m+2k+1)) for
// m = nmax (positive terms), then the downward recursion
// F_n = (2T F_(n+1) + e^-T) / (2n+1), which is stable.  T >= 30 (> nmax):
// F_0 = sqrt(pi/T)/2 erf(sqrt T) and the upward recursion
// F_(n+1) = ((2n+1) F_n - e^-T) / (2T), stable while 2n+1 < 2T.
__device__ inline void boys(int nmax, double T, double* F) {
  const double e = exp(-T);
  if (T < 30.0) {
    double term = 1.0 / (2 * nmax + 1), sum = term;
    for (int k = 1; k < 400; ++k) {
      term *= 2.0 * T / (2 * nmax + 2 * k + 1);
      sum += term;
      if (term < 1e-17 * sum) break;
    }
    F[nmax] = e * sum;
    for (int n = nmax - 1; n >= 0; --n) F[n] = (2.0 * T * F[n + 1] + e) / (2 * n + 1);
  } else {
    F[0] = 0.5 * sqrt(kPi / T) * erf(sqrt(T));
    for (int n = 0; n < nmax; ++n) F[n + 1] = ((2 * n + 1) * F[n] - e) / (2.0 * T);
  }
}

// Hermite coefficients E_t (t = 0..i+j) of x_A^i x_B^j e^(-a x_A^2 - b x_B^2)
// about P; XAB = A - B.  E^(i+1,j)_t = E^ij_(t-1)/(2p) + X_PA E^ij_t + (t+1) E^ij_(t+1),
// likewise for j with X_PB.
__device__ inline void hermite_e(int i, int j, double a, double b, double XAB, double* E) {
  const double p = a + b, h = 0.5 / p;
  const double XPA = -b * XAB / p, XPB = a * XAB / p;
  E[0] = exp(-a * b / p * XAB * XAB);
  int n = 0;
  for (int s = 0; s < i + j; ++s) {
    const double X = s < i ? XPA : XPB;
    double prev = 0.0;
    for (int t = 0; t <= n + 1; ++t) {
      const double cur = t <= n ? E[t] : 0.0;
      const double nxt = t + 1 <= n ? E[t + 1] : 0.0;
      E[t] = h * prev + X * cur + (t + 1) * nxt;
      prev = cur;
    }
    ++n;
  }
}

__device__ __forceinline__ int ridx(int t, int u, int v) {
  const int n = t + u + v, s = u + v;
  return n * (n + 1) * (n + 2) / 6 + s * (s + 1) / 2 + v;
}

// R_tuv = R^0_tuv for t+u+v <= L (<= LT) into R, with scratch W (rsize(LT) each):
// R^n_000 = (-2 alpha)^n F_n(alpha |PC|^2),
// R^n_(t+1)uv = t R^(n+1)_(t-1)uv + X R^(n+1)_tuv (and for u, v).
template <int LT>
__device__ void hermite_r(int L, double alpha, double X, double Y, double Z, double* R, double* W) {
  double F[LT + 1];
  boys(L, alpha * (X * X + Y * Y + Z * Z), F);
  double pw[LT + 1];
  pw[0] = 1.0;
  for (int n = 1; n <= L; ++n) pw[n] = pw[n - 1] * (-2.0 * alpha);
  for (int n = L; n >= 0; --n) {
    double* dst = (n & 1) ? W : R;
    const double* src = (n & 1) ? R : W;
    dst[0] = pw[n] * F[n];
    const int m = L - n;
    for (int s = 1; s <= m; ++s) {
      for (int t = s; t >= 0; --t) {
        for (int u = s - t; u >= 0; --u) {
          const int v = s - t - u;
          double val;
          if (t > 0) {
            val = X * src[ridx(t - 1, u, v)] + (t > 1 ? (t - 1) * src[ridx(t - 2, u, v)] : 0.0);
          } else if (u > 0) {
            val = Y * src[ridx(t, u - 1, v)] + (u > 1 ? (u - 1) * src[ridx(t, u - 2, v)] : 0.0);
          } else {
            val = Z * src[ridx(t, u, v - 1)] + (v > 1 ? (v - 1) * src[ridx(t, u, v - 2)] : 0.0);
          }
          dst[ridx(t, u, v)] = val;
        }
      }
    }
  }
}

struct Fn {          // one Cartesian function
  int l, x, y, z, p0, np;
  double A[3];
};

__device__ __forceinline__ Fn load_fn(const agb_basis& b, int mu) {
  Fn f;
  const int s = b.bf_shell[mu];
  f.l = b.shell_l[s];
  cart_pow(f.l, mu - b.shell_cart0[s], f.x, f.y, f.z);
  f.p0 = b.shell_prim0[s];
  f.np = b.shell_nprim[s];
  const int at = b.shell_atom[s];
  f.A[0] = b.atom_xyz[3 * at];
  f.A[1] = b.atom_xyz[3 * at + 1];
  f.A[2] = b.atom_xyz[3 * at + 2];
  return f;
}

// ------------------------------------------------------------- one-electron
// 1-D overlap table S[i][j], i <= ia, j <= jb (Obara-Saika):
// S_00 = sqrt(pi/p) exp(-mu X_AB^2); S_(i+1)j = X_PA S_ij + (i S_(i-1)j + j S_i(j-1)) / 2p;
// S_i(j+1) = X_PB S_ij + (i S_(i-1)j + j S_i(j-1)) / 2p.
template <int EM>
__device__ void os_table(int ia, int jb, double a, double b, double A, double B, double S[EM][EM]) {
  const double p = a + b, P = (a * A + b * B) / p, h = 0.5 / p;
  const double XPA = P - A, XPB = P - B, XAB = A - B;
  S[0][0] = sqrt(kPi / p) * exp(-a * b / p * XAB * XAB);
  for (int i = 0; i < ia; ++i) S[i + 1][0] = XPA * S[i][0] + (i > 0 ? i * S[i - 1][0] : 0.0) * h;
  for (int i = 0; i <= ia; ++i)
    for (int j = 0; j < jb; ++j)
      S[i][j + 1] = XPB * S[i][j] + ((i > 0 ? i * S[i - 1][j] : 0.0) + (j > 0 ? j * S[i][j - 1] : 0.0)) * h;
}

}  // namespace agbg
