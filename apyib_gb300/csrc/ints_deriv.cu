// Nuclear first derivatives of the AO integrals, FP64 (psi4's ao_oei_deriv1 /
// ao_tei_deriv1 / ao_overlap_half_deriv1, which apyib/analytic_aats.py:96-104 and
// apyib/analytic_apts.py read through MintsHelper).
//
// The derivative of a primitive Cartesian Gaussian with respect to its centre,
//   d/dA_x [x_A^i e^(-a r_A^2)] = 2a x_A^(i+1) e^(-a r_A^2) - i x_A^(i-1) e^(-a r_A^2),
// turns every derivative integral into two integrals with shifted powers, which
// the same Obara-Saika tables and McMurchie-Davidson Hermite expansions evaluate
// (the Hermite integrals to one order more).  Nuclear attraction also moves with
// its nucleus: each term -Z_C <a|1/r_C|b> is translation invariant, so its
// derivative with respect to C is minus the sum of those with respect to the two
// basis-function centres.  Outputs: out[atom][x,y,z][ncart][ncart] and
// out[atom][x,y,z][ncart^4] over Cartesian functions, zeroed by the call.
#include "common.cuh"
#include "gauss.cuh"

namespace {

using namespace agbg;

template <int EM>
__device__ __forceinline__ double s1(const double S[3][EM][EM], int k, int i, int j) {
  return (i >= 0 && j >= 0) ? S[k][i][j] : 0.0;
}

// Overlap, kinetic or dipole (-(r - 0), three components) integrals of the primitive
// pair for powers pa, pb (the tables hold the pair's one-dimensional overlaps; bexp
// is the ket exponent, A the bra centre).  Returns the number of components.
template <int EM>
__device__ int oei_value(int kind, const int pa[3], const int pb[3], double bexp, const double A[3],
                         const double S[3][EM][EM], double out[3]) {
  const double ss[3] = {s1<EM>(S, 0, pa[0], pb[0]), s1<EM>(S, 1, pa[1], pb[1]), s1<EM>(S, 2, pa[2], pb[2])};
  if (kind == AGB_OEI_DIPOLE) {
    for (int k = 0; k < 3; ++k) {
      const double mom = s1<EM>(S, k, pa[k] + 1, pb[k]) + A[k] * ss[k];
      out[k] = -mom * ss[(k + 1) % 3] * ss[(k + 2) % 3];
    }
    return 3;
  }
  if (kind != AGB_OEI_KINETIC) {
    out[0] = ss[0] * ss[1] * ss[2];
    return 1;
  }
  double lap[3];
  for (int k = 0; k < 3; ++k)
    lap[k] = pb[k] * (pb[k] - 1) * s1<EM>(S, k, pa[k], pb[k] - 2) -
             2.0 * bexp * (2 * pb[k] + 1) * s1<EM>(S, k, pa[k], pb[k]) +
             4.0 * bexp * bexp * s1<EM>(S, k, pa[k], pb[k] + 2);
  out[0] = -0.5 * (lap[0] * ss[1] * ss[2] + ss[0] * lap[1] * ss[2] + ss[0] * ss[1] * lap[2]);
  return 1;
}

__device__ __forceinline__ double herm_sum(const double* Ex, const double* Ey, const double* Ez, int nx, int ny,
                                           int nz, const double* R) {
  double s = 0.0;
  for (int t = 0; t <= nx; ++t)
    for (int u = 0; u <= ny; ++u)
      for (int v = 0; v <= nz; ++v) s += Ex[t] * Ey[u] * Ez[v] * R[ridx(t, u, v)];
  return s;
}

template <int LM>
__global__ void oei_deriv_kernel(agb_basis b, int kind, double* __restrict__ out) {
  constexpr int EM = emax(LM), LT = 2 * LM + 1;
  const int n = b.ncart;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * n) return;
  const int mu = (int)(idx / n), nu = (int)(idx % n);
  const Fn fa = load_fn(b, mu), fb = load_fn(b, nu);
  const int atA = b.shell_atom[b.bf_shell[mu]], atB = b.shell_atom[b.bf_shell[nu]];
  const int pa[3] = {fa.x, fa.y, fa.z}, pb[3] = {fb.x, fb.y, fb.z};
  const int64_t nn = (int64_t)n * n;
  const int ncomp = (kind == AGB_OEI_DIPOLE) ? 3 : 1;
  double dA[3][3] = {}, dB[3][3] = {};     // [direction][component]
  double S[3][EM][EM];
  double E0[3][EM], Ep[EM], Em[EM];
  double R[rsize(LT)], W[rsize(LT)];
  for (int i = 0; i < fa.np; ++i) {
    const double a = b.exps[fa.p0 + i], ca = b.coefs[fa.p0 + i];
    for (int j = 0; j < fb.np; ++j) {
      const double bb = b.exps[fb.p0 + j], cc = ca * b.coefs[fb.p0 + j];
      if (kind != AGB_OEI_POTENTIAL) {
        for (int k = 0; k < 3; ++k) os_table<EM>(pa[k] + 2, pb[k] + 3, a, bb, fa.A[k], fb.A[k], S[k]);
        for (int c = 0; c < 3; ++c) {
          double vp[3], vm[3] = {0.0, 0.0, 0.0};
          int q[3] = {pa[0], pa[1], pa[2]};
          q[c] += 1;
          oei_value<EM>(kind, q, pb, bb, fa.A, S, vp);
          if (pa[c] > 0) {
            q[c] -= 2;
            oei_value<EM>(kind, q, pb, bb, fa.A, S, vm);
          }
          for (int m = 0; m < ncomp; ++m) dA[c][m] += cc * (2.0 * a * vp[m] - pa[c] * vm[m]);
          if (kind == AGB_OEI_OVERLAP_HALF) continue;
          int r[3] = {pb[0], pb[1], pb[2]};
          r[c] += 1;
          oei_value<EM>(kind, pa, r, bb, fa.A, S, vp);
          vm[0] = vm[1] = vm[2] = 0.0;
          if (pb[c] > 0) {
            r[c] -= 2;
            oei_value<EM>(kind, pa, r, bb, fa.A, S, vm);
          }
          for (int m = 0; m < ncomp; ++m) dB[c][m] += cc * (2.0 * bb * vp[m] - pb[c] * vm[m]);
        }
        continue;
      }
      // nuclear attraction, McMurchie-Davidson with Hermite integrals to order L+1
      const double p = a + bb;
      double P[3];
      for (int k = 0; k < 3; ++k) {
        P[k] = (a * fa.A[k] + bb * fb.A[k]) / p;
        hermite_e(pa[k], pb[k], a, bb, fa.A[k] - fb.A[k], E0[k]);
      }
      const int L = fa.l + fb.l + 1;
      for (int at = 0; at < b.natom; ++at) {
        const double C[3] = {b.atom_xyz[3 * at], b.atom_xyz[3 * at + 1], b.atom_xyz[3 * at + 2]};
        hermite_r<LT>(L, p, P[0] - C[0], P[1] - C[1], P[2] - C[2], R, W);
        const double pref = -b.atom_charge[at] * 2.0 * kPi / p * cc;
        double vA[3], vB[3];
        for (int c = 0; c < 3; ++c) {
          const double* E[3] = {E0[0], E0[1], E0[2]};
          int ln[3] = {pa[0] + pb[0], pa[1] + pb[1], pa[2] + pb[2]};
          // centre A
          hermite_e(pa[c] + 1, pb[c], a, bb, fa.A[c] - fb.A[c], Ep);
          E[c] = Ep;
          ln[c] += 1;
          double v = 2.0 * a * herm_sum(E[0], E[1], E[2], ln[0], ln[1], ln[2], R);
          if (pa[c] > 0) {
            hermite_e(pa[c] - 1, pb[c], a, bb, fa.A[c] - fb.A[c], Em);
            E[c] = Em;
            ln[c] -= 2;
            v -= pa[c] * herm_sum(E[0], E[1], E[2], ln[0], ln[1], ln[2], R);
            ln[c] += 2;
          }
          vA[c] = v;
          // centre B
          ln[c] = pa[c] + pb[c] + 1;
          hermite_e(pa[c], pb[c] + 1, a, bb, fa.A[c] - fb.A[c], Ep);
          E[c] = Ep;
          v = 2.0 * bb * herm_sum(E[0], E[1], E[2], ln[0], ln[1], ln[2], R);
          if (pb[c] > 0) {
            hermite_e(pa[c], pb[c] - 1, a, bb, fa.A[c] - fb.A[c], Em);
            E[c] = Em;
            ln[c] -= 2;
            v -= pb[c] * herm_sum(E[0], E[1], E[2], ln[0], ln[1], ln[2], R);
          }
          vB[c] = v;
        }
        for (int c = 0; c < 3; ++c) {
          dA[c][0] += pref * vA[c];
          dB[c][0] += pref * vB[c];
          out[((int64_t)at * 3 + c) * nn + idx] -= pref * (vA[c] + vB[c]);
        }
      }
    }
  }
  for (int c = 0; c < 3; ++c)
    for (int m = 0; m < ncomp; ++m) {
      out[(((int64_t)atA * 3 + c) * ncomp + m) * nn + idx] += dA[c][m];
      if (kind != AGB_OEI_OVERLAP_HALF) out[(((int64_t)atB * 3 + c) * ncomp + m) * nn + idx] += dB[c][m];
    }
}

__device__ __forceinline__ int64_t tri(int64_t k) {
  int64_t i = (int64_t)((sqrt(8.0 * (double)k + 1.0) - 1.0) * 0.5);
  while (i * (i + 1) / 2 > k) --i;
  while ((i + 1) * (i + 2) / 2 <= k) ++i;
  return i;
}

// (ab|cd) for the bra Hermite vectors E1 (lengths m1) and ket vectors E2 (m2).
__device__ __forceinline__ double eri_sum(const double* const E1[3], const int m1[3], const double* const E2[3],
                                          const int m2[3], const double* R) {
  double s = 0.0;
  for (int t = 0; t <= m1[0]; ++t)
    for (int u = 0; u <= m1[1]; ++u)
      for (int v = 0; v <= m1[2]; ++v) {
        const double e1 = E1[0][t] * E1[1][u] * E1[2][v];
        double inner = 0.0;
        for (int t2 = 0; t2 <= m2[0]; ++t2)
          for (int u2 = 0; u2 <= m2[1]; ++u2)
            for (int v2 = 0; v2 <= m2[2]; ++v2) {
              const double e2 = E2[0][t2] * E2[1][u2] * E2[2][v2];
              const double r = R[ridx(t + t2, u + u2, v + v2)];
              inner += ((t2 + u2 + v2) & 1) ? -e2 * r : e2 * r;
            }
        s += e1 * inner;
      }
  return s;
}

// One warp per unique Cartesian quartet, its lanes splitting the primitive quartets
// (as the ERI kernel); the twelve derivative partials meet in a fixed shuffle order.
template <int LM>
__global__ void __launch_bounds__(128) eri_deriv_kernel(agb_basis b, int64_t nquart, double* __restrict__ out) {
  constexpr int EM = emax(LM), LT = 4 * LM + 1;
  const double two_pi52 = 2.0 * kPi * kPi * sqrt(kPi);
  const int64_t n = b.ncart, n4 = n * n * n * n;
  const int lane = threadIdx.x & 31;
  for (int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nquart;
       q += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t ij = tri(q), kl = q - ij * (ij + 1) / 2;
    const int64_t i = tri(ij), j = ij - i * (i + 1) / 2;
    const int64_t k = tri(kl), l = kl - k * (k + 1) / 2;
    const int64_t fidx[4] = {i, j, k, l};
    Fn f[4];
    int pw[4][3], at[4];
    for (int s = 0; s < 4; ++s) {
      f[s] = load_fn(b, (int)fidx[s]);
      pw[s][0] = f[s].x;
      pw[s][1] = f[s].y;
      pw[s][2] = f[s].z;
      at[s] = b.shell_atom[b.bf_shell[fidx[s]]];
    }
    const int L = f[0].l + f[1].l + f[2].l + f[3].l + 1;
    double d[4][3] = {};
    double E1[3][EM], E2[3][EM], Es[EM];
    double R[rsize(LT)], W[rsize(LT)];
    const int nprim = f[0].np * f[1].np * f[2].np * f[3].np;
    for (int pq = lane; pq < nprim; pq += 32) {
      int r = pq;
      const int i4 = r % f[3].np;
      r /= f[3].np;
      const int i3 = r % f[2].np;
      r /= f[2].np;
      const int i2 = r % f[1].np, i1 = r / f[1].np;
      const double e0 = b.exps[f[0].p0 + i1], c0 = b.coefs[f[0].p0 + i1];
      {
        const double e1 = b.exps[f[1].p0 + i2], c01 = c0 * b.coefs[f[1].p0 + i2];
        const double p = e0 + e1;
        double P[3];
        for (int c = 0; c < 3; ++c) {
          P[c] = (e0 * f[0].A[c] + e1 * f[1].A[c]) / p;
          hermite_e(pw[0][c], pw[1][c], e0, e1, f[0].A[c] - f[1].A[c], E1[c]);
        }
        {
          const double e2 = b.exps[f[2].p0 + i3], c012 = c01 * b.coefs[f[2].p0 + i3];
          {
            const double e3 = b.exps[f[3].p0 + i4], cc = c012 * b.coefs[f[3].p0 + i4];
            const double qq = e2 + e3;
            double Q[3];
            for (int c = 0; c < 3; ++c) {
              Q[c] = (e2 * f[2].A[c] + e3 * f[3].A[c]) / qq;
              hermite_e(pw[2][c], pw[3][c], e2, e3, f[2].A[c] - f[3].A[c], E2[c]);
            }
            hermite_r<LT>(L, p * qq / (p + qq), P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], R, W);
            const double pref = cc * two_pi52 / (p * qq * sqrt(p + qq));
            const double ex[4] = {e0, e1, e2, e3};
            for (int s = 0; s < 4; ++s) {
              const bool bra = s < 2;
              const int pairA = bra ? 0 : 2;       // first function of the pair holding s
              const double ea = ex[pairA], eb = ex[pairA + 1];
              for (int c = 0; c < 3; ++c) {
                const double* e1v[3] = {E1[0], E1[1], E1[2]};
                const double* e2v[3] = {E2[0], E2[1], E2[2]};
                int m1[3] = {pw[0][0] + pw[1][0], pw[0][1] + pw[1][1], pw[0][2] + pw[1][2]};
                int m2[3] = {pw[2][0] + pw[3][0], pw[2][1] + pw[3][1], pw[2][2] + pw[3][2]};
                const double XAB = f[pairA].A[c] - f[pairA + 1].A[c];
                const int ia = pw[pairA][c], ib = pw[pairA + 1][c];
                const bool first = (s == pairA);
                // +1 on function s
                hermite_e(first ? ia + 1 : ia, first ? ib : ib + 1, ea, eb, XAB, Es);
                if (bra) {
                  e1v[c] = Es;
                  m1[c] += 1;
                } else {
                  e2v[c] = Es;
                  m2[c] += 1;
                }
                double v = 2.0 * ex[s] * eri_sum(e1v, m1, e2v, m2, R);
                const int ps = pw[s][c];
                if (ps > 0) {
                  hermite_e(first ? ia - 1 : ia, first ? ib : ib - 1, ea, eb, XAB, Es);
                  if (bra)
                    m1[c] -= 2;
                  else
                    m2[c] -= 2;
                  v -= ps * eri_sum(e1v, m1, e2v, m2, R);
                }
                d[s][c] += pref * v;
              }
            }
          }
        }
      }
    }
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d[s][c] += __shfl_xor_sync(0xffffffffu, d[s][c], o);
    if (lane != 0) continue;
    const int64_t n2 = n * n, n3 = n2 * n;
    const int64_t pos[8] = {i * n3 + j * n2 + k * n + l, j * n3 + i * n2 + k * n + l, i * n3 + j * n2 + l * n + k,
                            j * n3 + i * n2 + l * n + k, k * n3 + l * n2 + i * n + j, l * n3 + k * n2 + i * n + j,
                            k * n3 + l * n2 + j * n + i, l * n3 + k * n2 + j * n + i};
    for (int s = 0; s < 4; ++s) {
      bool seen = false;
      for (int s2 = 0; s2 < s; ++s2) seen |= (at[s2] == at[s]);
      if (seen) continue;
      for (int c = 0; c < 3; ++c) {
        double v = 0.0;
        for (int s2 = s; s2 < 4; ++s2)
          if (at[s2] == at[s]) v += d[s2][c];
        double* o = out + ((int64_t)at[s] * 3 + c) * n4;
        for (int p8 = 0; p8 < 8; ++p8) o[pos[p8]] = v;
      }
    }
  }
}

}  // namespace

extern "C" agb_status agb_ao_one_electron_deriv(const agb_basis* basis, int kind, double* out, void* stream) {
  AGB_ARG_CHECK(basis != nullptr && out != nullptr, "NULL argument");
  AGB_ARG_CHECK(basis->lmax >= 0 && basis->lmax <= kLMax, "shell angular momentum above f (l = 3) is not supported");
  AGB_ARG_CHECK(kind == AGB_OEI_OVERLAP || kind == AGB_OEI_KINETIC || kind == AGB_OEI_POTENTIAL ||
                    kind == AGB_OEI_OVERLAP_HALF || kind == AGB_OEI_DIPOLE,
                "derivatives exist for overlap, kinetic, potential, dipole and the half-derivative overlap");
  const int64_t n2 = (int64_t)basis->ncart * basis->ncart;
  const int ncomp = (kind == AGB_OEI_DIPOLE) ? 3 : 1;
  cudaStream_t st = (cudaStream_t)stream;
  AGB_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * n2 * 3 * ncomp * basis->natom, st));
  const int threads = 128;
  const unsigned grid = (unsigned)((n2 + threads - 1) / threads);
  if (basis->lmax <= 1)
    oei_deriv_kernel<1><<<grid, threads, 0, st>>>(*basis, kind, out);
  else if (basis->lmax == 2)
    oei_deriv_kernel<2><<<grid, threads, 0, st>>>(*basis, kind, out);
  else
    oei_deriv_kernel<3><<<grid, threads, 0, st>>>(*basis, kind, out);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

extern "C" agb_status agb_ao_eri_deriv(const agb_basis* basis, double* out, void* stream) {
  AGB_ARG_CHECK(basis != nullptr && out != nullptr, "NULL argument");
  AGB_ARG_CHECK(basis->lmax >= 0 && basis->lmax <= kLMax, "shell angular momentum above f (l = 3) is not supported");
  const int64_t n = basis->ncart;
  const int64_t npair = n * (n + 1) / 2, nquart = npair * (npair + 1) / 2;
  cudaStream_t st = (cudaStream_t)stream;
  AGB_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * n * n * n * n * 3 * basis->natom, st));
  const int threads = 128;
  const int grid = agb::grid_for(nquart * 32, threads, 152LL * 16);
  if (basis->lmax <= 1)
    eri_deriv_kernel<1><<<grid, threads, 0, st>>>(*basis, nquart, out);
  else if (basis->lmax == 2)
    eri_deriv_kernel<2><<<grid, threads, 0, st>>>(*basis, nquart, out);
  else
    eri_deriv_kernel<3><<<grid, threads, 0, st>>>(*basis, nquart, out);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}
