// Gaussian AO integrals over contracted Cartesian shells, FP64 on the GB300.
//
// One-electron integrals (overlap, kinetic, dipole, nabla, angular momentum):
// one thread per Cartesian function pair, one-dimensional Obara-Saika overlap
// tables per primitive pair combined per component, the formulas of
// apyib/integrals.py:90-141 with its sign conventions (:143-146).
// Nuclear attraction and electron repulsion: McMurchie-Davidson Hermite
// expansion (McMurchie and Davidson, J. Comput. Phys. 26, 218 (1978)): per
// primitive pair the Hermite coefficients E_t of x_A^i x_B^j, per primitive
// quartet the Hermite integrals R_tuv from the Boys function by the downward
// recursion in n, then
//   (ab|cd) = 2 pi^(5/2) / (p q sqrt(p+q)) sum E^ab_tuv (-1)^(t'+u'+v') E^cd_t'u'v' R_(t+t')(u+u')(v+v').
// ERIs: one thread per unique quartet (mn|ls) with m>=n, l>=s, (mn)>=(ls),
// written to the eight symmetric positions.  These are set-up integrals
// (once per geometry, not per iteration), so the kernels are simple and exact
// rather than tuned.
#include <math.h>

#include "common.cuh"
#include "gauss.cuh"

namespace {

using namespace agbg;

template <int LM>
__global__ void oei_kernel(agb_basis b, int kind, double Ox, double Oy, double Oz, double* __restrict__ out) {
  constexpr int EM = emax(LM), LT = 2 * LM;
  const int n = b.ncart;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * n) return;
  const int mu = (int)(idx / n), nu = (int)(idx % n);
  const Fn fa = load_fn(b, mu), fb = load_fn(b, nu);
  const int pa[3] = {fa.x, fa.y, fa.z}, pb[3] = {fb.x, fb.y, fb.z};
  const double O[3] = {Ox, Oy, Oz};
  double acc[3] = {0.0, 0.0, 0.0};
  double S[3][EM][EM];
  double Ea[EM], Eb[EM], Ec[EM];
  double R[rsize(LT)], W[rsize(LT)];
  for (int i = 0; i < fa.np; ++i) {
    const double a = b.exps[fa.p0 + i], ca = b.coefs[fa.p0 + i];
    for (int j = 0; j < fb.np; ++j) {
      const double bb = b.exps[fb.p0 + j], cc = ca * b.coefs[fb.p0 + j];
      if (kind == AGB_OEI_POTENTIAL) {
        const double p = a + bb;
        hermite_e(pa[0], pb[0], a, bb, fa.A[0] - fb.A[0], Ea);
        hermite_e(pa[1], pb[1], a, bb, fa.A[1] - fb.A[1], Eb);
        hermite_e(pa[2], pb[2], a, bb, fa.A[2] - fb.A[2], Ec);
        double P[3];
        for (int k = 0; k < 3; ++k) P[k] = (a * fa.A[k] + bb * fb.A[k]) / p;
        const int L = fa.l + fb.l;
        for (int at = 0; at < b.natom; ++at) {
          hermite_r<LT>(L, p, P[0] - b.atom_xyz[3 * at], P[1] - b.atom_xyz[3 * at + 1], P[2] - b.atom_xyz[3 * at + 2],
                    R, W);
          double s = 0.0;
          for (int t = 0; t <= pa[0] + pb[0]; ++t)
            for (int u = 0; u <= pa[1] + pb[1]; ++u)
              for (int v = 0; v <= pa[2] + pb[2]; ++v) s += Ea[t] * Eb[u] * Ec[v] * R[ridx(t, u, v)];
          acc[0] -= b.atom_charge[at] * 2.0 * kPi / p * cc * s;
        }
        continue;
      }
      for (int k = 0; k < 3; ++k) os_table<EM>(pa[k] + 1, pb[k] + 2, a, bb, fa.A[k], fb.A[k], S[k]);
      auto s1 = [&](int k, int i1, int j1) { return (i1 >= 0 && j1 >= 0) ? S[k][i1][j1] : 0.0; };
      auto mom = [&](int k) {  // <a| (x_k - O_k) |b>
        return s1(k, pa[k] + 1, pb[k]) + (fa.A[k] - O[k]) * s1(k, pa[k], pb[k]);
      };
      auto der = [&](int k) { return pb[k] * s1(k, pa[k], pb[k] - 1) - 2.0 * bb * s1(k, pa[k], pb[k] + 1); };
      auto lap = [&](int k) {
        return pb[k] * (pb[k] - 1) * s1(k, pa[k], pb[k] - 2) - 2.0 * bb * (2 * pb[k] + 1) * s1(k, pa[k], pb[k]) +
               4.0 * bb * bb * s1(k, pa[k], pb[k] + 2);
      };
      const double sx = s1(0, pa[0], pb[0]), sy = s1(1, pa[1], pb[1]), sz = s1(2, pa[2], pb[2]);
      const double ss[3] = {sx, sy, sz};
      switch (kind) {
        case AGB_OEI_OVERLAP: acc[0] += cc * sx * sy * sz; break;
        case AGB_OEI_KINETIC: acc[0] += -0.5 * cc * (lap(0) * sy * sz + sx * lap(1) * sz + sx * sy * lap(2)); break;
        case AGB_OEI_DIPOLE:
          for (int k = 0; k < 3; ++k) acc[k] -= cc * mom(k) * ss[(k + 1) % 3] * ss[(k + 2) % 3];
          break;
        case AGB_OEI_NABLA:
          for (int k = 0; k < 3; ++k) acc[k] += cc * der(k) * ss[(k + 1) % 3] * ss[(k + 2) % 3];
          break;
        default:  // angular momentum: -(r - O) x nabla
          for (int k = 0; k < 3; ++k) {
            const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
            acc[k] -= cc * ss[k] * (mom(k1) * der(k2) - mom(k2) * der(k1));
          }
          break;
      }
    }
  }
  const int ncomp = (kind >= AGB_OEI_DIPOLE) ? 3 : 1;
  for (int k = 0; k < ncomp; ++k) out[(int64_t)k * n * n + idx] = acc[k];
}

// ------------------------------------------------------------- ERIs
__device__ __forceinline__ int64_t tri(int64_t k) {   // largest i with i(i+1)/2 <= k
  int64_t i = (int64_t)((sqrt(8.0 * (double)k + 1.0) - 1.0) * 0.5);
  while (i * (i + 1) / 2 > k) --i;
  while ((i + 1) * (i + 2) / 2 <= k) ++i;
  return i;
}

// One warp per unique Cartesian quartet; its lanes split the primitive quartets
// (contracted s shells of correlation-consistent bases have 9^4 of them, which a
// single thread would walk alone while the rest of the grid idles) and the partial
// sums meet in a fixed shuffle order, so the result is deterministic.
template <int LM>
__global__ void __launch_bounds__(128) eri_kernel(agb_basis b, int64_t nquart, double* __restrict__ out) {
  constexpr int EM = emax(LM), LT = 4 * LM;
  const double two_pi52 = 2.0 * kPi * kPi * sqrt(kPi);
  const int64_t n = b.ncart;
  const int lane = threadIdx.x & 31;
  for (int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nquart;
       q += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t ij = tri(q), kl = q - ij * (ij + 1) / 2;
    const int64_t i = tri(ij), j = ij - i * (i + 1) / 2;
    const int64_t k = tri(kl), l = kl - k * (k + 1) / 2;
    const Fn f1 = load_fn(b, (int)i), f2 = load_fn(b, (int)j), f3 = load_fn(b, (int)k), f4 = load_fn(b, (int)l);
    const int L = f1.l + f2.l + f3.l + f4.l;
    double E1[3][EM], E2[3][EM];
    double R[rsize(LT)], W[rsize(LT)];
    const int p1[3] = {f1.x, f1.y, f1.z}, p2[3] = {f2.x, f2.y, f2.z};
    const int p3[3] = {f3.x, f3.y, f3.z}, p4[3] = {f4.x, f4.y, f4.z};
    int m1[3], m2[3];
    for (int c = 0; c < 3; ++c) {
      m1[c] = p1[c] + p2[c];
      m2[c] = p3[c] + p4[c];
    }
    double acc = 0.0;
    const int nprim = f1.np * f2.np * f3.np * f4.np;
    for (int pq = lane; pq < nprim; pq += 32) {
      int r = pq;
      const int i4 = r % f4.np;
      r /= f4.np;
      const int i3 = r % f3.np;
      r /= f3.np;
      const int i2 = r % f2.np, i1 = r / f2.np;
      {
        const double a = b.exps[f1.p0 + i1], ca = b.coefs[f1.p0 + i1];
        const double bb = b.exps[f2.p0 + i2], cab = ca * b.coefs[f2.p0 + i2];
        const double p = a + bb;
        double P[3];
        for (int c = 0; c < 3; ++c) {
          P[c] = (a * f1.A[c] + bb * f2.A[c]) / p;
          hermite_e(p1[c], p2[c], a, bb, f1.A[c] - f2.A[c], E1[c]);
        }
        {
          const double cx = b.exps[f3.p0 + i3], cc = cab * b.coefs[f3.p0 + i3];
          {
            const double d = b.exps[f4.p0 + i4], cabcd = cc * b.coefs[f4.p0 + i4];
            const double qq = cx + d;
            double Q[3];
            for (int c = 0; c < 3; ++c) {
              Q[c] = (cx * f3.A[c] + d * f4.A[c]) / qq;
              hermite_e(p3[c], p4[c], cx, d, f3.A[c] - f4.A[c], E2[c]);
            }
            const double alpha = p * qq / (p + qq);
            hermite_r<LT>(L, alpha, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], R, W);
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
            acc += cabcd * two_pi52 / (p * qq * sqrt(p + qq)) * s;
          }
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane != 0) continue;
    const int64_t n2 = n * n, n3 = n2 * n;
    out[i * n3 + j * n2 + k * n + l] = acc;
    out[j * n3 + i * n2 + k * n + l] = acc;
    out[i * n3 + j * n2 + l * n + k] = acc;
    out[j * n3 + i * n2 + l * n + k] = acc;
    out[k * n3 + l * n2 + i * n + j] = acc;
    out[l * n3 + k * n2 + i * n + j] = acc;
    out[k * n3 + l * n2 + j * n + i] = acc;
    out[l * n3 + k * n2 + j * n + i] = acc;
  }
}

constexpr int kMaxRow = 16;

__global__ void transform_axis_kernel(const double* __restrict__ in, int64_t pre, int nin, int64_t post, int nout,
                                      const int* __restrict__ cart0, const int* __restrict__ len,
                                      const double* __restrict__ coef, double* __restrict__ out) {
  const int64_t total = pre * nout * post;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t bpos = e % post;
    const int64_t rest = e / post;
    const int s = (int)(rest % nout);
    const int64_t a = rest / nout;
    const int c0 = cart0[s], nl = len[s];
    if (nl < 0 || nl > kMaxRow || c0 < 0 || c0 + nl > nin) {   // malformed row: no access, NaN out
      out[e] = __longlong_as_double(0x7ff8000000000000LL);
      continue;
    }
    double acc = 0.0;
    for (int k = 0; k < nl; ++k) acc += coef[s * kMaxRow + k] * in[(a * nin + c0 + k) * post + bpos];
    out[e] = acc;
  }
}

agb_status check_basis(const agb_basis* b) {
  AGB_ARG_CHECK(b != nullptr, "basis is NULL");
  AGB_ARG_CHECK(b->natom > 0 && b->nshell > 0 && b->ncart > 0, "empty basis");
  AGB_ARG_CHECK(b->lmax >= 0 && b->lmax <= kLMax, "shell angular momentum above f (l = 3) is not supported");
  AGB_ARG_CHECK(b->atom_xyz && b->atom_charge && b->shell_l && b->shell_atom && b->shell_nprim && b->shell_prim0 &&
                    b->shell_cart0 && b->bf_shell && b->exps && b->coefs,
                "basis array is NULL");
  return AGB_OK;
}

}  // namespace

extern "C" agb_status agb_ao_one_electron(const agb_basis* basis, int kind, const double* origin, double* out,
                                          void* stream) {
  AGB_STATUS_TRY(check_basis(basis));
  AGB_ARG_CHECK(kind >= AGB_OEI_OVERLAP && kind <= AGB_OEI_ANGMOM, "unknown one-electron integral kind");
  AGB_ARG_CHECK(out != nullptr, "out is NULL");
  const double O[3] = {origin ? origin[0] : 0.0, origin ? origin[1] : 0.0, origin ? origin[2] : 0.0};
  const int64_t n2 = (int64_t)basis->ncart * basis->ncart;
  const int threads = 128;
  const unsigned grid = (unsigned)((n2 + threads - 1) / threads);
  cudaStream_t st = (cudaStream_t)stream;
  if (basis->lmax <= 1)
    oei_kernel<1><<<grid, threads, 0, st>>>(*basis, kind, O[0], O[1], O[2], out);
  else if (basis->lmax == 2)
    oei_kernel<2><<<grid, threads, 0, st>>>(*basis, kind, O[0], O[1], O[2], out);
  else
    oei_kernel<3><<<grid, threads, 0, st>>>(*basis, kind, O[0], O[1], O[2], out);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

extern "C" agb_status agb_ao_eri(const agb_basis* basis, double* out, void* stream) {
  AGB_STATUS_TRY(check_basis(basis));
  AGB_ARG_CHECK(out != nullptr, "out is NULL");
  const int64_t n = basis->ncart;
  const int64_t npair = n * (n + 1) / 2;
  const int64_t nquart = npair * (npair + 1) / 2;
  const int threads = 128;
  const int grid = agb::grid_for(nquart * 32, threads, 152LL * 16);
  cudaStream_t st = (cudaStream_t)stream;
  if (basis->lmax <= 1)
    eri_kernel<1><<<grid, threads, 0, st>>>(*basis, nquart, out);
  else if (basis->lmax == 2)
    eri_kernel<2><<<grid, threads, 0, st>>>(*basis, nquart, out);
  else
    eri_kernel<3><<<grid, threads, 0, st>>>(*basis, nquart, out);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

extern "C" agb_status agb_ao_transform_axis(const double* in, int64_t pre, int nin, int64_t post, int nout,
                                            const int* cart0, const int* len, const double* coef, double* out,
                                            void* stream) {
  AGB_ARG_CHECK(in && out && cart0 && len && coef, "NULL argument");
  AGB_ARG_CHECK(pre >= 1 && post >= 1 && nin >= 1 && nout >= 1, "bad shape");
  const int64_t total = pre * nout * post;
  const int threads = 256;
  transform_axis_kernel<<<agb::grid_for(total, threads), threads, 0, (cudaStream_t)stream>>>(in, pre, nin, post, nout,
                                                                                             cart0, len, coef, out);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}
