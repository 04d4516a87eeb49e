// Batched small complex linear algebra in FP64 for the overlap-based AAT terms:
// many products of matrices a few tens wide (one per wavefunction overlap) and the
// determinant and inverse of each overlap's occupied block.
//
//   batched_zgemm_kernel  C_b = alpha op(A_b) op(B_b) + beta C_b, one 32x32 output tile
//                         per CTA and batch entry (blockIdx.z), general strides, a batch
//                         stride of 0 broadcasts an operand.
//   det_inv_kernel        Gauss-Jordan elimination with partial pivoting, in place in
//                         shared memory, one CTA per matrix: the inverse and the
//                         determinant (product of the pivots times the permutation sign).
#include "common.cuh"

namespace agb {
namespace {

constexpr int TB = 32, TK = 16;

struct BGemmArgs {
  int64_t M, N, K;
  z64 alpha, beta;
  const z64* A; int64_t sAm, sAk, sAb; int conjA;
  const z64* B; int64_t sBk, sBn, sBb; int conjB;
  z64* C; int64_t ldc, sCb;
  int64_t b0;         // first batch entry of this launch
};

__global__ void __launch_bounds__(256) batched_zgemm_kernel(BGemmArgs p) {
  __shared__ z64 As[TK][TB + 1];
  __shared__ z64 Bs[TK][TB + 1];
  const int64_t b = p.b0 + blockIdx.z;
  const z64* A = p.A + b * p.sAb;
  const z64* B = p.B + b * p.sBb;
  z64* C = p.C + b * p.sCb;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * TB, n0 = (int64_t)blockIdx.x * TB;
  z64 acc[2][2] = {{zmk(0, 0), zmk(0, 0)}, {zmk(0, 0), zmk(0, 0)}};
  for (int64_t k0 = 0; k0 < p.K; k0 += TK) {
    for (int idx = threadIdx.x; idx < TB * TK; idx += 256) {
      const int m = idx % TB, k = idx / TB;
      const int64_t gm = m0 + m, gk = k0 + k;
      z64 a = zmk(0, 0);
      if (gm < p.M && gk < p.K) {
        a = A[gm * p.sAm + gk * p.sAk];
        if (p.conjA) a.y = -a.y;
      }
      As[k][m] = a;
      const int64_t gn = n0 + m;
      z64 bv = zmk(0, 0);
      if (gn < p.N && gk < p.K) {
        bv = B[gk * p.sBk + gn * p.sBn];
        if (p.conjB) bv.y = -bv.y;
      }
      Bs[k][m] = bv;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      const z64 a0 = As[kk][ty], a1 = As[kk][ty + 16];
      const z64 c0 = Bs[kk][tx], c1 = Bs[kk][tx + 16];
      zfma(acc[0][0], a0, c0);
      zfma(acc[0][1], a0, c1);
      zfma(acc[1][0], a1, c0);
      zfma(acc[1][1], a1, c1);
    }
    __syncthreads();
  }
  const bool use_beta = p.beta.x != 0.0 || p.beta.y != 0.0;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int64_t gm = m0 + ty + 16 * i;
    if (gm >= p.M) continue;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int64_t gn = n0 + tx + 16 * j;
      if (gn >= p.N) continue;
      z64* c = C + gm * p.ldc + gn;
      z64 out = zmul(p.alpha, acc[i][j]);
      if (use_beta) out = zadd(out, zmul(p.beta, *c));
      *c = out;
    }
  }
}

// In-place Gauss-Jordan inversion with partial pivoting of one n x n matrix per CTA.
// Step k: pick the row of largest |a_ik| (i >= k), swap it into row k (sign flip of the
// determinant), scale row k by 1 / pivot (the pivot's slot receives 1 / pivot), and
// subtract multiples of row k from every other row (their column-k slots receive
// -f / pivot).  After the last step the array holds (P A)^-1; undoing the row swaps as
// column swaps in reverse order gives A^-1.  An exactly zero pivot marks the matrix
// singular (info = step + 1) and leaves its outputs unspecified.
__global__ void __launch_bounds__(256) det_inv_kernel(int n, const z64* __restrict__ A, int64_t lda, int64_t sAb,
                                                      z64* __restrict__ Ainv, int64_t ldi, int64_t sIb,
                                                      z64* __restrict__ det, int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  z64* a = (z64*)smem_raw;                        // n x n, row stride n
  int* perm = (int*)(a + (size_t)n * n);
  __shared__ z64 s_det;
  __shared__ int s_piv, s_bad;
  const int64_t b = blockIdx.x;
  const z64* src = A + b * sAb;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) a[e] = src[(int64_t)(e / n) * lda + (e % n)];
  if (threadIdx.x == 0) {
    s_det = zmk(1, 0);
    s_bad = 0;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x < 32) {
      // warp 0: the pivot row (largest |a_ik|^2, first on ties)
      double best = -1.0;
      int bi = k;
      for (int i = k + (int)threadIdx.x; i < n; i += 32) {
        const z64 v = a[i * n + k];
        const double m2 = v.x * v.x + v.y * v.y;
        if (m2 > best) { best = m2; bi = i; }
      }
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (threadIdx.x == 0) {
        s_piv = bi;
        perm[k] = bi;
        if (best == 0.0 && !s_bad) s_bad = k + 1;
      }
    }
    __syncthreads();
    const int p = s_piv;
    if (p != k)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const z64 t = a[k * n + j];
        a[k * n + j] = a[p * n + j];
        a[p * n + j] = t;
      }
    __syncthreads();
    const z64 piv = a[k * n + k];
    const double pm = piv.x * piv.x + piv.y * piv.y;
    const z64 pinv = pm > 0.0 ? zmk(piv.x / pm, -piv.y / pm) : zmk(0, 0);
    if (threadIdx.x == 0) s_det = (p != k) ? zneg(zmul(s_det, piv)) : zmul(s_det, piv);
    __syncthreads();                                  // every thread has read the pivot
    for (int j = threadIdx.x; j < n; j += blockDim.x) a[k * n + j] = (j == k) ? pinv : zmul(a[k * n + j], pinv);
    __syncthreads();
    // rows i != k: a_ij -= a_ik a_kj (j != k), a_ik = -a_ik / pivot
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e / n, j = e % n;
      if (i == k || j == k) continue;
      const z64 f = a[i * n + k];
      const z64 r = a[k * n + j];
      a[i * n + j] = zsub(a[i * n + j], zmul(f, r));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      if (i != k) a[i * n + k] = zneg(zmul(a[i * n + k], pinv));
    __syncthreads();
  }
  // undo the row interchanges as column interchanges, last first (one thread per row)
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    for (int k = n - 1; k >= 0; --k) {
      const int p = perm[k];
      if (p != k) {
        const z64 t = a[i * n + k];
        a[i * n + k] = a[i * n + p];
        a[i * n + p] = t;
      }
    }
  __syncthreads();
  z64* dst = Ainv + b * sIb;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) dst[(int64_t)(e / n) * ldi + (e % n)] = a[e];
  if (threadIdx.x == 0) {
    det[b] = s_det;
    if (info) info[b] = s_bad;
  }
}

}  // namespace

constexpr int kDetInvMaxN = 96;

}  // namespace agb

extern "C" {

agb_status agb_zgemm_batched(int64_t batch, int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im,
                             const void* A, int64_t sAm, int64_t sAk, int64_t sAb, int conjA, const void* B,
                             int64_t sBk, int64_t sBn, int64_t sBb, int conjB, double beta_re, double beta_im,
                             void* C, int64_t ldc, int64_t sCb, void* stream) {
  using namespace agb;
  AGB_ARG_CHECK(batch >= 0 && M >= 0 && N >= 0 && K >= 0, "zgemm_batched: negative size");
  AGB_ARG_CHECK((conjA == 0 || conjA == 1) && (conjB == 0 || conjB == 1), "zgemm_batched: conj flags must be 0 or 1");
  if (batch == 0 || M == 0 || N == 0) return AGB_OK;
  AGB_ARG_CHECK(A && B && C, "zgemm_batched: null pointer");
  AGB_ARG_CHECK(M <= 1 || ldc >= N, "zgemm_batched: ldc must be at least N (C is row-major)");
  AGB_ARG_CHECK((M + TB - 1) / TB <= 65535 && (N + TB - 1) / TB <= 2147483647LL, "zgemm_batched: M too large");
  BGemmArgs p{M, N, K, zmk(alpha_re, alpha_im), zmk(beta_re, beta_im), (const z64*)A, sAm, sAk, sAb, conjA,
              (const z64*)B, sBk, sBn, sBb, conjB, (z64*)C, ldc, sCb, 0};
  const dim3 tiles((unsigned)((N + TB - 1) / TB), (unsigned)((M + TB - 1) / TB), 1);
  for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
    p.b0 = b0;
    const int64_t nb = batch - b0 < 65535 ? batch - b0 : 65535;
    batched_zgemm_kernel<<<dim3(tiles.x, tiles.y, (unsigned)nb), 256, 0, (cudaStream_t)stream>>>(p);
    AGB_LAUNCH_CHECK();
  }
  return AGB_OK;
}

agb_status agb_zdet_inv_batched(int64_t batch, int n, const void* A, int64_t lda, int64_t sAb, void* Ainv,
                                int64_t ldi, int64_t sIb, void* det, int* info, void* stream) {
  using namespace agb;
  AGB_ARG_CHECK(batch >= 0 && n >= 1 && n <= kDetInvMaxN, "zdet_inv_batched: need 1 <= n <= 96");
  if (batch == 0) return AGB_OK;
  AGB_ARG_CHECK(A && Ainv && det, "zdet_inv_batched: null pointer");
  AGB_ARG_CHECK(batch <= 2147483647LL && lda >= n && ldi >= n, "zdet_inv_batched: bad batch or leading dimension");
  const size_t smem = sizeof(z64) * (size_t)n * n + sizeof(int) * (size_t)n;
  static std::atomic<uint64_t> attr_done{0};
  AGB_STATUS_TRY(once_per_device(attr_done, [&]() -> agb_status {
    AGB_CUDA_TRY(cudaFuncSetAttribute(det_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(sizeof(z64) * kDetInvMaxN * kDetInvMaxN + sizeof(int) * kDetInvMaxN)));
    return AGB_OK;
  }));
  det_inv_kernel<<<(unsigned)batch, 256, smem, (cudaStream_t)stream>>>(n, (const z64*)A, lda, sAb, (z64*)Ainv, ldi, sIb,
                                                                       (z64*)det, info);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

}  // extern "C"
