// FP64 complex GEMM on the CUDA cores (DFMA), general strides.
//
// GB300 keeps only a small FP64 pipe, so this kernel is bound by DFMA issue,
// not by memory: a 64x64 complex tile per 256-thread CTA, 4x4 outputs per
// thread, operands staged through shared memory with the load order chosen by
// which operand stride is unit (coalesced either way).
#include "common.cuh"
#include "dfloat.cuh"

namespace agb {

namespace {
constexpr int BM = 64, BN = 64, BK = 16;
constexpr int PAD = 1;

struct ZGemmArgs {
  int64_t M, N, K;
  z64 alpha, beta;
  const z64* A; int64_t sAm, sAk; int conjA;
  const z64* B; int64_t sBk, sBn; int conjB;
  z64* C; int64_t ldc;
  int64_t kchunk;       // K range per split (blockIdx.z)
  z64* partial;         // [splits][M][N] when split-K, else null
};

__global__ void __launch_bounds__(256) zgemm_kernel(ZGemmArgs p) {
  __shared__ z64 As[BK][BM + PAD];
  __shared__ z64 Bs[BK][BN + PAD];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int tid = threadIdx.x;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  z64 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = zmk(0, 0);

  const bool a_kfast = (p.sAk == 1);
  const bool b_nfast = (p.sBn == 1);
  const int64_t kbeg = (int64_t)blockIdx.z * p.kchunk;
  const int64_t kend = (kbeg + p.kchunk < p.K) ? kbeg + p.kchunk : p.K;
  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int r = 0; r < (BM * BK) / 256; ++r) {
      int idx = tid + 256 * r;
      int m, k;
      if (a_kfast) { k = idx % BK; m = idx / BK; } else { m = idx % BM; k = idx / BM; }
      int64_t gm = m0 + m, gk = k0 + k;
      z64 val = zmk(0, 0);
      if (gm < p.M && gk < kend) {
        val = p.A[gm * p.sAm + gk * p.sAk];
        if (p.conjA) val.y = -val.y;
      }
      As[k][m] = val;
    }
#pragma unroll
    for (int r = 0; r < (BN * BK) / 256; ++r) {
      int idx = tid + 256 * r;
      int n, k;
      if (b_nfast) { n = idx % BN; k = idx / BN; } else { k = idx % BK; n = idx / BK; }
      int64_t gn = n0 + n, gk = k0 + k;
      z64 val = zmk(0, 0);
      if (gn < p.N && gk < kend) {
        val = p.B[gk * p.sBk + gn * p.sBn];
        if (p.conjB) val.y = -val.y;
      }
      Bs[k][n] = val;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      z64 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) zfma(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
  if (p.partial) {
    z64* dst = p.partial + (int64_t)blockIdx.z * p.M * p.N;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int64_t gm = m0 + ty + 16 * i;
      if (gm >= p.M) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        int64_t gn = n0 + tx + 16 * j;
        if (gn < p.N) dst[gm * p.N + gn] = acc[i][j];
      }
    }
    return;
  }
  const bool use_beta = (p.beta.x != 0.0 || p.beta.y != 0.0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int64_t gm = m0 + ty + 16 * i;
    if (gm >= p.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t gn = n0 + tx + 16 * j;
      if (gn >= p.N) continue;
      z64* c = p.C + gm * p.ldc + gn;
      z64 out = zmul(p.alpha, acc[i][j]);
      if (use_beta) out = zadd(out, zmul(p.beta, *c));
      *c = out;
    }
  }
}

// C = alpha * sum_s partial[s] + beta * C, summed in split order (deterministic).
__global__ void splitk_reduce_kernel(const z64* __restrict__ partial, int splits, int64_t M, int64_t N, z64 alpha,
                                     z64 beta, z64* C, int64_t ldc) {
  int64_t total = M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    z64 s = zmk(0, 0);
    for (int z = 0; z < splits; ++z) s = zadd(s, partial[(int64_t)z * total + e]);
    int64_t m = e / N, n = e % N;
    z64* c = C + m * ldc + n;
    z64 out = zmul(alpha, s);
    if (beta.x != 0.0 || beta.y != 0.0) out = zadd(out, zmul(beta, *c));
    *c = out;
  }
}

__global__ void zscale_kernel(z64* C, int64_t M, int64_t N, int64_t ldc, z64 beta) {
  int64_t total = M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t m = e / N, n = e % N;
    z64* c = C + m * ldc + n;
    *c = (beta.x == 0.0 && beta.y == 0.0) ? zmk(0, 0) : zmul(beta, *c);
  }
}
}  // namespace

// Number of K splits worth using for an M x N output given the partial buffer capacity.
int zgemm_splits(int64_t M, int64_t N, int64_t K, size_t scratch_bytes) {
  int64_t tiles = ((M + BM - 1) / BM) * ((N + BN - 1) / BN);
  if (tiles >= 152 || K < 8 * BK) return 1;
  int64_t want = (2 * 152 + tiles - 1) / tiles;
  int64_t kmax = K / (4 * BK);
  if (want > kmax) want = kmax;
  int64_t cap = (int64_t)(scratch_bytes / (sizeof(z64) * (size_t)(M * N)));
  if (want > cap) want = cap;
  if (want > 256) want = 256;
  return want < 1 ? 1 : (int)want;
}

agb_status zgemm_ex(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                    const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                    void* scratch, size_t scratch_bytes, cudaStream_t stream) {
  AGB_ARG_CHECK(M >= 0 && N >= 0 && K >= 0, "zgemm: negative size");
  if (M == 0 || N == 0) return AGB_OK;
  AGB_ARG_CHECK(C != nullptr, "zgemm: null C");
  if (K == 0 || (alpha.x == 0.0 && alpha.y == 0.0)) {
    zscale_kernel<<<grid_for(M * N, 256), 256, 0, stream>>>(C, M, N, ldc, beta);
    AGB_LAUNCH_CHECK();
    return AGB_OK;
  }
  AGB_ARG_CHECK(A != nullptr && B != nullptr, "zgemm: null operand");
  AGB_ARG_CHECK((M + BM - 1) / BM <= 65535, "zgemm: M too large for grid");
  int splits = scratch ? zgemm_splits(M, N, K, scratch_bytes) : 1;
  int64_t kchunk = K;
  if (splits > 1) {
    kchunk = (K + splits - 1) / splits;
    kchunk = (kchunk + BK - 1) / BK * BK;
    splits = (int)((K + kchunk - 1) / kchunk);
  }
  ZGemmArgs p{M, N, K, alpha, beta, A, sAm, sAk, conjA, B, sBk, sBn, conjB, C, ldc, kchunk,
              splits > 1 ? (z64*)scratch : nullptr};
  dim3 grid((unsigned)((N + BN - 1) / BN), (unsigned)((M + BM - 1) / BM), (unsigned)splits);
  zgemm_kernel<<<grid, 256, 0, stream>>>(p);
  AGB_LAUNCH_CHECK();
  if (splits > 1) {
    splitk_reduce_kernel<<<grid_for(M * N, 256), 256, 0, stream>>>((const z64*)scratch, splits, M, N, alpha, beta, C,
                                                                   ldc);
    AGB_LAUNCH_CHECK();
  }
  return AGB_OK;
}

agb_status zgemm(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                 const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                 cudaStream_t stream) {
  return zgemm_ex(M, N, K, alpha, A, sAm, sAk, conjA, B, sBk, sBn, conjB, beta, C, ldc, nullptr, 0, stream);
}

// y[m] = alpha * sum_k A[m*lda + k] x[k] + beta * y[m]: one warp per row, FP64.
namespace {
__global__ void zgemv_kernel(int64_t M, int64_t K, z64 alpha, const z64* __restrict__ A, int64_t lda,
                             const z64* __restrict__ x, z64 beta, z64* y) {
  int lane = threadIdx.x & 31;
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t m = warp; m < M; m += nwarps) {
    z64 s = zmk(0, 0);
    const z64* a = A + m * lda;
    for (int64_t k = lane; k < K; k += 32) zfma(s, a[k], x[k]);
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, off);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, off);
    }
    if (lane == 0) {
      z64 out = zmul(alpha, s);
      if (beta.x != 0.0 || beta.y != 0.0) out = zadd(out, zmul(beta, y[m]));
      y[m] = out;
    }
  }
}
// y = alpha A x + beta y with the products and sums in double-float on the FP32 pipe
// (~2^-44 relative): one warp per row, FP64 only for the per-row result.
__global__ void zgemv_df_kernel(int64_t M, int64_t K, z64 alpha, const z64* __restrict__ A, int64_t lda,
                                const z64* __restrict__ x, z64 beta, z64* y) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t m = warp; m < M; m += nwarps) {
    float re = 0.f, rec = 0.f, im = 0.f, imc = 0.f;
    const z64* a = A + m * lda;
    for (int64_t k = lane; k < K; k += 32) {
      const float4 av = split_z_fast(a[k]);
      const float4 xv = split_z_fast(x[k]);
      // a x = (ar xr - ai xi) + i (ar xi + ai xr)
      df_mac(re, rec, av.x, av.y, xv.x, xv.y);
      df_mac(re, rec, -av.z, -av.w, xv.z, xv.w);
      df_mac(im, imc, av.x, av.y, xv.z, xv.w);
      df_mac(im, imc, av.z, av.w, xv.x, xv.y);
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      df_add(re, rec, __shfl_xor_sync(0xffffffffu, re, off), __shfl_xor_sync(0xffffffffu, rec, off));
      df_add(im, imc, __shfl_xor_sync(0xffffffffu, im, off), __shfl_xor_sync(0xffffffffu, imc, off));
    }
    if (lane == 0) {
      z64 out = zmul(alpha, zmk(df_to_double(re, rec), df_to_double(im, imc)));
      if (beta.x != 0.0 || beta.y != 0.0) out = zadd(out, zmul(beta, y[m]));
      y[m] = out;
    }
  }
}
// y = alpha A x + beta y in FP32 arithmetic (each FP64 value truncated to its leading 24
// significant bits on the integer pipe, FP32 multiply-adds, a warp per row): for residuals
// whose other terms come from 3xTF32 tensor-core products (FP32-level error), where the
// double-float GEMV's instruction count, not the HBM stream, would set the time.
__global__ void zgemv_f32_kernel(int64_t M, int64_t K, z64 alpha, const z64* __restrict__ A, int64_t lda,
                                 const z64* __restrict__ x, z64 beta, z64* y) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t m = warp; m < M; m += nwarps) {
    float re = 0.f, im = 0.f;
    const z64* a = A + m * lda;
    for (int64_t k = lane; k < K; k += 32) {
      const float4 av = split_z_fast(__ldcs(&a[k]));
      const float4 xv = split_z_fast(x[k]);
      re = fmaf(av.x, xv.x, re);
      re = fmaf(-av.z, xv.z, re);
      im = fmaf(av.x, xv.z, im);
      im = fmaf(av.z, xv.x, im);
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, off);
      im += __shfl_xor_sync(0xffffffffu, im, off);
    }
    if (lane == 0) {
      z64 out = zmul(alpha, zmk(f2d_exact(re), f2d_exact(im)));
      if (beta.x != 0.0 || beta.y != 0.0) out = zadd(out, zmul(beta, y[m]));
      y[m] = out;
    }
  }
}
}  // namespace

agb_status zgemv_f32(int64_t M, int64_t K, z64 alpha, const z64* A, int64_t lda, const z64* x, z64 beta, z64* y,
                     cudaStream_t stream) {
  if (M == 0) return AGB_OK;
  zgemv_f32_kernel<<<grid_for(M * 32, 256), 256, 0, stream>>>(M, K, alpha, A, lda, x, beta, y);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

agb_status zgemv(int64_t M, int64_t K, z64 alpha, const z64* A, int64_t lda, const z64* x, z64 beta, z64* y,
                 cudaStream_t stream) {
  if (M == 0) return AGB_OK;
  zgemv_kernel<<<grid_for(M * 32, 256), 256, 0, stream>>>(M, K, alpha, A, lda, x, beta, y);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

agb_status zgemv_df(int64_t M, int64_t K, z64 alpha, const z64* A, int64_t lda, const z64* x, z64 beta, z64* y,
                    cudaStream_t stream) {
  if (M == 0) return AGB_OK;
  zgemv_df_kernel<<<grid_for(M * 32, 256), 256, 0, stream>>>(M, K, alpha, A, lda, x, beta, y);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

}  // namespace agb

extern "C" agb_status agb_zgemm(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im, const void* A,
                                int64_t sAm, int64_t sAk, int conjA, const void* B, int64_t sBk, int64_t sBn,
                                int conjB, double beta_re, double beta_im, void* C, int64_t ldc, void* stream) {
  AGB_ARG_CHECK((conjA == 0 || conjA == 1) && (conjB == 0 || conjB == 1), "gemm: conj flags must be 0 or 1");
  AGB_ARG_CHECK(M <= 1 || N <= 0 || ldc >= N, "gemm: ldc must be at least N (C is row-major)");
  return agb::zgemm(M, N, K, agb::zmk(alpha_re, alpha_im), (const agb::z64*)A, sAm, sAk, conjA,
                    (const agb::z64*)B, sBk, sBn, conjB, agb::zmk(beta_re, beta_im), (agb::z64*)C, ldc,
                    (cudaStream_t)stream);
}

extern "C" size_t agb_zgemm_scratch_bytes(int64_t M, int64_t N, int64_t K) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  const int splits = agb::zgemm_splits(M, N, K, (size_t)-1 / 2);
  return splits > 1 ? sizeof(agb::z64) * (size_t)splits * (size_t)M * (size_t)N : 0;
}

extern "C" agb_status agb_zgemm_ex(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im, const void* A,
                                   int64_t sAm, int64_t sAk, int conjA, const void* B, int64_t sBk, int64_t sBn,
                                   int conjB, double beta_re, double beta_im, void* C, int64_t ldc, void* scratch,
                                   size_t scratch_bytes, void* stream) {
  AGB_ARG_CHECK((conjA == 0 || conjA == 1) && (conjB == 0 || conjB == 1), "gemm: conj flags must be 0 or 1");
  AGB_ARG_CHECK(M <= 1 || N <= 0 || ldc >= N, "gemm: ldc must be at least N (C is row-major)");
  AGB_ARG_CHECK(scratch != nullptr || scratch_bytes == 0, "gemm: scratch is NULL with a nonzero size");
  return agb::zgemm_ex(M, N, K, agb::zmk(alpha_re, alpha_im), (const agb::z64*)A, sAm, sAk, conjA,
                       (const agb::z64*)B, sBk, sBn, conjB, agb::zmk(beta_re, beta_im), (agb::z64*)C, ldc,
                       scratch_bytes ? scratch : nullptr, scratch_bytes, (cudaStream_t)stream);
}
