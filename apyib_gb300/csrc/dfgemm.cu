// Complex GEMM in double-float ("df64") arithmetic on the FP32 CUDA cores.
//
// GB300's FP64 pipe issues about two DFMA per clock per SM, while the FP32 pipe
// issues 128 FMA per clock per SM.  Each FP64 operand is split into a float
// pair x = x_hi + x_lo (48 significant bits); products use the exact FMA split
// p = x_hi*y_hi, e = fma(x_hi, y_hi, -p) plus the two cross terms, and the
// running sum is a float pair updated with Knuth's two-sum, so the result
// carries ~2^-44 relative error after 10^4-term sums: far below what the
// iterative-refinement residual needs.  With scratch for the split operands the
// split happens once per element (not per tile load, which would keep the slow
// FP64 pipe busy) and the complex product uses three real products
// (Re = ArBr - AiBi, Im = (Ar+Ai)(Br+Bi) - ArBr - AiBi); without scratch the
// per-tile-split four-product kernel runs.  Same contract as the FP64 zgemm.
#include "common.cuh"
#include "dfloat.cuh"

namespace agb {

namespace {
constexpr int BM = 64, BN = 64, BK = 16;

struct DfArgs {
  int64_t M, N, K;
  z64 alpha, beta;
  const z64* A; int64_t sAm, sAk; int conjA;
  const z64* B; int64_t sBk, sBn; int conjB;
  z64* C; int64_t ldc;
  int64_t kchunk;
  z64* partial;
};

__global__ void __launch_bounds__(256) dfgemm_kernel(DfArgs p) {
  __shared__ float4 As[BK][BM + 1];
  __shared__ float4 Bs[BK][BN + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4, tid = threadIdx.x;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  float sr[4][4], cr[4][4], si[4][4], ci[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) sr[i][j] = cr[i][j] = si[i][j] = ci[i][j] = 0.f;
  const bool a_kfast = (p.sAk == 1), b_nfast = (p.sBn == 1);
  const int64_t kbeg = (int64_t)blockIdx.z * p.kchunk;
  const int64_t kend = (kbeg + p.kchunk < p.K) ? kbeg + p.kchunk : p.K;
  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int r = 0; r < (BM * BK) / 256; ++r) {
      int idx = tid + 256 * r, m, k;
      if (a_kfast) { k = idx % BK; m = idx / BK; } else { m = idx % BM; k = idx / BM; }
      int64_t gm = m0 + m, gk = k0 + k;
      z64 v = zmk(0, 0);
      if (gm < p.M && gk < kend) {
        v = p.A[gm * p.sAm + gk * p.sAk];
        if (p.conjA) v.y = -v.y;
      }
      As[k][m] = split_z(v);
    }
#pragma unroll
    for (int r = 0; r < (BN * BK) / 256; ++r) {
      int idx = tid + 256 * r, n, k;
      if (b_nfast) { n = idx % BN; k = idx / BN; } else { k = idx % BK; n = idx / BK; }
      int64_t gn = n0 + n, gk = k0 + k;
      z64 v = zmk(0, 0);
      if (gn < p.N && gk < kend) {
        v = p.B[gk * p.sBk + gn * p.sBn];
        if (p.conjB) v.y = -v.y;
      }
      Bs[k][n] = split_z(v);
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < BK; ++kk) {
      float4 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          // re += ar*br - ai*bi ; im += ar*bi + ai*br
          df_mac(sr[i][j], cr[i][j], a[i].x, a[i].y, b[j].x, b[j].y);
          df_mac(sr[i][j], cr[i][j], a[i].z, a[i].w, -b[j].z, -b[j].w);
          df_mac(si[i][j], ci[i][j], a[i].x, a[i].y, b[j].z, b[j].w);
          df_mac(si[i][j], ci[i][j], a[i].z, a[i].w, b[j].x, b[j].y);
        }
    }
    __syncthreads();
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
      z64 acc = zmk((double)sr[i][j] + (double)cr[i][j], (double)si[i][j] + (double)ci[i][j]);
      if (p.partial) {
        p.partial[((int64_t)blockIdx.z * p.M + gm) * p.N + gn] = acc;
      } else {
        z64* c = p.C + gm * p.ldc + gn;
        z64 out = zmul(p.alpha, acc);
        if (use_beta) out = zadd(out, zmul(p.beta, *c));
        *c = out;
      }
    }
  }
}

// ---- 3M variant: Re = P1 - P2, Im = P3 - P1 - P2 with P1 = Ar Br, P2 = Ai Bi,
// P3 = (Ar + Ai)(Br + Bi); three double-float products per complex multiply-add
// instead of four.  Operands are pre-split into float4 (re_hi, re_lo, im_hi, im_lo)
// and float2 (sum_hi, sum_lo) rows.
__global__ void df_split3_kernel(const z64* __restrict__ src, int64_t rows, int64_t K, int64_t s_row, int64_t s_k,
                                 int conj, int64_t Kp, float4* __restrict__ dst4, float2* __restrict__ dst2) {
  __shared__ z64 tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool kfast = (s_k == 1) || (s_row != 1 && s_k <= s_row);
  const int64_t tiles_k = (Kp + 31) / 32, tiles = ((rows + 31) / 32) * tiles_k;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t r0 = (t / tiles_k) * 32, k0 = (t % tiles_k) * 32;
    for (int i = ty; i < 32; i += 8) {
      int64_t r, k;
      if (kfast) { r = r0 + i; k = k0 + tx; } else { r = r0 + tx; k = k0 + i; }
      z64 v = zmk(0, 0);
      if (r < rows && k < K) {
        if (conj == kSrcReal) v.x = ((const double*)src)[r * s_row + k * s_k];
        else v = src[r * s_row + k * s_k];
      }
      if (conj == 1) v.y = -v.y;
      if (kfast) tile[i][tx] = v; else tile[tx][i] = v;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
      int64_t r = r0 + i, k = k0 + tx;
      if (r < rows && k < Kp) {
        z64 v = tile[i][tx];
        dst4[r * Kp + k] = split_z(v);
        uint32_t sh, sl;
        split_f32pair((uint64_t)__double_as_longlong(v.x + v.y), sh, sl);
        dst2[r * Kp + k] = make_float2(__uint_as_float(sh), __uint_as_float(sl));
      }
    }
    __syncthreads();
  }
}

constexpr int DF3_SMEM = BK * (BM + 1) * (16 + 8) + BK * (BN + 1) * (16 + 8);

__global__ void __launch_bounds__(256) dfgemm3m_kernel(int64_t M, int64_t N, int64_t Kp, int64_t kchunk, z64 alpha,
                                                       z64 beta, const float4* __restrict__ A4,
                                                       const float2* __restrict__ A2, const float4* __restrict__ B4,
                                                       const float2* __restrict__ B2, z64* C, int64_t ldc,
                                                       z64* partial) {
  extern __shared__ __align__(16) uint8_t df3_smem[];
  float4 (*As4)[BM + 1] = (float4 (*)[BM + 1])df3_smem;
  float4 (*Bs4)[BN + 1] = (float4 (*)[BN + 1])(df3_smem + BK * (BM + 1) * 16);
  float2 (*As2)[BM + 1] = (float2 (*)[BM + 1])(df3_smem + BK * (BM + 1) * 16 + BK * (BN + 1) * 16);
  float2 (*Bs2)[BN + 1] = (float2 (*)[BN + 1])(df3_smem + BK * (BM + 1) * 24 + BK * (BN + 1) * 16);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4, tid = threadIdx.x;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  float s1[4][4], c1[4][4], s2[4][4], c2[4][4], s3[4][4], c3[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) s1[i][j] = c1[i][j] = s2[i][j] = c2[i][j] = s3[i][j] = c3[i][j] = 0.f;
  const int64_t kbeg = (int64_t)blockIdx.z * kchunk;
  const int64_t kend = (kbeg + kchunk < Kp) ? kbeg + kchunk : Kp;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  const float2 z2 = make_float2(0.f, 0.f);
  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int r = 0; r < (BM * BK) / 256; ++r) {
      int idx = tid + 256 * r, k = idx % BK, m = idx / BK;
      int64_t gm = m0 + m, gk = k0 + k;
      bool in = gm < M && gk < kend;
      As4[k][m] = in ? A4[gm * Kp + gk] : z4;
      As2[k][m] = in ? A2[gm * Kp + gk] : z2;
    }
#pragma unroll
    for (int r = 0; r < (BN * BK) / 256; ++r) {
      int idx = tid + 256 * r, k = idx % BK, n = idx / BK;
      int64_t gn = n0 + n, gk = k0 + k;
      bool in = gn < N && gk < kend;
      Bs4[k][n] = in ? B4[gn * Kp + gk] : z4;
      Bs2[k][n] = in ? B2[gn * Kp + gk] : z2;
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < BK; ++kk) {
      float4 a[4], b[4];
      float2 as[4], bs[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) { a[i] = As4[kk][ty + 16 * i]; as[i] = As2[kk][ty + 16 * i]; }
#pragma unroll
      for (int j = 0; j < 4; ++j) { b[j] = Bs4[kk][tx + 16 * j]; bs[j] = Bs2[kk][tx + 16 * j]; }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          df_mac(s1[i][j], c1[i][j], a[i].x, a[i].y, b[j].x, b[j].y);
          df_mac(s2[i][j], c2[i][j], a[i].z, a[i].w, b[j].z, b[j].w);
          df_mac(s3[i][j], c3[i][j], as[i].x, as[i].y, bs[j].x, bs[j].y);
        }
    }
    __syncthreads();
  }
  const bool use_beta = (beta.x != 0.0 || beta.y != 0.0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int64_t gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      double p1 = (double)s1[i][j] + (double)c1[i][j];
      double p2 = (double)s2[i][j] + (double)c2[i][j];
      double p3 = (double)s3[i][j] + (double)c3[i][j];
      z64 acc = zmk(p1 - p2, p3 - p1 - p2);
      if (partial) {
        partial[((int64_t)blockIdx.z * M + gm) * N + gn] = acc;
      } else {
        z64* c = C + gm * ldc + gn;
        z64 out = zmul(alpha, acc);
        if (use_beta) out = zadd(out, zmul(beta, *c));
        *c = out;
      }
    }
  }
}

__global__ void df_splitk_sum_kernel(const z64* __restrict__ partial, int splits, int64_t M, int64_t N, z64 alpha,
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
}  // namespace

agb_status zgemm_ex(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                    const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                    void* scratch, size_t scratch_bytes, cudaStream_t stream);
int zgemm_splits(int64_t M, int64_t N, int64_t K, size_t scratch_bytes);

// Scratch that lets dfgemm_ex take the pre-split path for this shape (split operands
// plus split-K partials when the tile grid is small).
size_t dfgemm_scratch_bytes(int64_t M, int64_t N, int64_t K) {
  const int64_t Kp = (K + BK - 1) / BK * BK;
  size_t s = ((size_t)(M + N) * (size_t)Kp * (sizeof(float4) + sizeof(float2)) + 511) & ~(size_t)255;
  int64_t tiles = ((M + BM - 1) / BM) * ((N + BN - 1) / BN);
  if (tiles < 152 && Kp >= 8 * BK) s += (size_t)256 * M * N * sizeof(z64);
  return s;
}

agb_status dfgemm_ex(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                     const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                     void* scratch, size_t scratch_bytes, cudaStream_t stream) {
  AGB_ARG_CHECK(M >= 0 && N >= 0 && K >= 0, "dfgemm: negative size");
  if (M == 0 || N == 0) return AGB_OK;
  if (K == 0 || (alpha.x == 0.0 && alpha.y == 0.0))
    return zgemm_ex(M, N, K, alpha, A, sAm, sAk, conjA, B, sBk, sBn, conjB, beta, C, ldc, nullptr, 0, stream);
  AGB_ARG_CHECK(A && B && C, "dfgemm: null pointer");
  AGB_ARG_CHECK((M + BM - 1) / BM <= 65535, "dfgemm: M too large for grid");
  // Pre-split 3M path when the scratch holds both split operands (24 B per element).
  const int64_t Kp = (K + BK - 1) / BK * BK;
  const size_t split_bytes =
      ((size_t)(M + N) * (size_t)Kp * (sizeof(float4) + sizeof(float2)) + 511) & ~(size_t)255;
  if (scratch && scratch_bytes >= split_bytes) {
    float4* A4 = (float4*)scratch;
    float4* B4 = A4 + (size_t)M * Kp;
    float2* A2 = (float2*)(B4 + (size_t)N * Kp);
    float2* B2 = A2 + (size_t)M * Kp;
    void* rest = (char*)scratch + split_bytes;
    size_t rest_bytes = scratch_bytes - split_bytes;
    auto launch_split = [&](const z64* src, int64_t rows, int64_t s_row, int64_t s_k, int conj, float4* d4,
                            float2* d2) {
      int64_t tiles = ((rows + 31) / 32) * ((Kp + 31) / 32);
      int grid = (int)(tiles < 152 * 32 ? tiles : 152 * 32);
      df_split3_kernel<<<grid, 256, 0, stream>>>(src, rows, K, s_row, s_k, conj, Kp, d4, d2);
    };
    launch_split(A, M, sAm, sAk, conjA, A4, A2);
    AGB_LAUNCH_CHECK();
    launch_split(B, N, sBn, sBk, conjB, B4, B2);
    AGB_LAUNCH_CHECK();
    static std::atomic<uint64_t> attr_done{0};
    AGB_STATUS_TRY(once_per_device(attr_done, [&]() -> agb_status {
      AGB_CUDA_TRY(cudaFuncSetAttribute(dfgemm3m_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, DF3_SMEM));
      return AGB_OK;
    }));
    int sp = zgemm_splits(M, N, Kp, rest_bytes);
    int64_t kc = Kp;
    if (sp > 1) {
      kc = (Kp + sp - 1) / sp;
      kc = (kc + BK - 1) / BK * BK;
      sp = (int)((Kp + kc - 1) / kc);
    }
    dim3 grid((unsigned)((N + BN - 1) / BN), (unsigned)((M + BM - 1) / BM), (unsigned)sp);
    dfgemm3m_kernel<<<grid, 256, DF3_SMEM, stream>>>(M, N, Kp, kc, alpha, beta, A4, A2, B4, B2, C, ldc,
                                                     sp > 1 ? (z64*)rest : nullptr);
    AGB_LAUNCH_CHECK();
    if (sp > 1) {
      df_splitk_sum_kernel<<<grid_for(M * N, 256), 256, 0, stream>>>((const z64*)rest, sp, M, N, alpha, beta, C,
                                                                      ldc);
      AGB_LAUNCH_CHECK();
    }
    return AGB_OK;
  }
  if (conjA == kSrcReal || conjB == kSrcReal) {
    agb_set_error_message("dfgemm: a real operand needs scratch for the pre-split path", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  int splits = scratch ? zgemm_splits(M, N, K, scratch_bytes) : 1;
  int64_t kchunk = K;
  if (splits > 1) {
    kchunk = (K + splits - 1) / splits;
    kchunk = (kchunk + BK - 1) / BK * BK;
    splits = (int)((K + kchunk - 1) / kchunk);
  }
  DfArgs p{M, N, K, alpha, beta, A, sAm, sAk, conjA, B, sBk, sBn, conjB, C, ldc, kchunk,
           splits > 1 ? (z64*)scratch : nullptr};
  dim3 grid((unsigned)((N + BN - 1) / BN), (unsigned)((M + BM - 1) / BM), (unsigned)splits);
  dfgemm_kernel<<<grid, 256, 0, stream>>>(p);
  AGB_LAUNCH_CHECK();
  if (splits > 1) {
    df_splitk_sum_kernel<<<grid_for(M * N, 256), 256, 0, stream>>>((const z64*)scratch, splits, M, N, alpha, beta,
                                                                    C, ldc);
    AGB_LAUNCH_CHECK();
  }
  return AGB_OK;
}

}  // namespace agb

extern "C" size_t agb_zgemm_df64_scratch_bytes(int64_t M, int64_t N, int64_t K) {
  return agb::dfgemm_scratch_bytes(M, N, K);
}

extern "C" agb_status agb_zgemm_df64_ex(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im,
                                        const void* A, int64_t sAm, int64_t sAk, int conjA, const void* B,
                                        int64_t sBk, int64_t sBn, int conjB, double beta_re, double beta_im, void* C,
                                        int64_t ldc, void* scratch, size_t scratch_bytes, void* stream) {
  AGB_ARG_CHECK((conjA == 0 || conjA == 1) && (conjB == 0 || conjB == 1), "gemm: conj flags must be 0 or 1");
  AGB_ARG_CHECK(M <= 1 || N <= 0 || ldc >= N, "gemm: ldc must be at least N (C is row-major)");
  return agb::dfgemm_ex(M, N, K, agb::zmk(alpha_re, alpha_im), (const agb::z64*)A, sAm, sAk, conjA,
                        (const agb::z64*)B, sBk, sBn, conjB, agb::zmk(beta_re, beta_im), (agb::z64*)C, ldc, scratch,
                        scratch_bytes, (cudaStream_t)stream);
}

extern "C" agb_status agb_zgemm_df64(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im, const void* A,
                                     int64_t sAm, int64_t sAk, int conjA, const void* B, int64_t sBk, int64_t sBn,
                                     int conjB, double beta_re, double beta_im, void* C, int64_t ldc, void* stream) {
  AGB_ARG_CHECK((conjA == 0 || conjA == 1) && (conjB == 0 || conjB == 1), "gemm: conj flags must be 0 or 1");
  AGB_ARG_CHECK(M <= 1 || N <= 0 || ldc >= N, "gemm: ldc must be at least N (C is row-major)");
  return agb::dfgemm_ex(M, N, K, agb::zmk(alpha_re, alpha_im), (const agb::z64*)A, sAm, sAk, conjA,
                        (const agb::z64*)B, sBk, sBn, conjB, agb::zmk(beta_re, beta_im), (agb::z64*)C, ldc, nullptr, 0,
                        (cudaStream_t)stream);
}
