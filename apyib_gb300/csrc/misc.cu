// Spin-orbital expansion, amplitude pack/unpack, MP2_SO, the AO->MO
// four-index transform and the one-pass J/K Fock build.
#include "cisd_plan.h"
#include "dfloat.cuh"

namespace agb {

agb_status zgemm_ex(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                    const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                    void* scratch, size_t scratch_bytes, cudaStream_t stream);
agb_status cgemm_tf32x3(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk,
                        int conjA, const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                        void* scratch, size_t scratch_bytes, cudaStream_t stream);
size_t cgemm_tf32x3_scratch(int64_t M, int64_t N, int64_t K);
agb_status cgemm_tf32x3_fa(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk,
                           int conjA, const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C,
                           int64_t ldc, void* scratch, size_t scratch_bytes, cudaStream_t stream);
agb_status dfgemm_ex(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                     const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                     void* scratch, size_t scratch_bytes, cudaStream_t stream);
size_t dfgemm_scratch_bytes(int64_t M, int64_t N, int64_t K);
agb_status ozgemm_ex(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                     const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                     void* scratch, size_t scratch_bytes, cudaStream_t stream);
size_t ozgemm_scratch_bytes(int64_t M, int64_t N, int64_t K);
size_t ozgemm_scratch_bytes_fused(int64_t M, int64_t N, int64_t K);

namespace {

__global__ void f_so_kernel(const z64* __restrict__ F, int64_t n, z64* __restrict__ out) {
  int64_t m = 2 * n, total = m * m;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t p = e / m, q = e % m;
    out[e] = ((p ^ q) & 1) ? zmk(0, 0) : F[(p >> 1) * n + (q >> 1)];
  }
}

__global__ void eri_so_kernel(const z64* __restrict__ g, int64_t n0, int64_t n1, int64_t n2, int64_t n3,
                              z64* __restrict__ out) {
  int64_t m1 = 2 * n1, m2 = 2 * n2, m3 = 2 * n3;
  int64_t total = 2 * n0 * m1 * m2 * m3;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = e % m3, rest = e / m3;
    int64_t r = rest % m2; rest /= m2;
    int64_t q = rest % m1, p = rest / m1;
    z64 val = zmk(0, 0);
    if (!((p ^ q) & 1) && !((r ^ s) & 1)) val = g[(((p >> 1) * n1 + (q >> 1)) * n2 + (r >> 1)) * n3 + (s >> 1)];
    out[e] = val;
  }
}

__device__ __forceinline__ int sgnp(int x, int y) { return x < y ? 1 : (x > y ? -1 : 0); }

// full t2[i][j][a][b] from packed
__global__ void unpack_full_kernel(const z64* __restrict__ t2p, int o, int v, int64_t pv, z64* __restrict__ t2) {
  int64_t vv = (int64_t)v * v, total = (int64_t)o * o * vv;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t ij = e / vv, ab = e % vv;
    int i = (int)(ij / o), j = (int)(ij % o), a = (int)(ab / v), b = (int)(ab % v);
    int s = sgnp(i, j) * sgnp(a, b);
    z64 val = zmk(0, 0);
    if (s) {
      val = t2p[pair_index(min(i, j), max(i, j), o) * pv + pair_index(min(a, b), max(a, b), v)];
      if (s < 0) val = zneg(val);
    }
    t2[e] = val;
  }
}

__global__ void pack_kernel(const z64* __restrict__ t2, int o, int v, int64_t po, int64_t pv,
                            const int2* __restrict__ opairs, const int2* __restrict__ vpairs, z64* __restrict__ t2p) {
  int64_t total = po * pv;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int2 ij = opairs[e / pv], ab = vpairs[e % pv];
    t2p[e] = t2[(((int64_t)ij.x * o + ij.y) * v + ab.x) * v + ab.y];
  }
}

__global__ void copy_kernel(const z64* __restrict__ src, int64_t n, z64* __restrict__ dst) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    dst[e] = src[e];
}

__device__ __forceinline__ z64 warp_sum(z64 s) {
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, off);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, off);
  }
  return s;
}

constexpr int kMp2Blocks = 152 * 4;

// t2p = <ab||ij>_p * (1/D), partial[b] = sum t2p * <ij||ab>_p
// invD2: the plan's 1 / (e_i + e_j - e_a - e_b) of each packed doubles amplitude.
__global__ void __launch_bounds__(256) mp2_kernel(const z64* __restrict__ R0p, const z64* __restrict__ Wop,
                                                  const double* __restrict__ invD2, int64_t n2,
                                                  z64* __restrict__ t2p, z64* __restrict__ partial) {
  // t = <ab||ij> / D in FP64 (two multiplies); the energy sum W t in double-float on the
  // FP32 pipe (~2^-44 relative): complex FP64 multiply-adds per element would make this
  // stream FP64-pipe bound on GB300
  float er = 0.f, erc = 0.f, ei = 0.f, eic = 0.f;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n2; e += (int64_t)gridDim.x * blockDim.x) {
    const double inv = invD2[e];
    const z64 num = R0p[e];
    const z64 t = zmk(num.x * inv, num.y * inv);
    t2p[e] = t;
    const float4 w = split_z_fast(Wop[e]);
    const float4 tv = split_z_fast(t);
    // w t = (wr tr - wi ti) + i (wr ti + wi tr)
    df_mac(er, erc, w.x, w.y, tv.x, tv.y);
    df_mac(er, erc, -w.z, -w.w, tv.z, tv.w);
    df_mac(ei, eic, w.x, w.y, tv.z, tv.w);
    df_mac(ei, eic, w.z, w.w, tv.x, tv.y);
  }
  z64 acc = zmk(df_to_double(er, erc), df_to_double(ei, eic));
  __shared__ z64 sh[32];
  acc = warp_sum(acc);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = acc;
  __syncthreads();
  if (w == 0) {
    acc = lane < (int)(blockDim.x >> 5) ? sh[lane] : zmk(0, 0);
    acc = warp_sum(acc);
    if (lane == 0) partial[blockIdx.x] = acc;
  }
}

// *out = sum of partial[0 .. n), one 256-thread block: strided sums in order, then a fixed
// tree (deterministic).
__global__ void __launch_bounds__(256) sum_partials_kernel(const z64* __restrict__ partial, int n, z64* out) {
  __shared__ z64 sh[256];
  const int t = threadIdx.x;
  z64 s = zmk(0, 0);
  for (int b = t; b < n; b += 256) s = zadd(s, partial[b]);
  sh[t] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (t < w) sh[t] = zadd(sh[t], sh[t + w]);
    __syncthreads();
  }
  if (t == 0) *out = sh[0];
}

// ---- real FP64 GEMM (first AO->MO quarter step: real ERIs x interleaved complex C)
constexpr int DBM = 64, DBN = 64, DBK = 16;
__global__ void __launch_bounds__(256) dgemm_kernel(int64_t M, int64_t N, int64_t K, const double* __restrict__ A,
                                                    int64_t sAm, int64_t sAk, const double* __restrict__ B,
                                                    int64_t sBk, int64_t sBn, double* __restrict__ C, int64_t ldc) {
  __shared__ double As[DBK][DBM + 1];
  __shared__ double Bs[DBK][DBN + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4, tid = threadIdx.x;
  const int64_t m0 = (int64_t)blockIdx.y * DBM, n0 = (int64_t)blockIdx.x * DBN;
  double acc[4][4] = {};
  const bool a_kfast = (sAk == 1), b_nfast = (sBn == 1);
  for (int64_t k0 = 0; k0 < K; k0 += DBK) {
#pragma unroll
    for (int r = 0; r < (DBM * DBK) / 256; ++r) {
      int idx = tid + 256 * r, m, k;
      if (a_kfast) { k = idx % DBK; m = idx / DBK; } else { m = idx % DBM; k = idx / DBM; }
      int64_t gm = m0 + m, gk = k0 + k;
      As[k][m] = (gm < M && gk < K) ? A[gm * sAm + gk * sAk] : 0.0;
    }
#pragma unroll
    for (int r = 0; r < (DBN * DBK) / 256; ++r) {
      int idx = tid + 256 * r, n, k;
      if (b_nfast) { n = idx % DBN; k = idx / DBN; } else { k = idx % DBK; n = idx / DBK; }
      int64_t gn = n0 + n, gk = k0 + k;
      Bs[k][n] = (gn < N && gk < K) ? B[gk * sBk + gn * sBn] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < DBK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int64_t gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t gn = n0 + tx + 16 * j;
      if (gn < N) C[gm * ldc + gn] = acc[i][j];
    }
  }
}

__global__ void conj_kernel(const z64* __restrict__ src, int64_t n, z64* __restrict__ dst) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    dst[e] = zconj(src[e]);
}

// ---- J/K: one pass over the real (mn|ls), products and sums in double-float on the FP32 pipe
// (four complex-by-real multiply-adds per integral would otherwise keep the FP64 pipe, not HBM,
// the bound).  CTA per m.  The rows e[m][x][y][0..n) are walked in groups of JK_Y rows
// (fixed x, consecutive y): g = yb*n + x, yb = y / JK_Y, and each warp takes one contiguous
// range of groups.  Lane z-partials accumulate
//   J[m][x] += sum_yz e D[y][z]   (reduced over the lanes once per group)
//   K[m][y] += sum_xz e D[x][z]   (kept per lane while the warp stays in one y block)
// into per-warp slots; the slots are summed in a fixed order, so results are deterministic.
constexpr int JK_Y = 4;

__global__ void jk_split_kernel(const z64* __restrict__ D, int64_t nn, float4* __restrict__ D4) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x)
    D4[e] = split_z(D[e]);
}

__device__ __forceinline__ void df_warp_sum(float& s, float& c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float bs = __shfl_xor_sync(0xffffffffu, s, o), bc = __shfl_xor_sync(0xffffffffu, c, o);
    df_add(s, c, bs, bc);
  }
}

__global__ void __launch_bounds__(512) jk_df_kernel(const double* __restrict__ eri, int n,
                                                    const float4* __restrict__ D4, const z64* __restrict__ h,
                                                    double scale, z64* __restrict__ F) {
  extern __shared__ float4 jk_sh[];       // Jw[nw][n], Kw[nw][n]: (re_s, re_c, im_s, im_c)
  const int nw = blockDim.x >> 5;
  float4* Jw = jk_sh;
  float4* Kw = jk_sh + (size_t)nw * n;
  const int m = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < 2 * nw * n; i += blockDim.x) jk_sh[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncthreads();
  const int nyb = (n + JK_Y - 1) / JK_Y;
  const int64_t ngroups = (int64_t)nyb * n;
  const int64_t g0 = ngroups * w / nw, g1 = ngroups * (w + 1) / nw;
  const double* slab = eri + (int64_t)m * n * n * n;
  float ks[JK_Y][4];
#pragma unroll
  for (int i = 0; i < JK_Y; ++i) ks[i][0] = ks[i][1] = ks[i][2] = ks[i][3] = 0.f;
  int cur_yb = g0 < g1 ? (int)(g0 / n) : -1;
  auto flush_k = [&](int yb) {
#pragma unroll
    for (int i = 0; i < JK_Y; ++i) {
      df_warp_sum(ks[i][0], ks[i][1]);
      df_warp_sum(ks[i][2], ks[i][3]);
      const int y = yb * JK_Y + i;
      if (lane == 0 && y < n) {
        float4 k = Kw[(size_t)w * n + y];
        df_add(k.x, k.y, ks[i][0], ks[i][1]);
        df_add(k.z, k.w, ks[i][2], ks[i][3]);
        Kw[(size_t)w * n + y] = k;
      }
      ks[i][0] = ks[i][1] = ks[i][2] = ks[i][3] = 0.f;
    }
  };
  for (int64_t g = g0; g < g1; ++g) {
    const int yb = (int)(g / n), x = (int)(g % n);
    if (yb != cur_yb) {
      flush_k(cur_yb);
      cur_yb = yb;
    }
    float jr = 0.f, jrc = 0.f, ji = 0.f, jic = 0.f;
    const int y0 = yb * JK_Y;
    // rows past n re-read row n-1 (in bounds) and contribute zero, so every load is unconditional
    int64_t roff[JK_Y];
#pragma unroll
    for (int i = 0; i < JK_Y; ++i) roff[i] = (int64_t)min(y0 + i, n - 1);
    const double* xrows = slab + (int64_t)x * n * n;
    for (int z0 = lane; z0 < n; z0 += 64) {
      double ev[2][JK_Y];
      float4 dyv[2][JK_Y], dxv[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int z = min(z0 + 32 * u, n - 1);
        dxv[u] = __ldg(D4 + (int64_t)x * n + z);
#pragma unroll
        for (int i = 0; i < JK_Y; ++i) {
          ev[u][i] = __ldcs(xrows + roff[i] * n + z);
          dyv[u][i] = __ldg(D4 + roff[i] * n + z);
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const bool zok = z0 + 32 * u < n;
#pragma unroll
        for (int i = 0; i < JK_Y; ++i) {
          float eh, el;
          split_f32pair_fast((zok && y0 + i < n) ? ev[u][i] : 0.0, eh, el);
          df_mac(jr, jrc, eh, el, dyv[u][i].x, dyv[u][i].y);
          df_mac(ji, jic, eh, el, dyv[u][i].z, dyv[u][i].w);
          df_mac(ks[i][0], ks[i][1], eh, el, dxv[u].x, dxv[u].y);
          df_mac(ks[i][2], ks[i][3], eh, el, dxv[u].z, dxv[u].w);
        }
      }
    }
    df_warp_sum(jr, jrc);
    df_warp_sum(ji, jic);
    if (lane == 0) {
      float4 j = Jw[(size_t)w * n + x];
      df_add(j.x, j.y, jr, jrc);
      df_add(j.z, j.w, ji, jic);
      Jw[(size_t)w * n + x] = j;
    }
  }
  if (cur_yb >= 0) flush_k(cur_yb);
  __syncthreads();
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    double Jr = 0, Ji = 0, Kr = 0, Ki = 0;
    for (int v = 0; v < nw; ++v) {
      const float4 j = Jw[(size_t)v * n + p], k = Kw[(size_t)v * n + p];
      Jr += (double)j.x + (double)j.y; Ji += (double)j.z + (double)j.w;
      Kr += (double)k.x + (double)k.y; Ki += (double)k.z + (double)k.w;
    }
    const z64 hv = h ? h[(int64_t)m * n + p] : zmk(0, 0);
    F[(int64_t)m * n + p] = zmk(hv.x + scale * (2.0 * Jr - Kr), hv.y + scale * (2.0 * Ji - Ki));
  }
}

// ---- J/K for ERIs symmetric in their last pair, e[m][x][y][z] = e[m][x][z][y] (real AO
// integrals and their nuclear derivatives are): only z >= y is read.  With S = D + D^T off
// the diagonal and S[y][y] = D[y][y], each integral read adds
//   J[m][x] += e S[y][z],   K[m][y] += e D[x][z],   K[m][z] += e D[x][y] (z > y only),
// the full-tensor sums with the (x, z, y) partner folded in: six double-float multiply-adds
// per pair of integrals instead of eight, half the splits and half the bytes.  Groups of
// JK_Y rows of one x as in jk_df_kernel; the lanes own z = 32 c + lane from the chunk that
// holds the group's first row; the K[z] partials of a group's rows are summed in registers
// and added to the lane's own slot (Kz, never shared between lanes).  Warps take contiguous
// group ranges of equal work: groups further down the triangle have fewer chunks.
__global__ void jk_sym_split_kernel(const z64* __restrict__ D, int n, float4* __restrict__ D4,
                                    float4* __restrict__ S4) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t y = e / n, z = e % n;
    const z64 d = D[e];
    D4[e] = split_z(d);
    S4[e] = split_z(y == z ? d : zadd(d, D[z * n + y]));
  }
}

// Smallest group g whose preceding groups hold at least `target` chunk-units of work.
__device__ int64_t jk_sym_group_at(int64_t target, int n, int nyb, int nch) {
  int64_t cum = 0;
  for (int yb = 0; yb < nyb; ++yb) {
    const int64_t c = nch - (yb * JK_Y) / 32;
    if (cum + c * n >= target) return (int64_t)yb * n + (target - cum + c - 1) / c;
    cum += c * n;
  }
  return (int64_t)nyb * n;
}

__global__ void __launch_bounds__(512) jk_sym_kernel(const double* __restrict__ eri, int n,
                                                     const float4* __restrict__ D4, const float4* __restrict__ S4,
                                                     const z64* __restrict__ h, double scale, z64* __restrict__ F) {
  extern __shared__ float4 jk_sh[];       // Jw, Kw (K[y] per warp), Kz (K[z] per warp): [nw][n] each
  const int nw = blockDim.x >> 5;
  float4* Jw = jk_sh;
  float4* Kw = jk_sh + (size_t)nw * n;
  float4* Kz = jk_sh + (size_t)2 * nw * n;
  const int m = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < 3 * nw * n; i += blockDim.x) jk_sh[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncthreads();
  const int nyb = (n + JK_Y - 1) / JK_Y, nch = (n + 31) / 32;
  int64_t total = 0;
  for (int yb = 0; yb < nyb; ++yb) total += (int64_t)(nch - (yb * JK_Y) / 32) * n;
  const int64_t g0 = jk_sym_group_at(total * w / nw, n, nyb, nch);
  const int64_t g1 = jk_sym_group_at(total * (w + 1) / nw, n, nyb, nch);
  const double* slab = eri + (int64_t)m * n * n * n;
  float ks[JK_Y][4];
#pragma unroll
  for (int i = 0; i < JK_Y; ++i) ks[i][0] = ks[i][1] = ks[i][2] = ks[i][3] = 0.f;
  int cur_yb = g0 < g1 ? (int)(g0 / n) : -1;
  auto flush_k = [&](int yb) {
#pragma unroll
    for (int i = 0; i < JK_Y; ++i) {
      df_warp_sum(ks[i][0], ks[i][1]);
      df_warp_sum(ks[i][2], ks[i][3]);
      const int y = yb * JK_Y + i;
      if (lane == 0 && y < n) {
        float4 k = Kw[(size_t)w * n + y];
        df_add(k.x, k.y, ks[i][0], ks[i][1]);
        df_add(k.z, k.w, ks[i][2], ks[i][3]);
        Kw[(size_t)w * n + y] = k;
      }
      ks[i][0] = ks[i][1] = ks[i][2] = ks[i][3] = 0.f;
    }
  };
  for (int64_t g = g0; g < g1; ++g) {
    const int yb = (int)(g / n), x = (int)(g % n);
    if (yb != cur_yb) {
      flush_k(cur_yb);
      cur_yb = yb;
    }
    const int y0 = yb * JK_Y;
    // rows past n re-read row n-1 (in bounds) and contribute zero, so every load is unconditional
    int64_t roff[JK_Y];
    float4 dxy[JK_Y];
#pragma unroll
    for (int i = 0; i < JK_Y; ++i) {
      roff[i] = (int64_t)min(y0 + i, n - 1);
      dxy[i] = __ldg(D4 + (int64_t)x * n + roff[i]);
    }
    const double* xrows = slab + (int64_t)x * n * n;
    float jr = 0.f, jrc = 0.f, ji = 0.f, jic = 0.f;
    for (int c = y0 / 32; c < nch; ++c) {
      const int z = 32 * c + lane;
      const int zc = min(z, n - 1);
      const float4 dxz = __ldg(D4 + (int64_t)x * n + zc);
      double ev[JK_Y];
      float4 sv[JK_Y];
#pragma unroll
      for (int i = 0; i < JK_Y; ++i) {
        ev[i] = __ldcs(xrows + roff[i] * n + zc);
        sv[i] = __ldg(S4 + roff[i] * n + zc);
      }
      float kzr = 0.f, kzrc = 0.f, kzi = 0.f, kzic = 0.f;
#pragma unroll
      for (int i = 0; i < JK_Y; ++i) {
        const int y = y0 + i;
        float eh, el;
        split_f32pair_fast((z < n && y < n && z >= y) ? ev[i] : 0.0, eh, el);
        df_mac(jr, jrc, eh, el, sv[i].x, sv[i].y);
        df_mac(ji, jic, eh, el, sv[i].z, sv[i].w);
        df_mac(ks[i][0], ks[i][1], eh, el, dxz.x, dxz.y);
        df_mac(ks[i][2], ks[i][3], eh, el, dxz.z, dxz.w);
        const bool off = z > y;
        const float zh = off ? eh : 0.f, zl = off ? el : 0.f;
        df_mac(kzr, kzrc, zh, zl, dxy[i].x, dxy[i].y);
        df_mac(kzi, kzic, zh, zl, dxy[i].z, dxy[i].w);
      }
      if (z < n) {
        float4 k = Kz[(size_t)w * n + z];
        df_add(k.x, k.y, kzr, kzrc);
        df_add(k.z, k.w, kzi, kzic);
        Kz[(size_t)w * n + z] = k;
      }
    }
    df_warp_sum(jr, jrc);
    df_warp_sum(ji, jic);
    if (lane == 0) {
      float4 j = Jw[(size_t)w * n + x];
      df_add(j.x, j.y, jr, jrc);
      df_add(j.z, j.w, ji, jic);
      Jw[(size_t)w * n + x] = j;
    }
  }
  if (cur_yb >= 0) flush_k(cur_yb);
  __syncthreads();
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    double Jr = 0, Ji = 0, Kr = 0, Ki = 0;
    for (int v = 0; v < nw; ++v) {
      const float4 j = Jw[(size_t)v * n + p], k = Kw[(size_t)v * n + p], kz = Kz[(size_t)v * n + p];
      Jr += (double)j.x + (double)j.y; Ji += (double)j.z + (double)j.w;
      Kr += ((double)k.x + (double)k.y) + ((double)kz.x + (double)kz.y);
      Ki += ((double)k.z + (double)k.w) + ((double)kz.z + (double)kz.w);
    }
    const z64 hv = h ? h[(int64_t)m * n + p] : zmk(0, 0);
    F[(int64_t)m * n + p] = zmk(hv.x + scale * (2.0 * Jr - Kr), hv.y + scale * (2.0 * Ji - Ki));
  }
}
// ---- The same (l, s)-symmetric J/K in FP64 (the reference's arithmetic): six DFMAs per
// pair of integrals on the FP64 pipe.  Layout and work split as jk_sym_kernel; the density
// and S = D + D^T (diagonal D) are read as complex FP64.
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void jk_sym_s_kernel(const z64* __restrict__ D, int n, z64* __restrict__ S) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t y = e / n, z = e % n;
    S[e] = y == z ? D[e] : zadd(D[e], D[z * n + y]);
  }
}

__global__ void __launch_bounds__(512) jk_sym64_kernel(const double* __restrict__ eri, int n,
                                                       const z64* __restrict__ D, const z64* __restrict__ S,
                                                       const z64* __restrict__ h, double scale,
                                                       z64* __restrict__ F) {
  extern __shared__ z64 jk_sh64[];        // Jw, Kw, Kz: [nw][n] each
  const int nw = blockDim.x >> 5;
  z64* Jw = jk_sh64;
  z64* Kw = jk_sh64 + (size_t)nw * n;
  z64* Kz = jk_sh64 + (size_t)2 * nw * n;
  const int m = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < 3 * nw * n; i += blockDim.x) jk_sh64[i] = zmk(0, 0);
  __syncthreads();
  const int nyb = (n + JK_Y - 1) / JK_Y, nch = (n + 31) / 32;
  int64_t total = 0;
  for (int yb = 0; yb < nyb; ++yb) total += (int64_t)(nch - (yb * JK_Y) / 32) * n;
  const int64_t g0 = jk_sym_group_at(total * w / nw, n, nyb, nch);
  const int64_t g1 = jk_sym_group_at(total * (w + 1) / nw, n, nyb, nch);
  const double* slab = eri + (int64_t)m * n * n * n;
  double ks[JK_Y][2];
#pragma unroll
  for (int i = 0; i < JK_Y; ++i) ks[i][0] = ks[i][1] = 0.0;
  int cur_yb = g0 < g1 ? (int)(g0 / n) : -1;
  auto flush_k = [&](int yb) {
#pragma unroll
    for (int i = 0; i < JK_Y; ++i) {
      const double kr = warp_sum_d(ks[i][0]), ki = warp_sum_d(ks[i][1]);
      const int y = yb * JK_Y + i;
      if (lane == 0 && y < n) Kw[(size_t)w * n + y] = zadd(Kw[(size_t)w * n + y], zmk(kr, ki));
      ks[i][0] = ks[i][1] = 0.0;
    }
  };
  for (int64_t g = g0; g < g1; ++g) {
    const int yb = (int)(g / n), x = (int)(g % n);
    if (yb != cur_yb) {
      flush_k(cur_yb);
      cur_yb = yb;
    }
    const int y0 = yb * JK_Y;
    int64_t roff[JK_Y];
    z64 dxy[JK_Y];
#pragma unroll
    for (int i = 0; i < JK_Y; ++i) {
      roff[i] = (int64_t)min(y0 + i, n - 1);
      dxy[i] = __ldg(D + (int64_t)x * n + roff[i]);
    }
    const double* xrows = slab + (int64_t)x * n * n;
    double jr = 0.0, ji = 0.0;
    for (int c = y0 / 32; c < nch; ++c) {
      const int z = 32 * c + lane;
      const int zc = min(z, n - 1);
      const z64 dxz = __ldg(D + (int64_t)x * n + zc);
      double ev[JK_Y];
      z64 sv[JK_Y];
#pragma unroll
      for (int i = 0; i < JK_Y; ++i) {
        ev[i] = __ldcs(xrows + roff[i] * n + zc);
        sv[i] = __ldg(S + roff[i] * n + zc);
      }
      double kzr = 0.0, kzi = 0.0;
#pragma unroll
      for (int i = 0; i < JK_Y; ++i) {
        const int y = y0 + i;
        const double e = (z < n && y < n && z >= y) ? ev[i] : 0.0;
        jr = fma(e, sv[i].x, jr);
        ji = fma(e, sv[i].y, ji);
        ks[i][0] = fma(e, dxz.x, ks[i][0]);
        ks[i][1] = fma(e, dxz.y, ks[i][1]);
        const double ez = z > y ? e : 0.0;
        kzr = fma(ez, dxy[i].x, kzr);
        kzi = fma(ez, dxy[i].y, kzi);
      }
      if (z < n) Kz[(size_t)w * n + z] = zadd(Kz[(size_t)w * n + z], zmk(kzr, kzi));
    }
    jr = warp_sum_d(jr);
    ji = warp_sum_d(ji);
    if (lane == 0) Jw[(size_t)w * n + x] = zadd(Jw[(size_t)w * n + x], zmk(jr, ji));
  }
  if (cur_yb >= 0) flush_k(cur_yb);
  __syncthreads();
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    double Jr = 0, Ji = 0, Kr = 0, Ki = 0;
    for (int v = 0; v < nw; ++v) {
      const z64 j = Jw[(size_t)v * n + p], k = Kw[(size_t)v * n + p], kz = Kz[(size_t)v * n + p];
      Jr += j.x; Ji += j.y;
      Kr += k.x + kz.x; Ki += k.y + kz.y;
    }
    const z64 hv = h ? h[(int64_t)m * n + p] : zmk(0, 0);
    F[(int64_t)m * n + p] = zmk(hv.x + scale * (2.0 * Jr - Kr), hv.y + scale * (2.0 * Ji - Ki));
  }
}
}  // namespace

// Complex elements each of the transform's two intermediates must hold: the first
// quarter step writes nbf^3 nmo of them, the second nbf^2 nmo^2, the third nbf nmo^3
// (into the first buffer again); the fourth writes the caller's output.
int64_t ao2mo_intermediate_elems(int64_t nbf, int64_t nmo) {
  const int64_t q1 = nbf * nbf * nbf * nmo, q2 = nbf * nbf * nmo * nmo, q3 = nbf * nmo * nmo * nmo;
  return q1 > q2 ? (q1 > q3 ? q1 : q3) : (q2 > q3 ? q2 : q3);
}
}  // namespace agb

using namespace agb;

extern "C" {

agb_status agb_compute_f_so(const void* F_MO, int64_t n, void* F_SO, void* stream) {
  AGB_ARG_CHECK(F_MO && F_SO && n >= 0, "compute_f_so: bad argument");
  if (n == 0) return AGB_OK;
  f_so_kernel<<<grid_for(4 * n * n, 256), 256, 0, (cudaStream_t)stream>>>((const z64*)F_MO, n, (z64*)F_SO);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

agb_status agb_compute_eri_so(const void* ERI_MO, int64_t n0, int64_t n1, int64_t n2, int64_t n3, void* ERI_SO,
                              void* stream) {
  AGB_ARG_CHECK(ERI_MO && ERI_SO && n0 >= 0 && n1 >= 0 && n2 >= 0 && n3 >= 0, "compute_eri_so: bad argument");
  int64_t total = 16 * n0 * n1 * n2 * n3;
  if (total == 0) return AGB_OK;
  eri_so_kernel<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>((const z64*)ERI_MO, n0, n1, n2, n3,
                                                                        (z64*)ERI_SO);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

agb_status agb_cisd_unpack(agb_cisd_plan* P, const void* t, void* t1, void* t2, void* stream) {
  AGB_ARG_CHECK(P && P->ws && t, "unpack: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (t1 && P->n1) {
    copy_kernel<<<grid_for(P->n1, 256), 256, 0, st>>>((const z64*)t, P->n1, (z64*)t1);
    AGB_LAUNCH_CHECK();
  }
  if (t2) {
    int64_t total = (int64_t)P->o * P->o * P->v * P->v;
    unpack_full_kernel<<<grid_for(total, 256), 256, 0, st>>>((const z64*)t + P->n1, P->o, P->v, P->pv, (z64*)t2);
    AGB_LAUNCH_CHECK();
  }
  return AGB_OK;
}

agb_status agb_cisd_pack(agb_cisd_plan* P, const void* t1, const void* t2, void* t, void* stream) {
  AGB_ARG_CHECK(P && P->ws && t && t2 && (t1 || P->n1 == 0), "pack: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (P->n1) {
    copy_kernel<<<grid_for(P->n1, 256), 256, 0, st>>>((const z64*)t1, P->n1, (z64*)t);
    AGB_LAUNCH_CHECK();
  }
  if (P->n2) {
    pack_kernel<<<grid_for(P->n2, 256), 256, 0, st>>>((const z64*)t2, P->o, P->v, P->po, P->pv, P->opairs, P->vpairs,
                                                      (z64*)t + P->n1);
    AGB_LAUNCH_CHECK();
  }
  return AGB_OK;
}

agb_status agb_mp2_so(agb_cisd_plan* P, void* t, void* E_out, void* partials, size_t partials_bytes, void* stream) {
  AGB_ARG_CHECK(P && P->ws && t && E_out, "mp2_so: bad argument");
  if (!partials || partials_bytes < sizeof(z64) * kMp2Blocks) {
    agb_set_error_message("mp2_so: partials buffer too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (P->n1) {
    AGB_CUDA_TRY(cudaMemsetAsync(t, 0, sizeof(z64) * P->n1, st));
  }
  mp2_kernel<<<kMp2Blocks, 256, 0, st>>>(P->R0p, P->EW + P->n1, P->invD + P->n1, P->n2,
                                         (z64*)t + P->n1, (z64*)partials);
  AGB_LAUNCH_CHECK();
  sum_partials_kernel<<<1, 256, 0, st>>>((const z64*)partials, kMp2Blocks, (z64*)E_out);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

size_t agb_ao2mo_scratch_bytes(int64_t nbf, int64_t nmo, int precision) {
  size_t s = sizeof(z64) * (size_t)agb::ao2mo_intermediate_elems(nbf, nmo);
  s = (s + 255) & ~(size_t)255;
  size_t gs = (size_t)64 << 20;
  // the four quarter steps: rows (n l s), (l s p), (s p q), (p q r); N = nmo, K = nbf
  const int64_t rows[4] = {nbf * nbf * nbf, nbf * nbf * nmo, nbf * nmo * nmo, nmo * nmo * nmo};
  for (int i = 0; i < 4; ++i) {
    size_t need = 0;
    if (precision == AGB_PREC_TF32X3) need = cgemm_tf32x3_scratch(rows[i], nmo, nbf);
    else if (precision == AGB_PREC_DF64) need = dfgemm_scratch_bytes(rows[i], nmo, nbf);
    else if (precision == AGB_PREC_OZAKI) need = ozgemm_scratch_bytes_fused(rows[i], nmo, nbf);   // A sliced once
    if (need > gs) gs = need;
  }
  return 2 * s + sizeof(z64) * (size_t)(nbf * nmo) + 256 + gs + 256;
}

// Each quarter step contracts the leading AO index and appends the new MO index
// last: (m n l s) -> (n l s p) -> (l s p q) -> (s p q r) -> (p q r s).  The
// first step multiplies the real AO integrals by the complex C*: a real GEMM on
// interleaved columns in FP64 mode; in the tensor-core and double-float modes
// the split kernels read the real array directly (imaginary part zero).
agb_status agb_ao2mo(const double* ERI_AO, int64_t nbf, const void* C, int64_t nmo, void* ERI_MO, void* scratch,
                     size_t scratch_bytes, int precision, void* stream) {
  AGB_ARG_CHECK(ERI_AO && C && ERI_MO && nbf > 0 && nmo > 0, "ao2mo: bad argument");
  AGB_ARG_CHECK(precision == AGB_PREC_FP64 || precision == AGB_PREC_TF32X3 || precision == AGB_PREC_DF64 ||
                    precision == AGB_PREC_OZAKI,
                "ao2mo: unknown precision");
  if (!scratch || scratch_bytes < agb_ao2mo_scratch_bytes(nbf, nmo, precision)) {
    agb_set_error_message("ao2mo: scratch too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  size_t s = sizeof(z64) * (size_t)ao2mo_intermediate_elems(nbf, nmo);
  s = (s + 255) & ~(size_t)255;
  char* base = (char*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  z64* Y1 = (z64*)base;
  z64* Y2 = (z64*)(base + s);
  z64* Cc = (z64*)(base + 2 * s);
  char* gs = base + 2 * s + ((sizeof(z64) * nbf * nmo + 255) & ~(size_t)255);
  size_t gs_bytes = scratch_bytes - (size_t)(gs - (char*)scratch);
  if (precision == AGB_PREC_TF32X3 || precision == AGB_PREC_OZAKI)
    AGB_CUDA_TRY(cudaMemsetAsync(gs, 0, 256, st));  // GEMM status word
  conj_kernel<<<grid_for(nbf * nmo, 256), 256, 0, st>>>((const z64*)C, nbf * nmo, Cc);
  AGB_LAUNCH_CHECK();
  // out[(rest)][q] = sum_k T[k][(rest)] Cop[k][q]
  auto step = [&](const z64* T, int64_t Mrest, int kind, const z64* Cop, z64* out) -> agb_status {
    if (precision == AGB_PREC_TF32X3) {
      // outputs up to 256 wide: the GEMM converts the FP64 intermediate itself (no operand planes)
      if (nmo <= 256)
        return cgemm_tf32x3_fa(Mrest, nmo, nbf, zmk(1, 0), T, 1, Mrest, kind, Cop, nmo, 1, 0, zmk(0, 0), out, nmo,
                               gs, gs_bytes, st);
      return cgemm_tf32x3(Mrest, nmo, nbf, zmk(1, 0), T, 1, Mrest, kind, Cop, nmo, 1, 0, zmk(0, 0), out, nmo, gs,
                          gs_bytes, st);
    }
    if (precision == AGB_PREC_DF64)
      return dfgemm_ex(Mrest, nmo, nbf, zmk(1, 0), T, 1, Mrest, kind, Cop, nmo, 1, 0, zmk(0, 0), out, nmo, gs,
                       gs_bytes, st);
    if (precision == AGB_PREC_OZAKI)
      return ozgemm_ex(Mrest, nmo, nbf, zmk(1, 0), T, 1, Mrest, kind, Cop, nmo, 1, 0, zmk(0, 0), out, nmo, gs,
                       gs_bytes, st);
    return zgemm_ex(Mrest, nmo, nbf, zmk(1, 0), T, 1, Mrest, 0, Cop, nmo, 1, 0, zmk(0, 0), out, nmo, gs, gs_bytes,
                    st);
  };
  // step 1: Y1[(n l s)][p] = sum_m (mn|ls) C*[m,p]
  if (precision == AGB_PREC_FP64) {
    int64_t M = nbf * nbf * nbf, N = 2 * nmo, K = nbf;
    dim3 grid((unsigned)((N + DBN - 1) / DBN), (unsigned)((M + DBM - 1) / DBM));
    AGB_ARG_CHECK((M + DBM - 1) / DBM <= 65535, "ao2mo: nbf too large");
    dgemm_kernel<<<grid, 256, 0, st>>>(M, N, K, ERI_AO, 1, M, (const double*)Cc, N, 1, (double*)Y1, N);
    AGB_LAUNCH_CHECK();
  } else {
    AGB_STATUS_TRY(step((const z64*)ERI_AO, nbf * nbf * nbf, kSrcReal, Cc, Y1));
  }
  // step 2: Y2[(l s p)][q] = sum_n Y1[n][(l s p)] C[n,q]
  AGB_STATUS_TRY(step(Y1, nbf * nbf * nmo, 0, (const z64*)C, Y2));
  // step 3: Y1[(s p q)][r] = sum_l Y2[l][(s p q)] C*[l,r]
  AGB_STATUS_TRY(step(Y2, nbf * nmo * nmo, 0, Cc, Y1));
  // step 4: ERI_MO[(p q r)][s] = sum_s' Y1[s'][(p q r)] C[s',s]
  AGB_STATUS_TRY(step(Y1, nmo * nmo * nmo, 0, (const z64*)C, (z64*)ERI_MO));
  return AGB_OK;
}

size_t agb_jk_fock_scratch_bytes(int64_t nbf) { return 2 * sizeof(float4) * (size_t)nbf * (size_t)nbf + 512; }

agb_status agb_jk_fock(const double* ERI_AO, int64_t nbf, const void* D, const void* h, double scale, void* F,
                       void* scratch, size_t scratch_bytes, void* stream) {
  AGB_ARG_CHECK(ERI_AO && D && F && nbf > 0 && nbf < 65536, "jk_fock: bad argument");
  if (!scratch || scratch_bytes < agb_jk_fock_scratch_bytes(nbf)) {
    agb_set_error_message("jk_fock: scratch too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  // 16 warps while their J/K slots fit in shared memory, fewer for large nbf
  int nw = 16;
  while (nw > 1 && (size_t)2 * nw * nbf * sizeof(float4) > 200 * 1024) nw >>= 1;
  const size_t sh = (size_t)2 * nw * nbf * sizeof(float4);
  AGB_ARG_CHECK(sh <= 200 * 1024, "jk_fock: nbf too large for the shared J/K slots");
  float4* D4 = (float4*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  const int64_t nn = nbf * nbf;
  jk_split_kernel<<<grid_for(nn, 256), 256, 0, st>>>((const z64*)D, nn, D4);
  AGB_LAUNCH_CHECK();
  if (sh > 48 * 1024) AGB_CUDA_TRY(cudaFuncSetAttribute(jk_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  jk_df_kernel<<<(unsigned)nbf, 32 * nw, sh, st>>>(ERI_AO, (int)nbf, D4, (const z64*)h, scale, (z64*)F);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

agb_status agb_jk_fock_sym64(const double* ERI_AO, int64_t nbf, const void* D, const void* h, double scale, void* F,
                             void* scratch, size_t scratch_bytes, void* stream) {
  AGB_ARG_CHECK(ERI_AO && D && F && nbf > 0 && nbf < 65536, "jk_fock_sym64: bad argument");
  if (!scratch || scratch_bytes < agb_jk_fock_scratch_bytes(nbf)) {
    agb_set_error_message("jk_fock_sym64: scratch too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int nw = 16;
  while (nw > 1 && (size_t)3 * nw * nbf * sizeof(z64) > 200 * 1024) nw >>= 1;
  const size_t sh = (size_t)3 * nw * nbf * sizeof(z64);
  AGB_ARG_CHECK(sh <= 200 * 1024, "jk_fock_sym64: nbf too large for the shared J/K slots");
  z64* S = (z64*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  jk_sym_s_kernel<<<grid_for(nbf * nbf, 256), 256, 0, st>>>((const z64*)D, (int)nbf, S);
  AGB_LAUNCH_CHECK();
  if (sh > 48 * 1024)
    AGB_CUDA_TRY(cudaFuncSetAttribute(jk_sym64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  jk_sym64_kernel<<<(unsigned)nbf, 32 * nw, sh, st>>>(ERI_AO, (int)nbf, (const z64*)D, S, (const z64*)h, scale,
                                                       (z64*)F);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

agb_status agb_jk_fock_sym(const double* ERI_AO, int64_t nbf, const void* D, const void* h, double scale, void* F,
                           void* scratch, size_t scratch_bytes, void* stream) {
  AGB_ARG_CHECK(ERI_AO && D && F && nbf > 0 && nbf < 65536, "jk_fock_sym: bad argument");
  if (!scratch || scratch_bytes < agb_jk_fock_scratch_bytes(nbf)) {
    agb_set_error_message("jk_fock_sym: scratch too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int nw = 16;
  while (nw > 1 && (size_t)3 * nw * nbf * sizeof(float4) > 200 * 1024) nw >>= 1;
  const size_t sh = (size_t)3 * nw * nbf * sizeof(float4);
  AGB_ARG_CHECK(sh <= 200 * 1024, "jk_fock_sym: nbf too large for the shared J/K slots");
  const size_t plane = ((sizeof(float4) * (size_t)nbf * nbf) + 255) & ~(size_t)255;
  float4* D4 = (float4*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  float4* S4 = (float4*)((char*)D4 + plane);
  jk_sym_split_kernel<<<grid_for(nbf * nbf, 256), 256, 0, st>>>((const z64*)D, (int)nbf, D4, S4);
  AGB_LAUNCH_CHECK();
  if (sh > 48 * 1024)
    AGB_CUDA_TRY(cudaFuncSetAttribute(jk_sym_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  jk_sym_kernel<<<(unsigned)nbf, 32 * nw, sh, st>>>(ERI_AO, (int)nbf, D4, S4, (const z64*)h, scale, (z64*)F);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Closed-shell (spatial-orbital) MP2, apyib/mp2_wfn.py:42-59:
//   t2[i,j,a,b] = <ab|ij> / D_ijab,  E = sum (2 <ij|ab> - <ij|ba>) t2,  <pq|rs> = (pr|qs).
namespace agb {
namespace {
__global__ void __launch_bounds__(256) mp2_spatial_kernel(const z64* __restrict__ g, int64_t n, int no, int nv,
                                                          const double* __restrict__ eps, z64* __restrict__ t2,
                                                          z64* __restrict__ partial) {
  z64 acc = zmk(0, 0);
  const int64_t total = (int64_t)no * no * nv * nv;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int b = (int)(e % nv);
    int64_t r = e / nv;
    int a = (int)(r % nv);
    r /= nv;
    int j = (int)(r % no), i = (int)(r / no);
    int64_t A = no + a, B = no + b;
    z64 ab_ij = g[((A * n + i) * n + B) * n + j];   // (ai|bj)
    z64 ij_ab = g[(((int64_t)i * n + A) * n + j) * n + B];   // (ia|jb)
    z64 ij_ba = g[(((int64_t)i * n + B) * n + j) * n + A];   // (ib|ja)
    double inv = 1.0 / (eps[i] + eps[j] - eps[A] - eps[B]);
    z64 t = zmk(ab_ij.x * inv, ab_ij.y * inv);
    t2[e] = t;
    acc = zadd(acc, zmul(zsub(zscale(ij_ab, 2.0), ij_ba), t));
  }
  __shared__ z64 sh[32];
  acc = warp_sum(acc);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = acc;
  __syncthreads();
  if (w == 0) {
    acc = lane < (int)(blockDim.x >> 5) ? sh[lane] : zmk(0, 0);
    acc = warp_sum(acc);
    if (lane == 0) partial[blockIdx.x] = acc;
  }
}
}  // namespace
}  // namespace agb

extern "C" agb_status agb_mp2_spatial(const void* ERI_MO, int64_t nmo, int64_t no, const double* eps, void* t2,
                                      void* E_out, void* partials, size_t partials_bytes, void* stream) {
  using namespace agb;
  AGB_ARG_CHECK(ERI_MO && eps && t2 && E_out && nmo > 0 && no > 0 && no < nmo, "mp2_spatial: bad argument");
  if (!partials || partials_bytes < sizeof(z64) * kMp2Blocks) {
    agb_set_error_message("mp2_spatial: partials buffer too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  mp2_spatial_kernel<<<kMp2Blocks, 256, 0, st>>>((const z64*)ERI_MO, nmo, (int)no, (int)(nmo - no), eps, (z64*)t2,
                                                 (z64*)partials);
  AGB_LAUNCH_CHECK();
  sum_partials_kernel<<<1, 256, 0, st>>>((const z64*)partials, kMp2Blocks, (z64*)E_out);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}
