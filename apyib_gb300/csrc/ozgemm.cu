// FP64-accurate complex GEMM on the bf16 tensor cores (Ozaki splitting).
//
// Each FP64 row x_r (a row of A, or a column of B) is scaled by 2^-(E_r+1), E_r the
// largest binary exponent in the row, and rounded to a 42-bit fixed-point
// integer X (|x - 2^(E_r+1-42) X| <= 2^(E_r-42)).  X is cut into six balanced
// 7-bit digits, X = sum_s d_s 2^(35-7s) with |d_0| <= 128 and |d_s| <= 64, and
// slice s stores b_s = d_s 2^-7s in bf16 (exact: at most 8 significant bits),
// so x = 2^f_r sum_s b_s with f_r = E_r + 1 - 7 and
//     x_i . y_j = 2^(f_i + f_j) sum_{s,t} b_s c_t .
// The 21 slice pairs with s + t <= 5 are multiplied by tcgen05.mma kind::f16
// (bf16 in, FP32 accumulate); the dropped pairs and the rounding leave
// ~2^-41 of |x_i||y_j| per term.  The sum of group g = s + t is a multiple of
// 2^-7g bounded by 2^14 (g = 0, 1), 2^14 + 2^12 (g = 2) and 2^14 + 2^13 (g = 3)
// units per k, so groups 0..3 are EXACT in FP32 over 512 k (< 2^24 units): they
// accumulate in their own TMEM columns over one 512-k chunk, the epilogue drains
// them into int64 registers (exact) and the next chunk restarts them.  Groups
// 4 and 5 (scale <= 2^-28) share a fifth accumulator over the whole K.  The
// tensor core accumulates in FP32 with truncation (round toward zero), so only
// this small tail may round: group 3 kept in the tail gave 8x the error.
//
// Long K (> 1024): complex operands use three real products (3M): P1 = Re.Re,
// P2 = Im.Im, P3 = (Re+Im).(Re+Im); C = alpha (P1 - P2 + i (P3 - P1 - P2)) + beta C,
// each product's epilogue adding alpha * (1 - i, -1 - i, i)[part] * P into C.
// Short K (<= 1024, e.g. every AO->MO quarter step): the one-pass kernel (ozc_kernel,
// below) shares one exponent between a row's Re and Im parts, accumulates Re C and
// Im C side by side from the four real products and writes C once.
//
// Tiles of the 3M kernel: one CTA per 128x96 output tile (five 96-column accumulators fill 480 of
// TMEM's 512 columns), 2-stage TMA pipeline of 6 A (128 x 32 bf16) and 6 B
// (96 x 32 bf16) slice tiles, 64-byte swizzle, 84 KB per stage; warp 0 loads,
// warp 1 issues the MMAs from one thread, warps 2-9 drain TMEM (two warps per
// lane quadrant, 48 columns each).  Every mbarrier wait is bounded; a timeout
// records an error word at the start of the scratch and the kernel returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "tc05.cuh"

namespace agb {

namespace {
using namespace tc05;

constexpr int OZ_S = 6;                             // slices per operand
constexpr int BM = 128, BN = 96, BK = 32;           // BK in bf16 elements (64 bytes)
constexpr int NACC = 5;                             // exact groups 0..3, tail
constexpr int CHUNK_KB = 16;                        // k-blocks per exact chunk (512 k)
constexpr int STAGES = 2;
constexpr int A_TILE_BYTES = BM * BK * 2;           // 8 KB per A slice tile
constexpr int B_TILE_BYTES = BN * BK * 2;           // 6 KB per B slice tile
constexpr int STAGE_BYTES = OZ_S * (A_TILE_BYTES + B_TILE_BYTES);   // 84 KB
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr int THREADS = 320;
constexpr unsigned TMEM_COLS = 512;                 // G0 | G1 | G2 | G3 | tail, 96 columns each
constexpr int EPI_COLS = BN / 2;                    // columns per epilogue warp
constexpr int kGroupM = 12;

// Instruction descriptor: D = F32, A = B = BF16 (kind::f16), K-major both, N = 96, M = 128.
__host__ __device__ constexpr uint32_t make_idesc_bf16() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// tcgen05.ld of 16 columns without the wait (several loads, then one tcgen05.wait::ld).
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}


struct OzParams {
  int64_t M, N;
  int nkb;                   // k-blocks of BK
  const int* fA;             // per-row scale exponents f_r
  const int* fB;
  z64* C;                    // complex output [M][ldc]
  int64_t ldc;
  z64 coef;                  // C = (use_beta ? beta C : C) + coef * P  (first part: C = coef * P without beta)
  int csx, csy;              // coef.x, coef.y as -1 / 0 / 1 (applied as sign flips), or 2: multiply
  z64 beta;
  int mode;                  // 0: overwrite, 1: beta C + coef P, 2: C + coef P
  int fixed;                 // 1: combine groups and tail in int64 (|sum| < 2^62 for K <= 2^16)
  int* err;
  int64_t rowsA, rowsB;      // padded rows per slice plane
};

// round(t * 2^32) for a float t with |t| < 2^29, by integer instructions.
__device__ __forceinline__ long long f32_fixed32(float t) {
  const unsigned int f = __float_as_uint(t);
  const int ex = (int)((f >> 23) & 0xFFu);
  if (ex == 0) return 0;                                  // zero or subnormal: below 2^-32
  const long long mant = (long long)((f & 0x7FFFFFu) | 0x800000u);
  const int sh = ex - 118;                                // t * 2^32 = mant * 2^(ex - 150 + 32)
  long long r;
  if (sh >= 0) r = mant << sh;
  else if (sh < -25) r = 0;
  else r = (mant + (1ll << (-sh - 1))) >> (-sh);
  return (f >> 31) ? -r : r;
}

// T * 2^e2 rounded to the nearest double (ties to even, subnormal and overflowing results
// included), by integer instructions: GB300 runs FP64 conversions and multiplies on its
// narrow FP64 pipe, which made the FP64 epilogue the bottleneck of short-K products.
__device__ __forceinline__ double i64_ldexp_rn(long long T, int e2) {
  if (T == 0) return 0.0;
  const unsigned long long sgn = T < 0 ? (1ull << 63) : 0ull;
  const unsigned long long a = T < 0 ? 0ull - (unsigned long long)T : (unsigned long long)T;
  const int lz = __clzll((long long)a);
  const unsigned long long m = a << lz;                   // leading one at bit 63
  const int E = 1086 - lz + e2;                           // biased exponent of (m >> 11) * 2^(11 - lz + e2)
  unsigned long long bits;
  if (E >= 1) {
    unsigned long long mant = m >> 11;                    // 53 bits with the leading one
    const unsigned long long rem = m & 0x7FFull;
    mant += (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
    // (E - 1) << 52 plus the mantissa with its leading one: a carry out of rounding bumps E
    // (to the infinity pattern from E = 2046)
    bits = E >= 2047 ? (0x7FFull << 52) : (((unsigned long long)(E - 1)) << 52) + mant;
  } else {
    // subnormal: m * 2^-sh units of 2^-1074, rounded once
    const int sh = 12 - E;
    if (sh > 64) {
      bits = 0;
    } else if (sh == 64) {
      bits = m > (1ull << 63) ? 1ull : 0ull;
    } else {
      unsigned long long q = m >> sh;
      const unsigned long long r = m & ((1ull << sh) - 1), half = 1ull << (sh - 1);
      q += (r > half || (r == half && (q & 1ull))) ? 1ull : 0ull;
      bits = q;
    }
  }
  return __longlong_as_double((long long)(bits | sgn));
}

// c * v for a coefficient component c in {-1, 0, 1} (cs = c) by a sign flip, else a multiply.
__device__ __forceinline__ double coef_mul(int cs, double c, double v) {
  if (cs == 0) return 0.0;
  if (cs == 1) return v;
  if (cs == -1) return __longlong_as_double(__double_as_longlong(v) ^ (1ll << 63));
  return c * v;
}

__global__ void __launch_bounds__(THREADS, 1)
ozgemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, OzParams p) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full_bar = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty_bar = full_bar + STAGES;
  uint64_t* chunk_bar = empty_bar + STAGES;   // MMA -> epilogue: the chunk's MMAs completed
  uint64_t* drained_bar = chunk_bar + 1;      // epilogue -> MMA: exact accumulators read (8 warps)
  uint32_t* tmem_slot = (uint32_t*)(drained_bar + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntn = gridDim.x, ntm = gridDim.y;
  const int lin = blockIdx.y * ntn + blockIdx.x;
  const int gsz = kGroupM * ntn;
  const int first_m = (lin / gsz) * kGroupM;
  const int gm = min(ntm - first_m, kGroupM);
  const int tile_m = first_m + (lin % gsz) % gm;
  const int tile_n = (lin % gsz) / gm;
  const int nk = p.nkb;
  const int nchunks = (nk + CHUNK_KB - 1) / CHUNK_KB;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(chunk_bar, 1);
    mbar_init(drained_bar, 8);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int kb = 0; kb < nk; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
        if (!mbar_wait(&empty_bar[s], ph ^ 1u, p.err, abort_flag, 1)) break;
        uint8_t* st = smem + s * STAGE_BYTES;
        mbar_expect_tx(&full_bar[s], STAGE_BYTES);
        const int kx = kb * BK;
        for (int sl = 0; sl < OZ_S; ++sl) {
          tma_load_2d(st + sl * A_TILE_BYTES, &mapA, &full_bar[s], kx, (int)(sl * p.rowsA + tile_m * BM));
          tma_load_2d(st + OZ_S * A_TILE_BYTES + sl * B_TILE_BYTES, &mapB, &full_bar[s], kx,
                      (int)(sl * p.rowsB + tile_n * BN));
        }
        issued = kb + 1;
      }
      if (*abort_flag) {
        for (int kb = (issued > STAGES ? issued - STAGES : 0); kb < issued; ++kb) {
          long long t0 = clock64();
          while (!mbar_try_wait(&full_bar[kb % STAGES], (uint32_t)(kb / STAGES) & 1u) &&
                 clock64() - t0 < kWaitCycles) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = make_idesc_bf16();
      for (int kb = 0; kb < nk; ++kb) {
        const int kc = kb % CHUNK_KB, chunk = kb / CHUNK_KB;
        if (kc == 0 && chunk > 0) {
          // the epilogue must have read the previous chunk's exact accumulators
          if (!mbar_wait(drained_bar, (uint32_t)(chunk - 1) & 1u, p.err, abort_flag, 4)) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        const int s = kb % STAGES;
        const uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, p.err, abort_flag, 2)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // descriptors of the stage's first A tile; the others differ only in the start-address
        // field (byte offset / 16; no carry out of the 14-bit field within a 227 KB window)
        const uint64_t d0 = make_desc(smem_u32(smem + s * STAGE_BYTES));
#pragma unroll
        for (int ks = 0; ks < BK / 16; ++ks) {
#pragma unroll
          for (int sa = 0; sa < OZ_S; ++sa) {
#pragma unroll
            for (int tb = 0; tb + sa < OZ_S; ++tb) {
              const int g = sa + tb;
              const int d = g < NACC - 1 ? g : NACC - 1;
              const uint64_t a = d0 + (uint64_t)((sa * A_TILE_BYTES + ks * 32) >> 4);
              const uint64_t b = d0 + (uint64_t)((OZ_S * A_TILE_BYTES + tb * B_TILE_BYTES + ks * 32) >> 4);
              // first write of an exact group in a chunk, or of the tail in the whole K, overwrites
              const bool first =
                  sa == 0 && ks == 0 && ((g < NACC - 1 && kc == 0) || (g == NACC - 1 && kb == 0));
              mma_bf16(tmem_base + (uint32_t)(d * BN), a, b, idesc, first ? 0u : 1u);
            }
          }
        }
        mma_commit(&empty_bar[s]);
        if (kc == CHUNK_KB - 1 || kb == nk - 1) mma_commit(chunk_bar);
      }
    }
  } else {
    // epilogue: warps 2..9; TMEM lane quadrant q = warp % 4, column half h
    const int q = warp & 3, h = (warp - 2) >> 2;
    const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * EPI_COLS);
    long long acc[EPI_COLS];   // sum of the exact groups in units of 2^-21
#pragma unroll
    for (int j = 0; j < EPI_COLS; ++j) acc[j] = 0;
    bool ok = nk > 0;
    for (int c = 0; c < nchunks && ok; ++c) {
      int okw = 0;
      if (lane == 0) okw = mbar_wait(chunk_bar, (uint32_t)c & 1u, p.err, abort_flag, 3) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, okw, 0) != 0;
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int c4 = 0; c4 < EPI_COLS / 16; ++c4) {
        uint32_t g0[16], g1[16], g2[16], g3[16];
        tmem_ld16_async(lane_base + c4 * 16, g0);
        tmem_ld16_async(lane_base + BN + c4 * 16, g1);
        tmem_ld16_async(lane_base + 2 * BN + c4 * 16, g2);
        tmem_ld16_async(lane_base + 3 * BN + c4 * 16, g3);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const long long i0 = __float2int_rn(__uint_as_float(g0[j]));
          const long long i1 = __float2int_rn(__uint_as_float(g1[j]) * 128.0f);
          const long long i2 = __float2int_rn(__uint_as_float(g2[j]) * 16384.0f);
          const long long i3 = __float2int_rn(__uint_as_float(g3[j]) * 2097152.0f);
          acc[c4 * 16 + j] += (i0 << 21) + (i1 << 14) + (i2 << 7) + i3;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(drained_bar);
    }
    if (ok) {
      const int64_t m = (int64_t)tile_m * BM + q * 32 + lane;
      const int64_t n0 = (int64_t)tile_n * BN + h * EPI_COLS;
      const int fa = m < p.M ? p.fA[m] : 0;
#pragma unroll
      for (int c4 = 0; c4 < EPI_COLS / 16; ++c4) {
        float tl[16];
        tmem_ld16(lane_base + (NACC - 1) * BN + c4 * 16, tl);
        if (m < p.M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int64_t n = n0 + c4 * 16 + j;
            if (n < p.N) {
              double v;
              if (p.fixed) {
                // exact groups (units 2^-21) and the FP32 tail in units of 2^-32, one rounding
                const long long T = (acc[c4 * 16 + j] << 11) + f32_fixed32(tl[j]);
                v = i64_ldexp_rn(T, fa + p.fB[n] - 32);
              } else {
                // 2^(fa + fb) as a double built from its exponent field
                const double sc = __longlong_as_double((long long)(fa + p.fB[n] + 1023) << 52);
                v = ((double)acc[c4 * 16 + j] * 4.76837158203125e-07 + (double)tl[j]) * sc;   // I 2^-21 + tail
              }
              z64* c = p.C + m * p.ldc + n;
              z64 out = zmk(coef_mul(p.csx, p.coef.x, v), coef_mul(p.csy, p.coef.y, v));
              if (p.mode == 1) out = zadd(out, zmul(p.beta, *c));
              else if (p.mode == 2) out = zadd(out, *c);
              *c = out;
            }
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TMEM_COLS));
  }
}

// (Re, Im) of X(r, k) = src[r*s_row + k*s_k]; conj == 1 negates Im, conj == kSrcReal reads a real array.
__device__ __forceinline__ z64 oz_load(const z64* src, int64_t off, int conj) {
  if (conj == kSrcReal) return zmk(((const double*)src)[off], 0.0);
  const z64 v = src[off];
  return zmk(v.x, conj == 1 ? -v.y : v.y);
}

// Part `part` (0 Re, 1 Im, 2 Re + Im) of a loaded value.
__device__ __forceinline__ double oz_part(z64 v, int part) { return part == 0 ? v.x : (part == 1 ? v.y : v.x + v.y); }

__device__ __forceinline__ int oz_bexp(double v) { return (__double2hiint(v) >> 20) & 0x7ff; }

// Largest biased FP64 exponent per row of NP parts (part0, ...), from one read of the
// source; emax[p * estride + r] must start at zero.
template <int NP>
__global__ void oz_rowexp_kernel(const z64* __restrict__ src, int64_t rows, int64_t K, int64_t s_row, int64_t s_k,
                                 int conj, int part0, int64_t estride, int* __restrict__ emax) {
  __shared__ int tile[NP][32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool kfast = (s_k == 1) || (s_row != 1 && s_k <= s_row);
  const int64_t tiles_k = (K + 31) / 32, tiles = ((rows + 31) / 32) * tiles_k;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t r0 = (t / tiles_k) * 32, k0 = (t % tiles_k) * 32;
    for (int i = ty; i < 32; i += 8) {
      int64_t r, k;
      if (kfast) { r = r0 + i; k = k0 + tx; } else { r = r0 + tx; k = k0 + i; }
      z64 v = zmk(0.0, 0.0);
      if (r < rows && k < K) v = oz_load(src, r * s_row + k * s_k, conj);
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const int e = oz_bexp(oz_part(v, part0 + q));
        if (kfast) tile[q][i][tx] = e; else tile[q][tx][i] = e;
      }
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        int e = tile[q][i][tx];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
        if (tx == 0 && r0 + i < rows && e > 0) atomicMax(&emax[q * estride + r0 + i], e);
      }
    }
    __syncthreads();
  }
}

// bf16 bits of d * 2^-7s (exact: |d| <= 128).
__device__ __forceinline__ uint16_t oz_digit_bf16(long long d, float scale) {
  const float f = __fsub_rn(__int_as_float(0x4B400000 + (int)d), 12582912.0f);   // exactly d
  return (uint16_t)(__float_as_uint(__fmul_rn(f, scale)) >> 16);
}

// The OZ_S bf16 slices of v under the row's biased exponent eb (0: a zero row): v 2^-f,
// f = eb - 1023 + 1 - 7, rounded to the nearest integer X (|X| <= 2^42), split into
// balanced base-2^7 digits d_s; slice s is d_s 2^-7s, exact in bf16.
__device__ __forceinline__ void oz_digits(double v, int eb, uint16_t (&out)[OZ_S]) {
  const uint32_t hw = (uint32_t)__double2hiint(v), lw = (uint32_t)__double2loint(v);
  const int ex = (int)((hw >> 20) & 0x7ffu);
  long long X = 0;
  const int shift = 11 + (eb - ex);
  if (ex > 0 && eb > 0 && shift < 64) {
    const unsigned long long M = ((unsigned long long)(hw & 0xfffffu) << 32 | lw) | (1ull << 52);
    X = (long long)((M + (1ull << (shift - 1))) >> shift);   // nearest (|X| <= 2^42 keeps |d_0| <= 128)
    if (hw >> 31) X = -X;
  }
  long long d[OZ_S];
#pragma unroll
  for (int s = 0; s < OZ_S - 1; ++s) {
    const int sh = 35 - 7 * s;
    d[s] = (X + (1ll << (sh - 1))) >> sh;
    X -= d[s] << sh;
  }
  d[OZ_S - 1] = X;
  float sc = 1.0f;
#pragma unroll
  for (int s = 0; s < OZ_S; ++s) {
    out[s] = oz_digit_bf16(d[s], sc);
    sc *= 0.0078125f;   // 2^-7
  }
}

// Slices [OZ_S][rows_pad][Kp] (bf16, K-major, zero padded) and row scale exponents f_r of
// NP parts from one read of the source: part q's slices start at slices + q * OZ_S * rows_pad * Kp,
// its exponents at emax / fexp + q * estride (estride 0: one exponent shared by the parts).
template <int NP>
__global__ void oz_slice_kernel(const z64* __restrict__ src, int64_t rows, int64_t K, int64_t s_row, int64_t s_k,
                                int conj, int part0, int64_t rows_pad, int64_t Kp, int64_t estride,
                                const int* __restrict__ emax, int* __restrict__ fexp, uint16_t* __restrict__ slices) {
  __shared__ z64 tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool kfast = (s_k == 1) || (s_row != 1 && s_k <= s_row);
  const int64_t tiles_k = Kp / 32, tiles = (rows_pad / 32) * tiles_k;
  const int64_t plane = rows_pad * Kp;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t r0 = (t / tiles_k) * 32, k0 = (t % tiles_k) * 32;
    for (int i = ty; i < 32; i += 8) {
      int64_t r, k;
      if (kfast) { r = r0 + i; k = k0 + tx; } else { r = r0 + tx; k = k0 + i; }
      z64 v = zmk(0.0, 0.0);
      if (r < rows && k < K) v = oz_load(src, r * s_row + k * s_k, conj);
      if (kfast) tile[i][tx] = v; else tile[tx][i] = v;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
      const int64_t r = r0 + i, k = k0 + tx;
      const z64 vz = tile[i][tx];
#pragma unroll 1
      for (int q = 0; q < NP; ++q) {
        const int eb = r < rows ? emax[q * estride + r] : 0;
        if (k0 == 0 && tx == 0 && r < rows_pad) fexp[q * estride + r] = eb > 0 ? eb - 1023 + 1 - 7 : 0;
        uint16_t dg[OZ_S];
        oz_digits(oz_part(vz, part0 + q), eb, dg);
        uint16_t* dst = slices + (int64_t)q * OZ_S * plane + r * Kp + k;
#pragma unroll
        for (int s = 0; s < OZ_S; ++s) dst[s * plane] = dg[s];
      }
    }
    __syncthreads();
  }
}

// Slices of NP parts in the one-pass kernel's layout: each plane [Kp / 16][rows_pad][16],
// the two 16-byte halves of a row's 32 bytes swapped on rows r with (r >> 2) & 1 (the MMA's
// 32-byte swizzle), so a block of rows of one 16-k block is one contiguous run that lands in
// shared memory ready to use.  64-row x 32-k tiles are staged in shared memory (read along
// k or along rows, whichever is contiguous); each thread then converts 8 consecutive k of
// one row and writes them to each plane as one 16-byte store, a warp covering 16 rows x 32
// bytes of one k-block (512 contiguous bytes per plane).
template <int NP>
__global__ void __launch_bounds__(256) oz_slice_kblk_kernel(const z64* __restrict__ src, int64_t rows, int64_t K,
                                                            int64_t s_row, int64_t s_k, int conj, int part0,
                                                            int64_t rows_pad, int64_t Kp, int64_t estride,
                                                            const int* __restrict__ emax, int* __restrict__ fexp,
                                                            uint16_t* __restrict__ slices) {
  __shared__ z64 tile[64][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool kfast = (s_k == 1) || (s_row != 1 && s_k <= s_row);
  const int64_t tiles_k = Kp / 32, tiles = ((rows_pad + 63) / 64) * tiles_k;
  const int64_t plane = rows_pad * Kp;
  // conversion task of this thread: row rl of the tile, 8-k chunk c (warps 0..3 the first
  // k-block of the tile, 4..7 the second; a lane pair shares a row)
  const int rl = (ty & 3) * 16 + (tx >> 1), c = ((ty >> 2) << 1) | (tx & 1);
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t r0 = (t / tiles_k) * 64, k0 = (t % tiles_k) * 32;
    for (int i = ty; i < 64; i += 8) {
      int rr, kk;
      if (kfast) { rr = i; kk = tx; } else { rr = tx + ((i >> 5) << 5); kk = i & 31; }
      const int64_t r = r0 + rr, k = k0 + kk;
      tile[rr][kk] = (r < rows && k < K) ? oz_load(src, r * s_row + k * s_k, conj) : zmk(0.0, 0.0);
    }
    __syncthreads();
    const int64_t r = r0 + rl;
    if (r < rows_pad) {
      const int64_t kb = (k0 >> 4) + (c >> 1);
      const int64_t off = (kb * rows_pad + r) * 16 + (((c & 1) ^ (int)((r >> 2) & 1)) << 3);
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const int eb = r < rows ? emax[q * estride + r] : 0;
        if (k0 == 0 && c == 0) fexp[q * estride + r] = eb > 0 ? eb - 1023 + 1 - 7 : 0;
        uint32_t w[OZ_S][4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          uint16_t lo[OZ_S], hi[OZ_S];
          oz_digits(oz_part(tile[rl][c * 8 + j], part0 + q), eb, lo);
          oz_digits(oz_part(tile[rl][c * 8 + j + 1], part0 + q), eb, hi);
#pragma unroll
          for (int s2 = 0; s2 < OZ_S; ++s2) w[s2][j >> 1] = (uint32_t)lo[s2] | ((uint32_t)hi[s2] << 16);
        }
#pragma unroll
        for (int s2 = 0; s2 < OZ_S; ++s2)
          *(uint4*)(slices + (int64_t)(q * OZ_S + s2) * plane + off) = make_uint4(w[s2][0], w[s2][1], w[s2][2],
                                                                                  w[s2][3]);
      }
    }
    __syncthreads();
  }
}

// K (padded) up to which the one-pass kernel's operands are sliced in one read: 32 whole
// rows fit in shared memory (32 x 193 x 16 bytes at most).
constexpr int64_t kOzFusedMaxK = 192;

// Row exponents and slices of NP parts in one read of the source, for short K, in the
// layout of oz_slice_kblk_kernel: a block stages 32 whole rows (all Kp k) in shared memory,
// takes each row's largest exponent over its parts (one exponent shared by them; the row
// scale f_r goes to fexp), then converts 8 consecutive k of a row per thread and writes
// each plane with one 16-byte store.  Against a separate exponent pass this saves one
// read of the operand.
template <int NP>
__global__ void __launch_bounds__(256) oz_slice_fused_kernel(const z64* __restrict__ src, int64_t rows, int64_t K,
                                                             int64_t s_row, int64_t s_k, int conj, int64_t rows_pad,
                                                             int64_t Kp, int* __restrict__ fexp,
                                                             uint16_t* __restrict__ slices) {
  extern __shared__ __align__(16) uint8_t fused_smem[];
  z64* rowbuf = (z64*)fused_smem;                       // [32][Kp + 1]
  __shared__ int rexp[32];
  const int kp = (int)Kp, ld = kp + 1;
  const bool kfast = (s_k == 1) || (s_row != 1 && s_k <= s_row);
  const int64_t blocks = rows_pad / 32, plane = rows_pad * Kp;
  const int ntask = 32 * (kp / 8);                       // (row, 8-k chunk) pairs of a block
  for (int64_t b = blockIdx.x; b < blocks; b += gridDim.x) {
    const int64_t r0 = b * 32;
    for (int idx = threadIdx.x; idx < 32 * kp; idx += 256) {
      int rr, kk;
      if (kfast) {
        rr = idx / kp;
        kk = idx - rr * kp;
      } else {
        kk = idx >> 5;
        rr = idx & 31;
      }
      const int64_t r = r0 + rr;
      rowbuf[rr * ld + kk] = (r < rows && kk < K) ? oz_load(src, r * s_row + kk * s_k, conj) : zmk(0.0, 0.0);
    }
    __syncthreads();
    {
      // largest biased exponent of each row over its parts: 8 lanes per row
      const int rr = threadIdx.x >> 3, part = threadIdx.x & 7;
      int e = 0;
      for (int kk = part; kk < kp; kk += 8) {
        const z64 v = rowbuf[rr * ld + kk];
#pragma unroll
        for (int q = 0; q < NP; ++q) e = max(e, oz_bexp(oz_part(v, q)));
      }
      e = max(e, __shfl_xor_sync(0xffffffffu, e, 1));
      e = max(e, __shfl_xor_sync(0xffffffffu, e, 2));
      e = max(e, __shfl_xor_sync(0xffffffffu, e, 4));
      if (part == 0) {
        rexp[rr] = r0 + rr < rows ? e : 0;
        fexp[r0 + rr] = (r0 + rr < rows && e > 0) ? e - 1023 + 1 - 7 : 0;
      }
    }
    __syncthreads();
    // task t: k-block t / 64, row (t % 64) / 2, 8-k half t % 2 of the block, so a warp
    // writes 16 rows x 32 bytes of one k-block per plane
    for (int t = threadIdx.x; t < ntask; t += 256) {
      const int kb = t >> 6, rr = (t & 63) >> 1, hh = t & 1;
      const int64_t r = r0 + rr;
      const int eb = rexp[rr];
      const int64_t off = ((int64_t)kb * rows_pad + r) * 16 + ((hh ^ (int)((r >> 2) & 1)) << 3);
      const z64* x = rowbuf + rr * ld + kb * 16 + hh * 8;
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        uint32_t w[OZ_S][4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          uint16_t lo[OZ_S], hi[OZ_S];
          oz_digits(oz_part(x[j], q), eb, lo);
          oz_digits(oz_part(x[j + 1], q), eb, hi);
#pragma unroll
          for (int s2 = 0; s2 < OZ_S; ++s2) w[s2][j >> 1] = (uint32_t)lo[s2] | ((uint32_t)hi[s2] << 16);
        }
#pragma unroll
        for (int s2 = 0; s2 < OZ_S; ++s2)
          *(uint4*)(slices + (int64_t)(q * OZ_S + s2) * plane + off) = make_uint4(w[s2][0], w[s2][1], w[s2][2],
                                                                                  w[s2][3]);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// One-pass complex Ozaki GEMM for short K (4M, Re and Im accumulated side by side).
//
// Rows of A and columns of B are sliced with one exponent shared by their Re and Im
// parts, so the four real products Re.Re, Im.Im, Re.Im and Im.Re are sums in the same
// fixed-point units: Re C = Re.Re - Im.Im accumulates in one set of TMEM columns (the
// Im.Im MMAs negate A) and Im C = Re.Im + Im.Re in another.  Each set is the 3M kernel's
// five accumulators (exact groups 0..3 and the tail); two products per accumulator
// double the group bounds (group 3: 2 (2^14 + 2^13) units per k), so the exact chunk is
// 256 k (< 2^24 units).  The tile is 128 x 48 outputs: 2 sets x 5 x 48 = 480 TMEM
// columns, the widest tile that fits.  The epilogue turns the int64 group sums and the
// tail into FP64 with integer instructions and writes C once: no read-modify-write of C
// between products and no FP64 arithmetic when alpha = 1 and beta = 0.  A real A (the
// first AO->MO quarter step) has no Im slices and runs the Re.Re and Re.Im products
// only.
namespace ozc {
constexpr int BM = 128, BN = 48, BK = 16;            // BK in bf16 elements (32-byte rows)
constexpr int NSL = 2 * OZ_S;                         // slice tiles per operand: Re 0..5, Im 6..11
constexpr int A_TILE = BM * BK * 2;                   // 4 KB
constexpr int B_TILE = BN * BK * 2;                   // 1.5 KB
constexpr int STAGE_BYTES = NSL * (A_TILE + B_TILE);  // 66 KB
constexpr int STAGES = 3;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr int THREADS = 448;                          // load warp, MMA warp, 12 epilogue warps
constexpr unsigned TMEM_COLS = 512;                   // Re G0..G3 T | Im G0..G3 T, 48 columns each (480 used)
constexpr int CHUNK_KB = 16;                          // k-blocks per exact chunk (256 k)
constexpr int EPI_COLS = BN / 3;                      // columns per epilogue warp (two groups of 8)
}  // namespace ozc

// tcgen05.ld of 8 columns without the wait.
__device__ __forceinline__ void tmem_ld8_async(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

// Exact group sums g0..g3 (FP32, units 1, 2^-7, 2^-14, 2^-21) as one integer in units of 2^-21.
__device__ __forceinline__ long long oz_groups(uint32_t g0, uint32_t g1, uint32_t g2, uint32_t g3) {
  const long long i0 = __float2int_rn(__uint_as_float(g0));
  const long long i1 = __float2int_rn(__uint_as_float(g1) * 128.0f);
  const long long i2 = __float2int_rn(__uint_as_float(g2) * 16384.0f);
  const long long i3 = __float2int_rn(__uint_as_float(g3) * 2097152.0f);
  return (i0 << 21) + (i1 << 14) + (i2 << 7) + i3;
}

// Exact sum I (units 2^-21) plus the FP32 tail t, as an integer in units of 2^-32:
// t 2^21 = u_hi + u_lo with u_hi = rint(t 2^21) (both exact in FP32), then u_lo 2^11 is
// rounded once, as round(t 2^32) would be.  Needs |t| < 2^9.
__device__ __forceinline__ long long oz_fixed32(long long I, float t) {
  const float u = t * 2097152.0f;
  const float uh = rintf(u);
  return ((I + (long long)__float2int_rn(uh)) << 11) + (long long)__float2int_rn((u - uh) * 2048.0f);
}

// T * 2^e2 to the nearest double for e2 in [-1022, 960] (then every |T| < 2^63 gives a
// normal double): the branch-free part of i64_ldexp_rn.
__device__ __forceinline__ double i64_ldexp_normal(long long T, int e2) {
  const unsigned long long sgn = T < 0 ? (1ull << 63) : 0ull;
  const unsigned long long a = T < 0 ? 0ull - (unsigned long long)T : (unsigned long long)T;
  const int lz = __clzll((long long)a);
  const unsigned long long m = a << (lz & 63);
  unsigned long long mant = m >> 11;
  const unsigned long long rem = m & 0x7FFull;
  mant += (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
  const unsigned long long bits = (((unsigned long long)(1085 - lz + e2)) << 52) + mant;
  return __longlong_as_double((long long)(a == 0 ? 0ull : (bits | sgn)));
}

// tcgen05 shared-memory descriptor: K-major, 32-byte swizzle, 8-row groups 256 B apart.
__device__ __forceinline__ uint64_t make_desc_sw32(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(256 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)6 << 61;
  return d;
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, K-major both, M = 128, N = n (a
// multiple of 16, at most ozc::BN), optional -A.
__host__ __device__ constexpr uint32_t make_idesc_ozc(bool negA, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((negA ? 1u : 0u) << 13) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(ozc::BM >> 4) << 24);
}

struct OzcParams {
  int64_t M, N;
  int nkb;                   // k-blocks of ozc::BK
  int a_parts;               // 2, or 1 for a real A (no Im slices)
  int W;                     // column tile width: a multiple of 16, at most ozc::BN
  int ntn;                   // column tiles
  int64_t ntiles;            // row tiles x column tiles
  const uint16_t* sA;        // A slices [a_parts * 6][nkb][rowsA][16], each 32-byte row swizzled
  const uint16_t* sB;        // B slices [12][nkb][rowsB][16]
  const int* fA;             // per-row scale exponents of A (shared by Re and Im)
  const int* fB;             // per-column scale exponents of B
  z64* C;
  int64_t ldc;
  z64 alpha, beta;
  int plain;                 // alpha == 1 and beta == 0
  int* err;
  int64_t rowsA, rowsB;      // padded rows per slice plane
};

// MMA columns of column tile tn: W, or the rest of N rounded up to the MMA's 16.
__device__ __forceinline__ int ozc_tile_width(int64_t N, int W, int tn) {
  const int64_t rest = N - (int64_t)tn * W;
  return rest >= W ? W : (int)((rest + 15) & ~(int64_t)15);
}

// Persistent: each CTA takes tiles blockIdx.x, + gridDim.x, ... (the column tiles of a row
// tile adjacent, so the CTAs running at once share their A slices through L2).  Warp 0
// copies k-blocks of slices (contiguous runs, one bulk copy per plane) into a ring of
// stages that runs across tiles; warp 1 issues the MMAs; warps 2..13 read the accumulators
// into registers, release TMEM to the next tile's MMAs and only then convert and store,
// so a tile's epilogue overlaps the next tile's MMAs.
//
// A tile of width wn keeps its ten accumulators wn columns apart in TMEM and its B slice
// tiles wn rows apart in the stage, so the exact groups sa..3 and the tail of one A slice
// sa are one MMA against B slices 0..4-sa side by side (N = (5 - sa) wn), and the g = 5
// pair (sa, 5 - sa) a second one into the tail: 11 MMAs per product instead of one per
// slice pair (21).  Each MMA reads its A slice from shared memory once; the narrow ones
// cost about as much as the wide ones, so fewer, wider MMAs are faster.
__global__ void __launch_bounds__(ozc::THREADS, 1) ozc_kernel(OzcParams p) {
  constexpr int STAGES = ozc::STAGES, STAGE_BYTES = ozc::STAGE_BYTES, A_TILE = ozc::A_TILE, B_TILE = ozc::B_TILE;
  constexpr int CBM = ozc::BM, CBN = ozc::BN, CBK = ozc::BK, NSL = ozc::NSL, EPI = ozc::EPI_COLS;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full_bar = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty_bar = full_bar + STAGES;
  uint64_t* chunk_bar = empty_bar + STAGES;   // MMA -> epilogue: the chunk's MMAs completed
  uint64_t* drained_bar = chunk_bar + 1;      // epilogue -> MMA: the chunk's accumulators read (12 warps)
  uint64_t* done_bar = drained_bar + 1;       // MMA issuer, on abort: its MMAs completed
  uint32_t* tmem_slot = (uint32_t*)(done_bar + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = p.nkb;
  const int nchunks = (nk + ozc::CHUNK_KB - 1) / ozc::CHUNK_KB;
  const int na = p.a_parts;
  const int64_t tile0 = blockIdx.x, tstep = gridDim.x;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(chunk_bar, 1);
    mbar_init(drained_bar, 12);
    mbar_init(done_bar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(ozc::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      long long issued = 0;   // k-blocks whose copies were issued (the stage ring runs across tiles)
      bool ok = true;
      for (int64_t t = tile0; t < p.ntiles && ok; t += tstep) {
        const int64_t tm = t / p.ntn;
        const int tn = (int)(t % p.ntn);
        const uint32_t bbytes = (uint32_t)ozc_tile_width(p.N, p.W, tn) * CBK * 2;
        const uint32_t bytes = (uint32_t)(na * OZ_S * A_TILE) + (uint32_t)NSL * bbytes;
        const uint16_t* a0 = p.sA + tm * CBM * CBK;
        const uint16_t* b0 = p.sB + (int64_t)tn * p.W * CBK;
        for (int kb = 0; kb < nk; ++kb) {
          const int s = (int)(issued % STAGES);
          const uint32_t ph = (uint32_t)(issued / STAGES) & 1u;
          if (!mbar_wait(&empty_bar[s], ph ^ 1u, p.err, abort_flag, 1)) {
            ok = false;
            break;
          }
          uint8_t* st = smem + s * STAGE_BYTES;
          mbar_expect_tx(&full_bar[s], bytes);
          for (int q = 0; q < na * OZ_S; ++q)
            bulk_load(st + q * A_TILE, a0 + ((int64_t)q * nk + kb) * p.rowsA * CBK, (uint32_t)A_TILE, &full_bar[s]);
          // B slice tiles of this tile's width, packed wn rows apart
          for (int q = 0; q < NSL; ++q)
            bulk_load(st + NSL * A_TILE + q * bbytes, b0 + ((int64_t)q * nk + kb) * p.rowsB * CBK, bbytes,
                      &full_bar[s]);
          ++issued;
        }
      }
      if (!ok) {
        // let the copies in flight land before the CTA exits
        for (long long i = (issued > STAGES ? issued - STAGES : 0); i < issued; ++i) {
          long long t0 = clock64();
          while (!mbar_try_wait(&full_bar[i % STAGES], (uint32_t)(i / STAGES) & 1u) && clock64() - t0 < kWaitCycles) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      long long used = 0;   // k-blocks consumed
      long long chunks = 0;  // chunks committed
      bool ok = true;
      for (int64_t t = tile0; t < p.ntiles && ok; t += tstep) {
        const int wn = ozc_tile_width(p.N, p.W, (int)(t % p.ntn));
        for (int kb = 0; kb < nk; ++kb, ++used) {
          const int kc = kb % ozc::CHUNK_KB;
          if (kc == 0 && chunks > 0) {
            // the epilogue must have read the previous chunk's accumulators (this tile's or the last one's)
            if (!mbar_wait(drained_bar, (uint32_t)(chunks - 1) & 1u, p.err, abort_flag, 4)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          }
          const int s = (int)(used % STAGES);
          const uint32_t ph = (uint32_t)(used / STAGES) & 1u;
          if (!mbar_wait(&full_bar[s], ph, p.err, abort_flag, 2)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint64_t a0 = make_desc_sw32(smem_u32(smem + s * STAGE_BYTES));
          const uint64_t b0 = make_desc_sw32(smem_u32(smem + s * STAGE_BYTES + NSL * A_TILE));
          // products (A part, B part, accumulator set, -A): Re.Re, Im.Im -> Re; Re.Im, Im.Re -> Im
#pragma unroll
          for (int pr = 0; pr < 4; ++pr) {
            const int aq = (pr == 1 || pr == 3) ? 1 : 0, bq = (pr == 1 || pr == 2) ? 1 : 0;
            const int set = pr >= 2 ? 1 : 0;
            if (aq == 1 && na == 1) continue;                 // a real A has no Im part
            const bool neg = pr == 1;
            // the set's first product opens the exact groups at each chunk and the tail once per tile
            const bool opener = pr == 0 || pr == 2;
            const uint32_t acc0 = tmem_base + (uint32_t)(set * 5 * wn);
#pragma unroll
            for (int sa = 0; sa < OZ_S; ++sa) {
              const uint64_t a = a0 + (uint64_t)(((aq * OZ_S + sa) * A_TILE) >> 4);
              const uint64_t bs = b0 + (uint64_t)(((bq * OZ_S) * wn * CBK * 2) >> 4);   // B slice 0 of part bq
              if (sa < OZ_S - 1) {
                // groups sa..3 and the tail: B slices 0..4-sa
                const int run = OZ_S - 1 - sa;
                if (opener && sa == 0 && kc == 0 && kb > 0) {
                  // a later chunk: the exact groups restart, the tail carries on
                  mma_bf16(acc0, a, bs, make_idesc_ozc(neg, 4 * wn), 0u);
                  mma_bf16(acc0 + (uint32_t)(4 * wn), a, bs + (uint64_t)((4 * wn * CBK * 2) >> 4),
                           make_idesc_ozc(neg, wn), 1u);
                } else {
                  mma_bf16(acc0 + (uint32_t)(sa * wn), a, bs, make_idesc_ozc(neg, run * wn),
                           (opener && sa == 0 && kc == 0) ? 0u : 1u);
                }
              }
              // the g = 5 pair (sa, 5 - sa) into the tail
              mma_bf16(acc0 + (uint32_t)(4 * wn), a, bs + (uint64_t)(((OZ_S - 1 - sa) * wn * CBK * 2) >> 4),
                       make_idesc_ozc(neg, wn), 1u);
            }
          }
          mma_commit(&empty_bar[s]);
          if (kc == ozc::CHUNK_KB - 1 || kb == nk - 1) {
            mma_commit(chunk_bar);
            ++chunks;
          }
        }
      }
      if (!ok) {
        // the MMAs issued so far complete before TMEM is freed
        mma_commit(done_bar);
        long long t0 = clock64();
        while (!mbar_try_wait(done_bar, 0u) && clock64() - t0 < kWaitCycles) {
        }
      }
    }
  } else {
    // epilogue: warps 2..13; TMEM lane quadrant q = warp % 4, column third h
    const int q = warp & 3, h = (warp - 2) >> 2;
    const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * EPI);
    long long chunks = 0;
    bool ok = nk > 0;
    for (int64_t t = tile0; t < p.ntiles && ok; t += tstep) {
      const int64_t tm = t / p.ntn;
      const int tn = (int)(t % p.ntn);
      const int wn = ozc_tile_width(p.N, p.W, tn);
      const int64_t m = tm * CBM + q * 32 + lane;
      const int64_t n0 = (int64_t)tn * p.W + h * EPI;
      const bool cols = h * EPI < wn;   // warp-uniform: this third of the tile holds columns of C
      // the row's and the columns' scale exponents, read while the tile's MMAs run
      int fa = 0, fb[EPI];
#pragma unroll
      for (int j = 0; j < EPI; ++j) fb[j] = 0;
      if (cols && m < p.M) {
        fa = __ldg(p.fA + m);
#pragma unroll
        for (int j = 0; j < EPI; ++j)
          if (h * EPI + j < wn && n0 + j < p.N) fb[j] = __ldg(p.fB + n0 + j);
      }
      // exact group sums (units 2^-21); after the last chunk, with the tails, in units of 2^-32
      long long ar[EPI], ai[EPI];
#pragma unroll
      for (int j = 0; j < EPI; ++j) ar[j] = ai[j] = 0;
      for (int c = 0; c < nchunks; ++c, ++chunks) {
        int okw = 0;
        if (lane == 0) okw = mbar_wait(chunk_bar, (uint32_t)chunks & 1u, p.err, abort_flag, 3) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, okw, 0) != 0;
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (cols) {
#pragma unroll
          for (int set = 0; set < 2; ++set) {
#pragma unroll
            for (int c8 = 0; c8 < EPI / 8; ++c8) {
              uint32_t g0[8], g1[8], g2[8], g3[8];
              const uint32_t sb = lane_base + (uint32_t)(set * 5 * wn + c8 * 8);
              tmem_ld8_async(sb, g0);
              tmem_ld8_async(sb + wn, g1);
              tmem_ld8_async(sb + 2 * wn, g2);
              tmem_ld8_async(sb + 3 * wn, g3);
              asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const long long v = oz_groups(g0[j], g1[j], g2[j], g3[j]);
                if (set == 0) ar[c8 * 8 + j] += v; else ai[c8 * 8 + j] += v;
              }
            }
          }
          if (c == nchunks - 1) {
#pragma unroll
            for (int c8 = 0; c8 < EPI / 8; ++c8) {
              uint32_t tr[8], ti[8];
              tmem_ld8_async(lane_base + 4 * wn + c8 * 8, tr);
              tmem_ld8_async(lane_base + 9 * wn + c8 * 8, ti);
              asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                ar[c8 * 8 + j] = oz_fixed32(ar[c8 * 8 + j], __uint_as_float(tr[j]));
                ai[c8 * 8 + j] = oz_fixed32(ai[c8 * 8 + j], __uint_as_float(ti[j]));
              }
            }
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(drained_bar);
      }
      if (!ok) break;
      // TMEM is free for the next tile: convert (exact sums + tail, units 2^-32, rounded once to FP64) and store
      if (cols && m < p.M) {
        z64* crow = p.C + m * p.ldc;
#pragma unroll
        for (int j = 0; j < EPI; ++j) {
          const int64_t n = n0 + j;
          if (h * EPI + j < wn && n < p.N) {
            const int e2 = fa + fb[j] - 32;
            z64 out;
            if (e2 >= -1022 && e2 <= 960) out = zmk(i64_ldexp_normal(ar[j], e2), i64_ldexp_normal(ai[j], e2));
            else out = zmk(i64_ldexp_rn(ar[j], e2), i64_ldexp_rn(ai[j], e2));
            if (!p.plain) {
              out = zmul(p.alpha, out);
              if (p.beta.x != 0.0 || p.beta.y != 0.0) out = zadd(out, zmul(p.beta, crow[n]));
            }
            crow[n] = out;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(ozc::TMEM_COLS));
  }
}

int64_t rup(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

int sign_code(double c) { return c == 0.0 ? 0 : (c == 1.0 ? 1 : (c == -1.0 ? -1 : 2)); }

// Tensor map over slice planes [rows_total][Kp] (bf16) for the 3M kernel: boxes of BK x
// box_rows with the 64-byte swizzle.
bool encode_slices(CUtensorMap* map, uint16_t* base, int64_t rows_total, int64_t Kp, int box_rows) {
  auto enc = tma_encode_fn();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows_total};
  cuuint64_t strides[1] = {(cuuint64_t)(Kp * 2)};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1u, 1u};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// K up to which complex products take the one-pass kernel: there the 3M kernel's three
// passes, each re-reading and re-writing C, cost more than its 25 % fewer MMAs save.
constexpr int64_t kOzcMaxK = 1024;

struct OzcLayout {
  int64_t Mp, Np, Kp;
  size_t sA, sB, eA, eB, fA, fB, total;   // byte offsets from the scratch base
};

// na: parts of A sliced (2, or 1 for a real A); B always has both.
OzcLayout ozc_layout(int64_t M, int64_t N, int64_t K, int na) {
  OzcLayout L;
  L.Mp = rup(M, ozc::BM);
  L.Np = rup(rup(N, ozc::BN), 32);   // whole 48-wide column tiles, in the slicer's 32-row tiles
  L.Kp = rup(K, 32);      // the slicing kernels work on 32 x 32 tiles
  size_t off = 256;       // status word
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  L.sA = take((size_t)na * OZ_S * L.Mp * L.Kp * 2);
  L.sB = take((size_t)2 * OZ_S * L.Np * L.Kp * 2);
  L.eA = take((size_t)L.Mp * 4);
  L.eB = take((size_t)L.Np * 4);
  L.fA = take((size_t)L.Mp * 4);
  L.fB = take((size_t)L.Np * 4);
  L.total = off;
  return L;
}

struct OzLayout {
  int64_t Mp, Np, Kp;
  size_t sA, sB, eA, eB, fA, fB, total;   // byte offsets from the scratch base
};

// pa: parts of A whose slices are held at once (1, or 3 to slice Re, Im and Re + Im in one pass)
OzLayout oz_layout(int64_t M, int64_t N, int64_t K, int pa) {
  OzLayout L;
  L.Mp = rup(M, BM);
  L.Np = rup(N, BN);
  L.Kp = rup(K, BK);
  size_t off = 256;   // status word
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  L.sA = take((size_t)pa * OZ_S * L.Mp * L.Kp * 2);
  L.sB = take((size_t)OZ_S * L.Np * L.Kp * 2);
  L.eA = take((size_t)pa * L.Mp * 4);
  L.eB = take((size_t)L.Np * 4);
  L.fA = take((size_t)pa * L.Mp * 4);
  L.fB = take((size_t)L.Np * 4);
  L.total = off;
  return L;
}

}  // namespace

// Output tiles of the Ozaki GEMM (the dispatcher sends GEMMs with fewer than a wave
// of tiles to the double-float kernel, which splits K).
int64_t ozgemm_tiles(int64_t M, int64_t N) { return (rup(M, BM) / BM) * (rup(N, BN) / BN); }

size_t ozgemm_scratch_bytes(int64_t M, int64_t N, int64_t K) {
  if (M <= 0 || N <= 0 || K <= 0) return 256;
  if (K <= kOzcMaxK) return ozc_layout(M, N, K, 2).total;
  return oz_layout(M, N, K, 1).total;
}

// Scratch with which a complex A is sliced once for all three products (one read of A
// instead of three); ozgemm_ex uses that path whenever its scratch is this large.
size_t ozgemm_scratch_bytes_fused(int64_t M, int64_t N, int64_t K) {
  if (M <= 0 || N <= 0 || K <= 0) return 256;
  if (K <= kOzcMaxK) return ozc_layout(M, N, K, 2).total;
  return oz_layout(M, N, K, 3).total;
}

namespace {
// The one-pass complex product (K <= kOzcMaxK): slices with exponents shared by Re and Im.
agb_status ozc_gemm(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                    const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc, void* scratch,
                    size_t scratch_bytes, cudaStream_t stream) {
  const int na = conjA == kSrcReal ? 1 : 2;
  const OzcLayout L = ozc_layout(M, N, K, na);
  if (scratch_bytes < L.total) {
    agb_set_error_message("ozgemm: scratch too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  char* base = (char*)scratch;
  uint16_t* sA = (uint16_t*)(base + L.sA);
  uint16_t* sB = (uint16_t*)(base + L.sB);
  int* eA = (int*)(base + L.eA);
  int* eB = (int*)(base + L.eB);
  int* fA = (int*)(base + L.fA);
  int* fB = (int*)(base + L.fB);
  // both parts of an operand from one read, under one exponent per row (estride 0)
  auto slice = [&](const z64* src, int64_t rows, int64_t s_row, int64_t s_k, int conj, int np, int64_t rows_pad,
                   int* emax, int* fexp, uint16_t* dst) -> agb_status {
    if (L.Kp <= kOzFusedMaxK) {
      // one read: exponents and slices of 32 whole rows per block
      const size_t sh = (size_t)32 * (L.Kp + 1) * sizeof(z64);
      const int per_sm = (int)((227 * 1024) / (sh + 1024));
      const int64_t blocks = rows_pad / 32, cap = (int64_t)152 * (per_sm > 0 ? per_sm : 1);
      const int g = (int)(blocks < cap ? blocks : cap);
      if (np == 2) {
        AGB_CUDA_TRY(cudaFuncSetAttribute(oz_slice_fused_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sh));
        oz_slice_fused_kernel<2><<<g, 256, sh, stream>>>(src, rows, K, s_row, s_k, conj, rows_pad, L.Kp, fexp, dst);
      } else {
        AGB_CUDA_TRY(cudaFuncSetAttribute(oz_slice_fused_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sh));
        oz_slice_fused_kernel<1><<<g, 256, sh, stream>>>(src, rows, K, s_row, s_k, conj, rows_pad, L.Kp, fexp, dst);
      }
      AGB_LAUNCH_CHECK();
      return AGB_OK;
    }
    AGB_CUDA_TRY(cudaMemsetAsync(emax, 0, (size_t)rows_pad * 4, stream));
    const int64_t t1 = ((rows + 31) / 32) * ((K + 31) / 32);
    const int g1 = (int)(t1 < 152 * 32 ? t1 : 152 * 32);
    if (np == 2) oz_rowexp_kernel<2><<<g1, 256, 0, stream>>>(src, rows, K, s_row, s_k, conj, 0, 0, emax);
    else oz_rowexp_kernel<1><<<g1, 256, 0, stream>>>(src, rows, K, s_row, s_k, conj, 0, 0, emax);
    AGB_LAUNCH_CHECK();
    const int64_t t2 = ((rows_pad + 63) / 64) * (L.Kp / 32);
    const int g2 = (int)(t2 < 152 * 16 ? t2 : 152 * 16);
    if (np == 2)
      oz_slice_kblk_kernel<2><<<g2, 256, 0, stream>>>(src, rows, K, s_row, s_k, conj, 0, rows_pad, L.Kp, 0, emax,
                                                      fexp, dst);
    else
      oz_slice_kblk_kernel<1><<<g2, 256, 0, stream>>>(src, rows, K, s_row, s_k, conj, 0, rows_pad, L.Kp, 0, emax,
                                                      fexp, dst);
    AGB_LAUNCH_CHECK();
    return AGB_OK;
  };
  AGB_STATUS_TRY(slice(A, M, sAm, sAk, conjA, na, L.Mp, eA, fA, sA));
  AGB_STATUS_TRY(slice(B, N, sBn, sBk, conjB, 2, L.Np, eB, fB, sB));
  OzcParams p;
  p.M = M; p.N = N; p.nkb = (int)(L.Kp / ozc::BK); p.a_parts = na; p.fA = fA; p.fB = fB; p.C = C; p.ldc = ldc;
  p.alpha = alpha; p.beta = beta;
  p.plain = alpha.x == 1.0 && alpha.y == 0.0 && beta.x == 0.0 && beta.y == 0.0;
  p.err = (int*)base; p.rowsA = L.Mp; p.rowsB = L.Np;
  p.sA = sA; p.sB = sB;
  // ceil(N / 48) column tiles of equal width W (a multiple of 16; the last may be narrower)
  p.ntn = (int)((N + ozc::BN - 1) / ozc::BN);
  p.W = (int)rup((N + p.ntn - 1) / p.ntn, 16);
  p.ntiles = (L.Mp / ozc::BM) * p.ntn;
  AGB_CUDA_TRY(cudaFuncSetAttribute(ozc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ozc::SMEM_BYTES));
  int dev = 0, nsm = 0;
  AGB_CUDA_TRY(cudaGetDevice(&dev));
  AGB_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int64_t grid = p.ntiles < nsm ? p.ntiles : nsm;   // one persistent CTA per SM
  ozc_kernel<<<(unsigned)grid, ozc::THREADS, ozc::SMEM_BYTES, stream>>>(p);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}
}  // namespace

// C = alpha op(A) op(B) + beta C to ~1e-12 of sum |a||b| on the bf16 tensor cores.
// scratch: ozgemm_scratch_bytes(M, N, K), 256-byte aligned; its first int is the
// kernel's error word (read by agb_scratch_status).
agb_status ozgemm_ex(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                     const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                     void* scratch, size_t scratch_bytes, cudaStream_t stream) {
  AGB_ARG_CHECK(M >= 0 && N >= 0 && K >= 0, "ozgemm: negative size");
  if (M == 0 || N == 0) return AGB_OK;
  AGB_ARG_CHECK(K > 0, "ozgemm: K must be positive");
  AGB_ARG_CHECK(A && B && C && scratch, "ozgemm: null pointer");
  AGB_ARG_CHECK(((uintptr_t)scratch & 255) == 0, "ozgemm: scratch must be 256-byte aligned");
  if (K <= kOzcMaxK)
    return ozc_gemm(M, N, K, alpha, A, sAm, sAk, conjA, B, sBk, sBn, conjB, beta, C, ldc, scratch, scratch_bytes,
                    stream);
  const bool realA = conjA == kSrcReal, realB = conjB == kSrcReal;
  const int pa = (!realA && scratch_bytes >= oz_layout(M, N, K, 3).total) ? 3 : 1;
  const OzLayout L = oz_layout(M, N, K, pa);
  if (scratch_bytes < L.total) {
    agb_set_error_message("ozgemm: scratch too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  AGB_ARG_CHECK(L.Mp / BM <= 65535, "ozgemm: M too large for the grid");
  AGB_ARG_CHECK(OZ_S * L.Mp < (1ll << 31) && OZ_S * L.Np < (1ll << 31), "ozgemm: too many rows for a tensor map");
  char* base = (char*)scratch;
  uint16_t* sA = (uint16_t*)(base + L.sA);
  uint16_t* sB = (uint16_t*)(base + L.sB);
  int* eA = (int*)(base + L.eA);
  int* eB = (int*)(base + L.eB);
  int* fA = (int*)(base + L.fA);
  int* fB = (int*)(base + L.fB);
  const int64_t a_part = (int64_t)OZ_S * L.Mp * L.Kp;   // elements of one part's A slices
  CUtensorMap mA[3], mB;
  for (int q = 0; q < pa; ++q)
    if (!encode_slices(&mA[q], sA + q * a_part, OZ_S * L.Mp, L.Kp, BM)) {
      agb_set_error_message("ozgemm: cuTensorMapEncodeTiled failed", __FILE__, __LINE__);
      return AGB_ERR_CUDA;
    }
  if (!encode_slices(&mB, sB, OZ_S * L.Np, L.Kp, BN)) {
    agb_set_error_message("ozgemm: cuTensorMapEncodeTiled failed", __FILE__, __LINE__);
    return AGB_ERR_CUDA;
  }
  static std::atomic<uint64_t> attr_done{0};
  AGB_STATUS_TRY(once_per_device(attr_done, [&]() -> agb_status {
    AGB_CUDA_TRY(cudaFuncSetAttribute(ozgemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    return AGB_OK;
  }));
  // row exponents then slices of np parts (part0 ...) of an operand, one read of it each
  auto slice = [&](const z64* src, int64_t rows, int64_t s_row, int64_t s_k, int conj, int part0, int np,
                   int64_t rows_pad, int* emax, int* fexp, uint16_t* dst) -> agb_status {
    AGB_CUDA_TRY(cudaMemsetAsync(emax, 0, (size_t)np * rows_pad * 4, stream));
    const int64_t t1 = ((rows + 31) / 32) * ((K + 31) / 32);
    const int g1 = (int)(t1 < 152 * 32 ? t1 : 152 * 32);
    if (np == 3) oz_rowexp_kernel<3><<<g1, 256, 0, stream>>>(src, rows, K, s_row, s_k, conj, part0, rows_pad, emax);
    else oz_rowexp_kernel<1><<<g1, 256, 0, stream>>>(src, rows, K, s_row, s_k, conj, part0, rows_pad, emax);
    AGB_LAUNCH_CHECK();
    const int64_t t2 = (rows_pad / 32) * (L.Kp / 32);
    const int g2 = (int)(t2 < 152 * 32 ? t2 : 152 * 32);
    if (np == 3)
      oz_slice_kernel<3><<<g2, 256, 0, stream>>>(src, rows, K, s_row, s_k, conj, part0, rows_pad, L.Kp, rows_pad,
                                                 emax, fexp, dst);
    else
      oz_slice_kernel<1><<<g2, 256, 0, stream>>>(src, rows, K, s_row, s_k, conj, part0, rows_pad, L.Kp, rows_pad,
                                                 emax, fexp, dst);
    AGB_LAUNCH_CHECK();
    return AGB_OK;
  };
  OzParams p;
  p.M = M; p.N = N; p.nkb = (int)(L.Kp / BK); p.fB = fB; p.C = C; p.ldc = ldc; p.beta = beta;
  p.err = (int*)base; p.rowsA = L.Mp; p.rowsB = L.Np;
  // |exact sum| < K 2^35 (1 + 2^-6) units of 2^-21: shifted by 11 it stays below 2^63 for K <= 2^16
  p.fixed = L.Kp <= (1 << 16) ? 1 : 0;
  dim3 grid((unsigned)(L.Np / BN), (unsigned)(L.Mp / BM));
  // 3M coefficients of P1 = Re.Re, P2 = Im.Im, P3 = (Re+Im).(Re+Im)
  const z64 coef[3] = {zmk(1, -1), zmk(-1, -1), zmk(0, 1)};
  const bool use_beta = beta.x != 0.0 || beta.y != 0.0;
  if (pa == 3) AGB_STATUS_TRY(slice(A, M, sAm, sAk, conjA, 0, 3, L.Mp, eA, fA, sA));
  for (int part = 0; part < 3; ++part) {
    if (part == 1 && (realA || realB)) continue;   // Im.Im of a real operand is zero
    int qa = 0;                                     // A slice set of this product
    if (pa == 3) qa = part;
    else if (!(realA && part == 2))                 // a real A's Re + Im is its Re, still in place
      AGB_STATUS_TRY(slice(A, M, sAm, sAk, conjA, part, 1, L.Mp, eA, fA, sA));
    AGB_STATUS_TRY(slice(B, N, sBn, sBk, conjB, part, 1, L.Np, eB, fB, sB));
    p.fA = fA + qa * L.Mp;
    p.coef = zmul(alpha, coef[part]);
    p.csx = sign_code(p.coef.x);
    p.csy = sign_code(p.coef.y);
    p.mode = part > 0 ? 2 : (use_beta ? 1 : 0);
    ozgemm_kernel<<<grid, THREADS, SMEM_BYTES, stream>>>(mA[qa], mB, p);
    AGB_LAUNCH_CHECK();
  }
  return AGB_OK;
}

}  // namespace agb

extern "C" {

size_t agb_zgemm_oz_scratch_bytes(int64_t M, int64_t N, int64_t K) { return agb::ozgemm_scratch_bytes(M, N, K); }

agb_status agb_zgemm_oz(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im, const void* A,
                        int64_t sAm, int64_t sAk, int conjA, const void* B, int64_t sBk, int64_t sBn, int conjB,
                        double beta_re, double beta_im, void* C, int64_t ldc, void* scratch, size_t scratch_bytes,
                        void* stream) {
  AGB_ARG_CHECK((conjA == 0 || conjA == 1) && (conjB == 0 || conjB == 1), "gemm: conj flags must be 0 or 1");
  AGB_ARG_CHECK(M <= 1 || N <= 0 || ldc >= N, "gemm: ldc must be at least N (C is row-major)");
  return agb::ozgemm_ex(M, N, K, agb::zmk(alpha_re, alpha_im), (const agb::z64*)A, sAm, sAk, conjA,
                        (const agb::z64*)B, sBk, sBn, conjB, agb::zmk(beta_re, beta_im), (agb::z64*)C, ldc, scratch,
                        scratch_bytes, (cudaStream_t)stream);
}

}  // extern "C"
