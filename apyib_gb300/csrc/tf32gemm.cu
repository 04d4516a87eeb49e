// Complex GEMM as complex-FP32 with 3xTF32 split products on the sm_103a
// tensor cores (tcgen05.mma kind::tf32, accumulators in TMEM, operands staged
// by TMA with 64-byte swizzle).
//
//   x = x_hi + x_lo,  x_hi = tf32(x), x_lo = tf32(x - x_hi)   (|x - x_hi - x_lo| ~ 2^-22 |x|)
//   a*b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi
//   Re(C) += Ar Br - Ai Bi,  Im(C) += Ar Bi + Ai Br   (4M; the minus via the MMA negate-A bit)
//
// Operands arrive in FP64 (complex128, arbitrary strides); a prep kernel
// writes four K-major FP32 planes per operand (re_hi, re_lo, im_hi, im_lo),
// zero-padded to the tile grid.  Large outputs run on CTA pairs (cta_group::2,
// 256 x 256 tiles, 3 stages); the rest on single CTAs (128 x 256 tiles, or a tile
// and K split): warp 0 issues TMA loads, warp 1 issues the MMAs from one thread,
// warps 2-5 drain the two TMEM accumulators (Re in columns 0-255, Im in 256-511)
// and write FP64 results.  Outputs up to 256 wide whose A is an FP64 intermediate (the
// AO->MO quarter steps) take a persistent kernel whose converter warps split A into
// the planes in shared memory themselves.  Every mbarrier wait is bounded; on timeout
// the kernel records an error word and returns after releasing TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>

#include "common.cuh"
#include "dfloat.cuh"
#include "fsplit.cuh"
#include "tc05.cuh"

namespace agb {

PFN_cuTensorMapEncodeTiled_v12000 tma_encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* ptr = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)ptr;
  }
  return fn;
}

agb_status zgemm(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                 const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                 cudaStream_t stream);

namespace {
using namespace tc05;

constexpr int BM = 128, BN = 256, BK = 16;   // K padding of the planes, in fp32 elements (64 bytes)
constexpr int THREADS = 192;
// Single-CTA tile shapes: 128 x NB outputs, NB = 256 (2 stages of 96 KB, one CTA per SM),
// NB = 160 for outputs 65..160 wide (2 stages of 72 KB; the AO->MO quarter steps' 150-wide
// outputs), or, for outputs at most 64 wide, NB = 64 (2 stages of 48 KB, two CTAs per SM,
// so one CTA's epilogue overlaps the other's loads): a narrow output then pays for the
// MMA work and operand traffic of its own width, not of 256 columns.
template <int NB> struct Tile {
  static constexpr int STAGES = 2;
  static constexpr int CTAS_PER_SM = NB == 64 ? 2 : 1;
  static constexpr int A_TILE_BYTES = BM * BK * 4;
  static constexpr int B_TILE_BYTES = NB * BK * 4;
  static constexpr int STAGE_BYTES = 4 * (A_TILE_BYTES + B_TILE_BYTES);
  static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
  // Re and Im accumulators (2 NB columns), allocated as a power of two
  static constexpr unsigned TMEM_COLS = 2 * NB <= 128 ? 128u : (2 * NB <= 256 ? 256u : 512u);
};

// tcgen05 shared-memory descriptor of a K-major tile with 64-byte swizzle (16 fp32 per row),
// 8-row groups 512 bytes apart.
__device__ __forceinline__ uint64_t make_desc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(512 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)4 << 61;
  return d;
}
constexpr unsigned TMEM_COLS = 2 * BN;                       // Re and Im accumulators (256-wide tiles)
constexpr int kGroupM = 12;                      // tile rows per raster group

// Instruction descriptor: D=F32, A=B=TF32, K-major both, N=NB, M=128.
template <int NB>
__host__ __device__ constexpr uint32_t make_idesc(bool negA) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((negA ? 1u : 0u) << 13) | ((uint32_t)(NB >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

struct GemmParams {
  int64_t M, N;
  int nkb;          // k-blocks per split
  int nkb_total;
  z64 alpha, beta;
  z64* C;
  int64_t ldc;
  z64* partial;     // split-K partials [splits][M][N] or null
  int* err;
  int64_t rowsA, rowsB;  // padded rows per plane
  int trans_c;           // store C(m, n) at C[n * ldc + m] instead of C[m * ldc + n]
  int kblkA, kblkB;      // operand planes K-blocked ([k/16][row][16] per plane), read through 3D maps
  int c32;               // C holds complex FP32 (float2) values: C = AB (+ C when beta = 1)
};

template <int NB>
__global__ void __launch_bounds__(THREADS, Tile<NB>::CTAS_PER_SM)
tf32x3_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                   GemmParams p) {
  constexpr int STAGES = Tile<NB>::STAGES, STAGE_BYTES = Tile<NB>::STAGE_BYTES;
  constexpr int A_TILE_BYTES = Tile<NB>::A_TILE_BYTES, B_TILE_BYTES = Tile<NB>::B_TILE_BYTES;
  constexpr unsigned NCOLS = Tile<NB>::TMEM_COLS;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full_bar = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty_bar = full_bar + STAGES;
  uint64_t* tmem_bar = empty_bar + STAGES;
  uint32_t* tmem_slot = (uint32_t*)(tmem_bar + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Grouped raster: CTAs launched together cover a band of kGroupM tile rows
  // across a few tile columns, so the A and B panels they stream stay in L2.
  const int ntn = gridDim.x, ntm = gridDim.y;
  const int lin = blockIdx.y * ntn + blockIdx.x;
  const int gsz = kGroupM * ntn;
  const int first_m = (lin / gsz) * kGroupM;
  const int gm = min(ntm - first_m, kGroupM);
  const int tile_m = first_m + (lin % gsz) % gm;
  const int tile_n = (lin % gsz) / gm;
  const int split = blockIdx.z;
  const int kb0 = split * p.nkb;
  int nk = p.nkb_total - kb0;
  if (nk > p.nkb) nk = p.nkb;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(tmem_bar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(NCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // TMA producer
      int issued = 0;
      for (int kb = 0; kb < nk; ++kb) {
        int s = kb % STAGES;
        uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
        if (!mbar_wait(&empty_bar[s], ph ^ 1u, p.err, abort_flag, 1)) break;
        uint8_t* st = smem + s * STAGE_BYTES;
        mbar_expect_tx(&full_bar[s], STAGE_BYTES);
        const int kx = (kb0 + kb) * BK;
        for (int pl = 0; pl < 4; ++pl) {
          // K-blocked planes: one contiguous box per (plane, k-block); rows past the plane read zeros
          if (p.kblkA)
            tma_load_3d(st + pl * A_TILE_BYTES, &mapA, &full_bar[s], 0, tile_m * BM, pl * p.nkb_total + kb0 + kb);
          else
            tma_load_2d(st + pl * A_TILE_BYTES, &mapA, &full_bar[s], kx, (int)(pl * p.rowsA + tile_m * BM));
          if (p.kblkB)
            tma_load_3d(st + 4 * A_TILE_BYTES + pl * B_TILE_BYTES, &mapB, &full_bar[s], 0, tile_n * NB,
                        pl * p.nkb_total + kb0 + kb);
          else
            tma_load_2d(st + 4 * A_TILE_BYTES + pl * B_TILE_BYTES, &mapB, &full_bar[s], kx,
                        (int)(pl * p.rowsB + tile_n * NB));
        }
        issued = kb + 1;
      }
      // On abort, wait (bounded) for loads still in flight before the CTA exits.
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
      // MMA issuer
      const uint32_t id_pos = make_idesc<NB>(false), id_neg = make_idesc<NB>(true);
      const uint32_t d_re = tmem_base, d_im = tmem_base + NB;
      bool ok = true;
      for (int kb = 0; kb < nk; ++kb) {
        int s = kb % STAGES;
        uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, p.err, abort_flag, 2)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        uint32_t st = smem_u32(smem + s * STAGE_BYTES);
        // planes: 0 Ar_hi 1 Ar_lo 2 Ai_hi 3 Ai_lo | 4 Br_hi 5 Br_lo 6 Bi_hi 7 Bi_lo
#pragma unroll
        for (int ks = 0; ks < BK / 8; ++ks) {
          uint64_t a[4], b[4];
#pragma unroll
          for (int pl = 0; pl < 4; ++pl) {
            a[pl] = make_desc_sw64(st + pl * A_TILE_BYTES + ks * 32);
            b[pl] = make_desc_sw64(st + 4 * A_TILE_BYTES + pl * B_TILE_BYTES + ks * 32);
          }
          uint32_t acc0 = (kb > 0 || ks > 0) ? 1u : 0u;
          // Re: Ar Br - Ai Bi
          mma_tf32(d_re, a[1], b[0], id_pos, acc0);
          mma_tf32(d_re, a[0], b[1], id_pos, 1u);
          mma_tf32(d_re, a[0], b[0], id_pos, 1u);
          mma_tf32(d_re, a[3], b[2], id_neg, 1u);
          mma_tf32(d_re, a[2], b[3], id_neg, 1u);
          mma_tf32(d_re, a[2], b[2], id_neg, 1u);
          // Im: Ar Bi + Ai Br
          mma_tf32(d_im, a[1], b[2], id_pos, acc0);
          mma_tf32(d_im, a[0], b[3], id_pos, 1u);
          mma_tf32(d_im, a[0], b[2], id_pos, 1u);
          mma_tf32(d_im, a[3], b[0], id_pos, 1u);
          mma_tf32(d_im, a[2], b[1], id_pos, 1u);
          mma_tf32(d_im, a[2], b[0], id_pos, 1u);
        }
        mma_commit(&empty_bar[s]);   // frees the stage once these MMAs finish
      }
      if (ok) mma_commit(tmem_bar);
    }
  } else {
    // Epilogue warps 2..5: TMEM lane quadrant = warp % 4
    const int q = warp & 3;
    int okw = 0;
    if (lane == 0) okw = mbar_wait(tmem_bar, 0, p.err, abort_flag, 3) ? 1 : 0;
    const bool ok = __shfl_sync(0xffffffffu, okw, 0) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok && nk > 0) {
      const int64_t m = (int64_t)tile_m * BM + q * 32 + lane;
      const bool use_beta = (p.beta.x != 0.0 || p.beta.y != 0.0);
      // FP32 -> FP64 by exponent rebias on the integer pipe, and no complex scaling in the
      // common alpha = 1, beta in {0, 1} case: GB300's FP64 pipe would otherwise bound the
      // epilogue of short-K GEMMs
      const bool unit_alpha = p.alpha.x == 1.0 && p.alpha.y == 0.0;
      const bool unit_beta = p.beta.x == 1.0 && p.beta.y == 0.0;
#pragma unroll 1
      for (int c = 0; c < NB / 32; ++c) {
        float vr[32], vi[32];
        uint32_t tl = tmem_base + ((uint32_t)(q * 32) << 16) + c * 32;
        tmem_ld32(tl, vr);
        tmem_ld32(tl + NB, vi);
        if (m < p.M) {
          int64_t n0 = (int64_t)tile_n * NB + c * 32;
          if (p.partial) {
            z64* dst = p.partial + ((int64_t)split * p.M + m) * p.N + n0;
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (n0 + j < p.N) dst[j] = zmk(f2d_exact(vr[j]), f2d_exact(vi[j]));
          } else if (p.c32) {
            const int64_t sj = p.trans_c ? p.ldc : 1;
            float2* dst = (float2*)p.C + (p.trans_c ? n0 * p.ldc + m : m * p.ldc + n0);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              if (n0 + j < p.N) {
                float2 out = make_float2(vr[j], vi[j]);
                if (unit_beta) {
                  const float2 c = dst[j * sj];
                  out.x += c.x;
                  out.y += c.y;
                }
                dst[j * sj] = out;
              }
            }
          } else {
            // row-major C: a thread writes its row's 32 columns; transposed C: for each column
            // the warp's 32 rows are consecutive addresses
            const int64_t sj = p.trans_c ? p.ldc : 1;
            z64* dst = p.trans_c ? p.C + n0 * p.ldc + m : p.C + m * p.ldc + n0;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              if (n0 + j < p.N) {
                z64 out = zmk(f2d_exact(vr[j]), f2d_exact(vi[j]));
                if (!unit_alpha) out = zmul(p.alpha, out);
                if (unit_beta) out = zadd(out, dst[j * sj]);
                else if (use_beta) out = zadd(out, zmul(p.beta, dst[j * sj]));
                dst[j * sj] = out;
              }
            }
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(NCOLS));
  }
}


// ---------------------------------------------------------------------------
// The single-CTA GEMM with A converted from FP64 inside the kernel (the AO->MO quarter
// steps, whose A is the FP64 intermediate read column by column).  A separate operand split
// reads the intermediate and writes its TF32 planes (8.7 GB per quarter step at nbf = 150),
// which the GEMM then reads back; here eight converter warps load each 128-row x 16-k block
// of A straight from FP64 (coalesced along M), split it into the four planes and store them
// into the stage in the MMA's 64-byte-swizzled K-major layout, then signal the stage.  B
// (the small coefficient matrix) arrives by TMA from its planes as before.  N fits one
// column tile, so a tile is a 128-row band of C.
//
// Persistent: each CTA takes bands blockIdx.x, + gridDim.x, ...; the converters and the B
// loads run through a ring of stages that continues across bands, so the next band's
// operands are converted while this band's epilogue drains TMEM and stores.  A band's
// MMAs wait only until the previous band's accumulators have been read.  Warps: 0 B loads,
// 1 MMAs, 2-9 epilogue (TMEM lane quadrant warp % 4, column half), 10-17 converters
// (thread c: row c % 128, k-half c / 128 of each 16-wide block).  Three stages where they
// fit (64- and 160-wide tiles).
constexpr int FA_EPI_WARPS = 8;
constexpr int FA_THREADS = 64 + 32 * FA_EPI_WARPS + 256;   // B loads, MMAs, epilogue, converters
constexpr int FA_CONV0 = 64 + 32 * FA_EPI_WARPS;            // first converter thread
template <int NB> struct FaTile {
  static constexpr int STAGES = NB == 256 ? 2 : 3;
  static constexpr int SMEM_BYTES = STAGES * Tile<NB>::STAGE_BYTES + 1024 + 256;
};

struct FaParams {
  int64_t M, N, K;
  const z64* A;          // A(m, k) = A[m * sAm + k * sAk]; conjA == kSrcReal: a real FP64 array
  int64_t sAm, sAk;
  int conjA;
  int nkb;               // 16-wide k-blocks
  int64_t ntiles;        // 128-row bands
  z64 alpha, beta;
  z64* C;
  int64_t ldc;
  int* err;
  int64_t rowsB;         // padded rows per B plane
};

// Byte offset of fp32 element (row, k < 16) in a K-major tile of 64-byte rows with the
// 64-byte swizzle: 16-byte chunk c of row r sits at chunk c ^ ((r >> 1) & 3).
__device__ __forceinline__ uint32_t sw64_chunk_off(int row, int chunk) {
  return (uint32_t)(row * 64 + ((chunk ^ ((row >> 1) & 3)) << 4));
}

template <int NB>
__global__ void __launch_bounds__(FA_THREADS, 1)
tf32x3_gemm_fa_kernel(const __grid_constant__ CUtensorMap mapB, FaParams p) {
  constexpr int STAGES = FaTile<NB>::STAGES, STAGE_BYTES = Tile<NB>::STAGE_BYTES;
  constexpr int A_TILE_BYTES = Tile<NB>::A_TILE_BYTES, B_TILE_BYTES = Tile<NB>::B_TILE_BYTES;
  constexpr unsigned NCOLS = Tile<NB>::TMEM_COLS;
  constexpr int HALF = NB / 2;               // columns per epilogue warp
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full_bar = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty_bar = full_bar + STAGES;
  uint64_t* tmem_full = empty_bar + STAGES;   // MMA -> epilogue: the band's MMAs completed
  uint64_t* tmem_empty = tmem_full + 1;       // epilogue -> MMA: the band's accumulators read (8 warps)
  uint64_t* done_bar = tmem_empty + 1;        // MMA issuer, on abort: its MMAs completed
  uint32_t* tmem_slot = (uint32_t*)(done_bar + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  volatile int* conv_ok = abort_flag + 1;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = p.nkb;
  const bool real_a = p.conjA == kSrcReal;   // no Im planes: six of the twelve MMAs, half the stores
  const int64_t tile0 = blockIdx.x, tstep = gridDim.x;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 2);      // B's expect_tx arrival + the converters' arrival
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(tmem_full, 1);
    mbar_init(tmem_empty, FA_EPI_WARPS);
    mbar_init(done_bar, 1);
    *abort_flag = 0;
    *conv_ok = 1;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(NCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // B planes by TMA, stage by stage across bands
      long long issued = 0;
      bool ok = true;
      for (int64_t t = tile0; t < p.ntiles && ok; t += tstep) {
        for (int kb = 0; kb < nk; ++kb) {
          const int s = (int)(issued % STAGES);
          const uint32_t ph = (uint32_t)(issued / STAGES) & 1u;
          if (!mbar_wait(&empty_bar[s], ph ^ 1u, p.err, abort_flag, 1)) {
            ok = false;
            break;
          }
          uint8_t* st = smem + s * STAGE_BYTES;
          mbar_expect_tx(&full_bar[s], 4 * B_TILE_BYTES);
          for (int pl = 0; pl < 4; ++pl)
            tma_load_2d(st + 4 * A_TILE_BYTES + pl * B_TILE_BYTES, &mapB, &full_bar[s], kb * BK, (int)(pl * p.rowsB));
          ++issued;
        }
      }
      if (!ok) {
        for (long long i = (issued > STAGES ? issued - STAGES : 0); i < issued; ++i) {
          long long t0 = clock64();
          while (!mbar_try_wait(&full_bar[i % STAGES], (uint32_t)(i / STAGES) & 1u) && clock64() - t0 < kWaitCycles) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t id_pos = make_idesc<NB>(false), id_neg = make_idesc<NB>(true);
      const uint32_t d_re = tmem_base, d_im = tmem_base + NB;
      long long used = 0, bands = 0;
      bool ok = true;
      for (int64_t t = tile0; t < p.ntiles && ok; t += tstep) {
        if (bands > 0) {
          // the epilogue must have read the previous band's accumulators
          if (!mbar_wait(tmem_empty, (uint32_t)(bands - 1) & 1u, p.err, abort_flag, 4)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        for (int kb = 0; kb < nk; ++kb, ++used) {
          const int s = (int)(used % STAGES);
          const uint32_t ph = (uint32_t)(used / STAGES) & 1u;
          if (!mbar_wait(&full_bar[s], ph, p.err, abort_flag, 2)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          uint32_t st = smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
          for (int ks = 0; ks < BK / 8; ++ks) {
            uint64_t a[4], b[4];
#pragma unroll
            for (int pl = 0; pl < 4; ++pl) {
              a[pl] = make_desc_sw64(st + pl * A_TILE_BYTES + ks * 32);
              b[pl] = make_desc_sw64(st + 4 * A_TILE_BYTES + pl * B_TILE_BYTES + ks * 32);
            }
            uint32_t acc0 = (kb > 0 || ks > 0) ? 1u : 0u;
            mma_tf32(d_re, a[1], b[0], id_pos, acc0);
            mma_tf32(d_re, a[0], b[1], id_pos, 1u);
            mma_tf32(d_re, a[0], b[0], id_pos, 1u);
            if (!real_a) {
              mma_tf32(d_re, a[3], b[2], id_neg, 1u);
              mma_tf32(d_re, a[2], b[3], id_neg, 1u);
              mma_tf32(d_re, a[2], b[2], id_neg, 1u);
            }
            mma_tf32(d_im, a[1], b[2], id_pos, acc0);
            mma_tf32(d_im, a[0], b[3], id_pos, 1u);
            mma_tf32(d_im, a[0], b[2], id_pos, 1u);
            if (!real_a) {
              mma_tf32(d_im, a[3], b[0], id_pos, 1u);
              mma_tf32(d_im, a[2], b[1], id_pos, 1u);
              mma_tf32(d_im, a[2], b[0], id_pos, 1u);
            }
          }
          mma_commit(&empty_bar[s]);
        }
        if (!ok) break;
        mma_commit(tmem_full);
        ++bands;
      }
      if (!ok) {
        // the MMAs issued so far complete before TMEM is freed
        mma_commit(done_bar);
        long long t0 = clock64();
        while (!mbar_try_wait(done_bar, 0u) && clock64() - t0 < kWaitCycles) {
        }
      }
    }
  } else if (threadIdx.x >= FA_CONV0) {
    // converters: thread c owns row c % 128 of the band and half (8 k) of each k-block
    const int c = threadIdx.x - FA_CONV0;
    const int row = c & 127, kh = c >> 7;
    long long it = 0;
    bool ok = true;
    for (int64_t t = tile0; t < p.ntiles && ok; t += tstep) {
      const int64_t m = t * BM + row;
      const bool live = m < p.M;
      for (int kb = 0; kb < nk; ++kb, ++it) {
        const int s = (int)(it % STAGES);
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        if (c == 0) *conv_ok = mbar_wait(&empty_bar[s], ph ^ 1u, p.err, abort_flag, 5) ? 1 : 0;
        asm volatile("bar.sync 1, 256;" ::: "memory");   // the eight converter warps; c == 0's wait is bounded
        if (!*conv_ok) {
          ok = false;
          break;
        }
        z64 v[BK / 2];
#pragma unroll
        for (int kk = 0; kk < BK / 2; ++kk) {
          const int64_t k = (int64_t)kb * BK + kh * (BK / 2) + kk;
          v[kk] = zmk(0, 0);
          if (live && k < p.K) {
            if (p.conjA == kSrcReal) {
              v[kk].x = ((const double*)p.A)[m * p.sAm + k * p.sAk];
            } else {
              v[kk] = p.A[m * p.sAm + k * p.sAk];
              if (p.conjA == 1) v[kk].y = -v[kk].y;
            }
          }
        }
        uint8_t* st = smem + s * STAGE_BYTES;
#pragma unroll
        for (int cl = 0; cl < BK / 8; ++cl) {
          const int ch = kh * (BK / 8) + cl;          // 16-byte chunk of the row
          float4 rh, rl, ih, il;
          float* prh = &rh.x;
          float* prl = &rl.x;
          float* pih = &ih.x;
          float* pil = &il.x;
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            uint32_t a0, a1, b0, b1;
            const z64 x = v[4 * cl + u];
            split_tf32_fast((uint32_t)__double2hiint(x.x), (uint32_t)__double2loint(x.x), a0, a1);
            split_tf32_fast((uint32_t)__double2hiint(x.y), (uint32_t)__double2loint(x.y), b0, b1);
            prh[u] = __uint_as_float(a0);
            prl[u] = __uint_as_float(a1);
            pih[u] = __uint_as_float(b0);
            pil[u] = __uint_as_float(b1);
          }
          const uint32_t off = sw64_chunk_off(row, ch);
          *(float4*)(st + off) = rh;
          *(float4*)(st + A_TILE_BYTES + off) = rl;
          if (!real_a) {
            *(float4*)(st + 2 * A_TILE_BYTES + off) = ih;
            *(float4*)(st + 3 * A_TILE_BYTES + off) = il;
          }
        }
        // the generic-proxy stores must be visible to the tensor core's (async-proxy) reads
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("bar.sync 1, 256;" ::: "memory");
        if (c == 0) mbar_arrive(&full_bar[s]);
      }
    }
  } else {
    // epilogue warps 2..9: TMEM lane quadrant q = warp % 4, column half h
    const int q = warp & 3, h = (warp - 2) >> 2;
    const bool use_beta = (p.beta.x != 0.0 || p.beta.y != 0.0);
    const bool unit_alpha = p.alpha.x == 1.0 && p.alpha.y == 0.0;
    long long bands = 0;
    for (int64_t t = tile0; t < p.ntiles; t += tstep, ++bands) {
      int okw = 0;
      if (lane == 0) okw = mbar_wait(tmem_full, (uint32_t)bands & 1u, p.err, abort_flag, 3) ? 1 : 0;
      if (__shfl_sync(0xffffffffu, okw, 0) == 0) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int64_t m = t * BM + q * 32 + lane;
#pragma unroll 1
      for (int cc = 0; cc < HALF / 16; ++cc) {
        float vr[16], vi[16];
        const uint32_t tl = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * HALF + cc * 16);
        tmem_ld16(tl, vr);
        tmem_ld16(tl + NB, vi);
        if (cc == HALF / 16 - 1) {
          // the band's accumulators are in registers: the next band's MMAs may start
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(tmem_empty);
        }
        if (m < p.M) {
          const int64_t n0 = (int64_t)h * HALF + cc * 16;
          z64* dst = p.C + m * p.ldc + n0;
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            if (n0 + j < p.N) {
              z64 out = zmk(f2d_exact(vr[j]), f2d_exact(vi[j]));
              if (!unit_alpha) out = zmul(p.alpha, out);
              if (use_beta) out = zadd(out, zmul(p.beta, dst[j]));
              dst[j] = out;
            }
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(NCOLS));
  }
}

// The same GEMM on CTA pairs (tcgen05 cta_group::2): a cluster of two CTAs on two
// SMs computes a 256 x 256 output tile with 256-row MMAs issued by the even CTA.
// Each CTA stages its own 128 rows of A and its own 128 of the 256 rows of B (the
// MMA reads B from both CTAs' shared memory), so per SM the operand traffic from L2
// and the tensor core's shared-memory reads are two thirds of the single-CTA tile's.
// Each CTA's TMEM holds its 128 output rows (Re | Im, 512 columns).  Both CTAs'
// TMA loads complete on the even CTA's "full" barrier; the even CTA's MMA commit
// arrives on both CTAs' "empty" barriers and, at the end, on both "tmem" barriers.
// Every wait is bounded as in the single-CTA kernel; the pair meets at cluster
// barriers after set-up and before freeing TMEM, which every thread reaches.
constexpr int P2_STAGES = 3;
constexpr int P2_A_TILE = 128 * BK * 4;                    // 8 KB per plane (own 128 rows)
constexpr int P2_B_TILE = 128 * BK * 4;                    // 8 KB per plane (own half of 256 rows)
constexpr int P2_STAGE_BYTES = 4 * (P2_A_TILE + P2_B_TILE);  // 64 KB
constexpr int P2_SMEM_BYTES = P2_STAGES * P2_STAGE_BYTES + 1024 + 256;

// Instruction descriptor for the pair MMA: D = F32, A = B = TF32, K-major, N = 256, M = 256.
__host__ __device__ constexpr uint32_t make_idesc_pair(bool negA) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((negA ? 1u : 0u) << 13) | ((uint32_t)(256 >> 3) << 17) |
         ((uint32_t)(256 >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32_pair(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                              uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Commit of the pair MMAs issued so far: one arrival on the barrier at this shared
// offset in both CTAs of the pair.
__device__ __forceinline__ void mma_commit_pair(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
      ::"r"(smem_u32(bar)), "h"((uint16_t)3)
      : "memory");
}

// TMA load whose completion is counted on a barrier of either CTA of the pair (bar is a
// shared::cluster address, here the even CTA's).
__device__ __forceinline__ void tma_load_2d_pair(void* dst, const CUtensorMap* map, uint32_t bar_cluster, int x,
                                                 int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4}], [%2];"
      ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(bar_cluster), "r"(x), "r"(y)
      : "memory");
}

// Shared::cluster address of the object at local shared address a in CTA rank 'rank'.
__device__ __forceinline__ uint32_t map_to_rank(uint32_t a, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS, 1)
tf32x3_gemm2_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                    GemmParams p) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full_bar = (uint64_t*)(smem + P2_STAGES * P2_STAGE_BYTES);
  uint64_t* empty_bar = full_bar + P2_STAGES;
  uint64_t* tmem_bar = empty_bar + P2_STAGES;
  uint32_t* tmem_slot = (uint32_t*)(tmem_bar + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_rank();             // 0: issues the MMAs; 1: its peer
  // pair tiles in a grouped raster (kGroupM pair rows per group); x = 2 * tile_n + rank
  const int ntn = gridDim.x / 2, ntm = gridDim.y;
  const int lin = blockIdx.y * ntn + (blockIdx.x >> 1);
  const int gsz = kGroupM * ntn;
  const int first_m = (lin / gsz) * kGroupM;
  const int gm = min(ntm - first_m, kGroupM);
  const int tile_m = first_m + (lin % gsz) % gm;    // 256-row pair tile
  const int tile_n = (lin % gsz) / gm;              // 256-column tile
  const int split = blockIdx.z;
  const int kb0 = split * p.nkb;
  int nk = p.nkb_total - kb0;
  if (nk > p.nkb) nk = p.nkb;

  if (threadIdx.x == 0) {
    for (int s = 0; s < P2_STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(tmem_bar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  cluster_sync_all();                               // the peer's barriers exist before any load targets them
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // TMA producer of this CTA's operand halves; completion counted on the even CTA's barrier
      int issued = 0;
      for (int kb = 0; kb < nk; ++kb) {
        const int s = kb % P2_STAGES;
        const uint32_t ph = (uint32_t)(kb / P2_STAGES) & 1u;
        if (!mbar_wait(&empty_bar[s], ph ^ 1u, p.err, abort_flag, 1)) break;
        uint8_t* st = smem + s * P2_STAGE_BYTES;
        if (rank == 0) mbar_expect_tx(&full_bar[s], 2 * P2_STAGE_BYTES);
        const uint32_t bar0 = map_to_rank(smem_u32(&full_bar[s]), 0);
        const int kx = (kb0 + kb) * BK;
        for (int pl = 0; pl < 4; ++pl) {
          tma_load_2d_pair(st + pl * P2_A_TILE, &mapA, bar0, kx, (int)(pl * p.rowsA + tile_m * 256 + rank * 128));
          tma_load_2d_pair(st + 4 * P2_A_TILE + pl * P2_B_TILE, &mapB, bar0, kx,
                           (int)(pl * p.rowsB + tile_n * 256 + rank * 128));
        }
        issued = kb + 1;
      }
      if (*abort_flag && rank == 0) {
        // wait (bounded) for the stages in flight: the even CTA's barrier counts both halves
        for (int kb = (issued > P2_STAGES ? issued - P2_STAGES : 0); kb < issued; ++kb) {
          long long t0 = clock64();
          while (!mbar_try_wait(&full_bar[kb % P2_STAGES], (uint32_t)(kb / P2_STAGES) & 1u) &&
                 clock64() - t0 < kWaitCycles) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && rank == 0) {
      // MMA issuer (even CTA only)
      const uint32_t id_pos = make_idesc_pair(false), id_neg = make_idesc_pair(true);
      const uint32_t d_re = tmem_base, d_im = tmem_base + BN;
      bool ok = true;
      for (int kb = 0; kb < nk; ++kb) {
        const int s = kb % P2_STAGES;
        const uint32_t ph = (uint32_t)(kb / P2_STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, p.err, abort_flag, 2)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = smem_u32(smem + s * P2_STAGE_BYTES);
#pragma unroll
        for (int ks = 0; ks < BK / 8; ++ks) {
          uint64_t a[4], b[4];
#pragma unroll
          for (int pl = 0; pl < 4; ++pl) {
            a[pl] = make_desc_sw64(st + pl * P2_A_TILE + ks * 32);
            b[pl] = make_desc_sw64(st + 4 * P2_A_TILE + pl * P2_B_TILE + ks * 32);
          }
          const uint32_t acc0 = (kb > 0 || ks > 0) ? 1u : 0u;
          mma_tf32_pair(d_re, a[1], b[0], id_pos, acc0);
          mma_tf32_pair(d_re, a[0], b[1], id_pos, 1u);
          mma_tf32_pair(d_re, a[0], b[0], id_pos, 1u);
          mma_tf32_pair(d_re, a[3], b[2], id_neg, 1u);
          mma_tf32_pair(d_re, a[2], b[3], id_neg, 1u);
          mma_tf32_pair(d_re, a[2], b[2], id_neg, 1u);
          mma_tf32_pair(d_im, a[1], b[2], id_pos, acc0);
          mma_tf32_pair(d_im, a[0], b[3], id_pos, 1u);
          mma_tf32_pair(d_im, a[0], b[2], id_pos, 1u);
          mma_tf32_pair(d_im, a[3], b[0], id_pos, 1u);
          mma_tf32_pair(d_im, a[2], b[1], id_pos, 1u);
          mma_tf32_pair(d_im, a[2], b[0], id_pos, 1u);
        }
        mma_commit_pair(&empty_bar[s]);              // frees stage s in both CTAs once these MMAs finish
      }
      if (ok) mma_commit_pair(tmem_bar);
    }
  } else {
    // Epilogue warps 2..5 of each CTA drain that CTA's 128 rows
    const int q = warp & 3;
    int okw = 0;
    if (lane == 0) okw = mbar_wait(tmem_bar, 0, p.err, abort_flag, 3) ? 1 : 0;
    const bool ok = __shfl_sync(0xffffffffu, okw, 0) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok && nk > 0) {
      const int64_t m = (int64_t)tile_m * 256 + rank * 128 + q * 32 + lane;
      const bool use_beta = (p.beta.x != 0.0 || p.beta.y != 0.0);
      const bool unit_alpha = p.alpha.x == 1.0 && p.alpha.y == 0.0;
      const bool unit_beta = p.beta.x == 1.0 && p.beta.y == 0.0;
#pragma unroll 1
      for (int c = 0; c < BN / 32; ++c) {
        float vr[32], vi[32];
        const uint32_t tl = tmem_base + ((uint32_t)(q * 32) << 16) + c * 32;
        tmem_ld32(tl, vr);
        tmem_ld32(tl + BN, vi);
        if (m < p.M) {
          const int64_t n0 = (int64_t)tile_n * BN + c * 32;
          if (p.partial) {
            z64* dst = p.partial + ((int64_t)split * p.M + m) * p.N + n0;
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (n0 + j < p.N) dst[j] = zmk(f2d_exact(vr[j]), f2d_exact(vi[j]));
          } else if (p.c32) {
            float2* dst = (float2*)p.C + m * p.ldc + n0;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              if (n0 + j < p.N) {
                float2 out = make_float2(vr[j], vi[j]);
                if (unit_beta) {
                  const float2 c = dst[j];
                  out.x += c.x;
                  out.y += c.y;
                }
                dst[j] = out;
              }
            }
          } else {
            z64* dst = p.C + m * p.ldc + n0;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              if (n0 + j < p.N) {
                z64 out = zmk(f2d_exact(vr[j]), f2d_exact(vi[j]));
                if (!unit_alpha) out = zmul(p.alpha, out);
                if (unit_beta) out = zadd(out, dst[j]);
                else if (use_beta) out = zadd(out, zmul(p.beta, dst[j]));
                dst[j] = out;
              }
            }
          }
        }
      }
    }
  }
  if (*abort_flag) {
    // after a timed-out wait, give loads still in flight into this CTA time to land
    const long long t0 = clock64();
    while (clock64() - t0 < 2000000LL) {
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  cluster_sync_all();                               // neither CTA frees TMEM while its peer may still use it
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TMEM_COLS));
  }
}

// planes[4][rows][Kp]: re_hi, re_lo, im_hi, im_lo of X(row, k) = src[row*s_row + k*s_k], zero padded.
__global__ void prep_kernel(const z64* __restrict__ src, int64_t nrows, int64_t K, int64_t s_row, int64_t s_k,
                            int conj, int64_t rows_pad, int64_t Kp, int kblk, float* __restrict__ planes) {
  __shared__ z64 tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const bool kfast = (s_k == 1) || (s_row != 1 && s_k <= s_row);
  const int64_t tiles_k = (Kp + 31) / 32, tiles = (rows_pad / 32) * tiles_k;
  const int64_t plane = rows_pad * Kp;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t r0 = (t / tiles_k) * 32, k0 = (t % tiles_k) * 32;
    for (int i = ty; i < 32; i += 8) {
      int64_t r, k;
      if (kfast) { r = r0 + i; k = k0 + tx; } else { r = r0 + tx; k = k0 + i; }
      z64 v = zmk(0, 0);
      if (r < nrows && k < K) {
        if (conj == kSrcReal) v.x = ((const double*)src)[r * s_row + k * s_k];
        else v = src[r * s_row + k * s_k];
      }
      if (conj == 1) v.y = -v.y;
      if (kfast) tile[i][tx] = v; else tile[tx][i] = v;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
      int64_t r = r0 + i, k = k0 + tx;
      if (r >= rows_pad || k >= Kp) continue;
      z64 v = tile[i][tx];
      uint32_t rh, rl, ih, il;
      split_tf32_fast((uint32_t)__double2hiint(v.x), (uint32_t)__double2loint(v.x), rh, rl);
      split_tf32_fast((uint32_t)__double2hiint(v.y), (uint32_t)__double2loint(v.y), ih, il);
      const int64_t off = kblk ? ((k >> 4) * rows_pad + r) * 16 + (k & 15) : r * Kp + k;
      planes[off] = __uint_as_float(rh);
      planes[plane + off] = __uint_as_float(rl);
      planes[2 * plane + off] = __uint_as_float(ih);
      planes[3 * plane + off] = __uint_as_float(il);
    }
    __syncthreads();
  }
}

__global__ void splitk_sum_kernel(const z64* __restrict__ partial, int splits, int64_t M, int64_t N, z64 alpha,
                                  z64 beta, z64* C, int64_t ldc, int trans_c) {
  int64_t total = M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    // e runs along C's rows in memory: (m, n) for a row-major C, (n, m) for a transposed one
    int64_t m, n;
    if (trans_c) { n = e / M; m = e % M; } else { m = e / N; n = e % N; }
    const int64_t pe = m * N + n;
    z64 s = zmk(0, 0);
    for (int z = 0; z < splits; ++z) s = zadd(s, partial[(int64_t)z * total + pe]);
    z64* c = trans_c ? C + n * ldc + m : C + m * ldc + n;
    z64 out = zmul(alpha, s);
    if (beta.x != 0.0 || beta.y != 0.0) out = zadd(out, zmul(beta, *c));
    *c = out;
  }
}

int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

PFN_cuTensorMapEncodeTiled_v12000 get_encode() { return tma_encode_fn(); }

// K-blocked planes [4][Kp/16][rows_pad][16] as a 3D tensor (16 k, rows_pad rows, 4 Kp/16 plane-k-blocks):
// a box of 16 k x box_rows rows is one contiguous run.
bool encode_planes_kblk(CUtensorMap* map, float* base, int64_t rows_pad, int64_t Kp, int box_rows) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[3] = {16u, (cuuint64_t)rows_pad, (cuuint64_t)(4 * (Kp / 16))};
  cuuint64_t strides[2] = {16u * sizeof(float), (cuuint64_t)rows_pad * 16u * sizeof(float)};
  cuuint32_t box[3] = {16u, (cuuint32_t)box_rows, 1u};
  cuuint32_t estr[3] = {1u, 1u, 1u};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

bool encode_planes(CUtensorMap* map, float* base, int64_t rows_total, int64_t Kp, int box_rows, int kb) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows_total};
  cuuint64_t strides[1] = {(cuuint64_t)(Kp * sizeof(float))};
  cuuint32_t box[2] = {(cuuint32_t)kb, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1u, 1u};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, kb == 16 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// The CTA-pair kernel for large outputs (both extents at least 1024, no K split): its
// 256-row pair tiles would mostly compute padding on a short M.
bool use_pair(int64_t M, int64_t N, int splits) { return M >= 1024 && N >= 1024 && splits == 1; }

}  // namespace

// Plane rows are padded to the 256-row tile edge, or to 64 rows for operands of at most 64
// rows (the narrow B tile), so one layout serves as A or B.  A 128-row A tile over a 64-row
// plane reads past it (the next plane, or zeros beyond the last): those rows only feed
// output rows >= M, which are never stored; a 256-row B tile over it likewise.
int64_t tf32_rows_pad(int64_t rows) { return rows <= 64 ? 64 : round_up(rows, BN); }
int64_t tf32_k_pad(int64_t K) { return round_up(K, BK); }
size_t tf32_planes_bytes(int64_t rows, int64_t K) {
  return (size_t)4 * (size_t)tf32_rows_pad(rows) * (size_t)tf32_k_pad(K) * sizeof(float);
}

// Split an FP64 complex operand X(row,k) = src[row*s_row + k*s_k] into the four
// zero-padded K-major TF32 planes the tensor-core kernel reads.
// kblk: K-blocked layout [4][Kp/16][rows_pad][16] (for GEMMs whose K is long and whose rows,
// Kp apart in the plain layout, would each cost the TMA a separate DRAM page per k-block).
agb_status tf32_prep_planes(const z64* src, int64_t rows, int64_t K, int64_t s_row, int64_t s_k, int conj,
                            float* dst, cudaStream_t stream, int kblk) {
  int64_t rp = tf32_rows_pad(rows), kp = tf32_k_pad(K);
  int64_t tiles = (rp / 32) * ((kp + 31) / 32);
  int grid = (int)(tiles < 152 * 32 ? tiles : 152 * 32);
  prep_kernel<<<grid, 256, 0, stream>>>(src, rows, K, s_row, s_k, conj, rp, kp, kblk, dst);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

namespace {
// Tile width of the single-CTA kernel for an N-wide output.
int tile_n_for(int64_t N) { return N <= 64 ? 64 : (N <= 160 ? 160 : BN); }

int choose_splits(int64_t M, int64_t N, int64_t nkb, size_t partial_cap) {
  const int nb = tile_n_for(N);
  int64_t tiles = (round_up(M, BM) / BM) * (round_up(N, nb) / nb);
  if (tiles >= 152 || nkb < 16) return 1;
  int64_t want = (2 * 152 + tiles - 1) / tiles;
  int64_t kmax = nkb / 8;
  if (want > kmax) want = kmax;
  if (want > 152) want = 152;
  int64_t fit = (int64_t)(partial_cap / ((size_t)M * N * sizeof(z64)));
  if (want > fit) want = fit;
  return want < 2 ? 1 : (int)want;
}
}  // namespace

// Bytes of split-K partials a planes GEMM may use (0 when no split is chosen).
size_t tf32_partials_bytes(int64_t M, int64_t N, int64_t K) {
  int64_t nkb = tf32_k_pad(K) / BK;
  int s = choose_splits(M, N, nkb, (size_t)-1 / 2);
  return s > 1 ? (size_t)s * M * N * sizeof(z64) : 0;
}

// C = alpha * A B^T + beta C on prepared planes (A: rows M, B: rows N, both K-major over K).
// trans_c: C(m, n) lives at C[n * ldc + m] (the output written column by column, which keeps
// the stores of an output with a short row extent coalesced).
// kblkA / kblkB: that operand's planes are K-blocked (single-CTA kernel only).  c32: C holds
// complex FP32 values (ldc in float2 units), alpha = 1, beta 0 or 1, no K split.  timing:
// when not null, CUDA events around the GEMM kernel are appended to it (the caller's log).
agb_status tf32_gemm_planes(int64_t M, int64_t N, int64_t K, z64 alpha, const float* PA, const float* PB, z64 beta,
                            z64* C, int64_t ldc, int* err, z64* partials, size_t partial_bytes, cudaStream_t stream,
                            int trans_c, int kblkA, int kblkB, int c32, GemmTimingLog* timing) {
  AGB_ARG_CHECK(M >= 0 && N >= 0 && K > 0, "tf32_gemm_planes: bad size");
  if (M == 0 || N == 0) return AGB_OK;
  AGB_ARG_CHECK(PA && PB && C && err, "tf32_gemm_planes: null pointer");
  constexpr int kb = 16;
  const int64_t Mp = tf32_rows_pad(M), Np = tf32_rows_pad(N), Kp = tf32_k_pad(K), nkb = Kp / kb;
  AGB_ARG_CHECK(Mp / BM <= 65535, "tf32_gemm_planes: grid too large");
  AGB_ARG_CHECK(!c32 || (alpha.x == 1.0 && alpha.y == 0.0 && beta.y == 0.0 && (beta.x == 0.0 || beta.x == 1.0)),
                "tf32_gemm_planes: an FP32 output takes alpha = 1 and beta = 0 or 1");
  int splits = (partials && !c32) ? choose_splits(M, N, Kp / BK, partial_bytes) : 1;
  int nkb_split = (int)((nkb + splits - 1) / splits);
  splits = (int)((nkb + nkb_split - 1) / nkb_split);
  const bool pair = use_pair(M, N, splits) && !trans_c && !kblkA && !kblkB;
  const int nb = tile_n_for(N);
  CUtensorMap mA, mB;
  const bool okA = kblkA ? encode_planes_kblk(&mA, (float*)PA, Mp, Kp, BM) : encode_planes(&mA, (float*)PA, 4 * Mp, Kp, BM, kb);
  const bool okB = kblkB ? encode_planes_kblk(&mB, (float*)PB, Np, Kp, nb)
                         : encode_planes(&mB, (float*)PB, 4 * Np, Kp, pair ? 128 : nb, kb);
  if (!okA || !okB) {
    agb_set_error_message("tf32_gemm_planes: cuTensorMapEncodeTiled failed", __FILE__, __LINE__);
    return AGB_ERR_CUDA;
  }
  static std::atomic<uint64_t> attr_done{0};
  AGB_STATUS_TRY(once_per_device(attr_done, [&]() -> agb_status {
    AGB_CUDA_TRY(cudaFuncSetAttribute(tf32x3_gemm_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile<256>::SMEM_BYTES));
    AGB_CUDA_TRY(cudaFuncSetAttribute(tf32x3_gemm_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile<64>::SMEM_BYTES));
    AGB_CUDA_TRY(cudaFuncSetAttribute(tf32x3_gemm_kernel<160>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile<160>::SMEM_BYTES));
    AGB_CUDA_TRY(cudaFuncSetAttribute(tf32x3_gemm2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      P2_SMEM_BYTES));
    return AGB_OK;
  }));
  GemmParams p;
  p.M = M; p.N = N; p.nkb = nkb_split; p.nkb_total = (int)nkb;
  p.alpha = alpha; p.beta = beta; p.C = C; p.ldc = ldc; p.partial = splits > 1 ? partials : nullptr; p.err = err;
  p.rowsA = Mp; p.rowsB = Np; p.trans_c = trans_c; p.kblkA = kblkA; p.kblkB = kblkB; p.c32 = c32;
  dim3 grid((unsigned)(round_up(N, nb) / nb), (unsigned)(round_up(M, BM) / BM), (unsigned)splits);
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (timing) {
    AGB_CUDA_TRY(cudaEventCreate(&ev0));
    AGB_CUDA_TRY(cudaEventCreate(&ev1));
    AGB_CUDA_TRY(cudaEventRecord(ev0, stream));
  }
  if (pair) {
    AGB_ARG_CHECK(Mp / 256 <= 65535, "tf32_gemm_planes: grid too large");
    const dim3 grid2((unsigned)(2 * (Np / 256)), (unsigned)(Mp / 256), (unsigned)splits);
    tf32x3_gemm2_kernel<<<grid2, THREADS, P2_SMEM_BYTES, stream>>>(mA, mB, p);
  } else {
    if (nb == 64) tf32x3_gemm_kernel<64><<<grid, THREADS, Tile<64>::SMEM_BYTES, stream>>>(mA, mB, p);
    else if (nb == 160) tf32x3_gemm_kernel<160><<<grid, THREADS, Tile<160>::SMEM_BYTES, stream>>>(mA, mB, p);
    else tf32x3_gemm_kernel<256><<<grid, THREADS, Tile<256>::SMEM_BYTES, stream>>>(mA, mB, p);
  }
  AGB_LAUNCH_CHECK();
  if (ev0) {
    AGB_CUDA_TRY(cudaEventRecord(ev1, stream));
    timing->push_back(GemmTimingRec{ev0, ev1, 8.0 * (double)M * (double)N * (double)K, M, N, K});
  }
  if (splits > 1) {
    splitk_sum_kernel<<<grid_for(M * N, 256), 256, 0, stream>>>(partials, splits, M, N, alpha, beta, C, ldc,
                                                                 trans_c);
    AGB_LAUNCH_CHECK();
  }
  return AGB_OK;
}

// C = alpha op(A) op(B) + beta C with A read as FP64 by the kernel's converter warps (no A
// planes): scratch = [256-byte status header][B planes].  For outputs up to 256 wide.
size_t cgemm_tf32x3_fa_scratch(int64_t N, int64_t K) {
  return 256 + round_up((int64_t)tf32_planes_bytes(N, K), 256);
}

agb_status cgemm_tf32x3_fa(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk,
                           int conjA, const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C,
                           int64_t ldc, void* scratch, size_t scratch_bytes, cudaStream_t stream) {
  AGB_ARG_CHECK(M >= 0 && N >= 0 && K >= 0, "cgemm_tf32x3_fa: negative size");
  if (M == 0 || N == 0) return AGB_OK;
  AGB_ARG_CHECK(K > 0 && N <= BN, "cgemm_tf32x3_fa: K must be positive and N at most 256");
  AGB_ARG_CHECK(A && B && C && scratch && ((uintptr_t)scratch & 255) == 0, "cgemm_tf32x3_fa: bad pointer");
  if (scratch_bytes < cgemm_tf32x3_fa_scratch(N, K)) {
    agb_set_error_message("cgemm_tf32x3_fa: scratch too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  const int64_t Mp = round_up(M, BM), Np = tf32_rows_pad(N), Kp = tf32_k_pad(K);
  char* base = (char*)scratch;
  float* PB = (float*)(base + 256);
  AGB_STATUS_TRY(tf32_prep_planes(B, N, K, sBn, sBk, conjB, PB, stream, 0));
  const int nb = tile_n_for(N);
  CUtensorMap mB;
  if (!encode_planes(&mB, PB, 4 * Np, Kp, nb, BK)) {
    agb_set_error_message("cgemm_tf32x3_fa: cuTensorMapEncodeTiled failed", __FILE__, __LINE__);
    return AGB_ERR_CUDA;
  }
  AGB_CUDA_TRY(cudaFuncSetAttribute(tf32x3_gemm_fa_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    FaTile<64>::SMEM_BYTES));
  AGB_CUDA_TRY(cudaFuncSetAttribute(tf32x3_gemm_fa_kernel<160>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    FaTile<160>::SMEM_BYTES));
  AGB_CUDA_TRY(cudaFuncSetAttribute(tf32x3_gemm_fa_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    FaTile<256>::SMEM_BYTES));
  FaParams p;
  p.M = M; p.N = N; p.K = K; p.A = A; p.sAm = sAm; p.sAk = sAk; p.conjA = conjA; p.nkb = (int)(Kp / BK);
  p.ntiles = Mp / BM;
  p.alpha = alpha; p.beta = beta; p.C = C; p.ldc = ldc; p.err = (int*)base; p.rowsB = Np;
  int dev = 0, nsm = 0;
  AGB_CUDA_TRY(cudaGetDevice(&dev));
  AGB_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const unsigned grid = (unsigned)(p.ntiles < nsm ? p.ntiles : nsm);   // one persistent CTA per SM
  if (nb == 64) tf32x3_gemm_fa_kernel<64><<<grid, FA_THREADS, FaTile<64>::SMEM_BYTES, stream>>>(mB, p);
  else if (nb == 160) tf32x3_gemm_fa_kernel<160><<<grid, FA_THREADS, FaTile<160>::SMEM_BYTES, stream>>>(mB, p);
  else tf32x3_gemm_fa_kernel<256><<<grid, FA_THREADS, FaTile<256>::SMEM_BYTES, stream>>>(mB, p);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

// Scratch layout of the all-in-one entry: [256-byte status header][A planes][B planes][split-K partials].
size_t cgemm_tf32x3_scratch(int64_t M, int64_t N, int64_t K) {
  if (M <= 0 || N <= 0 || K <= 0) return 256;
  return 256 + round_up((int64_t)tf32_planes_bytes(M, K), 256) + round_up((int64_t)tf32_planes_bytes(N, K), 256) +
         tf32_partials_bytes(M, N, K);
}

agb_status cgemm_tf32x3(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk,
                        int conjA, const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                        void* scratch, size_t scratch_bytes, cudaStream_t stream) {
  AGB_ARG_CHECK(M >= 0 && N >= 0 && K >= 0, "cgemm_tf32x3: negative size");
  if (M == 0 || N == 0) return AGB_OK;
  AGB_ARG_CHECK(A && B && C && scratch, "cgemm_tf32x3: null pointer");
  AGB_ARG_CHECK(((uintptr_t)scratch & 255) == 0, "cgemm_tf32x3: scratch must be 256-byte aligned");
  if (K == 0) return zgemm(M, N, 0, zmk(0, 0), A, sAm, sAk, 0, B, sBk, sBn, 0, beta, C, ldc, stream);
  size_t a_bytes = round_up((int64_t)tf32_planes_bytes(M, K), 256);
  size_t b_bytes = round_up((int64_t)tf32_planes_bytes(N, K), 256);
  if (scratch_bytes < 256 + a_bytes + b_bytes) {
    agb_set_error_message("cgemm_tf32x3: scratch too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  char* base = (char*)scratch;
  float* PA = (float*)(base + 256);
  float* PB = (float*)(base + 256 + a_bytes);
  AGB_STATUS_TRY(tf32_prep_planes(A, M, K, sAm, sAk, conjA, PA, stream, 0));
  AGB_STATUS_TRY(tf32_prep_planes(B, N, K, sBn, sBk, conjB, PB, stream, 0));
  size_t used = 256 + a_bytes + b_bytes;
  return tf32_gemm_planes(M, N, K, alpha, PA, PB, beta, C, ldc, (int*)base, (z64*)(base + used),
                          scratch_bytes - used, stream, 0, 0, 0, 0, nullptr);
}

}  // namespace agb

extern "C" {

size_t agb_cgemm_tf32x3_scratch_bytes(int64_t M, int64_t N, int64_t K) { return agb::cgemm_tf32x3_scratch(M, N, K); }

agb_status agb_cgemm_tf32x3(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im, const void* A,
                            int64_t sAm, int64_t sAk, int conjA, const void* B, int64_t sBk, int64_t sBn, int conjB,
                            double beta_re, double beta_im, void* C, int64_t ldc, void* scratch, size_t scratch_bytes,
                            void* stream) {
  AGB_ARG_CHECK((conjA == 0 || conjA == 1) && (conjB == 0 || conjB == 1), "gemm: conj flags must be 0 or 1");
  AGB_ARG_CHECK(M <= 1 || N <= 0 || ldc >= N, "gemm: ldc must be at least N (C is row-major)");
  return agb::cgemm_tf32x3(M, N, K, agb::zmk(alpha_re, alpha_im), (const agb::z64*)A, sAm, sAk, conjA,
                           (const agb::z64*)B, sBk, sBn, conjB, agb::zmk(beta_re, beta_im), (agb::z64*)C, ldc,
                           scratch, scratch_bytes, (cudaStream_t)stream);
}


/* Reads and clears the error word a 3xTF32 GEMM keeps at the start of its scratch
 * (non-zero: a bounded wait inside the kernel ran out). Synchronises the stream. */
agb_status agb_scratch_status(void* scratch, void* stream) {
  if (!scratch) return AGB_ERR_ARG;
  int h = 0;
  AGB_CUDA_TRY(cudaMemcpyAsync(&h, scratch, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  AGB_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  if (h != 0) {
    AGB_CUDA_TRY(cudaMemsetAsync(scratch, 0, sizeof(int), (cudaStream_t)stream));
    agb_set_error_message("tcgen05 GEMM: a bounded wait timed out", __FILE__, __LINE__);
    return AGB_ERR_TIMEOUT;
  }
  return AGB_OK;
}

}  // extern "C"
