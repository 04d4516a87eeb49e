// Spin-orbital CISD / CID residual on the GPU: block builders, per-iteration
// amplitude layouts, the residual as a sequence of complex GEMMs plus one
// packed assembly kernel, the amplitude update, DIIS dot products and the
// fused DIIS combination / energy / norm reduction.
//
// Amplitudes are kept packed: t2p[p(i<j)][p(a<b)] = t2[i,j,a,b].  Every
// quantity of the reference with full (i,j,a,b) ranges is recovered through
// the antisymmetry t2[i,j,a,b] = -t2[j,i,a,b] = -t2[i,j,b,a]; the full-vector
// sums of the reference (energy, DIIS Gram, rms) equal 4x the packed sums.
#include <cuda.h>

#include <vector>
#include <string>
#include <mutex>
#include <atomic>

#include "cisd_plan.h"
#include "dfloat.cuh"

namespace agb {

agb_status zgemm_ex(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                    const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                    void* scratch, size_t scratch_bytes, cudaStream_t stream);
agb_status dfgemm_ex(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                     const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                     void* scratch, size_t scratch_bytes, cudaStream_t stream);
agb_status zgemv(int64_t M, int64_t K, z64 alpha, const z64* A, int64_t lda, const z64* x, z64 beta, z64* y,
                 cudaStream_t stream);
agb_status zgemv_f32(int64_t M, int64_t K, z64 alpha, const z64* A, int64_t lda, const z64* x, z64 beta, z64* y,
                     cudaStream_t stream);
agb_status zgemv_df(int64_t M, int64_t K, z64 alpha, const z64* A, int64_t lda, const z64* x, z64 beta, z64* y,
                    cudaStream_t stream);
agb_status cgemm_tf32x3(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk,
                        int conjA, const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                        void* scratch, size_t scratch_bytes, cudaStream_t stream);
size_t cgemm_tf32x3_scratch(int64_t M, int64_t N, int64_t K);
size_t tf32_planes_bytes(int64_t rows, int64_t K);
int64_t tf32_rows_pad(int64_t rows);
int64_t tf32_k_pad(int64_t K);
size_t tf32_partials_bytes(int64_t M, int64_t N, int64_t K);
size_t dfgemm_scratch_bytes(int64_t M, int64_t N, int64_t K);
size_t ozgemm_scratch_bytes(int64_t M, int64_t N, int64_t K);
int64_t ozgemm_tiles(int64_t M, int64_t N);
agb_status ozgemm_ex(int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm, int64_t sAk, int conjA,
                     const z64* B, int64_t sBk, int64_t sBn, int conjB, z64 beta, z64* C, int64_t ldc,
                     void* scratch, size_t scratch_bytes, cudaStream_t stream);
// GEMMs with at least this many 128x128 output tiles take the Ozaki tensor-core path in
// AGB_PREC_OZAKI mode; smaller ones (few tiles, long K) the split-K double-float kernel.
constexpr int64_t kOzMinTiles = 152;
agb_status tf32_prep_planes(const z64* src, int64_t rows, int64_t K, int64_t s_row, int64_t s_k, int conj,
                            float* dst, cudaStream_t stream, int kblk);
agb_status tf32_gemm_planes(int64_t M, int64_t N, int64_t K, z64 alpha, const float* PA, const float* PB, z64 beta,
                            z64* C, int64_t ldc, int* err, z64* partials, size_t partial_bytes, cudaStream_t stream,
                            int trans_c, int kblkA, int kblkB, int c32, GemmTimingLog* timing);

namespace {

// ----------------------------------------------------------------- blocks --

enum BlockId { B_R0p = 0, B_Wop, B_VT, B_Wvovv, B_Wooov, B_Wovoo, B_Wvvvo, B_Woooo, B_Wvvvv, B_COUNT };
// Orbital-range letters of each block's <PQ||RS> (o = occupied, v = virtual).
const char* kBlockRanges[B_COUNT] = {"vvoo", "oovv", "ovvo", "vovv", "ooov", "ovoo", "vvvo", "oooo", "vvvv"};

struct Dims {
  int o, v;
  int64_t ov, po, pv;
  const int2* opairs;
  const int2* vpairs;
};

// Output element e of block id -> spin-orbital indices (P,Q,R,S) of <PQ||RS>.
__device__ __forceinline__ void block_indices(int id, int64_t e, const Dims& d, int& P, int& Q, int& R, int& S) {
  const int o = d.o, v = d.v;
  switch (id) {
    case B_R0p: {  // [p(ij)][p(ab)] <ab||ij>
      int2 ij = d.opairs[e / d.pv], ab = d.vpairs[e % d.pv];
      P = o + ab.x; Q = o + ab.y; R = ij.x; S = ij.y; break;
    }
    case B_Wop: {  // [p(ij)][p(ab)] <ij||ab>
      int2 ij = d.opairs[e / d.pv], ab = d.vpairs[e % d.pv];
      P = ij.x; Q = ij.y; R = o + ab.x; S = o + ab.y; break;
    }
    case B_VT: {  // [(j,b)][(k,c)] <kb||cj>
      int64_t row = e / d.ov, col = e % d.ov;
      int j = (int)(row / v), b = (int)(row % v), k = (int)(col / v), c = (int)(col % v);
      P = k; Q = o + b; R = o + c; S = j; break;
    }
    case B_Wvovv: {  // [a][j][p(cb)] <aj||cb>
      int2 cb = d.vpairs[e % d.pv];
      int64_t rest = e / d.pv;
      int j = (int)(rest % o), a = (int)(rest / o);
      P = o + a; Q = j; R = o + cb.x; S = o + cb.y; break;
    }
    case B_Wooov: {  // [i][p(kj)][b] <kj||ib>
      int b = (int)(e % v);
      int64_t rest = e / v;
      int2 kj = d.opairs[rest % d.po];
      int i = (int)(rest / d.po);
      P = kj.x; Q = kj.y; R = i; S = o + b; break;
    }
    case B_Wovoo: {  // [p(ij)][b][k] <kb||ij>
      int k = (int)(e % o);
      int64_t rest = e / o;
      int b = (int)(rest % v);
      int2 ij = d.opairs[rest / v];
      P = k; Q = o + b; R = ij.x; S = ij.y; break;
    }
    case B_Wvvvo: {  // [c][j][p(ab)] <ab||cj>
      int2 ab = d.vpairs[e % d.pv];
      int64_t rest = e / d.pv;
      int j = (int)(rest % o), c = (int)(rest / o);
      P = o + ab.x; Q = o + ab.y; R = o + c; S = j; break;
    }
    case B_Woooo: {  // [p(ij)][p(kl)] <kl||ij>
      int2 ij = d.opairs[e / d.po], kl = d.opairs[e % d.po];
      P = kl.x; Q = kl.y; R = ij.x; S = ij.y; break;
    }
    default: {  // B_Wvvvv [p(ab)][p(cd)] <ab||cd>
      int2 ab = d.vpairs[e / d.pv], cd = d.vpairs[e % d.pv];
      P = o + ab.x; Q = o + ab.y; R = o + cd.x; S = o + cd.y; break;
    }
  }
}

int64_t block_elems(int id, const agb_cisd_plan* p) {
  switch (id) {
    case B_R0p: case B_Wop: return p->po * p->pv;
    case B_VT: return p->ov * p->ov;
    case B_Wvovv: return (int64_t)p->v * p->o * p->pv;
    case B_Wooov: return (int64_t)p->o * p->po * p->v;
    case B_Wovoo: return p->po * p->v * p->o;
    case B_Wvvvo: return (int64_t)p->v * p->o * p->pv;
    case B_Woooo: return p->po * p->po;
    default: return p->pv * p->pv;
  }
}

// Chemist sources (pq|rs) in spin orbitals.
struct SrcMO {  // spatial ERI_MO[n^4] with the spin integration of compute_ERI_SO
  const z64* g; int64_t n;
  __device__ __forceinline__ z64 chem(int p, int q, int r, int s) const {
    if (((p ^ q) & 1) || ((r ^ s) & 1)) return zmk(0, 0);
    return g[(((int64_t)(p >> 1) * n + (q >> 1)) * n + (r >> 1)) * n + (s >> 1)];
  }
};
struct SrcSO {  // full spin-orbital chemist tensor
  const z64* g; int64_t n;
  __device__ __forceinline__ z64 chem(int p, int q, int r, int s) const {
    return g[(((int64_t)p * n + q) * n + r) * n + s];
  }
};
struct SrcChem {  // chemist sub-block over index ranges [off_i, off_i + len_i)
  const z64* g; int off0, off1, off2, off3; int64_t len1, len2, len3;
  __device__ __forceinline__ z64 chem(int p, int q, int r, int s) const {
    return g[((((int64_t)(p - off0)) * len1 + (q - off1)) * len2 + (r - off2)) * len3 + (s - off3)];
  }
};

template <class SD, class SE>
__global__ void build_block_kernel(int id, Dims d, int64_t total, SD sd, SE se, z64* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int P, Q, R, S;
    block_indices(id, e, d, P, Q, R, S);
    // <PQ||RS> = (PR|QS) - (PS|QR)
    out[e] = zsub(sd.chem(P, R, Q, S), se.chem(P, S, Q, R));
  }
}

// Bsub[(x,y)][L] = Bf[L][x0+x][y0+y]
__global__ void extract_factor_kernel(const z64* __restrict__ Bf, int64_t naux, int64_t nso, int x0, int nx, int y0,
                                      int ny, z64* __restrict__ out) {
  int64_t total = (int64_t)nx * ny * naux;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t L = e % naux, xy = e / naux;
    int64_t x = xy / ny, y = xy % ny;
    out[e] = Bf[(L * nso + x0 + x) * nso + y0 + y];
  }
}

// ------------------------------------------------------- Fock and tables --

__global__ void fock_extract_kernel(const z64* __restrict__ F, const double* __restrict__ eps_in, int o, int v,
                                    z64* FvoT, z64* Foo, z64* Fvv, z64* Fov, double* eps, int* offdiag) {
  int nso = o + v;
  int64_t total = (int64_t)nso * nso;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int p = (int)(e / nso), q = (int)(e % nso);
    z64 f = F[e];
    if (p < o && q < o) {
      Foo[p * o + q] = f;
      if (p != q && (f.x != 0.0 || f.y != 0.0)) atomicOr(offdiag, 1);
    } else if (p >= o && q >= o) {
      Fvv[(p - o) * v + (q - o)] = f;
      if (p != q && (f.x != 0.0 || f.y != 0.0)) atomicOr(offdiag, 1);
    } else if (p < o) {
      if (Fov) Fov[p * v + (q - o)] = f;
    } else {
      if (FvoT) FvoT[q * v + (p - o)] = f;  // F[a,i] at [i][a]
    }
    if (e < nso) eps[e] = eps_in[e];
  }
}

// ------------------------------------------------- per-iteration layouts --

__device__ __forceinline__ int sgn_pair(int x, int y) { return x < y ? 1 : (x > y ? -1 : 0); }

// Tring[(i,a)][(k,c)] = t2[i,k,a,c]
__global__ void unpack_ring_kernel(const z64* __restrict__ t2p, int o, int v, int64_t pv, z64* __restrict__ out) {
  int64_t ov = (int64_t)o * v, total = ov * ov;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t row = e / ov, col = e % ov;
    int i = (int)(row / v), a = (int)(row % v), k = (int)(col / v), c = (int)(col % v);
    int s = sgn_pair(i, k) * sgn_pair(a, c);
    z64 val = zmk(0, 0);
    if (s != 0) {
      int64_t p = pair_index(min(i, k), max(i, k), o), q = pair_index(min(a, c), max(a, c), v);
      val = t2p[p * pv + q];
      if (s < 0) val = zneg(val);
    }
    out[e] = val;
  }
}

// The ring GEMM's A operand straight from the packed amplitudes, as the four zero-padded
// K-major TF32 planes the tensor-core GEMM reads (re_hi, re_lo, im_hi, im_lo of
// Tring[(i,a)][(k,c)] = t2[i,k,a,c]), for 3xTF32 residuals: no FP64 Tring is written and
// re-read by a separate operand split.  One warp per row (i,a), lanes along (k,c), so the
// plane writes are coalesced; with Fov it also forms the singles term
// r1x[(i,a)] = sum_(k,c) t2[i,k,a,c] F_kc (apyib/ci_wfn.py:313, F_jb t2_ijab) from the values
// it has just unpacked, in FP32 (the 3xTF32 residual's own level).
__global__ void unpack_ring_planes_kernel(const z64* __restrict__ t2p, int o, int v, int64_t pv, int64_t rows_pad,
                                          int64_t Kp, const z64* __restrict__ Fov, z64* __restrict__ r1x,
                                          float* __restrict__ planes) {
  const int lane = threadIdx.x & 31;
  const int64_t ov = (int64_t)o * v, plane = rows_pad * Kp;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = warp; row < rows_pad; row += nwarps) {
    const bool live = row < ov;
    const int i = live ? (int)(row / v) : 0, a = live ? (int)(row % v) : 0;
    float re = 0.f, im = 0.f;
    // (k, c) of col, advanced by 32 per pass without divisions; pair offsets in 32-bit
    // (o, v < 2^15 keeps p(ab) and p(ik) below 2^31)
    int k = v > 0 ? lane / v : 0, c = v > 0 ? lane % v : 0;
    for (int64_t col = lane; col < Kp; col += 32) {
      z64 val = zmk(0, 0);
      const bool in = live && col < ov;
      if (in) {
        const int sg = sgn_pair(i, k) * sgn_pair(a, c);
        if (sg != 0) {
          const int lo = min(i, k), hi = max(i, k), la = min(a, c), ha = max(a, c);
          const int pik = lo * o - lo * (lo + 1) / 2 + (hi - lo - 1);
          const int pac = la * v - la * (la + 1) / 2 + (ha - la - 1);
          val = t2p[(int64_t)pik * pv + pac];
          if (sg < 0) val = zneg(val);
        }
      }
      c += 32;
      while (v > 0 && c >= v) {
        c -= v;
        ++k;
      }
      uint32_t rh, rl, ih, il;
      split_tf32_fast((uint32_t)__double2hiint(val.x), (uint32_t)__double2loint(val.x), rh, rl);
      split_tf32_fast((uint32_t)__double2hiint(val.y), (uint32_t)__double2loint(val.y), ih, il);
      const int64_t e = row * Kp + col;
      planes[e] = __uint_as_float(rh);
      planes[plane + e] = __uint_as_float(rl);
      planes[2 * plane + e] = __uint_as_float(ih);
      planes[3 * plane + e] = __uint_as_float(il);
      if (Fov && in) {
        const float tr = __uint_as_float(rh) + __uint_as_float(rl), ti = __uint_as_float(ih) + __uint_as_float(il);
        const float4 f = split_z_fast(Fov[col]);
        re = fmaf(tr, f.x, re);
        re = fmaf(-ti, f.z, re);
        im = fmaf(tr, f.z, im);
        im = fmaf(ti, f.x, im);
      }
    }
    if (Fov && live) {
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, off);
        im += __shfl_xor_sync(0xffffffffu, im, off);
      }
      if (lane == 0) r1x[row] = zmk(f2d_exact(re), f2d_exact(im));
    }
  }
}

// t2h[i][j][q] = t2[i,j,(a<b)_q]
__global__ void unpack_h_kernel(const z64* __restrict__ t2p, int o, int64_t pv, z64* __restrict__ out) {
  int64_t total = (int64_t)o * o * pv;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = e % pv, ij = e / pv;
    int i = (int)(ij / o), j = (int)(ij % o);
    int s = sgn_pair(i, j);
    z64 val = zmk(0, 0);
    if (s != 0) {
      val = t2p[pair_index(min(i, j), max(i, j), o) * pv + q];
      if (s < 0) val = zneg(val);
    }
    out[e] = val;
  }
}

// t2q[p][a][b] = t2[(i<j)_p, a, b]
// Offset of (row, k) in one TF32 plane: K-blocked [k/16][row][16] or plain [row][Kp].
__device__ __forceinline__ int64_t plane_off(int64_t row, int64_t k, int64_t rows_pad, int64_t Kp, int kblk) {
  return kblk ? ((k >> 4) * rows_pad + row) * 16 + (k & 15) : row * Kp + k;
}
// (row, k) of the plane element at offset e (the inverse of plane_off).
__device__ __forceinline__ void plane_pos(int64_t e, int64_t rows_pad, int64_t Kp, int kblk, int64_t& row,
                                          int64_t& k) {
  if (kblk) {
    const int64_t blk = e / (rows_pad * 16), rem = e % (rows_pad * 16);
    row = rem >> 4;
    k = blk * 16 + (rem & 15);
  } else {
    row = e / Kp;
    k = e % Kp;
  }
}

__device__ __forceinline__ void write_planes4(float* planes, int64_t plane, int64_t e, z64 val) {
  uint32_t rh, rl, ih, il;
  split_tf32_fast((uint32_t)__double2hiint(val.x), (uint32_t)__double2loint(val.x), rh, rl);
  split_tf32_fast((uint32_t)__double2hiint(val.y), (uint32_t)__double2loint(val.y), ih, il);
  planes[e] = __uint_as_float(rh);
  planes[plane + e] = __uint_as_float(rl);
  planes[2 * plane + e] = __uint_as_float(ih);
  planes[3 * plane + e] = __uint_as_float(il);
}

// The TF32 planes of the singles GEMMs' amplitude operands straight from the packed
// amplitudes (3xTF32 residuals with a diagonal Fock matrix, where no FP64 t2h / t2q is
// needed): t2h as rows i, k = (j, p(ab)) -> t2[i,j,(a<b)]; t2q as rows a, k = (p(ij), b) ->
// t2[i,j,b,a].  Threads run over plane offsets, so the writes are coalesced in either layout.
__global__ void unpack_h_planes_kernel(const z64* __restrict__ t2p, int o, int64_t pv, int64_t rows_pad, int64_t Kp,
                                       int kblk, float* __restrict__ planes) {
  const int64_t plane = rows_pad * Kp, K = (int64_t)o * pv;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < plane; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t row, k;
    plane_pos(e, rows_pad, Kp, kblk, row, k);
    z64 val = zmk(0, 0);
    if (row < o && k < K) {
      const int i = (int)row, j = (int)(k / pv);
      const int s = sgn_pair(i, j);
      if (s != 0) {
        val = t2p[pair_index(min(i, j), max(i, j), o) * pv + k % pv];
        if (s < 0) val = zneg(val);
      }
    }
    write_planes4(planes, plane, e, val);
  }
}

__global__ void unpack_q_planes_kernel(const z64* __restrict__ t2p, int64_t po, int v, int64_t pv, int64_t rows_pad,
                                       int64_t Kp, int kblk, float* __restrict__ planes) {
  const int64_t plane = rows_pad * Kp, K = po * v;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < plane; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t row, k;
    plane_pos(e, rows_pad, Kp, kblk, row, k);
    z64 val = zmk(0, 0);
    if (row < v && k < K) {
      const int a = (int)row, b = (int)(k % v);
      const int s = sgn_pair(b, a);
      if (s != 0) {
        val = t2p[(k / v) * pv + pair_index(min(a, b), max(a, b), v)];
        if (s < 0) val = zneg(val);
      }
    }
    write_planes4(planes, plane, e, val);
  }
}

__global__ void unpack_q_kernel(const z64* __restrict__ t2p, int64_t po, int v, int64_t pv, z64* __restrict__ out) {
  int64_t vv = (int64_t)v * v, total = po * vv;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t p = e / vv, ab = e % vv;
    int a = (int)(ab / v), b = (int)(ab % v);
    int s = sgn_pair(a, b);
    z64 val = zmk(0, 0);
    if (s != 0) {
      val = t2p[p * pv + pair_index(min(a, b), max(a, b), v)];
      if (s < 0) val = zneg(val);
    }
    out[e] = val;
  }
}

// y = x (or 0) , optionally y -= E*t
// r = src (or 0), plus add (when given)
__global__ void r1_init_kernel(const z64* __restrict__ src, const z64* __restrict__ add, int64_t n,
                               z64* __restrict__ r) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    z64 x = src ? src[e] : zmk(0, 0);
    if (add) x = zadd(x, add[e]);
    r[e] = x;
  }
}
__global__ void axpy_kernel(int64_t n, z64 alpha, const z64* __restrict__ x, z64* __restrict__ y) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    z64 t = y[e];
    zfma(t, alpha, x[e]);
    y[e] = t;
  }
}

// ------------------------------------------------------------- assembly --

struct AsmArgs {
  int o, v;
  int64_t ov, po, pv;
  const int2* opairs;
  const z64 *R0p, *PQ, *X, *Zq, *Yh, *Gq, *H2h, *t2p;
  int out32;             // PQ, X, Zq, Yh hold complex FP32 (3xTF32 residuals)
  const double* eps;     // SO energies (for the diagonal-Fock fast path)
  const z64 *Foo, *Fvv;  // diagonal-Fock fast path reads F[p,p]
  z64 E;
  int use_const, use_e, singles, f_diag;
  z64* r2p;
};

constexpr int TS = 32;  // (a,b) tile edge

// Element arithmetic of the assembly: FP64 (z64), or FP32 (float2) for 3xTF32 residuals, whose
// GEMM terms carry FP32-level error anyway (FP64 loads rounded to float on the integer pipe,
// the result widened exactly).
__device__ __forceinline__ float f64_to_f32(double x) {
  float h, l;
  split_f32pair_fast(x, h, l);
  return __fadd_rn(h, l);
}
template <typename T> __device__ __forceinline__ T ldz(const z64* p);
// (read-only loads: the assembly's inputs are never written while it runs, which lets the
// compiler issue a thread's loads ahead of its stores)
template <> __device__ __forceinline__ z64 ldz<z64>(const z64* p) { return __ldg(p); }
template <> __device__ __forceinline__ float2 ldz<float2>(const z64* p) {
  const z64 v = __ldg(p);
  return make_float2(f64_to_f32(v.x), f64_to_f32(v.y));
}
template <typename T> __device__ __forceinline__ T cz(z64 v);
template <> __device__ __forceinline__ z64 cz<z64>(z64 v) { return v; }
template <> __device__ __forceinline__ float2 cz<float2>(z64 v) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ z64 tz(z64 v) { return v; }
__device__ __forceinline__ z64 tz(float2 v) { return zmk(f2d_exact(v.x), f2d_exact(v.y)); }
__device__ __forceinline__ z64 vadd(z64 a, z64 b) { return zadd(a, b); }
__device__ __forceinline__ z64 vsub(z64 a, z64 b) { return zsub(a, b); }
__device__ __forceinline__ z64 vneg(z64 a) { return zneg(a); }
__device__ __forceinline__ z64 vmul(z64 a, z64 b) { return zmul(a, b); }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 vsub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 vneg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 vmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// Element idx of a GEMM product array stored in complex FP32 (f32) or FP64.
template <typename T> __device__ __forceinline__ T ldo(const z64* base, int64_t idx, int f32);
template <> __device__ __forceinline__ float2 ldo<float2>(const z64* base, int64_t idx, int f32) {
  return f32 ? __ldg((const float2*)base + idx) : ldz<float2>(base + idx);
}
template <> __device__ __forceinline__ z64 ldo<z64>(const z64* base, int64_t idx, int f32) {
  if (f32) {
    const float2 v = __ldg((const float2*)base + idx);
    return zmk(f2d_exact(v.x), f2d_exact(v.y));
  }
  return base[idx];
}
template <typename T> __device__ __forceinline__ T zzero();
template <> __device__ __forceinline__ z64 zzero<z64>() { return zmk(0, 0); }
template <> __device__ __forceinline__ float2 zzero<float2>() { return make_float2(0.f, 0.f); }

// One CTA per (pair p(ij), upper-triangle tile of (a,b)).  Terms whose source
// is indexed [b][a] are summed first along a (coalesced) into shared memory
// and read transposed; the rest are read along b.
// Four blocks per SM (at most 64 registers): the kernel is bound by load latency (ncu at
// 40/160: long-scoreboard stalls first, 25 % of DRAM bandwidth at 3 blocks per SM).
template <typename T>
__global__ void __launch_bounds__(256, 4) assemble_r2_kernel(AsmArgs A) {
  __shared__ T tr[TS][TS + 1];
  const int ntile = (A.v + TS - 1) / TS;
  // decode tile pair (ta <= tb) from blockIdx.x
  int tp = blockIdx.x, ta = 0;
  while (tp >= ntile - ta) { tp -= ntile - ta; ++ta; }
  const int tb = ta + tp;
  const int64_t p = blockIdx.y;
  const int2 ij = A.opairs[p];
  const int i = ij.x, j = ij.y;
  const int a0 = ta * TS, b0 = tb * TS;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int v = A.v;
  const int64_t vv = (int64_t)v * v;
  // Phase 1: transposed terms T[b][a] for b in tile tb, a in tile ta (coalesced along a).
  for (int rb = ty; rb < TS; rb += 8) {
    int b = b0 + rb, a = a0 + tx;
    T s = zzero<T>();
    if (a < v && b < v) {
      // -X[(i,b),(j,a)] + X[(j,b),(i,a)]
      s = vneg(ldo<T>(A.X, ((int64_t)i * v + b) * A.ov + (int64_t)j * v + a, A.out32));
      s = vadd(s, ldo<T>(A.X, ((int64_t)j * v + b) * A.ov + (int64_t)i * v + a, A.out32));
      if (A.singles) s = vsub(s, ldo<T>(A.Zq, p * vv + (int64_t)b * v + a, A.out32));      // -Zq[p][b][a]
      if (!A.f_diag) s = vsub(s, ldz<T>(A.Gq + p * vv + (int64_t)b * v + a));      // -Gq[p][b][a]
    }
    tr[rb][tx] = s;
  }
  __syncthreads();
  // Phase 2: direct terms along b, plus tr[b][a].
  for (int ra = ty; ra < TS; ra += 8) {
    int a = a0 + ra, b = b0 + tx;
    if (a >= v || b >= v || b <= a) continue;
    int64_t q = pair_index(a, b, v);
    int64_t pq = p * A.pv + q;
    T s = tr[tx][ra];
    s = vadd(s, ldo<T>(A.PQ, pq, A.out32));
    s = vadd(s, ldo<T>(A.X, ((int64_t)i * v + a) * A.ov + (int64_t)j * v + b, A.out32));
    s = vsub(s, ldo<T>(A.X, ((int64_t)j * v + a) * A.ov + (int64_t)i * v + b, A.out32));
    if (A.singles) {
      s = vadd(s, ldo<T>(A.Zq, p * vv + (int64_t)a * v + b, A.out32));
      s = vadd(s, ldo<T>(A.Yh, ((int64_t)i * A.o + j) * A.pv + q, A.out32));
      s = vsub(s, ldo<T>(A.Yh, ((int64_t)j * A.o + i) * A.pv + q, A.out32));
    }
    T t = ldz<T>(A.t2p + pq);
    if (A.f_diag) {
      // sum_c F[b,c] t2[ijac] + F[a,c] t2[ijcb] - F[k,j] t2[ikab] - F[k,i] t2[kjab] with F diagonal
      const T fs = vsub(vadd(ldz<T>(A.Fvv + (int64_t)a * v + a), ldz<T>(A.Fvv + (int64_t)b * v + b)),
                        vadd(ldz<T>(A.Foo + (int64_t)i * A.o + i), ldz<T>(A.Foo + (int64_t)j * A.o + j)));
      s = vadd(s, vmul(fs, t));
    } else {
      s = vadd(s, ldz<T>(A.Gq + p * vv + (int64_t)a * v + b));
      s = vadd(s, ldz<T>(A.H2h + ((int64_t)j * A.o + i) * A.pv + q));
      s = vsub(s, ldz<T>(A.H2h + ((int64_t)i * A.o + j) * A.pv + q));
    }
    if (A.use_const) s = vadd(s, ldz<T>(A.R0p + pq));
    if (A.use_e) s = vsub(s, vmul(cz<T>(A.E), t));
    A.r2p[pq] = tz(s);
  }
}

// ------------------------------------------------------- update / guess --

struct VecDims {
  int o, v;
  int64_t n1, pv;
  const int2* opairs;
  const int2* vpairs;
  const double* eps;
  const double* invD;    // 1 / denom_at, stored by agb_cisd_set_fock
};

__device__ __forceinline__ double denom_at(const VecDims& d, int64_t k) {
  if (k < d.n1) {
    int i = (int)(k / d.v), a = (int)(k % d.v);
    return d.eps[i] - d.eps[d.o + a];
  }
  int64_t e = k - d.n1;
  int2 ij = d.opairs[e / d.pv], ab = d.vpairs[e % d.pv];
  return d.eps[ij.x] + d.eps[ij.y] - d.eps[d.o + ab.x] - d.eps[d.o + ab.y];
}

// invD[k] = 1 / D_k, once per set of orbital energies: the pair lookups and the FP64
// reciprocal (several operations on GB300's narrow FP64 pipe per element) leave the
// per-iteration update, which then streams t, r and invD at HBM rate.
__global__ void inv_denom_kernel(VecDims d, int64_t n, double* __restrict__ invD) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    invD[k] = 1.0 / denom_at(d, k);
}

// t_out = t + r * (1/D), the exact operation numpy performs for complex / real.
__global__ void update_kernel(VecDims d, int64_t n, const z64* __restrict__ t, const z64* __restrict__ r,
                              z64* __restrict__ t_out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double inv = d.invD[k];
    z64 rr = r[k], tt = t[k];
    t_out[k] = zmk(tt.x + rr.x * inv, tt.y + rr.y * inv);
  }
}

// guess: t1 = F_ai / D_ia, t2p = <ab||ij> / D
__global__ void guess_kernel(VecDims d, int64_t n, const z64* __restrict__ FvoT, const z64* __restrict__ R0p,
                             z64* __restrict__ t) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double inv = d.invD[k];
    z64 num = k < d.n1 ? FvoT[k] : R0p[k - d.n1];
    t[k] = zmk(num.x * inv, num.y * inv);
  }
}

// ------------------------------------------------------------ reductions --

__device__ __forceinline__ z64 warp_sum(z64 s) {
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, off);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, off);
  }
  return s;
}

// Block-reduce NV complex accumulators; thread 0 writes them to out[blockIdx.x*NV + k].
template <int NV>
__device__ __forceinline__ void block_reduce_store(z64 (&acc)[NV], z64* out) {
  __shared__ z64 sh[NV][32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    z64 s = warp_sum(acc[k]);
    if (lane == 0) sh[k][w] = s;
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      z64 s = lane < nw ? sh[k][lane] : zmk(0, 0);
      s = warp_sum(s);
      if (lane == 0) out[(int64_t)blockIdx.x * NV + k] = s;
    }
  }
}

// out[k] = sum over blocks of partial[b*nv + k], one 256-thread block per slot k < count <= nv:
// thread t sums blocks t, t + 256, ... in order, then a fixed tree (deterministic; a single
// thread's dependent chain of nblocks loads made this tail ~90 us).
__global__ void __launch_bounds__(256) finish_partials_kernel(const z64* __restrict__ partial, int nblocks, int nv,
                                                              int count, z64* out) {
  __shared__ z64 sh[256];
  const int k = blockIdx.x, t = threadIdx.x;
  if (k >= count || k >= nv) return;
  z64 s = zmk(0, 0);
  for (int b = t; b < nblocks; b += 256) s = zadd(s, partial[(int64_t)b * nv + k]);
  sh[t] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (t < w) sh[t] = zadd(sh[t], sh[t + w]);
    __syncthreads();
  }
  if (t == 0) out[k] = sh[0];
}

constexpr int kRedBlocks = 152 * 4;
constexpr int kMaxVec = 16;

struct DotArgs {
  int64_t n1, n2;
  double w1, w2;
  const z64* x;
  const z64* ys[kMaxVec];
  int ny;
};

// First index >= lo of the grid-stride sequence k0, k0 + stride, ...
__device__ __forceinline__ int64_t stride_start(int64_t k0, int64_t stride, int64_t lo) {
  return k0 >= lo ? k0 : k0 + (lo - k0 + stride - 1) / stride * stride;
}

// Weighted Gram row: out_j = w(k) sum_k conj(y_j[k]) x[k], w = w1 on the t1 part (k < n1), w2 on t2.
// Products and running sums in double-float on the FP32 pipe (~2^-44 relative; GB300's FP64
// pipe would bound this HBM stream), fixed reduction order.  Block 0 sums the small t1 part
// alone and the other blocks the packed doubles.  The two halves of a block take the even and
// the odd vectors of the same elements (x is read by both, the second time from L1), so a
// thread carries half the double-float sums: fewer registers, four blocks per SM, and each
// thread's loads and math alternate over half as many vectors.
constexpr int kDotBlocks = 152 * 4;

template <int NY>
__global__ void __launch_bounds__(256, 4) dots_kernel(DotArgs A, z64* partial) {
  constexpr int NH = (NY + 1) / 2;
  const int half = threadIdx.x >> 7, tid = threadIdx.x & 127;
  const bool t1 = blockIdx.x == 0;
  const int64_t lo = t1 ? 0 : A.n1, hi = t1 ? A.n1 : A.n1 + A.n2;
  const int64_t stride = (int64_t)(t1 ? 1 : gridDim.x - 1) * 128;
  const int64_t k0 = lo + (int64_t)(t1 ? 0 : blockIdx.x - 1) * 128 + tid;
  float s[NH][4];
#pragma unroll
  for (int h = 0; h < NH; ++h) s[h][0] = s[h][1] = s[h][2] = s[h][3] = 0.f;
  for (int64_t k = k0; k < hi; k += stride) {
    const float4 x = split_z_fast(A.x[k]);
    z64 yv[NH];
#pragma unroll
    for (int h = 0; h < NH; ++h) {
      const int j = 2 * h + half;
      yv[h] = j < A.ny ? __ldcs(&A.ys[j][k]) : zmk(0, 0);
    }
#pragma unroll
    for (int h = 0; h < NH; ++h) {
      if (2 * h + half < A.ny) {
        const float4 y = split_z_fast(yv[h]);
        // conj(y) * x = (yr xr + yi xi) + i (yr xi - yi xr)
        df_mac(s[h][0], s[h][1], y.x, y.y, x.x, x.y);
        df_mac(s[h][0], s[h][1], y.z, y.w, x.z, x.w);
        df_mac(s[h][2], s[h][3], y.x, y.y, x.z, x.w);
        df_mac(s[h][2], s[h][3], -y.z, -y.w, x.x, x.y);
      }
    }
  }
  const double w = t1 ? A.w1 : A.w2;
  z64 acc[NY];
#pragma unroll
  for (int j = 0; j < NY; ++j) acc[j] = zmk(0, 0);
#pragma unroll
  for (int h = 0; h < NH; ++h) {
    const z64 v = zmk(w * df_to_double(s[h][0], s[h][1]), w * df_to_double(s[h][2], s[h][3]));
    if (half == 0 && 2 * h < NY) acc[2 * h] = v;
    if (half == 1 && 2 * h + 1 < NY) acc[2 * h + 1] = v;
  }
  block_reduce_store<NY>(acc, partial);
}

// The Gram-row kernel for ny vectors (partials [kRedBlocks][nv]); returns nv, the slot stride.
int launch_dots(const DotArgs& A, int ny, z64* part, cudaStream_t st) {
  if (ny <= 4) {
    dots_kernel<4><<<kDotBlocks, 256, 0, st>>>(A, part);
    return 4;
  }
  if (ny <= 8) {
    dots_kernel<8><<<kDotBlocks, 256, 0, st>>>(A, part);
    return 8;
  }
  if (ny <= 12) {
    dots_kernel<12><<<kDotBlocks, 256, 0, st>>>(A, part);
    return 12;
  }
  dots_kernel<16><<<kDotBlocks, 256, 0, st>>>(A, part);
  return 16;
}

struct CombArgs {
  int64_t n1, n2;
  const z64* ys[kMaxVec];
  double c[2 * kMaxVec];
  z64 csum;        // sum_j c_j
  int ny;
  const z64* t_old;
  z64* t_new;
  const z64* ew;   // energy weights [F_ov | <ij||ab>_p]
};

// (ah + al) - (bh + bl) as a float pair (two-sum of the leading parts, then a fast
// renormalisation): absolute error ~2^-48 of the operands.
__device__ __forceinline__ void df_diff(float ah, float al, float bh, float bl, float& h, float& l) {
  const float s = __fsub_rn(ah, bh);
  const float z = __fsub_rn(s, ah);
  float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, z)), __fsub_rn(-bh, z));
  e = __fadd_rn(e, __fsub_rn(al, bl));
  h = __fadd_rn(s, e);
  l = __fsub_rn(e, __fsub_rn(h, s));
}

// t_new = sum_j c_j y_j, E = sum t_new ew, s1 = sum_{t1} (t_old - t_new)^2 and
// s2 = 4 sum_{t2} (t_old - t_new)^2 (apyib/utils.py:138, ci_wfn.py:355,361-365).
// t_new = (sum_j c_j) y_0 + sum_{j>0} c_j (y_j - y_0): the first product in FP64 (so a
// copy, ny = 1 with c = 1, is exact), the differences, the small sum, the energy and the
// squared norms (old - t_new taken in double-float) in double-float on the FP32 pipe
// (~2^-46 of |y_j| per element), which leaves 4 FP64 operations per element (GB300's FP64
// pipe bounded the FP64 version).
// t_old / t_new and any y_j may alias: each element is read before it is written.
__global__ void __launch_bounds__(256) combine_kernel(CombArgs A, z64* partial) {
  __shared__ float4 cs[kMaxVec];
  if (threadIdx.x < A.ny) cs[threadIdx.x] = split_z(zmk(A.c[2 * threadIdx.x], A.c[2 * threadIdx.x + 1]));
  __syncthreads();
  const bool csum_real = A.csum.y == 0.0;
  float er = 0.f, erc = 0.f, ei = 0.f, eic = 0.f;  // E = sum t ew
  z64 acc[3] = {zmk(0, 0), zmk(0, 0), zmk(0, 0)};  // E, s1, s2
  const int64_t n = A.n1 + A.n2, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t k0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (int part = 0; part < 2; ++part) {
    float q[4] = {0.f, 0.f, 0.f, 0.f};
    const int64_t hi = part ? n : A.n1;
    for (int64_t k = stride_start(k0, stride, part ? A.n1 : 0); k < hi; k += stride) {
      const z64 y0 = A.ys[0][k];
      z64 t = zmk(0, 0);
      float dr = 0.f, drc = 0.f, di = 0.f, dic = 0.f;
      if (A.ny > 1) {
        const float4 y0s = split_z_fast(y0);
        for (int j = 1; j < A.ny; ++j) {
          const float4 yj = split_z_fast(A.ys[j][k]);
          float4 d;
          df_diff(yj.x, yj.y, y0s.x, y0s.y, d.x, d.y);
          df_diff(yj.z, yj.w, y0s.z, y0s.w, d.z, d.w);
          const float4 c = cs[j];
          // c d = (cr dr - ci di) + i (cr di + ci dr)
          df_mac(dr, drc, c.x, c.y, d.x, d.y);
          df_mac(dr, drc, -c.z, -c.w, d.z, d.w);
          df_mac(di, dic, c.x, c.y, d.z, d.w);
          df_mac(di, dic, c.z, c.w, d.x, d.y);
        }
      }
      // t = (sum c) y0 + the double-float sum: one FMA and one add per part on the FP64 pipe
      if (csum_real) {
        t.x = fma(A.csum.x, y0.x, f2d_exact(dr)) + f2d_exact(drc);
        t.y = fma(A.csum.x, y0.y, f2d_exact(di)) + f2d_exact(dic);
      } else {
        t = zmul(A.csum, y0);
        t.x += df_to_double(dr, drc);
        t.y += df_to_double(di, dic);
      }
      const z64 old = A.t_old[k];
      const z64 w = A.ew[k];
      A.t_new[k] = t;
      const float4 ts = split_z_fast(t);
      const float4 ws = split_z_fast(w);
      // t w = (tr wr - ti wi) + i (tr wi + ti wr)
      df_mac(er, erc, ts.x, ts.y, ws.x, ws.y);
      df_mac(er, erc, -ts.z, -ts.w, ws.z, ws.w);
      df_mac(ei, eic, ts.x, ts.y, ws.z, ws.w);
      df_mac(ei, eic, ts.z, ts.w, ws.x, ws.y);
      // old - t in double-float from the float pairs (absolute error ~2^-46 |t|; no FP64 subtract)
      const float4 os = split_z_fast(old);
      float4 e;
      df_diff(os.x, os.y, ts.x, ts.y, e.x, e.y);
      df_diff(os.z, os.w, ts.z, ts.w, e.z, e.w);
      // (old - t)^2, unconjugated
      df_mac(q[0], q[1], e.x, e.y, e.x, e.y);
      df_mac(q[0], q[1], -e.z, -e.w, e.z, e.w);
      df_mac(q[2], q[3], 2.f * e.x, 2.f * e.y, e.z, e.w);
    }
    const z64 qs = zmk(df_to_double(q[0], q[1]), df_to_double(q[2], q[3]));
    if (part) acc[2] = zadd(acc[2], qs);
    else acc[1] = zadd(acc[1], qs);
  }
  acc[0] = zmk(df_to_double(er, erc), df_to_double(ei, eic));
  acc[2] = zscale(acc[2], 4.0);
  block_reduce_store<3>(acc, partial);
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace
}  // namespace agb

using namespace agb;

// =================================================================== plan ==

static void plan_layout(agb_cisd_plan* P, char* base, size_t* total) {
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* ptr = base ? base + off : nullptr;
    off += align256(bytes);
    return ptr;
  };
  const size_t Z = sizeof(z64);
  const int64_t o = P->o, v = P->v, ov = P->ov, po = P->po, pv = P->pv;
  P->FvoT = (z64*)take(Z * ov);
  P->Foo = (z64*)take(Z * o * o);
  P->Fvv = (z64*)take(Z * v * v);
  P->EW = (z64*)take(Z * (P->n1 + P->n2));
  P->eps = (double*)take(sizeof(double) * P->nso);
  P->invD = (double*)take(sizeof(double) * (P->n1 + P->n2));
  P->opairs = (int2*)take(sizeof(int2) * (po > 0 ? po : 1));
  P->vpairs = (int2*)take(sizeof(int2) * (pv > 0 ? pv : 1));
  P->R0p = (z64*)take(Z * po * pv);
  if (P->mp2_only) {
    P->VT = P->WooooT = P->Wvp = P->Tring = P->X = P->PQ = P->t2h = P->t2q = P->Gq = P->H2h = P->R1x = nullptr;
    P->WvovvH = P->WooovP = P->WovooP = P->WvvvoP = P->Zq = P->Yh = nullptr;
    P->gemm_scratch = take(4096);
    P->gemm_scratch_bytes = 4096;
    *total = off;
    return;
  }
  P->VT = (z64*)take(Z * ov * ov);
  P->WooooT = (z64*)take(Z * po * po);
  P->Wvp = (z64*)take(Z * pv * pv);
  // FP64 Tring, or (mixed plans) the ring operand's TF32 planes in 3xTF32 residuals
  P->Tring = (z64*)take(P->mixed ? std::max(Z * ov * ov, agb::tf32_planes_bytes(ov, ov)) : Z * ov * ov);
  P->X = (z64*)take(Z * ov * ov);
  P->PQ = (z64*)take(Z * po * pv);
  // t2h/t2q serve the singles terms and the non-diagonal Fock terms
  // (mixed plans: or the TF32 planes of the singles GEMMs' operands, written straight from t2p)
  P->t2h = (z64*)take(P->mixed ? std::max(Z * o * o * pv, agb::tf32_planes_bytes(o, (int64_t)o * pv)) : Z * o * o * pv);
  P->t2q = (z64*)take(P->mixed ? std::max(Z * po * v * v, agb::tf32_planes_bytes(v, po * v)) : Z * po * v * v);
  P->Gq = (z64*)take(Z * po * v * v);
  P->H2h = (z64*)take(Z * o * o * pv);
  P->R1x = (z64*)take(Z * ov);
  if (P->singles) {
    P->WvovvH = (z64*)take(Z * v * o * pv);
    P->WooovP = (z64*)take(Z * o * po * v);
    P->WovooP = (z64*)take(Z * po * v * o);
    P->WvvvoP = (z64*)take(Z * v * o * pv);
    P->Zq = (z64*)take(Z * po * v * v);
    P->Yh = (z64*)take(Z * o * o * pv);
  } else {
    P->WvovvH = P->WooovP = P->WovooP = P->WvvvoP = P->Zq = P->Yh = nullptr;
  }
  // GEMM scratch: split-K partials (FP64) or 3xTF32 operand planes.
  size_t gs = (size_t)64 << 20;
  if (P->mixed) {
    // status header + planes of the operands prepared per call + split-K partials
    // (mixed plans also run the double-float base residual: room for its split operands)
    auto upd = [&](int64_t M, int64_t N, int64_t K, bool a_static, bool b_static) {
      size_t s = 256 + agb::tf32_partials_bytes(M, N, K);
      if (!a_static) s += align256(agb::tf32_planes_bytes(M, K));
      if (!b_static) s += align256(agb::tf32_planes_bytes(N, K));
      if (s > gs) gs = s;
      size_t d = 256 + agb::dfgemm_scratch_bytes(M, N, K);
      if (d > gs) gs = d;
      if (agb::ozgemm_tiles(M, N) >= agb::kOzMinTiles) {
        size_t z = agb::ozgemm_scratch_bytes(M, N, K);
        if (z > gs) gs = z;
      }
    };
    upd(o, v, o, false, false);
    upd(o, v, v, false, false);
    upd(ov, ov, ov, false, true);
    upd(po, pv, pv, false, true);
    upd(po, pv, po, true, false);
    upd(po * v, v, v, false, false);
    upd(o, o * pv, o, false, false);
    if (P->singles) {
      // the singles GEMMs in both orientations (3xTF32 runs them with transposed outputs)
      upd(o, v, o * pv, false, true);
      upd(o, v, po * v, true, false);
      upd(po * v, v, o, true, false);
      upd(o, o * pv, v, false, true);
      upd(v, o, o * pv, true, false);
      upd(v, o, po * v, false, true);
      upd(v, po * v, o, false, true);
      upd(o * pv, o, v, true, false);
    }
    P->P_VT = (float*)take(agb::tf32_planes_bytes(ov, ov));
    P->P_Wvp = (float*)take(agb::tf32_planes_bytes(pv, pv));
    P->P_Woooo = (float*)take(agb::tf32_planes_bytes(po, po));
    if (P->singles) {
      P->P_Wvovv = (float*)take(agb::tf32_planes_bytes(v, o * pv));
      P->P_Wooov = (float*)take(agb::tf32_planes_bytes(o, po * v));
      P->P_Wovoo = (float*)take(agb::tf32_planes_bytes(po * v, o));
      P->P_Wvvvo = (float*)take(agb::tf32_planes_bytes(o * pv, v));
    }
  }
  P->gemm_scratch = take(gs);
  P->gemm_scratch_bytes = gs;
  *total = off;
}

namespace {
thread_local std::string g_last_error;
}

void agb_set_error_message(const char* msg, const char* file, int line) {
  g_last_error = std::string(msg) + " (" + file + ":" + std::to_string(line) + ")";
}

static std::atomic<unsigned long long> g_launches{0};
void agb_count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
extern "C" unsigned long long agb_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

namespace agb {
namespace {

// GEMM on the selected backend.  conj flags are never needed on the hot path.
// PA / PB: TF32 planes of a static operand prepared at set-up (tensor-core path only).
// trans_c: C(m, n) lives at C[n * ldc + m]; the 3xTF32 kernel stores it so, the other
// backends compute the same product as C^T = B^T A^T.  kblk: both operands' planes are
// K-blocked (static ones prepared so at set-up; the singles GEMMs, whose operands are up to
// 1.7M elements long in K).  c32 (3xTF32 only): C holds complex FP32 values (the
// products only the assembly reads, which works at FP32 level in 3xTF32 residuals).
agb_status gemm(agb_cisd_plan* P, int prec, int64_t M, int64_t N, int64_t K, z64 alpha, const z64* A, int64_t sAm,
                int64_t sAk, const z64* B, int64_t sBk, int64_t sBn, z64 beta, z64* C, int64_t ldc,
                cudaStream_t st, const float* PA = nullptr, const float* PB = nullptr, int trans_c = 0,
                int kblk = 0, int c32 = 0) {
  if (prec == AGB_PREC_TF32X3) {
    if (M == 0 || N == 0) return AGB_OK;
    AGB_ARG_CHECK(!(c32 && K == 0), "residual: empty contraction into an FP32 product");
    if (K == 0) return zgemm_ex(M, N, 0, zmk(0, 0), A, sAm, sAk, 0, B, sBk, sBn, 0, beta, C, ldc, nullptr, 0, st);
    char* base = (char*)P->gemm_scratch;
    size_t off = 256;
    if (!PA) {
      PA = (const float*)(base + off);
      AGB_STATUS_TRY(tf32_prep_planes(A, M, K, sAm, sAk, 0, (float*)PA, st, kblk));
      off += align256(tf32_planes_bytes(M, K));
    }
    if (!PB) {
      PB = (const float*)(base + off);
      AGB_STATUS_TRY(tf32_prep_planes(B, N, K, sBn, sBk, 0, (float*)PB, st, kblk));
      off += align256(tf32_planes_bytes(N, K));
    }
    if (off > P->gemm_scratch_bytes) {
      agb_set_error_message("residual: GEMM scratch too small", __FILE__, __LINE__);
      return AGB_ERR_WORKSPACE;
    }
    return tf32_gemm_planes(M, N, K, alpha, PA, PB, beta, C, ldc, (int*)base, (z64*)(base + off),
                            P->gemm_scratch_bytes - off, st, trans_c, kblk, kblk, c32,
                            P->gemm_timing ? &P->gemm_timing_log : nullptr);
  }
  if (trans_c) return gemm(P, prec, N, M, K, alpha, B, sBn, sBk, A, sAk, sAm, beta, C, ldc, st);
  if (prec == AGB_PREC_OZAKI && ozgemm_tiles(M, N) >= kOzMinTiles)
    return ozgemm_ex(M, N, K, alpha, A, sAm, sAk, 0, B, sBk, sBn, 0, beta, C, ldc, P->gemm_scratch,
                     P->gemm_scratch_bytes, st);
  if (prec == AGB_PREC_DF64 || prec == AGB_PREC_OZAKI)
    return dfgemm_ex(M, N, K, alpha, A, sAm, sAk, 0, B, sBk, sBn, 0, beta, C, ldc, (char*)P->gemm_scratch + 256,
                     P->gemm_scratch_bytes - 256, st);
  // FP64 split-K partials start past the 256-byte status header of the scratch.
  return zgemm_ex(M, N, K, alpha, A, sAm, sAk, 0, B, sBk, sBn, 0, beta, C, ldc, (char*)P->gemm_scratch + 256,
                  P->gemm_scratch_bytes - 256, st);
}

// The singles GEMMs read K-blocked planes when every operand they take as A (v-row and
// (j,p(ab))-row operands) has more than 64 rows, so that its planes hold whole 128-row boxes.
int singles_kblk(const agb_cisd_plan* P) { return (P->v > 64 && (int64_t)P->o * P->pv > 64) ? 1 : 0; }

// TF32 planes of every static ERI-block operand, in the orientation its GEMM reads it.
agb_status prepare_static_planes(agb_cisd_plan* P, cudaStream_t st) {
  if (!P->mixed || P->mp2_only) return AGB_OK;
  const int64_t o = P->o, v = P->v, ov = P->ov, po = P->po, pv = P->pv;
  AGB_STATUS_TRY(tf32_prep_planes(P->VT, ov, ov, ov, 1, 0, P->P_VT, st, 0));
  AGB_STATUS_TRY(tf32_prep_planes(P->Wvp, pv, pv, pv, 1, 0, P->P_Wvp, st, 0));
  AGB_STATUS_TRY(tf32_prep_planes(P->WooooT, po, po, po, 1, 0, P->P_Woooo, st, 0));
  if (P->singles) {
    const int kb = singles_kblk(P);
    AGB_STATUS_TRY(tf32_prep_planes(P->WvovvH, v, o * pv, o * pv, 1, 0, P->P_Wvovv, st, kb));
    AGB_STATUS_TRY(tf32_prep_planes(P->WooovP, o, po * v, po * v, 1, 0, P->P_Wooov, st, kb));
    AGB_STATUS_TRY(tf32_prep_planes(P->WovooP, po * v, o, o, 1, 0, P->P_Wovoo, st, kb));
    AGB_STATUS_TRY(tf32_prep_planes(P->WvvvoP, o * pv, v, 1, o * pv, 0, P->P_Wvvvo, st, kb));
  }
  return AGB_OK;
}

Dims dims_of(const agb_cisd_plan* P) { return Dims{P->o, P->v, P->ov, P->po, P->pv, P->opairs, P->vpairs}; }
VecDims vdims_of(const agb_cisd_plan* P) {
  return VecDims{P->o, P->v, P->n1, P->pv, P->opairs, P->vpairs, P->eps, P->invD};
}

z64* block_ptr(agb_cisd_plan* P, int id) {
  switch (id) {
    case B_R0p: return P->R0p;
    case B_Wop: return P->EW + P->n1;
    case B_VT: return P->VT;
    case B_Wvovv: return P->WvovvH;
    case B_Wooov: return P->WooovP;
    case B_Wovoo: return P->WovooP;
    case B_Wvvvo: return P->WvvvoP;
    case B_Woooo: return P->WooooT;
    default: return P->Wvp;
  }
}

bool block_needed(const agb_cisd_plan* P, int id) {
  if (P->mp2_only) return id == B_R0p || id == B_Wop;
  if (P->singles) return true;
  return id == B_R0p || id == B_Wop || id == B_VT || id == B_Woooo || id == B_Wvvvv;
}

template <class SD, class SE>
agb_status launch_build(agb_cisd_plan* P, int id, SD sd, SE se, cudaStream_t st) {
  int64_t n = block_elems(id, P);
  if (n == 0) return AGB_OK;
  build_block_kernel<SD, SE><<<grid_for(n, 256), 256, 0, st>>>(id, dims_of(P), n, sd, se, block_ptr(P, id));
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

}  // namespace
}  // namespace agb

extern "C" {

int agb_version(void) { return 100; }
const char* agb_last_error(void) { return g_last_error.c_str(); }

agb_status agb_cisd_plan_create(int o, int v, int flags, agb_cisd_plan** plan) {
  AGB_ARG_CHECK(plan != nullptr, "plan_create: null output");
  AGB_ARG_CHECK(o >= 2 && v >= 2 && o % 2 == 0 && v % 2 == 0, "plan_create: o, v must be even and >= 2");
  agb_cisd_plan* P = new agb_cisd_plan();
  P->o = o; P->v = v; P->flags = flags;
  P->nso = o + v; P->ov = (int64_t)o * v; P->po = npairs(o); P->pv = npairs(v);
  P->mp2_only = (flags & AGB_PLAN_MP2) != 0;
  P->singles = !(flags & (AGB_PLAN_NO_SINGLES | AGB_PLAN_MP2));
  P->mixed = (flags & AGB_PLAN_MIXED) != 0;
  P->n1 = P->singles ? P->ov : 0;
  P->n2 = P->po * P->pv;
  P->f_diag = true;
  P->ws = nullptr;
  plan_layout(P, nullptr, &P->ws_bytes);
  *plan = P;
  return AGB_OK;
}

agb_status agb_cisd_plan_destroy(agb_cisd_plan* plan) {
  if (plan)
    for (auto& r : plan->gemm_timing_log) {
      cudaEventDestroy(r.e0);
      cudaEventDestroy(r.e1);
    }
  delete plan;
  return AGB_OK;
}

agb_status agb_cisd_plan_gemm_timing(agb_cisd_plan* plan, int on) {
  AGB_ARG_CHECK(plan != nullptr, "gemm_timing: null plan");
  plan->gemm_timing = on != 0;
  return AGB_OK;
}

agb_status agb_cisd_plan_gemm_timing_collect(agb_cisd_plan* plan, double min_mnk, int* launches, double* ms,
                                             double* flops) {
  AGB_ARG_CHECK(plan != nullptr, "gemm_timing_collect: null plan");
  int n = 0;
  double tms = 0, tfl = 0;
  agb_status st = AGB_OK;
  for (auto& r : plan->gemm_timing_log) {
    if (st == AGB_OK && cudaEventSynchronize(r.e1) == cudaSuccess) {
      if ((double)r.M * (double)r.N * (double)r.K >= min_mnk) {
        float e = 0;
        if (cudaEventElapsedTime(&e, r.e0, r.e1) != cudaSuccess) st = AGB_ERR_CUDA;
        ++n;
        tms += e;
        tfl += r.flops;
      }
    } else if (st == AGB_OK) {
      agb_set_error_message("gemm_timing_collect: event synchronisation failed", __FILE__, __LINE__);
      st = AGB_ERR_CUDA;
    }
    cudaEventDestroy(r.e0);
    cudaEventDestroy(r.e1);
  }
  plan->gemm_timing_log.clear();
  if (launches) *launches = n;
  if (ms) *ms = tms;
  if (flops) *flops = tfl;
  return st;
}

agb_status agb_cisd_plan_workspace_bytes(const agb_cisd_plan* plan, size_t* bytes) {
  AGB_ARG_CHECK(plan && bytes, "workspace_bytes: null argument");
  *bytes = plan->ws_bytes;
  return AGB_OK;
}

agb_status agb_cisd_plan_sizes(const agb_cisd_plan* plan, int64_t* n1, int64_t* n2) {
  AGB_ARG_CHECK(plan && n1 && n2, "plan_sizes: null argument");
  *n1 = plan->n1;
  *n2 = plan->n2;
  return AGB_OK;
}

agb_status agb_cisd_plan_set_workspace(agb_cisd_plan* P, void* workspace, size_t bytes) {
  AGB_ARG_CHECK(P != nullptr, "set_workspace: null plan");
  if (workspace == nullptr || bytes < P->ws_bytes) {
    agb_set_error_message("set_workspace: workspace missing or smaller than agb_cisd_plan_workspace_bytes",
                          __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  AGB_ARG_CHECK(((uintptr_t)workspace & 255) == 0, "set_workspace: workspace must be 256-byte aligned");
  size_t total;
  P->ws = workspace;
  plan_layout(P, (char*)workspace, &total);
  // pair tables
  std::vector<int2> op(P->po > 0 ? P->po : 1), vp(P->pv > 0 ? P->pv : 1);
  for (int p = 0, k = 0; p < P->o; ++p)
    for (int q = p + 1; q < P->o; ++q) op[k++] = make_int2(p, q);
  for (int p = 0, k = 0; p < P->v; ++p)
    for (int q = p + 1; q < P->v; ++q) vp[k++] = make_int2(p, q);
  AGB_CUDA_TRY(cudaMemcpy(P->opairs, op.data(), sizeof(int2) * op.size(), cudaMemcpyHostToDevice));
  AGB_CUDA_TRY(cudaMemcpy(P->vpairs, vp.data(), sizeof(int2) * vp.size(), cudaMemcpyHostToDevice));
  AGB_CUDA_TRY(cudaMemset(P->gemm_scratch, 0, 256));  // error word of the tcgen05 GEMM
  return AGB_OK;
}

agb_status agb_cisd_set_fock(agb_cisd_plan* P, const void* F_SO, const double* eps_so, void* stream) {
  AGB_ARG_CHECK(P && P->ws, "set_fock: plan without workspace");
  AGB_ARG_CHECK(F_SO && eps_so, "set_fock: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  int* flag = (int*)((char*)P->gemm_scratch + 128);  // scratch word, consumed synchronously below
  AGB_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), st));
  int64_t nn = P->nso * P->nso;
  fock_extract_kernel<<<grid_for(nn, 256), 256, 0, st>>>((const z64*)F_SO, eps_so, P->o, P->v,
                                                          P->singles ? P->FvoT : nullptr, P->Foo, P->Fvv,
                                                          P->singles ? P->EW : nullptr, P->eps, flag);
  AGB_LAUNCH_CHECK();
  const int64_t n = P->n1 + P->n2;
  inv_denom_kernel<<<grid_for(n, 256), 256, 0, st>>>(vdims_of(P), n, P->invD);
  AGB_LAUNCH_CHECK();
  int h = 0;
  AGB_CUDA_TRY(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  AGB_CUDA_TRY(cudaStreamSynchronize(st));
  P->f_diag = (h == 0);
  return AGB_OK;
}

agb_status agb_cisd_blocks_from_mo(agb_cisd_plan* P, const void* ERI_MO, void* stream) {
  AGB_ARG_CHECK(P && P->ws && ERI_MO, "blocks_from_mo: bad argument");
  SrcMO s{(const z64*)ERI_MO, P->nso / 2};
  for (int id = 0; id < B_COUNT; ++id)
    if (block_needed(P, id)) AGB_STATUS_TRY(launch_build(P, id, s, s, (cudaStream_t)stream));
  return prepare_static_planes(P, (cudaStream_t)stream);
}

agb_status agb_cisd_blocks_from_so(agb_cisd_plan* P, const void* ERI_SO, void* stream) {
  AGB_ARG_CHECK(P && P->ws && ERI_SO, "blocks_from_so: bad argument");
  SrcSO s{(const z64*)ERI_SO, P->nso};
  for (int id = 0; id < B_COUNT; ++id)
    if (block_needed(P, id)) AGB_STATUS_TRY(launch_build(P, id, s, s, (cudaStream_t)stream));
  return prepare_static_planes(P, (cudaStream_t)stream);
}

static int64_t rlen(const agb_cisd_plan* P, char c) { return c == 'o' ? P->o : P->v; }
static int roff(const agb_cisd_plan* P, char c) { return c == 'o' ? 0 : P->o; }

size_t agb_cisd_factor_scratch_bytes(const agb_cisd_plan* P, int64_t naux) {
  size_t fac = sizeof(z64) * (size_t)(P->nso * P->nso * naux) + 4 * 256;
  size_t best = 0;
  for (int id = 0; id < B_COUNT; ++id) {
    if (!block_needed(P, id)) continue;
    const char* r = kBlockRanges[id];
    // direct (X Z | Y W), exchange (X W | Y Z)
    size_t d = align256(sizeof(z64) * rlen(P, r[0]) * rlen(P, r[2]) * rlen(P, r[1]) * rlen(P, r[3]));
    bool same = (r[2] == r[3]);
    size_t e = same ? 0 : align256(sizeof(z64) * rlen(P, r[0]) * rlen(P, r[3]) * rlen(P, r[1]) * rlen(P, r[2]));
    if (d + e > best) best = d + e;
  }
  return fac + best + 256;
}

agb_status agb_cisd_blocks_from_factors(agb_cisd_plan* P, const void* Bf, int64_t naux, void* scratch,
                                        size_t scratch_bytes, int precision, void* stream) {
  AGB_ARG_CHECK(P && P->ws && Bf && naux > 0, "blocks_from_factors: bad argument");
  AGB_ARG_CHECK(precision == AGB_PREC_FP64 || precision == AGB_PREC_DF64 || precision == AGB_PREC_OZAKI,
                "blocks_from_factors: precision must be AGB_PREC_FP64, AGB_PREC_DF64 or AGB_PREC_OZAKI");
  if (!scratch || scratch_bytes < agb_cisd_factor_scratch_bytes(P, naux)) {
    agb_set_error_message("blocks_from_factors: scratch too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char* base = (char*)(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  // sub-factors Bsub_XY[(x,y)][L] for XY in {oo, ov, vo, vv}
  z64* sub[2][2];
  size_t off = 0;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      char ca = a ? 'v' : 'o', cb = b ? 'v' : 'o';
      int64_t nx = rlen(P, ca), ny = rlen(P, cb);
      sub[a][b] = (z64*)(base + off);
      off += align256(sizeof(z64) * nx * ny * naux);
      extract_factor_kernel<<<grid_for(nx * ny * naux, 256), 256, 0, st>>>(
          (const z64*)Bf, naux, P->nso, roff(P, ca), (int)nx, roff(P, cb), (int)ny, sub[a][b]);
      AGB_LAUNCH_CHECK();
    }
  char* chem_base = base + off;
  auto chem_block = [&](char c0, char c1, char c2, char c3, z64* out) -> agb_status {
    // (c0 c1 | c2 c3) = sum_L Bsub_{c0c1}[(x,y)][L] * Bsub_{c2c3}[(z,w)][L]
    const z64* A = sub[c0 == 'v'][c1 == 'v'];
    const z64* B = sub[c2 == 'v'][c3 == 'v'];
    int64_t M = rlen(P, c0) * rlen(P, c1), N = rlen(P, c2) * rlen(P, c3);
    if (precision == AGB_PREC_OZAKI && ozgemm_tiles(M, N) >= kOzMinTiles &&
        ozgemm_scratch_bytes(M, N, naux) <= P->gemm_scratch_bytes)
      return ozgemm_ex(M, N, naux, zmk(1, 0), A, naux, 1, 0, B, 1, naux, 0, zmk(0, 0), out, N, P->gemm_scratch,
                       P->gemm_scratch_bytes, st);
    if (precision == AGB_PREC_DF64 || precision == AGB_PREC_OZAKI)
      return dfgemm_ex(M, N, naux, zmk(1, 0), A, naux, 1, 0, B, 1, naux, 0, zmk(0, 0), out, N,
                       (char*)P->gemm_scratch + 256, P->gemm_scratch_bytes - 256, st);
    return zgemm_ex(M, N, naux, zmk(1, 0), A, naux, 1, 0, B, 1, naux, 0, zmk(0, 0), out, N,
                    (char*)P->gemm_scratch + 256, P->gemm_scratch_bytes - 256, st);
  };
  for (int id = 0; id < B_COUNT; ++id) {
    if (!block_needed(P, id)) continue;
    const char* r = kBlockRanges[id];
    z64* cd = (z64*)chem_base;
    AGB_STATUS_TRY(chem_block(r[0], r[2], r[1], r[3], cd));
    SrcChem sd{cd, roff(P, r[0]), roff(P, r[2]), roff(P, r[1]), roff(P, r[3]),
               rlen(P, r[2]), rlen(P, r[1]), rlen(P, r[3])};
    SrcChem se = sd;
    if (r[2] != r[3]) {
      z64* ce = (z64*)(chem_base + align256(sizeof(z64) * rlen(P, r[0]) * rlen(P, r[2]) * rlen(P, r[1]) *
                                            rlen(P, r[3])));
      AGB_STATUS_TRY(chem_block(r[0], r[3], r[1], r[2], ce));
      se = SrcChem{ce, roff(P, r[0]), roff(P, r[3]), roff(P, r[1]), roff(P, r[2]),
                   rlen(P, r[3]), rlen(P, r[1]), rlen(P, r[2])};
    }
    AGB_STATUS_TRY(launch_build(P, id, sd, se, st));
  }
  return prepare_static_planes(P, st);
}

agb_status agb_cisd_residual(agb_cisd_plan* P, int prec, const void* tv, double E_re, double E_im, int flags, void* rv,
                             void* stream) {
  AGB_ARG_CHECK(P && P->ws && tv && rv, "residual: bad argument");
  AGB_ARG_CHECK(!P->mp2_only, "residual: plan created with AGB_PLAN_MP2");
  AGB_ARG_CHECK(prec == AGB_PREC_FP64 || prec == AGB_PREC_TF32X3 || prec == AGB_PREC_DF64 ||
                    prec == AGB_PREC_OZAKI,
                "residual: unknown precision");
  AGB_ARG_CHECK((prec != AGB_PREC_TF32X3 && prec != AGB_PREC_OZAKI) || P->mixed,
                "residual: plan created without AGB_PLAN_MIXED");
  cudaStream_t st = (cudaStream_t)stream;
  const int o = P->o, v = P->v;
  const int64_t ov = P->ov, po = P->po, pv = P->pv, n1 = P->n1;
  const z64* t1 = (const z64*)tv;
  const z64* t2p = t1 + n1;
  z64* r1 = (z64*)rv;
  z64* r2p = r1 + n1;
  const z64 one = zmk(1, 0), zero = zmk(0, 0);
  const z64 E = zmk(E_re, E_im);
  const bool need_hq = P->singles || !P->f_diag;

  // 3xTF32 residuals take the ring operand as TF32 planes written straight from t2p, and keep
  // the products that only the assembly reads (X, PQ, Zq, Yh) in complex FP32
  const bool ring_planes = prec == AGB_PREC_TF32X3;
  const int out32 = ring_planes ? 1 : 0;
  if (ring_planes) {
    const int64_t rp = tf32_rows_pad(ov), kp = tf32_k_pad(ov);
    // one warp per plane row; with singles it also forms the F_jb t2_ijab term into R1x
    unpack_ring_planes_kernel<<<grid_for(rp * 32, 256), 256, 0, st>>>(t2p, o, v, pv, rp, kp,
                                                                      P->singles ? P->EW : nullptr, P->R1x,
                                                                      (float*)P->Tring);
  } else {
    unpack_ring_kernel<<<grid_for(ov * ov, 256), 256, 0, st>>>(t2p, o, v, pv, P->Tring);
  }
  AGB_LAUNCH_CHECK();
  // 3xTF32 with a diagonal Fock matrix: t2h / t2q serve only the singles GEMMs, as planes
  const bool hq_planes = ring_planes && P->singles && P->f_diag;
  if (hq_planes) {
    const int kb = singles_kblk(P);
    const int64_t rh = tf32_rows_pad(o), kh = tf32_k_pad((int64_t)o * pv);
    unpack_h_planes_kernel<<<grid_for(rh * kh, 256), 256, 0, st>>>(t2p, o, pv, rh, kh, kb, (float*)P->t2h);
    AGB_LAUNCH_CHECK();
    const int64_t rq = tf32_rows_pad(v), kq = tf32_k_pad(po * v);
    unpack_q_planes_kernel<<<grid_for(rq * kq, 256), 256, 0, st>>>(t2p, po, v, pv, rq, kq, kb, (float*)P->t2q);
    AGB_LAUNCH_CHECK();
  } else if (need_hq) {
    unpack_h_kernel<<<grid_for((int64_t)o * o * pv, 256), 256, 0, st>>>(t2p, o, pv, P->t2h);
    AGB_LAUNCH_CHECK();
    unpack_q_kernel<<<grid_for(po * v * v, 256), 256, 0, st>>>(t2p, po, v, pv, P->t2q);
    AGB_LAUNCH_CHECK();
  }

  if (P->singles) {
    // r1 = F_ai - F_ji t1_ja + F_ab t1_ib + <ja||bi> t1_jb + F_jb t2_ijab + 1/2 <aj||cb> t2_ijcb
    //      - 1/2 <kj||ib> t2_kjab - E t1                                    (apyib/ci_wfn.py:309-316)
    r1_init_kernel<<<grid_for(n1, 256), 256, 0, st>>>((flags & AGB_RES_CONST) ? P->FvoT : nullptr,
                                                      ring_planes ? P->R1x : nullptr, n1, r1);
    AGB_LAUNCH_CHECK();
    AGB_STATUS_TRY(gemm(P, prec, o, v, o, zmk(-1, 0), P->Foo, 1, o, t1, v, 1, one, r1, v, st));
    AGB_STATUS_TRY(gemm(P, prec, o, v, v, one, t1, v, 1, P->Fvv, 1, v, one, r1, v, st));
    // FP64 mode keeps the FP64 pipe, the FP64-accurate modes take the double-float GEMV
    // (~2^-44), the 3xTF32 mode an FP32 one (its GEMM terms carry FP32-level error)
    auto gemv = prec == AGB_PREC_FP64 ? zgemv : (prec == AGB_PREC_TF32X3 ? zgemv_f32 : zgemv_df);
    AGB_STATUS_TRY(gemv(ov, ov, one, P->VT, ov, t1, one, r1, st));
    // (3xTF32: the F_jb t2_ijab term came with the ring planes, added by r1_init)
    if (!ring_planes) {
      AGB_STATUS_TRY(gemv(ov, ov, one, P->Tring, ov, P->EW, one, r1, st));
    }
    // The singles GEMMs run with the long or static extent as M and the o-wide one as N:
    // under 3xTF32 an o-wide N takes the 64-wide tile and the transposed store keeps the
    // output's writes coalesced (r1 and Yh are i-major, Zq a-minor).
    // r1[i][a] += sum_(j,p(cb)) <aj||cb> t2h[i][j][p(cb)]
    const int kb = singles_kblk(P);
    AGB_STATUS_TRY(gemm(P, prec, v, o, (int64_t)o * pv, one, P->WvovvH, (int64_t)o * pv, 1, P->t2h, 1,
                        (int64_t)o * pv, one, r1, v, st, P->P_Wvovv, hq_planes ? (const float*)P->t2h : nullptr, 1,
                        kb));
    // r1[i][a] += sum_(p(kj),b) <kj||ib> t2q[p(kj)][b][a]
    AGB_STATUS_TRY(gemm(P, prec, v, o, po * v, one, P->t2q, 1, v, P->WooovP, 1, po * v, one, r1, v, st,
                        hq_planes ? (const float*)P->t2q : nullptr, P->P_Wooov, 1, kb));
    if (flags & AGB_RES_ETERM) {
      axpy_kernel<<<grid_for(n1, 256), 256, 0, st>>>(n1, zneg(E), t1, r1);
      AGB_LAUNCH_CHECK();
    }
    // Zq[p(ij)][b][a] = sum_k <kb||ij> t1[k,a];  Yh[i][j][p(ab)] = sum_c t1[i,c] <ab||cj>
    AGB_STATUS_TRY(gemm(P, prec, v, po * v, o, one, t1, 1, v, P->WovooP, 1, o, zero, P->Zq, v, st, nullptr,
                        P->P_Wovoo, 1, kb, out32));
    AGB_STATUS_TRY(gemm(P, prec, (int64_t)o * pv, o, v, one, P->WvvvoP, 1, (int64_t)o * pv, t1, 1, v, zero, P->Yh,
                        (int64_t)o * pv, st, P->P_Wvvvo, nullptr, 1, kb, out32));
  }
  // ladders: PQ = sum_{k<l} <kl||ij> t2p[kl,ab] + sum_{c<d} t2p[ij,cd] <ab||cd>
  AGB_STATUS_TRY(gemm(P, prec, po, pv, po, one, P->WooooT, po, 1, t2p, pv, 1, zero, P->PQ, pv, st, P->P_Woooo,
                      nullptr, 0, 0, out32));
  AGB_STATUS_TRY(gemm(P, prec, po, pv, pv, one, t2p, pv, 1, P->Wvp, 1, pv, one, P->PQ, pv, st, nullptr, P->P_Wvp, 0,
                      0, out32));
  // rings: X[(i,a),(j,b)] = sum_(k,c) t2[i,k,a,c] <kb||cj>
  AGB_STATUS_TRY(gemm(P, prec, ov, ov, ov, one, P->Tring, ov, 1, P->VT, 1, ov, zero, P->X, ov, st,
                      ring_planes ? (const float*)P->Tring : nullptr, P->P_VT, 0, 0, out32));
  if (!P->f_diag) {
    AGB_STATUS_TRY(gemm(P, prec, po * v, v, v, one, P->t2q, v, 1, P->Fvv, 1, v, zero, P->Gq, v, st));
    AGB_STATUS_TRY(gemm(P, prec, o, (int64_t)o * pv, o, one, P->Foo, 1, o, P->t2h, (int64_t)o * pv, 1, zero, P->H2h,
                        (int64_t)o * pv, st));
  }
  if (po > 0 && pv > 0) {
    AsmArgs A;
    A.o = o; A.v = v; A.ov = ov; A.po = po; A.pv = pv; A.opairs = P->opairs;
    A.R0p = P->R0p; A.PQ = P->PQ; A.X = P->X; A.Zq = P->Zq; A.Yh = P->Yh; A.Gq = P->Gq; A.H2h = P->H2h;
    A.out32 = out32;
    A.t2p = t2p; A.eps = P->eps; A.Foo = P->Foo; A.Fvv = P->Fvv; A.E = E;
    A.use_const = (flags & AGB_RES_CONST) != 0; A.use_e = (flags & AGB_RES_ETERM) != 0;
    A.singles = P->singles; A.f_diag = P->f_diag; A.r2p = r2p;
    int nt = (v + TS - 1) / TS;
    dim3 grid(nt * (nt + 1) / 2, (unsigned)po);
    if (prec == AGB_PREC_TF32X3) assemble_r2_kernel<float2><<<grid, 256, 0, st>>>(A);
    else assemble_r2_kernel<z64><<<grid, 256, 0, st>>>(A);
    AGB_LAUNCH_CHECK();
  }
  return AGB_OK;
}

agb_status agb_scratch_status(void* scratch, void* stream);

agb_status agb_cisd_status(agb_cisd_plan* P, void* stream) {
  AGB_ARG_CHECK(P && P->ws, "status: plan without workspace");
  return agb_scratch_status(P->gemm_scratch, stream);
}

agb_status agb_cisd_update(agb_cisd_plan* P, const void* t, const void* r, void* t_out, void* stream) {
  AGB_ARG_CHECK(P && P->ws && t && r && t_out, "update: bad argument");
  int64_t n = P->n1 + P->n2;
  update_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(vdims_of(P), n, (const z64*)t, (const z64*)r,
                                                                    (z64*)t_out);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

agb_status agb_cisd_guess(agb_cisd_plan* P, void* t, void* stream) {
  AGB_ARG_CHECK(P && P->ws && t, "guess: bad argument");
  int64_t n = P->n1 + P->n2;
  guess_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(vdims_of(P), n, P->FvoT, P->R0p, (z64*)t);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

// Each block stores the full slot width of the kernel instance that serves ny vectors
// (4, 8, 12 or 16; 3 for the combination's E, s1, s2), not just ny.
size_t agb_vec_partials_bytes(int ny) {
  const int nv = ny <= 4 ? 4 : (ny <= 8 ? 8 : (ny <= 12 ? 12 : 16));
  return sizeof(z64) * (size_t)kRedBlocks * (size_t)(nv > 3 ? nv : 3);
}

agb_status agb_vec_dots(int64_t n1, int64_t n2, double w1, double w2, const void* x, const void* const* ys, int ny,
                        void* out, void* partials, size_t partials_bytes, void* stream) {
  AGB_ARG_CHECK(x && ys && out && n1 >= 0 && n2 >= 0 && ny >= 1 && ny <= kMaxVec, "vec_dots: bad argument");
  if (!partials || partials_bytes < agb_vec_partials_bytes(ny)) {
    agb_set_error_message("vec_dots: partials buffer too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  DotArgs A;
  A.n1 = n1; A.n2 = n2; A.w1 = w1; A.w2 = w2; A.x = (const z64*)x; A.ny = ny;
  for (int j = 0; j < kMaxVec; ++j) A.ys[j] = j < ny ? (const z64*)ys[j] : nullptr;
  z64* part = (z64*)partials;
  const int nv = launch_dots(A, ny, part, st);
  AGB_LAUNCH_CHECK();
  // finish only the first ny of the nv slots (stride nv)
  finish_partials_kernel<<<ny, 256, 0, st>>>(part, kDotBlocks, nv, ny, (z64*)out);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// agb_vec_dots_noalloc: the DIIS Gram-row reduction for callers that cannot
// allocate device memory.  Its block partial sums live in the file-scope array
// below (kRedBlocks x 16 complex doubles = 155,648 bytes), which every context
// that loads this library keeps until the process exits.
//
// The host-side name of a __device__ array is not a device address: its address
// is looked up with cudaGetSymbolAddress in the context current at the call and
// cached under that context's unique id (cuCtxGetId ids are never reused within a
// process), so a device reset, or a caller that makes its own non-primary context
// current, gets a fresh lookup instead of a stale pointer.
namespace {
constexpr int kNoAllocMaxVec = 16;
__device__ __align__(256) z64 g_dots_noalloc_scratch[kRedBlocks * kNoAllocMaxVec];
std::mutex g_noalloc_mu;
constexpr size_t kNoAllocMaxContexts = 64;
std::vector<std::pair<unsigned long long, void*>> g_noalloc_cache;   // (context id, array address)

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

// Unique id of the calling thread's current context; false if no context is bound to
// the thread yet (the runtime binds the device's primary context at its first call that
// needs one, e.g. cudaGetSymbolAddress) or the driver cannot tell.
bool current_context_id(unsigned long long* id) {
  struct Fns {
    PfnCtxGetCurrent get_cur = nullptr;
    PfnCtxGetId get_id = nullptr;
  };
  // looked up once, by the first caller (a function-local static is initialised exactly once)
  static const Fns fns = [] {
    Fns r;
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      r.get_cur = (PfnCtxGetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      r.get_id = (PfnCtxGetId)f;
    return r;
  }();
  const PfnCtxGetCurrent get_cur = fns.get_cur;
  const PfnCtxGetId get_id = fns.get_id;
  if (!get_cur || !get_id) return false;
  CUcontext ctx = nullptr;
  if (get_cur(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}
}  // namespace

extern "C" {

agb_status agb_vec_dots_noalloc(int64_t n1, int64_t n2, double w1, double w2, const void* x, const void* const* ys,
                                int ny, void* out, void* stream) {
  AGB_ARG_CHECK(x && ys && out && n1 >= 0 && n2 >= 0, "vec_dots_noalloc: bad argument");
  if (ny < 1 || ny > kNoAllocMaxVec) {
    agb_set_error_message("vec_dots_noalloc: ny must be between 1 and 16 (the fixed scratch holds 16 partial sums "
                          "per block)", __FILE__, __LINE__);
    return AGB_ERR_ARG;
  }
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    unsigned long long ctx_id = 0;
    if (current_context_id(&ctx_id))
      for (auto& e : g_noalloc_cache)
        if (e.first == ctx_id) scratch = e.second;
    if (!scratch) {
      // Set-up for this context (its device is current): look the address up once.
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_dots_noalloc_scratch);
      if (e != cudaSuccess || p == nullptr) {
        agb_set_error_message(cudaGetErrorString(e), __FILE__, __LINE__);
        return AGB_ERR_CUDA;
      }
      scratch = p;
      if (current_context_id(&ctx_id) && g_noalloc_cache.size() < kNoAllocMaxContexts)
        g_noalloc_cache.emplace_back(ctx_id, p);
    }
  }
  cudaStream_t st = (cudaStream_t)stream;
  DotArgs A;
  A.n1 = n1; A.n2 = n2; A.w1 = w1; A.w2 = w2; A.x = (const z64*)x; A.ny = ny;
  for (int j = 0; j < kMaxVec; ++j) A.ys[j] = j < ny ? (const z64*)ys[j] : nullptr;
  // Every partial slot read below is written earlier in this same call, so the
  // array's previous contents never leak into the result.
  z64* part = (z64*)scratch;
  const int nv = launch_dots(A, ny, part, st);
  AGB_LAUNCH_CHECK();
  finish_partials_kernel<<<ny, 256, 0, st>>>(part, kDotBlocks, nv, ny, (z64*)out);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

agb_status agb_cisd_combine(agb_cisd_plan* P, const void* const* ys, const double* coefs, int ny, const void* t_old,
                            void* t_new, void* out3, void* partials, size_t partials_bytes, void* stream) {
  AGB_ARG_CHECK(P && P->ws && ys && coefs && t_old && t_new && out3, "combine: bad argument");
  AGB_ARG_CHECK(ny >= 1 && ny <= kMaxVec, "combine: 1 <= ny <= 16");
  if (!partials || partials_bytes < agb_vec_partials_bytes(3)) {
    agb_set_error_message("combine: partials buffer too small", __FILE__, __LINE__);
    return AGB_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  CombArgs A;
  A.n1 = P->n1; A.n2 = P->n2; A.ny = ny;
  for (int j = 0; j < kMaxVec; ++j) {
    A.ys[j] = j < ny ? (const z64*)ys[j] : nullptr;
    A.c[2 * j] = j < ny ? coefs[2 * j] : 0.0;
    A.c[2 * j + 1] = j < ny ? coefs[2 * j + 1] : 0.0;
  }
  A.csum = zmk(0, 0);
  for (int j = 0; j < ny; ++j) A.csum = zadd(A.csum, zmk(coefs[2 * j], coefs[2 * j + 1]));
  A.t_old = (const z64*)t_old; A.t_new = (z64*)t_new; A.ew = P->EW;
  combine_kernel<<<kRedBlocks, 256, 0, st>>>(A, (z64*)partials);
  AGB_LAUNCH_CHECK();
  finish_partials_kernel<<<3, 256, 0, st>>>((const z64*)partials, kRedBlocks, 3, 3, (z64*)out3);
  AGB_LAUNCH_CHECK();
  return AGB_OK;
}

}  // extern "C"
