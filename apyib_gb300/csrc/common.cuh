// Shared helpers for the apyib_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <vector>

#include "../../include/apyib_gb300.h"

namespace agb {

typedef double2 z64;   // complex double, interleaved (re, im)

// Benchmark instrumentation a plan keeps for itself: CUDA events bracketing each of its
// tcgen05 GEMM launches on the launch stream, with the launch's shape.
struct GemmTimingRec {
  cudaEvent_t e0, e1;
  double flops;          // 8 M N K
  int64_t M, N, K;
};
typedef std::vector<GemmTimingRec> GemmTimingLog;

// Operand-conjugation flag of the internal split kernels: 0 as stored, 1 conjugated,
// kSrcReal the operand is a real FP64 array (same strides, in doubles; imaginary part zero).
constexpr int kSrcReal = 2;

__host__ __device__ __forceinline__ z64 zmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ z64 zadd(z64 a, z64 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ z64 zsub(z64 a, z64 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ z64 zmul(z64 a, z64 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ z64 zscale(z64 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ z64 zneg(z64 a) { return make_double2(-a.x, -a.y); }
__host__ __device__ __forceinline__ z64 zconj(z64 a) { return make_double2(a.x, -a.y); }
// acc += a*b
__host__ __device__ __forceinline__ void zfma(z64& acc, z64 a, z64 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}

// Packed index of the pair p<q among n: rows p = 0..n-2, each holding q = p+1..n-1.
__host__ __device__ __forceinline__ int64_t pair_index(int64_t p, int64_t q, int64_t n) {
  return p * n - p * (p + 1) / 2 + (q - p - 1);
}
__host__ __device__ __forceinline__ int64_t npairs(int64_t n) { return n * (n - 1) / 2; }

// Inverse of pair_index (row p for packed index k), computed by a float guess then exact fix-up.
__host__ __device__ __forceinline__ void pair_from_index(int64_t k, int64_t n, int& p, int& q) {
  // row start s(p) = p*n - p(p+1)/2 ; find the largest p with s(p) <= k
  float b = 2.0f * (float)n - 1.0f;
  float disc = b * b - 8.0f * (float)k;
  int pp = (int)((b - sqrtf(disc > 0.f ? disc : 0.f)) * 0.5f);
  if (pp < 0) pp = 0;
  if (pp > n - 2) pp = (int)n - 2;
  while (pp > 0 && (int64_t)pp * n - (int64_t)pp * (pp + 1) / 2 > k) --pp;
  while (pp < n - 2 && (int64_t)(pp + 1) * n - (int64_t)(pp + 1) * (pp + 2) / 2 <= k) ++pp;
  p = pp;
  q = (int)(k - ((int64_t)pp * n - (int64_t)pp * (pp + 1) / 2)) + pp + 1;
}

inline int grid_for(int64_t n, int threads, int64_t cap = 152LL * 64) {
  int64_t g = (n + threads - 1) / threads;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace agb

#define AGB_CUDA_TRY(expr)                                                    \
  do {                                                                        \
    cudaError_t _e = (expr);                                                  \
    if (_e != cudaSuccess) {                                                  \
      agb_set_error_message(cudaGetErrorString(_e), __FILE__, __LINE__);      \
      return AGB_ERR_CUDA;                                                    \
    }                                                                         \
  } while (0)

#define AGB_LAUNCH_CHECK()          \
  do {                              \
    agb_count_launch();             \
    AGB_CUDA_TRY(cudaGetLastError()); \
  } while (0)

#define AGB_STATUS_TRY(expr)            \
  do {                                  \
    agb_status _s = (expr);             \
    if (_s != AGB_OK) return _s;        \
  } while (0)

#define AGB_ARG_CHECK(cond, msg)                                  \
  do {                                                            \
    if (!(cond)) {                                                \
      agb_set_error_message(msg, __FILE__, __LINE__);             \
      return AGB_ERR_ARG;                                         \
    }                                                             \
  } while (0)

namespace agb {
// Runs setup() once per device (CUDA keeps kernel attributes per device): `done` holds one
// bit per device ordinal; a setup that fails, or a device past ordinal 63, is tried again
// on the next call.
template <class F>
agb_status once_per_device(std::atomic<uint64_t>& done, F setup) {
  int dev = -1;
  const uint64_t bit = (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return AGB_OK;
  const agb_status st = setup();
  if (st == AGB_OK && bit) done.fetch_or(bit, std::memory_order_release);
  return st;
}
}  // namespace agb

void agb_set_error_message(const char* msg, const char* file, int line);
// Process-wide count of kernels this library has launched (diagnostics only).
void agb_count_launch();
