// Double-float (float pair) arithmetic on the FP32 pipe: FP64-level products
// and sums for kernels whose FP64 instruction count would otherwise bound them
// (GB300 issues FP32 about 64x faster than FP64).
#pragma once
#include "common.cuh"
#include "fsplit.cuh"

namespace agb {

// (re_hi, re_lo, im_hi, im_lo) of a complex FP64 value, split on the integer pipe.
__device__ __forceinline__ float4 split_z(z64 v) {
  uint32_t rh, rl, ih, il;
  split_f32pair((uint64_t)__double_as_longlong(v.x), rh, rl);
  split_f32pair((uint64_t)__double_as_longlong(v.y), ih, il);
  return make_float4(__uint_as_float(rh), __uint_as_float(rl), __uint_as_float(ih), __uint_as_float(il));
}

// (s, c) += (xh + xl) * (yh + yl): exact FMA product split, cross terms, Knuth two-sum.
// The _rn intrinsics keep the compiler from contracting the rounded product into
// the two-sum (which would void it).
__device__ __forceinline__ void df_mac(float& s, float& c, float xh, float xl, float yh, float yl) {
  float p = __fmul_rn(xh, yh);
  float e = fmaf(xh, yh, -p);
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  float t = __fadd_rn(s, p);
  float z = __fsub_rn(t, s);
  float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
  c = __fadd_rn(c, __fadd_rn(err, e));
  s = t;
}

// (s, c) += (bs, bc): sum of two float pairs (two-sum of the leading parts).
__device__ __forceinline__ void df_add(float& s, float& c, float bs, float bc) {
  float t = __fadd_rn(s, bs);
  float z = __fsub_rn(t, s);
  float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(bs, z));
  c = __fadd_rn(__fadd_rn(c, bc), err);
  s = t;
}

// Streamed complex value as (re_hi, re_lo, im_hi, im_lo) with the cheap split (~2^-46 relative).
__device__ __forceinline__ float4 split_z_fast(z64 v) {
  float4 r;
  split_f32pair_fast(v.x, r.x, r.y);
  split_f32pair_fast(v.y, r.z, r.w);
  return r;
}

// Exact double of a float, integer pipe only (FP32 subnormals give zero).
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  const uint64_t s = (uint64_t)(u >> 31) << 63;
  if (e == 0) return __longlong_as_double((long long)s);
  return __longlong_as_double((long long)(s | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(u & 0x7fffffu) << 29)));
}

// hi + lo as a double (one FP64 add).
__device__ __forceinline__ double df_to_double(float hi, float lo) { return f2d_exact(hi) + f2d_exact(lo); }

// Renormalise a float pair so that |lo| <= ulp(hi)/2 (two-sum of its parts).
__device__ __forceinline__ void df_norm(float& s, float& c) {
  const float t = __fadd_rn(s, c);
  const float z = __fsub_rn(t, s);
  c = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(c, z));
  s = t;
}

}  // namespace agb
