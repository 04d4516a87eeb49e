// Integer-only splits of an FP64 value into float pieces.  GB300 executes
// double<->float conversions on its narrow FP64 pipe; these use the integer
// pipe instead (sign / exponent / significand arithmetic on the bit pattern).
// Values below the FP32 normal range flush to zero.
#pragma once
#include <stdint.h>

namespace agb {

// float from sign, unbiased exponent E of the leading bit, and a normalized 24-bit significand sig (bit 23 set),
// flushed to zero below the normal range.
__device__ __forceinline__ uint32_t pack_f32(uint32_t s, int E, uint32_t sig) {
  int fe = E + 127;
  if (fe <= 0 || sig == 0) return s << 31;
  if (fe >= 255) return (s << 31) | 0x7f800000u;
  return (s << 31) | ((uint32_t)fe << 23) | (sig & 0x7fffffu);
}
// x = hi + lo + O(2^-23 |x|) in TF32 (10-bit mantissas) from the two 32-bit words of an FP64
// value, on 32-bit integer operations and one int -> float conversion (a 64-bit-integer
// version kept the operand-split kernel integer-issue bound).  hi: the top 11 significant bits rounded half
// away from zero, straight from the high word (adding 2^9 there is adding 2^41 to the
// significand; a carry into the exponent is the IEEE rounding overflow), rebiased to FP32.
// lo: the remainder x - hi is the low 42 bits of the significand read as a two's-complement
// number (negative when the rounding went up), times 2^(E-52); its top 32 bits convert to
// float, the scale 2^(E-42) goes into the exponent field, and the result rounds to TF32.
// |x - hi - lo| <= 2^-23 |x| (tests/test_split_spec.py restates these steps in NumPy and
// checks the bound over 60 decades); values below the FP32 normal range give zero.
__device__ __forceinline__ void split_tf32_fast(uint32_t hw, uint32_t lw, uint32_t& hi, uint32_t& lo) {
  const uint32_t sign = hw & 0x80000000u;
  const int e = (int)((hw >> 20) & 0x7ffu);
  const uint32_t hr = (hw + 0x200u) & 0xfffffc00u;
  const int eh = (int)((hr >> 20) & 0x7ffu);
  hi = e > 896 ? (sign | ((uint32_t)(eh - 896) << 23) | ((hr & 0x000ffc00u) << 3)) : sign;
  const int q = (int)(((hw & 0x3ffu) << 22) | (lw >> 10));          // remainder / 2^10, sign-extended
  const uint32_t qf = __float_as_uint((float)q);
  const int sh = e - 1023 - 42;
  const int ne = (int)((qf >> 23) & 0xffu) + sh;
  uint32_t l = (q != 0 && ne > 0 && e > 896) ? qf + ((uint32_t)sh << 23) : 0u;
  l = (l + 0x1000u) & 0xffffe000u;                                   // round to TF32, half away
  lo = l ^ sign;
}

// x = hi + lo with hi = float(x) (nearest-even) and lo = float(x - hi): the double-float split.
__device__ __forceinline__ void split_f32pair(uint64_t u, uint32_t& hi, uint32_t& lo) {
  uint32_t s = (uint32_t)(u >> 63);
  int e = (int)((u >> 52) & 0x7ff);
  if (e == 0 || e == 0x7ff) { hi = s << 31; lo = s << 31; return; }
  int64_t S = (int64_t)((u & ((1ull << 52) - 1)) | (1ull << 52));
  int E = e - 1023;
  // round to 24 bits, nearest-even on bit 28
  int64_t keep = S >> 29, rem = S & ((1ll << 29) - 1);
  int64_t half = 1ll << 28;
  if (rem > half || (rem == half && (keep & 1))) keep += 1;
  int64_t Shi = keep << 29;
  int64_t r = S - Shi;
  int Eh = E;
  if (keep == (1ll << 24)) { Eh = E + 1; keep >>= 1; }
  hi = pack_f32(s, Eh, (uint32_t)keep);
  if (r == 0) { lo = s << 31; return; }
  uint32_t ls = s ^ (r < 0 ? 1u : 0u);
  uint64_t ar = (uint64_t)(r < 0 ? -r : r);
  int lz = __clzll(ar);
  int msb = 63 - lz;                                                  // <= 28
  uint64_t A = ar << (52 - msb);
  // round to 24 bits nearest-even (|r| has at most 29 bits, so this is exact or one rounding)
  uint64_t k2 = A >> 29, rm = A & ((1ull << 29) - 1);
  if (rm > (1ull << 28) || (rm == (1ull << 28) && (k2 & 1))) k2 += 1;
  int El = E - 52 + msb;
  if (k2 == (1ull << 24)) { El += 1; k2 >>= 1; }
  lo = pack_f32(ls, El, (uint32_t)k2);
}

// Cheap x ~ hi + lo for streamed operands: hi = x truncated to 24 significant bits,
// lo = the next 23 bits (the last 6 of x's 52 fraction bits dropped), so
// |x - hi - lo| < 2^-46 |x|.  About 20 integer/FP32 operations and no FP64 instruction.
// Range: |x| < 2^128 is split as above; |x| >= 2^128 (and inf / NaN) gives hi = +-inf and
// lo = 0, so a sum fed out-of-range values comes out non-finite instead of plausibly wrong;
// |x| < 2^-126 gives hi = 0 and |x| < 2^-112 gives lo = 0 (an absolute error below 2^-112).
__device__ __forceinline__ void split_f32pair_fast(double x, float& hi, float& lo) {
  const uint32_t hw = (uint32_t)__double2hiint(x), lw = (uint32_t)__double2loint(x);
  const uint32_t ex = (hw >> 20) & 0x7ffu;                          // biased FP64 exponent
  const uint32_t sign = hw & 0x80000000u;
  const uint32_t frac23 = __funnelshift_l(lw, hw, 3) & 0x7fffffu;    // top 23 fraction bits
  const bool big = ex >= 1151u;                                     // |x| >= 2^128: no FP32 exponent
  hi = __uint_as_float(big ? (sign | 0x7f800000u) : (ex > 896u ? (sign | ((ex - 896u) << 23) | frac23) : sign));
  const uint32_t m = (lw >> 6) & 0x7fffffu;                         // next 23 fraction bits, weight 2^(E-46)
  const float mf = __fsub_rn(__uint_as_float(0x4b000000u | m), 8388608.0f);   // exactly m
  // 2^(E-46) = 2^(E-14) * 2^-32, so the scale factor stays a normal float down to E = -112
  lo = (ex > 910u && !big)
           ? __fmul_rn(__fmul_rn(__uint_as_float(sign | ((ex - 910u) << 23)), mf), 2.3283064365386963e-10f)
           : 0.0f;
}

}  // namespace agb
