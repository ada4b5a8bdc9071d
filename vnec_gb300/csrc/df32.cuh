// Double-float arithmetic on the FP32 pipe (a value held as an unevaluated sum
// hi + lo of two floats), shared by the DF32 forms of the merge-path, sliced
// and batched kernels.  GB300 runs FP64 FMA at 1/64 of the FP32 rate; these
// operations give products and sums with ~2^-46 relative error from FP32
// instructions only.
#pragma once

namespace vnec {

struct DF {
  float s, c;  // value = s + c
};

// Truncation split of a double into hi + lo floats (integer operations only):
// hi keeps the top 24 significand bits, lo the next 29 rounded down to 24.
// Returns false when a nonzero v lies outside [2^-40, 2^41) or is not finite
// (both halves and their products must stay normal FP32 numbers).
__device__ __forceinline__ bool df_split(double v, float& hi, float& lo) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
  const unsigned sign = static_cast<unsigned>(b >> 63) << 31;
  const int e = static_cast<int>((b >> 52) & 0x7ff);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  if (e == 0 && m == 0) {
    hi = 0.0f;
    lo = 0.0f;
    return true;
  }
  const int E = e - 1023;
  const bool ok = (E >= -40) && (E <= 40);
  hi = __uint_as_float(sign | (static_cast<unsigned>(E + 127) << 23) | static_cast<unsigned>(m >> 29));
  const unsigned rem = static_cast<unsigned>(m & 0x1FFFFFFFull);
  const int msb = 31 - __clz(rem | 1u);  // 0..28 (rem == 0 handled below)
  const unsigned mant = msb > 23 ? (rem >> (msb - 23)) : (rem << (23 - msb));
  lo = rem ? __uint_as_float(sign | (static_cast<unsigned>(E - 52 + msb + 127) << 23) | (mant & 0x7FFFFFu)) : 0.0f;
  return ok;
}

// acc + (ah + al) (xh + xl): Dekker's exact product of the high parts with an
// FMA (ah xh = p + e), the cross terms folded into e, and Knuth's TwoSum of
// the running high part with p; the low-order terms collect in acc.c.
__device__ __forceinline__ DF df_mac(DF acc, float ah, float al, float xh, float xl) {
  const float p = __fmul_rn(ah, xh);
  const float e = fmaf(ah, xh, -p);
  const float q = fmaf(ah, xl, fmaf(al, xh, e));
  const float t = __fadd_rn(acc.s, p);
  const float bb = __fsub_rn(t, acc.s);
  const float r = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
  return DF{t, __fadd_rn(acc.c, __fadd_rn(r, q))};
}

__device__ __forceinline__ double df_to_f64(DF a) { return static_cast<double>(a.s) + static_cast<double>(a.c); }

}  // namespace vnec
