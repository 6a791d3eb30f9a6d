// Device helpers of the slice-product kernels (gemm_tc.cu): strided index
// decoding, the per-row binary exponents, the
// cut of a scaled double into balanced BF16-exact digits, and the exact
// conversion of an int64 sum back to a scaled double.
#pragma once

#include <cstdint>

#include "engine.h"

namespace tdcc {

// Offset of index l < prod(dim) of a mode group (last mode fastest).
__device__ __forceinline__ void decomp_tc(const ModeGroup& g, int l, long long& o0) {
  if (g.n == 1) {  // l < dim[0]: no division
    o0 = (long long)l * g.s0[0];
    return;
  }
  o0 = 0;
#pragma unroll
  for (int q = kMaxModes - 1; q >= 1; --q) {
    if (q < g.n) {
      const int d = g.dim[q];
      const int r = l % d;
      l /= d;
      o0 += (long long)r * g.s0[q];
    }
  }
  o0 += (long long)l * g.s0[0];  // l < dim[0]: the outermost mode needs no division
}

// Row exponents are stored biased (e + kExpBias; 0 = all-zero row) so that
// zero-initialised memory and atomicMax give the maximum directly.
constexpr int kExpBias = 4096;
__device__ __forceinline__ int row_exp(int biased) { return biased > 0 ? biased - kExpBias : 0; }

// floor(|x| 2^(nbits - e)) as an integer, from the bits of x (exact; no FP64
// arithmetic).  Requires |x| < 2^e and nbits <= 56, so the result < 2^nbits.
__device__ __forceinline__ unsigned long long fixed_point(double x, int e, int nbits) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
  const int E = (int)(u >> 52);
  if (E == 0) return 0ull;  // zero or subnormal: below every slice
  const unsigned long long M = (u & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
  const int sh = E - 1075 - e + nbits;  // |x| = M 2^(E-1075)
  if (sh >= 0) return M << sh;
  if (sh <= -64) return 0ull;
  return M >> (-sh);
}

// The digits of f < 2^(7S) in balanced form, least significant first:
// every digit below the top one in [-64, 63] (a digit >= 64 becomes d - 128
// with a carry into the next), the top one in [0, 128].  The value is f
// itself, sum_s q[s] 2^(7(S-1-s)), and products of digits stay within 2^14.
template <int SMAX>
__device__ __forceinline__ void balanced_digits(unsigned long long f, int S, int (&q)[SMAX]) {
#pragma unroll
  for (int i = SMAX - 1; i >= 1; --i)
    if (i < S) {
      int d = (int)(f & 127ull);
      f >>= 7;
      if (d >= 64) {
        d -= 128;
        ++f;
      }
      q[i] = d;
    }
  q[0] = (int)f;
}

// (float)d for |d| < 2^22 with one integer and one FP32 addition, both on
// full-rate pipes (an int-to-float conversion runs at a quarter of that):
// 0x4B400000 is the float 1.5 * 2^23, whose neighbours are 1 apart, so its
// bits + d are the float 1.5 * 2^23 + d, and the subtraction is exact.  d = 0
// gives +0, as the conversion does.
__device__ __forceinline__ float small_int_to_float(int d) {
  return __int_as_float(0x4B400000 + d) - 12582912.0f;
}

// Two digits (|d| <= 128, at most 8 significant bits: exact in BF16, whose
// bits are then the upper half of the float's) as a BF16 pair, d0 in the low
// half (the lower address).
__device__ __forceinline__ uint32_t digit_pair_bf16x2(int d0, int d1) {
  return __byte_perm(__float_as_uint(small_int_to_float(d0)), __float_as_uint(small_int_to_float(d1)), 0x7632);
}

// Subnormal or overflowing results (not met by the contractions here) take
// the FP64 path, out of line so that nothing of it is evaluated on the
// normal path.
static __device__ __noinline__ double scaled_i64_to_double_rare(long long x, int E) { return ldexp((double)x, E); }

// x * 2^E rounded to nearest (ties to even) from the integer's bits, without
// branches on the normal-range path and no FP64 arithmetic (GB300's FP64
// pipe is narrow): the magnitude is normalised to bit 63, its top 53 bits
// are the significand, the 11 bits below round it, and a carry out of the
// significand rounds up into the exponent field by the integer addition.
__device__ __forceinline__ double scaled_i64_to_double(long long x, int E) {
  const unsigned long long sgn = (unsigned long long)(x >> 63);  // all ones when negative
  const unsigned long long u = ((unsigned long long)x ^ sgn) - sgn;
  if (u == 0ull) return 0.0;
  const int lz = __clzll((long long)u);
  const unsigned long long m = u << lz;  // leading one at bit 63
  const unsigned long long mant = m >> 11;  // 53 bits, leading one at bit 52
  const unsigned rem = (unsigned)(m & 0x7FFull);
  const unsigned long long up = (rem > 0x400u || (rem == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
  const int be = 63 - lz + E + 1023;  // biased exponent before rounding
  if (be <= 0 || be >= 2047) return scaled_i64_to_double_rare(x, E);
  // the leading one of mant adds 1 to the exponent field (be - 1 + 1)
  const unsigned long long bits = ((unsigned long long)(be - 1) << 52) + mant + up;
  return __longlong_as_double((long long)(bits | (sgn << 63)));
}

}  // namespace tdcc
