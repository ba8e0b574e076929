// Correctly rounded binary64 multiplication on the integer pipes.
//
// GB300 executes 2 FP64 lane-operations per clock per SM, 1/64 of its FP32
// rate, while the integer and FP32 pipes and most issue slots sit idle in
// the FP64-bound SD-ADER kernels.  emul_mul computes the IEEE-754
// round-to-nearest-even product of two doubles with 64-bit integer
// arithmetic (IMAD / shifts), so part of the multiplications run beside the
// FP64 pipe instead of on it.  The result is the same bits as the FP64
// multiply (it is the same mathematical operation: exact 106-bit product of
// the significands, then rounding to 53 bits), which keeps the kernels
// bit-identical to the reference.
//
// Fast path: both operands normal and the rounded product normal.  Zero,
// subnormal, infinite and NaN operands, and products that overflow or fall
// below the normal range, take the FP64 multiply (mul_slow), so every
// special case has the hardware's own result.
#pragma once
#include <cstdint>

namespace spd {

static __device__ __noinline__ double mul_slow(double a, double b) { return __dmul_rn(a, b); }

__device__ __forceinline__ double emul_mul(double a, double b) {
  const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
  const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
  const unsigned ea = (unsigned)(ua >> 52) & 0x7ffu;
  const unsigned eb = (unsigned)(ub >> 52) & 0x7ffu;
  const unsigned long long frac = 0x000FFFFFFFFFFFFFull;
  const unsigned long long ma = (ua & frac) | 0x0010000000000000ull;  // 53-bit significands
  const unsigned long long mb = (ub & frac) | 0x0010000000000000ull;
  // high 64 bits of (ma * 2^11) * (mb * 2^11) = ma*mb / 2^42, in [2^62, 2^64)
  const unsigned long long hi = __umul64hi(ma << 11, mb << 11);
  const unsigned top = (unsigned)(hi >> 63);  // ma*mb >= 2^105
  const unsigned sh = 10u + top;              // bits of hi below the 53-bit result
  unsigned long long m = hi >> sh;
  const unsigned guard = (unsigned)(hi >> (sh - 1u)) & 1u;
  // the bits below the guard bit are nonzero iff the exact product has a set
  // bit below position 42 + sh - 1; its lowest set bit is tz(ma) + tz(mb)
  const unsigned tz = (unsigned)(__ffsll((long long)ma) - 1) + (unsigned)(__ffsll((long long)mb) - 1);
  const unsigned sticky = tz < 41u + sh;
  m += (unsigned long long)(guard & (sticky | (unsigned)(m & 1ull)));
  int e = (int)ea + (int)eb - 1023 + (int)top;
  const unsigned carry = (unsigned)(m >> 53);  // rounding overflowed to 2^53
  m >>= carry;
  e += (int)carry;
  const bool fast = (ea - 1u < 2046u) & (eb - 1u < 2046u) & (e >= 1) & (e <= 2046);
  if (!fast) return mul_slow(a, b);
  const unsigned long long r = ((ua ^ ub) & 0x8000000000000000ull) | ((unsigned long long)e << 52) | (m & frac);
  return __longlong_as_double((long long)r);
}

}  // namespace spd
