// Conversions between binary32 and binary64 on the integer pipe.
//
// GB300 executes binary64 arithmetic, and the hardware conversions between binary32 and binary64,
// on a narrow pipe (about 2 lanes per SM per clock, 1/64 of binary32).  The binary32 node update
// converts every force to binary64 and every new velocity and displacement back to binary32, which
// made those conversions two thirds of its binary64 instructions.  Both directions are plain
// re-encodings of the IEEE 754 formats (1 sign, 8 exponent bits biased by 127, 23 fraction bits;
// 1 sign, 11 exponent bits biased by 1023, 52 fraction bits), done here entirely with integer
// operations, so that no path of the node update issues on the binary64 pipe for a conversion:
//   widen:  exact for every input (normal, subnormal, zero, infinity; a NaN stays a NaN);
//   narrow: round to nearest, ties to even, including the carry into the exponent, overflow to
//           infinity, and results in the binary32 subnormal range or below; a NaN stays a NaN.
// They give the hardware conversions' bits on every non-NaN input (eqd_gpu_check_conversions).
#pragma once

namespace eqd {

__device__ __forceinline__ double widen_f32(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u, mag = u & 0x7fffffffu;
  unsigned hi, lo;
  if (mag - 0x00800000u < 0x7f000000u) {  // normal: biased exponent 1..254
    // the exponent field moves from bit 23 to bit 52 (hi bit 20) with the bias 1023 - 127 = 896
    // added; the 23 fraction bits become the top of the 52-bit fraction
    hi = ((mag >> 3) + (896u << 20)) | sign;
    lo = u << 29;
  } else if (mag >= 0x7f800000u) {  // infinity (fraction 0) or NaN (fraction kept)
    hi = sign | 0x7ff00000u | ((mag & 0x007fffffu) >> 3);
    lo = mag << 29;
  } else if (mag == 0u) {
    hi = sign;
    lo = 0u;
  } else {  // subnormal: value = mag * 2^-149; normalise on its leading one at bit k
    const int k = 31 - __clz(mag);
    const unsigned long long frac = (unsigned long long)(mag & ((1u << k) - 1u)) << (52 - k);
    hi = sign | ((unsigned)(k + 874) << 20) | (unsigned)(frac >> 32);
    lo = (unsigned)frac;
  }
  return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ float narrow_f64(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned sign = hi & 0x80000000u, mag = hi & 0x7fffffffu;
  if (mag - (897u << 20) < (254u << 20)) {  // binary64 exponent 897..1150: binary32 exponent 1..254
    // top 23 fraction bits under the rebased exponent; the 29 dropped bits decide the rounding
    unsigned b = ((mag - (896u << 20)) << 3) | (lo >> 29);
    const unsigned r = lo & 0x1fffffffu;
    b += (unsigned)(r > 0x10000000u) | ((unsigned)(r == 0x10000000u) & b);
    return __uint_as_float(b | sign);
  }
  const unsigned e = mag >> 20;
  if (e >= 2047u) {  // infinity or NaN
    const bool nan = ((mag & 0x000fffffu) | lo) != 0u;
    return __uint_as_float(sign | (nan ? 0x7fc00000u : 0x7f800000u));
  }
  if (e >= 1151u) return __uint_as_float(sign | 0x7f800000u);  // above the binary32 range
  // binary32 subnormal range or below: value = M 2^(e - 1075) with the 53-bit significand M (or
  // the subnormal binary64 fraction); the result's units are 2^-149, so shift M right by 926 - e
  if (e == 0u) return __uint_as_float(sign);  // binary64 subnormal or zero: far below 2^-150
  const unsigned long long M = ((unsigned long long)(mag & 0x000fffffu) << 32 | lo) | (1ull << 52);
  const unsigned s = 926u - e;  // >= 30
  if (s > 53u) return __uint_as_float(sign);  // below half of the smallest subnormal
  unsigned long long q = M >> s;
  const unsigned long long rem = M & ((1ull << s) - 1ull), half = 1ull << (s - 1u);
  q += (rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull;
  return __uint_as_float(sign | (unsigned)q);
}

}  // namespace eqd
