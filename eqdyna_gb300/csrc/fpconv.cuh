// Conversions between binary32 and binary64 on the integer pipe.
//
// GB300 executes binary64 arithmetic, and the hardware conversions between binary32 and binary64,
// on a narrow pipe (about 2 lanes per SM per clock, 1/64 of binary32).  The binary32 node update
// converts every force to binary64 and every new velocity and displacement back to binary32, which
// made those conversions two thirds of its binary64 instructions.  Both directions are plain
// re-encodings of the IEEE 754 formats (1 sign, 8 exponent bits biased by 127, 23 fraction bits;
// 1 sign, 11 exponent bits biased by 1023, 52 fraction bits), so for the common operands they are
// done here with a few 32-bit integer operations, and give the same bits as the hardware
// conversions:
//   widen:  binary32 normal numbers and zeros; subnormals, infinities and NaNs use the hardware
//           conversion (exact in every case);
//   narrow: results in the binary32 normal range (round to nearest, ties to even, including the
//           carry into the exponent and the overflow of the largest binade to infinity) and zeros;
//           results that would be binary32 subnormals, and infinities and NaNs, use the hardware
//           conversion.
#pragma once

namespace eqd {

__device__ __forceinline__ double widen_f32(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned mag = u & 0x7fffffffu;
  if (mag - 0x00800000u < 0x7f000000u) {  // biased exponent 1..254
    // exponent field moves from bit 23 to bit 52 (hi bit 20) with the bias 1023 - 127 = 896 added;
    // the 23 fraction bits become the top of the 52-bit fraction
    const unsigned hi = ((mag >> 3) + (896u << 20)) | (u & 0x80000000u);
    return __hiloint2double((int)hi, (int)(u << 29));
  }
  if (mag == 0u) return __hiloint2double((int)u, 0);  // signed zero
  return (double)f;
}

__device__ __forceinline__ float narrow_f64(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned mag = hi & 0x7fffffffu;
  if (mag - (897u << 20) < (254u << 20)) {  // binary64 exponent 897..1150: binary32 exponent 1..254
    // top 23 fraction bits under the rebased exponent; the 29 dropped bits decide the rounding
    unsigned b = ((mag - (896u << 20)) << 3) | (lo >> 29);
    const unsigned r = lo & 0x1fffffffu;
    b += (unsigned)(r > 0x10000000u) | ((unsigned)(r == 0x10000000u) & b);
    return __uint_as_float(b | (hi & 0x80000000u));
  }
  if ((mag | lo) == 0u) return __uint_as_float(hi);  // signed zero
  return (float)d;
}

}  // namespace eqd
