// Small MLP (6 -> 64 -> 64 -> 1) that predicts log10 of the converged rate-and-state slip rate
// from (log V_trial, state, normal traction, trial shear traction, a, b).  The prediction only
// replaces the Newton initial guess; Newton then runs to the reference's own exit test.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "eqd_internal.h"

namespace eqd {

constexpr int kMlpIn = 6;
constexpr int kMlpHidden = 64;

struct MlpDevice {
  // weights in bf16 (what the tensor cores consume), biases and normalisation in fp32
  __nv_bfloat16 W1[kMlpHidden * 16];          // [64][16], input padded from 6 to 16
  __nv_bfloat16 W2[kMlpHidden * kMlpHidden];  // [64][64]
  __nv_bfloat16 W3[16 * kMlpHidden];          // [16][64], row 0 used
  float b1[kMlpHidden], b2[kMlpHidden], b3[16];
  float in_shift[16], in_scale[16];
  float out_shift, out_scale;
  int valid;
};

const void *mlp_device_params(Context &c);

// Scalar evaluation with the same bf16 weights and fp32 accumulation as the tensor-core
// kernels (used per thread inside the fault kernel).
__device__ __forceinline__ double mlp_guess(const MlpDevice &m, const double feat[kMlpIn]) {
  float x[kMlpIn];
#pragma unroll
  for (int i = 0; i < kMlpIn; ++i) {
    float v = (float)feat[i];
    v = (v - m.in_shift[i]) * m.in_scale[i];
    x[i] = __bfloat162float(__float2bfloat16(v));
  }
  float h1[kMlpHidden];
#pragma unroll 8
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = m.b1[j];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) s = fmaf(__bfloat162float(m.W1[j * 16 + i]), x[i], s);
    s = s > 0.f ? s : 0.f;
    h1[j] = __bfloat162float(__float2bfloat16(s));
  }
  float out = m.b3[0];
  for (int j = 0; j < kMlpHidden; ++j) {
    float s = m.b2[j];
#pragma unroll 8
    for (int i = 0; i < kMlpHidden; ++i) s = fmaf(__bfloat162float(m.W2[j * kMlpHidden + i]), h1[i], s);
    s = s > 0.f ? s : 0.f;
    out = fmaf(__bfloat162float(m.W3[j]), __bfloat162float(__float2bfloat16(s)), out);
  }
  const float lg = out * m.out_scale + m.out_shift;  // log10 V
  return exp10((double)lg);
}

}  // namespace eqd
