// Learned initial guess for the rate-and-state Newton solve: a 6 -> 64 -> 64 -> 1 MLP (ReLU) in
// BF16 weights and activations with FP32 accumulation.  This header holds the model block and the
// inference fused into the fault kernel: each warp evaluates its 32 pairs with the warp-level
// tensor-core MMA (mma.sync.m16n8k16, bf16 x bf16 -> f32), so no CTA-wide barrier or tensor memory
// enters the per-pair solve.  Training runs on tcgen05 (kernels_mlp.cu).
//
// Inputs (raw features of one solve): ln V_trial (the slip rate the plain method starts from),
// ln |state|, effective normal traction, trial shear traction, a, b.  Output: ln(V / V_trial) of the
// converged slip rate V, so the guess is V_trial * exp(output).  The guess only replaces the
// starting point; Newton then runs to the reference's own exit test, which still decides
// convergence, and the plain starting point stays the fallback.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "eqd_internal.h"

namespace eqd {

constexpr int kMlpIn = 6;
constexpr int kMlpK1 = 16;   // input padded to one k16 step
constexpr int kMlpH = 64;
constexpr int kMlpN3 = 8;    // output padded to one n8 tile (row 0 used)
// FP32 master parameter vector: W1 [64][16], b1 [64], W2 [64][64], b2 [64], W3 [64], b3
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kMlpH * kMlpK1, kOffW2 = kOffB1 + kMlpH;
constexpr int kOffB2 = kOffW2 + kMlpH * kMlpH, kOffW3 = kOffB2 + kMlpH, kOffB3 = kOffW3 + kMlpH;
constexpr int kMlpParams = kOffB3 + 1;
constexpr int kMlpNorm = 2 * 8 + 2 + 2 * 8;  // in_shift[8], in_scale[8], out_shift, out_scale, in_lo[8], in_hi[8]

struct MlpDevice {
  __nv_bfloat16 W1[kMlpH * kMlpK1];  // [64][16], columns 6-15 zero
  __nv_bfloat16 W2[kMlpH * kMlpH];   // [64][64]
  __nv_bfloat16 W3[kMlpN3 * kMlpH];  // [8][64], rows 1-7 zero
  float b1[kMlpH], b2[kMlpH], b3;
  float in_shift[8], in_scale[8];    // x = (f - shift) * scale
  float out_shift, out_scale;        // ln(V / V_trial) = y * scale + shift
  float in_lo[8], in_hi[8];          // range of each raw feature over the training data
};

const void *mlp_device_params(Context &c);

// ---- tensor-core primitives -------------------------------------------------------------------
// D = A B + D for one 16x8x16 tile; fragments as in the PTX ISA for mma.m16n8k16 with .bf16:
// g = lane / 4, t = lane % 4; A regs: (g, 2t..2t+1), (g+8, 2t..), (g, 2t+8..), (g+8, 2t+8..);
// B regs: (k = 2t..2t+1, n = g), (k = 2t+8.., n = g); D: (g, 2t..2t+1), (g+8, 2t..2t+1).
__device__ __forceinline__ void mma_bf16(float d[4], const unsigned a[4], const unsigned b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<unsigned *>(&v);
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16(x)); }
__device__ __forceinline__ unsigned ld32(const __nv_bfloat16 *p) { return *reinterpret_cast<const unsigned *>(p); }
// A fragment of rows m0.., columns k0.. of a row-major bf16 matrix with leading dimension lda.
__device__ __forceinline__ void frag_a(unsigned a[4], const __nv_bfloat16 *A, int lda, int m0, int k0) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  a[0] = ld32(A + (m0 + g) * lda + k0 + 2 * t);
  a[1] = ld32(A + (m0 + g + 8) * lda + k0 + 2 * t);
  a[2] = ld32(A + (m0 + g) * lda + k0 + 8 + 2 * t);
  a[3] = ld32(A + (m0 + g + 8) * lda + k0 + 8 + 2 * t);
}
// B fragment (k0.., n0..) of B = Bt^T, Bt row-major [N][ldb] (each output column's K values
// contiguous), e.g. a weight matrix W [out][in] for y = x W^T.
__device__ __forceinline__ void frag_bt(unsigned b[2], const __nv_bfloat16 *Bt, int ldb, int n0, int k0) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  b[0] = ld32(Bt + (n0 + g) * ldb + k0 + 2 * t);
  b[1] = ld32(Bt + (n0 + g) * ldb + k0 + 8 + 2 * t);
}
// Two adjacent n8 accumulator tiles (columns 16 kk ..) after ReLU, as the A fragment of k-step kk.
__device__ __forceinline__ void relu_to_a(unsigned a[4], const float lo[4], const float hi[4]) {
  a[0] = pack_bf16(fmaxf(lo[0], 0.f), fmaxf(lo[1], 0.f));
  a[1] = pack_bf16(fmaxf(lo[2], 0.f), fmaxf(lo[3], 0.f));
  a[2] = pack_bf16(fmaxf(hi[0], 0.f), fmaxf(hi[1], 0.f));
  a[3] = pack_bf16(fmaxf(hi[2], 0.f), fmaxf(hi[3], 0.f));
}

// Forward pass of 16 rows (one m16 tile) whose input A fragment is xa: pre-activations z1, z2
// (accumulator layout) and the output (column 0 of `out`: rows g in out[0], g + 8 in out[2], on
// lanes with t == 0).  Weights may live in global or shared memory.
__device__ __forceinline__ void mlp_forward16(const unsigned xa[4], const __nv_bfloat16 *W1, const __nv_bfloat16 *W2,
                                              const __nv_bfloat16 *W3, const float *b1, const float *b2, float b3,
                                              float z1[8][4], float z2[8][4], float out[4]) {
  const int t = threadIdx.x & 3;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float c0 = b1[8 * j + 2 * t], c1 = b1[8 * j + 2 * t + 1];
    z1[j][0] = c0, z1[j][1] = c1, z1[j][2] = c0, z1[j][3] = c1;
    unsigned b[2];
    frag_bt(b, W1, kMlpK1, 8 * j, 0);
    mma_bf16(z1[j], xa, b);
  }
  unsigned h1[4][4];
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) relu_to_a(h1[kk], z1[2 * kk], z1[2 * kk + 1]);
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float c0 = b2[8 * j + 2 * t], c1 = b2[8 * j + 2 * t + 1];
    z2[j][0] = c0, z2[j][1] = c1, z2[j][2] = c0, z2[j][3] = c1;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      unsigned b[2];
      frag_bt(b, W2, kMlpH, 8 * j, 16 * kk);
      mma_bf16(z2[j], h1[kk], b);
    }
  }
  out[0] = out[1] = out[2] = out[3] = b3;
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    unsigned a[4], b[2];
    relu_to_a(a, z2[2 * kk], z2[2 * kk + 1]);
    frag_bt(b, W3, kMlpH, 0, 16 * kk);
    mma_bf16(out, a, b);
  }
}

// Raw features of one solve.
__device__ __forceinline__ void mlp_features(double v0, double state0, double tn, double trial, double a,
                                             double b, float f[kMlpIn]) {
  f[0] = (float)log(fmax(v0, 1e-30));
  f[1] = (float)log(fmax(fabs(state0), 1e-30));
  f[2] = (float)tn;
  f[3] = (float)trial;
  f[4] = (float)a;
  f[5] = (float)b;
}

// Scalar evaluation with the same bf16 weights and activations (used by lanes of a warp that is
// not complete, where the warp-wide tensor-core path cannot run).
__device__ __forceinline__ float mlp_eval_scalar(const MlpDevice &m, const float f[kMlpIn]) {
  float x[kMlpIn];
#pragma unroll
  for (int i = 0; i < kMlpIn; ++i) x[i] = bf16r((f[i] - m.in_shift[i]) * m.in_scale[i]);
  float h1[kMlpH];
#pragma unroll 8
  for (int j = 0; j < kMlpH; ++j) {
    float s = m.b1[j];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) s = fmaf(__bfloat162float(m.W1[j * kMlpK1 + i]), x[i], s);
    h1[j] = bf16r(fmaxf(s, 0.f));
  }
  float out = m.b3;
  for (int j = 0; j < kMlpH; ++j) {
    float s = m.b2[j];
#pragma unroll 8
    for (int i = 0; i < kMlpH; ++i) s = fmaf(__bfloat162float(m.W2[j * kMlpH + i]), h1[i], s);
    out = fmaf(__bfloat162float(m.W3[j]), bf16r(fmaxf(s, 0.f)), out);
  }
  return out;
}

// Learned guess for each lane's solve.  `full` must be the same on all lanes of the warp and true
// only when all 32 lanes are here; xs: 32 x 16 bf16 of shared scratch owned by this warp.  Returns
// V_trial * exp(prediction); V_trial itself (the plain guess) when that is not a positive finite
// number, or when a feature of the solve lies outside its range over the training data (the model
// would extrapolate).
__device__ __forceinline__ double mlp_guess_warp(const MlpDevice &m, const float f[kMlpIn], double v0, bool full,
                                                 __nv_bfloat16 *xs) {
  float y;
  if (full) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    unsigned row[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) row[i] = 0u;
    row[0] = pack_bf16((f[0] - m.in_shift[0]) * m.in_scale[0], (f[1] - m.in_shift[1]) * m.in_scale[1]);
    row[1] = pack_bf16((f[2] - m.in_shift[2]) * m.in_scale[2], (f[3] - m.in_shift[3]) * m.in_scale[3]);
    row[2] = pack_bf16((f[4] - m.in_shift[4]) * m.in_scale[4], (f[5] - m.in_shift[5]) * m.in_scale[5]);
    uint4 *dst = reinterpret_cast<uint4 *>(xs + lane * kMlpK1);
    dst[0] = make_uint4(row[0], row[1], row[2], row[3]);
    dst[1] = make_uint4(row[4], row[5], row[6], row[7]);
    __syncwarp();
    float out[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      unsigned xa[4];
      frag_a(xa, xs, kMlpK1, 16 * mt, 0);
      float z1[8][4], z2[8][4];
      mlp_forward16(xa, m.W1, m.W2, m.W3, m.b1, m.b2, m.b3, z1, z2, out[mt]);
    }
    // row r of tile r / 16 sits on lane ((r % 16) % 8) * 4, in out[0] (r % 16 < 8) or out[2]
    const int src = (lane & 7) * 4;
    const float o00 = __shfl_sync(0xffffffffu, out[0][0], src), o02 = __shfl_sync(0xffffffffu, out[0][2], src);
    const float o10 = __shfl_sync(0xffffffffu, out[1][0], src), o12 = __shfl_sync(0xffffffffu, out[1][2], src);
    const int r = lane & 15;
    y = lane < 16 ? (r < 8 ? o00 : o02) : (r < 8 ? o10 : o12);
    __syncwarp();
  } else {
    y = mlp_eval_scalar(m, f);
  }
  bool inside = true;
#pragma unroll
  for (int i = 0; i < kMlpIn; ++i) inside = inside && f[i] >= m.in_lo[i] && f[i] <= m.in_hi[i];
  const double g = fmax(v0, 1e-30) * exp((double)(y * m.out_scale + m.out_shift));
  return (inside && g > 0.0 && isfinite(g)) ? g : v0;
}

}  // namespace eqd
