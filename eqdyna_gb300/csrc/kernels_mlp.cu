// Learned Newton initial guess: logged solves -> features, tensor-core training (forward,
// backward, Adam), replay of logged solves, and the model's device parameter block.
//
// Training data are the rate-and-state Newton solves the plain method itself performs
// (eqd_gpu_newton_log).  Training runs its products on the 5th-generation tensor cores
// (tcgen05.mma with accumulators in tensor memory, tcgen05.cuh), 128 samples per CTA; inference
// inside the fault and replay kernels is warp-cooperative (mma.sync.m16n8k16, mlp_common.cuh).
// Both use bf16 operands and fp32 accumulation; biases, losses, Adam and the rank-1 output layer
// are fp32 on the CUDA cores.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "eqd_device.cuh"
#include "mlp_common.cuh"
#include "rsf_newton.cuh"
#include "tcgen05.cuh"

namespace eqd {

namespace {

constexpr int kTrainRows = 128;  // samples per CTA = threads = the M of every tensor-core product

// ---- records -> raw features ---------------------------------------------------------------------
// raw[r][0..5] features, [6] target ln(V / V_trial), [7] 1 if finite
__global__ void record_features_kernel(const double *__restrict__ rec, long long n, float *__restrict__ raw) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const double *q = rec + r * kNewtonRecord;
  float f[kMlpIn];
  mlp_features(q[13], q[7], q[9], q[10], q[0], q[1], f);
  const double tgt = log(fmax(q[14], 1e-30)) - log(fmax(q[13], 1e-30));
  bool ok = isfinite(tgt) && q[14] > 0.0;
  for (int k = 0; k < kMlpIn; ++k) {
    raw[r * 8 + k] = f[k];
    ok = ok && isfinite(f[k]);
  }
  raw[r * 8 + 6] = (float)tgt;
  raw[r * 8 + 7] = ok ? 1.f : 0.f;
}

// normalised inputs (bf16, padded to 16) and targets
__global__ void normalise_kernel(const float *__restrict__ raw, long long n, const float *__restrict__ norm,
                                 __nv_bfloat16 *__restrict__ X, float *__restrict__ Y) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int k = 0; k < kMlpK1; ++k)
    X[r * kMlpK1 + k] = __float2bfloat16(k < kMlpIn ? (raw[r * 8 + k] - norm[k]) * norm[8 + k] : 0.f);
  Y[r] = (raw[r * 8 + 6] - norm[16]) / norm[17];
}

// FP32 master parameters -> the bf16 / fp32 block the kernels read
__device__ __forceinline__ void write_param(MlpDevice *m, int i, float v) {
  if (i < kOffB1) m->W1[i] = __float2bfloat16(v);
  else if (i < kOffW2) m->b1[i - kOffB1] = v;
  else if (i < kOffB2) m->W2[i - kOffW2] = __float2bfloat16(v);
  else if (i < kOffW3) m->b2[i - kOffB2] = v;
  else if (i < kOffB3) m->W3[i - kOffW3] = __float2bfloat16(v);
  else m->b3 = v;
}

static_assert(kMlpNorm == EQD_MLP_NORM, "normalisation block of the C ABI");

__global__ void mlp_sync_kernel(const float *__restrict__ P, MlpDevice *m, const float *__restrict__ norm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kMlpParams) write_param(m, i, P[i]);
  if (i < (kMlpN3 - 1) * kMlpH) m->W3[kMlpH + i] = __float2bfloat16(0.f);
  if (norm && i < 8) {
    m->in_shift[i] = norm[i];
    m->in_scale[i] = norm[8 + i];
  }
  if (norm && i == 0) {
    m->out_shift = norm[16];
    m->out_scale = norm[17];
  }
  if (norm && i < 8) {
    m->in_lo[i] = norm[18 + i];
    m->in_hi[i] = norm[26 + i];
  }
}

// Adam step on the FP32 masters (gradients are zeroed for the next step), then the device block.
__global__ void mlp_adam_kernel(float *__restrict__ P, float *__restrict__ G, float *__restrict__ M,
                                float *__restrict__ V, MlpDevice *m, float lr_t, float beta1, float beta2,
                                float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kMlpParams) return;
  const float g = G[i];
  G[i] = 0.f;
  const float mi = beta1 * M[i] + (1.f - beta1) * g;
  const float vi = beta2 * V[i] + (1.f - beta2) * g * g;
  M[i] = mi;
  V[i] = vi;
  const float p = P[i] - lr_t * mi / (sqrtf(vi) + eps);
  P[i] = p;
  write_param(m, i, p);
}

struct TrainBatch {
  const __nv_bfloat16 *X;  // [n][16]
  const float *Y;          // [n]
  const int *order;        // sample ids, or null for 0..n-1
  long long start, count;  // this batch: order[start .. start + count)
  float inv_count;         // 1 / samples in the batch
};

// Shared memory of the training kernel: the tensor-core operands (bf16, tc::kmaj_off layout), then
// the fp32 bias / output-weight rows, the mbarrier and the tensor-memory address.
struct GradSmem {
  static constexpr int W1 = 0;                                   // B of Z1: [64 n1][16 k]
  static constexpr int W2 = W1 + kMlpH * kMlpK1 * 2;             // B of Z2: [64 n2][64 k1]
  static constexpr int W2T = W2 + kMlpH * kMlpH * 2;             // B of dH1: [64 k1][64 n2]
  static constexpr int X = W2T + kMlpH * kMlpH * 2;              // A of Z1: [128 s][16 k]
  static constexpr int AT = X + kTrainRows * kMlpK1 * 2;         // A of dW: [64 n2 | 64 n1][128 s]
  static constexpr int H1 = AT + 2 * kMlpH * kTrainRows * 2;     // A of Z2: [128 s][64 k1]
  static constexpr int DZ2 = H1 + kTrainRows * kMlpH * 2;        // A of dH1: [128 s][64 n2]
  static constexpr int BT = DZ2 + kTrainRows * kMlpH * 2;        // B of dW: [64 k1 | 16 k][128 s]
  static constexpr int VEC = BT + (kMlpH + kMlpK1) * kTrainRows * 2;  // b1[64], b2[64], w3[64] fp32
  static constexpr int BAR = VEC + 3 * kMlpH * 4;
  static constexpr int TMEM = BAR + 8;
  static constexpr int BYTES = TMEM + 8;
};
// 2 CTAs per SM at most (3 x 108 KB exceed the SM's shared memory), so the 2 x kGradCols columns
// they allocate never exceed the SM's 512 and the allocation never waits.
constexpr uint32_t kGradCols = 256;
static_assert(GradSmem::BYTES > 228 * 1024 / 3, "the shared memory must keep a third CTA off the SM");
static_assert(2 * kGradCols <= 512, "tensor memory of two CTAs");

// Forward + backward of one batch, kTrainRows = 128 samples per CTA (thread i owns sample i, which is
// row / tensor-memory lane i of every product): loss += sum (y - t)^2 / (2 count), G += d loss /
// d params.  The four products run on the 5th-generation tensor cores (tcgen05.mma, kind::f16, bf16
// operands from shared memory, fp32 accumulators in tensor memory), issued by thread 0:
//   Z1 = X W1^T (cols 0-63), Z2 = H1 W2^T (cols 64-127), dH1 = dZ2 W2 (cols 128-191),
//   [dW2 | . ; . | dW1] = [dZ2^T ; dZ1^T] [H1 | X] over the CTA's samples (cols 0-79, M 128, N 80).
// Biases, ReLU, the rank-1 output layer and its error are fp32 on the CUDA cores; the bias and
// output-weight gradients are column sums over the CTA's rows; all gradients reach G by fp32
// atomics.  Every wait is bounded: on a timeout bit 2 of *err is set and the CTA frees its tensor
// memory and returns.
__global__ void __launch_bounds__(kTrainRows, 1) mlp_grad_kernel(const MlpDevice *__restrict__ m, TrainBatch tb,
                                                                 float *__restrict__ G, float *__restrict__ loss,
                                                                 int *__restrict__ err) {
  using S = GradSmem;
  extern __shared__ __align__(128) unsigned char smem[];
  float *sb1 = reinterpret_cast<float *>(smem + S::VEC), *sb2 = sb1 + kMlpH, *sw3 = sb2 + kMlpH;
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem + S::BAR);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + S::TMEM);
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  auto st16 = [&](int off, const uint4 &v) { *reinterpret_cast<uint4 *>(smem + off) = v; };
  auto st2 = [&](int off, __nv_bfloat16 v) { *reinterpret_cast<__nv_bfloat16 *>(smem + off) = v; };

  if (w == 0) tc::tmem_alloc(tslot, kGradCols);
  if (tid == 0) e32::mbar_init(bar, 1);
  // weights (16-byte rows of 8 bf16), the transposed W2, biases and the output row
  {
    const uint4 *w1 = reinterpret_cast<const uint4 *>(m->W1);  // [64][16] = 2 chunks per row
    st16(S::W1 + tc::kmaj_off(tid >> 1, 8 * (tid & 1), kMlpK1), w1[tid]);
    const uint4 *w2 = reinterpret_cast<const uint4 *>(m->W2);  // [64][64] = 8 chunks per row
    for (int q = tid; q < kMlpH * 8; q += kTrainRows) st16(S::W2 + tc::kmaj_off(q >> 3, 8 * (q & 7), kMlpH), w2[q]);
    for (int q = tid; q < kMlpH * kMlpH; q += kTrainRows) {
      const int n2 = q >> 6, k1 = q & 63;
      st2(S::W2T + tc::kmaj_off(k1, n2, kMlpH), m->W2[q]);
    }
    if (tid < kMlpH) {
      sb1[tid] = m->b1[tid];
      sb2[tid] = m->b2[tid];
      sw3[tid] = __bfloat162float(m->W3[tid]);
    }
  }
  // this thread's sample: X row (zero past the batch) into X and, transposed, rows 64-79 of BT
  const long long q = tb.start + (long long)blockIdx.x * kTrainRows + tid;
  const bool valid = q < tb.start + tb.count;
  const long long sid = valid ? (tb.order ? (long long)tb.order[q] : q) : -1;
  {
    uint4 x0 = make_uint4(0u, 0u, 0u, 0u), x1 = x0;
    if (valid) {
      const uint4 *xr = reinterpret_cast<const uint4 *>(tb.X + sid * kMlpK1);
      x0 = xr[0];
      x1 = xr[1];
    }
    st16(S::X + tc::kmaj_off(tid, 0, kMlpK1), x0);
    st16(S::X + tc::kmaj_off(tid, 8, kMlpK1), x1);
    const __nv_bfloat16 *e0 = reinterpret_cast<const __nv_bfloat16 *>(&x0);
    const __nv_bfloat16 *e1 = reinterpret_cast<const __nv_bfloat16 *>(&x1);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      st2(S::BT + tc::kmaj_off(kMlpH + k, tid, kTrainRows), e0[k]);
      st2(S::BT + tc::kmaj_off(kMlpH + 8 + k, tid, kTrainRows), e1[k]);
    }
  }
  const float target = valid ? tb.Y[sid] : 0.f;
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t trow = tmem + ((uint32_t)(32 * w) << 16);  // this warp's lanes
  const uint32_t id64 = tc::idesc_bf16_f32(128, 64), id80 = tc::idesc_bf16_f32(128, 80);
  unsigned phase = 0;
  bool ok = true;
  // issue, commit, and wait for one group of MMAs; false (on every thread) after a timeout
  auto run = [&](auto issue) -> bool {
    if (tid == 0) {
      issue();
      tc::commit(bar);
    }
    bool done = tc::mbar_wait_parity(bar, phase);
    if (!done) {
      atomicOr(err, 2);
      done = tc::mbar_wait_parity(bar, phase);  // let the MMAs end before the memory is freed
    }
    phase ^= 1u;
    tc::fence_after_sync();
    return __syncthreads_and(done) != 0;
  };

  // ---- Z1 = X W1^T -----------------------------------------------------------------------------
  ok = run([&] { tc::mma_bf16(tmem + 0, tc::kmaj_desc(smem + S::X, kMlpK1, 0), tc::kmaj_desc(smem + S::W1, kMlpK1, 0), id64, false); });
  if (ok) {
    // H1 = bf16(relu(Z1 + b1)) as the A rows of Z2 and, transposed, rows 0-63 of BT
#pragma unroll
    for (int c = 0; c < kMlpH / 16; ++c) {
      float z[16];
      tc::tmem_ld16(trow + 16 * c, z);
      __align__(16) __nv_bfloat16 h[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) h[i] = __float2bfloat16(fmaxf(z[i] + sb1[16 * c + i], 0.f));
      st16(S::H1 + tc::kmaj_off(tid, 16 * c, kMlpH), *reinterpret_cast<const uint4 *>(h));
      st16(S::H1 + tc::kmaj_off(tid, 16 * c + 8, kMlpH), *reinterpret_cast<const uint4 *>(h + 8));
#pragma unroll
      for (int i = 0; i < 16; ++i) st2(S::BT + tc::kmaj_off(16 * c + i, tid, kTrainRows), h[i]);
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- Z2 = H1 W2^T ----------------------------------------------------------------------------
    ok = run([&] {
      for (int kk = 0; kk < kMlpH / 16; ++kk)
        tc::mma_bf16(tmem + 64, tc::kmaj_desc(smem + S::H1, kMlpH, kk), tc::kmaj_desc(smem + S::W2, kMlpH, kk), id64,
                     kk > 0);
    });
  }
  if (ok) {
    // output y = relu(Z2 + b2) . w3 + b3 (bf16 activations), its error, dZ2 = (z2 > 0) dy w3; Z2 is
    // read from tensor memory twice rather than held in registers
    float y = m->b3;
#pragma unroll
    for (int c = 0; c < kMlpH / 16; ++c) {
      float z[16];
      tc::tmem_ld16(trow + 64 + 16 * c, z);
#pragma unroll
      for (int i = 0; i < 16; ++i) y = fmaf(sw3[16 * c + i], bf16r(fmaxf(z[i] + sb2[16 * c + i], 0.f)), y);
    }
    const float d = valid ? y - target : 0.f;
    const float dy = d * tb.inv_count;
    float lsum = d * d * 0.5f * tb.inv_count, db3 = dy;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
      db3 += __shfl_xor_sync(0xffffffffu, db3, o);
    }
    if (lane == 0) {
      atomicAdd(loss, lsum);
      atomicAdd(G + kOffB3, db3);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {  // 32 columns at a time
      float gw3[32], gb2[32];
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        float z[16];
        tc::tmem_ld16(trow + 64 + 32 * h + 16 * c, z);
        __align__(16) __nv_bfloat16 e[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int j = 32 * h + 16 * c + i;
          const float z2 = z[i] + sb2[j];
          const float dz = z2 > 0.f ? dy * sw3[j] : 0.f;
          gw3[16 * c + i] = dy * bf16r(fmaxf(z2, 0.f));
          gb2[16 * c + i] = dz;
          e[i] = __float2bfloat16(dz);
          st2(S::AT + tc::kmaj_off(j, tid, kTrainRows), e[i]);
        }
        st16(S::DZ2 + tc::kmaj_off(tid, 32 * h + 16 * c, kMlpH), *reinterpret_cast<const uint4 *>(e));
        st16(S::DZ2 + tc::kmaj_off(tid, 32 * h + 16 * c + 8, kMlpH), *reinterpret_cast<const uint4 *>(e + 8));
      }
      const float a = tc::warp_column_sums32(gw3), b = tc::warp_column_sums32(gb2);
      atomicAdd(G + kOffW3 + 32 * h + lane, a);
      atomicAdd(G + kOffB2 + 32 * h + lane, b);
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- dH1 = dZ2 W2 ----------------------------------------------------------------------------
    ok = run([&] {
      for (int kk = 0; kk < kMlpH / 16; ++kk)
        tc::mma_bf16(tmem + 128, tc::kmaj_desc(smem + S::DZ2, kMlpH, kk), tc::kmaj_desc(smem + S::W2T, kMlpH, kk),
                     id64, kk > 0);
    });
  }
  if (ok) {
    // dZ1 = (z1 > 0) dH1: rows 64-127 of AT (transposed) and the b1 column sums
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float gb1[32];
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        float z1[16], dh[16];
        tc::tmem_ld16(trow + 32 * h + 16 * c, z1);
        tc::tmem_ld16(trow + 128 + 32 * h + 16 * c, dh);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int j = 32 * h + 16 * c + i;
          const float dz = (z1[i] + sb1[j]) > 0.f ? dh[i] : 0.f;
          gb1[16 * c + i] = dz;
          st2(S::AT + tc::kmaj_off(kMlpH + j, tid, kTrainRows), __float2bfloat16(dz));
        }
      }
      atomicAdd(G + kOffB1 + 32 * h + lane, tc::warp_column_sums32(gb1));
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- [dW2 ; dW1] = [dZ2^T ; dZ1^T] [H1 | X] ----------------------------------------------------
    ok = run([&] {
      for (int kk = 0; kk < kTrainRows / 16; ++kk)
        tc::mma_bf16(tmem + 0, tc::kmaj_desc(smem + S::AT, kTrainRows, kk), tc::kmaj_desc(smem + S::BT, kTrainRows, kk),
                     id80, kk > 0);
    });
  }
  if (ok) {
    if (w < 2) {  // rows 0-63: dW2 [n2 = tid][k1]
#pragma unroll
      for (int c = 0; c < kMlpH / 16; ++c) {
        float g[16];
        tc::tmem_ld16(trow + 16 * c, g);
#pragma unroll
        for (int i = 0; i < 16; ++i) atomicAdd(G + kOffW2 + tid * kMlpH + 16 * c + i, g[i]);
      }
    } else {  // rows 64-127: dW1 [n1 = tid - 64][k], columns 64-79
      float g[16];
      tc::tmem_ld16(trow + kMlpH, g);
#pragma unroll
      for (int k = 0; k < kMlpIn; ++k) atomicAdd(G + kOffW1 + (tid - kMlpH) * kMlpK1 + k, g[k]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(tmem, kGradCols);
}

constexpr size_t kGradSmem = GradSmem::BYTES;

// Replays logged solves from the plain guess or the learned one; ghost lanes past n re-solve the
// last record so every warp is complete for the tensor-core guess, and write nothing.
template <bool FAST>
__global__ void __launch_bounds__(128) newton_replay_kernel(const double *__restrict__ rec, long long n,
                                                            int friclaw, double dt, const MlpDevice *m,
                                                            double *__restrict__ v_out,
                                                            double *__restrict__ step_out,
                                                            int *__restrict__ flag_out,
                                                            unsigned long long *__restrict__ counts) {
  __shared__ __align__(16) __nv_bfloat16 xs[4][32 * kMlpK1];
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const bool live = i < n;
  const double *q = rec + (live ? i : n - 1) * kNewtonRecord;
  NewtonSolve s;
  s.r = RsfParams{q[0], q[1], q[2], q[3], q[4], q[5], q[6]};
  s.state0 = q[7];
  s.th0 = q[8];
  s.tn = q[9];
  s.trial = q[10];
  s.Tc = q[11];
  s.c0 = q[12];
  double v0 = q[13];
  if (m) {
    float f[kMlpIn];
    mlp_features(q[13], q[7], q[9], q[10], q[0], q[1], f);
    v0 = mlp_guess_warp(*m, f, q[13], true, xs[threadIdx.x >> 5]);
  }
  NewtonOut o = rsf_newton<FAST>(friclaw, dt, s, v0);
  unsigned fallback = 0;
  if (m && !newton_settled(o)) {  // as the fault kernel: repeat from the plain guess
    const NewtonOut first = o;
    o = rsf_newton<FAST>(friclaw, dt, s, q[13]);
    o.iters += first.iters;
    o.executed += first.executed;
    fallback = 1;
  }
  if (live) {
    if (v_out) v_out[i] = o.v;
    if (step_out) step_out[i] = o.step;
    if (flag_out) flag_out[i] = o.iters | o.capped << 8 | (int)fallback << 9 | o.exit_kind << 10;
    warp_count_add(counts + 0, (unsigned)o.iters);
    warp_count_add(counts + 1, (unsigned)o.capped);
    warp_count_add(counts + 2, (unsigned)o.executed);
    warp_count_add(counts + 3, fallback);
  }
}

// He-normal initial weights (seeded), zero biases.
std::vector<float> init_params(unsigned long long seed) {
  std::vector<float> p(kMlpParams, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  const float s1 = std::sqrt(2.f / kMlpIn), s2 = std::sqrt(2.f / kMlpH), s3 = std::sqrt(1.f / kMlpH);
  for (int n = 0; n < kMlpH; ++n)
    for (int k = 0; k < kMlpIn; ++k) p[kOffW1 + n * kMlpK1 + k] = s1 * nd(rng);
  for (int k = 0; k < kMlpH * kMlpH; ++k) p[kOffW2 + k] = s2 * nd(rng);
  for (int k = 0; k < kMlpH; ++k) p[kOffW3 + k] = s3 * nd(rng);
  return p;
}

int dmalloc(void **p, size_t bytes) { return cudaMalloc(p, bytes) == cudaSuccess ? EQD_OK : EQD_ERR_OOM; }

#define MRC(x)               \
  do {                       \
    const int r_ = (x);      \
    if (r_) return r_;       \
  } while (0)

}  // namespace

const void *mlp_device_params(Context &c) { return c.mlp_on ? c.mlp : nullptr; }

int mlp_init(Context &c) {
  if (c.mlp) return EQD_OK;
  MRC(dmalloc(&c.mlp, sizeof(MlpDevice)));
  EQD_CUDA_OK(cudaMemset(c.mlp, 0, sizeof(MlpDevice)));
  MRC(dmalloc(reinterpret_cast<void **>(&c.mlp_p), 4 * sizeof(float) * kMlpParams));
  c.mlp_g = c.mlp_p + kMlpParams;
  c.mlp_m = c.mlp_g + kMlpParams;
  c.mlp_v = c.mlp_m + kMlpParams;
  EQD_CUDA_OK(cudaMemset(c.mlp_p, 0, 4 * sizeof(float) * kMlpParams));
  return EQD_OK;
}

void mlp_free(Context &c) {
  if (c.mlp) cudaFree(c.mlp);
  if (c.mlp_p) cudaFree(c.mlp_p);
  if (c.nlog) cudaFree(c.nlog);
  c.mlp = nullptr;
  c.mlp_p = c.mlp_g = c.mlp_m = c.mlp_v = nullptr;
  c.nlog = nullptr;
  c.mlp_on = 0;
}

int newton_log_start(Context &c, int nsteps, int stride) {
  if (nsteps < 0 || stride < 1) return EQD_ERR_INPUT;
  if (c.sc.friclaw < 3 || c.sc.friclaw > 4 || c.npair == 0) return EQD_ERR_UNSUPPORTED;
  if (c.nlog) cudaFree(c.nlog);
  c.nlog = nullptr;
  c.nlog_steps = 0;
  if (nsteps == 0) return EQD_OK;
  MRC(dmalloc(reinterpret_cast<void **>(&c.nlog), sizeof(double) * kNewtonRecord * (size_t)nsteps * c.npair));
  c.nlog_nt0 = c.nt;
  c.nlog_steps = nsteps;
  c.nlog_stride = stride;
  return EQD_OK;
}

long long newton_log_count(const Context &c) {
  if (!c.nlog) return 0;
  const int done = std::min(c.nlog_steps, (c.nt - c.nlog_nt0) / c.nlog_stride);
  return (long long)std::max(done, 0) * c.npair;
}

int newton_records(Context &c, double *host, long long cap, long long *count) {
  const long long n = newton_log_count(c);
  if (count) *count = n;
  if (host && n > 0) EQD_CUDA_OK(cudaMemcpy(host, c.nlog, sizeof(double) * kNewtonRecord * std::min(n, cap),
                                            cudaMemcpyDeviceToHost));
  return EQD_OK;
}

int mlp_set(Context &c, const float *params, const float *norm) {
  MRC(mlp_init(c));
  EQD_CUDA_OK(cudaMemcpy(c.mlp_p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
  EQD_CUDA_OK(cudaMemset(c.mlp_g, 0, 3 * sizeof(float) * kMlpParams));
  std::memcpy(c.mlp_norm, norm, sizeof(float) * kMlpNorm);
  float *dn = nullptr;
  MRC(dmalloc(reinterpret_cast<void **>(&dn), sizeof(float) * kMlpNorm));
  cudaMemcpy(dn, norm, sizeof(float) * kMlpNorm, cudaMemcpyHostToDevice);
  mlp_sync_kernel<<<(kMlpParams + 255) / 256, 256>>>(c.mlp_p, static_cast<MlpDevice *>(c.mlp), dn);
  const cudaError_t e = cudaDeviceSynchronize();
  cudaFree(dn);
  c.mlp_steps = 0;
  return e == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

int mlp_get(Context &c, float *params, float *norm) {
  if (!c.mlp_p) return EQD_ERR_STATE;
  if (params) EQD_CUDA_OK(cudaMemcpy(params, c.mlp_p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
  if (norm) std::memcpy(norm, c.mlp_norm, sizeof(float) * kMlpNorm);
  return EQD_OK;
}

// Trains the guess on the logged solves: normalisation from the data, a seeded shuffle with a
// held-out tail, mini-batch Adam.  epoch_loss[e] (mean training loss of epoch e) and the
// held-out loss are optional outputs.
int mlp_train(Context &c, const eqd_mlp_train_options &o, float *epoch_loss, float *holdout_loss) {
  const long long n = newton_log_count(c);
  if (n <= 0) return EQD_ERR_STATE;
  if (o.epochs < 0 || o.batch < kTrainRows || o.holdout < 0.f || o.holdout >= 1.f) return EQD_ERR_INPUT;
  MRC(mlp_init(c));
  float *raw = nullptr, *Y = nullptr, *dnorm = nullptr, *dloss = nullptr;
  __nv_bfloat16 *X = nullptr;
  int *order = nullptr;
  int rc = EQD_OK;
  std::vector<float> hraw(8 * (size_t)n);
  std::vector<int> valid;
  float norm[kMlpNorm];
  long long ntrain = 0, nhold = 0;
  const int bs = (o.batch + kTrainRows - 1) / kTrainRows * kTrainRows;
  do {
    if ((rc = dmalloc(reinterpret_cast<void **>(&raw), sizeof(float) * 8 * n))) break;
    record_features_kernel<<<(unsigned)((n + 255) / 256), 256>>>(c.nlog, n, raw);
    if (cudaMemcpy(hraw.data(), raw, sizeof(float) * 8 * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = EQD_ERR_CUDA;
      break;
    }
    // normalisation over the valid records
    double sum[7] = {0}, sq[7] = {0};
    for (long long r = 0; r < n; ++r) {
      if (hraw[r * 8 + 7] == 0.f) continue;
      valid.push_back((int)r);
      for (int k = 0; k < 7; ++k) sum[k] += hraw[r * 8 + k], sq[k] += (double)hraw[r * 8 + k] * hraw[r * 8 + k];
    }
    if (valid.size() < (size_t)kTrainRows) {
      rc = EQD_ERR_STATE;
      break;
    }
    const double nv = (double)valid.size();
    for (int k = 0; k < 8; ++k) norm[k] = 0.f, norm[8 + k] = 0.f;
    // range of each raw feature over the training records: the guess is used inside it only
    for (int k = 0; k < 8; ++k) norm[18 + k] = 0.f, norm[26 + k] = 0.f;
    for (int k = 0; k < kMlpIn; ++k) {
      float lo = hraw[(size_t)valid[0] * 8 + k], hi = lo;
      for (const int r : valid) {
        lo = std::min(lo, hraw[(size_t)r * 8 + k]);
        hi = std::max(hi, hraw[(size_t)r * 8 + k]);
      }
      norm[18 + k] = lo;
      norm[26 + k] = hi;
    }
    for (int k = 0; k < 7; ++k) {
      const double mean = sum[k] / nv, var = std::max(sq[k] / nv - mean * mean, 0.0), sd = std::sqrt(var);
      const bool flat = sd <= 1e-7 * std::max(std::fabs(mean), 1e-30);
      if (k < kMlpIn) {
        norm[k] = (float)mean;
        norm[8 + k] = flat ? 0.f : (float)(1.0 / sd);
      } else {
        norm[16] = (float)mean;
        norm[17] = flat ? 1.f : (float)sd;
      }
    }
    std::memcpy(c.mlp_norm, norm, sizeof(norm));
    if ((rc = dmalloc(reinterpret_cast<void **>(&dnorm), sizeof(norm)))) break;
    cudaMemcpy(dnorm, norm, sizeof(norm), cudaMemcpyHostToDevice);
    if ((rc = dmalloc(reinterpret_cast<void **>(&X), sizeof(__nv_bfloat16) * kMlpK1 * n))) break;
    if ((rc = dmalloc(reinterpret_cast<void **>(&Y), sizeof(float) * n))) break;
    normalise_kernel<<<(unsigned)((n + 255) / 256), 256>>>(raw, n, dnorm, X, Y);
    // seeded shuffle, held-out tail
    std::mt19937_64 rng(o.seed);
    std::shuffle(valid.begin(), valid.end(), rng);
    nhold = (long long)(o.holdout * valid.size());
    ntrain = (long long)valid.size() - nhold;
    if ((rc = dmalloc(reinterpret_cast<void **>(&order), sizeof(int) * valid.size()))) break;
    // dloss[0] the loss sum, dloss[1] (as int) the kernels' error word
    if ((rc = dmalloc(reinterpret_cast<void **>(&dloss), 2 * sizeof(float)))) break;
    cudaMemset(dloss, 0, 2 * sizeof(float));
    int *derr = reinterpret_cast<int *>(dloss + 1);
    // parameters
    const std::vector<float> p0 = init_params(o.seed);
    cudaMemcpy(c.mlp_p, p0.data(), sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
    cudaMemset(c.mlp_g, 0, 3 * sizeof(float) * kMlpParams);
    mlp_sync_kernel<<<(kMlpParams + 255) / 256, 256>>>(c.mlp_p, static_cast<MlpDevice *>(c.mlp), dnorm);
    if (cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem) !=
        cudaSuccess) {
      rc = EQD_ERR_CUDA;
      break;
    }
    const float beta1 = 0.9f, beta2 = 0.999f;
    c.mlp_steps = 0;
    for (int ep = 0; ep < o.epochs && !rc; ++ep) {
      std::shuffle(valid.begin(), valid.begin() + ntrain, rng);
      cudaMemcpy(order, valid.data(), sizeof(int) * valid.size(), cudaMemcpyHostToDevice);
      cudaMemset(dloss, 0, sizeof(float));
      long long nb = 0;
      for (long long b0 = 0; b0 < ntrain; b0 += bs, ++nb) {
        TrainBatch tb{X, Y, order, b0, std::min<long long>(bs, ntrain - b0), 0.f};
        tb.inv_count = 1.f / (float)tb.count;
        const unsigned grid = (unsigned)((tb.count + kTrainRows - 1) / kTrainRows);
        mlp_grad_kernel<<<grid, kTrainRows, kGradSmem>>>(static_cast<MlpDevice *>(c.mlp), tb, c.mlp_g, dloss, derr);
        ++c.mlp_steps;
        const double t = (double)c.mlp_steps;
        const float lr_t = (float)(o.lr * std::sqrt(1.0 - std::pow(beta2, t)) / (1.0 - std::pow(beta1, t)));
        mlp_adam_kernel<<<(kMlpParams + 255) / 256, 256>>>(c.mlp_p, c.mlp_g, c.mlp_m, c.mlp_v,
                                                             static_cast<MlpDevice *>(c.mlp), lr_t, beta1, beta2,
                                                             1e-8f);
      }
      float l = 0.f;
      if (cudaMemcpy(&l, dloss, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) rc = EQD_ERR_CUDA;
      if (epoch_loss) epoch_loss[ep] = nb > 0 ? l / (float)nb : 0.f;
    }
    if (rc) break;
    if (holdout_loss) {
      *holdout_loss = 0.f;
      if (nhold > 0) {
        float *gscratch = nullptr;
        if ((rc = dmalloc(reinterpret_cast<void **>(&gscratch), sizeof(float) * kMlpParams))) break;
        cudaMemset(gscratch, 0, sizeof(float) * kMlpParams);
        cudaMemset(dloss, 0, sizeof(float));
        TrainBatch tb{X, Y, order, ntrain, nhold, 1.f / (float)nhold};
        mlp_grad_kernel<<<(unsigned)((nhold + kTrainRows - 1) / kTrainRows), kTrainRows, kGradSmem>>>(
            static_cast<MlpDevice *>(c.mlp), tb, gscratch, dloss, derr);
        if (cudaMemcpy(holdout_loss, dloss, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) rc = EQD_ERR_CUDA;
        cudaFree(gscratch);
      }
    }
    if (cudaDeviceSynchronize() != cudaSuccess) rc = EQD_ERR_CUDA;
    int herr = 0;
    if (!rc && cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) rc = EQD_ERR_CUDA;
    if (!rc && herr) rc = EQD_ERR_TIMEOUT;
  } while (false);
  if (raw) cudaFree(raw);
  if (X) cudaFree(X);
  if (Y) cudaFree(Y);
  if (dnorm) cudaFree(dnorm);
  if (order) cudaFree(order);
  if (dloss) cudaFree(dloss);
  return rc;
}

int newton_replay(Context &c, int learned, int fast, long long counts[5], double *v_host, double *step_host,
                  int *flag_host) {
  const long long n = newton_log_count(c);
  if (n <= 0) return EQD_ERR_STATE;
  if (learned && !c.mlp) return EQD_ERR_STATE;
  unsigned long long *dc = nullptr;
  double *dv = nullptr, *ds = nullptr;
  int *df = nullptr;
  MRC(dmalloc(reinterpret_cast<void **>(&dc), 4 * sizeof(unsigned long long)));
  cudaMemset(dc, 0, 4 * sizeof(unsigned long long));
  int rc = EQD_OK;
  if (v_host) rc = dmalloc(reinterpret_cast<void **>(&dv), sizeof(double) * n);
  if (!rc && step_host) rc = dmalloc(reinterpret_cast<void **>(&ds), sizeof(double) * n);
  if (!rc && flag_host) rc = dmalloc(reinterpret_cast<void **>(&df), sizeof(int) * n);
  if (!rc) {
    const unsigned grid = (unsigned)((n + 127) / 128);
    const MlpDevice *m = learned ? static_cast<const MlpDevice *>(c.mlp) : nullptr;
    if (fast) newton_replay_kernel<true><<<grid, 128>>>(c.nlog, n, c.sc.friclaw, c.sc.dt, m, dv, ds, df, dc);
    else newton_replay_kernel<false><<<grid, 128>>>(c.nlog, n, c.sc.friclaw, c.sc.dt, m, dv, ds, df, dc);
    unsigned long long h[4] = {0, 0, 0, 0};
    if (cudaMemcpy(h, dc, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) rc = EQD_ERR_CUDA;
    if (!rc && v_host && cudaMemcpy(v_host, dv, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = EQD_ERR_CUDA;
    if (!rc && step_host && cudaMemcpy(step_host, ds, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = EQD_ERR_CUDA;
    if (!rc && flag_host && cudaMemcpy(flag_host, df, sizeof(int) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = EQD_ERR_CUDA;
    for (int k = 0; k < 3; ++k) counts[k] = (long long)h[k];
    counts[3] = n;
    counts[4] = (long long)h[3];
  }
  cudaFree(dc);
  if (dv) cudaFree(dv);
  if (ds) cudaFree(ds);
  if (df) cudaFree(df);
  return rc;
}

}  // namespace eqd

using namespace eqd;

// Standalone loss and gradient of the MLP on a batch (for gradient checks): x [n][6] normalised
// inputs, y [n] normalised targets, params [kMlpParams] FP32 masters.
extern "C" int eqd_mlp_gradient(int32_t device, const float *params, const float *x, const float *y, int32_t n,
                                float *loss, float *grad) {
  if (!params || !x || !y || n <= 0 || !loss || !grad) return EQD_ERR_INPUT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return EQD_ERR_NO_DEVICE;
  }
  EQD_CUDA_OK(cudaSetDevice(device));
  std::vector<__nv_bfloat16> hx((size_t)n * kMlpK1, __float2bfloat16(0.f));
  for (int r = 0; r < n; ++r)
    for (int k = 0; k < kMlpIn; ++k) hx[(size_t)r * kMlpK1 + k] = __float2bfloat16(x[(size_t)r * kMlpIn + k]);
  MlpDevice *m = nullptr;
  float *P = nullptr, *G = nullptr, *Y = nullptr, *dl = nullptr;
  __nv_bfloat16 *X = nullptr;
  int rc = EQD_OK;
  do {
    if ((rc = dmalloc(reinterpret_cast<void **>(&m), sizeof(MlpDevice)))) break;
    cudaMemset(m, 0, sizeof(MlpDevice));
    if ((rc = dmalloc(reinterpret_cast<void **>(&P), sizeof(float) * 2 * kMlpParams))) break;
    G = P + kMlpParams;
    if ((rc = dmalloc(reinterpret_cast<void **>(&X), sizeof(__nv_bfloat16) * hx.size()))) break;
    if ((rc = dmalloc(reinterpret_cast<void **>(&Y), sizeof(float) * n))) break;
    if ((rc = dmalloc(reinterpret_cast<void **>(&dl), 2 * sizeof(float)))) break;  // loss, error word
    cudaMemcpy(P, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
    cudaMemset(G, 0, sizeof(float) * kMlpParams);
    cudaMemcpy(X, hx.data(), sizeof(__nv_bfloat16) * hx.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(Y, y, sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemset(dl, 0, 2 * sizeof(float));
    mlp_sync_kernel<<<(kMlpParams + 255) / 256, 256>>>(P, m, nullptr);
    if (cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem) !=
        cudaSuccess) {
      rc = EQD_ERR_CUDA;
      break;
    }
    TrainBatch tb{X, Y, nullptr, 0, n, 1.f / (float)n};
    mlp_grad_kernel<<<(unsigned)((n + kTrainRows - 1) / kTrainRows), kTrainRows, kGradSmem>>>(
        m, tb, G, dl, reinterpret_cast<int *>(dl + 1));
    float h[2] = {0.f, 0.f};
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(grad, G, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(h, dl, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = EQD_ERR_CUDA;
      break;
    }
    *loss = h[0];
    int herr = 0;
    std::memcpy(&herr, &h[1], sizeof(int));
    if (herr) rc = EQD_ERR_TIMEOUT;
  } while (false);
  if (m) cudaFree(m);
  if (P) cudaFree(P);
  if (X) cudaFree(X);
  if (Y) cudaFree(Y);
  if (dl) cudaFree(dl);
  return rc;
}
