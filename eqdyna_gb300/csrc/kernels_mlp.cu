// Learned Newton initial guess: logged solves -> features, tensor-core training (forward,
// backward, Adam), replay of logged solves, and the model's device parameter block.
//
// Training data are the rate-and-state Newton solves the plain method itself performs
// (eqd_gpu_newton_log).  Every kernel that touches the MLP runs its matrix products on the tensor
// cores with mma.sync.m16n8k16 (bf16 operands, fp32 accumulation; fragment helpers in
// mlp_common.cuh); biases, losses, Adam and the rank-1 output layer's gradient are fp32 on the
// CUDA cores.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "eqd_device.cuh"
#include "mlp_common.cuh"
#include "rsf_newton.cuh"

namespace eqd {

namespace {

constexpr int kTrainRows = 64;  // samples per CTA (4 warps x 16)

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

__device__ __forceinline__ void to_a(unsigned a[4], const float lo[4], const float hi[4]) {
  a[0] = pack_bf16(lo[0], lo[1]);
  a[1] = pack_bf16(lo[2], lo[3]);
  a[2] = pack_bf16(hi[0], hi[1]);
  a[3] = pack_bf16(hi[2], hi[3]);
}

struct TrainBatch {
  const __nv_bfloat16 *X;  // [n][16]
  const float *Y;          // [n]
  const int *order;        // sample ids, or null for 0..n-1
  long long start, count;  // this batch: order[start .. start + count)
  float inv_count;         // 1 / samples in the batch
};

// Forward + backward of one batch, 64 samples per CTA: loss += sum (y - t)^2 / (2 count),
// G += d loss / d params.  Weight gradients contract over the CTA's samples on the tensor cores
// (transposed activations staged in shared memory) and are reduced across CTAs with fp32 atomics.
__global__ void __launch_bounds__(128) mlp_grad_kernel(const MlpDevice *__restrict__ m, TrainBatch tb,
                                                       float *__restrict__ G, float *__restrict__ loss) {
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16 *sW1 = reinterpret_cast<__nv_bfloat16 *>(smem);  // [64][16]
  __nv_bfloat16 *sW2 = sW1 + kMlpH * kMlpK1;                     // [64][64]
  __nv_bfloat16 *sW2T = sW2 + kMlpH * kMlpH;                     // [64][64] transposed
  __nv_bfloat16 *sW3 = sW2T + kMlpH * kMlpH;                     // [8][64]
  __nv_bfloat16 *XT = sW3 + kMlpN3 * kMlpH;                      // [16][64 samples]
  __nv_bfloat16 *H1T = XT + kMlpK1 * kTrainRows;                 // [64][64 samples]
  __nv_bfloat16 *dZ2T = H1T + kMlpH * kTrainRows;
  __nv_bfloat16 *dZ1T = dZ2T + kMlpH * kTrainRows;
  float *sb1 = reinterpret_cast<float *>(dZ1T + kMlpH * kTrainRows);
  float *sb2 = sb1 + kMlpH;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, g = lane >> 2, t = lane & 3;
  for (int k = tid; k < kMlpH * kMlpK1; k += blockDim.x) sW1[k] = m->W1[k];
  for (int k = tid; k < kMlpH * kMlpH; k += blockDim.x) {
    sW2[k] = m->W2[k];
    sW2T[(k % kMlpH) * kMlpH + k / kMlpH] = m->W2[k];
  }
  for (int k = tid; k < kMlpN3 * kMlpH; k += blockDim.x) sW3[k] = m->W3[k];
  for (int k = tid; k < kMlpH; k += blockDim.x) sb1[k] = m->b1[k], sb2[k] = m->b2[k];
  __syncthreads();
  const float b3 = m->b3;
  const int s0 = w * 16;
  const long long base = tb.start + (long long)blockIdx.x * kTrainRows + s0;
  const long long end = tb.start + tb.count;
  auto sid = [&](int r) -> long long {
    const long long q = base + r;
    if (q >= end) return -1;
    return tb.order ? (long long)tb.order[q] : q;
  };
  const long long ig = sid(g), ig8 = sid(g + 8);
  unsigned xa[4] = {0u, 0u, 0u, 0u};
  if (ig >= 0) {
    xa[0] = ld32(tb.X + ig * kMlpK1 + 2 * t);
    xa[2] = ld32(tb.X + ig * kMlpK1 + 8 + 2 * t);
  }
  if (ig8 >= 0) {
    xa[1] = ld32(tb.X + ig8 * kMlpK1 + 2 * t);
    xa[3] = ld32(tb.X + ig8 * kMlpK1 + 8 + 2 * t);
  }
  {  // X^T for the first layer's weight gradient
    const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(xa);
    XT[(2 * t) * kTrainRows + s0 + g] = e[0];
    XT[(2 * t + 1) * kTrainRows + s0 + g] = e[1];
    XT[(2 * t) * kTrainRows + s0 + g + 8] = e[2];
    XT[(2 * t + 1) * kTrainRows + s0 + g + 8] = e[3];
    XT[(8 + 2 * t) * kTrainRows + s0 + g] = e[4];
    XT[(9 + 2 * t) * kTrainRows + s0 + g] = e[5];
    XT[(8 + 2 * t) * kTrainRows + s0 + g + 8] = e[6];
    XT[(9 + 2 * t) * kTrainRows + s0 + g + 8] = e[7];
  }
  float z1[8][4], z2[8][4], out[4];
  mlp_forward16(xa, sW1, sW2, sW3, sb1, sb2, b3, z1, z2, out);
  // output error on the lanes that hold column 0
  float d0 = 0.f, d2 = 0.f;
  if (t == 0) {
    if (ig >= 0) d0 = out[0] - tb.Y[ig];
    if (ig8 >= 0) d2 = out[2] - tb.Y[ig8];
  }
  float lsum = (d0 * d0 + d2 * d2) * 0.5f * tb.inv_count;
  const float dg = __shfl_sync(0xffffffffu, d0 * tb.inv_count, lane & ~3);
  const float dg8 = __shfl_sync(0xffffffffu, d2 * tb.inv_count, lane & ~3);
  // layer 3 and 2 backward
  float dz2[8][4], gw3[8][2], gb2[8][2];
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int n = 8 * j + 2 * t + (q & 1);
      const float dv = q < 2 ? dg : dg8;
      const float h2 = bf16r(fmaxf(z2[j][q], 0.f));
      dz2[j][q] = z2[j][q] > 0.f ? dv * __bfloat162float(sW3[n]) : 0.f;
      if (q < 2) gw3[j][q] = dv * h2, gb2[j][q] = dz2[j][q];
      else gw3[j][q - 2] += dv * h2, gb2[j][q - 2] += dz2[j][q];
    }
  // dH1 = dZ2 W2 (tensor cores, B = W2 read transposed), then dZ1
  float dz1[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) dz1[j][0] = dz1[j][1] = dz1[j][2] = dz1[j][3] = 0.f;
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    unsigned a[4];
    to_a(a, dz2[2 * kk], dz2[2 * kk + 1]);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      unsigned b[2];
      frag_bt(b, sW2T, kMlpH, 8 * j, 16 * kk);
      mma_bf16(dz1[j], a, b);
    }
  }
  float gb1[8][2];
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      dz1[j][q] = z1[j][q] > 0.f ? dz1[j][q] : 0.f;
      if (q < 2) gb1[j][q] = dz1[j][q];
      else gb1[j][q - 2] += dz1[j][q];
    }
  // transposed activations / errors of this warp's 16 samples
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int n = 8 * j + 2 * t + (q & 1), r = s0 + g + (q < 2 ? 0 : 8);
      H1T[n * kTrainRows + r] = __float2bfloat16(fmaxf(z1[j][q], 0.f));
      dZ2T[n * kTrainRows + r] = __float2bfloat16(dz2[j][q]);
      dZ1T[n * kTrainRows + r] = __float2bfloat16(dz1[j][q]);
    }
  // column sums over the warp's rows: reduce across the 8 row groups (lane bits 2-4)
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) {
        gw3[j][q] += __shfl_xor_sync(0xffffffffu, gw3[j][q], o);
        gb2[j][q] += __shfl_xor_sync(0xffffffffu, gb2[j][q], o);
        gb1[j][q] += __shfl_xor_sync(0xffffffffu, gb1[j][q], o);
      }
      if (g == 0) {
        const int n = 8 * j + 2 * t + q;
        atomicAdd(G + kOffW3 + n, gw3[j][q]);
        atomicAdd(G + kOffB2 + n, gb2[j][q]);
        atomicAdd(G + kOffB1 + n, gb1[j][q]);
      }
    }
  float db3 = (t == 0) ? (d0 + d2) * tb.inv_count : 0.f;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    db3 += __shfl_xor_sync(0xffffffffu, db3, o);
    lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  }
  if (lane == 0) {
    atomicAdd(G + kOffB3, db3);
    atomicAdd(loss, lsum);
  }
  __syncthreads();
  // dW2 [n2][k1] = dZ2^T H1 and dW1 [n1][k0] = dZ1^T X over the CTA's 64 samples; warp w owns
  // output rows 16 w .. 16 w + 15
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kk = 0; kk < kTrainRows / 16; ++kk) {
      unsigned a[4], b[2];
      frag_a(a, dZ2T, kTrainRows, 16 * w, 16 * kk);
      frag_bt(b, H1T, kTrainRows, 8 * j, 16 * kk);
      mma_bf16(c, a, b);
    }
    float *gw = G + kOffW2 + (16 * w + g) * kMlpH + 8 * j + 2 * t;
    atomicAdd(gw, c[0]);
    atomicAdd(gw + 1, c[1]);
    atomicAdd(gw + 8 * kMlpH, c[2]);
    atomicAdd(gw + 8 * kMlpH + 1, c[3]);
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kk = 0; kk < kTrainRows / 16; ++kk) {
      unsigned a[4], b[2];
      frag_a(a, dZ1T, kTrainRows, 16 * w, 16 * kk);
      frag_bt(b, XT, kTrainRows, 8 * j, 16 * kk);
      mma_bf16(c, a, b);
    }
    const int k0 = 8 * j + 2 * t;
    float *gw = G + kOffW1 + (16 * w + g) * kMlpK1 + k0;
    if (k0 < kMlpIn) {
      atomicAdd(gw, c[0]);
      atomicAdd(gw + 8 * kMlpK1, c[2]);
    }
    if (k0 + 1 < kMlpIn) {
      atomicAdd(gw + 1, c[1]);
      atomicAdd(gw + 8 * kMlpK1 + 1, c[3]);
    }
  }
}

constexpr size_t kGradSmem = (size_t)(kMlpH * kMlpK1 + 2 * kMlpH * kMlpH + kMlpN3 * kMlpH + kMlpK1 * kTrainRows +
                                      3 * kMlpH * kTrainRows) * 2 + 2 * kMlpH * 4;

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
    if ((rc = dmalloc(reinterpret_cast<void **>(&dloss), sizeof(float)))) break;
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
        mlp_grad_kernel<<<grid, 128, kGradSmem>>>(static_cast<MlpDevice *>(c.mlp), tb, c.mlp_g, dloss);
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
        mlp_grad_kernel<<<(unsigned)((nhold + kTrainRows - 1) / kTrainRows), 128, kGradSmem>>>(
            static_cast<MlpDevice *>(c.mlp), tb, gscratch, dloss);
        if (cudaMemcpy(holdout_loss, dloss, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) rc = EQD_ERR_CUDA;
        cudaFree(gscratch);
      }
    }
    if (cudaDeviceSynchronize() != cudaSuccess) rc = EQD_ERR_CUDA;
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
    if ((rc = dmalloc(reinterpret_cast<void **>(&dl), sizeof(float)))) break;
    cudaMemcpy(P, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
    cudaMemset(G, 0, sizeof(float) * kMlpParams);
    cudaMemcpy(X, hx.data(), sizeof(__nv_bfloat16) * hx.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(Y, y, sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemset(dl, 0, sizeof(float));
    mlp_sync_kernel<<<(kMlpParams + 255) / 256, 256>>>(P, m, nullptr);
    if (cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem) !=
        cudaSuccess) {
      rc = EQD_ERR_CUDA;
      break;
    }
    TrainBatch tb{X, Y, nullptr, 0, n, 1.f / (float)n};
    mlp_grad_kernel<<<(unsigned)((n + kTrainRows - 1) / kTrainRows), 128, kGradSmem>>>(m, tb, G, dl);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(grad, G, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(loss, dl, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = EQD_ERR_CUDA;
  } while (false);
  if (m) cudaFree(m);
  if (P) cudaFree(P);
  if (X) cudaFree(X);
  if (Y) cudaFree(Y);
  if (dl) cudaFree(dl);
  return rc;
}
