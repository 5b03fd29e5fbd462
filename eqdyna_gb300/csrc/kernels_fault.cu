// Node update and split-node fault kernels.
//
// node_update  : the mass division of the previous step (src/driver.f90:29) fused with
//                velDispUpdate (src/driver.f90:89-155): central-difference update of 3-DOF nodes,
//                damped split-field update of 12-DOF PML nodes (comdampv precomputed per node),
//                NaN detection, and zeroing of the force accumulators for this step.
// fault_kernel : one thread per split-node pair: thermop (src/thermop.f90), faulting
//                (src/faulting.f90:3-541) with the friction laws (src/fric.f90), station capture
//                (src/faulting.f90:518-541, src/driver.f90:157-180) and rupture time.
#include <algorithm>
#include <vector>

#include "eqd_device.cuh"
#include "fpconv.cuh"
#include "mlp_common.cuh"
#include "rsf_newton.cuh"
#include "elem32r_body.cuh"

namespace eqd {

namespace {

constexpr int kBlockNode = 256;       // default node-update block
constexpr int kBlockNodeMax = 512;
constexpr int kBlockFault = 128;      // default and largest fault-kernel block

// Node update of the binary64 form (velDispUpdate, src/driver.f90:89-155; comdampv for PML nodes).
template <bool F_IS_ACC>
__global__ void __launch_bounds__(kBlockNodeMax)
    node_update(double *__restrict__ vel, double *__restrict__ disp, double *__restrict__ F,
                const double *__restrict__ inv_mass, double *__restrict__ F9,
                double *__restrict__ v9, double *__restrict__ vh,
                const double *__restrict__ pml_ab, int nnode, int n_int, int npml, double dt,
                int *__restrict__ d_nt, int *__restrict__ d_err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *d_nt += 1;
  if (i >= nnode) return;
  const double im = inv_mass[i];
  double v[3];
  if (i < n_int) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double f = F[c * nnode + i];
      const double acc = F_IS_ACC ? f : f * im;
      v[c] = fma(acc, dt, vel[c * nnode + i]);
      vel[c * nnode + i] = v[c];
      disp[c * nnode + i] = fma(v[c], dt, disp[c * nnode + i]);
      F[c * nnode + i] = 0.0;
    }
  } else {
    const int p = i - n_int;
    if (im == 0.0) {  // fixed boundary node: eq = -1 (src/driver.f90:141-144)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        v[c] = 0.0;
        vel[c * nnode + i] = 0.0;
        disp[c * nnode + i] = 0.0;
        F[c * nnode + i] = 0.0;
      }
#pragma unroll
      for (int j = 0; j < 9; ++j) F9[j * npml + p] = 0.0;
    } else {
      double vs[3] = {0, 0, 0};
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        const int ax = j % 3;
        const double f = F9[j * npml + p];
        const double acc = F_IS_ACC ? f : f * im;
        const double nv = fma(pml_ab[ax * npml + p], v9[j * npml + p], acc) * pml_ab[(3 + ax) * npml + p];
        v9[j * npml + p] = nv;
        vs[j / 3] += nv;
        F9[j * npml + p] = 0.0;
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double f = F[c * nnode + i];
        const double acc = F_IS_ACC ? f : f * im;
        const double nh = fma(acc, dt, vh[c * npml + p]);
        vh[c * npml + p] = nh;
        v[c] = vs[c] + nh;
        vel[c * nnode + i] = v[c];
        disp[c * nnode + i] = fma(v[c], dt, disp[c * nnode + i]);
        F[c * nnode + i] = 0.0;
      }
    }
  }
  if (isnan(v[0]) || isnan(v[1]) || isnan(v[2])) atomicOr(d_err, 1);
}

// Arguments of the binary32 node update (one context).
struct NodeArgs32 {
  double *vel, *disp;
  float *F;
  const float *inv_mass;
  float *F9, *v9;
  double *vh;
  const float *pml_ab;
  int nnode, n_int, npml, nsplit;
  int n_split, npml_live;  // device order: split nodes first, fixed PML nodes after the live ones
  float dt;
  double dtd, rdampk;
  int *d_nt, *d_err;
  float *vel32, *dl32;
  const double *Fsplit;
  const int *split_slot;
  int f_is_acc;  // used by the batched launch (the single launch selects a template instead)
  int damp;      // rdampk != 0: the element kernels read u + rdampk v instead of u
  float rdampk32;
  int skip_split;  // split nodes are left to split_update32 (overlapped step schedule)
};

// Split (fault) node i, slot q of Fsplit: the fault kernel set its force in binary64; the update is
// binary64 so that the slave-master relative motion keeps binary64 resolution (creep rates
// ~1e-12..1e-16 m/s).
template <bool F_IS_ACC>
__device__ __forceinline__ void split_node_update(const NodeArgs32 &a, int i, int q) {
  const int nnode = a.nnode;
  const double imd = -(double)a.inv_mass[i];
  double v[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double f = a.Fsplit[(size_t)c * a.nsplit + q];
    const double acc = F_IS_ACC ? f : f * imd;
    v[c] = fma(acc, a.dtd, a.vel[c * nnode + i]);
    a.vel[c * nnode + i] = v[c];
    const double u = fma(v[c], a.dtd, a.disp[c * nnode + i]);
    a.disp[c * nnode + i] = u;
    a.F[c * nnode + i] = 0.f;
    a.vel32[c * nnode + i] = (float)v[c];
    a.dl32[c * nnode + i] = (float)fma(a.rdampk, v[c], u);
  }
  if (isnan(v[0]) || isnan(v[1]) || isnan(v[2])) atomicOr(a.d_err, 1);
}

// Node update of the binary32 form.  The force sums arrive in binary32 (Kahan-compensated per
// tile); acceleration, its increment a*dt and the PML split-field velocities are binary32, while
// velocity and displacement of every node stay binary64 (increments are small against the state,
// which is accumulated over 10^3 - 10^4 steps).  Two binary64 operations per component (v += dv,
// u += v dt; two more for the PML split sum), no binary64 conversion: the conversions between the
// formats run on the integer pipe (fpconv.cuh) and u + rdampk v is formed in binary32.  Split
// (fault) nodes are updated entirely in binary64.
template <bool F_IS_ACC, bool DAMP>
__device__ __forceinline__ void node_update32_body(const NodeArgs32 &a, int i) {
  double *__restrict__ vel = a.vel;
  double *__restrict__ disp = a.disp;
  float *__restrict__ F = a.F;
  const float *__restrict__ inv_mass = a.inv_mass;
  float *__restrict__ F9 = a.F9;
  float *__restrict__ v9 = a.v9;
  double *__restrict__ vh = a.vh;
  const float *__restrict__ pml_ab = a.pml_ab;
  const int nnode = a.nnode, n_int = a.n_int, npml = a.npml;
  const float dt = a.dt;
  const double dtd = a.dtd;
  const float rdampk32 = a.rdampk32;
  int *__restrict__ d_err = a.d_err;
  float *__restrict__ vel32 = a.vel32;
  float *__restrict__ dl32 = a.dl32;
  const int *__restrict__ split_slot = a.split_slot;
  if (i == 0) *a.d_nt += 1;
  if (i >= nnode) return;
  // the node classes are index ranges (device order), so no test waits for a loaded value
  if (i < a.n_split) {
    if (!a.skip_split) split_node_update<F_IS_ACC>(a, i, split_slot[i]);
    return;
  }
  const float im = inv_mass[i];
  double v[3];
  if (i < n_int) {
    float v32[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float f = F[c * nnode + i];
      const float dv = F_IS_ACC ? f * dt : f * im * dt;
      const double vn = vel[c * nnode + i] + widen_f32(dv);
      vel[c * nnode + i] = vn;
      const double u = fma(vn, dtd, disp[c * nnode + i]);
      disp[c * nnode + i] = u;
      F[c * nnode + i] = 0.f;
      v32[c] = narrow_f64(vn);
      vel32[c * nnode + i] = v32[c];
      // u + rdampk v for the element kernels, formed in binary32 from the rounded u and v (within
      // 1.5 units in the last place of the binary32 value, against 0.5 when formed in binary64)
      dl32[c * nnode + i] = DAMP ? fmaf(rdampk32, v32[c], narrow_f64(u)) : narrow_f64(u);
    }
    if (isnan(v32[0]) || isnan(v32[1]) || isnan(v32[2])) atomicOr(d_err, 1);
    return;
  } else {
    const int p = i - n_int;
    if (p >= a.npml_live) {  // fixed PML node (or padding): 1/m = 0
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        v[c] = 0.0;
        vel[c * nnode + i] = 0.0;
        disp[c * nnode + i] = 0.0;
        F[c * nnode + i] = 0.f;
        vel32[c * nnode + i] = 0.f;
        dl32[c * nnode + i] = 0.f;
      }
#pragma unroll
      for (int j = 0; j < 9; ++j) F9[j * npml + p] = 0.f;
    } else {
      float vs[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        const int ax = j % 3;
        const float f = F9[j * npml + p];
        const float acc = F_IS_ACC ? f : f * im;
        const float nv = fmaf(pml_ab[ax * npml + p], v9[j * npml + p], acc) * pml_ab[(3 + ax) * npml + p];
        v9[j * npml + p] = nv;
        vs[j / 3] += nv;
        F9[j * npml + p] = 0.f;
      }
      float v32[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float f = F[c * nnode + i];
        const float dv = F_IS_ACC ? f * dt : f * im * dt;
        const double nh = vh[c * npml + p] + widen_f32(dv);
        vh[c * npml + p] = nh;
        const double vn = widen_f32(vs[c]) + nh;
        vel[c * nnode + i] = vn;
        const double u = fma(vn, dtd, disp[c * nnode + i]);
        disp[c * nnode + i] = u;
        F[c * nnode + i] = 0.f;
        v32[c] = narrow_f64(vn);
        vel32[c * nnode + i] = v32[c];
        dl32[c * nnode + i] = DAMP ? fmaf(rdampk32, v32[c], narrow_f64(u)) : narrow_f64(u);
      }
      if (isnan(v32[0]) || isnan(v32[1]) || isnan(v32[2])) atomicOr(d_err, 1);
      return;
    }
  }
  if (isnan(v[0]) || isnan(v[1]) || isnan(v[2])) atomicOr(d_err, 1);
}

template <bool F_IS_ACC, bool DAMP>
__global__ void __launch_bounds__(kBlockNodeMax) node_update32(NodeArgs32 a) {
  node_update32_body<F_IS_ACC, DAMP>(a, blockIdx.x * blockDim.x + threadIdx.x);
}

// Member of a batch that owns block b: the largest m with start[m] <= b (start: n + 1 prefix sums).
__device__ __forceinline__ int batch_member(const int *__restrict__ start, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Node update of every member of an ensemble in one launch.
__global__ void __launch_bounds__(kBlockNode) node_update32_batched(const NodeArgs32 *__restrict__ args,
                                                                    const int *__restrict__ start, int n) {
  __shared__ NodeArgs32 a;
  __shared__ int lb;
  if (threadIdx.x == 0) {
    const int m = batch_member(start, n, blockIdx.x);
    a = args[m];
    lb = blockIdx.x - start[m];
  }
  __syncthreads();
  const int i = lb * blockDim.x + threadIdx.x;
  if (a.f_is_acc) {
    if (a.damp) node_update32_body<true, true>(a, i);
    else node_update32_body<true, false>(a, i);
  } else {
    if (a.damp) node_update32_body<false, true>(a, i);
    else node_update32_body<false, false>(a, i);
  }
}

struct FaultArgs {
  int npair, nnode, nstep, nOnSt, nOffRows, nftmx_tp;
  int friclaw, TPV, C_nuclea_here, C_elastic, insertFaultType;
  double dt, nucR, nucRuptVel, nucdtau0, nucT, slipRateThres, fric_tp_h;
  const int *pair_s, *pair_m;
  const double *geo;          // [13][np]
  double *fric;               // [100][np]
  double *fnft;
  double *tp_hist;            // (2, np, nstep) or null
  const PairStation *onst;
  double *onhist;
  const int *off_rows;
  double *offhist;
  double *F;                  // binary64 form forces, or null
  float *F32;                 // binary32 form element-force sums, or null
  double *Fsplit;             // binary32 form: binary64 output forces [3][2 * npair]
  const double *vel, *disp;
  const int *d_nt;
  const double *d_times;
  unsigned long long *stats;
  const MlpDevice *mlp;       // learned initial guess, or null
  double *newton_log;         // [log_steps][npair][kNewtonRecord] logged solves, or null
  int log_nt0, log_steps, log_stride;  // steps log_nt0 + k log_stride, k = 1 .. log_steps
};

// Force of node `node`, component c, in the form's own precision.
template <bool F32>
__device__ __forceinline__ double force_get(const FaultArgs &p, int c, int node) {
  return F32 ? (double)p.F32[(size_t)c * p.nnode + node] : p.F[(size_t)c * p.nnode + node];
}
// Writes the pair's new force.  The binary32 form keeps split-node forces in binary64 (slot
// 2 i for the slave, 2 i + 1 for the master of pair i).
template <bool F32>
__device__ __forceinline__ void force_set(const FaultArgs &p, int c, int node, int slot, double v) {
  if (F32) p.Fsplit[(size_t)c * 2 * p.npair + slot] = v;
  else p.F[(size_t)c * p.nnode + node] = v;
}

// Thermal pressurization (src/thermop.f90:1-40): pore pressure and temperature change of every
// pair by convolution of its slip-rate x shear-stress history with the diffusion kernels, O(nt)
// per pair per step.  32 pairs per CTA of 8 warps; warp w takes history rows w, w + 8, ... (each
// row a coalesced 32-pair read of the step-major history), the warps' partial sums are added in
// shared memory.
constexpr int kTpWarps = 8;
__global__ void __launch_bounds__(32 * kTpWarps) thermop_kernel(FaultArgs p) {
  __shared__ double part[kTpWarps][2][32];
  const int nt = *p.d_nt;
  const int np = p.npair;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  double tp = 0.0, tt = 0.0;
  if (i < np) {
    const double *fr = p.fric + i;
#define FR(k) fr[((k)-1) * np]
    const double omega = FR(16), kapa = FR(17), h2 = 2.0 * p.fric_tp_h * p.fric_tp_h;
    const double dt = p.dt;
    const int jmax = nt - 1 < p.nstep ? nt - 1 : p.nstep;  // history rows that exist
    for (int j = 1 + w; j <= jmax; j += kTpWarps) {
      const double *hh = p.tp_hist + 2 * ((size_t)i + (size_t)np * (j - 1));
      const double q = fabs(hh[1]) * hh[0];
      const double s1 = sqrt(4.0 * kapa * (nt - j) * dt + h2);
      const double s2 = sqrt(4.0 * omega * (nt - j) * dt + h2);
      const double ker = -kapa / (omega - kapa) / s1 + omega / (omega - kapa) / s2;
      tp += q * ker * dt;
      tt += q * (1.0 / s1) * dt;
    }
#undef FR
  }
  part[w][0][lane] = tp;
  part[w][1][lane] = tt;
  __syncthreads();
  if (w == 0 && i < np) {
    for (int k = 1; k < kTpWarps; ++k) tp += part[k][0][lane], tt += part[k][1][lane];
    double *fr = p.fric + i;
#define FR(k) fr[((k)-1) * np]
    const double gama = FR(19) / FR(18);
    const double rpi = sqrt(3.14159265358979323846);
    FR(51) = tp * gama / rpi;
    FR(52) = tt / FR(18) / rpi + FR(41);
#undef FR
  }
}

// RSF = false leaves the rate-and-state branch (friclaw 3-5) out of the instantiation: a kernel
// that runs slip- or time-weakening faults only then carries none of the Newton solve's registers.
template <bool F32, bool RSF = true>
__device__ __forceinline__ void fault_body(const FaultArgs &p, int tid,
                                           __nv_bfloat16 (*mlp_xs)[32 * kMlpK1]) {
  const int nt = *p.d_nt;
  const double t = p.d_times[nt];
  const int np = p.npair;
  const int nn = p.nnode;
  if (tid >= np) {
    // off-fault station rows (storeOffFaultStData): row 0 is the time
    const int r = tid - np;
    if (r <= p.nOffRows && nt >= 1 && nt <= p.nstep && p.offhist) {
      double val = t;
      if (r > 0) {
        const int node = p.off_rows[r - 1], comp = p.off_rows[p.nOffRows + r - 1];
        const int type = p.off_rows[2 * p.nOffRows + r - 1];
        val = (type == 1) ? p.disp[comp * nn + node] : p.vel[comp * nn + node];
      }
      p.offhist[(size_t)(p.nOffRows + 1) * (nt - 1) + r] = val;
    }
    return;
  }
  const int i = tid;
  double *fr = p.fric + i;
#define FR(k) fr[((k)-1) * np]
  const double dt = p.dt;
  const int sl = p.pair_s[i], ms = p.pair_m[i];
  const double un[3] = {p.geo[0 * np + i], p.geo[1 * np + i], p.geo[2 * np + i]};
  const double us[3] = {p.geo[3 * np + i], p.geo[4 * np + i], p.geo[5 * np + i]};
  const double ud[3] = {p.geo[6 * np + i], p.geo[7 * np + i], p.geo[8 * np + i]};
  const double arn = p.geo[9 * np + i], mS = p.geo[10 * np + i], mM = p.geo[11 * np + i];
  const double radius = p.geo[12 * np + i];

  // thermal pressurization (src/thermop.f90): fric(51), fric(52) come from thermop_kernel, which
  // runs just before this kernel

  // getNsdSlipSliprateTraction (src/faulting.f90:54-134)
  const double init[3] = {FR(7), FR(8), FR(49)};
  const double totalMass = (mS + mM) * arn;
  double q[3][2][3];  // [n|s|d][slave|master][force|vel|disp]
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int node = j == 0 ? sl : ms;
    double x[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      x[0][c] = force_get<F32>(p, c, node);
      x[1][c] = p.vel[c * nn + node];
      x[2][c] = p.disp[c * nn + node];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      q[0][j][k] = x[k][0] * un[0] + x[k][1] * un[1] + x[k][2] * un[2];
      q[1][j][k] = x[k][0] * us[0] + x[k][1] * us[1] + x[k][2] * us[2];
      q[2][j][k] = x[k][0] * ud[0] + x[k][1] * ud[1] + x[k][2] * ud[2];
    }
  }
  double slip[4], rate[4], tr[4];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    slip[j] = q[j][1][2] - q[j][0][2];
    rate[j] = q[j][1][1] - q[j][0][1];
  }
  slip[3] = sqrt(slip[0] * slip[0] + slip[1] * slip[1] + slip[2] * slip[2]);
  rate[3] = sqrt(rate[0] * rate[0] + rate[1] * rate[1] + rate[2] * rate[2]);
  FR(71) = slip[1];
  FR(72) = slip[2];
  FR(73) = slip[0];
  FR(74) = rate[1];
  FR(75) = rate[2];
  if (rate[3] > FR(76)) FR(76) = rate[3];
  FR(77) = FR(77) + rate[3] * dt;
  const double mSM = mS * mM;
  tr[0] = (mSM * ((q[0][1][1] - q[0][0][1]) + (q[0][1][2] - q[0][0][2]) / dt) / dt + mS * q[0][1][0] -
           mM * q[0][0][0]) / totalMass + init[0] * p.C_elastic;
  tr[1] = (mSM * (q[1][1][1] - q[1][0][1]) / dt + mS * q[1][1][0] - mM * q[1][0][0]) / totalMass +
          init[1] * p.C_elastic;
  tr[2] = (mSM * (q[2][1][1] - q[2][0][1]) / dt + mS * q[2][1][0] - mM * q[2][0][0]) / totalMass +
          init[2] * p.C_elastic;
  if (RSF && p.friclaw >= 3 && p.C_nuclea_here) {  // rsfNucleation (src/faulting.f90:367-414)
    double dtau = 0.0, Fn = 0.0, G = 1.0;
    if (radius < p.nucR) Fn = exp(radius * radius / (radius * radius - p.nucR * p.nucR));
    if (t <= p.nucT) G = exp((t - p.nucT) * (t - p.nucT) / (t * (t - 2.0 * p.nucT)));
    if (p.TPV == 105 || p.TPV == 104) {
      dtau = p.nucdtau0 * Fn * G;
    } else if (p.TPV == 2802) {
      if (nt == 1) {
        FR(81) = p.nucdtau0;
        const double ttao = sqrt(tr[1] * tr[1] + tr[2] * tr[2]);
        const double bs = sqrt((rate[1] + FR(26)) * (rate[1] + FR(26)) + (rate[2] + FR(27)) * (rate[2] + FR(27)));
        FR(20) = FR(9) * log(2.0 * FR(12) / bs * sinh(ttao / fabs(tr[0]) / FR(9)));
        FR(23) = fabs(tr[0]);
      }
      dtau = FR(81) * Fn * G;
    }
    tr[1] += dtau;
  }
  tr[3] = sqrt(tr[1] * tr[1] + tr[2] * tr[2]);

  unsigned iters = 0, maxhit = 0, executed = 0, learned = 0, fallback = 0;
  if (!RSF || p.friclaw <= 2) {
    // solveSWTW (src/faulting.f90:136-188)
    double mu;
    if (p.friclaw == 1) {
      const double slp = FR(77);
      mu = 0.0;
      if (fabs(slp) < 1.0e-10) mu = FR(1);
      else if (slp < FR(3)) mu = FR(1) - (FR(1) - FR(2)) * slp / FR(3);
      if (slp >= FR(3)) mu = FR(2);
    } else {
      const double tru = t - p.fnft[i];
      if (tru <= 0.0) mu = FR(1);
      else if (tru < FR(5)) mu = FR(1) - (FR(1) - FR(2)) * tru / FR(5);
      else mu = FR(2);
    }
    if (p.C_nuclea_here) {  // swtwNucleation (src/faulting.f90:416-443)
      double trr = 1.0e9;
      if (radius <= p.nucR) {
        if (p.TPV == 201 || p.TPV == 36 || p.TPV == 37)
          trr = (radius + 0.081 * p.nucR * (1.0 / (1.0 - (radius / p.nucR) * (radius / p.nucR)) - 1.0)) / (0.7 * 3464.0);
        if (p.TPV == 202) trr = radius / p.nucRuptVel;
      }
      double tc = 1.0;
      if (t < trr) tc = 0.0;
      else if (t < trr + FR(5) && t >= trr) tc = (t - trr) / FR(5);
      mu = fmin(FR(1) + (FR(2) - FR(1)) * tc, mu);
    }
    const double ens = (tr[0] + FR(6) > 0) ? 0.0 : tr[0] + FR(6);
    const double strength = FR(4) - mu * ens;
    if (tr[3] > strength) {
      tr[1] = tr[1] * strength / tr[3];
      tr[2] = tr[2] * strength / tr[3];
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double xt = (tr[0] * un[j] + tr[1] * us[j] + tr[2] * ud[j]) * arn;
      const double xi = (init[0] * un[j] + init[1] * us[j] + init[2] * ud[j]) * arn;
      force_set<F32>(p, j, sl, 2 * i, force_get<F32>(p, j, sl) + xt - xi * p.C_elastic);
      force_set<F32>(p, j, ms, 2 * i + 1, force_get<F32>(p, j, ms) - xt + xi * p.C_elastic);
    }
    FR(78) = tr[0];
    FR(79) = tr[1];
    FR(80) = tr[2];
  } else if constexpr (RSF) {
    // solveRSF (src/faulting.f90:190-327)
    tr[0] += (p.friclaw == 5) ? FR(51) : FR(6);
    if (p.insertFaultType > 0 && p.C_elastic == 1) {
      if (tr[0] >= -10.0e6) tr[0] = -10.0e6;
      else if (tr[0] <= -40.0e6) tr[0] = -40.0e6;
    }
    if (tr[0] > 0.0) tr[0] = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      slip[j] += FR(25 + j) * t;
      rate[j] += FR(25 + j);
    }
    slip[3] = sqrt(slip[1] * slip[1] + slip[2] * slip[2]);
    rate[3] = sqrt(rate[1] * rate[1] + rate[2] * rate[2]);
    double vt = rate[3];
    const double thpc0 = FR(23);
    const double L = FR(11);
    {
      const double thdot = -vt / L * (FR(23) - fabs(tr[0]));
      FR(23) = FR(23) + thdot * dt;
      FR(24) = thdot;
    }
    const double state0 = FR(20);
    const RsfParams rp{FR(9), FR(10), FR(11), FR(12), FR(13), FR(14), FR(15)};
    double xmu, dxmudv;
    {
      double st = FR(20);
      rsf_law(p.friclaw, vt, st, rp, dt, xmu, dxmudv);
      FR(20) = st;
    }
    const double taoc_old = (p.friclaw == 5) ? FR(4) - xmu * tr[0] : xmu * thpc0;
    const double mr = mM * mS / (mM + mS);
    const double Tc = arn * dt / mr;
    double trial[4];
#pragma unroll
    for (int j = 1; j <= 2; ++j) trial[j] = tr[j] - taoc_old * 0.5 * (rate[j] / rate[3]) + FR(25 + j) / Tc;
    trial[3] = sqrt(trial[1] * trial[1] + trial[2] * trial[2]);
    const NewtonSolve ns{rp, state0, thpc0, tr[0], trial[3], Tc, FR(4)};
    // learned initial guess for the Newton iteration (same residual, same exit test): the
    // tensor-core MLP over the warp's 32 pairs (the scalar path in the last, incomplete warp)
    double v0 = vt;
    if (p.mlp) {
      float f[kMlpIn];
      mlp_features(vt, state0, tr[0], trial[3], rp.A, rp.B, f);
      const bool full = (tid & ~31) + 32 <= np;
      v0 = mlp_guess_warp(*p.mlp, f, vt, full, mlp_xs[threadIdx.x >> 5]);
      learned = 1;
    }
    NewtonOut no = rsf_newton<true>(p.friclaw, dt, ns, v0);
    if (learned && !newton_settled(no)) {  // the learned guess was outside the Newton's basin
      const NewtonOut first = no;
      no = rsf_newton<true>(p.friclaw, dt, ns, vt);
      no.iters += first.iters;
      no.executed += first.executed;
      fallback = 1;
    }
    const int lstep = nt - p.log_nt0;
    if (p.newton_log && lstep > 0 && lstep % p.log_stride == 0 && lstep / p.log_stride <= p.log_steps) {
      double *rec = p.newton_log + (size_t)kNewtonRecord * ((size_t)(lstep / p.log_stride - 1) * np + i);
      const double vals[kNewtonRecord] = {rp.A,  rp.B,     rp.L,  rp.V0,    rp.f0,    rp.fw, rp.Vw, state0,
                                          thpc0, tr[0],    trial[3], Tc, FR(4), vt,    no.v,  (double)no.iters};
#pragma unroll
      for (int k = 0; k < kNewtonRecord; ++k) rec[k] = vals[k];
    }
    vt = no.v;
    const double stateTmp = no.state, thTmp = no.th, taoc_new = no.taoc;
    iters = no.iters;
    maxhit = no.capped;
    executed = no.executed;
    if (p.TPV == 105 && vt < FR(46)) vt = FR(46);
    FR(20) = stateTmp;
    FR(23) = thTmp;
#pragma unroll
    for (int j = 1; j <= 2; ++j) tr[j] = taoc_old * 0.5 * (rate[j] / rate[3]) + taoc_new * 0.5 * (trial[j] / trial[3]);
    FR(78) = tr[0];
    FR(79) = tr[1];
    FR(80) = tr[2];
    FR(47) = vt;
    FR(48) = sqrt(tr[1] * tr[1] + tr[2] * tr[2]);
    if (p.tp_hist && nt >= 1 && nt <= p.nstep) {
      double *hh = p.tp_hist + 2 * ((size_t)i + (size_t)np * (nt - 1));
      hh[0] = FR(47);
      hh[1] = FR(48);
    }
    const double acc[3] = {-rate[0] / dt - slip[0] / dt / dt, (vt * (trial[1] / trial[3]) - rate[1]) / dt,
                           (vt * (trial[2] / trial[3]) - rate[2]) / dt};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double xa = acc[0] * un[j] + acc[1] * us[j] + acc[2] * ud[j];
      const double R = force_get<F32>(p, j, sl) + force_get<F32>(p, j, ms);
      force_set<F32>(p, j, sl, 2 * i, (-xa + R / mM) * mr);
      force_set<F32>(p, j, ms, 2 * i + 1, (xa + R / mS) * mr);
      FR(31 + j) = p.vel[j * nn + ms] + (xa + R / mS) * dt;
      FR(34 + j) = p.vel[j * nn + sl] + (-xa + R / mM) * dt;
    }
  }
  if (RSF && p.friclaw >= 3) {
    warp_count_add(p.stats + 0, iters);
    warp_count_add(p.stats + 1, maxhit);
    warp_count_add(p.stats + 2, executed);
    warp_count_add(p.stats + 3, learned);
    warp_count_add(p.stats + 4, fallback);
  }
  // storeOnFaultStationQuantSCEC
  if (nt >= 1 && nt <= p.nstep) {
    for (int j = 0; j < p.nOnSt; ++j) {
      if (p.onst[j].pair != i) continue;
      double *h = p.onhist + 12 * ((size_t)(nt - 1) + (size_t)p.nstep * p.onst[j].column);
      h[0] = t;
      h[1] = rate[1];
      h[2] = rate[2];
      h[3] = FR(20);
      h[4] = slip[1];
      h[5] = slip[2];
      h[6] = slip[0];
      h[7] = tr[1];
      h[8] = tr[2];
      h[9] = tr[0];
      h[10] = FR(51) + FR(42);
      h[11] = FR(52);
    }
  }
  // storeRuptureTime
  if (p.fnft[i] > 5000.0 && rate[3] >= p.slipRateThres) p.fnft[i] = t;
#undef FR
}

template <bool F32>
__global__ void __launch_bounds__(kBlockFault) fault_kernel(FaultArgs p) {
  __shared__ __align__(16) __nv_bfloat16 mlp_xs[kBlockFault / 32][32 * kMlpK1];
  fault_body<F32>(p, blockIdx.x * blockDim.x + threadIdx.x, mlp_xs);
}

// Fault pairs (and station rows) of every member of an ensemble in one launch.
__global__ void __launch_bounds__(kBlockFault) fault_kernel_batched(const FaultArgs *__restrict__ args,
                                                                    const int *__restrict__ start, int n) {
  __shared__ __align__(16) __nv_bfloat16 mlp_xs[kBlockFault / 32][32 * kMlpK1];
  __shared__ FaultArgs p;
  __shared__ int lb;
  if (threadIdx.x == 0) {
    const int m = batch_member(start, n, blockIdx.x);
    p = args[m];
    lb = blockIdx.x - start[m];
  }
  __syncthreads();
  fault_body<true>(p, lb * blockDim.x + threadIdx.x, mlp_xs);
}

NodeArgs32 node_args32(const Context &c) {
  NodeArgs32 a;
  a.vel = c.vel;
  a.disp = c.disp;
  a.F = c.F32;
  a.inv_mass = c.inv_mass32;
  a.F9 = c.F9_32;
  a.v9 = c.v9_32;
  a.vh = c.vh;
  a.pml_ab = c.pml_ab32;
  a.nnode = c.nnode;
  a.n_int = c.n_int;
  a.npml = c.npml;
  a.n_split = c.n_split;
  a.npml_live = c.npml_live;
  a.dt = (float)c.sc.dt;
  a.dtd = c.sc.dt;
  a.d_nt = c.d_nt;
  a.d_err = c.d_err;
  a.vel32 = c.vel32;
  a.dl32 = c.dl32;
  a.rdampk = c.sc.rdampk;
  a.Fsplit = c.Fsplit;
  a.split_slot = c.split_slot;
  a.nsplit = 2 * c.npair;
  a.f_is_acc = c.f_is_acc;
  a.damp = c.sc.rdampk != 0.0;
  a.rdampk32 = (float)c.sc.rdampk;
  a.skip_split = 0;
  return a;
}

FaultArgs fault_args(Context &c) {
  FaultArgs p;
  p.npair = c.npair;
  p.nnode = c.nnode;
  p.nstep = c.nstep;
  p.nOnSt = c.nOnSt;
  p.nOffRows = c.nOffRows;
  p.nftmx_tp = c.npair;
  p.friclaw = c.sc.friclaw;
  p.TPV = c.sc.TPV;
  p.C_nuclea_here = (c.sc.C_nuclea == 1 && c.sc.nucfault == 1) ? 1 : 0;
  p.C_elastic = c.sc.C_elastic;
  p.insertFaultType = c.sc.insertFaultType;
  p.dt = c.sc.dt;
  p.nucR = c.sc.nucR;
  p.nucRuptVel = c.sc.nucRuptVel;
  p.nucdtau0 = c.sc.nucdtau0;
  p.nucT = c.sc.nucT;
  p.slipRateThres = c.sc.slipRateThres;
  p.fric_tp_h = c.sc.fric_tp_h;
  p.pair_s = c.pair_s;
  p.pair_m = c.pair_m;
  p.geo = c.pair_geo;
  p.fric = c.fric;
  p.fnft = c.fnft;
  p.tp_hist = c.tp_hist;
  p.onst = c.onst;
  p.onhist = c.onhist;
  p.off_rows = c.off_rows;
  p.offhist = c.offhist;
  p.F = c.fp32 ? nullptr : c.F;
  p.F32 = c.fp32 ? c.F32 : nullptr;
  p.Fsplit = c.Fsplit;
  p.vel = c.vel;
  p.disp = c.disp;
  p.d_nt = c.d_nt;
  p.d_times = c.d_times;
  p.stats = c.d_stats;
  p.mlp = static_cast<const MlpDevice *>(mlp_device_params(c));
  p.newton_log = c.nlog;
  p.log_nt0 = c.nlog_nt0;
  p.log_steps = c.nlog_steps;
  p.log_stride = c.nlog_stride;
  return p;
}

}  // namespace

int launch_node_update(Context &c, cudaStream_t s, bool skip_split) {
  const int bn = c.opt.block_node > 0 ? c.opt.block_node : kBlockNode;
  const int grid = (c.nnode + bn - 1) / bn;
#define EQD_NODE_ARGS c.vel, c.disp, c.F, c.inv_mass, c.F9, c.v9, c.vh, c.pml_ab, c.nnode, c.n_int, \
    c.npml, c.sc.dt, c.d_nt, c.d_err
  if (c.fp32) {
    NodeArgs32 a = node_args32(c);
    a.skip_split = skip_split ? 1 : 0;
    if (c.f_is_acc) {
      if (a.damp) node_update32<true, true><<<grid, bn, 0, s>>>(a);
      else node_update32<true, false><<<grid, bn, 0, s>>>(a);
    } else {
      if (a.damp) node_update32<false, true><<<grid, bn, 0, s>>>(a);
      else node_update32<false, false><<<grid, bn, 0, s>>>(a);
    }
  } else {
    if (c.f_is_acc) node_update<true><<<grid, bn, 0, s>>>(EQD_NODE_ARGS);
    else node_update<false><<<grid, bn, 0, s>>>(EQD_NODE_ARGS);
  }
#undef EQD_NODE_ARGS
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

namespace {
struct NodeFaultBatch {
  int n = 0;
  NodeArgs32 *d_node = nullptr;
  FaultArgs *d_fault = nullptr;
  int *d_node_start = nullptr, *d_fault_start = nullptr;  // [n + 1] block prefix sums
  int node_blocks = 0, fault_blocks = 0;
  int *d_node_start_tile = nullptr;  // [n + 1] prefix sums of blocks of kTile nodes (persistent kernel)
  int node_blocks_tile = 0;
  int max_friclaw = 0;
  std::vector<NodeArgs32> h_node;
  std::vector<FaultArgs> h_fault;
};
}  // namespace

int node_fault_batch_update(void **handle, Context *const *m, int n) {
  if (n <= 0) return EQD_ERR_INPUT;
  for (int i = 0; i < n; ++i)
    if (!m[i]->fp32 || (m[i]->sc.friclaw == 5 && m[i]->tp_hist)) return EQD_ERR_UNSUPPORTED;
  NodeFaultBatch *b = static_cast<NodeFaultBatch *>(*handle);
  if (!b) {
    b = new NodeFaultBatch();
    b->n = n;
    std::vector<int> ns(n + 1, 0), fs(n + 1, 0);
    for (int i = 0; i < n; ++i) {
      ns[i + 1] = ns[i] + (m[i]->nnode + kBlockNode - 1) / kBlockNode;
      const int nthreads = m[i]->npair + (m[i]->nOffRows > 0 ? m[i]->nOffRows + 1 : 0);
      fs[i + 1] = fs[i] + (nthreads + kBlockFault - 1) / kBlockFault;
    }
    b->node_blocks = ns[n];
    b->fault_blocks = fs[n];
    std::vector<int> nt(n + 1, 0);
    for (int i = 0; i < n; ++i) {
      nt[i + 1] = nt[i] + (m[i]->nnode + kTile - 1) / kTile;
      b->max_friclaw = std::max(b->max_friclaw, m[i]->sc.friclaw);
    }
    b->node_blocks_tile = nt[n];
    if (cudaMalloc(&b->d_node_start_tile, sizeof(int) * (n + 1)) != cudaSuccess) {
      node_fault_batch_free(b);
      return EQD_ERR_OOM;
    }
    cudaMemcpy(b->d_node_start_tile, nt.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice);
    if (cudaMalloc(&b->d_node, sizeof(NodeArgs32) * n) != cudaSuccess ||
        cudaMalloc(&b->d_fault, sizeof(FaultArgs) * n) != cudaSuccess ||
        cudaMalloc(&b->d_node_start, sizeof(int) * (n + 1)) != cudaSuccess ||
        cudaMalloc(&b->d_fault_start, sizeof(int) * (n + 1)) != cudaSuccess) {
      node_fault_batch_free(b);
      return EQD_ERR_OOM;
    }
    cudaMemcpy(b->d_node_start, ns.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(b->d_fault_start, fs.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice);
    b->h_node.resize(n);
    b->h_fault.resize(n);
    *handle = b;
  }
  if (b->n != n) return EQD_ERR_INPUT;
  for (int i = 0; i < n; ++i) {
    b->h_node[i] = node_args32(*m[i]);
    b->h_fault[i] = fault_args(*m[i]);
  }
  EQD_CUDA_OK(cudaMemcpy(b->d_node, b->h_node.data(), sizeof(NodeArgs32) * n, cudaMemcpyHostToDevice));
  EQD_CUDA_OK(cudaMemcpy(b->d_fault, b->h_fault.data(), sizeof(FaultArgs) * n, cudaMemcpyHostToDevice));
  return EQD_OK;
}

int launch_node_update_batched(const void *handle, cudaStream_t s) {
  const NodeFaultBatch *b = static_cast<const NodeFaultBatch *>(handle);
  if (b->node_blocks > 0) node_update32_batched<<<b->node_blocks, kBlockNode, 0, s>>>(b->d_node, b->d_node_start, b->n);
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

int launch_fault_batched(const void *handle, cudaStream_t s) {
  const NodeFaultBatch *b = static_cast<const NodeFaultBatch *>(handle);
  if (b->fault_blocks > 0) fault_kernel_batched<<<b->fault_blocks, kBlockFault, 0, s>>>(b->d_fault, b->d_fault_start, b->n);
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

void node_fault_batch_free(void *handle) {
  NodeFaultBatch *b = static_cast<NodeFaultBatch *>(handle);
  if (!b) return;
  if (b->d_node) cudaFree(b->d_node);
  if (b->d_fault) cudaFree(b->d_fault);
  if (b->d_node_start) cudaFree(b->d_node_start);
  if (b->d_fault_start) cudaFree(b->d_fault_start);
  if (b->d_node_start_tile) cudaFree(b->d_node_start_tile);
  delete b;
}

// ---- persistent ensemble step ------------------------------------------------------------------
// One cooperative launch advances every member by many steps: per step the node update of every
// member, then the interior and PML tiles of every member, then the fault pairs (and station rows)
// of every member, each phase split over the resident CTAs and closed by a grid-wide barrier.  The
// device bodies are those of the batched launches, so the arithmetic is the same.
namespace {

static_assert(kBlockFault == kTile, "fault blocks and tiles share the persistent CTA");
constexpr unsigned long long kGridWaitNs = 2000000000ull;  // a barrier wait gives up after 2 s
constexpr unsigned kGridWaitPolls = 1u << 26;             // or after this many polls

struct PersistentArgs {
  const NodeArgs32 *node;
  const int *node_start;      // [n + 1] prefix sums of blocks of kTile nodes
  int node_blocks;
  const ElemArgs32 *elem[2];  // interior, PML
  const int *elem_start[2];   // [n + 1] tile prefix sums
  int tiles[2];
  const FaultArgs *fault;
  const int *fault_start;     // [n + 1] prefix sums of blocks of kBlockFault pairs
  int fault_blocks;
  int n, nsteps;
  unsigned *bar;  // [0] arrivals, [1] generation; zero at launch
  int *err;       // bit 2 set when a barrier wait gave up
};

// Grid-wide barrier of a cooperative launch (all CTAs resident).  Thread 0 of each CTA arrives on
// the counter; the last one resets it and advances the generation the others wait for.  The wait is
// bounded in polls and in time: a CTA that gives up flags bit 2 of the error word and returns false,
// and every other CTA then gives up at a barrier too.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *err) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned *gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const unsigned long long t0 = globaltimer_ns();
      for (unsigned it = 0; *gen == g; ++it) {
        if (it >= kGridWaitPolls || ((it & 255u) == 255u && globaltimer_ns() - t0 > kGridWaitNs)) {
          atomicOr(err, 2);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

template <class T>
__device__ __forceinline__ void copy_args(T *dst, const T *src) {
  static_assert(sizeof(T) % 4 == 0, "argument block of whole words");
  const int *s = reinterpret_cast<const int *>(src);
  int *d = reinterpret_cast<int *>(dst);
  for (int q = threadIdx.x; q < (int)(sizeof(T) / 4); q += blockDim.x) d[q] = s[q];
}

// Slip- and time-weakening members only (the fault body without the Newton solve), no Q; every
// step but a member's first (stored acceleration).  At most 72 registers a thread: 7 CTAs of
// kTile threads per SM, as many as the element passes' shared memory allows.
template <bool BODY, bool PLASTIC, int HG, bool S0>
__global__ void __launch_bounds__(kTile, 7) ensemble_persistent(const __grid_constant__ PersistentArgs P) {
  __shared__ __align__(16) NodeArgs32 na;
  __shared__ __align__(16) ElemArgs32 ea;
  __shared__ __align__(16) FaultArgs fa;
  __shared__ int lb;
  for (int step = 0; step < P.nsteps; ++step) {
    for (int b = blockIdx.x; b < P.node_blocks; b += gridDim.x) {
      const int m = batch_member(P.node_start, P.n, b);
      copy_args(&na, P.node + m);
      if (threadIdx.x == 0) lb = b - P.node_start[m];
      __syncthreads();
      const int i = lb * kTile + threadIdx.x;
      if (na.damp) node_update32_body<false, true>(na, i);
      else node_update32_body<false, false>(na, i);
      __syncthreads();
    }
    if (!grid_barrier(P.bar, P.err)) return;
    for (int grp = 0; grp < 2; ++grp) {
      for (int b = blockIdx.x; b < P.tiles[grp]; b += gridDim.x) {
        const int m = elem_batch_member(P.elem_start[grp], P.n, b);
        copy_args(&ea, P.elem[grp] + m);
        __syncthreads();
        const int tile = b - P.elem_start[grp][m];
        if (grp == 0) {
          if (ea.g.nrec == 1) interior_rec_body<BODY, PLASTIC, HG, true, false>(ea, tile);
          else interior_rec_body<BODY, PLASTIC, HG, false, false>(ea, tile);
        } else {
          if (ea.g.nrec == 1) pml_rec_body<BODY, S0, HG, true>(ea, tile);
          else pml_rec_body<BODY, S0, HG, false>(ea, tile);
        }
        __syncthreads();  // the next tile's copies land in the same shared memory
      }
    }
    if (!grid_barrier(P.bar, P.err)) return;
    for (int b = blockIdx.x; b < P.fault_blocks; b += gridDim.x) {
      const int m = batch_member(P.fault_start, P.n, b);
      copy_args(&fa, P.fault + m);
      if (threadIdx.x == 0) lb = b - P.fault_start[m];
      __syncthreads();
      fault_body<true, false>(fa, lb * kTile + threadIdx.x, nullptr);
      __syncthreads();
    }
    if (!grid_barrier(P.bar, P.err)) return;
  }
}

template <bool BODY, bool PLASTIC, int HG, bool S0>
int launch_persistent_variant(const PersistentArgs &P, const int Mmax[2], cudaStream_t s) {
  auto kern = ensemble_persistent<BODY, PLASTIC, HG, S0>;
  const size_t sm = std::max(rec_smem<RecInterior<BODY, PLASTIC, HG, false>>(std::max(Mmax[0], 1)),
                             rec_smem<RecPml<BODY, S0, HG>>(std::max(Mmax[1], 1)));
  if (allow_smem(kern, sm)) return EQD_ERR_CUDA;
  int dev = 0, nsm = 0, per = 0;
  EQD_CUDA_OK(cudaGetDevice(&dev));
  EQD_CUDA_OK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  EQD_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kTile, sm));
  if (per <= 0) return EQD_ERR_UNSUPPORTED;
  const int work = std::max({P.node_blocks, P.tiles[0], P.tiles[1], P.fault_blocks, 1});
  const int grid = std::min(per * nsm, work);
  void *args[] = {const_cast<PersistentArgs *>(&P)};
  EQD_CUDA_OK(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(kern), dim3(grid), dim3(kTile), args, sm, s));
  return EQD_OK;
}

}  // namespace

int launch_ensemble_persistent(const void *nf, const void *eb, int nsteps, unsigned *bar, int *err,
                               cudaStream_t s) {
  const NodeFaultBatch *b = static_cast<const NodeFaultBatch *>(nf);
  if (!b || !eb || nsteps <= 0) return EQD_ERR_STATE;
  if (b->max_friclaw > 2) return EQD_ERR_UNSUPPORTED;
  PersistentArgs P{};
  const void *eargs[2];
  const int *estart[2];
  int tiles[2], Mmax[2], v[5];
  const int rc = elem_batch_tables(eb, eargs, estart, tiles, Mmax, v);
  if (rc) return rc;
  const bool body = v[0], plastic = v[1], s0 = v[2];
  const int hg = v[3];
  if (v[4] || (body != plastic)) return EQD_ERR_UNSUPPORTED;  // Q, or mass damping without plasticity
  P.node = b->d_node;
  P.node_start = b->d_node_start_tile;
  P.node_blocks = b->node_blocks_tile;
  for (int grp = 0; grp < 2; ++grp) {
    P.elem[grp] = static_cast<const ElemArgs32 *>(eargs[grp]);
    P.elem_start[grp] = estart[grp];
    P.tiles[grp] = tiles[grp];
  }
  P.fault = b->d_fault;
  P.fault_start = b->d_fault_start;
  P.fault_blocks = b->fault_blocks;
  P.n = b->n;
  P.nsteps = nsteps;
  P.bar = bar;
  P.err = err;
  EQD_CUDA_OK(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s));
  if (hg == 2) {
    if (plastic) return s0 ? launch_persistent_variant<true, true, 2, true>(P, Mmax, s)
                           : launch_persistent_variant<true, true, 2, false>(P, Mmax, s);
    return s0 ? launch_persistent_variant<false, false, 2, true>(P, Mmax, s)
              : launch_persistent_variant<false, false, 2, false>(P, Mmax, s);
  }
  if (plastic) return s0 ? launch_persistent_variant<true, true, 1, true>(P, Mmax, s)
                         : launch_persistent_variant<true, true, 1, false>(P, Mmax, s);
  return s0 ? launch_persistent_variant<false, false, 1, true>(P, Mmax, s)
            : launch_persistent_variant<false, false, 1, false>(P, Mmax, s);
}

namespace {
struct OutputArgs {
  const double *vel, *fric;
  const int *surf, *d_nt;
  double *frames;
  int *count;
  int nnode, npair, nsurf, every, ring;
};

// output_gm + output_src_evol (src/library_output.f90:267-312) of step nt when
// (nt - 1) % every == 0 (src/driver.f90:30: mod(nt, 10) == 1): frame (nt - 1) / every of the ring
// gets the velocity of every surface node and fric(47) of every pair.
// part 1: the surface velocities, part 2: fric(47), 3: both
__global__ void __launch_bounds__(256) output_capture_kernel(OutputArgs o, int part) {
  const int nt = *o.d_nt;
  if (nt < 1 || (nt - 1) % o.every != 0) return;
  const int f = (nt - 1) / o.every;
  const size_t len = 3 * (size_t)o.nsurf + o.npair;
  double *fr = o.frames + (size_t)(f % o.ring) * len;
  const int t = blockIdx.x * blockDim.x + threadIdx.x + ((part & 1) ? 0 : o.nsurf);
  if (t < o.nsurf) {
    const int d = o.surf[t];
#pragma unroll
    for (int c = 0; c < 3; ++c) fr[3 * t + c] = o.vel[(size_t)c * o.nnode + d];
  } else if (t < o.nsurf + o.npair) {
    const int i = t - o.nsurf;
    fr[3 * (size_t)o.nsurf + i] = o.fric[46 * (size_t)o.npair + i];
  }
  if (t == 0) atomicMax(o.count, f + 1);
}
}  // namespace

int launch_output_capture(Context &c, cudaStream_t s, int part, bool overlapped) {
  if (!c.out_frames) return EQD_OK;
  // the fault-side part of the overlapped schedule runs beside the next step's node update
  const OutputArgs o{c.vel, c.fric, c.out_surf, (overlapped && part == 2) ? c.d_nt_c : c.d_nt, c.out_frames,
                     c.out_count, c.nnode, c.npair, c.out_nsurf, c.out_every, c.out_ring};
  const int n = ((part & 1) ? c.out_nsurf : 0) + ((part & 2) ? c.npair : 0);
  if (n > 0) output_capture_kernel<<<(n + 255) / 256, 256, 0, s>>>(o, part);
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

namespace {
// Split nodes of the overlapped schedule (after the fault kernel of the previous step and the bulk
// node update of this one): slot q of Fsplit is the slave (even q) or master (odd q) of pair q / 2.
// Thread 0 also publishes the step number to d_nt_c for the fault phase of this step.
template <bool F_IS_ACC>
__global__ void __launch_bounds__(256) split_update32(NodeArgs32 a, const int *__restrict__ pair_s,
                                                     const int *__restrict__ pair_m, int npair, int *d_nt_c) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q == 0) *d_nt_c = *a.d_nt;
  if (q >= 2 * npair) return;
  split_node_update<F_IS_ACC>(a, (q & 1) ? pair_m[q >> 1] : pair_s[q >> 1], q);
}

// Off-fault station rows (storeOffFaultStData, src/driver.f90:157-180) of the overlapped schedule:
// taken after every node of the step is updated, before the element kernels.
__global__ void __launch_bounds__(128) station_capture_kernel(FaultArgs p) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = *p.d_nt;
  if (r > p.nOffRows || nt < 1 || nt > p.nstep || !p.offhist) return;
  double val = p.d_times[nt];
  if (r > 0) {
    const int node = p.off_rows[r - 1], comp = p.off_rows[p.nOffRows + r - 1];
    const int type = p.off_rows[2 * p.nOffRows + r - 1];
    val = (type == 1) ? p.disp[comp * p.nnode + node] : p.vel[comp * p.nnode + node];
  }
  p.offhist[(size_t)(p.nOffRows + 1) * (nt - 1) + r] = val;
}
}  // namespace

int launch_split_update(Context &c, cudaStream_t s) {
  const NodeArgs32 a = node_args32(c);
  const int n = std::max(2 * c.npair, 1);
  if (c.f_is_acc) split_update32<true><<<(n + 255) / 256, 256, 0, s>>>(a, c.pair_s, c.pair_m, c.npair, c.d_nt_c);
  else split_update32<false><<<(n + 255) / 256, 256, 0, s>>>(a, c.pair_s, c.pair_m, c.npair, c.d_nt_c);
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

int launch_station_capture(Context &c, cudaStream_t s) {
  if (c.nOffRows <= 0 || !c.offhist) return EQD_OK;
  const FaultArgs p = fault_args(c);
  station_capture_kernel<<<(c.nOffRows + 1 + 127) / 128, 128, 0, s>>>(p);
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

int launch_fault(Context &c, cudaStream_t s, bool overlapped) {
  // overlapped schedule: the off-fault station rows are taken by station_capture_kernel, and the
  // step number comes from d_nt_c (the bulk node update of the next step may already count it)
  const int nthreads = c.npair + (!overlapped && c.nOffRows > 0 ? c.nOffRows + 1 : 0);
  if (nthreads == 0) return EQD_OK;
  FaultArgs p = fault_args(c);
  if (overlapped) {
    p.d_nt = c.d_nt_c;
    p.offhist = nullptr;  // the last block's spare threads must not take station rows either
  }
  if (p.friclaw == 5 && p.tp_hist)
    thermop_kernel<<<(c.npair + 31) / 32, 32 * kTpWarps, 0, s>>>(p);
  const int bf = c.opt.block_fault > 0 ? c.opt.block_fault : kBlockFault;
  const int grid = (nthreads + bf - 1) / bf;
  if (overlapped) {
    // beside the PML pass: the launch carries the highest priority itself, so that a captured
    // graph node keeps it (a graph does not take the priority of the capturing stream).  (One
    // single-warp CTA per SM, which fits beside a full complement of PML CTAs, was slower: each
    // warp's 20-iteration binary64 solves are latency-bound, and six rounds of them outlast the
    // PML pass, 2.61 -> 3.05 ms per C1 step.)
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = hi;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(bf);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = c.fp32 ? cudaLaunchKernelEx(&cfg, fault_kernel<true>, p)
                                 : cudaLaunchKernelEx(&cfg, fault_kernel<false>, p);
    return e == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
  }
  if (c.fp32) fault_kernel<true><<<grid, bf, 0, s>>>(p);
  else fault_kernel<false><<<grid, bf, 0, s>>>(p);
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// widen_f32 / narrow_f64 against the hardware conversions: every binary32 pattern class (random
// bits), and binary64 values with exponents 880..1160 (around and inside the binary32 normal range)
// whose dropped 29 fraction bits are random, exactly half (ties), just below and just above half,
// or whose kept 23 bits are all ones (carry into the exponent).
__global__ void fpconv_check_kernel(long long n, unsigned long long seed, unsigned long long *bad) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const unsigned long long h = mix64(seed ^ (unsigned long long)k);
    const float f = __uint_as_float((unsigned)h);
    const double w1 = widen_f32(f), w2 = (double)f;
    const bool okw = __double_as_longlong(w1) == __double_as_longlong(w2) || (isnan(w1) && isnan(w2));
    const unsigned long long g = mix64(h);
    // exponents around and inside the binary32 range; one draw in four anywhere (0 .. 2047)
    const unsigned long long e = ((g >> 40) & 3ull) == 0ull ? g % 2048ull : 880ull + g % 281ull;
    unsigned long long frac = mix64(g) & ((1ull << 52) - 1ull);
    const unsigned long long low = 0x1fffffffull;
    switch (k & 7) {
      case 1: frac = (frac & ~low) | 0x10000000ull; break;
      case 2: frac = (frac & ~low) | 0x0fffffffull; break;
      case 3: frac = (frac & ~low) | 0x10000001ull; break;
      case 4: frac |= ~low & ((1ull << 52) - 1ull); break;
      case 5: frac = (frac | (~low & ((1ull << 52) - 1ull)) & ~low) | 0x10000000ull; break;
      default: break;
    }
    const double d = __longlong_as_double((long long)(((h >> 63) << 63) | (e << 52) | frac));
    const float n1 = narrow_f64(d), n2 = (float)d;
    const bool okn = __float_as_uint(n1) == __float_as_uint(n2) || (isnan(n1) && isnan(n2));
    if (!okw) atomicAdd(bad, 1ull);
    if (!okn) atomicAdd(bad + 1, 1ull);
  }
}

}  // namespace

}  // namespace eqd

namespace eqd {
namespace {
// Self-tests of the bounded waits: a completion that never comes must make the wait give up and
// flag bit 2 of the error word, not hang.
__global__ void wait_selftest_mbar(int *err) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_expect_tx(&bar, 16u);  // 16 bytes that no copy delivers
  }
  __syncthreads();
  mbar_wait_bounded(&bar, err);
}
__global__ void wait_selftest_grid(unsigned *bar, int *err) {
  if (blockIdx.x == 1) return;  // this CTA leaves without arriving at the barrier
  grid_barrier(bar, err);
}
}  // namespace
}  // namespace eqd

extern "C" int eqd_gpu_wait_selftest(int32_t device, int32_t which, int32_t *status, double *ms) {
  using namespace eqd;
  if (!status || (which != 0 && which != 1)) return EQD_ERR_INPUT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return EQD_ERR_NO_DEVICE;
  }
  EQD_CUDA_OK(cudaSetDevice(device));
  if (which == 1) {
    int coop = 0;
    EQD_CUDA_OK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
    if (!coop) return EQD_ERR_UNSUPPORTED;
  }
  int *err = nullptr;
  unsigned *bar = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = EQD_OK;
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess || cudaMalloc(&bar, 2 * sizeof(unsigned)) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    rc = EQD_ERR_OOM;
  }
  if (!rc) {
    cudaMemset(err, 0, sizeof(int));
    cudaMemset(bar, 0, 2 * sizeof(unsigned));
    cudaEventRecord(e0);
    if (which == 0) {
      wait_selftest_mbar<<<1, 32>>>(err);
    } else {
      void *args[] = {&bar, &err};
      if (cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(wait_selftest_grid), dim3(2), dim3(32), args, 0,
                                      nullptr) != cudaSuccess)
        rc = EQD_ERR_CUDA;
    }
    cudaEventRecord(e1);
    int h = 0;
    if (!rc && (cudaEventSynchronize(e1) != cudaSuccess ||
                cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess))
      rc = EQD_ERR_CUDA;
    float t = 0.f;
    if (!rc) cudaEventElapsedTime(&t, e0, e1);
    if (ms) *ms = t;
    *status = (h & 2) ? EQD_ERR_TIMEOUT : EQD_OK;
  }
  if (err) cudaFree(err);
  if (bar) cudaFree(bar);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return rc;
}

extern "C" int eqd_gpu_check_conversions(int32_t device, int64_t n, uint64_t seed, int64_t mismatches[2]) {
  using namespace eqd;
  if (n <= 0 || !mismatches) return EQD_ERR_INPUT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return EQD_ERR_NO_DEVICE;
  }
  EQD_CUDA_OK(cudaSetDevice(device));
  unsigned long long *bad = nullptr;
  if (cudaMalloc(reinterpret_cast<void **>(&bad), 2 * sizeof(unsigned long long)) != cudaSuccess) return EQD_ERR_OOM;
  int rc = EQD_OK;
  unsigned long long hb[2] = {0, 0};
  cudaMemset(bad, 0, sizeof(hb));
  fpconv_check_kernel<<<4 * 152, 256>>>(n, seed, bad);
  if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = EQD_ERR_CUDA;
  cudaFree(bad);
  mismatches[0] = (int64_t)hb[0];
  mismatches[1] = (int64_t)hb[1];
  return rc;
}
