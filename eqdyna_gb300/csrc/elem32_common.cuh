// Shared parts of the binary32 element kernels (kernels_elem32.cu: per-element tables streamed by
// bulk copy; kernels_elem32r.cu: record-indexed tables).
//
// Both layouts run one CTA per tile of 128 consecutive elements of a brick-ordered element list.
// The element math below is written once against a table "source" S that answers
//   S.g(row)  geometry / material value of the element, rows numbered as in TabCommon
//   S.em(a)   lumped corner mass,   S.str(i) stress component,   S.por() pore pressure
//   S.st0(i)  PML initial stress,   S.pa(k), S.pb(k)  PML factors a_k, b_k
// and is that of the binary64 kernels (src/calcElemKU.f90, src/hrglss.f90,
// src/assembleGlobalKU.f90:70-346) in binary32.
#pragma once
#include "eqd_device.cuh"

namespace eqd {
namespace e32 {

constexpr int kTile = 128;                          // elements per tile = CTA size
constexpr unsigned kWaitLimit = 1u << 22;           // polls of one bounded wait
constexpr unsigned long long kWaitNs = 100000000ull;  // and at most 100 ms

struct ElemConst32 {
  float dt, rdampk, rdampm, gz, ccosphi, sinphi, relax;
};

__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// Kahan step on two independent sums at once with the packed binary32 pair instructions of sm_100
// and later (__fadd2_rn / __ffma2_rn: two lanes per issued instruction, each lane rounded as the
// scalar operation).  fma(a, -1, b) is b - a rounded once, so every lane is bit for bit kahan_add.
__device__ __forceinline__ void kahan_add2(float2 &s, float2 &c, float2 x) {
  const float2 m1 = make_float2(-1.f, -1.f);
  const float2 y = __ffma2_rn(c, m1, x);                // x - c
  const float2 t = __fadd2_rn(s, y);                    // s + y
  c = __ffma2_rn(y, m1, __ffma2_rn(s, m1, t));          // (t - s) - y
  s = t;
}

__device__ __forceinline__ float viscous_pattern_f(int m, int a) {
  const unsigned neg[4] = {0x3Cu, 0x96u, 0xAAu, 0x5Au};
  return ((neg[m] >> a) & 1u) ? -1.0f : 1.0f;
}

// ---- mbarrier and bulk-copy primitives --------------------------------------------------------
__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
// global -> shared bulk copy completing `bytes` of transaction count on `bar`; both addresses
// 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for phase 0 for at most kWaitLimit polls and kWaitNs nanoseconds.
__device__ __forceinline__ bool mbar_wait_for(unsigned long long *bar) {
  const unsigned long long t0 = globaltimer_ns();
  for (unsigned it = 0; it < kWaitLimit; ++it) {
    if (mbar_try_wait(bar, 0)) return true;
    if ((it & 63u) == 63u && globaltimer_ns() - t0 > kWaitNs) break;
  }
  return false;
}
// Bounded wait for the tile's copies.  On timeout: flag bit 2 of the error word, wait once more
// (bounded) so no copy is still writing into shared memory when the CTA exits, report failure.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, int *err) {
  if (mbar_wait_for(bar)) return true;
  atomicOr(err, 2);
  mbar_wait_for(bar);
  return false;
}

// Issues one 512-byte bulk copy per table row: rows row..row+n-1 of the slab <- chunk e0 of the
// component-major table src (row stride ld, a multiple of kTile).
__device__ __forceinline__ void copy_rows(float *tab, int row, const void *src, int n, int ld, int e0,
                                          unsigned long long *bar) {
  const float *s = static_cast<const float *>(src);
  for (int k = 0; k < n; ++k) bulk_g2s(tab + (row + k) * kTile, s + (size_t)k * ld + e0, kTile * 4, bar);
}

// Row offsets shared by both layouts: the geometry / material part of an element's table
// (record-indexed layout: the record itself).
template <int HG>
struct TabCommon {
  static constexpr int SHP = 0;                          // 24 shape-function gradients (3 a + k)
  static constexpr int PHI = 24;                         // 32 hourglass vectors (8 m + a), KF78
  static constexpr int SS = PHI + (HG == 1 ? 32 : 0);    // 6 hourglass stiffness, KF78
  static constexpr int HGC = SS + (HG == 1 ? 6 : 0);     // 1 viscous hourglass coefficient
  static constexpr int DET = HGC + (HG == 2 ? 1 : 0);    // det * weight
  static constexpr int LAM = DET + 1;
  static constexpr int MU = LAM + 1;
  static constexpr int STR = MU + 1;
};

// Shared memory of a tile after its per-element rows: the incidence list, the slot table, the
// staged node data, the tile's incidence pointers and (optionally) its node ids.
struct TileSmem {
  unsigned short *sinc;     // [8 * kTile] incidences (corner * kTile + element), node-major
  unsigned short *slot_of;  // [8 * kTile] local node of (corner, element), layout slot_index
  float *sv, *sd;           // [3][Mmax] binary32 velocity and u + rdampk v of the tile's nodes
  unsigned short *sincp;    // [Mmax + 1] first incidence of each tile node
  int *sids;                // [Mmax] global node ids, or null (read again from the tile list)
};
// slot_over: where slot_of lives when it overlays rows of the tile (null: its own 2 KB)
__device__ __forceinline__ TileSmem tile_smem(float *rows_end, int Mmax, bool ids,
                                              unsigned short *slot_over = nullptr) {
  TileSmem t;
  t.sinc = reinterpret_cast<unsigned short *>(rows_end);
  t.slot_of = slot_over ? slot_over : t.sinc + 8 * kTile;
  t.sv = reinterpret_cast<float *>(t.sinc + (slot_over ? 8 : 16) * kTile);
  t.sd = t.sv + 3 * Mmax;
  t.sids = ids ? reinterpret_cast<int *>(t.sd + 3 * Mmax) : nullptr;
  t.sincp = reinterpret_cast<unsigned short *>(t.sd + 3 * Mmax + (ids ? Mmax : 0));
  return t;
}
inline size_t tile_smem_bytes(int Mmax, bool ids, bool slot_over = false) {
  return (slot_over ? 1 : 2) * (8 * kTile * 2) + 6 * (size_t)Mmax * 4 + (ids ? 4 * (size_t)Mmax : 0) +
         (((size_t)Mmax + 2) & ~(size_t)1) * 2;
}

// Slot table layout: the two 16-bit entries of corners 2k and 2k + 1 of element e share one 32-bit
// word at word k * kTile + e, so that the table is four rows of kTile words whose column e belongs
// to element e alone (it can overlay rows of per-element data).
__host__ __device__ __forceinline__ int slot_index(int r) {  // r = corner * kTile + element
  const int a = r / kTile, e = r - a * kTile;
  return (a >> 1) * (2 * kTile) + 2 * e + (a & 1);
}

// The local node of each corner of this thread's element (garbage for an empty slot, unused).
__device__ __forceinline__ void load_slots(const unsigned short *slot_of, int tid, int (&sl)[8]) {
  const unsigned *w = reinterpret_cast<const unsigned *>(slot_of);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const unsigned v = w[k * kTile + tid];
    sl[2 * k] = (int)(v & 0xffffu);
    sl[2 * k + 1] = (int)(v >> 16);
  }
}

// slot_of from the staged incidence list (node j of the tile owns incidences incp[j] .. incp[j+1]).
__device__ __forceinline__ void build_slots(const unsigned short *incp, int M, const unsigned short *sinc,
                                            unsigned short *slot_of) {
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    const int q1 = incp[j + 1];
    for (int q = incp[j]; q < q1; ++q) slot_of[slot_index(sinc[q])] = (unsigned short)j;
  }
}

// Stages tile t: the binary32 node data, the incidence pointers and (optionally) the node ids
// into shared memory, all loads of a node issued together; returns the tile's node count.
__device__ __forceinline__ int stage_nodes(const ElemGroup<float> &g, int t, const float *__restrict__ vel32,
                                           const float *__restrict__ dl32, int nnode, int Mmax,
                                           const TileSmem &ts, int &nb) {
  nb = g.tile_node_ptr[t];
  const int M = g.tile_node_ptr[t + 1] - nb;
  const unsigned short *__restrict__ incp = g.tile_incp + g.tile_incp_off[t];
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    const int n = g.tile_nodes[nb + j];
    ts.sincp[j] = incp[j];
    if (ts.sids) ts.sids[j] = n;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      ts.sv[c * Mmax + j] = vel32[c * nnode + n];
      ts.sd[c * Mmax + j] = dl32[c * nnode + n];
    }
  }
  if (threadIdx.x == 0) ts.sincp[M] = incp[M];
  return M;
}

// ---- element math ------------------------------------------------------------------------------
// Interior element (types 1, 11-13): stress update, optional Drucker-Prager return, stiffness +
// Rayleigh + hourglass + body forces per corner into fs[(c * 8 + a) * kTile + tid].  fs may
// overlay the hourglass-vector rows of S: each corner's rows are written only after they were read.
// QM: coarse-grained Q (src/calcElemKU.f90:77-132): the stress follows from the strain of the
// displacement u = (u + rdampk v) - rdampk v and the 6 memory variables (stress rows 6-11), with
// the element's constants S.q(0..4) = exp(-dt / tau_k), mu c_s, (lambda + 2 mu) c_v, 8 w_kp, 8 w_ks.
template <bool BODY, bool PLASTIC, int HG, bool QM, class Src>
__device__ __forceinline__ void interior_element(const Src &S, const float *sv, const float *sd, int Mmax,
                                                 const int (&sl_in)[8], int tid,
                                                 const ElemConst32 &k, double *pstrain_e,
                                                 float *stress_e, size_t ld, float *fs) {
  using C = TabCommon<HG>;
  float sr[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  float sn[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // strain (QM only)
  float ph[4][3];
#pragma unroll
  for (int m = 0; m < 4; ++m) ph[m][0] = ph[m][1] = ph[m][2] = 0.f;
  int sl[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    sl[a] = sl_in[a];
    const float bx = S.g(C::SHP + 3 * a), by = S.g(C::SHP + 3 * a + 1), bz = S.g(C::SHP + 3 * a + 2);
    const float vx = sv[sl[a]], vy = sv[Mmax + sl[a]], vz = sv[2 * Mmax + sl[a]];
    sr[0] = fmaf(bx, vx, sr[0]);
    sr[1] = fmaf(by, vy, sr[1]);
    sr[2] = fmaf(bz, vz, sr[2]);
    sr[3] = fmaf(by, vz, fmaf(bz, vy, sr[3]));
    sr[4] = fmaf(bx, vz, fmaf(bz, vx, sr[4]));
    sr[5] = fmaf(bx, vy, fmaf(by, vx, sr[5]));
    if constexpr (QM) {
      const float ux = fmaf(-k.rdampk, vx, sd[sl[a]]), uy = fmaf(-k.rdampk, vy, sd[Mmax + sl[a]]);
      const float uz = fmaf(-k.rdampk, vz, sd[2 * Mmax + sl[a]]);
      sn[0] = fmaf(bx, ux, sn[0]);
      sn[1] = fmaf(by, uy, sn[1]);
      sn[2] = fmaf(bz, uz, sn[2]);
      sn[3] = fmaf(by, uz, fmaf(bz, uy, sn[3]));
      sn[4] = fmaf(bx, uz, fmaf(bz, ux, sn[4]));
      sn[5] = fmaf(bx, uy, fmaf(by, ux, sn[5]));
    }
    if (HG == 1) {
      const float lx = sd[sl[a]], ly = sd[Mmax + sl[a]], lz = sd[2 * Mmax + sl[a]];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float p = S.g(C::PHI + 8 * m + a);
        ph[m][0] = fmaf(p, lx, ph[m][0]);
        ph[m][1] = fmaf(p, ly, ph[m][1]);
        ph[m][2] = fmaf(p, lz, ph[m][2]);
      }
    } else {
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float s = viscous_pattern_f(m, a);
        ph[m][0] = fmaf(s, vx, ph[m][0]);
        ph[m][1] = fmaf(s, vy, ph[m][1]);
        ph[m][2] = fmaf(s, vz, ph[m][2]);
      }
    }
  }
  const float lam = S.g(C::LAM), mu = S.g(C::MU), cd = lam + 2.0f * mu;
  const float srate[6] = {cd * sr[0] + lam * sr[1] + lam * sr[2], lam * sr[0] + cd * sr[1] + lam * sr[2],
                          lam * sr[0] + lam * sr[1] + cd * sr[2], mu * sr[3], mu * sr[4], mu * sr[5]};
  float s[6];
  if constexpr (!QM) {
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] = fmaf(srate[i], k.dt, S.str(i));
  } else {
    const float ex = S.q(0), miuu = S.q(1), Mu = S.q(2), wkp = S.q(3), wks = S.q(4);
    const float vols = sn[0] + sn[1] + sn[2];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const float a1 = S.str(6 + i);
      const float drive = (i < 3) ? 2.f * miuu * sn[i] * wks + (Mu * wkp - 2.f * miuu * wks) * vols
                                  : miuu * sn[i] * wks;
      const float an = ex * a1 + (1.f - ex) * drive;
      stress_e[(6 + i) * ld] = an;
      s[i] = (i < 3) ? 2.f * miuu * sn[i] + (Mu - 2.f * miuu) * vols - 0.5f * (an + a1)
                     : miuu * sn[i] - 0.5f * (an + a1);
    }
  }
  if (PLASTIC) {
    const float strmea = (s[0] + s[1] + s[2]) / 3.0f;
    const float dev[6] = {s[0] - strmea, s[1] - strmea, s[2] - strmea, s[3], s[4], s[5]};
    const float taomax = sqrtf(0.5f * (dev[0] * dev[0] + dev[1] * dev[1] + dev[2] * dev[2]) +
                               dev[3] * dev[3] + dev[4] * dev[4] + dev[5] * dev[5]);
    float yield = k.ccosphi - k.sinphi * (strmea + S.por());
    if (yield < 0.f) yield = 0.f;
    if (taomax > yield) {
      const float r = yield / taomax + (1.f - yield / taomax) * k.relax;
      float pinc[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const float v = dev[i] * r;
        pinc[i] = (dev[i] - v) / mu;
        s[i] = (i < 3) ? v + strmea : v;
      }
      const float pm = (pinc[0] + pinc[1] + pinc[2]) / 3.0f;
      float mag = 0.f;
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const float q = pinc[i] - pm;
        mag += (i < 3 ? 0.5f : 1.0f) * q * q;
      }
      *pstrain_e += (double)sqrtf(mag);
    }
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) stress_e[i * ld] = s[i];
  const float tw = -S.g(C::DET);
  float st[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) st[i] = tw * fmaf(k.rdampk, srate[i], s[i]);
  float h[4][3];
  if (HG == 1) {
    const float s1 = S.g(C::SS), s2 = S.g(C::SS + 1), s3 = S.g(C::SS + 2);
    const float s4 = S.g(C::SS + 3), s5 = S.g(C::SS + 4), s6 = S.g(C::SS + 5);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      h[m][0] = s1 * ph[m][0] + s2 * ph[m][1] + s3 * ph[m][2];
      h[m][1] = s2 * ph[m][0] + s4 * ph[m][1] + s5 * ph[m][2];
      h[m][2] = s3 * ph[m][0] + s5 * ph[m][1] + s6 * ph[m][2];
    }
  } else {
    const float coef = S.g(C::HGC);
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int c = 0; c < 3; ++c) h[m][c] = coef * ph[m][c];
  }
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const float bx = S.g(C::SHP + 3 * a), by = S.g(C::SHP + 3 * a + 1), bz = S.g(C::SHP + 3 * a + 2);
    float f0 = bx * st[0] + bz * st[4] + by * st[5];
    float f1 = by * st[1] + bz * st[3] + bx * st[5];
    float f2 = bz * st[2] + by * st[3] + bx * st[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const float p = (HG == 1) ? S.g(C::PHI + 8 * m + a) : viscous_pattern_f(m, a);
      f0 = fmaf(-p, h[m][0], f0);
      f1 = fmaf(-p, h[m][1], f1);
      f2 = fmaf(-p, h[m][2], f2);
    }
    if (BODY) {
      const float em = S.em(a);
      f0 -= em * (k.rdampm * sv[sl[a]]);
      f1 -= em * (k.rdampm * sv[Mmax + sl[a]]);
      f2 -= em * (k.rdampm * sv[2 * Mmax + sl[a]] + k.gz);
    }
    fs[(0 * 8 + a) * kTile + tid] = f0;
    fs[(1 * 8 + a) * kTile + tid] = f1;
    fs[(2 * 8 + a) * kTile + tid] = f2;
  }
}

// Interior gather: one thread per tile node, Kahan-compensated sums of its incidences in a fixed
// order, one binary32 L2 reduction per component.  The x and y sums run as one packed pair.
__device__ __forceinline__ void interior_gather(const ElemGroup<float> &g, int M, int nb,
                                                const unsigned short *incp, const unsigned short *sinc,
                                                const float *fs, float *__restrict__ F, int nnode,
                                                const int *sids) {
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    // the node id is loaded first: its latency runs under the sums
    const int n = sids ? sids[j] : __ldg(g.tile_nodes + nb + j);
    float2 hxy = make_float2(0.f, 0.f), lxy = make_float2(0.f, 0.f);
    float hz = 0.f, lz = 0.f;
    const int q1 = incp[j + 1];
    for (int q = incp[j]; q < q1; ++q) {
      const int r = sinc[q];  // corner * kTile + local element
      const int a = r / kTile, el = r - a * kTile;
      kahan_add2(hxy, lxy, make_float2(fs[(0 * 8 + a) * kTile + el], fs[(1 * 8 + a) * kTile + el]));
      kahan_add(hz, lz, fs[(2 * 8 + a) * kTile + el]);
    }
    atomicAdd(F + n, hxy.x - lxy.x);
    atomicAdd(F + (size_t)nnode + n, hxy.y - lxy.y);
    atomicAdd(F + 2 * (size_t)nnode + n, hz - lz);
  }
}

// PML element (type 2): split-field stress update (15 components) into es (6 sums per element,
// es[r * kTile + tid]) and s0 + hourglass + body force per corner into cfh.  es may overlay the
// stress rows of S (read first), cfh the hourglass-vector rows (as fs above).
template <bool BODY, bool S0, int HG, class Src>
__device__ __forceinline__ void pml_element(const Src &S, const float *sv, const float *sd, int Mmax,
                                            const int (&sl_in)[8], int tid, const ElemConst32 &k,
                                            float *stress_e, size_t ld, float *es, float *cfh) {
  using C = TabCommon<HG>;
  float D[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i) D[i][0] = D[i][1] = D[i][2] = 0.f;
  float ph[4][3];
#pragma unroll
  for (int m = 0; m < 4; ++m) ph[m][0] = ph[m][1] = ph[m][2] = 0.f;
  int sl[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    sl[a] = sl_in[a];
    const float b[3] = {S.g(C::SHP + 3 * a), S.g(C::SHP + 3 * a + 1), S.g(C::SHP + 3 * a + 2)};
    const float v[3] = {sv[sl[a]], sv[Mmax + sl[a]], sv[2 * Mmax + sl[a]]};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) D[i][j] = fmaf(b[i], v[j], D[i][j]);
    if (HG == 1) {
      const float l[3] = {sd[sl[a]], sd[Mmax + sl[a]], sd[2 * Mmax + sl[a]]};
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float p = S.g(C::PHI + 8 * m + a);
#pragma unroll
        for (int c = 0; c < 3; ++c) ph[m][c] = fmaf(p, l[c], ph[m][c]);
      }
    } else {
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float s = viscous_pattern_f(m, a);
#pragma unroll
        for (int c = 0; c < 3; ++c) ph[m][c] = fmaf(s, v[c], ph[m][c]);
      }
    }
  }
  const float lam = S.g(C::LAM), mu = S.g(C::MU), cd = lam + 2.0f * mu;
  const float src[15] = {cd * D[0][0], lam * D[1][1], lam * D[2][2], lam * D[0][0], cd * D[1][1],
                         lam * D[2][2], lam * D[0][0], lam * D[1][1], cd * D[2][2], mu * D[0][1],
                         mu * D[1][0], mu * D[0][2], mu * D[2][0], mu * D[1][2], mu * D[2][1]};
  const int axis[15] = {0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 0, 2, 1, 2};
  const float pa[3] = {S.pa(0), S.pa(1), S.pa(2)}, pb[3] = {S.pb(0), S.pb(1), S.pb(2)};
  float sp[15];
#pragma unroll
  for (int i = 0; i < 15; ++i) {
    sp[i] = fmaf(pa[axis[i]], S.str(i), src[i]) * pb[axis[i]];
    stress_e[i * ld] = sp[i];
  }
  es[0 * kTile + tid] = sp[0] + sp[1] + sp[2];
  es[1 * kTile + tid] = sp[3] + sp[4] + sp[5];
  es[2 * kTile + tid] = sp[6] + sp[7] + sp[8];
  es[3 * kTile + tid] = sp[9] + sp[10];
  es[4 * kTile + tid] = sp[11] + sp[12];
  es[5 * kTile + tid] = sp[13] + sp[14];
  const float sr[6] = {D[0][0], D[1][1], D[2][2], D[2][1] + D[1][2], D[2][0] + D[0][2], D[1][0] + D[0][1]};
  float s0[6] = {k.rdampk * (cd * sr[0] + lam * sr[1] + lam * sr[2]),
                 k.rdampk * (lam * sr[0] + cd * sr[1] + lam * sr[2]),
                 k.rdampk * (lam * sr[0] + lam * sr[1] + cd * sr[2]), k.rdampk * (mu * sr[3]),
                 k.rdampk * (mu * sr[4]), k.rdampk * (mu * sr[5])};
  if (S0) {
#pragma unroll
    for (int i = 0; i < 6; ++i) s0[i] += S.st0(i);
  }
  float h[4][3];
  if (HG == 1) {
    const float s1 = S.g(C::SS), s2 = S.g(C::SS + 1), s3 = S.g(C::SS + 2);
    const float s4 = S.g(C::SS + 3), s5 = S.g(C::SS + 4), s6 = S.g(C::SS + 5);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      h[m][0] = s1 * ph[m][0] + s2 * ph[m][1] + s3 * ph[m][2];
      h[m][1] = s2 * ph[m][0] + s4 * ph[m][1] + s5 * ph[m][2];
      h[m][2] = s3 * ph[m][0] + s5 * ph[m][1] + s6 * ph[m][2];
    }
  } else {
    const float coef = S.g(C::HGC);
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int c = 0; c < 3; ++c) h[m][c] = coef * ph[m][c];
  }
  const float dw = S.g(C::DET);
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const float wx = dw * S.g(C::SHP + 3 * a), wy = dw * S.g(C::SHP + 3 * a + 1);
    const float wz = dw * S.g(C::SHP + 3 * a + 2);
    float fh[3] = {-(wx * s0[0] + wz * s0[4] + wy * s0[5]), -(wy * s0[1] + wz * s0[3] + wx * s0[5]),
                   -(wz * s0[2] + wy * s0[3] + wx * s0[4])};
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const float p = (HG == 1) ? S.g(C::PHI + 8 * m + a) : viscous_pattern_f(m, a);
#pragma unroll
      for (int c = 0; c < 3; ++c) fh[c] = fmaf(-p, h[m][c], fh[c]);
    }
    if (BODY) {
      const float em = S.em(a);
      fh[0] -= em * (k.rdampm * sv[sl[a]]);
      fh[1] -= em * (k.rdampm * sv[Mmax + sl[a]]);
      fh[2] -= em * (k.rdampm * sv[2 * Mmax + sl[a]] + k.gz);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) cfh[(c * 8 + a) * kTile + tid] = fh[c];
  }
}

// PML gather: one thread per tile node; the split-field forces of an incidence are rebuilt from
// the element's det * shape gradient of the corner and its split-stress sums.  w2_of(el, a, wxx,
// wyy, wzz, wxy) gives the negated binary32 products -dw * shp of corner a of local element el as
// the pairs (wx, wx), (wy, wy), (wz, wz), (wx, wy) (as in pml_element).  The nine split components
// run as four packed pairs, (0, 3) = wx (sxx, sxy), (1, 4) = wy (sxy, syy), (2, 5) = wz (sxz, syz),
// (6, 7) = (wx, wy) (sxz, syz), and a single 8 = wz szz; the hourglass forces as (x, y) and z.
// 12-DOF nodes reduce 9 split components + 3 into F9 / F; 3-DOF nodes on the PML boundary take
// the compensated sum of their 4 partials.
template <class W2Of>
__device__ __forceinline__ void pml_gather(const ElemGroup<float> &g, int M, int nb, const unsigned short *incp,
                                           const unsigned short *sinc, const float *es, const float *cfh,
                                           const W2Of &w2_of, float *__restrict__ F, float *__restrict__ F9,
                                           int nnode, int n_int, int npml, const int *sids) {
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    // the node id is loaded first: its latency runs under the sums
    const int n = sids ? sids[j] : __ldg(g.tile_nodes + nb + j);
    const float2 z2 = make_float2(0.f, 0.f);
    float2 h03 = z2, l03 = z2, h14 = z2, l14 = z2, h25 = z2, l25 = z2, h67 = z2, l67 = z2, hf = z2, lf = z2;
    float h8 = 0.f, l8 = 0.f, hfz = 0.f, lfz = 0.f;
    const int q1 = incp[j + 1];
    for (int q = incp[j]; q < q1; ++q) {
      const int r = sinc[q];
      const int a = r / kTile, el = r - a * kTile;
      float2 wxx, wyy, wzz, wxy;
      w2_of(el, a, wxx, wyy, wzz, wxy);
      const float sxx = es[el], syy = es[kTile + el], szz = es[2 * kTile + el];
      const float sxy = es[3 * kTile + el], sxz = es[4 * kTile + el], syz = es[5 * kTile + el];
      kahan_add2(h03, l03, __fmul2_rn(wxx, make_float2(sxx, sxy)));
      kahan_add2(h14, l14, __fmul2_rn(wyy, make_float2(sxy, syy)));
      kahan_add2(h25, l25, __fmul2_rn(wzz, make_float2(sxz, syz)));
      kahan_add2(h67, l67, __fmul2_rn(wxy, make_float2(sxz, syz)));
      kahan_add(h8, l8, wzz.x * szz);
      kahan_add2(hf, lf, make_float2(cfh[(0 * 8 + a) * kTile + el], cfh[(1 * 8 + a) * kTile + el]));
      kahan_add(hfz, lfz, cfh[(2 * 8 + a) * kTile + el]);
    }
    const float hi[12] = {h03.x, h14.x, h25.x, h03.y, h14.y, h25.y, h67.x, h67.y, h8, hf.x, hf.y, hfz};
    const float lo[12] = {l03.x, l14.x, l25.x, l03.y, l14.y, l25.y, l67.x, l67.y, l8, lf.x, lf.y, lfz};
    if (n >= n_int) {
      const int slot = n - n_int;
#pragma unroll
      for (int i = 0; i < 9; ++i) atomicAdd(F9 + (size_t)i * npml + slot, hi[i] - lo[i]);
#pragma unroll
      for (int c = 0; c < 3; ++c) atomicAdd(F + (size_t)c * nnode + n, hi[9 + c] - lo[9 + c]);
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float s = 0.f, e2 = 0.f;
        kahan_add(s, e2, hi[3 * c] - lo[3 * c]);
        kahan_add(s, e2, hi[3 * c + 1] - lo[3 * c + 1]);
        kahan_add(s, e2, hi[3 * c + 2] - lo[3 * c + 2]);
        kahan_add(s, e2, hi[9 + c] - lo[9 + c]);
        atomicAdd(F + (size_t)c * nnode + n, s - e2);
      }
    }
  }
}

// w2_of for table sources: the negated products -dw * shape gradient of corner a of the element
// that src_of(el) reads, as the pairs pml_gather takes.
template <int HG, class SrcOf>
struct WFromSrc {
  SrcOf src_of;
  __device__ void operator()(int el, int a, float2 &wxx, float2 &wyy, float2 &wzz, float2 &wxy) const {
    using C = TabCommon<HG>;
    const auto S = src_of(el);
    const float dw = S.g(C::DET);
    const float wx = -(dw * S.g(C::SHP + 3 * a)), wy = -(dw * S.g(C::SHP + 3 * a + 1));
    const float wz = -(dw * S.g(C::SHP + 3 * a + 2));
    wxx = make_float2(wx, wx);
    wyy = make_float2(wy, wy);
    wzz = make_float2(wz, wz);
    wxy = make_float2(wx, wy);
  }
};
template <int HG, class SrcOf>
__device__ __forceinline__ WFromSrc<HG, SrcOf> w_from_src(const SrcOf &f) {
  return WFromSrc<HG, SrcOf>{f};
}

template <class K>
inline int allow_smem(K kern, size_t sm) {
  if (sm > 48 * 1024 &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
    return EQD_ERR_CUDA;
  return EQD_OK;
}

}  // namespace e32

// record-indexed layout (kernels_elem32r.cu)
int launch_elements_rec(Context &c, cudaStream_t s, const e32::ElemConst32 &k, bool interior);

}  // namespace eqd
