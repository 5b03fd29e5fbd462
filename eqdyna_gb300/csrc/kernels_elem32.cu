// Element kernels of the binary32 form: element strain, stress and hourglass forces in binary32,
// nodal accumulation in binary32 with Kahan compensation, binary64 node state.
//
// One CTA per tile.  A tile is `tile` consecutive elements of a brick-ordered element list
// (4 x 4 x 8 elements), so its ~225 distinct nodes are few and come in short runs along y.  Per tile:
//   stage  : the binary32 copies of velocity and (u + rdampk v) of the tile's nodes -> shared memory
//   element: one thread per element computes its forces from shared memory and stores them per
//            (corner, element) slot in shared memory
//   gather : one thread per tile node sums its incidences in a fixed order with Kahan-compensated
//            binary32 and adds the result to the binary32 node force with one L2 reduction per
//            component (no binary64 arithmetic: GB300 runs binary64 at 1/64 of binary32)
// The element math is that of the binary64 kernels (src/calcElemKU.f90, src/hrglss.f90,
// src/assembleGlobalKU.f90:70-346).
#include "eqd_device.cuh"

namespace eqd {

namespace {

constexpr int kTileI = 128;  // interior tile = CTA size
constexpr int kTileP = 128;  // PML tile = CTA size

__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

__device__ __forceinline__ float viscous_pattern_f(int m, int a) {
  const unsigned neg[4] = {0x3Cu, 0x96u, 0xAAu, 0x5Au};
  return ((neg[m] >> a) & 1u) ? -1.0f : 1.0f;
}

struct ElemConst32 {
  float dt, rdampk, rdampm, gz, ccosphi, sinphi, relax;
};

// Stages the tile's node data and builds slot_of[corner * tile + e] = local node index.
template <int TILE>
__device__ __forceinline__ int stage_tile(const ElemGroup<float> &g, const float *__restrict__ vel32,
                                          const float *__restrict__ dl32, int nnode, int Mmax,
                                          float *sv, float *sd, unsigned short *slot_of,
                                          int &nb, const unsigned short *&incp,
                                          const unsigned short *&inc) {
  const int t = blockIdx.x;
  nb = g.tile_node_ptr[t];
  const int M = g.tile_node_ptr[t + 1] - nb;
  incp = g.tile_incp + g.tile_incp_off[t];
  inc = g.tile_inc + (size_t)t * TILE * 8;
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    const int n = g.tile_nodes[nb + j];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      sv[c * Mmax + j] = vel32[c * nnode + n];
      sd[c * Mmax + j] = dl32[c * nnode + n];
    }
    const int q1 = incp[j + 1];
    for (int q = incp[j]; q < q1; ++q) slot_of[inc[q]] = (unsigned short)j;
  }
  return M;
}

template <bool BODY, bool PLASTIC, int HG>
__global__ void __launch_bounds__(kTileI)
    elem_interior_f32(ElemGroup<float> g, const float *__restrict__ vel32,
                      const float *__restrict__ dl32, float *__restrict__ F, int nnode,
                      ElemConst32 k) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int Mmax = g.max_tile_nodes;
  float *sv = reinterpret_cast<float *>(smem);
  float *sd = sv + 3 * Mmax;
  float *fs = sd + 3 * Mmax;                                        // [3][8][TILE]
  unsigned short *slot_of = reinterpret_cast<unsigned short *>(fs + 24 * kTileI);  // [8][TILE]
  int nb;
  const unsigned short *incp, *inc;
  const int M = stage_tile<kTileI>(g, vel32, dl32, nnode, Mmax, sv, sd, slot_of, nb, incp, inc);
  __syncthreads();
  const int tid = threadIdx.x;
  const int e = blockIdx.x * kTileI + tid;
  if (e < g.ne) {
    const int ne = g.ne;
    float sr[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float ph[4][3];
#pragma unroll
    for (int m = 0; m < 4; ++m) ph[m][0] = ph[m][1] = ph[m][2] = 0.f;
    int sl[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      sl[a] = slot_of[a * kTileI + tid];
      const float bx = __ldg(g.shp + (3 * a + 0) * ne + e);
      const float by = __ldg(g.shp + (3 * a + 1) * ne + e);
      const float bz = __ldg(g.shp + (3 * a + 2) * ne + e);
      const float vx = sv[sl[a]], vy = sv[Mmax + sl[a]], vz = sv[2 * Mmax + sl[a]];
      sr[0] = fmaf(bx, vx, sr[0]);
      sr[1] = fmaf(by, vy, sr[1]);
      sr[2] = fmaf(bz, vz, sr[2]);
      sr[3] = fmaf(by, vz, fmaf(bz, vy, sr[3]));
      sr[4] = fmaf(bx, vz, fmaf(bz, vx, sr[4]));
      sr[5] = fmaf(bx, vy, fmaf(by, vx, sr[5]));
      if (HG == 1) {
        const float lx = sd[sl[a]], ly = sd[Mmax + sl[a]], lz = sd[2 * Mmax + sl[a]];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          const float p = __ldg(g.phi + (8 * m + a) * ne + e);
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
    const float lam = g.lam[e], mu = g.mu[e], cd = lam + 2.0f * mu;
    const float srate[6] = {cd * sr[0] + lam * sr[1] + lam * sr[2], lam * sr[0] + cd * sr[1] + lam * sr[2],
                            lam * sr[0] + lam * sr[1] + cd * sr[2], mu * sr[3], mu * sr[4], mu * sr[5]};
    float s[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] = fmaf(srate[i], k.dt, g.stress[i * ne + e]);
    if (PLASTIC) {
      const float strmea = (s[0] + s[1] + s[2]) / 3.0f;
      const float dev[6] = {s[0] - strmea, s[1] - strmea, s[2] - strmea, s[3], s[4], s[5]};
      const float taomax = sqrtf(0.5f * (dev[0] * dev[0] + dev[1] * dev[1] + dev[2] * dev[2]) +
                                 dev[3] * dev[3] + dev[4] * dev[4] + dev[5] * dev[5]);
      float yield = k.ccosphi - k.sinphi * (strmea + g.porep[e]);
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
        g.pstrain[e] += (double)sqrtf(mag);
      }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) g.stress[i * ne + e] = s[i];
    const float tw = -g.detw[e];
    float st[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) st[i] = tw * fmaf(k.rdampk, srate[i], s[i]);
    float h[4][3];
    if (HG == 1) {
      const float s1 = g.ss[e], s2 = g.ss[ne + e], s3 = g.ss[2 * ne + e];
      const float s4 = g.ss[3 * ne + e], s5 = g.ss[4 * ne + e], s6 = g.ss[5 * ne + e];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        h[m][0] = s1 * ph[m][0] + s2 * ph[m][1] + s3 * ph[m][2];
        h[m][1] = s2 * ph[m][0] + s4 * ph[m][1] + s5 * ph[m][2];
        h[m][2] = s3 * ph[m][0] + s5 * ph[m][1] + s6 * ph[m][2];
      }
    } else {
      const float coef = g.hgcoef[e];
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int c = 0; c < 3; ++c) h[m][c] = coef * ph[m][c];
    }
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const float bx = __ldg(g.shp + (3 * a + 0) * ne + e);
      const float by = __ldg(g.shp + (3 * a + 1) * ne + e);
      const float bz = __ldg(g.shp + (3 * a + 2) * ne + e);
      float f0 = bx * st[0] + bz * st[4] + by * st[5];
      float f1 = by * st[1] + bz * st[3] + bx * st[5];
      float f2 = bz * st[2] + by * st[3] + bx * st[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float p = (HG == 1) ? __ldg(g.phi + (8 * m + a) * ne + e) : viscous_pattern_f(m, a);
        f0 = fmaf(-p, h[m][0], f0);
        f1 = fmaf(-p, h[m][1], f1);
        f2 = fmaf(-p, h[m][2], f2);
      }
      if (BODY) {
        const float em = g.em[a * ne + e];
        f0 -= em * (k.rdampm * sv[sl[a]]);
        f1 -= em * (k.rdampm * sv[Mmax + sl[a]]);
        f2 -= em * (k.rdampm * sv[2 * Mmax + sl[a]] + k.gz);
      }
      fs[(0 * 8 + a) * kTileI + tid] = f0;
      fs[(1 * 8 + a) * kTileI + tid] = f1;
      fs[(2 * 8 + a) * kTileI + tid] = f2;
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
    const int q1 = incp[j + 1];
    for (int q = incp[j]; q < q1; ++q) {
      const int r = inc[q];  // corner * TILE + e_local
      const int a = r / kTileI, el = r - a * kTileI;
#pragma unroll
      for (int c = 0; c < 3; ++c) kahan_add(hi[c], lo[c], fs[(c * 8 + a) * kTileI + el]);
    }
    const int n = g.tile_nodes[nb + j];
#pragma unroll
    for (int c = 0; c < 3; ++c) atomicAdd(F + (size_t)c * nnode + n, hi[c] - lo[c]);
  }
}

template <bool BODY, bool S0, int HG>
__global__ void __launch_bounds__(kTileP)
    elem_pml_f32(ElemGroup<float> g, const float *__restrict__ vel32, const float *__restrict__ dl32,
                 float *__restrict__ F, float *__restrict__ F9, int nnode, int n_int, int npml,
                 ElemConst32 k) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int Mmax = g.max_tile_nodes;
  float *sv = reinterpret_cast<float *>(smem);
  float *sd = sv + 3 * Mmax;
  float *cw = sd + 3 * Mmax;            // [3][8][TILE] dw * shape gradient of each corner
  float *cfh = cw + 24 * kTileP;        // [3][8][TILE] hourglass / s0 / body force of each corner
  float *es = cfh + 24 * kTileP;        // [6][TILE] split-stress sums sxx syy szz sxy sxz syz
  unsigned short *slot_of = reinterpret_cast<unsigned short *>(es + 6 * kTileP);
  int nb;
  const unsigned short *incp, *inc;
  const int M = stage_tile<kTileP>(g, vel32, dl32, nnode, Mmax, sv, sd, slot_of, nb, incp, inc);
  __syncthreads();
  const int tid = threadIdx.x;
  const int e = blockIdx.x * kTileP + tid;
  if (e < g.ne) {
    const int ne = g.ne;
    float D[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) D[i][0] = D[i][1] = D[i][2] = 0.f;
    float ph[4][3];
#pragma unroll
    for (int m = 0; m < 4; ++m) ph[m][0] = ph[m][1] = ph[m][2] = 0.f;
    int sl[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      sl[a] = slot_of[a * kTileP + tid];
      const float b[3] = {__ldg(g.shp + (3 * a + 0) * ne + e), __ldg(g.shp + (3 * a + 1) * ne + e),
                          __ldg(g.shp + (3 * a + 2) * ne + e)};
      const float v[3] = {sv[sl[a]], sv[Mmax + sl[a]], sv[2 * Mmax + sl[a]]};
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) D[i][j] = fmaf(b[i], v[j], D[i][j]);
      if (HG == 1) {
        const float l[3] = {sd[sl[a]], sd[Mmax + sl[a]], sd[2 * Mmax + sl[a]]};
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          const float p = __ldg(g.phi + (8 * m + a) * ne + e);
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
    const float lam = g.lam[e], mu = g.mu[e], cd = lam + 2.0f * mu;
    const float a0 = g.pml_ab[e], a1 = g.pml_ab[ne + e], a2 = g.pml_ab[2 * ne + e];
    const float b0 = g.pml_ab[3 * ne + e], b1 = g.pml_ab[4 * ne + e], b2 = g.pml_ab[5 * ne + e];
    const float src[15] = {cd * D[0][0], lam * D[1][1], lam * D[2][2], lam * D[0][0], cd * D[1][1],
                           lam * D[2][2], lam * D[0][0], lam * D[1][1], cd * D[2][2], mu * D[0][1],
                           mu * D[1][0], mu * D[0][2], mu * D[2][0], mu * D[1][2], mu * D[2][1]};
    const int axis[15] = {0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 0, 2, 1, 2};
    float sp[15];
#pragma unroll
    for (int i = 0; i < 15; ++i) {
      const float aa = axis[i] == 0 ? a0 : (axis[i] == 1 ? a1 : a2);
      const float bb = axis[i] == 0 ? b0 : (axis[i] == 1 ? b1 : b2);
      sp[i] = fmaf(aa, g.stress[i * ne + e], src[i]) * bb;
      g.stress[i * ne + e] = sp[i];
    }
    es[0 * kTileP + tid] = sp[0] + sp[1] + sp[2];
    es[1 * kTileP + tid] = sp[3] + sp[4] + sp[5];
    es[2 * kTileP + tid] = sp[6] + sp[7] + sp[8];
    es[3 * kTileP + tid] = sp[9] + sp[10];
    es[4 * kTileP + tid] = sp[11] + sp[12];
    es[5 * kTileP + tid] = sp[13] + sp[14];
    const float sr[6] = {D[0][0], D[1][1], D[2][2], D[2][1] + D[1][2], D[2][0] + D[0][2], D[1][0] + D[0][1]};
    float s0[6] = {k.rdampk * (cd * sr[0] + lam * sr[1] + lam * sr[2]),
                   k.rdampk * (lam * sr[0] + cd * sr[1] + lam * sr[2]),
                   k.rdampk * (lam * sr[0] + lam * sr[1] + cd * sr[2]), k.rdampk * (mu * sr[3]),
                   k.rdampk * (mu * sr[4]), k.rdampk * (mu * sr[5])};
    if (S0) {
#pragma unroll
      for (int i = 0; i < 6; ++i) s0[i] += g.stress0[i * ne + e];
    }
    float h[4][3];
    if (HG == 1) {
      const float s1 = g.ss[e], s2 = g.ss[ne + e], s3 = g.ss[2 * ne + e];
      const float s4 = g.ss[3 * ne + e], s5 = g.ss[4 * ne + e], s6 = g.ss[5 * ne + e];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        h[m][0] = s1 * ph[m][0] + s2 * ph[m][1] + s3 * ph[m][2];
        h[m][1] = s2 * ph[m][0] + s4 * ph[m][1] + s5 * ph[m][2];
        h[m][2] = s3 * ph[m][0] + s5 * ph[m][1] + s6 * ph[m][2];
      }
    } else {
      const float coef = g.hgcoef[e];
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int c = 0; c < 3; ++c) h[m][c] = coef * ph[m][c];
    }
    const float dw = g.detw[e];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const float wx = dw * __ldg(g.shp + (3 * a + 0) * ne + e);
      const float wy = dw * __ldg(g.shp + (3 * a + 1) * ne + e);
      const float wz = dw * __ldg(g.shp + (3 * a + 2) * ne + e);
      float fh[3] = {-(wx * s0[0] + wz * s0[4] + wy * s0[5]), -(wy * s0[1] + wz * s0[3] + wx * s0[5]),
                     -(wz * s0[2] + wy * s0[3] + wx * s0[4])};
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float p = (HG == 1) ? __ldg(g.phi + (8 * m + a) * ne + e) : viscous_pattern_f(m, a);
#pragma unroll
        for (int c = 0; c < 3; ++c) fh[c] = fmaf(-p, h[m][c], fh[c]);
      }
      if (BODY) {
        const float em = g.em[a * ne + e];
        fh[0] -= em * (k.rdampm * sv[sl[a]]);
        fh[1] -= em * (k.rdampm * sv[Mmax + sl[a]]);
        fh[2] -= em * (k.rdampm * sv[2 * Mmax + sl[a]] + k.gz);
      }
      cw[(0 * 8 + a) * kTileP + tid] = wx;
      cw[(1 * 8 + a) * kTileP + tid] = wy;
      cw[(2 * 8 + a) * kTileP + tid] = wz;
#pragma unroll
      for (int c = 0; c < 3; ++c) cfh[(c * 8 + a) * kTileP + tid] = fh[c];
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < M; j += blockDim.x) {
    float hi[12], lo[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) hi[q] = lo[q] = 0.f;
    const int q1 = incp[j + 1];
    for (int q = incp[j]; q < q1; ++q) {
      const int r = inc[q];
      const int a = r / kTileP, el = r - a * kTileP;
      const float wx = cw[(0 * 8 + a) * kTileP + el], wy = cw[(1 * 8 + a) * kTileP + el];
      const float wz = cw[(2 * 8 + a) * kTileP + el];
      const float sxx = es[el], syy = es[kTileP + el], szz = es[2 * kTileP + el];
      const float sxy = es[3 * kTileP + el], sxz = es[4 * kTileP + el], syz = es[5 * kTileP + el];
      const float f9[9] = {-wx * sxx, -wy * sxy, -wz * sxz, -wx * sxy, -wy * syy,
                           -wz * syz, -wx * sxz, -wy * syz, -wz * szz};
#pragma unroll
      for (int i = 0; i < 9; ++i) kahan_add(hi[i], lo[i], f9[i]);
#pragma unroll
      for (int c = 0; c < 3; ++c) kahan_add(hi[9 + c], lo[9 + c], cfh[(c * 8 + a) * kTileP + el]);
    }
    const int n = g.tile_nodes[nb + j];
    if (n >= n_int) {
      const int slot = n - n_int;
#pragma unroll
      for (int i = 0; i < 9; ++i) atomicAdd(F9 + (size_t)i * npml + slot, hi[i] - lo[i]);
#pragma unroll
      for (int c = 0; c < 3; ++c) atomicAdd(F + (size_t)c * nnode + n, hi[9 + c] - lo[9 + c]);
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float s = 0.f, e = 0.f;
        kahan_add(s, e, hi[3 * c] - lo[3 * c]);
        kahan_add(s, e, hi[3 * c + 1] - lo[3 * c + 1]);
        kahan_add(s, e, hi[3 * c + 2] - lo[3 * c + 2]);
        kahan_add(s, e, hi[9 + c] - lo[9 + c]);
        atomicAdd(F + (size_t)c * nnode + n, s - e);
      }
    }
  }
}

size_t smem_interior(int Mmax) { return 6 * (size_t)Mmax * 4 + 24 * kTileI * 4 + 8 * kTileI * 2; }
size_t smem_pml(int Mmax) { return 6 * (size_t)Mmax * 4 + 48 * kTileP * 4 + 6 * kTileP * 4 + 8 * kTileP * 2; }

template <bool BODY, bool PLASTIC>
int launch_interior32(Context &c, cudaStream_t s, const ElemConst32 &k) {
  const ElemGroup<float> &g = c.gi32;
  if (g.ne == 0) return EQD_OK;
  const size_t sm = smem_interior(g.max_tile_nodes);
  if (c.sc.C_hg == 2) {
    auto kern = elem_interior_f32<BODY, PLASTIC, 2>;
    if (sm > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kern<<<g.ntiles, kTileI, sm, s>>>(g, c.vel32, c.dl32, c.F32, c.nnode, k);
  } else {
    auto kern = elem_interior_f32<BODY, PLASTIC, 1>;
    if (sm > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kern<<<g.ntiles, kTileI, sm, s>>>(g, c.vel32, c.dl32, c.F32, c.nnode, k);
  }
  return EQD_OK;
}

template <bool BODY, bool S0>
int launch_pml32(Context &c, cudaStream_t s, const ElemConst32 &k) {
  const ElemGroup<float> &g = c.gp32;
  if (g.ne == 0) return EQD_OK;
  const size_t sm = smem_pml(g.max_tile_nodes);
  if (c.sc.C_hg == 2) {
    auto kern = elem_pml_f32<BODY, S0, 2>;
    if (sm > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kern<<<g.ntiles, kTileP, sm, s>>>(g, c.vel32, c.dl32, c.F32, c.F9_32, c.nnode, c.n_int, c.npml, k);
  } else {
    auto kern = elem_pml_f32<BODY, S0, 1>;
    if (sm > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kern<<<g.ntiles, kTileP, sm, s>>>(g, c.vel32, c.dl32, c.F32, c.F9_32, c.nnode, c.n_int, c.npml, k);
  }
  return EQD_OK;
}

}  // namespace

int tile_size_interior() { return kTileI; }
int tile_size_pml() { return kTileP; }

int launch_elements_f32(Context &c, cudaStream_t s, const ElemConst &kd, int part) {
  ElemConst32 k{(float)kd.dt, (float)kd.rdampk, (float)kd.rdampm, (float)kd.gz,
                (float)kd.ccosphi, (float)kd.sinphi, (float)kd.relax};
  const bool body = (c.sc.rdampm != 0.0) || (c.sc.C_elastic == 0);
  const bool plastic = (c.sc.C_elastic == 0);
  int rc = EQD_OK;
  if (part != 1) {
    if (plastic) rc = body ? launch_interior32<true, true>(c, s, k) : launch_interior32<false, true>(c, s, k);
    else rc = body ? launch_interior32<true, false>(c, s, k) : launch_interior32<false, false>(c, s, k);
    if (rc) return rc;
  }
  if (part != 0) {
    const bool s0 = c.gp32.stress0 != nullptr;
    if (body) rc = s0 ? launch_pml32<true, true>(c, s, k) : launch_pml32<true, false>(c, s, k);
    else rc = s0 ? launch_pml32<false, true>(c, s, k) : launch_pml32<false, false>(c, s, k);
    if (rc) return rc;
  }
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

}  // namespace eqd
