// Element internal-force kernels: one-point hexahedron / degenerated wedge with hourglass control
// (interior elements) and the split-field PML element, each fused with its hourglass force and
// scattered to the nodes with hardware float64 reductions in L2.
//
// Reference: assembleGlobalKU + calcElemKU + calcB + calcElemMass (src/assembleGlobalKU.f90:3-67,
// src/calcElemKU.f90:3-191, src/calcB.f90, src/calcElemMass.f90), calcPMLElemKU
// (src/assembleGlobalKU.f90:70-346) and hrglss (src/hrglss.f90:3-100).  The reference makes two
// element passes (forces, then hourglass) and adds every contribution to nodalForceArr in element
// order; here one pass adds the sum of both per node, so the summation order (not the terms)
// differs.
#include "eqd_device.cuh"

namespace eqd {

namespace {

constexpr int kBlockElem = 128;

// ---------------------------------------------------------------------------------------------
// Interior elements, binary64.
//   BODY    : -m (rdampm v + g_z e_z) body term of calcElemMass (plastic form or rdampm != 0)
//   PLASTIC : Drucker-Prager visco-plastic return (C_elastic == 0, src/calcElemKU.f90:133-167)
//   QM      : coarse-grained Q memory variables (C_Q == 1, src/calcElemKU.f90:77-132)
//   HG      : 1 = Kosloff-Frazier stiffness hourglass, 2 = viscous hourglass
template <bool BODY, bool PLASTIC, bool QM, int HG>
__global__ void __launch_bounds__(kBlockElem)
    elem_interior_f64(ElemGroup<double> g, const double *__restrict__ vel,
                      const double *__restrict__ disp, double *__restrict__ F, int nnode,
                      ElemConst k) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.ne) return;
  const size_t ne = g.ne;  // 64-bit: the 32 hourglass rows of a group of 10^8 elements pass 2^31
  int n[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) n[a] = __ldg(g.conn + a * ne + e);

  double sr[6] = {0, 0, 0, 0, 0, 0};  // strain rate, Voigt order xx yy zz yz xz xy
  double sn[6] = {0, 0, 0, 0, 0, 0};  // strain (Q form only)
  double ph[4][3];                    // per hourglass mode: phi^T (u + rdampk v), or q for HG 2
#pragma unroll
  for (int m = 0; m < 4; ++m) ph[m][0] = ph[m][1] = ph[m][2] = 0.0;

#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double bx = __ldg(g.shp + (3 * a + 0) * ne + e);
    const double by = __ldg(g.shp + (3 * a + 1) * ne + e);
    const double bz = __ldg(g.shp + (3 * a + 2) * ne + e);
    const double vx = vel[n[a]], vy = vel[nnode + n[a]], vz = vel[2 * nnode + n[a]];
    sr[0] = fma(bx, vx, sr[0]);
    sr[1] = fma(by, vy, sr[1]);
    sr[2] = fma(bz, vz, sr[2]);
    sr[3] = fma(by, vz, fma(bz, vy, sr[3]));
    sr[4] = fma(bx, vz, fma(bz, vx, sr[4]));
    sr[5] = fma(bx, vy, fma(by, vx, sr[5]));
    if (HG == 1 || QM) {
      const double dx = disp[n[a]], dy = disp[nnode + n[a]], dz = disp[2 * nnode + n[a]];
      if (QM) {
        sn[0] = fma(bx, dx, sn[0]);
        sn[1] = fma(by, dy, sn[1]);
        sn[2] = fma(bz, dz, sn[2]);
        sn[3] = fma(by, dz, fma(bz, dy, sn[3]));
        sn[4] = fma(bx, dz, fma(bz, dx, sn[4]));
        sn[5] = fma(bx, dy, fma(by, dx, sn[5]));
      }
      if (HG == 1) {
        const double lx = fma(k.rdampk, vx, dx), ly = fma(k.rdampk, vy, dy), lz = fma(k.rdampk, vz, dz);
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          const double p = __ldg(g.phi + (8 * m + a) * ne + e);
          ph[m][0] = fma(p, lx, ph[m][0]);
          ph[m][1] = fma(p, ly, ph[m][1]);
          ph[m][2] = fma(p, lz, ph[m][2]);
        }
      }
    }
    if (HG == 2) {
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const double s = viscous_pattern(m, a);
        ph[m][0] = fma(s, vx, ph[m][0]);
        ph[m][1] = fma(s, vy, ph[m][1]);
        ph[m][2] = fma(s, vz, ph[m][2]);
      }
    }
  }

  // ---- stress update (src/calcElemKU.f90:63-76) ----
  const double lam = g.lam[e], mu = g.mu[e], cd = lam + 2.0 * mu;
  double srate[6];
  srate[0] = cd * sr[0] + lam * sr[1] + lam * sr[2];
  srate[1] = lam * sr[0] + cd * sr[1] + lam * sr[2];
  srate[2] = lam * sr[0] + lam * sr[1] + cd * sr[2];
  srate[3] = mu * sr[3];
  srate[4] = mu * sr[4];
  srate[5] = mu * sr[5];
  double s[6];
  if (!QM) {
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] = fma(srate[i], k.dt, g.stress[i * ne + e]);
  } else {
    // coarse-grained memory variables: per-element coefficients precomputed from qconstant
    const double ex = g.qcoef[e], miuu = g.qcoef[ne + e], Mu = g.qcoef[2 * ne + e];
    const double wkp = g.qcoef[3 * ne + e], wks = g.qcoef[4 * ne + e];
    const double vols = sn[0] + sn[1] + sn[2];
    double *mem = g.stress + 6 * ne;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const double a1 = mem[i * ne + e];
      const double drive = (i < 3) ? (2 * miuu * sn[i] * wks + (Mu * wkp - 2 * miuu * wks) * vols)
                                   : (miuu * sn[i] * wks);
      const double an = ex * a1 + (1 - ex) * drive;
      mem[i * ne + e] = an;
      s[i] = (i < 3) ? (2.0 * miuu * sn[i] + (Mu - 2.0 * miuu) * vols - 0.5 * (an + a1))
                     : (2.0 * miuu * sn[i] / 2.0 - 0.5 * (an + a1));
    }
  }
  if (PLASTIC) {
    const double strmea = (s[0] + s[1] + s[2]) / 3.0;
    double dev[6] = {s[0] - strmea, s[1] - strmea, s[2] - strmea, s[3], s[4], s[5]};
    const double taomax = sqrt(0.5 * (dev[0] * dev[0] + dev[1] * dev[1] + dev[2] * dev[2]) +
                               dev[3] * dev[3] + dev[4] * dev[4] + dev[5] * dev[5]);
    double yield = k.ccosphi - k.sinphi * (strmea + g.porep[e]);
    if (yield < 0.0) yield = 0.0;
    if (taomax > yield) {
      const double r = yield / taomax + (1 - yield / taomax) * k.relax;
      double pinc[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const double sv = dev[i] * r;
        pinc[i] = (dev[i] - sv) / mu;
        s[i] = (i < 3) ? sv + strmea : sv;
      }
      const double pm = (pinc[0] + pinc[1] + pinc[2]) / 3.0;
      double mag = 0.0;
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const double q = pinc[i] - pm;
        mag += (i < 3 ? 0.5 : 1.0) * q * q;
      }
      g.pstrain[e] += sqrt(mag);
    }
  }
  if (!QM) {
#pragma unroll
    for (int i = 0; i < 6; ++i) g.stress[i * ne + e] = s[i];
  } else {
#pragma unroll
    for (int i = 0; i < 6; ++i) g.stress[i * ne + e] = s[i];
  }
  const double tw = -g.detw[e];
  double st[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) st[i] = tw * fma(k.rdampk, srate[i], s[i]);

  // ---- hourglass resistance per mode ----
  double h[4][3];
  if (HG == 1) {
    const double s1 = g.ss[e], s2 = g.ss[ne + e], s3 = g.ss[2 * ne + e];
    const double s4 = g.ss[3 * ne + e], s5 = g.ss[4 * ne + e], s6 = g.ss[5 * ne + e];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const double p0 = ph[m][0], p1 = ph[m][1], p2 = ph[m][2];
      h[m][0] = s1 * p0 + s2 * p1 + s3 * p2;
      h[m][1] = s2 * p0 + s4 * p1 + s5 * p2;
      h[m][2] = s3 * p0 + s5 * p1 + s6 * p2;
    }
  } else {
    const double coef = g.hgcoef[e];
#pragma unroll
    for (int m = 0; m < 4; ++m)
      for (int c = 0; c < 3; ++c) h[m][c] = coef * ph[m][c];
  }

  // ---- nodal forces: B^T st - sum_m phi_m h_m [- m (rdampm v + g)] and scatter ----
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double bx = __ldg(g.shp + (3 * a + 0) * ne + e);
    const double by = __ldg(g.shp + (3 * a + 1) * ne + e);
    const double bz = __ldg(g.shp + (3 * a + 2) * ne + e);
    double fx = bx * st[0] + bz * st[4] + by * st[5];
    double fy = by * st[1] + bz * st[3] + bx * st[5];
    double fz = bz * st[2] + by * st[3] + bx * st[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const double p = (HG == 1) ? __ldg(g.phi + (8 * m + a) * ne + e) : viscous_pattern(m, a);
      fx = fma(-p, h[m][0], fx);
      fy = fma(-p, h[m][1], fy);
      fz = fma(-p, h[m][2], fz);
    }
    if (BODY) {
      const double em = g.em[a * ne + e];
      fx -= em * (k.rdampm * vel[n[a]]);
      fy -= em * (k.rdampm * vel[nnode + n[a]]);
      fz -= em * (k.rdampm * vel[2 * nnode + n[a]] + k.gz);
    }
    atomicAdd(F + n[a], fx);
    atomicAdd(F + nnode + n[a], fy);
    atomicAdd(F + 2 * nnode + n[a], fz);
  }
}

// ---------------------------------------------------------------------------------------------
// PML elements, binary64 (src/assembleGlobalKU.f90:36-63 and :70-346).
//   S0 : element carries a constant initial stress s(16..21) (plastic form)
template <bool BODY, bool S0, int HG>
__global__ void __launch_bounds__(kBlockElem)
    elem_pml_f64(ElemGroup<double> g, const double *__restrict__ vel,
                 const double *__restrict__ disp, double *__restrict__ F, double *__restrict__ F9,
                 int nnode, int n_int, int npml, ElemConst k) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.ne) return;
  const size_t ne = g.ne;  // 64-bit: the 32 hourglass rows of a group of 10^8 elements pass 2^31
  int n[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) n[a] = __ldg(g.conn + a * ne + e);
  double D[3][3];  // D[i][j] = d v_j / d x_i
#pragma unroll
  for (int i = 0; i < 3; ++i) D[i][0] = D[i][1] = D[i][2] = 0.0;
  double ph[4][3];
#pragma unroll
  for (int m = 0; m < 4; ++m) ph[m][0] = ph[m][1] = ph[m][2] = 0.0;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double b[3] = {__ldg(g.shp + (3 * a + 0) * ne + e), __ldg(g.shp + (3 * a + 1) * ne + e),
                         __ldg(g.shp + (3 * a + 2) * ne + e)};
    const double v[3] = {vel[n[a]], vel[nnode + n[a]], vel[2 * nnode + n[a]]};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) D[i][j] = fma(b[i], v[j], D[i][j]);
    if (HG == 1) {
      const double l[3] = {fma(k.rdampk, v[0], disp[n[a]]), fma(k.rdampk, v[1], disp[nnode + n[a]]),
                           fma(k.rdampk, v[2], disp[2 * nnode + n[a]])};
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const double p = __ldg(g.phi + (8 * m + a) * ne + e);
#pragma unroll
        for (int c = 0; c < 3; ++c) ph[m][c] = fma(p, l[c], ph[m][c]);
      }
    } else {
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const double s = viscous_pattern(m, a);
#pragma unroll
        for (int c = 0; c < 3; ++c) ph[m][c] = fma(s, v[c], ph[m][c]);
      }
    }
  }
  const double lam = g.lam[e], mu = g.mu[e], cd = lam + 2.0 * mu;
  // split-field stress update: s_new = (source + a s) * b, per damping axis
  const double a0 = g.pml_ab[e], a1 = g.pml_ab[ne + e], a2 = g.pml_ab[2 * ne + e];
  const double b0 = g.pml_ab[3 * ne + e], b1 = g.pml_ab[4 * ne + e], b2 = g.pml_ab[5 * ne + e];
  // (source, axis) of the 15 split components, src/assembleGlobalKU.f90:277-311
  const double src[15] = {cd * D[0][0], lam * D[1][1], lam * D[2][2], lam * D[0][0], cd * D[1][1],
                          lam * D[2][2], lam * D[0][0], lam * D[1][1], cd * D[2][2], mu * D[0][1],
                          mu * D[1][0], mu * D[0][2], mu * D[2][0], mu * D[1][2], mu * D[2][1]};
  const int axis[15] = {0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 0, 2, 1, 2};
  double sp[15];
#pragma unroll
  for (int i = 0; i < 15; ++i) {
    const double aa = axis[i] == 0 ? a0 : (axis[i] == 1 ? a1 : a2);
    const double bb = axis[i] == 0 ? b0 : (axis[i] == 1 ? b1 : b2);
    sp[i] = fma(aa, g.stress[i * ne + e], src[i]) * bb;
    g.stress[i * ne + e] = sp[i];
  }
  const double sxx = sp[0] + sp[1] + sp[2], syy = sp[3] + sp[4] + sp[5], szz = sp[6] + sp[7] + sp[8];
  const double sxy = sp[9] + sp[10], sxz = sp[11] + sp[12], syz = sp[13] + sp[14];
  // s0 = initial stress + rdampk * stress rate (Voigt xx yy zz yz xz xy)
  const double sr[6] = {D[0][0], D[1][1], D[2][2], D[2][1] + D[1][2], D[2][0] + D[0][2], D[1][0] + D[0][1]};
  double s0[6];
  s0[0] = k.rdampk * (cd * sr[0] + lam * sr[1] + lam * sr[2]);
  s0[1] = k.rdampk * (lam * sr[0] + cd * sr[1] + lam * sr[2]);
  s0[2] = k.rdampk * (lam * sr[0] + lam * sr[1] + cd * sr[2]);
  s0[3] = k.rdampk * (mu * sr[3]);
  s0[4] = k.rdampk * (mu * sr[4]);
  s0[5] = k.rdampk * (mu * sr[5]);
  if (S0) {
#pragma unroll
    for (int i = 0; i < 6; ++i) s0[i] += g.stress0[i * ne + e];
  }
  const double dw = g.detw[e];
  double h[4][3];
  if (HG == 1) {
    const double s1 = g.ss[e], s2 = g.ss[ne + e], s3 = g.ss[2 * ne + e];
    const double s4 = g.ss[3 * ne + e], s5 = g.ss[4 * ne + e], s6 = g.ss[5 * ne + e];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      h[m][0] = s1 * ph[m][0] + s2 * ph[m][1] + s3 * ph[m][2];
      h[m][1] = s2 * ph[m][0] + s4 * ph[m][1] + s5 * ph[m][2];
      h[m][2] = s3 * ph[m][0] + s5 * ph[m][1] + s6 * ph[m][2];
    }
  } else {
    const double coef = g.hgcoef[e];
#pragma unroll
    for (int m = 0; m < 4; ++m)
      for (int c = 0; c < 3; ++c) h[m][c] = coef * ph[m][c];
  }
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double bx = __ldg(g.shp + (3 * a + 0) * ne + e);
    const double by = __ldg(g.shp + (3 * a + 1) * ne + e);
    const double bz = __ldg(g.shp + (3 * a + 2) * ne + e);
    const double wx = dw * bx, wy = dw * by, wz = dw * bz;
    double f9[9] = {-wx * sxx, -wy * sxy, -wz * sxz, -wx * sxy, -wy * syy,
                    -wz * syz, -wx * sxz, -wy * syz, -wz * szz};
    double fh[3] = {-(wx * s0[0] + wz * s0[4] + wy * s0[5]), -(wy * s0[1] + wz * s0[3] + wx * s0[5]),
                    -(wz * s0[2] + wy * s0[3] + wx * s0[4])};
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const double p = (HG == 1) ? __ldg(g.phi + (8 * m + a) * ne + e) : viscous_pattern(m, a);
#pragma unroll
      for (int c = 0; c < 3; ++c) fh[c] = fma(-p, h[m][c], fh[c]);
    }
    if (BODY) {
      const double em = g.em[a * ne + e];
      fh[0] -= em * (k.rdampm * vel[n[a]]);
      fh[1] -= em * (k.rdampm * vel[nnode + n[a]]);
      fh[2] -= em * (k.rdampm * vel[2 * nnode + n[a]] + k.gz);
    }
    const int node = n[a];
    if (node >= n_int) {
      const int slot = node - n_int;
#pragma unroll
      for (int j = 0; j < 9; ++j) atomicAdd(F9 + j * npml + slot, f9[j]);
#pragma unroll
      for (int c = 0; c < 3; ++c) atomicAdd(F + c * nnode + node, fh[c]);
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c)
        atomicAdd(F + c * nnode + node, f9[3 * c] + f9[3 * c + 1] + f9[3 * c + 2] + fh[c]);
    }
  }
}

template <bool BODY, bool PLASTIC, bool QM>
int launch_interior_hg(Context &c, cudaStream_t s, const ElemConst &k) {
  const int ne = c.gi64.ne;
  if (ne == 0) return EQD_OK;
  const int grid = (ne + kBlockElem - 1) / kBlockElem;
  if (c.sc.C_hg == 2)
    elem_interior_f64<BODY, PLASTIC, QM, 2><<<grid, kBlockElem, 0, s>>>(c.gi64, c.vel, c.disp, c.F, c.nnode, k);
  else
    elem_interior_f64<BODY, PLASTIC, QM, 1><<<grid, kBlockElem, 0, s>>>(c.gi64, c.vel, c.disp, c.F, c.nnode, k);
  return EQD_OK;
}

template <bool BODY, bool S0>
int launch_pml_hg(Context &c, cudaStream_t s, const ElemConst &k) {
  const int ne = c.gp64.ne;
  if (ne == 0) return EQD_OK;
  const int grid = (ne + kBlockElem - 1) / kBlockElem;
  if (c.sc.C_hg == 2)
    elem_pml_f64<BODY, S0, 2><<<grid, kBlockElem, 0, s>>>(c.gp64, c.vel, c.disp, c.F, c.F9, c.nnode,
                                                          c.n_int, c.npml, k);
  else
    elem_pml_f64<BODY, S0, 1><<<grid, kBlockElem, 0, s>>>(c.gp64, c.vel, c.disp, c.F, c.F9, c.nnode,
                                                          c.n_int, c.npml, k);
  return EQD_OK;
}

}  // namespace

ElemConst make_elem_const(const Context &c) {
  ElemConst k;
  const eqd_scalars &s = c.sc;
  k.dt = s.dt;
  k.rdampk = s.rdampk;
  k.rdampm = s.rdampm;
  k.gz = (1.0 - s.C_elastic) * s.grav * (s.roumax - (s.gamar + 1.0) * s.rhow) / (s.roumax != 0 ? s.roumax : 1.0);
  k.ccosphi = s.ccosphi;
  k.sinphi = s.sinphi;
  k.relax = (s.tv > 0) ? exp(-s.dt / s.tv) : 0.0;
  return k;
}

int launch_elements_f32(Context &c, cudaStream_t s, const ElemConst &k, int part);

int launch_elements(Context &c, cudaStream_t s, int part) {
  const ElemConst k = make_elem_const(c);
  if (c.fp32) return launch_elements_f32(c, s, k, part);
  const bool body = (c.sc.rdampm != 0.0) || (c.sc.C_elastic == 0);
  const bool plastic = (c.sc.C_elastic == 0);
  const bool qm = (c.sc.C_Q != 0);
  int rc = EQD_OK;
  if (part != 1) {
  if (qm && plastic) rc = body ? launch_interior_hg<true, true, true>(c, s, k) : launch_interior_hg<false, true, true>(c, s, k);
  else if (qm) rc = body ? launch_interior_hg<true, false, true>(c, s, k) : launch_interior_hg<false, false, true>(c, s, k);
  else if (plastic) rc = body ? launch_interior_hg<true, true, false>(c, s, k) : launch_interior_hg<false, true, false>(c, s, k);
  else rc = body ? launch_interior_hg<true, false, false>(c, s, k) : launch_interior_hg<false, false, false>(c, s, k);
  if (rc) return rc;
  }
  if (part != 0) {
    const bool s0 = c.gp64.stress0 != nullptr;
    if (body) rc = s0 ? launch_pml_hg<true, true>(c, s, k) : launch_pml_hg<true, false>(c, s, k);
    else rc = s0 ? launch_pml_hg<false, true>(c, s, k) : launch_pml_hg<false, false>(c, s, k);
    if (rc) return rc;
  }
  return cudaGetLastError() == cudaSuccess ? EQD_OK : EQD_ERR_CUDA;
}

}  // namespace eqd
