// Per-element tables of the one-point hexahedron, written once for the host case builder
// (case_builder.cpp, g++) and the device table build (setup_device.cu, nvcc with --fmad=false).
// Both compile this same source without floating-point contraction, so the two builds give the
// same bits.
//
// Restated from the reference's setup:
//   calcGlobalShapeFunc      src/calcGlobalShapeFunc.f90:1-75 (wedge column merge :21-28)
//   one-point local gradients src/calcLocalShapeFunc.f90
//   lumped element mass      src/assembleGlobalMass.f90:376-406
//   hourglass tables         calcSSPhi4Hrgls, src/assembleGlobalMass.f90:328-374
//   hexahedron volume        src/library.f90:60-93
#pragma once
#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define EQD_HD __host__ __device__
#else
#define EQD_HD
#endif

namespace eqd {
namespace geom {

// Hexahedron volume, the Flanagan-Belytschko form of src/library.f90:60-93: it(r, i) is node r of
// the permutation used for node i (src/library.f90:73-76).
EQD_HD inline double hex_volume(const double xl[3][8]) {
  const int it[8][8] = {{1, 2, 3, 4, 5, 6, 7, 8}, {2, 3, 4, 1, 6, 7, 8, 5}, {3, 4, 1, 2, 7, 8, 5, 6},
                        {4, 1, 2, 3, 8, 5, 6, 7}, {5, 8, 7, 6, 1, 4, 3, 2}, {6, 5, 8, 7, 2, 1, 4, 3},
                        {7, 6, 5, 8, 3, 2, 1, 4}, {8, 7, 6, 5, 4, 3, 2, 1}};
  double vol = 0.0;
  for (int i = 0; i < 8; ++i) {
    double Yv[9], Zv[9];
    for (int r = 1; r <= 8; ++r) {
      Yv[r] = xl[1][it[i][r - 1] - 1];
      Zv[r] = xl[2][it[i][r - 1] - 1];
    }
    const double b = Yv[2] * (Zv[6] - Zv[3] + Zv[5] - Zv[4]) + Yv[3] * (Zv[2] - Zv[4]) +
                     Yv[4] * (Zv[3] - Zv[8] + Zv[2] - Zv[5]) + Yv[5] * (Zv[8] - Zv[6] + Zv[4] - Zv[2]) +
                     Yv[6] * (Zv[5] - Zv[2]) + Yv[8] * (Zv[4] - Zv[5]);
    vol += xl[0][i] * b;
  }
  return vol / 12.0;
}

// Tables of one element from its corner coordinates xl[component][corner], its type (11 and 12
// are degenerated wedges) and its material row m = (vp, vs, rho, lambda, mu):
//   shp[3 k + q]  d N_k / d x_q at the centre        (eleshp(q, k))
//   det           Jacobian determinant               (eledet)
//   em[k]         lumped mass of corner k            (elemass(3 k + q), equal for q = 1..3)
//   ss[6]         hourglass stiffness                (ss)
//   phi[8 m + k]  hourglass base vector m at corner k (phi(k, m))
// Returns false (tables unset) for a non-positive determinant.
EQD_HD inline bool element_tables(const double xl[3][8], int et, const double m[5], double shp[24], double &det,
                                  double em[8], double ss[6], double phi[32]) {
  // one-point local derivatives (src/calcLocalShapeFunc.f90): corner signs
  const double sgn[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                            {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  const int ha[4][8] = {{1, 1, -1, -1, -1, -1, 1, 1}, {1, -1, -1, 1, -1, 1, 1, -1},
                        {1, -1, 1, -1, 1, -1, 1, -1}, {-1, 1, -1, 1, 1, -1, 1, -1}};
  const double w = 8.0;
  double g[4][8];
  for (int k = 0; k < 8; ++k) {
    for (int q = 0; q < 3; ++q) g[q][k] = sgn[k][q] / 8.0;
    g[3][k] = 1.0 / 8.0;
  }
  if (et == 11 || et == 12) {  // wedge column merge, src/calcGlobalShapeFunc.f90:21-28
    for (int r = 0; r < 4; ++r) {
      g[r][2] = g[r][2] + g[r][3];
      g[r][3] = 0.0;
      g[r][6] = g[r][6] + g[r][7];
      g[r][7] = 0.0;
    }
  }
  double xs[3][3];  // xs(j,i) = sum_k g(i,k) xl(j,k)
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double t = 0.0;
      for (int k = 0; k < 8; ++k) t += g[i][k] * xl[j][k];
      xs[j][i] = t;
    }
  const double c11 = xs[1][1] * xs[2][2] - xs[1][2] * xs[2][1];
  const double c12 = xs[1][2] * xs[2][0] - xs[1][0] * xs[2][2];
  const double c13 = xs[1][0] * xs[2][1] - xs[1][1] * xs[2][0];
  const double c21 = xs[2][1] * xs[0][2] - xs[2][2] * xs[0][1];
  const double c22 = xs[2][2] * xs[0][0] - xs[2][0] * xs[0][2];
  const double c23 = xs[2][0] * xs[0][1] - xs[2][1] * xs[0][0];
  const double c31 = xs[0][1] * xs[1][2] - xs[0][2] * xs[1][1];
  const double c32 = xs[0][2] * xs[1][0] - xs[0][0] * xs[1][2];
  const double c33 = xs[0][0] * xs[1][1] - xs[0][1] * xs[1][0];
  det = xs[0][0] * c11 + xs[0][1] * c12 + xs[0][2] * c13;
  if (!(det > 0.0)) return false;
  double gs[4][8];
  for (int k = 0; k < 8; ++k) {
    gs[0][k] = (g[0][k] * c11 + g[1][k] * c12 + g[2][k] * c13) / det;
    gs[1][k] = (g[0][k] * c21 + g[1][k] * c22 + g[2][k] * c23) / det;
    gs[2][k] = (g[0][k] * c31 + g[1][k] * c32 + g[2][k] * c33) / det;
    gs[3][k] = g[3][k];
  }
  // returned xs = cofactor matrix / det, column-major reshape of (c11,c12,c13,c21,...)
  const double xi[3][3] = {{c11 / det, c21 / det, c31 / det},
                           {c12 / det, c22 / det, c32 / det},
                           {c13 / det, c23 / det, c33 / det}};
  // lumped mass, src/assembleGlobalMass.f90:376-406
  const double totmas = m[2] * w * det;
  double work[8], dsum = 0.0;
  for (int k = 0; k < 8; ++k) {
    const double t2 = totmas * gs[3][k] * gs[3][k];
    dsum += t2;
    work[k] = t2;
  }
  const double t1 = totmas / dsum;
  for (int k = 0; k < 8; ++k) em[k] = t1 * work[k];
  for (int k = 0; k < 8; ++k)
    for (int q = 0; q < 3; ++q) shp[3 * k + q] = gs[q][k];
  // hourglass tables, src/assembleGlobalMass.f90:328-374
  const double vol = hex_volume(xl);
  double ce = m[4] * (3 * m[3] + 2 * m[4]) / (m[3] + m[4]);
  ce = 16.0 * ce / 15.0;
  const double co = ce * vol / 48.0;
  ss[0] = co * (xi[0][0] * xi[0][0] + xi[1][0] * xi[1][0] + xi[2][0] * xi[2][0]);
  ss[1] = co * (xi[0][0] * xi[0][1] + xi[1][0] * xi[1][1] + xi[2][0] * xi[2][1]);
  ss[2] = co * (xi[0][0] * xi[0][2] + xi[1][0] * xi[1][2] + xi[2][0] * xi[2][2]);
  ss[3] = co * (xi[0][1] * xi[0][1] + xi[1][1] * xi[1][1] + xi[2][1] * xi[2][1]);
  ss[4] = co * (xi[0][1] * xi[0][2] + xi[1][1] * xi[1][2] + xi[2][1] * xi[2][2]);
  ss[5] = co * (xi[0][2] * xi[0][2] + xi[1][2] * xi[1][2] + xi[2][2] * xi[2][2]);
  for (int mode = 0; mode < 4; ++mode) {
    double pm[8];
    for (int j = 0; j < 8; ++j) {
      double t = 0.0;
      for (int k = 0; k < 8; ++k)
        t += ha[mode][k] * (xl[0][k] * gs[0][j] + xl[1][k] * gs[1][j] + xl[2][k] * gs[2][j]);
      pm[j] = ha[mode][j] - t;
    }
    double nrm = 0.0;
    for (int j = 0; j < 8; ++j) nrm += pm[j] * pm[j];
    nrm = std::sqrt(nrm / 8.0);
    for (int j = 0; j < 8; ++j) phi[8 * mode + j] = pm[j] / nrm;
  }
  return true;
}

}  // namespace geom
}  // namespace eqd
