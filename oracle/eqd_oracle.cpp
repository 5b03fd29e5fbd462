// ORACLE — test infrastructure only.  A plain C++ binary64 restatement of EQdyna's per-time-step
// hot path, used by the tests, by __graft_entry__.smoke() and by the CPU-baseline leg of
// bench.py as the checker.  It is never linked into, loaded by or called from the product path
// (eqdyna_gb300/), which must fail loudly rather than fall back to this code.
//
// Parity is pinned: the oracle, fed by the case builder, is compared against the reference's
// own golden outputs test.reference.results/<case>/frt.txt* for the seven shipped cases
// (tests/test_oracle_golden.py).
//
// It operates in place on the Fortran globalvar arrays described by eqd_host_arrays and follows
// the reference loops statement by statement:
//   driver ............... src/driver.f90:9-34
//   velDispUpdate ........ src/driver.f90:89-155, comdampv src/comdampv.f90:1-120
//   storeOffFaultStData .. src/driver.f90:157-180
//   assembleGlobalKU ..... src/assembleGlobalKU.f90:3-67, calcPMLElemKU :70-346
//   calcElemKU ........... src/calcElemKU.f90:3-191 (calcB, calcElemMass inlined)
//   qconstant ............ src/qconstant.f90:3-35
//   hrglss ............... src/hrglss.f90:3-100
//   faulting ............. src/faulting.f90:3-541, friction laws src/fric.f90:3-95
//   thermop .............. src/thermop.f90:1-40
// Optional OpenMP: elements are greedily coloured so that no two elements of one colour share
// a node; each colour is a parallel loop.  With one thread the loops run in the reference order.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/eqdyna_gb300.h"

namespace {

struct Oracle {
  eqd_scalars s;
  eqd_host_arrays a;
  double timeElapsed;
  int nthreads;
  int64_t newton_iters = 0, newton_maxhits = 0;
  std::vector<std::vector<int32_t>> colours;  // element ids (0-based) per colour
  std::vector<double> patnode, Tatnode;
  // Newton logging (initial-guess training data): per solve, 6 features + converged V
  std::vector<double> *log = nullptr;
  int64_t log_cap = 0;
};

// ---- Fortran-view accessors (1-based indices) ------------------------------------------------
struct View {
  Oracle &o;
  const eqd_scalars &s;
  eqd_host_arrays &a;
  explicit View(Oracle &x) : o(x), s(x.s), a(x.a) {}
  int conn(int k, int e) const { return a.nodeElemIdRelation[8 * (size_t)(e - 1) + (k - 1)]; }
  int eqidx(int loc) const { return a.eqNumIndexArr[loc - 1]; }       // eqNumIndexArr(loc)
  int eq(int node, int j) const { return eqidx(a.eqNumStartIndexLoc[node - 1] + j); }
  int ndof(int node) const { return a.numOfDofPerNodeArr[node - 1]; }
  double &F(int e) { return a.nodalForceArr[e - 1]; }
  double &V1(int e) { return a.v1[e - 1]; }
  double &vel(int k, int n) { return a.velArr[3 * (size_t)(n - 1) + (k - 1)]; }
  double &disp(int k, int n) { return a.dispArr[3 * (size_t)(n - 1) + (k - 1)]; }
  double xc(int k, int n) const { return a.meshCoor[3 * (size_t)(n - 1) + (k - 1)]; }
  double shp(int k, int i, int e) const { return a.eleshp[24 * (size_t)(e - 1) + 3 * (i - 1) + (k - 1)]; }
  double mat(int e, int k) const { return a.mat[(size_t)(k - 1) * a.nelem + (e - 1)]; }
  double phi(int j, int m, int e) const { return a.phi[32 * (size_t)(e - 1) + 8 * (m - 1) + (j - 1)]; }
  double ss(int k, int e) const { return a.ss[6 * (size_t)(e - 1) + (k - 1)]; }
  double elemass(int k, int e) const { return a.elemass[24 * (size_t)(e - 1) + (k - 1)]; }
  double &fric(int k, int i) { return a.fric[100 * (size_t)(i - 1) + (k - 1)]; }
  int nsmp(int j, int i) const { return a.nsmp[2 * (size_t)(i - 1) + (j - 1)]; }
  double un(int k, int i) const { return a.un[3 * (size_t)(i - 1) + (k - 1)]; }
  double us(int k, int i) const { return a.us[3 * (size_t)(i - 1) + (k - 1)]; }
  double ud(int k, int i) const { return a.ud[3 * (size_t)(i - 1) + (k - 1)]; }
};

// ---- src/comdampv.f90:1-120 (the node damping profile; the element profile in
//      calcPMLElemKU is the same with strict inequalities) ---------------------------------------
void damping_profile(const eqd_scalars &s, double x, double y, double z, bool strict, double d[3]) {
  const double xmax0 = s.PMLb[0], xmin0 = s.PMLb[1], ymax0 = s.PMLb[2], ymin0 = s.PMLb[3];
  const double zmin0 = s.PMLb[4];
  auto ge = [&](double p, double q) { return strict ? (p > q) : (p >= q); };
  auto le = [&](double p, double q) { return strict ? (p < q) : (p <= q); };
  bool lower = strict ? (z < zmin0) : (z <= zmin0);
  bool upper = strict ? (z > zmin0) : (z > zmin0);
  d[0] = d[1] = d[2] = 0.0;
  if (!lower && !upper) return;  // z == zmin0 with strict tests: damps untouched (zero-initialised)
  d[2] = lower ? std::fabs(z - zmin0) : 0.0;
  if (ge(x, xmax0) && ge(y, ymax0)) {
    d[0] = std::fabs(x - xmax0); d[1] = std::fabs(y - ymax0);
  } else if (ge(x, xmax0) && le(y, ymin0)) {
    d[0] = std::fabs(x - xmax0); d[1] = std::fabs(y - ymin0);
  } else if (le(x, xmin0) && le(y, ymin0)) {
    d[0] = std::fabs(x - xmin0); d[1] = std::fabs(y - ymin0);
  } else if (le(x, xmin0) && ge(y, xmax0)) {  // the reference compares y with xmax here
    d[0] = std::fabs(x - xmin0); d[1] = std::fabs(y - ymax0);
  } else if (ge(x, xmax0) && y > ymin0 && y < ymax0) {
    d[0] = std::fabs(x - xmax0); d[1] = 0.0;
  } else if (le(y, ymin0) && x > xmin0 && x < xmax0) {
    d[0] = 0.0; d[1] = std::fabs(y - ymin0);
  } else if (le(x, xmin0) && y > ymin0 && y < ymax0) {
    d[0] = std::fabs(x - xmin0); d[1] = 0.0;
  } else if (ge(y, ymax0) && x > xmin0 && x < xmax0) {
    d[0] = 0.0; d[1] = std::fabs(y - ymax0);
  } else {
    d[0] = 0.0; d[1] = 0.0;
  }
}

void damping_values(const eqd_scalars &s, double d[3], bool node_form) {
  const double maxd[3] = {s.PMLb[5], s.PMLb[6], s.PMLb[7]};
  for (int i = 0; i < 3; ++i) {
    const double delta = s.nPML * maxd[i];
    if (node_form)
      d[i] = 3.0 * s.vmaxPML / 2.0 / delta * std::log(1.0 / s.R) * std::pow(d[i] / delta, 2.0);
    else
      d[i] = 3 * s.vmaxPML / 2 / delta * std::log(1 / s.R) * std::pow(d[i] / delta, 2.0);
  }
}

// ---- src/driver.f90:89-155 ------------------------------------------------------------------
int vel_disp_update(Oracle &o) {
  View v(o);
  const double dt = o.s.dt;
  int status = EQD_OK;
  const int nn = o.a.nnode;
#pragma omp parallel for num_threads(o.nthreads) schedule(static) reduction(max : status)
  for (int i = 1; i <= nn; ++i) {
    if (v.ndof(i) == 3) {
      for (int j = 1; j <= 3; ++j) {
        const int e = v.eq(i, j);
        v.V1(e) = v.V1(e) + v.F(e) * dt;
        v.vel(j, i) = v.V1(e);
        v.disp(j, i) = v.disp(j, i) + v.V1(e) * dt;
      }
    } else if (v.ndof(i) == 12) {
      double dampv[9] = {0};
      if (v.eq(i, 1) > 0) {
        double d[3];
        damping_profile(o.s, v.xc(1, i), v.xc(2, i), v.xc(3, i), false, d);
        damping_values(o.s, d, true);
        for (int k = 0; k < 9; ++k) dampv[k] = d[k % 3];
      }
      for (int j = 1; j <= 9; ++j) {
        const int e = v.eq(i, j);
        if (e > 0)
          v.V1(e) = (v.F(e) + v.V1(e) * (1.0 / dt - dampv[j - 1] / 2.0)) / (1.0 / dt + dampv[j - 1] / 2.0);
      }
      for (int j = 10; j <= 12; ++j) {
        const int e = v.eq(i, j);
        if (e > 0) v.V1(e) = v.V1(e) + v.F(e) * dt;
      }
      const int e1 = v.eq(i, 1);
      if (e1 > 0) {
        v.vel(1, i) = v.V1(v.eq(i, 1)) + v.V1(v.eq(i, 2)) + v.V1(v.eq(i, 3)) + v.V1(v.eq(i, 10));
        v.vel(2, i) = v.V1(v.eq(i, 4)) + v.V1(v.eq(i, 5)) + v.V1(v.eq(i, 6)) + v.V1(v.eq(i, 11));
        v.vel(3, i) = v.V1(v.eq(i, 7)) + v.V1(v.eq(i, 8)) + v.V1(v.eq(i, 9)) + v.V1(v.eq(i, 12));
        for (int k = 1; k <= 3; ++k) v.disp(k, i) = v.disp(k, i) + v.vel(k, i) * dt;
      } else if (e1 == -1) {
        for (int k = 1; k <= 3; ++k) v.vel(k, i) = 0.0, v.disp(k, i) = 0.0;
      }
    }
    if (std::isnan(v.vel(1, i)) || std::isnan(v.vel(2, i)) || std::isnan(v.vel(3, i))) status = EQD_ERR_NAN;
  }
  return status;
}

// ---- src/driver.f90:157-180 ------------------------------------------------------------------
void store_off_fault(Oracle &o, int nt) {
  View v(o);
  const int n = o.a.numOffFaultSt * 6;
  if (n <= 0 || !o.a.OffFaultStGramSCEC || nt < 1 || nt > o.s.nstep) return;  // rows exist for 1..nstep
  double *g = o.a.OffFaultStGramSCEC + (size_t)(n + 1) * (nt - 1);
  g[0] = o.timeElapsed;
  for (int i = 1; i <= n; ++i) {
    const int node = o.a.idhist[3 * (i - 1)], k = o.a.idhist[3 * (i - 1) + 1], q = o.a.idhist[3 * (i - 1) + 2];
    if (q == 1) g[i] = v.disp(k, node);
    else if (q == 2) g[i] = v.vel(k, node);
    else if (q == 3) g[i] = v.F(v.eq(node, k));
  }
}

// ---- src/qconstant.f90:3-35 ------------------------------------------------------------------
void qconstant(double Q, int k, double &rtaok, double &rwk, double &c1) {
  // relaxation times and weights of the 8 mechanisms (Liu & Archuleta 2006), single-precision
  // literals in the reference
  static const float taok[8] = {1.72333e-3f, 1.80701e-3f, 5.38887e-3f, 1.99322e-2f,
                                8.49833e-2f, 4.09335e-1f, 2.05951f, 13.2629f};
  static const float alfk[8] = {1.66958e-2f, 3.81644e-2f, 9.84666e-3f, -1.36803e-2f,
                                -2.85125e-2f, -5.37309e-2f, -6.65035e-2f, -1.33696e-1f};
  static const float betk[8] = {8.98758e-2f, 6.84635e-2f, 9.67052e-2f, 1.20172e-1f,
                                1.30728e-1f, 1.38746e-1f, 1.40705e-1f, 2.14647e-1f};
  const double pi = 4.0 * std::atan(1.0);
  double kapa = 3.071f + 1.433f * std::pow(Q, (double)-1.158f) * std::log(Q / 5);
  kapa = kapa / (1 + 0.415f * Q);
  rwk = kapa * (kapa * (double)alfk[k - 1] + (double)betk[k - 1]);
  rtaok = taok[k - 1];
  const double ref = 2.0 * pi;
  const double ak0 = 1.0 - rwk * 8.0 / (1.0 + (rtaok * ref) * (rtaok * ref));
  const double bk0 = rwk * 8.0 * ref * rtaok / (1.0 + (rtaok * ref) * (rtaok * ref));
  c1 = 0.5 * std::pow(ak0 * ak0 + bk0 * bk0, -0.5);
  c1 = c1 * (1.0 + ak0 * std::pow(ak0 * ak0 + bk0 * bk0, -0.5));
}

// ---- src/calcElemKU.f90:3-191 ----------------------------------------------------------------
void calc_elem_ku(Oracle &o, int nel, double elresf[24], double &pstrinc_mag) {
  View v(o);
  const eqd_scalars &s = o.s;
  const double dt = s.dt;
  double *stress = o.a.stressArr + o.a.stressCompIndexArr[nel - 1];  // stress(1..12) = stress[0..11]
  const double lam = v.mat(nel, 4), miu = v.mat(nel, 5);
  double vl[24], dl[24];
  for (int i = 1; i <= 8; ++i)
    for (int j = 1; j <= 3; ++j) {
      vl[3 * (i - 1) + j - 1] = v.vel(j, v.conn(i, nel));
      dl[3 * (i - 1) + j - 1] = v.disp(j, v.conn(i, nel));
    }
  double sr[6] = {0}, sn[6] = {0};
  for (int i = 1; i <= 8; ++i) {
    const double bx = v.shp(1, i, nel), by = v.shp(2, i, nel), bz = v.shp(3, i, nel);
    const double *vv = &vl[3 * (i - 1)], *dd = &dl[3 * (i - 1)];
    sr[0] += bx * vv[0];
    sr[1] += by * vv[1];
    sr[2] += bz * vv[2];
    sr[3] = sr[3] + bz * vv[1] + by * vv[2];
    sr[4] = sr[4] + bz * vv[0] + bx * vv[2];
    sr[5] = sr[5] + by * vv[0] + bx * vv[1];
    sn[0] += bx * dd[0];
    sn[1] += by * dd[1];
    sn[2] += bz * dd[2];
    sn[3] = sn[3] + bz * dd[1] + by * dd[2];
    sn[4] = sn[4] + bz * dd[0] + bx * dd[2];
    sn[5] = sn[5] + by * dd[0] + bx * dd[1];
  }
  const double cd = lam + 2 * miu;
  double srate[6];
  srate[0] = cd * sr[0] + lam * sr[1] + lam * sr[2];
  srate[1] = lam * sr[0] + cd * sr[1] + lam * sr[2];
  srate[2] = lam * sr[0] + lam * sr[1] + cd * sr[2];
  srate[3] = miu * sr[3];
  srate[4] = miu * sr[4];
  srate[5] = miu * sr[5];
  double strdev[6];
  if (s.C_Q == 0) {
    for (int i = 0; i < 6; ++i) {
      stress[i] = stress[i] + srate[i] * dt;
      strdev[i] = stress[i];
    }
  } else {
    double ctr[3] = {0, 0, 0};
    for (int i = 1; i <= 3; ++i)
      for (int j = 1; j <= 8; ++j) ctr[i - 1] += v.xc(i, v.conn(j, nel));
    for (double &c : ctr) c = c / 8.0;
    double Qs, Qp;
    if (s.C_Q == 2) {  // extension: Qs = 50 Vs (km/s), Qp = 2 Qs
      Qs = 50.0 * v.mat(nel, 2) / 1000.0;
      Qp = 2.0 * Qs;
    } else if (ctr[2] > -1000.0) {
      Qs = 10.0;
      Qp = 20.0;
    } else {
      Qs = 50.0;
      Qp = 100.0;
    }
    const int ip = (int)((ctr[0] - (s.PMLb[1] + s.dx / 2)) / s.dx + 1);
    const int iq = (int)((ctr[1] - (s.PMLb[3] + s.dx / 2)) / s.dx + 1);
    const int ir = (int)((ctr[2] - (s.PMLb[4] + s.dx / 2)) / s.dx + 1);
    const int k = 1 + ip % 2 + 2 * (iq % 2) + 4 * (ir % 2);
    double taok, wkp, wks, cv, cs;
    qconstant(Qp, k, taok, wkp, cv);
    qconstant(Qs, k, taok, wks, cs);
    wkp = wkp * 8.0;
    wks = wks * 8.0;
    const double miuu = miu * cs, Mu = (lam + 2 * miu) * cv;
    const double vols = sn[0] + sn[1] + sn[2];
    double an1[6], an[6];
    for (int i = 0; i < 6; ++i) an1[i] = stress[i + 6];
    const double ex = std::exp(-dt / taok);
    for (int i = 0; i < 3; ++i) an[i] = ex * an1[i] + (1 - ex) * (2 * miuu * sn[i] * wks + (Mu * wkp - 2 * miuu * wks) * vols);
    for (int i = 3; i < 6; ++i) an[i] = ex * an1[i] + (1 - ex) * (miuu * sn[i] * wks);
    for (int i = 0; i < 6; ++i) stress[i + 6] = an[i];
    for (int i = 0; i < 3; ++i) stress[i] = 2.0 * miuu * sn[i] + (Mu - 2.0 * miuu) * vols - 0.5 * (an[i] + an1[i]);
    for (int i = 3; i < 6; ++i) stress[i] = 2.0 * miuu * sn[i] / 2.0 - 0.5 * (an[i] + an1[i]);
  }
  pstrinc_mag = 0.0;
  if (s.C_elastic == 0) {
    const double porep = o.a.eleporep[nel - 1];
    const double strmea = (stress[0] + stress[1] + stress[2]) / 3.0;
    for (int i = 0; i < 3; ++i) strdev[i] = stress[i] - strmea;
    if (s.C_Q != 0)
      for (int i = 3; i < 6; ++i) strdev[i] = stress[i];
    double taomax = 0.5 * (strdev[0] * strdev[0] + strdev[1] * strdev[1] + strdev[2] * strdev[2]) +
                    strdev[3] * strdev[3] + strdev[4] * strdev[4] + strdev[5] * strdev[5];
    taomax = std::sqrt(taomax);
    double yield = s.ccosphi - s.sinphi * (strmea + porep);
    if (yield < 0.0) yield = 0.0;
    if (taomax > yield) {
      const double rjust = yield / taomax + (1 - yield / taomax) * std::exp(-dt / s.tv);
      double pinc[6];
      for (int i = 0; i < 6; ++i) {
        stress[i] = strdev[i] * rjust;
        pinc[i] = (strdev[i] - stress[i]) / miu;
        if (i < 3) stress[i] = stress[i] + strmea;
      }
      const double pm = (pinc[0] + pinc[1] + pinc[2]) / 3.0;
      for (double &p : pinc) p = p - pm;
      double mag = 0.5 * (pinc[0] * pinc[0] + pinc[1] * pinc[1] + pinc[2] * pinc[2]) + pinc[3] * pinc[3] +
                   pinc[4] * pinc[4] + pinc[5] * pinc[5];
      pstrinc_mag = std::sqrt(mag);
    }
  }
  const double temp = -o.a.eledet[nel - 1] * s.w;
  double st[6];
  for (int i = 0; i < 6; ++i) st[i] = temp * (stress[i] + s.rdampk * srate[i]);
  for (int i = 1; i <= 8; ++i) {
    const double bx = v.shp(1, i, nel), by = v.shp(2, i, nel), bz = v.shp(3, i, nel);
    elresf[3 * (i - 1) + 0] += bx * st[0] + bz * st[4] + by * st[5];
    elresf[3 * (i - 1) + 1] += by * st[1] + bz * st[3] + bx * st[5];
    elresf[3 * (i - 1) + 2] += bz * st[2] + by * st[3] + bx * st[4];
  }
}

// ---- src/assembleGlobalKU.f90:70-346 ---------------------------------------------------------
void calc_pml_elem_ku(Oracle &o, int nel, double f[96]) {
  View v(o);
  const eqd_scalars &s = o.s;
  const double dt = s.dt;
  double *st = o.a.stressArr + o.a.stressCompIndexArr[nel - 1];  // s(1..21) = st[0..20]
  const double lam = v.mat(nel, 4), miu = v.mat(nel, 5);
  const double det = o.a.eledet[nel - 1];
  double ctr[3] = {0, 0, 0};
  for (int i = 1; i <= 3; ++i)
    for (int j = 1; j <= 8; ++j) ctr[i - 1] += v.xc(i, v.conn(j, nel));
  for (double &c : ctr) c = c / 8;
  double damps[3];
  damping_profile(s, ctr[0], ctr[1], ctr[2], true, damps);
  damping_values(s, damps, false);
  double va[24];
  for (int i = 1; i <= 8; ++i)
    for (int j = 1; j <= 3; ++j) va[3 * (i - 1) + j - 1] = v.vel(j, v.conn(i, nel));
  double sr[6] = {0};
  for (int i = 1; i <= 8; ++i) {
    const double bx = v.shp(1, i, nel), by = v.shp(2, i, nel), bz = v.shp(3, i, nel);
    const double *vv = &va[3 * (i - 1)];
    sr[0] += bx * vv[0];
    sr[1] += by * vv[1];
    sr[2] += bz * vv[2];
    sr[3] = sr[3] + bz * vv[1] + by * vv[2];
    sr[4] = sr[4] + bz * vv[0] + bx * vv[2];
    sr[5] = sr[5] + by * vv[0] + bx * vv[1];
  }
  double srate[6];
  srate[0] = (lam + 2.0 * miu) * sr[0] + lam * sr[1] + lam * sr[2];
  srate[1] = lam * sr[0] + (lam + 2.0 * miu) * sr[1] + lam * sr[2];
  srate[2] = lam * sr[0] + lam * sr[1] + (lam + 2.0 * miu) * sr[2];
  srate[3] = miu * sr[3];
  srate[4] = miu * sr[4];
  srate[5] = miu * sr[5];
  double D[3][3] = {{0}};  // D[a][b] = d v_b / d x_a  (Dx_vy = D[0][1])
  for (int i = 1; i <= 8; ++i)
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) D[a][b] += v.shp(a + 1, i, nel) * va[3 * (i - 1) + b];
  const double Dx_vx = D[0][0], Dy_vy = D[1][1], Dz_vz = D[2][2], Dx_vy = D[0][1], Dy_vx = D[1][0];
  const double Dx_vz = D[0][2], Dz_vx = D[2][0], Dy_vz = D[1][2], Dz_vy = D[2][1];
  auto upd = [&](int idx, double src, int ax) {
    st[idx] = src + (1 / dt - damps[ax] / 2) * st[idx];
    st[idx] = st[idx] / (1 / dt + damps[ax] / 2);
  };
  upd(0, (lam + 2 * miu) * Dx_vx, 0);
  upd(1, lam * Dy_vy, 1);
  upd(2, lam * Dz_vz, 2);
  upd(3, lam * Dx_vx, 0);
  upd(4, (lam + 2 * miu) * Dy_vy, 1);
  upd(5, lam * Dz_vz, 2);
  upd(6, lam * Dx_vx, 0);
  upd(7, lam * Dy_vy, 1);
  upd(8, (lam + 2 * miu) * Dz_vz, 2);
  upd(9, miu * Dx_vy, 0);
  upd(10, miu * Dy_vx, 1);
  upd(11, miu * Dx_vz, 0);
  upd(12, miu * Dz_vx, 2);
  upd(13, miu * Dy_vz, 1);
  upd(14, miu * Dz_vy, 2);
  const double sxx = st[0] + st[1] + st[2], syy = st[3] + st[4] + st[5], szz = st[6] + st[7] + st[8];
  const double sxy = st[9] + st[10], sxz = st[11] + st[12], syz = st[13] + st[14];
  double s0[6];
  for (int i = 0; i < 6; ++i) s0[i] = st[15 + i] + s.rdampk * srate[i];
  const double dw = det * s.w;
  for (int i = 1; i <= 8; ++i) {
    const double bx = v.shp(1, i, nel), by = v.shp(2, i, nel), bz = v.shp(3, i, nel);
    double *g = &f[12 * (i - 1)];
    g[0] = g[0] - dw * bx * sxx;
    g[1] = g[1] - dw * by * sxy;
    g[2] = g[2] - dw * bz * sxz;
    g[3] = g[3] - dw * bx * sxy;
    g[4] = g[4] - dw * by * syy;
    g[5] = g[5] - dw * bz * syz;
    g[6] = g[6] - dw * bx * sxz;
    g[7] = g[7] - dw * by * syz;
    g[8] = g[8] - dw * bz * szz;
    g[9] = g[9] - dw * (bx * s0[0] + bz * s0[4] + by * s0[5]);
    g[10] = g[10] - dw * (by * s0[1] + bz * s0[3] + bx * s0[5]);
    g[11] = g[11] - dw * (bz * s0[2] + by * s0[3] + bx * s0[4]);
  }
}

// one element of assembleGlobalKU (src/assembleGlobalKU.f90:13-64)
void assemble_element(Oracle &o, int nel) {
  View v(o);
  const eqd_scalars &s = o.s;
  double al[24];
  for (int i = 1; i <= 8; ++i)
    for (int j = 1; j <= 3; ++j) al[3 * (i - 1) + j - 1] = s.rdampm * v.vel(j, v.conn(i, nel));
  for (int i = 1; i <= 8; ++i)
    al[3 * (i - 1) + 2] = al[3 * (i - 1) + 2] + (1.0 - s.C_elastic) * s.grav * (s.roumax - (s.gamar + 1.0) * s.rhow) / s.roumax;
  double elresf[24];
  for (int k = 0; k < 24; ++k) elresf[k] = 0.0 - al[k] * v.elemass(k + 1, nel);
  const int et = o.a.elemTypeArr[nel - 1];
  if (et == 1 || et > 10) {
    double pinc;
    calc_elem_ku(o, nel, elresf, pinc);
    o.a.pstrain[nel - 1] = o.a.pstrain[nel - 1] + pinc;
    for (int i = 1; i <= 8; ++i)
      for (int j = 1; j <= 3; ++j) {
        const int e = v.eq(v.conn(i, nel), j);
        if (e > 0) v.F(e) = v.F(e) + elresf[3 * (i - 1) + j - 1];
      }
  } else if (et == 2) {
    double f[96] = {0};
    for (int i = 1; i <= 8; ++i)
      for (int j = 1; j <= 3; ++j) f[12 * (i - 1) + 9 + j - 1] = elresf[3 * (i - 1) + j - 1];
    calc_pml_elem_ku(o, nel, f);
    for (int i = 1; i <= 8; ++i) {
      const int node = v.conn(i, nel);
      const double *g = &f[12 * (i - 1)];
      if (v.ndof(node) == 12) {
        for (int j = 1; j <= 12; ++j) {
          const int e = v.eq(node, j);
          if (e > 0) v.F(e) = v.F(e) + g[j - 1];
        }
      } else if (v.ndof(node) == 3) {
        int e = v.eq(node, 1);
        v.F(e) = v.F(e) + g[0] + g[1] + g[2] + g[9];
        e = v.eq(node, 2);
        v.F(e) = v.F(e) + g[3] + g[4] + g[5] + g[10];
        e = v.eq(node, 3);
        v.F(e) = v.F(e) + g[6] + g[7] + g[8] + g[11];
      }
    }
  }
}

// one element of hrglss (src/hrglss.f90:13-98)
void hourglass_element(Oracle &o, int nel) {
  View v(o);
  const eqd_scalars &s = o.s;
  double vl[3][8], dl[3][8];
  for (int i = 1; i <= 8; ++i)
    for (int j = 1; j <= 3; ++j) {
      vl[j - 1][i - 1] = v.vel(j, v.conn(i, nel));
      dl[j - 1][i - 1] = v.disp(j, v.conn(i, nel)) + s.rdampk * vl[j - 1][i - 1];
    }
  auto target = [&](int node, int j) {
    int itag = 0;
    if (v.ndof(node) == 3) itag = o.a.eqNumStartIndexLoc[node - 1] + j;
    else if (v.ndof(node) == 12) itag = o.a.eqNumStartIndexLoc[node - 1] + j + 9;
    return v.eqidx(itag);
  };
  if (s.C_hg == 1) {
    for (int m = 1; m <= 4; ++m) {
      double phid[3];
      for (int i = 0; i < 3; ++i) {
        phid[i] = 0.0;
        for (int j = 1; j <= 8; ++j) phid[i] = phid[i] + v.phi(j, m, nel) * dl[i][j - 1];
      }
      const double s1 = v.ss(1, nel), s2 = v.ss(2, nel), s3 = v.ss(3, nel);
      const double s4 = v.ss(4, nel), s5 = v.ss(5, nel), s6 = v.ss(6, nel);
      double fhr[3][8];
      for (int i = 1; i <= 8; ++i) {
        const double p = v.phi(i, m, nel);
        fhr[0][i - 1] = p * (s1 * phid[0] + s2 * phid[1] + s3 * phid[2]);
        fhr[1][i - 1] = p * (s2 * phid[0] + s4 * phid[1] + s5 * phid[2]);
        fhr[2][i - 1] = p * (s3 * phid[0] + s5 * phid[1] + s6 * phid[2]);
      }
      for (int i = 1; i <= 8; ++i)
        for (int j = 1; j <= 3; ++j) {
          const int k = target(v.conn(i, nel), j);
          if (k > 0) v.F(k) = v.F(k) - fhr[j - 1][i - 1];
        }
    }
  } else if (s.C_hg == 2) {
    const double coef = 0.25 * s.kapa_hg * v.mat(nel, 3) * v.mat(nel, 1) *
                        std::pow(o.a.eledet[nel - 1] * s.w, 2.0 / 3.0);
    static const int fi[4][8] = {{1, 1, -1, -1, -1, -1, 1, 1}, {1, -1, -1, 1, -1, 1, 1, -1},
                                 {1, -1, 1, -1, 1, -1, 1, -1}, {1, -1, 1, -1, -1, 1, -1, 1}};
    double q[3][4] = {{0}};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 8; ++k) q[i][j] = q[i][j] + vl[i][k] * fi[j][k];
    double f[24] = {0};
    for (int k = 0; k < 8; ++k)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 4; ++j) f[3 * k + i] = f[3 * k + i] - coef * q[i][j] * fi[j][k];
    for (int i = 1; i <= 8; ++i)
      for (int j = 1; j <= 3; ++j) {
        const int k = target(v.conn(i, nel), j);
        if (k > 0) v.F(k) = v.F(k) + f[3 * (i - 1) + j - 1];
      }
  }
}

// ---- friction laws, src/fric.f90:3-95 --------------------------------------------------------
double slip_weak(double slip, const double *fr) {  // fr[k] == fricsgl(k)
  double xmu = 0.0;
  if (std::fabs(slip) < 1.0e-10) xmu = fr[1];
  else if (slip < fr[3]) xmu = fr[1] - (fr[1] - fr[2]) * slip / fr[3];
  if (slip >= fr[3]) xmu = fr[2];
  return xmu;
}

double time_weak(double trupt, const double *fr) {
  if (trupt <= 0.0) return fr[1];
  if (trupt < fr[5]) return fr[1] - (fr[1] - fr[2]) * trupt / fr[5];
  return fr[2];
}

void rsf_aging(double V2, double &theta, const double *fr, double dt, double &xmu, double &dxmudv) {
  const double A = fr[9], B = fr[10], L = fr[11], f0 = fr[13], V0 = fr[12];
  const double tmpc = 1.0 / (2.0 * V0) * std::exp((f0 + B * std::log(V0 * theta / L)) / A);
  const double tmp = (V2 + 1.e-30) * tmpc;
  xmu = A * std::log(tmp + std::sqrt(tmp * tmp + 1.0));
  dxmudv = A * tmpc / std::sqrt(1.0 + tmp * tmp);
  theta = L / V2 + (theta - L / V2) * std::exp(-V2 * dt / L);
}

void rsf_slip(double V2, double &psi, const double *fr, double dt, double &xmu, double &dxmudv) {
  const double A = fr[9], B = fr[10], L = fr[11], f0 = fr[13], V0 = fr[12], fw = fr[14], Vw = fr[15];
  const double tmpc = 1.0 / (2.0 * V0) * std::exp(psi / A);
  const double tmp = (V2 + 1.e-30) * tmpc;
  xmu = A * std::log(tmp + std::sqrt(tmp * tmp + 1.0));
  dxmudv = A * tmpc / std::sqrt(1.0 + tmp * tmp);
  const double fLV = f0 - (B - A) * std::log(V2 / V0);
  const double fss = fw + (fLV - fw) / std::pow(1.0 + std::pow(V2 / Vw, 8), 0.125);
  const double fssa = fss / A;
  const double psiss = A * std::log(2.0 * V0 / V2 * (std::exp(fssa) - std::exp(-fssa)) / 2.0);
  psi = psiss + (psi - psiss) * std::exp(-V2 * dt / L);
}

void rsf_law(int friclaw, double V2, double &state, const double *fr, double dt, double &xmu, double &dxmudv) {
  if (friclaw == 3) rsf_aging(V2, state, fr, dt, xmu, dxmudv);
  else rsf_slip(V2, state, fr, dt, xmu, dxmudv);
}

// ---- src/faulting.f90 ------------------------------------------------------------------------
void fault_pair(Oracle &o, int i, int nt) {
  View v(o);
  const eqd_scalars &s = o.s;
  const double dt = s.dt, t = o.timeElapsed;
  double *fr = &v.fric(1, i) - 1;  // fr[k] == fric(k,i)
  const int sl = v.nsmp(1, i), ms = v.nsmp(2, i);
  // getNsdSlipSliprateTraction, :54-134
  const double dtau = 0.0;
  double init[3] = {fr[7], fr[8] + dtau, fr[49]};
  const double mS = o.a.fnms[sl - 1], mM = o.a.fnms[ms - 1];
  const double totalMass = (mS + mM) * o.a.arn[i - 1];
  double xyz[3][2][3];  // xyz[k][j][q]: component k, node j (slave, master), quantity q
  for (int j = 0; j < 2; ++j) {
    const int node = (j == 0) ? sl : ms;
    for (int k = 1; k <= 3; ++k) {
      xyz[k - 1][j][0] = v.F(v.eq(node, k));
      xyz[k - 1][j][1] = v.vel(k, node);
      xyz[k - 1][j][2] = v.disp(k, node);
    }
  }
  double nsd[3][2][3];
  for (int q = 0; q < 3; ++q)
    for (int j = 0; j < 2; ++j) {
      nsd[0][j][q] = xyz[0][j][q] * v.un(1, i) + xyz[1][j][q] * v.un(2, i) + xyz[2][j][q] * v.un(3, i);
      nsd[1][j][q] = xyz[0][j][q] * v.us(1, i) + xyz[1][j][q] * v.us(2, i) + xyz[2][j][q] * v.us(3, i);
      nsd[2][j][q] = xyz[0][j][q] * v.ud(1, i) + xyz[1][j][q] * v.ud(2, i) + xyz[2][j][q] * v.ud(3, i);
    }
  double slip[4], rate[4], tr[4];
  for (int j = 0; j < 3; ++j) slip[j] = nsd[j][1][2] - nsd[j][0][2];
  slip[3] = std::sqrt(slip[0] * slip[0] + slip[1] * slip[1] + slip[2] * slip[2]);
  for (int j = 0; j < 3; ++j) rate[j] = nsd[j][1][1] - nsd[j][0][1];
  rate[3] = std::sqrt(rate[0] * rate[0] + rate[1] * rate[1] + rate[2] * rate[2]);
  fr[71] = slip[1];
  fr[72] = slip[2];
  fr[73] = slip[0];
  fr[74] = rate[1];
  fr[75] = rate[2];
  if (rate[3] > fr[76]) fr[76] = rate[3];
  fr[77] = fr[77] + rate[3] * dt;
  tr[0] = (mS * mM * ((nsd[0][1][1] - nsd[0][0][1]) + (nsd[0][1][2] - nsd[0][0][2]) / dt) / dt +
           mS * nsd[0][1][0] - mM * nsd[0][0][0]) / totalMass + init[0] * s.C_elastic;
  tr[1] = (mS * mM * (nsd[1][1][1] - nsd[1][0][1]) / dt + mS * nsd[1][1][0] - mM * nsd[1][0][0]) / totalMass +
          init[1] * s.C_elastic;
  tr[2] = (mS * mM * (nsd[2][1][1] - nsd[2][0][1]) / dt + mS * nsd[2][1][0] - mM * nsd[2][0][0]) / totalMass +
          init[2] * s.C_elastic;
  const double sx = v.xc(1, sl), sy = v.xc(2, sl), sz = v.xc(3, sl);
  if (s.friclaw >= 3 && s.C_nuclea == 1 && 1 == s.nucfault) {
    // rsfNucleation, :367-414
    double dt2 = 0.0;
    const double radius = std::sqrt((sx - s.xsource) * (sx - s.xsource) + (sy - s.ysource) * (sy - s.ysource) +
                                    (sz - s.zsource) * (sz - s.zsource));
    double F = 0.0, G = 1.0;
    if (radius < s.nucR) F = std::exp(radius * radius / (radius * radius - s.nucR * s.nucR));
    if (t <= s.nucT) G = std::exp((t - s.nucT) * (t - s.nucT) / (t * (t - 2.0 * s.nucT)));
    if (s.TPV == 105 || s.TPV == 104) {
      dt2 = s.nucdtau0 * F * G;
    } else if (s.TPV == 2802) {
      if (nt == 1) {
        fr[81] = s.nucdtau0;
        const double ttao = std::sqrt(tr[1] * tr[1] + tr[2] * tr[2]);
        const double back = std::sqrt((rate[1] + fr[26]) * (rate[1] + fr[26]) + (rate[2] + fr[27]) * (rate[2] + fr[27]));
        fr[20] = fr[9] * std::log(2.0 * fr[12] / back * std::sinh(ttao / std::fabs(tr[0]) / fr[9]));
        fr[23] = std::fabs(tr[0]);
      }
      dt2 = fr[81] * F * G;
    }
    tr[1] = tr[1] + dt2;
  }
  tr[3] = std::sqrt(tr[1] * tr[1] + tr[2] * tr[2]);

  if (s.friclaw <= 2) {
    // solveSWTW, :136-188
    double mu = 0.0;
    if (s.friclaw == 1) mu = slip_weak(fr[77], fr);
    else mu = time_weak(t - o.a.fnft[i - 1], fr);
    if (s.C_nuclea == 1 && 1 == s.nucfault) {  // swtwNucleation, :416-443
      const double radius = std::sqrt((sx - s.xsource) * (sx - s.xsource) + (sy - s.ysource) * (sy - s.ysource) +
                                      (sz - s.zsource) * (sz - s.zsource));
      double trr = 1.0e9;
      if (radius <= s.nucR) {
        if (s.TPV == 201 || s.TPV == 36 || s.TPV == 37)
          trr = (radius + 0.081 * s.nucR * (1.0 / (1.0 - (radius / s.nucR) * (radius / s.nucR)) - 1.0)) / (0.7 * 3464.0);
        if (s.TPV == 202) trr = radius / s.nucRuptVel;
      }
      double tc = 1.0;
      if (t < trr) tc = 0.0;
      else if (t < trr + fr[5] && t >= trr) tc = (t - trr) / fr[5];
      mu = std::fmin(fr[1] + (fr[2] - fr[1]) * tc, mu);
    }
    const double ens = (tr[0] + fr[6] > 0) ? 0.0 : tr[0] + fr[6];
    const double strength = fr[4] - mu * ens;
    if (tr[3] > strength) {
      tr[1] = tr[1] * strength / tr[3];
      tr[2] = tr[2] * strength / tr[3];
    }
    double xt[3], xi[3];
    for (int j = 1; j <= 3; ++j) {
      xt[j - 1] = (tr[0] * v.un(j, i) + tr[1] * v.us(j, i) + tr[2] * v.ud(j, i)) * o.a.arn[i - 1];
      xi[j - 1] = (init[0] * v.un(j, i) + init[1] * v.us(j, i) + init[2] * v.ud(j, i)) * o.a.arn[i - 1];
    }
    for (int j = 1; j <= 3; ++j) {
      double &fs = v.F(v.eq(sl, j));
      fs = fs + xt[j - 1] - xi[j - 1] * s.C_elastic;
      double &fm = v.F(v.eq(ms, j));
      fm = fm - xt[j - 1] + xi[j - 1] * s.C_elastic;
    }
    for (int j = 0; j < 3; ++j) fr[78 + j] = tr[j];
  } else {
    // solveRSF, :190-327
    if (s.friclaw == 5) tr[0] = tr[0] + fr[51];
    else tr[0] = tr[0] + fr[6];
    if (s.insertFaultType > 0 && s.C_elastic == 1) {
      const double max_norm = -40.0e6, min_norm = -10.0e6;
      if (tr[0] >= min_norm) tr[0] = min_norm;
      else if (tr[0] <= max_norm) tr[0] = max_norm;
    }
    if (tr[0] > 0.0) tr[0] = 0.0;
    for (int j = 0; j < 3; ++j) {
      slip[j] = slip[j] + fr[25 + j] * t;
      rate[j] = rate[j] + fr[25 + j];
    }
    slip[3] = std::sqrt(slip[1] * slip[1] + slip[2] * slip[2]);
    rate[3] = std::sqrt(rate[1] * rate[1] + rate[2] * rate[2]);
    double vt = rate[3];
    const double thpc0 = fr[23];
    // rate_state_normal_stress on fric(23) with the trial rate
    double thdot = -vt / fr[11] * (fr[23] - std::fabs(tr[0]));
    fr[23] = fr[23] + thdot * dt;
    fr[24] = thdot;
    double state0 = fr[20];
    double xmu, dxmudv;
    rsf_law(s.friclaw, vt, fr[20], fr, dt, xmu, dxmudv);
    double taoc_old;
    if (s.friclaw == 5) taoc_old = fr[4] - xmu * tr[0];
    else taoc_old = xmu * thpc0;
    const double mr = mM * mS / (mM + mS);
    const double Tc = o.a.arn[i - 1] * dt / mr;
    double trial[4];
    for (int j = 1; j <= 2; ++j)
      trial[j] = tr[j] - taoc_old * 0.5 * (rate[j] / rate[3]) + fr[25 + j] / Tc;
    trial[3] = std::sqrt(trial[1] * trial[1] + trial[2] * trial[2]);
    // NewtonRaphson, :459-516
    const double nf[6] = {std::log(vt), state0, tr[0], trial[3], fr[9], fr[10]};
    double stateTmp = state0, thTmp = thpc0, taoc_new = 0.0;
    int iv;
    for (iv = 1; iv <= 20; ++iv) {
      stateTmp = state0;
      rsf_law(s.friclaw, vt, stateTmp, fr, dt, xmu, dxmudv);
      double rsfeq, dr;
      if (s.friclaw < 5) {
        thTmp = thpc0;
        thdot = -vt / fr[11] * (thTmp - std::fabs(tr[0]));
        thTmp = thTmp + thdot * dt;
        taoc_new = xmu * thTmp;
        rsfeq = vt + Tc * (taoc_new * 0.5 - trial[3]);
        dr = 1.0 + Tc * (dxmudv * thTmp) * 0.5;
      } else {
        taoc_new = fr[4] - xmu * std::fmin(tr[0], 0.0);
        rsfeq = vt + Tc * (taoc_new * 0.5 - trial[3]);
        dr = 1.0 + Tc * (-dxmudv * std::fmin(tr[0], 0.0)) * 0.5;
      }
      if (std::fabs(rsfeq / dr) < 1.e-14 * std::fabs(vt) && std::fabs(rsfeq) < 1.e-6 * std::fabs(vt)) break;
      const double vn = vt - rsfeq / dr;
      if (vn <= 0.0) vt = vt / 2.0;
      else vt = vn;
    }
    o.newton_iters += (iv > 20) ? 20 : iv;
    if (iv > 20) ++o.newton_maxhits;
    if (s.TPV == 105 && vt < fr[46]) vt = fr[46];
    if (o.log && (int64_t)o.log->size() < o.log_cap * 7) {
      o.log->insert(o.log->end(), nf, nf + 6);
      o.log->push_back(vt);
    }
    fr[20] = stateTmp;
    fr[23] = thTmp;
    for (int j = 1; j <= 2; ++j)
      tr[j] = taoc_old * 0.5 * (rate[j] / rate[3]) + taoc_new * 0.5 * (trial[j] / trial[3]);
    for (int j = 0; j < 3; ++j) fr[78 + j] = tr[j];
    fr[47] = vt;
    fr[48] = std::sqrt(tr[1] * tr[1] + tr[2] * tr[2]);
    if (o.a.onFaultTPHist && nt >= 1 && nt <= s.nstep) {
      double *h = o.a.onFaultTPHist + 2 * ((size_t)(i - 1) + (size_t)o.a.nftmx * (nt - 1));
      h[0] = fr[47];
      h[1] = fr[48];
    }
    double acc[3];
    acc[0] = -rate[0] / dt - slip[0] / dt / dt;
    acc[1] = (vt * (trial[1] / trial[3]) - rate[1]) / dt;
    acc[2] = (vt * (trial[2] / trial[3]) - rate[2]) / dt;
    double xa[3], R[3];
    for (int j = 1; j <= 3; ++j) {
      xa[j - 1] = acc[0] * v.un(j, i) + acc[1] * v.us(j, i) + acc[2] * v.ud(j, i);
      R[j - 1] = v.F(v.eq(sl, j)) + v.F(v.eq(ms, j));
    }
    for (int j = 1; j <= 3; ++j) {
      v.F(v.eq(sl, j)) = (-xa[j - 1] + R[j - 1] / mM) * mr;
      v.F(v.eq(ms, j)) = (xa[j - 1] + R[j - 1] / mS) * mr;
      fr[31 + j - 1] = v.vel(j, ms) + (xa[j - 1] + R[j - 1] / mS) * dt;
      fr[34 + j - 1] = v.vel(j, sl) + (-xa[j - 1] + R[j - 1] / mM) * dt;
    }
  }
  // storeOnFaultStationQuantSCEC, :518-541
  for (int j = 1; j <= o.a.numOnFaultSt && nt >= 1 && nt <= s.nstep; ++j) {
    if (o.a.anonfs[3 * (j - 1)] == i && o.a.anonfs[3 * (j - 1) + 2] == 1) {
      double *h = o.a.onFaultQuantHistSCECForm + 12 * ((size_t)(nt - 1) + (size_t)s.nstep * (j - 1));
      h[0] = t;
      h[1] = rate[1];
      h[2] = rate[2];
      h[3] = fr[20];
      h[4] = slip[1];
      h[5] = slip[2];
      h[6] = slip[0];
      h[7] = tr[1];
      h[8] = tr[2];
      h[9] = tr[0];
      h[10] = fr[51] + fr[42];
      h[11] = fr[52];
    }
  }
  // storeRuptureTime, :329-341
  if (o.a.fnft[i - 1] > 5000.0 && rate[3] >= s.slipRateThres) o.a.fnft[i - 1] = t;
}

// ---- src/thermop.f90:1-40 --------------------------------------------------------------------
void thermop(Oracle &o, int nt) {
  View v(o);
  const eqd_scalars &s = o.s;
  const double dt = s.dt, pi = 4.0 * std::atan(1.0), h = s.fric_tp_h;
  const int n = o.a.nftnd[0];
  if (!o.a.onFaultTPHist) return;
#pragma omp parallel for num_threads(o.nthreads) schedule(static)
  for (int i = 1; i <= n; ++i) {
    double *fr = &v.fric(1, i) - 1;
    const double gama = fr[19] / fr[18], omega = fr[16], kapa = fr[17];
    double tmp = 0.0;
    const int jmax = nt - 1 < s.nstep ? nt - 1 : s.nstep;
    for (int j = 1; j <= jmax; ++j) {
      double ker = -kapa / (omega - kapa) / std::pow(4.0 * kapa * (nt - j) * dt + 2.0 * h * h, 0.5);
      ker = ker + omega / (omega - kapa) / std::pow(4.0 * omega * (nt - j) * dt + 2.0 * h * h, 0.5);
      const double *hh = o.a.onFaultTPHist + 2 * ((size_t)(i - 1) + (size_t)o.a.nftmx * (j - 1));
      tmp = tmp + std::fabs(hh[1]) * hh[0] * ker * dt;
    }
    o.patnode[i - 1] = tmp * gama / std::pow(pi, 0.5);
    tmp = 0.0;
    for (int j = 1; j <= jmax; ++j) {
      const double ker = 1.0 / std::pow(4.0 * kapa * (nt - j) * dt + 2.0 * h * h, 0.5);
      const double *hh = o.a.onFaultTPHist + 2 * ((size_t)(i - 1) + (size_t)o.a.nftmx * (j - 1));
      tmp = tmp + std::fabs(hh[1]) * hh[0] * ker * dt;
    }
    o.Tatnode[i - 1] = tmp / fr[18] / std::pow(pi, 0.5);
    fr[51] = o.patnode[i - 1];
    fr[52] = o.Tatnode[i - 1] + fr[41];
  }
}

void colour_elements(Oracle &o) {
  const int ne = o.a.nelem;
  std::vector<uint64_t> used(o.a.nnode, 0);
  std::vector<int> col(ne, 0);
  int ncol = 0;
  for (int e = 1; e <= ne; ++e) {
    uint64_t m = 0;
    for (int k = 0; k < 8; ++k) m |= used[o.a.nodeElemIdRelation[8 * (size_t)(e - 1) + k] - 1];
    int c = 0;
    while (c < 64 && (m >> c & 1)) ++c;
    col[e - 1] = c;
    for (int k = 0; k < 8; ++k) used[o.a.nodeElemIdRelation[8 * (size_t)(e - 1) + k] - 1] |= (uint64_t)1 << c;
    if (c + 1 > ncol) ncol = c + 1;
  }
  o.colours.assign(ncol, {});
  for (int e = 0; e < ne; ++e) o.colours[col[e]].push_back(e + 1);
}

int step(Oracle &o, int nt) {
  View v(o);
  o.timeElapsed = o.timeElapsed + o.s.dt;
  int st = vel_disp_update(o);
  store_off_fault(o, nt);
  std::memset(o.a.nodalForceArr, 0, sizeof(double) * (size_t)o.a.neq);
  if (o.nthreads <= 1) {
    for (int e = 1; e <= o.a.nelem; ++e) assemble_element(o, e);
    for (int e = 1; e <= o.a.nelem; ++e) hourglass_element(o, e);
  } else {
    for (auto &c : o.colours) {
      const int n = (int)c.size();
#pragma omp parallel for num_threads(o.nthreads) schedule(static)
      for (int k = 0; k < n; ++k) assemble_element(o, c[k]);
    }
    for (auto &c : o.colours) {
      const int n = (int)c.size();
#pragma omp parallel for num_threads(o.nthreads) schedule(static)
      for (int k = 0; k < n; ++k) hourglass_element(o, c[k]);
    }
  }
  if (o.s.friclaw == 5) thermop(o, nt);
  const int np = o.a.nftnd[0];
  for (int i = 1; i <= np; ++i) fault_pair(o, i, nt);
  const int neq = o.a.neq;
#pragma omp parallel for num_threads(o.nthreads) schedule(static)
  for (int e = 0; e < neq; ++e) o.a.nodalForceArr[e] = o.a.nodalForceArr[e] / o.a.nodalMassArr[e];
  return st;
}

}  // namespace

extern "C" {

// Creates an oracle bound to caller-owned arrays (they are updated in place).
void *oracle_create(const eqd_scalars *s, const eqd_host_arrays *a, int nthreads) {
  auto *o = new Oracle();
  o->s = *s;
  o->a = *a;
  o->timeElapsed = s->time0;
  o->nthreads = nthreads < 1 ? 1 : nthreads;
  o->patnode.assign(a->nftmx, 0.0);
  o->Tatnode.assign(a->nftmx, 0.0);
  if (o->nthreads > 1) colour_elements(*o);
  return o;
}

// Runs steps nt_begin .. nt_begin+nsteps-1; returns 0 or EQD_ERR_NAN.
int oracle_step(void *h, int nt_begin, int nsteps) {
  Oracle &o = *static_cast<Oracle *>(h);
  for (int k = 0; k < nsteps; ++k) {
    int st = step(o, nt_begin + k);
    if (st) return st;
  }
  return 0;
}

double oracle_time(void *h) { return static_cast<Oracle *>(h)->timeElapsed; }

void oracle_stats(void *h, int64_t *iters, int64_t *maxhits, int32_t *ncolours) {
  Oracle &o = *static_cast<Oracle *>(h);
  if (iters) *iters = o.newton_iters;
  if (maxhits) *maxhits = o.newton_maxhits;
  if (ncolours) *ncolours = (int32_t)o.colours.size();
}

// Records (log V_trial, state0, normal traction, trial shear traction, a, b, converged V) for up
// to `cap` Newton solves into `buf` (7 doubles per solve); returns the count recorded so far.
int64_t oracle_log_newton(void *h, double *buf, int64_t cap) {
  Oracle &o = *static_cast<Oracle *>(h);
  if (buf == nullptr) {
    if (!o.log) return 0;
    return (int64_t)o.log->size() / 7;
  }
  if (!o.log) {
    o.log = new std::vector<double>();
    o.log_cap = cap;
    return 0;
  }
  const int64_t n = std::min<int64_t>((int64_t)o.log->size() / 7, cap);
  std::memcpy(buf, o.log->data(), sizeof(double) * 7 * (size_t)n);
  return n;
}

void oracle_free(void *h) {
  Oracle *o = static_cast<Oracle *>(h);
  delete o->log;
  delete o;
}

}  // extern "C"
