// Rate-and-state friction law and the per-pair Newton solve for the slip rate
// (src/fric.f90:39-95, src/faulting.f90:459-516), shared by the fault kernel and the kernel that
// replays logged solves.
#pragma once
#include <cuda_runtime.h>

namespace eqd {

// fric(9..15) of one pair: a, b, L, V0, f0, fw, Vw
struct RsfParams {
  double A, B, L, V0, f0, fw, Vw;
};

// Inputs of one Newton solve: the law's parameters, state and fric(23) before the solve, the
// effective normal traction, the trial shear traction, Tc = area dt / reduced mass, fric(4).
struct NewtonSolve {
  RsfParams r;
  double state0, th0, tn, trial, Tc, c0;
};

struct NewtonOut {
  double v, state, th, taoc;
  double step;   // |last Newton step| / |slip rate where it was evaluated|
  int iters;     // as the reference counts them (20 when the cap is reached)
  int capped;    // 1 when the 20 iterations ran out without meeting the tolerance
  int executed;  // iterations actually evaluated
  int exit_kind; // FAST: 0 exit test or cap, 1 fixed point, 2 2-cycle ending on the last
                 // evaluation, 3 2-cycle ending on the one before it
};

// Logged solve: NewtonSolve (13 doubles), the plain initial guess, the converged slip rate and
// the reference iteration count.
constexpr int kNewtonRecord = 16;

__device__ __forceinline__ void rsf_law(int friclaw, double V2, double &state, const RsfParams &p, double dt,
                                        double &xmu, double &dxmudv) {
  if (friclaw == 3) {  // aging law
    const double tmpc = 1.0 / (2.0 * p.V0) * exp((p.f0 + p.B * log(p.V0 * state / p.L)) / p.A);
    const double tmp = (V2 + 1.e-30) * tmpc;
    xmu = p.A * log(tmp + sqrt(tmp * tmp + 1.0));
    dxmudv = p.A * tmpc / sqrt(1.0 + tmp * tmp);
    state = p.L / V2 + (state - p.L / V2) * exp(-V2 * dt / p.L);
  } else {  // slip law with strong rate weakening
    const double tmpc = 1.0 / (2.0 * p.V0) * exp(state / p.A);
    const double tmp = (V2 + 1.e-30) * tmpc;
    xmu = p.A * log(tmp + sqrt(tmp * tmp + 1.0));
    dxmudv = p.A * tmpc / sqrt(1.0 + tmp * tmp);
    const double fLV = p.f0 - (p.B - p.A) * log(V2 / p.V0);
    const double r = V2 / p.Vw, r2 = r * r, r4 = r2 * r2;
    const double fss = p.fw + (fLV - p.fw) / pow(1.0 + r4 * r4, 0.125);
    const double fssa = fss / p.A;
    const double psiss = p.A * log(2.0 * p.V0 / V2 * (exp(fssa) - exp(-fssa)) / 2.0);
    state = psiss + (state - psiss) * exp(-V2 * dt / p.L);
  }
}

// State evolution of the law at slip rate V2 (the state half of rsf_law).
__device__ __forceinline__ double rsf_state(int friclaw, double V2, double state, const RsfParams &p, double dt) {
  if (friclaw == 3) return p.L / V2 + (state - p.L / V2) * exp(-V2 * dt / p.L);
  const double fLV = p.f0 - (p.B - p.A) * log(V2 / p.V0);
  const double r = V2 / p.Vw, r2 = r * r, r4 = r2 * r2;
  const double fss = p.fw + (fLV - p.fw) / pow(1.0 + r4 * r4, 0.125);
  const double fssa = fss / p.A;
  const double psiss = p.A * log(2.0 * p.V0 / V2 * (exp(fssa) - exp(-fssa)) / 2.0);
  return psiss + (state - psiss) * exp(-V2 * dt / p.L);
}

// NewtonRaphson, at most 20 iterations from v0.  Iteration k evaluates the law at v_(k-1) and
// forms v_k = f(v_(k-1)), a deterministic map; after 20 iterations the outputs are v_20 and the
// law evaluated at v_19.
//
// FAST = false is the reference's loop statement by statement.  FAST = true gives the same values
// bit for bit with less work:
//  * the law's prefactor 1/(2 V0) exp(...) depends only on the state before the solve, which every
//    iteration restarts from, so it is evaluated once; the state update (another exp) is needed
//    only at the last evaluation point, so it is evaluated once after the loop;
//  * when an iterate repeats (a fixed point v_k = v_(k-1), or a 2-cycle v_k = v_(k-2)) every later
//    iteration is known and the loop stops with the values iteration 20 would give.
template <bool FAST>
__device__ __forceinline__ NewtonOut rsf_newton(int friclaw, double dt, const NewtonSolve &s, double v0) {
  const RsfParams &p = s.r;
  double vt = v0;
  double stateTmp = s.state0, thTmp = s.th0, taoc_new = 0.0;
  double tmpc = 0.0;
  if (FAST) tmpc = (friclaw == 3) ? 1.0 / (2.0 * p.V0) * exp((p.f0 + p.B * log(p.V0 * s.state0 / p.L)) / p.A)
                                  : 1.0 / (2.0 * p.V0) * exp(s.state0 / p.A);
  double v_eval = v0;                        // FAST: where the law was last evaluated
  double vA = 0.0, thA = 0.0, tcA = 0.0;     // FAST: v_(k-2) and the law evaluated at it
  double dvA = 0.0;                          // FAST: the Newton step evaluated at v_(k-2)
  double dv_last = 0.0, vt_last = 1.0;       // Newton step and iterate of the last evaluation
  int iv, executed = 0, exit_kind = 0;
  for (iv = 1; iv <= 20; ++iv) {
    ++executed;
    double xmu, dxmudv;
    if (FAST) {
      v_eval = vt;
      const double tmp = (vt + 1.e-30) * tmpc;
      xmu = p.A * log(tmp + sqrt(tmp * tmp + 1.0));
      dxmudv = p.A * tmpc / sqrt(1.0 + tmp * tmp);
    } else {
      stateTmp = s.state0;
      rsf_law(friclaw, vt, stateTmp, p, dt, xmu, dxmudv);
    }
    double rsfeq, dr;
    if (friclaw < 5) {
      thTmp = s.th0;
      const double thdot = -vt / p.L * (thTmp - fabs(s.tn));
      thTmp = thTmp + thdot * dt;
      taoc_new = xmu * thTmp;
      rsfeq = vt + s.Tc * (taoc_new * 0.5 - s.trial);
      dr = 1.0 + s.Tc * (dxmudv * thTmp) * 0.5;
    } else {
      taoc_new = s.c0 - xmu * fmin(s.tn, 0.0);
      rsfeq = vt + s.Tc * (taoc_new * 0.5 - s.trial);
      dr = 1.0 + s.Tc * (-dxmudv * fmin(s.tn, 0.0)) * 0.5;
    }
    const double dv = rsfeq / dr;
    dv_last = dv;
    vt_last = vt;
    if (fabs(dv) < 1.e-14 * fabs(vt) && fabs(rsfeq) < 1.e-6 * fabs(vt)) break;
    const double vn = vt - dv;
    const double vnew = (vn <= 0.0) ? vt / 2.0 : vn;
    if (FAST && iv < 20) {
      if (vnew == vt) {  // fixed point: v_20 = v_19 = vt
        exit_kind = 1;
        iv = 21;
        break;
      }
      if (iv >= 2 && vnew == vA) {  // 2-cycle vA, vt, vA, ...
        if ((20 - iv) % 2 == 0) {
          vt = vnew;  // v_20 = vA, v_19 = vt: the evaluation just made
          exit_kind = 2;
        } else {      // v_20 = vt, v_19 = vA: the previous evaluation, step ratio included
          v_eval = vA;
          thTmp = thA;
          taoc_new = tcA;
          dv_last = dvA;
          vt_last = vA;
          exit_kind = 3;
        }
        iv = 21;
        break;
      }
    }
    if (FAST) {
      vA = vt;
      thA = thTmp;
      tcA = taoc_new;
      dvA = dv;
    }
    vt = vnew;
  }
  if (FAST) stateTmp = rsf_state(friclaw, v_eval, s.state0, p, dt);
  // the step ratio of the last evaluation, formed once here rather than in every iteration
  const double step = fabs(dv_last) / fabs(vt_last);
  NewtonOut o;
  o.v = vt;
  o.state = stateTmp;
  o.th = thTmp;
  o.taoc = taoc_new;
  o.step = step;
  o.iters = iv > 20 ? 20 : iv;
  o.capped = iv > 20 ? 1 : 0;
  o.executed = executed;
  o.exit_kind = exit_kind;
  return o;
}

// A solve from the learned initial guess is kept when it settled: it met the exit test, or its
// last Newton step was below 1e-12 of the slip rate (the iterate had reached round-off, as the
// plain method's capped solves of creeping pairs do).  A guess outside the Newton's basin ends
// with the cap reached while the iterate still moves; that solve is repeated from the plain guess
// and the repeat's result is kept, so a poor guess costs iterations but never changes a result.
__device__ __forceinline__ bool newton_settled(const NewtonOut &o) { return !o.capped || o.step <= 1.e-12; }

}  // namespace eqd
