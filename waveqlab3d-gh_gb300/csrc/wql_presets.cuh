// Fault-physics presets evaluated per fault point on the device (and host).
//
// The reference selects prestress, strength, rate-and-state parameters and
// initial stress by the `problem` string inside every per-point call
// (src/Interface_Condition.f90:1268-2476, src/initial_stress_condition.f90).
// Here the string is resolved once to an integer preset and the formulas are
// evaluated branch-free of string compares.  `param` presets (sw_param,
// rs_param) take their constants from the &fault_list extension group.
#pragma once
#include <math.h>

#include "wql_sbp.cuh"

namespace wql {

enum Preset : int {
  PRE_NONE = 0,
  PRE_TPV5 = 1,   // also LOH1 / OKLAHOMA prestress
  PRE_TPV26 = 2,
  PRE_TPV27 = 3,
  PRE_TPV28 = 4,
  PRE_TPV29 = 5,
  PRE_TPV30 = 6,
  PRE_TPV10 = 7,
  PRE_TPV101 = 8,
  PRE_TPV102 = 9,
  PRE_SW_PARAM = 10,
  PRE_RS_PARAM = 11,
  // TPV28 with the SCEC benchmark's szz = -60 MPa in place of the +60 of
  // src/initial_stress_condition.f90:80 (&gb300_list tpv28_prestress = 'benchmark')
  PRE_TPV28_BENCH = 12,
  // problem = 'rate-weakening': rate and state with strong velocity
  // weakening (src/Interface_Condition.f90:410-416, 438-443, 2387-2423,
  // 2819-2843; src/initial_stress_condition.f90:184-193)
  PRE_RATE_WEAKENING = 13,
};

enum Coupling : int { CPL_LOCKED = 0, CPL_LINEAR = 1, CPL_SW = 2, CPL_RS = 3 };

struct FaultParams {
  int preset;
  int coupling;
  double fs, fd, Dc, barrier_y, barrier_z;
  double a, b, V0, f0, L, Vini;
  double s0[6], nuc_amp, nuc_radius, nuc_y, nuc_z, nuc_rise;
  int s0_profile;  // preset whose initial stress replaces s0 (PRE_NONE: uniform s0)
};

// boxcar / smooth_boxcar: src/Interface_Condition.f90:2438-2476
WQL_HD double boxcar(double x, double w) {
  const double tol = 100.0 * 2.220446049250313e-16;
  if (-w + tol < x && x < w - tol) return 1.0;
  if (fabs(-w - x) <= tol || fabs(x - w) <= tol) return 0.5;
  return 0.0;
}

WQL_HD double smooth_boxcar(double x, double w, double wr) {
  if (-w <= x && x <= w) return 1.0;
  const double ax = fabs(x);
  if (ax > w && ax < w + wr) return 0.5 * (1.0 + tanh(wr / (ax - w - wr) + wr / (ax - w)));
  return 0.0;
}

// The uniform tensor of problem 'rate-weakening' (src/initial_stress_condition.f90:
// 184-193), with that routine's pi = 3.14159265359.
WQL_HD void rate_weakening_stress(double s0[6]) {
  const double psi = 50.0 / 180.0 * 3.14159265359;
  s0[0] = -126.0;
  s0[4] = 42.0;
  s0[2] = (1.0 - 2.0 * s0[4] / (s0[0] * tan(2.0 * psi))) * s0[0];
  s0[1] = 0.5 * (s0[0] + s0[2]);
  s0[3] = 0.0;
  s0[5] = 0.0;
}

// initial_stress_tensor (src/initial_stress_condition.f90:8-254): s0 =
// (sxx, syy, szz, sxy, sxz, syz).  Returns false for presets without one.
WQL_HD bool initial_stress(int preset, const double x[3], double s0[6]) {
  switch (preset) {
    case PRE_TPV26:
    case PRE_TPV27:
    case PRE_TPV29:
    case PRE_TPV30: {
      const bool p29 = preset == PRE_TPV29 || preset == PRE_TPV30;
      const double y1 = p29 ? 17.0 : 15.0, y2 = p29 ? 22.0 : 20.0;
      double Om = 0.0;
      if (x[1] <= y1) Om = 1.0;
      else if (x[1] >= y1 && x[1] <= y2) Om = (y2 - x[1]) / 5.0;
      const double b11 = p29 ? 1.025837 : 0.926793, b33 = p29 ? 0.974162 : 1.073206;
      const double b13 = p29 ? -0.158649 : -0.169029;
      const double Pf = 9.8 * x[1], s22 = -2.67 * 9.8 * x[1];
      s0[0] = Om * (b33 * (s22 + Pf) - Pf) + (1.0 - Om) * s22 + Pf;
      s0[1] = s22 + Pf;
      s0[2] = Om * (b11 * (s22 + Pf) - Pf) + (1.0 - Om) * s22 + Pf;
      s0[3] = 0.0;
      s0[4] = Om * (b13 * (s22 + Pf));
      s0[5] = 0.0;
      return true;
    }
    case PRE_TPV28:
    case PRE_TPV28_BENCH:
      s0[0] = -60.0; s0[1] = 0.0; s0[2] = preset == PRE_TPV28 ? 60.0 : -60.0;
      s0[3] = 0.0; s0[4] = 29.38; s0[5] = 0.0;
      return true;
    case PRE_TPV101:
    case PRE_TPV102:
      s0[0] = -120.0; s0[1] = 0.0; s0[2] = -120.0; s0[3] = 0.0; s0[4] = 75.0; s0[5] = 0.0;
      return true;
    case PRE_TPV10:
      s0[0] = -7.378 * x[1]; s0[1] = 0.0; s0[2] = -7.378 * x[1]; s0[3] = 0.0;
      s0[4] = -0.55 * s0[0]; s0[5] = 0.0;
      return true;
    case PRE_RATE_WEAKENING:
      rate_weakening_stress(s0);
      return true;
    case PRE_SW_PARAM:
    case PRE_RS_PARAM:
      return false;  // uniform tensor: supplied by the caller (FaultParams::s0)
    default:
      return false;
  }
}

// initial_stress for the plastic update in the field precision R: the same
// expressions on the depth y (R = double gives the values above).
template <typename R>
WQL_HD bool initial_stress_y(int preset, R y, R s0[6]) {
  switch (preset) {
    case PRE_TPV26:
    case PRE_TPV27:
    case PRE_TPV29:
    case PRE_TPV30: {
      const bool p29 = preset == PRE_TPV29 || preset == PRE_TPV30;
      const R y1 = p29 ? R(17.0) : R(15.0), y2 = p29 ? R(22.0) : R(20.0);
      R Om = R(0.0);
      if (y <= y1) Om = R(1.0);
      else if (y >= y1 && y <= y2) Om = (y2 - y) / R(5.0);
      const R b11 = p29 ? R(1.025837) : R(0.926793), b33 = p29 ? R(0.974162) : R(1.073206);
      const R b13 = p29 ? R(-0.158649) : R(-0.169029);
      const R Pf = R(9.8) * y, s22 = R(-2.67) * R(9.8) * y;
      s0[0] = Om * (b33 * (s22 + Pf) - Pf) + (R(1.0) - Om) * s22 + Pf;
      s0[1] = s22 + Pf;
      s0[2] = Om * (b11 * (s22 + Pf) - Pf) + (R(1.0) - Om) * s22 + Pf;
      s0[3] = R(0.0);
      s0[4] = Om * (b13 * (s22 + Pf));
      s0[5] = R(0.0);
      return true;
    }
    case PRE_TPV28:
    case PRE_TPV28_BENCH:
      s0[0] = R(-60.0); s0[1] = R(0.0); s0[2] = preset == PRE_TPV28 ? R(60.0) : R(-60.0);
      s0[3] = R(0.0); s0[4] = R(29.38); s0[5] = R(0.0);
      return true;
    case PRE_TPV101:
    case PRE_TPV102:
      s0[0] = R(-120.0); s0[1] = R(0.0); s0[2] = R(-120.0); s0[3] = R(0.0); s0[4] = R(75.0); s0[5] = R(0.0);
      return true;
    case PRE_TPV10:
      s0[0] = R(-7.378) * y; s0[1] = R(0.0); s0[2] = R(-7.378) * y; s0[3] = R(0.0);
      s0[4] = R(-0.55) * s0[0]; s0[5] = R(0.0);
      return true;
    case PRE_RATE_WEAKENING: {  // uniform: the FP64 values rounded to R
      double d[6];
      rate_weakening_stress(d);
      for (int c = 0; c < 6; ++c) s0[c] = R(d[c]);
      return true;
    }
    default:
      return false;
  }
}

WQL_HD void tensor_traction(const double s0[6], const double n[3], const double m[3],
                            const double l[3], double& Tn, double& Tm, double& Tl) {
  const double Tx = n[0] * s0[0] + n[1] * s0[3] + n[2] * s0[4];
  const double Ty = n[0] * s0[3] + n[1] * s0[1] + n[2] * s0[5];
  const double Tz = n[0] * s0[4] + n[1] * s0[5] + n[2] * s0[2];
  Tn = n[0] * Tx + n[1] * Ty + n[2] * Tz;
  Tm = m[0] * Tx + m[1] * Ty + m[2] * Tz;
  Tl = l[0] * Tx + l[1] * Ty + l[2] * Tz;
}

// TPV101/102 nucleation time function G(t) (src/Interface_Condition.f90:2344-2351)
WQL_HD double smooth_ramp(double t) {
  double G = 0.0;
  if (t > 0.0 && t < 1.0) G = exp((t - 1.0) * (t - 1.0) / (t * (t - 2.0)));
  if (t >= 1.0) G = 1.0;
  return G;
}

// prestress (src/Interface_Condition.f90:1802-2435), split as
//   (Tn, Tm, Tl) = static(x) + (0, 0, nucleation_weight(x) * nucleation_ramp(t))
// because the only time dependence of every preset is a fault-uniform ramp
// of a nucleation patch; the static part and the weight are evaluated once
// per fault point, the ramp once per stage.  prestress() recombines them
// with the reference's arithmetic order (Tl + (weight * ramp)).
WQL_HD void prestress_static(const FaultParams& fp, const double x[3], const double l[3], const double m[3],
                             const double n[3], double& Tn, double& Tm, double& Tl) {
  double s0[6];
  switch (fp.preset) {
    case PRE_TPV5:
      Tn = -120.0;
      Tm = 0.0;
      Tl = 70.0;
      Tl = Tl + 8.0 * boxcar(x[1] - 7.5, 1.5) * boxcar(x[2] + 7.5, 1.5);
      Tl = Tl + 11.6 * boxcar(x[1] - 7.5, 1.5) * boxcar(x[2], 1.5);
      Tl = Tl - 8.0 * boxcar(x[1] - 7.5, 1.5) * boxcar(x[2] - 7.5, 1.5);
      return;
    case PRE_TPV26:
    case PRE_TPV27:
    case PRE_TPV29:
    case PRE_TPV30:
    case PRE_TPV101:
    case PRE_TPV102:
    case PRE_RATE_WEAKENING:
      initial_stress(fp.preset, x, s0);
      tensor_traction(s0, n, m, l, Tn, Tm, Tl);
      return;
    case PRE_TPV28:
    case PRE_TPV28_BENCH: {
      initial_stress(fp.preset, x, s0);
      tensor_traction(s0, n, m, l, Tn, Tm, Tl);
      const double r = sqrt((x[1] - 7.5) * (x[1] - 7.5) + x[2] * x[2]);
      double nuke = 0.0;
      if (r <= 1.4) nuke = 11.60;
      else if (r >= 1.4 && r <= 2.0) nuke = 5.8 * (1.0 + cos(3.141592653589793 * (r - 1.4) / 0.6));
      Tl = Tl + nuke;
      return;
    }
    case PRE_TPV10: {
      const double g = 2.0 / sqrt(3.0);
      Tn = -7.378 * x[1] * g;
      Tm = -0.55 * Tn;
      Tl = 0.0;
      Tm = Tm + (-(0.760 + 0.0057) * Tn + 0.2 - Tm) * boxcar(x[1] * g - 12.0, 1.5) * boxcar(x[2], 1.5);
      return;
    }
    case PRE_SW_PARAM:
    case PRE_RS_PARAM:
      if (fp.s0_profile != PRE_NONE && initial_stress(fp.s0_profile, x, s0))
        tensor_traction(s0, n, m, l, Tn, Tm, Tl);
      else
        tensor_traction(fp.s0, n, m, l, Tn, Tm, Tl);
      return;
    default:
      Tn = Tm = Tl = 0.0;
  }
}

// Amplitude of the time-ramped nucleation traction at x (MPa); Tn is the
// static normal traction there.
WQL_HD double nucleation_weight(const FaultParams& fp, const double x[3], double Tn) {
  switch (fp.preset) {
    case PRE_RATE_WEAKENING: {
      // a Gaussian pulse of twice tau_pulse = -0.2429 Tn
      const double tau_pulse = -0.2429 * Tn;
      const double r0 = 3.0 * 1.5 * 0.3;
      const double y0 = 8.0, z0 = 0.0;
      const double r = sqrt((x[1] - y0) * (x[1] - y0) + (x[2] + z0) * (x[2] + z0));
      const double F = exp(-((r / r0) * (r / r0)) / 2.0);
      return 2.0 * tau_pulse * F;
    }
    case PRE_TPV101:
    case PRE_TPV102: {
      const double r = sqrt((x[1] - 7.5) * (x[1] - 7.5) + x[2] * x[2]);
      double F = 0.0;
      if (r < 3.0) F = exp(r * r / (r * r - 9.0));
      return 25.0 * F;
    }
    case PRE_SW_PARAM:
    case PRE_RS_PARAM: {
      const double dy = x[1] - fp.nuc_y, dz = x[2] - fp.nuc_z;
      const double F = exp(-(dy * dy + dz * dz) / (2.0 * fp.nuc_radius * fp.nuc_radius));
      return fp.nuc_amp * F;
    }
    default:
      return 0.0;
  }
}

// The fault-uniform ramp of the nucleation traction at time t.
WQL_HD double nucleation_ramp(const FaultParams& fp, double t) {
  switch (fp.preset) {
    case PRE_TPV101:
    case PRE_TPV102:
      return smooth_ramp(t);
    case PRE_SW_PARAM:
    case PRE_RS_PARAM:
      return fp.nuc_rise > 0.0 ? smooth_ramp(t / fp.nuc_rise) : 1.0;
    case PRE_RATE_WEAKENING:
      return t > 0.0 ? 1.0 : 0.0;
    default:
      return 0.0;
  }
}

WQL_HD void prestress(const FaultParams& fp, const double x[3], double t, const double l[3],
                      const double m[3], const double n[3], double& Tn, double& Tm, double& Tl) {
  prestress_static(fp, x, l, m, n, Tn, Tm, Tl);
  const double w = nucleation_weight(fp, x, Tn);
  if (w != 0.0) Tl = Tl + w * nucleation_ramp(fp, t);
}

WQL_HD double forced_rupture_time(double r, double Vs) {
  const double rc = 4.0;
  if (r < rc - 1.0e-9) return r / (0.7 * Vs) + 0.081 * rc / (0.7 * Vs) * (1.0 / (1.0 - (r / rc) * (r / rc)) - 1.0);
  return 1.0e9;
}

// Tau_strength (src/Interface_Condition.f90:1268-1797)
WQL_HD double tau_strength(const FaultParams& fp, double sigma_n, double D, const double x[3],
                           double t) {
  switch (fp.preset) {
    case PRE_TPV5: {
      double fs = 0.677 + 1.0e10 * (1.0 - boxcar(x[1], 15.0) * boxcar(x[2], 15.0));
      const double fd = 0.525, Dc = 0.4;
      return sigma_n * (fs - (fs - fd) * fmin(D, Dc) / Dc);
    }
    case PRE_TPV28:
    case PRE_TPV28_BENCH: {
      double fs = 0.677 + 1.0e10 * (1.0 - boxcar(x[1], 15.0) * boxcar(x[2], 18.0));
      const double fd = 0.373, Dc = 0.4;
      return sigma_n * (fs - (fs - fd) * fmin(D, Dc) / Dc);
    }
    case PRE_TPV26:
    case PRE_TPV27:
    case PRE_TPV29:
    case PRE_TPV30: {
      const bool p29 = fp.preset == PRE_TPV29 || fp.preset == PRE_TPV30;
      double fs = 0.18;
      const double fd = 0.12, Dc = 0.3, t0 = 0.5, Vs = 3.464;
      const double r = sqrt((x[1] - 10.0) * (x[1] - 10.0) + (x[2] + 5.0) * (x[2] + 5.0));
      const double depth = x[1];
      double C0;
      if (p29) C0 = depth <= 4.0 ? 0.4 + 0.2 * (4.0 - depth) : 0.4;
      else C0 = depth <= 5.0 ? 0.4 + 0.72 * (5.0 - depth) : 0.4;
      const double box = boxcar(x[1], 20.0) * boxcar(x[2], 20.0);
      if (p29) C0 = C0 + 1.0e10 * (1.0 - box);
      const double tf = forced_rupture_time(r, Vs);
      const double f1 = fmin(D / Dc, 1.0);
      double f2 = 0.0;
      if (t < tf) f2 = 0.0;
      else if (t >= tf && t < tf + t0) f2 = (t - tf) / t0;
      else if (t >= tf + t0) f2 = 1.0;
      if (!p29) fs = fs + 1.0e10 * (1.0 - box);
      const double f = fs - (fs - fd) * fmax(f1, f2);
      return C0 + f * sigma_n;
    }
    case PRE_TPV10: {
      const double g = 2.0 / sqrt(3.0);
      const double bb = boxcar(x[1] * g, 15.0) * boxcar(x[2], 15.0);
      const double fs = 0.760 + (1.0e4 - 0.760) * (1.0 - bb);
      const double fd = 0.448, Dc = 0.50;
      const double f = fs - (fs - fd) * fmin(D, Dc) / Dc;
      const double C0 = 0.2 + 1.0e3 * (1.0 - bb);
      return C0 + fmax(sigma_n, 0.0) * f;
    }
    case PRE_SW_PARAM: {
      double fs = fp.fs + 1.0e10 * (1.0 - boxcar(x[1], fp.barrier_y) * boxcar(x[2], fp.barrier_z));
      return sigma_n * (fs - (fs - fp.fd) * fmin(D, fp.Dc) / fp.Dc);
    }
    default:
      return 0.0;
  }
}

struct RSParams {
  double L0, f0, b, V0, a;
};

// rate-and-state constants per point (src/Interface_Condition.f90:384-417);
// only the direct-effect parameter a varies along the fault
WQL_HD double rs_direct_a(const FaultParams& fp, const double x[3]) {
  if (fp.preset == PRE_RS_PARAM) return fp.a;
  if (fp.preset == PRE_RATE_WEAKENING)
    return 0.016 + 0.016 * (1.0 - smooth_boxcar(x[1], 20.0, 2.5) * smooth_boxcar(x[2], 20.0, 2.5));
  return 0.008 + 0.008 * (1.0 - smooth_boxcar(x[1], 15.0, 3.0) * smooth_boxcar(x[2], 15.0, 3.0));
}

// Weakening velocity V_w(x) of problem 'rate-weakening' (src/Interface_Condition.f90:439-440).
WQL_HD double rs_weakening_velocity(const double x[3]) {
  return 0.17 + 5.0 * (1.0 - smooth_boxcar(x[1], 20.0, 2.5) * smooth_boxcar(x[2], 20.0, 2.5));
}

// Rate of the state variable psi at slip rate V: the aging law of TPV101/102
// and rs_param (src/Interface_Condition.f90:431-436), or for
// 'rate-weakening' the slip law with a steady state that weakens above V_w
// (:438-443):
//   Fss = 0.13 + (f0 - (b-a) ln(V/V0) - 0.13) / (1 + (V/V_w)^8)^(1/8),
//   dpsi/dt = -V/L0 (a asinh(V/(2 V0) e^{psi/a}) - Fss).
WQL_HD double rs_rate_weakening_state_rate(double psi, double V, double a, double b, double V0, double f0,
                                           double L0, double Vw) {
  double Fss = f0 - (b - a) * log(V / V0);
  const double r = V / Vw, r2 = r * r, r4 = r2 * r2;  // (V/V_w)**8 by squaring, as an integer power
  Fss = 0.13 + (Fss - 0.13) / pow(1.0 + r4 * r4, 0.125);
  return -V / L0 * (a * asinh(V / (2.0 * V0) * exp(psi / a)) - Fss);
}

WQL_HD RSParams rs_params(const FaultParams& fp, const double x[3], double a) {
  (void)x;
  RSParams r;
  if (fp.preset == PRE_RS_PARAM) {
    r.L0 = fp.L; r.f0 = fp.f0; r.b = fp.b; r.V0 = fp.V0;
  } else if (fp.preset == PRE_RATE_WEAKENING) {
    r.L0 = 2.0 * 0.2572; r.f0 = 0.7; r.b = 0.02; r.V0 = 1.0e-6;
  } else {
    r.L0 = 0.02; r.f0 = 0.6; r.b = 0.012; r.V0 = 1.0e-6;
  }
  r.a = a;
  return r;
}

WQL_HD RSParams rs_params(const FaultParams& fp, const double x[3]) { return rs_params(fp, x, rs_direct_a(fp, x)); }

}  // namespace wql
