// Interface kernel: on-device block coupling and fault friction, one thread
// per (fault point, block copy), always in FP64.
//
// The reference swaps the two blocks' fault faces over MPI
// (src/domain.f90:665-690, src/mpi3d_interface.f90:483-520) and every rank
// pair solves the interface condition for its own block with its own copy of
// the interface state (src/domain.f90:262-263, 586-611).  Here one kernel
// reads both blocks' faces straight from HBM; copy b = 0 is block 1's solve
// (its +q face normals and metrics), copy b = 1 is block 2's (-q face).  Each
// copy keeps its own slip S(4), state W and their rates, which is what an
// even-rank reference run does.  Per point and copy:
//   tractions, rotation to (n,m,l) ....... src/CouplingForcing.f90:115-210, 469-522
//   hat variables from friction .......... src/Interface_Condition.f90:12-1265
//   stage-1 outputs, rupture front ...... src/CouplingForcing.f90:211-228, 584-605
//   SAT vector u_bc / v_bc ............... src/CouplingForcing.f90:238-466
//   DS/DW accumulation and RK update ..... src/Interface_Condition.f90:433,475-476,
//                                          src/iface.f90:51-76
#include <cuda_runtime.h>

#include "wql_internal.h"

namespace wql {
namespace {

// Regula falsi for V + a*sigma_n/eta*asinh(V/(2V0)*exp(psi/a)) = Phi/eta on
// [0, Phi/eta] (src/Interface_Condition.f90:1170-1265), including the
// reference's acceptance test `fv*fl > tol`.  tol and maxit are the
// reference's 1e-12 and 5000 unless the input overrides them.  Returns false
// when the iteration budget is exhausted.  exp(psi/a) is evaluated once; the
// residual is otherwise formed exactly as the reference forms it.
__device__ bool regula_falsi(double& V, double Phi, double eta, double sn, double psi, double V0,
                             double a, double tol, int maxit) {
  const double ek = exp(psi / a);
  auto f = [&](double v) { return v + a * sn / eta * asinh(0.5 * v / V0 * ek) - Phi / eta; };
  double Vl = 0.0, Vr = Phi / eta;
  double fv = f(V), fl = f(Vl), fr = f(Vr);
  if (fabs(fv) <= tol) return true;
  if (fabs(fl) <= tol) { V = Vl; return true; }
  if (fabs(fr) <= tol) { V = Vr; return true; }
  double err = 1.0;
  int k = 1;
  while (k <= maxit && err >= tol) {
    const double V1 = V;
    if (fv * fl > tol) {
      Vl = V;
      V = Vr - (Vr - Vl) * fr / (fr - fl);
      fl = fv;
    } else if (fv * fr > tol) {
      Vr = V;
      V = Vr - (Vr - Vl) * fr / (fr - fl);
      fr = fv;
    }
    fv = f(V);
    err = fabs(V - V1);
    ++k;
  }
  return !(k >= maxit);
}

// The same equation for FP32 fields, by Newton's method in u = ln V.  With
// s = V/(2V0)*exp(psi/a) = exp(w), w = u + ln(exp(psi/a)/(2V0)), the function
// g(u) = e^u + c*asinh(s) - Phi/eta is increasing and convex in u
// (d asinh(s)/du = s/sqrt(1+s^2) grows with u), so Newton iterates clamped to
// u <= ln(Phi/eta) (where g >= 0) decrease monotonically to the root after at
// most one step from the left.  asinh(e^w) is evaluated as w + ln 2 for
// w > 20 and as e^w for w < -20 (relative error below 1e-17 in both), so
// nothing overflows although exp(psi/a) exceeds the FP32 range.  The
// iteration runs in FP32 until the step is below 1e-4 (relative to u; the
// FP32 residual cannot resolve much less), then two FP64 Newton steps square
// the remaining error twice (1e-4 -> 1e-8 -> 1e-16).  Returns false when the
// second FP64 step is still above 1e-9.
__device__ __forceinline__ void asinh_exp(double w, double& A, double& dA) {
  if (w > 20.0) {
    A = w + 0.69314718055994531;
    dA = 1.0;
  } else if (w < -20.0) {
    A = exp(w);
    dA = A;
  } else {
    const double sw = exp(w);
    A = asinh(sw);
    dA = sw / sqrt(1.0 + sw * sw);
  }
}

__device__ bool newton_mixed(double& V, double Phi, double eta, double sn, double psi, double V0, double a,
                             double lnV0h) {
  const double target = Phi / eta;
  if (!(target > 0.0)) {
    V = 0.0;
    return true;
  }
  const double c = a * sn / eta;
  const double L = psi / a + lnV0h;  // ln(exp(psi/a)/(2 V0))
  const float tf = (float)target, cf = (float)c, Lf = (float)L;
  const float uhi = logf(tf);
  const float vf = (float)V;
  float u = vf > 0.0f ? fminf(logf(vf), uhi) : uhi;
  for (int it = 0; it < 40; ++it) {
    const float w = u + Lf;
    const float v = expf(u);
    float A, dA;
    if (w > 20.0f) {
      A = w + 0.6931471806f;
      dA = 1.0f;
    } else if (w < -20.0f) {
      A = expf(w);
      dA = A;
    } else {
      const float sw = expf(w);
      A = asinhf(sw);
      dA = sw / sqrtf(1.0f + sw * sw);
    }
    const float un = fminf(u - (v + cf * A - tf) / (v + cf * dA), uhi);
    const float du = un - u;
    u = un;
    if (fabsf(du) <= 1.0e-4f * fmaxf(1.0f, fabsf(u))) break;
  }
  double ud = (double)u, du = 0.0, v = 0.0;
  for (int it = 0; it < 2; ++it) {
    v = exp(ud);
    double A, dA;
    asinh_exp(ud + L, A, dA);
    du = -(v + c * A - target) / (v + c * dA);
    ud += du;
  }
  // exp(ud + du) from the last exp(ud): the series in du is exact to
  // rounding once |du| <= 1e-9 (the acceptance bound below)
  V = v * (1.0 + du * (1.0 + 0.5 * du));
  return fabs(du) <= 1.0e-9 * fmax(1.0, fabs(ud));
}

// The nine fields of one face point in the algebra type R.  With C (the
// Kahan compensation of FP32 fields) the value is the compensated one,
// F - C in FP64: the field to about twice the FP32 precision.
template <typename T, typename R>
__device__ __forceinline__ void load_face(const void* F, const void* C, long long np, long long p, R out[9]) {
  const T* f = (const T*)F;
  const comp_t* k = (const comp_t*)C;
#pragma unroll
  for (int c = 0; c < 9; ++c) out[c] = k ? (R)f[c * np + p] - (R)comp_get(k, c * np + p) : (R)f[c * np + p];
}

// T is the field type, R the arithmetic type of the characteristic algebra.
// FP64 fields (R = T = double) keep every operation of the FP64 restatement.
// FP32 fields either do the algebra in FP32 (R = float) or read the
// compensated face values and do it in FP64 (R = double); the slip, state,
// their rates and the friction law are FP64 in every case.  FP32 algebra:
// capped at 96 registers so that five 128-thread CTAs share an SM and a 201^2
// fault (2 x 40401 threads) runs in about one round (measured 0.092 -> 0.078
// ms per launch on config 1 despite some spilling).
template <typename T, typename R>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 5 : 3) interface_kernel(const __grid_constant__ InterfaceArgs a) {
  constexpr bool F64 = sizeof(T) == 8;
  const long long nf = (long long)a.nr * a.ns;
  const long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (f >= nf) return;
  const int j = (int)(f % a.nr), k = (int)(f / a.nr);
  // fields on both faces: block 0 at q = nq0-1, block 1 at q = 0
  R u[9], v[9];
  const long long pu = (a.nq0 - 1) + (long long)a.pq0 * (j + (long long)a.nr * k);
  const long long pv = (long long)a.pq1 * (j + (long long)a.nr * k);
  const bool comp = sizeof(R) > sizeof(T);
  load_face<T, R>(a.F0, comp ? a.C0 : nullptr, a.np0, pu, u);
  load_face<T, R>(a.F1, comp ? a.C1 : nullptr, a.np1, pv, v);
  if (a.ms0) {
    // manufactured solution: both sides' velocities and tractions less the
    // exact solution at their own fault points (src/CouplingForcing.f90:147-185)
    const T* s0 = (const T*)a.ms0;
    const T* s1 = (const T*)a.ms1;
    const R Tt = (R)a.mms_T;
    const R u_v = Tt * s0[pu], u_s = Tt * s0[a.np0 + pu];
    const R v_v = Tt * s1[pv], v_s = Tt * s1[a.np1 + pv];
#pragma unroll
    for (int c = 0; c < 9; ++c) {
      u[c] -= c < 3 ? u_v : u_s;
      v[c] -= c < 3 ? v_v : v_s;
    }
  }
  const double* face = b == 0 ? a.face0 : a.face1;
  R n[3], m[3], l[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    n[c] = (R)face[(0 + c) * nf + f];
    m[c] = (R)face[(3 + c) * nf + f];
    l[c] = (R)face[(6 + c) * nf + f];
  }
  const R gx = (R)face[9 * nf + f], gy = (R)face[10 * nf + f], gz = (R)face[11 * nf + f];
  // material on each side (block 0 / block 1 face)
  const R lam1 = (R)a.face0[12 * nf + f], mu1 = (R)a.face0[13 * nf + f], rho1 = (R)a.face0[14 * nf + f];
  const R lam2 = (R)a.face1[12 * nf + f], mu2 = (R)a.face1[13 * nf + f], rho2 = (R)a.face1[14 * nf + f];
  const R c1p = sqrt((R(2) * mu1 + lam1) / rho1), c1s = sqrt(mu1 / rho1);
  const R c2p = sqrt((R(2) * mu2 + lam2) / rho2), c2s = sqrt(mu2 / rho2);
  const R Z1p = rho1 * c1p, Z1s = rho1 * c1s, Z2p = rho2 * c2p, Z2s = rho2 * c2s;
  double x[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) x[c] = a.xij[(b * 3 + c) * nf + f];

  // tractions on the face, then rotate velocities and tractions to (n,m,l)
  R ur[6], vr[6];
  {
    const R Tu0 = n[0] * u[3] + n[1] * u[6] + n[2] * u[7];
    const R Tu1 = n[0] * u[6] + n[1] * u[4] + n[2] * u[8];
    const R Tu2 = n[0] * u[7] + n[1] * u[8] + n[2] * u[5];
    const R Tv0 = n[0] * v[3] + n[1] * v[6] + n[2] * v[7];
    const R Tv1 = n[0] * v[6] + n[1] * v[4] + n[2] * v[8];
    const R Tv2 = n[0] * v[7] + n[1] * v[8] + n[2] * v[5];
    ur[0] = n[0] * u[0] + n[1] * u[1] + n[2] * u[2];
    ur[1] = m[0] * u[0] + m[1] * u[1] + m[2] * u[2];
    ur[2] = l[0] * u[0] + l[1] * u[1] + l[2] * u[2];
    ur[3] = n[0] * Tu0 + n[1] * Tu1 + n[2] * Tu2;
    ur[4] = m[0] * Tu0 + m[1] * Tu1 + m[2] * Tu2;
    ur[5] = l[0] * Tu0 + l[1] * Tu1 + l[2] * Tu2;
    vr[0] = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
    vr[1] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
    vr[2] = l[0] * v[0] + l[1] * v[1] + l[2] * v[2];
    vr[3] = n[0] * Tv0 + n[1] * Tv1 + n[2] * Tv2;
    vr[4] = m[0] * Tv0 + m[1] * Tv1 + m[2] * Tv2;
    vr[5] = l[0] * Tv0 + l[1] * Tv1 + l[2] * Tv2;
  }

  // characteristics (src/Interface_Condition.f90:809-828)
  const R p_n = Z1p * ur[0] - ur[3], p_m = Z1s * ur[1] - ur[4], p_l = Z1s * ur[2] - ur[5];
  const R q_n = Z2p * vr[0] + vr[3], q_m = Z2s * vr[1] + vr[4], q_l = Z2s * vr[2] + vr[5];
  const R eta_s = R(1) / (R(1) / Z1s + R(1) / Z2s);
  const R eta_p = R(1) / (R(1) / Z1p + R(1) / Z2p);
  const R phi_n = eta_p * (q_n / Z2p - p_n / Z1p);
  const R phi_m = eta_s * (q_m / Z2s - p_m / Z1s);
  const R phi_l = eta_s * (q_l / Z2s - p_l / Z1s);

  double* S = a.S + (long long)b * 4 * nf;
  double* DS = a.DS + (long long)b * 4 * nf;
  double* W = a.W + (long long)b * nf;
  double* DW = a.DW + (long long)b * nf;
  double* trup = a.trup + (long long)b * nf;

  R P[6], Q[6];
  double T0n = 0.0, T0m = 0.0, T0l = 0.0;
  const int cpl = a.fp.coupling;
  if (cpl == CPL_LOCKED) {
    // Welded_Interface (src/Interface_Condition.f90:516-637)
    P[0] = (q_n - phi_n) / Z2p; P[1] = (q_m - phi_m) / Z2s; P[2] = (q_l - phi_l) / Z2s;
    Q[0] = (p_n + phi_n) / Z1p; Q[1] = (p_m + phi_m) / Z1s; Q[2] = (p_l + phi_l) / Z1s;
    P[3] = Q[3] = phi_n; P[4] = Q[4] = phi_m; P[5] = Q[5] = phi_l;
  } else if (cpl == CPL_LINEAR) {
    // Linear_Friction with alpha = 1e14 (src/Interface_Condition.f90:639-742)
    const R al = R(1.0e14);
    const R tm = al / (al + eta_s) * phi_m, tl = al / (al + eta_s) * phi_l;
    P[0] = (q_n - phi_n) / Z2p; Q[0] = (p_n + phi_n) / Z1p;
    Q[1] = (p_m + tm) / Z1s + R(1) / (al + eta_s) * phi_m;
    Q[2] = (p_l + tl) / Z1s + R(1) / (al + eta_s) * phi_l;
    P[1] = R(0);
    P[2] = (q_l - tl) / Z2s - R(1) / (al + eta_s) * phi_l;
    P[3] = Q[3] = phi_n; P[4] = Q[4] = tm; P[5] = Q[5] = tl;
  } else {
    // prestress: static part + nucleation weight x the stage's uniform ramp
    const double* pre = a.pre + (long long)b * 5 * nf;
    T0n = pre[f];
    T0m = pre[nf + f];
    T0l = pre[2 * nf + f];
    const double wn = pre[3 * nf + f];
    if (wn != 0.0) T0l = T0l + wn * a.ramp;
    // the friction law in FP64 for both field types
    const double phm = phi_m, phl = phi_l, phn = phi_n, es = eta_s;
    double tau_m_hat, tau_l_hat, vv_m, vv_l;
    const double phi_1 = T0m + phm, phi_2 = T0l + phl;
    if (cpl == CPL_SW) {
      // Slip_Weakening_Friction + solve (src/Interface_Condition.f90:745-916, 1147-1166)
      const double tau_lock = sqrt((T0l + phl) * (T0l + phl) + (T0m + phm) * (T0m + phm));
      const double sn = fmax(0.0, -(T0n + phn));
      const double tau_str = tau_strength(a.fp, sn, S[3 * nf + f], x, a.t);
      if (tau_lock > tau_str) {
        const double Phi = sqrt(phi_1 * phi_1 + phi_2 * phi_2);
        const double V = (Phi - tau_str) / es;
        vv_m = phi_1 / (es + tau_str / V);
        vv_l = phi_2 / (es + tau_str / V);
        tau_m_hat = (phi_1 - es * vv_m) - T0m;
        tau_l_hat = (phi_2 - es * vv_l) - T0l;
      } else {
        tau_m_hat = phm;
        tau_l_hat = phl;
        vv_m = vv_l = 0.0;
      }
    } else {
      // rate_state_friction + solve + Regula_Falsi (src/Interface_Condition.f90:918-1146)
      const double ra = pre[4 * nf + f];  // direct-effect parameter a(x)
      const RSParams rs = rs_params(a.fp, x, ra);
      const double psi = W[f];
      const double sn = fmax(0.0, -(T0n + phn));
      const double Phi = sqrt(phi_1 * phi_1 + phi_2 * phi_2);
      const double d1 = (double)vr[1] - (double)ur[1], d2 = (double)vr[2] - (double)ur[2];
      double V = sqrt(d1 * d1 + d2 * d2);
      if (V > Phi) V = 0.5 * Phi / es;
      const bool ok = F64 ? regula_falsi(V, Phi, es, sn, psi, rs.V0, rs.a, a.rs_tol, a.rs_maxit)
                          : newton_mixed(V, Phi, es, sn, psi, rs.V0, rs.a, a.lnV0h);
      if (!ok && a.solver_fail) atomicAdd(a.solver_fail, 1u);
      if (F64) {
        const double fv = sn * rs.a * asinh(0.5 * V / rs.V0 * exp(psi / rs.a));
        vv_m = phi_1 / (es + fv / V);
        vv_l = phi_2 / (es + fv / V);
      } else {
        // at the root the friction stress is Phi - eta*V, so
        // phi/(eta + fv/V) = phi*V/Phi
        const double ratio = Phi > 0.0 ? V / Phi : 0.0;
        vv_m = phi_1 * ratio;
        vv_l = phi_2 * ratio;
      }
      tau_m_hat = (phi_1 - es * vv_m) - T0m;
      tau_l_hat = (phi_2 - es * vv_l) - T0l;
      // aging law (src/Interface_Condition.f90:431-436); the FP32-field mode
      // multiplies by the reciprocals (FP64 division is slow on this part)
      if (a.fp.preset == PRE_RATE_WEAKENING) {
        DW[f] = a.A * DW[f] + rs_rate_weakening_state_rate(psi, V, rs.a, rs.b, rs.V0, rs.f0, rs.L0,
                                                            rs_weakening_velocity(x));
      } else if (F64) {
        DW[f] = a.A * DW[f] + (rs.b * rs.V0 / rs.L0 * exp(-(psi - rs.f0) / rs.b) - V * rs.b / rs.L0);
      } else {
        DW[f] = a.A * DW[f] + (a.rs_bL * rs.V0 * exp((rs.f0 - psi) * a.rs_binv) - V * a.rs_bL);
      }
    }
    const R tmh = (R)tau_m_hat, tlh = (R)tau_l_hat, vm = (R)vv_m, vl = (R)vv_l;
    P[0] = (q_n - phi_n) / Z2p;
    Q[0] = (p_n + phi_n) / Z1p;
    P[3] = Q[3] = phi_n;
    P[4] = Q[4] = tmh;
    P[5] = Q[5] = tlh;
    Q[1] = (tmh + p_m) / Z1s + vm;
    Q[2] = (tlh + p_l) / Z1s + vl;
    P[1] = (q_m - tmh) / Z2s - vm;
    P[2] = (q_l - tlh) / Z2s - vl;
  }
  const R srate = sqrt((Q[1] - P[1]) * (Q[1] - P[1]) + (Q[2] - P[2]) * (Q[2] - P[2]));

  // stage-1 outputs: rupture front and the fault frame (block 1's copy)
  if (a.stage == 1) {
    const R sv1 = Q[1] - P[1], sv2 = Q[2] - P[2];
    if (sqrt(sv1 * sv1 + sv2 * sv2) > R(1.0e-3)) trup[f] = fmin(trup[f], a.t);
    if (b == 0 && a.frame) {
      float* fr = a.frame;
#pragma unroll
      for (int c = 0; c < 9; ++c) {
        fr[(FR_UFACE + c) * nf + f] = (float)((const T*)a.F0)[c * a.np0 + pu];
        fr[(FR_VFACE + c) * nf + f] = (float)((const T*)a.F1)[c * a.np1 + pv];
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) fr[(FR_S + c) * nf + f] = (float)S[c * nf + f];
      const double T0[3] = {T0n, T0m, T0l};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float sv = (float)(Q[c] - P[c]);
        fr[(FR_UHAT + c) * nf + f] = sv;
        fr[(FR_VHAT + c) * nf + f] = sv;
        fr[(FR_SVEL + c) * nf + f] = sv;
        fr[(FR_UHAT + 3 + c) * nf + f] = (float)(P[3 + c] + T0[c]);
        fr[(FR_VHAT + 3 + c) * nf + f] = (float)(Q[3 + c] + T0[c]);
      }
      fr[FR_TRUP * nf + f] = (float)trup[f];
      fr[FR_STATE * nf + f] = (float)W[f];
    }
  }

  // slip and state: DS <- A*DS + rates, then the RK update of S and W
#pragma unroll
  for (int c = 0; c < 3; ++c) DS[c * nf + f] = a.A * DS[c * nf + f] + (double)(Q[c] - P[c]);
  DS[3 * nf + f] = a.A * DS[3 * nf + f] + (double)srate;
#pragma unroll
  for (int c = 0; c < 4; ++c) S[c * nf + f] += a.Bdt * DS[c * nf + f];
  if (cpl == CPL_RS) W[f] += a.Bdt * DW[f];

  // hat variables back to (x,y,z); grid values rotate back to themselves
  R uh[6], vh[6];
  auto back = [&](const R h[6], R o[6]) {
    o[0] = n[0] * h[0] + m[0] * h[1] + l[0] * h[2];
    o[1] = n[1] * h[0] + m[1] * h[1] + l[1] * h[2];
    o[2] = n[2] * h[0] + m[2] * h[1] + l[2] * h[2];
    o[3] = n[0] * h[3] + m[0] * h[4] + l[0] * h[5];
    o[4] = n[1] * h[3] + m[1] * h[4] + l[1] * h[5];
    o[5] = n[2] * h[3] + m[2] * h[4] + l[2] * h[5];
  };
  back(P, uh);
  back(Q, vh);
  R ug[6], vg[6];
  back(ur, ug);
  back(vr, vg);

  // SAT vector for this copy's block (src/CouplingForcing.f90:238-466)
  const R norm = sqrt(gx * gx + gy * gy + gz * gz);
  const R Zp = b == 0 ? Z1p : Z2p, Zs = b == 0 ? Z1s : Z2s;
  R Mm[3][3], Pm[3][3];
  const R* e[3] = {n, m, l};
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      // M = sum_k e_r[k] e_c[k] Z_k with Z = (Zp, Zs, Zs) by component index
      Mm[r][c] = e[r][0] * e[c][0] * Zp + e[r][1] * e[c][1] * Zs + e[r][2] * e[c][2] * Zs;
      Pm[r][c] = e[r][0] * e[c][0] * R(1) / Zp + e[r][1] * e[c][1] * R(1) / Zs + e[r][2] * e[c][2] * R(1) / Zs;
    }
  R dch[3];
  if (b == 0) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const R ph = R(0.5) * (Mm[r][0] * uh[0] + Mm[r][1] * uh[1] + Mm[r][2] * uh[2] + uh[3 + r]);
      const R pg = R(0.5) * (Mm[r][0] * ug[0] + Mm[r][1] * ug[1] + Mm[r][2] * ug[2] + ug[3 + r]);
      dch[r] = pg - ph;
    }
  } else {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const R qh = R(0.5) * (Mm[r][0] * vh[0] + Mm[r][1] * vh[1] + Mm[r][2] * vh[2] - vh[3 + r]);
      const R qg = R(0.5) * (Mm[r][0] * vg[0] + Mm[r][1] * vg[1] + Mm[r][2] * vg[2] - vg[3 + r]);
      dch[r] = qg - qh;
    }
  }
  R rr[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) rr[r] = Pm[r][0] * dch[0] + Pm[r][1] * dch[1] + Pm[r][2] * dch[2];
  const R lam = b == 0 ? lam1 : lam2, mu = b == 0 ? mu1 : mu2, rho = b == 0 ? rho1 : rho2;
  const R sgn = b == 0 ? R(1) : R(-1);
  const R l2m = R(2) * mu + lam;
  R sat[9];
  sat[0] = norm / rho * dch[0];
  sat[1] = norm / rho * dch[1];
  sat[2] = norm / rho * dch[2];
  sat[3] = sgn * (l2m * gx * rr[0] + lam * gy * rr[1] + lam * gz * rr[2]);
  sat[4] = sgn * (l2m * gy * rr[1] + lam * gz * rr[2] + lam * gx * rr[0]);
  sat[5] = sgn * (l2m * gz * rr[2] + lam * gy * rr[1] + lam * gx * rr[0]);
  sat[6] = sgn * (mu * (gy * rr[0] + gx * rr[1]));
  sat[7] = sgn * (mu * (gz * rr[0] + gx * rr[2]));
  sat[8] = sgn * (mu * (gz * rr[1] + gy * rr[2]));
  T* out = (T*)a.sat + (long long)b * 9 * nf;
  const R th = (R)a.tau_h[b];
#pragma unroll
  for (int c = 0; c < 9; ++c) out[c * nf + f] = th * sat[c];
}

}  // namespace

void launch_interface(const InterfaceArgs& a, void* stream) {
  const long long nf = (long long)a.nr * a.ns;
  dim3 blk(128), grd((unsigned)((nf + 127) / 128), 2);
  if (a.fp64) interface_kernel<double, double><<<grd, blk, 0, (cudaStream_t)stream>>>(a);
  else if (a.fault_comp) interface_kernel<float, double><<<grd, blk, 0, (cudaStream_t)stream>>>(a);
  else interface_kernel<float, float><<<grd, blk, 0, (cudaStream_t)stream>>>(a);
}

}  // namespace wql
