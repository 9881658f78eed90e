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
// reference's acceptance test `fv*fl > tol`.  Returns false when the
// iteration budget (5000) is exhausted.
__device__ bool regula_falsi(double& V, double Phi, double eta, double sn, double psi, double V0,
                             double a) {
  auto f = [&](double v) { return v + a * sn / eta * asinh(0.5 * v / V0 * exp(psi / a)) - Phi / eta; };
  const double tol = 1.0e-12;
  double Vl = 0.0, Vr = Phi / eta;
  double fv = f(V), fl = f(Vl), fr = f(Vr);
  if (fabs(fv) <= tol) return true;
  if (fabs(fl) <= tol) { V = Vl; return true; }
  if (fabs(fr) <= tol) { V = Vr; return true; }
  double err = 1.0;
  int k = 1;
  while (k <= 5000 && err >= tol) {
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
  return !(k >= 5000);
}

template <typename T>
__device__ __forceinline__ void load_face(const void* F, long long np, long long p, double out[9]) {
  const T* f = (const T*)F;
#pragma unroll
  for (int c = 0; c < 9; ++c) out[c] = (double)f[c * np + p];
}

template <typename T>
__global__ void interface_kernel(const InterfaceArgs a) {
  const long long nf = (long long)a.nr * a.ns;
  const long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (f >= nf) return;
  const int j = (int)(f % a.nr), k = (int)(f / a.nr);
  // fields on both faces: block 0 at q = nq0-1, block 1 at q = 0
  double u[9], v[9];
  load_face<T>(a.F0, a.np0, (a.nq0 - 1) + (long long)a.nq0 * (j + (long long)a.nr * k), u);
  {
    // block 1 has the same (nr, ns) face; its q stride is its own nq
    const long long nq1 = a.np1 / nf;
    load_face<T>(a.F1, a.np1, (long long)nq1 * (j + (long long)a.nr * k), v);
  }
  const double* face = b == 0 ? a.face0 : a.face1;
  double n[3], m[3], l[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    n[c] = face[(0 + c) * nf + f];
    m[c] = face[(3 + c) * nf + f];
    l[c] = face[(6 + c) * nf + f];
  }
  const double gx = face[9 * nf + f], gy = face[10 * nf + f], gz = face[11 * nf + f];
  // material on each side (block 0 / block 1 face)
  const double lam1 = a.face0[12 * nf + f], mu1 = a.face0[13 * nf + f], rho1 = a.face0[14 * nf + f];
  const double lam2 = a.face1[12 * nf + f], mu2 = a.face1[13 * nf + f], rho2 = a.face1[14 * nf + f];
  const double c1p = sqrt((2.0 * mu1 + lam1) / rho1), c1s = sqrt(mu1 / rho1);
  const double c2p = sqrt((2.0 * mu2 + lam2) / rho2), c2s = sqrt(mu2 / rho2);
  const double Z1p = rho1 * c1p, Z1s = rho1 * c1s, Z2p = rho2 * c2p, Z2s = rho2 * c2s;
  double x[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) x[c] = a.xij[(b * 3 + c) * nf + f];

  // tractions on the face, then rotate velocities and tractions to (n,m,l)
  double ur[6], vr[6];
  {
    const double Tu0 = n[0] * u[3] + n[1] * u[6] + n[2] * u[7];
    const double Tu1 = n[0] * u[6] + n[1] * u[4] + n[2] * u[8];
    const double Tu2 = n[0] * u[7] + n[1] * u[8] + n[2] * u[5];
    const double Tv0 = n[0] * v[3] + n[1] * v[6] + n[2] * v[7];
    const double Tv1 = n[0] * v[6] + n[1] * v[4] + n[2] * v[8];
    const double Tv2 = n[0] * v[7] + n[1] * v[8] + n[2] * v[5];
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
  const double p_n = Z1p * ur[0] - ur[3], p_m = Z1s * ur[1] - ur[4], p_l = Z1s * ur[2] - ur[5];
  const double q_n = Z2p * vr[0] + vr[3], q_m = Z2s * vr[1] + vr[4], q_l = Z2s * vr[2] + vr[5];
  const double eta_s = 1.0 / (1.0 / Z1s + 1.0 / Z2s);
  const double eta_p = 1.0 / (1.0 / Z1p + 1.0 / Z2p);
  const double phi_n = eta_p * (q_n / Z2p - p_n / Z1p);
  const double phi_m = eta_s * (q_m / Z2s - p_m / Z1s);
  const double phi_l = eta_s * (q_l / Z2s - p_l / Z1s);

  double* S = a.S + (long long)b * 4 * nf;
  double* DS = a.DS + (long long)b * 4 * nf;
  double* W = a.W + (long long)b * nf;
  double* DW = a.DW + (long long)b * nf;
  double* trup = a.trup + (long long)b * nf;

  double P[6], Q[6], Vel = 0.0;
  double T0n = 0.0, T0m = 0.0, T0l = 0.0;
  const int cpl = a.fp.coupling;
  if (cpl == CPL_LOCKED) {
    // Welded_Interface (src/Interface_Condition.f90:516-637)
    P[0] = (q_n - phi_n) / Z2p; P[1] = (q_m - phi_m) / Z2s; P[2] = (q_l - phi_l) / Z2s;
    Q[0] = (p_n + phi_n) / Z1p; Q[1] = (p_m + phi_m) / Z1s; Q[2] = (p_l + phi_l) / Z1s;
    P[3] = Q[3] = phi_n; P[4] = Q[4] = phi_m; P[5] = Q[5] = phi_l;
  } else if (cpl == CPL_LINEAR) {
    // Linear_Friction with alpha = 1e14 (src/Interface_Condition.f90:639-742)
    const double al = 1.0e14;
    const double tm = al / (al + eta_s) * phi_m, tl = al / (al + eta_s) * phi_l;
    P[0] = (q_n - phi_n) / Z2p; Q[0] = (p_n + phi_n) / Z1p;
    Q[1] = (p_m + tm) / Z1s + 1.0 / (al + eta_s) * phi_m;
    Q[2] = (p_l + tl) / Z1s + 1.0 / (al + eta_s) * phi_l;
    P[1] = 0.0;
    P[2] = (q_l - tl) / Z2s - 1.0 / (al + eta_s) * phi_l;
    P[3] = Q[3] = phi_n; P[4] = Q[4] = tm; P[5] = Q[5] = tl;
  } else {
    prestress(a.fp, x, a.t, l, m, n, T0n, T0m, T0l);
    double tau_m_hat, tau_l_hat, vv_m, vv_l;
    const double phi_1 = T0m + phi_m, phi_2 = T0l + phi_l;
    if (cpl == CPL_SW) {
      // Slip_Weakening_Friction + solve (src/Interface_Condition.f90:745-916, 1147-1166)
      const double tau_lock = sqrt((T0l + phi_l) * (T0l + phi_l) + (T0m + phi_m) * (T0m + phi_m));
      const double sn = fmax(0.0, -(T0n + phi_n));
      const double tau_str = tau_strength(a.fp, sn, S[3 * nf + f], x, a.t);
      if (tau_lock > tau_str) {
        const double Phi = sqrt(phi_1 * phi_1 + phi_2 * phi_2);
        const double V = (Phi - tau_str) / eta_s;
        Vel = V;
        vv_m = phi_1 / (eta_s + tau_str / V);
        vv_l = phi_2 / (eta_s + tau_str / V);
        tau_m_hat = (phi_1 - eta_s * vv_m) - T0m;
        tau_l_hat = (phi_2 - eta_s * vv_l) - T0l;
      } else {
        tau_m_hat = phi_m;
        tau_l_hat = phi_l;
        vv_m = vv_l = 0.0;
        Vel = 0.0;
      }
    } else {
      // rate_state_friction + solve + Regula_Falsi (src/Interface_Condition.f90:918-1146)
      const RSParams rs = rs_params(a.fp, x);
      const double psi = W[f];
      const double sn = fmax(0.0, -(T0n + phi_n));
      const double Phi = sqrt(phi_1 * phi_1 + phi_2 * phi_2);
      double V = sqrt((vr[1] - ur[1]) * (vr[1] - ur[1]) + (vr[2] - ur[2]) * (vr[2] - ur[2]));
      if (V > Phi) V = 0.5 * Phi / eta_s;
      if (!regula_falsi(V, Phi, eta_s, sn, psi, rs.V0, rs.a) && a.solver_fail)
        atomicAdd(a.solver_fail, 1u);
      Vel = V;
      const double fv = sn * rs.a * asinh(0.5 * V / rs.V0 * exp(psi / rs.a));
      vv_m = phi_1 / (eta_s + fv / V);
      vv_l = phi_2 / (eta_s + fv / V);
      tau_m_hat = (phi_1 - eta_s * vv_m) - T0m;
      tau_l_hat = (phi_2 - eta_s * vv_l) - T0l;
      // aging law (src/Interface_Condition.f90:431-436)
      DW[f] = a.A * DW[f] + (rs.b * rs.V0 / rs.L0 * exp(-(psi - rs.f0) / rs.b) - Vel * rs.b / rs.L0);
    }
    P[0] = (q_n - phi_n) / Z2p;
    Q[0] = (p_n + phi_n) / Z1p;
    P[3] = Q[3] = phi_n;
    P[4] = Q[4] = tau_m_hat;
    P[5] = Q[5] = tau_l_hat;
    Q[1] = (tau_m_hat + p_m) / Z1s + vv_m;
    Q[2] = (tau_l_hat + p_l) / Z1s + vv_l;
    P[1] = (q_m - tau_m_hat) / Z2s - vv_m;
    P[2] = (q_l - tau_l_hat) / Z2s - vv_l;
  }
  (void)Vel;
  const double srate = sqrt((Q[1] - P[1]) * (Q[1] - P[1]) + (Q[2] - P[2]) * (Q[2] - P[2]));

  // stage-1 outputs: rupture front and the fault frame (block 1's copy)
  if (a.stage == 1) {
    const double sv1 = Q[1] - P[1], sv2 = Q[2] - P[2];
    if (sqrt(sv1 * sv1 + sv2 * sv2) > 1.0e-3) trup[f] = fmin(trup[f], a.t);
    if (b == 0 && a.frame) {
      float* fr = a.frame;
#pragma unroll
      for (int c = 0; c < 9; ++c) {
        fr[(FR_UFACE + c) * nf + f] = (float)u[c];
        fr[(FR_VFACE + c) * nf + f] = (float)v[c];
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
  for (int c = 0; c < 3; ++c) DS[c * nf + f] = a.A * DS[c * nf + f] + (Q[c] - P[c]);
  DS[3 * nf + f] = a.A * DS[3 * nf + f] + srate;
#pragma unroll
  for (int c = 0; c < 4; ++c) S[c * nf + f] += a.Bdt * DS[c * nf + f];
  if (cpl == CPL_RS) W[f] += a.Bdt * DW[f];

  // hat variables back to (x,y,z); grid values rotate back to themselves
  double uh[6], vh[6];
  auto back = [&](const double h[6], double o[6]) {
    o[0] = n[0] * h[0] + m[0] * h[1] + l[0] * h[2];
    o[1] = n[1] * h[0] + m[1] * h[1] + l[1] * h[2];
    o[2] = n[2] * h[0] + m[2] * h[1] + l[2] * h[2];
    o[3] = n[0] * h[3] + m[0] * h[4] + l[0] * h[5];
    o[4] = n[1] * h[3] + m[1] * h[4] + l[1] * h[5];
    o[5] = n[2] * h[3] + m[2] * h[4] + l[2] * h[5];
  };
  back(P, uh);
  back(Q, vh);
  double ug[6], vg[6];
  back(ur, ug);
  back(vr, vg);

  // SAT vector for this copy's block (src/CouplingForcing.f90:238-466)
  const double norm = sqrt(gx * gx + gy * gy + gz * gz);
  const double Zp = b == 0 ? Z1p : Z2p, Zs = b == 0 ? Z1s : Z2s;
  double Mm[3][3], Pm[3][3];
  const double* e[3] = {n, m, l};
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      // M = sum_k e_r[k] e_c[k] Z_k with Z = (Zp, Zs, Zs) by component index
      Mm[r][c] = e[r][0] * e[c][0] * Zp + e[r][1] * e[c][1] * Zs + e[r][2] * e[c][2] * Zs;
      Pm[r][c] = e[r][0] * e[c][0] * 1.0 / Zp + e[r][1] * e[c][1] * 1.0 / Zs + e[r][2] * e[c][2] * 1.0 / Zs;
    }
  double dch[3];
  if (b == 0) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const double ph = 0.5 * (Mm[r][0] * uh[0] + Mm[r][1] * uh[1] + Mm[r][2] * uh[2] + uh[3 + r]);
      const double pg = 0.5 * (Mm[r][0] * ug[0] + Mm[r][1] * ug[1] + Mm[r][2] * ug[2] + ug[3 + r]);
      dch[r] = pg - ph;
    }
  } else {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const double qh = 0.5 * (Mm[r][0] * vh[0] + Mm[r][1] * vh[1] + Mm[r][2] * vh[2] - vh[3 + r]);
      const double qg = 0.5 * (Mm[r][0] * vg[0] + Mm[r][1] * vg[1] + Mm[r][2] * vg[2] - vg[3 + r]);
      dch[r] = qg - qh;
    }
  }
  double rr[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) rr[r] = Pm[r][0] * dch[0] + Pm[r][1] * dch[1] + Pm[r][2] * dch[2];
  const double lam = b == 0 ? lam1 : lam2, mu = b == 0 ? mu1 : mu2, rho = b == 0 ? rho1 : rho2;
  const double sgn = b == 0 ? 1.0 : -1.0;
  const double l2m = 2.0 * mu + lam;
  double sat[9];
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
#pragma unroll
  for (int c = 0; c < 9; ++c) out[c * nf + f] = (T)(a.tau_h[b] * sat[c]);
}

}  // namespace

void launch_interface(const InterfaceArgs& a, void* stream) {
  const long long nf = (long long)a.nr * a.ns;
  dim3 blk(128), grd((unsigned)((nf + 127) / 128), 2);
  if (a.fp64) interface_kernel<double><<<grd, blk, 0, (cudaStream_t)stream>>>(a);
  else interface_kernel<float><<<grd, blk, 0, (cudaStream_t)stream>>>(a);
}

}  // namespace wql
