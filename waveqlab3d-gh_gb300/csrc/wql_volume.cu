// Fused volume kernel: one RK stage of the elastic velocity-stress system on
// one block, per grid point:
//
//   DF <- A*DF + L(F)                 (scale_rates + set_rates,
//                                      src/fields.f90:49-108,
//                                      src/JU_xJU_yJU_z6.f90:12-812, 16141-16449,
//                                      src/RHS_Interior.f90:133-274)
//   DF -= PML damping, DQ <- A*DQ+..  (src/RHS_Interior.f90:1782-2201)
//   DF -= tau0/h * boundary SAT       (src/RHS_Interior.f90:1516-1703,
//                                      src/BoundaryConditions.f90:777-918 or
//                                      src/BoundaryConditions3.f90:777-903)
//   DF -= tau0/h * fault SAT          (src/RHS_Interior.f90:1706-1779; the SAT
//                                      vector comes from the interface kernel)
//   F_out = F_in + B*dt*DF            (update_fields, src/fields.f90:111-171;
//                                      Kahan-compensated in FP32 mode)
//   plastic return map on the last stage (src/plastic.f90:11-217)
//
// Curvilinear blocks use the conservative flux form for the stress
// divergence, D_d(J*metric*sigma)/(rho*J), and metric(centre)*D_d(v) for the
// velocity gradient; the three per-direction fluxes of each momentum
// component are combined before differencing (D is linear), so each point
// differences 6 quantities per axis.  Cartesian blocks use the diagonal
// constant metric.
#include <cuda_runtime.h>

#include "wql_internal.h"
#include "wql_sbp.cuh"

namespace wql {
namespace {

__constant__ double c_sbp_d[6][9] = WQL_SBP_TABLE;
__constant__ float c_sbp_f[6][9] = WQL_SBP_TABLE;

template <typename T>
__device__ __forceinline__ T sbp_w(int row, int col);
template <>
__device__ __forceinline__ double sbp_w<double>(int row, int col) { return c_sbp_d[row][col]; }
template <>
__device__ __forceinline__ float sbp_w<float>(int row, int col) { return c_sbp_f[row][col]; }

// sigma_{c,j} component index in F: rows x,y,z of the symmetric stress.
__device__ __forceinline__ int sig(int c, int j) {
  // sxx=3 syy=4 szz=5 sxy=6 sxz=7 syz=8
  const int t[3][3] = {{3, 6, 7}, {6, 4, 8}, {7, 8, 5}};
  return t[c][j];
}

// Load the six differenced quantities at point q for axis d: velocities
// and the momentum fluxes through the d-faces.
template <typename T, bool CURV>
__device__ __forceinline__ void load6(const T* __restrict__ F, const T* __restrict__ coef,
                                      long long np, long long q, int d, T o[6]) {
  o[0] = F[q];
  o[1] = F[np + q];
  o[2] = F[2 * np + q];
  if (CURV) {
    const T a = coef[(d * 3 + 0) * np + q], b = coef[(d * 3 + 1) * np + q],
            c = coef[(d * 3 + 2) * np + q];
    const T sxx = F[3 * np + q], syy = F[4 * np + q], szz = F[5 * np + q];
    const T sxy = F[6 * np + q], sxz = F[7 * np + q], syz = F[8 * np + q];
    o[3] = a * sxx + b * sxy + c * sxz;
    o[4] = a * sxy + b * syy + c * syz;
    o[5] = a * sxz + b * syz + c * szz;
  } else {
    o[3] = F[sig(0, d) * np + q];
    o[4] = F[sig(1, d) * np + q];
    o[5] = F[sig(2, d) * np + q];
  }
}

// Apply the SBP-6 derivative along axis d (0-based index i of n, stride st)
// to the six quantities of load6.  Result is not yet divided by h.
template <typename T, bool CURV>
__device__ __forceinline__ void diff6(const T* __restrict__ F, const T* __restrict__ coef,
                                      long long np, long long p, int i, int n, long long st, int d,
                                      T r[6]) {
  T t[6], u[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) r[c] = T(0);
  const int kind = sbp_kind(i, n);
  if (kind == 0) {
    const T cs[3] = {T(kC1), T(kC2), T(kC3)};
#pragma unroll
    for (int s = 1; s <= 3; ++s) {
      load6<T, CURV>(F, coef, np, p + s * st, d, t);
      load6<T, CURV>(F, coef, np, p - s * st, d, u);
#pragma unroll
      for (int c = 0; c < 6; ++c) r[c] += cs[s - 1] * (t[c] - u[c]);
    }
  } else if (kind < 0) {
    const int row = -kind - 1;
    const long long p0 = p - (long long)i * st;
    for (int col = 0; col < 9; ++col) {
      const T w = sbp_w<T>(row, col);
      if (w != T(0)) {
        load6<T, CURV>(F, coef, np, p0 + col * st, d, t);
#pragma unroll
        for (int c = 0; c < 6; ++c) r[c] += w * t[c];
      }
    }
  } else {
    const int row = kind - 1;
    const long long pn = p + (long long)(n - 1 - i) * st;
    for (int col = 0; col < 9; ++col) {
      const T w = -sbp_w<T>(row, col);
      if (w != T(0)) {
        load6<T, CURV>(F, coef, np, pn - col * st, d, t);
#pragma unroll
        for (int c = 0; c < 6; ++c) r[c] += w * t[c];
      }
    }
  }
}

// D_d of the three fluxes J*metric_j(d)*sigma_{c,j} (fixed physical axis j),
// needed only inside PML slabs (the per-axis split of the divergence).
template <typename T>
__device__ void diff_pml_flux(const T* __restrict__ F, const T* __restrict__ coef, long long np,
                              long long p, int i, int n, long long st, int d, int j, T r[3]) {
  r[0] = r[1] = r[2] = T(0);
  const int kind = sbp_kind(i, n);
  auto acc = [&](long long q, T w) {
    const T a = coef[(d * 3 + j) * np + q];
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c] += w * (a * F[sig(c, j) * np + q]);
  };
  if (kind == 0) {
    const T cs[3] = {T(kC1), T(kC2), T(kC3)};
    for (int s = 1; s <= 3; ++s) {
      acc(p + s * st, cs[s - 1]);
      acc(p - s * st, -cs[s - 1]);
    }
  } else if (kind < 0) {
    const int row = -kind - 1;
    const long long p0 = p - (long long)i * st;
    for (int col = 0; col < 9; ++col) {
      const T w = sbp_w<T>(row, col);
      if (w != T(0)) acc(p0 + col * st, w);
    }
  } else {
    const int row = kind - 1;
    const long long pn = p + (long long)(n - 1 - i) * st;
    for (int col = 0; col < 9; ++col) {
      const T w = -sbp_w<T>(row, col);
      if (w != T(0)) acc(pn - col * st, w);
    }
  }
}

// Characteristic boundary forcing (BCm / BCp), src/BoundaryConditions.f90:777-918,
// followed by structure() (src/RHS_Interior.f90:2203-2223); or the weighted
// alpha/theta form of src/BoundaryConditions3.f90:777-903 added directly.
// Returns sat (added to DF with -tau/h) and ubc (added to DQ in a PML).
__device__ void boundary_sat(const double u[9], const double* __restrict__ face, long long nf,
                             long long f, int code, bool plus, int form, double sat[9],
                             double ubc[9]) {
  double n[3], m[3], l[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    n[c] = face[(0 + c) * nf + f];
    m[c] = face[(3 + c) * nf + f];
    l[c] = face[(6 + c) * nf + f];
  }
  const double gx = face[9 * nf + f], gy = face[10 * nf + f], gz = face[11 * nf + f];
  const double lam = face[12 * nf + f], mu = face[13 * nf + f], rho = face[14 * nf + f];
  const double norm = sqrt(gx * gx + gy * gy + gz * gz);
  const double cp = sqrt((2.0 * mu + lam) / rho), cs = sqrt(mu / rho);
  const double Zp = rho * cp, Zs = rho * cs;
  double r, alpha, theta;
  if (code == 1) { r = 0.0; alpha = 2.0; theta = 0.0; }
  else if (code == 2) { r = 1.0; alpha = 1.0; theta = 0.0; }
  else { r = -1.0; alpha = 0.0; theta = plus ? 1.0 : -1.0; }
  const double T0 = n[0] * u[3] + n[1] * u[6] + n[2] * u[7];
  const double T1 = n[0] * u[6] + n[1] * u[4] + n[2] * u[8];
  const double T2 = n[0] * u[7] + n[1] * u[8] + n[2] * u[5];
  const double vl = l[0] * u[0] + l[1] * u[1] + l[2] * u[2];
  const double vm = m[0] * u[0] + m[1] * u[1] + m[2] * u[2];
  const double vn = n[0] * u[0] + n[1] * u[1] + n[2] * u[2];
  const double Tl = l[0] * T0 + l[1] * T1 + l[2] * T2;
  const double Tm = m[0] * T0 + m[1] * T1 + m[2] * T2;
  const double Tn = n[0] * T0 + n[1] * T1 + n[2] * T2;
  const double sg = plus ? 1.0 : -1.0;
  const double pl = 0.5 * ((1.0 - r) * Zs * vl + sg * (1.0 + r) * Tl);
  const double pm = 0.5 * ((1.0 - r) * Zs * vm + sg * (1.0 + r) * Tm);
  const double pn = 0.5 * ((1.0 - r) * Zp * vn + sg * (1.0 + r) * Tn);
  const double ql = 0.5 * ((1.0 - r) * vl + sg * (1.0 + r) / Zs * Tl);
  const double qm = 0.5 * ((1.0 - r) * vm + sg * (1.0 + r) / Zs * Tm);
  const double qn = 0.5 * ((1.0 - r) * vn + sg * (1.0 + r) / Zp * Tn);
  const double Fx = l[0] * pl + m[0] * pm + n[0] * pn;
  const double Fy = l[1] * pl + m[1] * pm + n[1] * pn;
  const double Fz = l[2] * pl + m[2] * pm + n[2] * pn;
  const double F_x = l[0] * ql + m[0] * qm + n[0] * qn;
  const double F_y = l[1] * ql + m[1] * qm + n[1] * qn;
  const double F_z = l[2] * ql + m[2] * qm + n[2] * qn;
  if (form == BC_WEIGHTED) {
    const double l2m = lam + 2.0 * mu;
    ubc[0] = alpha * norm / rho * Fx;
    ubc[1] = alpha * norm / rho * Fy;
    ubc[2] = alpha * norm / rho * Fz;
    ubc[3] = theta * norm * (l2m * n[0] * F_x + lam * (n[1] * F_y + n[2] * F_z));
    ubc[4] = theta * norm * (l2m * n[1] * F_y + lam * (n[0] * F_x + n[2] * F_z));
    ubc[5] = theta * norm * (l2m * n[2] * F_z + lam * (n[0] * F_x + n[1] * F_y));
    ubc[6] = theta * mu * norm * (n[1] * F_x + n[0] * F_y);
    ubc[7] = theta * mu * norm * (n[2] * F_x + n[0] * F_z);
    ubc[8] = theta * mu * norm * (n[2] * F_y + n[1] * F_z);
#pragma unroll
    for (int c = 0; c < 9; ++c) sat[c] = ubc[c];
    return;
  }
  ubc[0] = norm * Fx;
  ubc[1] = norm * Fy;
  ubc[2] = norm * Fz;
  ubc[3] = sg * (norm * n[0] * F_x);
  ubc[4] = sg * (norm * n[1] * F_y);
  ubc[5] = sg * (norm * n[2] * F_z);
  ubc[6] = sg * (norm * (n[1] * F_x + n[0] * F_y));
  ubc[7] = sg * (norm * (n[2] * F_x + n[0] * F_z));
  ubc[8] = sg * (norm * (n[2] * F_y + n[1] * F_z));
  sat[0] = 1.0 / rho * ubc[0];
  sat[1] = 1.0 / rho * ubc[1];
  sat[2] = 1.0 / rho * ubc[2];
  sat[3] = (2.0 * mu + lam) * ubc[3] + lam * (ubc[4] + ubc[5]);
  sat[4] = (2.0 * mu + lam) * ubc[4] + lam * (ubc[3] + ubc[5]);
  sat[5] = (2.0 * mu + lam) * ubc[5] + lam * (ubc[3] + ubc[4]);
  sat[6] = mu * ubc[6];
  sat[7] = mu * ubc[7];
  sat[8] = mu * ubc[8];
}

template <typename T, bool CURV, bool KAHAN>
__global__ void __launch_bounds__(256) volume_kernel(const VolumeArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= a.nq || j >= a.nr) return;
  const int nq = a.nq, nr = a.nr, ns = a.ns;
  const long long np = a.np;
  const long long p = i + (long long)nq * (j + (long long)nr * k);
  const long long st[3] = {1, nq, (long long)nq * nr};
  const int idx[3] = {i, j, k};
  const int nn[3] = {nq, nr, ns};
  const T* __restrict__ F = a.Fin;
  const T* __restrict__ coef = a.coef;

  T res[3][6];
#pragma unroll
  for (int d = 0; d < 3; ++d) diff6<T, CURV>(F, coef, np, p, idx[d], nn[d], st[d], d, res[d]);

  T lam, mu, rinv, Jinv = T(1);
  T g[3][3];  // g[c][j] = d v_c / d x_j
  T dv[3];    // momentum: divergence of stress
  if (CURV) {
    Jinv = coef[9 * np + p];
    lam = coef[10 * np + p];
    mu = coef[11 * np + p];
    rinv = coef[12 * np + p];  // 1/(rho J)
    T met[3][3];               // met[j][d] = metric_j(d) at the centre
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) met[jj][d] = coef[(d * 3 + jj) * np + p] * Jinv;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dv[c] = a.rh[0] * res[0][3 + c] + a.rh[1] * res[1][3 + c] + a.rh[2] * res[2][3 + c];
#pragma unroll
      for (int jj = 0; jj < 3; ++jj)
        g[c][jj] = met[jj][0] * (a.rh[0] * res[0][c]) + met[jj][1] * (a.rh[1] * res[1][c]) +
                   met[jj][2] * (a.rh[2] * res[2][c]);
    }
  } else {
    lam = coef[0 * np + p];
    mu = coef[1 * np + p];
    rinv = coef[2 * np + p];  // 1/rho
    T sc[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) sc[d] = a.cart_metric[d] * a.rh[d];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dv[c] = sc[0] * res[0][3 + c] + sc[1] * res[1][3 + c] + sc[2] * res[2][3 + c];
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) g[c][jj] = sc[jj] * res[jj][c];
    }
  }
  const T l2m = lam + T(2) * mu;
  T du[9];
  du[0] = rinv * dv[0];
  du[1] = rinv * dv[1];
  du[2] = rinv * dv[2];
  du[3] = l2m * g[0][0] + lam * (g[1][1] + g[2][2]);
  du[4] = l2m * g[1][1] + lam * (g[0][0] + g[2][2]);
  du[5] = l2m * g[2][2] + lam * (g[0][0] + g[1][1]);
  du[6] = mu * (g[0][1] + g[1][0]);
  du[7] = mu * (g[0][2] + g[2][0]);
  du[8] = mu * (g[1][2] + g[2][1]);

  // ---------------- PML (slabs of npml layers on the active sides) -------
  if (a.npml > 0) {
    const double d0 = 6.0 / (2.0 * 1.0) * log(1.0 / 1.0e-3);
    const T cfs = T(1);
    // reference order of the layers: s-low, s-high, r-low, r-high, q-low, q-high
    const int order[6] = {4, 5, 2, 3, 0, 1};
    for (int oi = 0; oi < 6; ++oi) {
      const int side = order[oi];
      if (!a.pml[side]) continue;
      const int axis = side >> 1;
      const bool hi = side & 1;
      const int ii = idx[axis], n = nn[axis], npml = a.npml;
      const bool in = hi ? (ii >= n - npml) : (ii < npml);
      if (!in) continue;
      // damping profile in grid-index units (src/RHS_Interior.f90:1855,1973,2092)
      double dd;
      if (axis == 2) dd = hi ? fabs((double)(ii + 1 - (n - npml)) / npml) : fabs((double)(ii + 1 - npml) / npml);
      else dd = hi ? fabs((double)(ii + 1 - (n - npml)) / npml) : fabs((double)(ii - npml) / npml);
      const T damp = (T)(d0 * dd);
      // slab index
      long long sp;
      if (axis == 0) sp = (hi ? ii - (n - npml) : ii) + (long long)npml * (j + (long long)nr * k);
      else if (axis == 1) sp = i + (long long)nq * ((hi ? ii - (n - npml) : ii) + (long long)npml * k);
      else sp = i + (long long)nq * (j + (long long)nr * (hi ? ii - (n - npml) : ii));
      const long long snp = a.slab_np[side];
      T* Q = a.Q[side];
      T* DQ = a.DQ[side];
      T q[9];
#pragma unroll
      for (int c = 0; c < 9; ++c) q[c] = Q[c * snp + sp];
      // per-axis stress derivative for the auxiliary sources
      T sd[3];
      const int jx = axis;  // physical axis paired with this side
      if (CURV) {
        T acc3[3] = {T(0), T(0), T(0)};
        for (int d = 0; d < 3; ++d) {
          T r3[3];
          diff_pml_flux<T>(F, coef, np, p, idx[d], nn[d], st[d], d, jx, r3);
#pragma unroll
          for (int c = 0; c < 3; ++c) acc3[c] += a.rh[d] * r3[c];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) sd[c] = acc3[c] * Jinv;
      } else {
        const T sc = a.cart_metric[jx] * a.rh[jx];
#pragma unroll
        for (int c = 0; c < 3; ++c) sd[c] = sc * res[jx][3 + c];
      }
      const T rhoinv = CURV ? (rinv / Jinv) : rinv;  // J/(rho J) = 1/rho
      du[0] -= damp * q[0] * rhoinv;
      du[1] -= damp * q[1] * rhoinv;
      du[2] -= damp * q[2] * rhoinv;
      du[3] -= damp * (l2m * q[3] + lam * q[4] + lam * q[5]);
      du[4] -= damp * (lam * q[3] + l2m * q[4] + lam * q[5]);
      du[5] -= damp * (lam * q[3] + lam * q[4] + l2m * q[5]);
      du[6] -= mu * damp * q[6];
      du[7] -= mu * damp * q[7];
      du[8] -= mu * damp * q[8];
      T src[9];
#pragma unroll
      for (int c = 0; c < 9; ++c) src[c] = T(0);
      src[0] = sd[0];
      src[1] = sd[1];
      src[2] = sd[2];
      // velocity-gradient sources (src/RHS_Interior.f90:1890-1907, 2008-2025, 2125-2142)
      if (jx == 0) { src[3] = g[0][0]; src[6] = g[1][0]; src[7] = g[2][0]; }
      else if (jx == 1) { src[4] = g[1][1]; src[6] = g[0][1]; src[8] = g[2][1]; }
      else { src[5] = g[2][2]; src[7] = g[0][2]; src[8] = g[1][2]; }
      T dq[9];
#pragma unroll
      for (int c = 0; c < 9; ++c) dq[c] = a.A * DQ[c * snp + sp] + src[c] - (damp + cfs) * q[c];
      // boundary SAT on this side's own face also drives DQ
      const bool on_face = hi ? (ii == n - 1) : (ii == 0);
      if (on_face && a.bc[side] >= 1 && a.bc[side] <= 3) {
        double u[9], sat[9], ubc[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) u[c] = (double)F[c * np + p];
        const int na = axis == 0 ? nr : nq;
        const long long f = axis == 0 ? (j + (long long)nr * k) : (axis == 1 ? (i + (long long)nq * k) : (i + (long long)nq * j));
        const long long nf = (long long)na * (axis == 2 ? nr : ns);
        boundary_sat(u, a.face[side], nf, f, a.bc[side], hi, a.bc_form, sat, ubc);
#pragma unroll
        for (int c = 0; c < 9; ++c) dq[c] -= a.tau_h[axis] * (T)ubc[c];
      }
#pragma unroll
      for (int c = 0; c < 9; ++c) {
        DQ[c * snp + sp] = dq[c];
        Q[c * snp + sp] = q[c] + a.Bdt * dq[c];
      }
    }
  }

  // ---------------- RK register: DF <- A*DF + L(F) -------------------------
  T df[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) df[c] = a.A * a.DF[c * np + p] + du[c];

  // ---------------- outer-boundary SAT --------------------------------------
  const bool on_boundary = (i == 0) | (i == nq - 1) | (j == 0) | (j == nr - 1) | (k == 0) | (k == ns - 1);
  if (on_boundary) {
    double u[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) u[c] = (double)F[c * np + p];
    for (int side = 0; side < 6; ++side) {
      const int code = a.bc[side];
      if (code < 1 || code > 3) continue;
      const int axis = side >> 1;
      const bool hi = side & 1;
      if (idx[axis] != (hi ? nn[axis] - 1 : 0)) continue;
      const int na = axis == 0 ? nr : nq;
      const long long nf = (long long)na * (axis == 2 ? nr : ns);
      const long long f = axis == 0 ? (j + (long long)nr * k) : (axis == 1 ? (i + (long long)nq * k) : (i + (long long)nq * j));
      double sat[9], ubc[9];
      boundary_sat(u, a.face[side], nf, f, code, hi, a.bc_form, sat, ubc);
#pragma unroll
      for (int c = 0; c < 9; ++c) df[c] -= a.tau_h[axis] * (T)sat[c];
    }
    // fault SAT on the interface face
    if (a.fault_sat && ((a.block == 0 && i == nq - 1) || (a.block == 1 && i == 0))) {
      const long long nf = (long long)nr * ns;
      const long long f = j + (long long)nr * k;
#pragma unroll
      for (int c = 0; c < 9; ++c) df[c] -= a.fault_sat[c * nf + f];
    }
  }

  // ---------------- update ---------------------------------------------------
  T fo[9];
  if (KAHAN) {
    T cc[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) {
      const T f0 = F[c * np + p];
      const T y = a.Bdt * df[c] - a.C[c * np + p];
      const T t = f0 + y;
      cc[c] = (t - f0) - y;
      fo[c] = t;
    }
    if (a.plastic) {
      // fall through to the plastic update below with the compensation kept
    }
#pragma unroll
    for (int c = 0; c < 9; ++c) a.C[c * np + p] = cc[c];
  } else {
#pragma unroll
    for (int c = 0; c < 9; ++c) fo[c] = F[c * np + p] + a.Bdt * df[c];
  }

  // ---------------- plasticity (last stage, non-PML points) ----------------
  if (a.plastic) {
    bool inside = true;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      if (a.pml[2 * ax] && idx[ax] < a.npml) inside = false;
      if (a.pml[2 * ax + 1] && idx[ax] >= nn[ax] - a.npml) inside = false;
    }
    if (inside) {
      double xs[3] = {0.0, (double)a.ycoord[p], 0.0}, s0[6];
      if (!initial_stress(a.preset, xs, s0))
        for (int c = 0; c < 6; ++c) s0[c] = a.s0u[c];
      T sa[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) sa[c] = fo[3 + c] + (T)s0[c];
      const T sigma = (sa[0] + sa[1] + sa[2]) / T(3);
      const T J2 = ((sa[0] - sa[1]) * (sa[0] - sa[1]) + (sa[1] - sa[2]) * (sa[1] - sa[2]) +
                    (sa[2] - sa[0]) * (sa[2] - sa[0])) / T(6) +
                   sa[3] * sa[3] + sa[4] * sa[4] + sa[5] * sa[5];
      const T tau = sqrt(J2);
      const T Ys = fmax(T(0), (T)(a.pl_c * cos(atan(a.pl_nu))) - sigma * (T)sin(atan(a.pl_nu)));
      if (tau - Ys > T(0)) {
        const T e = (T)exp(-a.dt / a.pl_Tv);
        const T r = e + (T(1) - e) * Ys / tau;
        const T delta[6] = {T(1), T(1), T(1), T(0), T(0), T(0)};
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const T sd = sa[c] - sigma * delta[c];
          fo[3 + c] = (sigma * delta[c] + r * sd) - (T)s0[c];
        }
        if (KAHAN)
#pragma unroll
          for (int c = 3; c < 9; ++c) a.C[c * np + p] = T(0);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    a.DF[c * np + p] = df[c];
    a.Fout[c * np + p] = fo[c];
  }
}

}  // namespace

template <typename T>
void launch_volume(const VolumeArgs<T>& a, bool curv, void* stream) {
  dim3 blk(32, 8, 1), grd((a.nq + 31) / 32, (a.nr + 7) / 8, a.ns);
  cudaStream_t s = (cudaStream_t)stream;
  const bool kahan = a.C != nullptr;
  if (curv) {
    if (kahan) volume_kernel<T, true, true><<<grd, blk, 0, s>>>(a);
    else volume_kernel<T, true, false><<<grd, blk, 0, s>>>(a);
  } else {
    if (kahan) volume_kernel<T, false, true><<<grd, blk, 0, s>>>(a);
    else volume_kernel<T, false, false><<<grd, blk, 0, s>>>(a);
  }
}

template void launch_volume<double>(const VolumeArgs<double>&, bool, void*);
template void launch_volume<float>(const VolumeArgs<float>&, bool, void*);

}  // namespace wql
