// Device helpers shared by the stencil kernels: the SBP-6 closure weights in
// constant memory, the row lookup of the first-derivative operator, the
// stress-component map, the tile ownership rule of the tiled kernels and
// the boundary/fault penalty of a face point.
// Included by each CUDA translation unit that differences fields (every
// unit gets its own constant-memory copy of the table).
#pragma once

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

// Upwind SBP-6 closure rows: [0] D+, [1] D-.
__constant__ double c_up_d[2][6][10] = WQL_UP_TABLE;
__constant__ float c_up_f[2][6][10] = WQL_UP_TABLE;

template <typename T>
__device__ __forceinline__ T up_w(int op, int row, int col);
template <>
__device__ __forceinline__ double up_w<double>(int op, int row, int col) { return c_up_d[op][row][col]; }
template <>
__device__ __forceinline__ float up_w<float>(int op, int row, int col) { return c_up_f[op][row][col]; }

// sigma_{c,j} component index in F: rows x,y,z of the symmetric stress.
__host__ __device__ constexpr int sig(int c, int j) {
  // sxx=3 syy=4 szz=5 sxy=6 sxz=7 syz=8
  return c == j ? 3 + c : 5 + c + j;
}

// ---------------------------------------------------------------------------
// SBP row lookup shared by every stencil: for a point at 0-based index i of
// n, entry t (0..8) of its row is weight w at offset off from i.  Central
// rows use entries 0..5, closure rows all nine (src/JU_xJU_yJU_z6.f90:55-164).
template <typename T>
__device__ __forceinline__ void row_entry(int kind, int t, T& w, int& off) {
  if (kind == 0) {
    const int k = t < 3 ? 3 - t : t - 2;  // 3,2,1 then 1,2,3
    const T c = k == 1 ? T(kC1) : (k == 2 ? T(kC2) : T(kC3));
    w = t < 3 ? -c : c;
    off = t < 3 ? -k : k;
    if (t > 5) { w = T(0); off = 0; }
  } else if (kind < 0) {  // left closure row i = -kind-1, columns are points 0..8
    const int i = -kind - 1;
    w = sbp_w<T>(i, t);
    off = t - i;
  } else {  // right closure row k = n-1-i, columns are points n-1..n-9
    const int k = kind - 1;
    w = -sbp_w<T>(k, t);
    off = k - t;
  }
}

// Closure entry t (0..9) of the upwind pair at a closure row (kind as
// sbp_kind, nonzero): the D+ weight wv (velocities), the D- weight wf
// (fluxes) and the offset from the point.  Left rows read points 0..9,
// right rows the mirror images; the right rows of D+ are the negated left
// rows of D- and the other way round.
template <typename T>
__device__ __forceinline__ void up_entry(int kind, int t, T& wv, T& wf, int& off) {
  if (kind < 0) {
    const int i = -kind - 1;
    wv = up_w<T>(0, i, t);
    wf = up_w<T>(1, i, t);
    off = t - i;
  } else {
    const int k = kind - 1;
    wv = -up_w<T>(1, k, t);
    wf = -up_w<T>(0, k, t);
    off = k - t;
  }
}


// The upwind pair of a kernel's operator FD (1: order 6, 2: order 5):
// closure rows R per end, closure columns NCOL, interior D+ offsets
// -2..PHI (D- offsets -PHI..2).
__constant__ double c_up5_d[2][4][7] = WQL_UP5_TABLE;
__constant__ float c_up5_f[2][4][7] = WQL_UP5_TABLE;
template <int FD>
struct UpOp {
  static constexpr int R = FD == 2 ? 4 : 6, NCOL = FD == 2 ? 7 : 10, PHI = FD == 2 ? 3 : 4;
};
template <int FD>
__device__ __forceinline__ int up_kind(int i, int n) {
  constexpr int R = UpOp<FD>::R;
  if (i < R) return -(i + 1);
  if (i >= n - R) return n - i;
  return 0;
}
template <typename T, int FD>
__device__ __forceinline__ T upw(int op, int row, int col) {
  if (FD == 2) return sizeof(T) == 8 ? (T)c_up5_d[op][row][col] : (T)c_up5_f[op][row][col];
  return up_w<T>(op, row, col);
}
// Interior D+ weight at offset o (-2..PHI).
template <typename T, int FD>
__device__ __forceinline__ T up_cf(int o) {
  if (FD == 2) {
    const T cf[6] = WQL_UP5_CF;
    return cf[o + 2];
  }
  const T cf[7] = WQL_UP_CF;
  return cf[o + 2];
}
// Closure entry t (0..NCOL-1) of operator FD on axis ax, as up_entry.
template <typename T, int FD>
__device__ __forceinline__ void upx_entry(int kind, int t, int ax, T& wv, T& wf, int& off) {
  if (kind < 0) {
    const int i = -kind - 1;
    wv = upw<T, FD>(0, i, t);
    wf = upw<T, FD>(1, i, t);
    off = t - i;
  } else {
    const int k = kind - 1;
    wv = -upw<T, FD>(1, k, t);
    wf = -upw<T, FD>(0, k, t);
    off = k - t;
  }
}

struct TileSpan {
  int origin, own_lo, own_hi;
};
__device__ __forceinline__ TileSpan tile_span(int t, int n, int T_) {
  const int ntiles = (n + T_ - 1) / T_;
  TileSpan sp;
  if (n <= T_) {
    sp.origin = 0; sp.own_lo = 0; sp.own_hi = n;
  } else if (t == ntiles - 1) {
    sp.origin = n - T_; sp.own_lo = n - T_; sp.own_hi = n;
  } else {
    sp.origin = t * T_; sp.own_lo = t * T_; sp.own_hi = min((t + 1) * T_, n - T_);
  }
  return sp;
}

// Characteristic boundary forcing (BCm / BCp), src/BoundaryConditions.f90:777-918,
// followed by structure() (src/RHS_Interior.f90:2203-2223); or the weighted
// alpha/theta form of src/BoundaryConditions3.f90:777-903 added directly.
// Returns sat (added to DF with -tau/h) and ubc (added to DQ in a PML).
template <typename R>
__device__ void boundary_sat(const R u[9], const double* __restrict__ face, long long nf, long long f, int code,
                             bool plus, int form, R sat[9], R ubc[9]) {
  R n[3], m[3], l[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    n[c] = (R)face[(0 + c) * nf + f];
    m[c] = (R)face[(3 + c) * nf + f];
    l[c] = (R)face[(6 + c) * nf + f];
  }
  const R gx = (R)face[9 * nf + f], gy = (R)face[10 * nf + f], gz = (R)face[11 * nf + f];
  const R lam = (R)face[12 * nf + f], mu = (R)face[13 * nf + f], rho = (R)face[14 * nf + f];
  const R norm = sqrt(gx * gx + gy * gy + gz * gz);
  const R cp = sqrt((R(2.0) * mu + lam) / rho), cs = sqrt(mu / rho);
  const R Zp = rho * cp, Zs = rho * cs;
  R r, alpha, theta;
  if (code == 1) { r = R(0.0); alpha = R(2.0); theta = R(0.0); }
  else if (code == 2) { r = R(1.0); alpha = R(1.0); theta = R(0.0); }
  else { r = -R(1.0); alpha = R(0.0); theta = plus ? R(1.0) : -R(1.0); }
  const R T0 = n[0] * u[3] + n[1] * u[6] + n[2] * u[7];
  const R T1 = n[0] * u[6] + n[1] * u[4] + n[2] * u[8];
  const R T2 = n[0] * u[7] + n[1] * u[8] + n[2] * u[5];
  const R vl = l[0] * u[0] + l[1] * u[1] + l[2] * u[2];
  const R vm = m[0] * u[0] + m[1] * u[1] + m[2] * u[2];
  const R vn = n[0] * u[0] + n[1] * u[1] + n[2] * u[2];
  const R Tl = l[0] * T0 + l[1] * T1 + l[2] * T2;
  const R Tm = m[0] * T0 + m[1] * T1 + m[2] * T2;
  const R Tn = n[0] * T0 + n[1] * T1 + n[2] * T2;
  const R sg = plus ? R(1.0) : -R(1.0);
  const R pl = R(0.5) * ((R(1.0) - r) * Zs * vl + sg * (R(1.0) + r) * Tl);
  const R pm = R(0.5) * ((R(1.0) - r) * Zs * vm + sg * (R(1.0) + r) * Tm);
  const R pn = R(0.5) * ((R(1.0) - r) * Zp * vn + sg * (R(1.0) + r) * Tn);
  const R ql = R(0.5) * ((R(1.0) - r) * vl + sg * (R(1.0) + r) / Zs * Tl);
  const R qm = R(0.5) * ((R(1.0) - r) * vm + sg * (R(1.0) + r) / Zs * Tm);
  const R qn = R(0.5) * ((R(1.0) - r) * vn + sg * (R(1.0) + r) / Zp * Tn);
  const R Fx = l[0] * pl + m[0] * pm + n[0] * pn;
  const R Fy = l[1] * pl + m[1] * pm + n[1] * pn;
  const R Fz = l[2] * pl + m[2] * pm + n[2] * pn;
  const R F_x = l[0] * ql + m[0] * qm + n[0] * qn;
  const R F_y = l[1] * ql + m[1] * qm + n[1] * qn;
  const R F_z = l[2] * ql + m[2] * qm + n[2] * qn;
  if (form == BC_WEIGHTED) {
    const R l2m = lam + R(2.0) * mu;
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
  sat[0] = R(1.0) / rho * ubc[0];
  sat[1] = R(1.0) / rho * ubc[1];
  sat[2] = R(1.0) / rho * ubc[2];
  sat[3] = (R(2.0) * mu + lam) * ubc[3] + lam * (ubc[4] + ubc[5]);
  sat[4] = (R(2.0) * mu + lam) * ubc[4] + lam * (ubc[3] + ubc[5]);
  sat[5] = (R(2.0) * mu + lam) * ubc[5] + lam * (ubc[3] + ubc[4]);
  sat[6] = mu * ubc[6];
  sat[7] = mu * ubc[7];
  sat[8] = mu * ubc[8];
}

// Adds corr to DF and B*dt*corr to the updated field of one point
// (compensated in FP32C).
template <typename T, bool KAHAN>
__device__ __forceinline__ void add_correction(const VolumeArgs<T>& a, long long p, const T (&corr)[9]) {
  const long long np = a.np;
  // DF, F_out and C are distinct arrays: a component's loads need not wait
  // for the previous component's stores
  T* __restrict__ DF = a.DF;
  T* __restrict__ Fo = a.Fout;
  comp_t* __restrict__ Ck = a.C;
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    if (corr[c] == T(0)) continue;
    DF[c * np + p] += corr[c];
    const T f0 = Fo[c * np + p];
    if (KAHAN) {
      const T y = a.Bdt * corr[c] - (T)comp_get(Ck, c * np + p);
      const T t = f0 + y;
      comp_put(Ck, c * np + p, (float)((t - f0) - y));
      Fo[c * np + p] = t;
    } else {
      Fo[c * np + p] = f0 + a.Bdt * corr[c];
    }
  }
}

// Sum of the penalty terms at a block-face point (i, j, k) with fields u:
// the outer-boundary SAT of every side with a boundary code 1..3 that the
// point lies on, times that axis's tau0/h (src/RHS_Interior.f90:1516-1703),
// plus the fault SAT on the interface face (src/RHS_Interior.f90:1757-1772).
// The caller subtracts tot from the rates.  Returns false if the point has
// no penalised face.  Inlined: as a call its array arguments went through
// the stack.
template <typename T>
__device__ __forceinline__ bool face_penalty(const VolumeArgs<T>& a, int i, int j, int k, const T* u, T* tot) {
  const int nq = a.nq, nr = a.nr, ns = a.ns;
  bool any = false;
  for (int c = 0; c < 9; ++c) tot[c] = T(0);
  for (int s2 = 0; s2 < 6; ++s2) {
    const int code = a.bc[s2];
    if (code < 1 || code > 3) continue;
    const int ax2 = s2 >> 1;
    const bool hi = s2 & 1;
    // selects, not arrays indexed by ax2 (those went to local memory)
    const int ii = ax2 == 0 ? i : (ax2 == 1 ? j : k), n2 = ax2 == 0 ? nq : (ax2 == 1 ? nr : ns);
    if (ii != (hi ? n2 - 1 : 0)) continue;
    const int na = ax2 == 0 ? nr : nq;
    const long long nf = (long long)na * (ax2 == 2 ? nr : ns);
    const long long f = ax2 == 0 ? (j + (long long)nr * k) : (ax2 == 1 ? (i + (long long)nq * k) : (i + (long long)nq * j));
    T sat[9], ubc[9];
    boundary_sat(u, a.face[s2], nf, f, code, hi, a.bc_form, sat, ubc);
    for (int c = 0; c < 9; ++c) tot[c] += a.tau_h[ax2] * sat[c];
    any = true;
  }
  if (a.fault_sat && ((a.block == 0 && i == nq - 1) || (a.block == 1 && i == 0))) {
    const long long nf = (long long)nr * ns;
    const long long f = j + (long long)nr * k;
    for (int c = 0; c < 9; ++c) tot[c] += a.fault_sat[c * nf + f];
    any = true;
  }
  return any;
}

}  // namespace
}  // namespace wql
