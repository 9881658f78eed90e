// One-time FP64 precompute on the device: metric terms, Jacobian, face
// frames and the per-point stencil coefficients.
//
//   metrics + J ....... derivatives (src/grid.f90:396-469) with the SBP-6
//                       operator (src/metrics.f90:16-488)
//   face frames ....... local_orth_vectors_{q,r,s} + gen_orth_vectors
//                       (src/unit_normals.f90:8-282)
//   coefficients ...... J*metric, 1/J, lambda, mu, 1/(rho*J), the terms the
//                       stencils of src/JU_xJU_yJU_z6.f90 multiply by
#include <cuda_runtime.h>

#include "wql_internal.h"
#include "wql_sbp.cuh"

namespace wql {
namespace {

__constant__ double c_sbp_setup[6][9] = WQL_SBP_TABLE;

// D(u)/h along one axis at 0-based index i (stride between neighbours `st`).
__device__ double deriv_fp64(const double* __restrict__ u, long long p, int i, int n,
                             long long st, double rh) {
  const int kind = sbp_kind(i, n);
  double s;
  if (kind == 0) {
    s = kC1 * (u[p + st] - u[p - st]) + kC2 * (u[p + 2 * st] - u[p - 2 * st]) +
        kC3 * (u[p + 3 * st] - u[p - 3 * st]);
  } else if (kind < 0) {
    const int row = -kind - 1;
    const long long p0 = p - (long long)i * st;
    s = 0.0;
    for (int c = 0; c < 9; ++c) s += c_sbp_setup[row][c] * u[p0 + c * st];
  } else {
    const int row = kind - 1;
    const long long pn = p + (long long)(n - 1 - i) * st;
    s = 0.0;
    for (int c = 0; c < 9; ++c) s += c_sbp_setup[row][c] * u[pn - c * st];
    s = -s;
  }
  return rh * s;
}

__global__ void metrics_kernel(int nq, int nr, int ns, const double* __restrict__ x,
                               double* __restrict__ metric, double* __restrict__ J) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nq || j >= nr || k >= ns) return;
  const long long np = (long long)nq * nr * ns;
  const long long p = i + (long long)nq * (j + (long long)nr * k);
  const long long st[3] = {1, nq, (long long)nq * nr};
  const int idx[3] = {i, j, k};
  const int n[3] = {nq, nr, ns};
  double Xd[3][3];  // Xd[d][c] = d x_c / d xi_d
  for (int d = 0; d < 3; ++d)
    for (int c = 0; c < 3; ++c)
      Xd[d][c] = deriv_fp64(x + c * np, p, idx[d], n[d], st[d], (double)(n[d] - 1));
  const double* Xq = Xd[0];
  const double* Xr = Xd[1];
  const double* Xs = Xd[2];
  const double Jp = Xq[0] * (Xr[1] * Xs[2] - Xr[2] * Xs[1]) - Xq[1] * (Xr[0] * Xs[2] - Xr[2] * Xs[0]) +
                    Xq[2] * (Xr[0] * Xs[1] - Xr[1] * Xs[0]);
  const double iJ = 1.0 / Jp;
  J[p] = Jp;
  // metric[3*j + d]: j = x,y,z component, d = q,r,s
  metric[0 * np + p] = iJ * (Xr[1] * Xs[2] - Xr[2] * Xs[1]);
  metric[1 * np + p] = iJ * (Xq[2] * Xs[1] - Xq[1] * Xs[2]);
  metric[2 * np + p] = iJ * (Xq[1] * Xr[2] - Xq[2] * Xr[1]);
  metric[3 * np + p] = iJ * (Xr[2] * Xs[0] - Xr[0] * Xs[2]);
  metric[4 * np + p] = iJ * (Xq[0] * Xs[2] - Xq[2] * Xs[0]);
  metric[5 * np + p] = iJ * (Xq[2] * Xr[0] - Xq[0] * Xr[2]);
  metric[6 * np + p] = iJ * (Xr[0] * Xs[1] - Xr[1] * Xs[0]);
  metric[7 * np + p] = iJ * (Xq[1] * Xs[0] - Xq[0] * Xs[1]);
  metric[8 * np + p] = iJ * (Xq[0] * Xr[1] - Xq[1] * Xr[0]);
}

struct FacePtrs {
  double* f[6];
};

__global__ void faces_kernel(int nq, int nr, int ns, const double* __restrict__ metric,
                             const double* __restrict__ lam, const double* __restrict__ mu,
                             const double* __restrict__ rho, FacePtrs out) {
  const int side = blockIdx.z;
  const int axis = side / 2;
  const bool hi = side & 1;
  const int na = axis == 0 ? nr : nq;
  const int nb = axis == 2 ? nr : ns;
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y * blockDim.y + threadIdx.y;
  if (a >= na || b >= nb) return;
  int i, j, k;
  if (axis == 0) { i = hi ? nq - 1 : 0; j = a; k = b; }
  else if (axis == 1) { i = a; j = hi ? nr - 1 : 0; k = b; }
  else { i = a; j = b; k = hi ? ns - 1 : 0; }
  const long long np = (long long)nq * nr * ns;
  const long long p = i + (long long)nq * (j + (long long)nr * k);
  const double gx = metric[(0 * 3 + axis) * np + p];
  const double gy = metric[(1 * 3 + axis) * np + p];
  const double gz = metric[(2 * 3 + axis) * np + p];
  const double norm = sqrt(gx * gx + gy * gy + gz * gz);
  const double n[3] = {gx / norm, gy / norm, gz / norm};
  // gen_orth_vectors: m seeded with y, Gram-Schmidt; z if n is parallel to y
  double m[3] = {0.0, 1.0, 0.0};
  const double d1 = sqrt((n[0] - m[0]) * (n[0] - m[0]) + (n[1] - m[1]) * (n[1] - m[1]) + (n[2] - m[2]) * (n[2] - m[2]));
  const double d2 = sqrt((n[0] + m[0]) * (n[0] + m[0]) + (n[1] + m[1]) * (n[1] + m[1]) + (n[2] + m[2]) * (n[2] + m[2]));
  if (!(d1 >= 1.0e-12 && d2 >= 1.0e-12)) { m[1] = 0.0; m[2] = 1.0; }
  const double an = n[0] * m[0] + n[1] * m[1] + n[2] * m[2];
  for (int c = 0; c < 3; ++c) m[c] -= an * n[c];
  const double inv = 1.0 / sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
  for (int c = 0; c < 3; ++c) m[c] *= inv;
  const double l[3] = {n[1] * m[2] - n[2] * m[1], n[2] * m[0] - n[0] * m[2], n[0] * m[1] - n[1] * m[0]};
  const long long nf = (long long)na * nb;
  const long long f = a + (long long)na * b;
  double* o = out.f[side];
  for (int c = 0; c < 3; ++c) {
    o[(0 + c) * nf + f] = n[c];
    o[(3 + c) * nf + f] = m[c];
    o[(6 + c) * nf + f] = l[c];
  }
  o[9 * nf + f] = gx;
  o[10 * nf + f] = gy;
  o[11 * nf + f] = gz;
  o[12 * nf + f] = lam[p];
  o[13 * nf + f] = mu[p];
  o[14 * nf + f] = rho[p];
}

template <typename T>
__global__ void coef_kernel(int nq, long long npd, int pq, long long np, int curv, const double* __restrict__ metric,
                            const double* __restrict__ J, const double* __restrict__ lam,
                            const double* __restrict__ mu, const double* __restrict__ rho,
                            T* __restrict__ coef) {
  // p: dense index of the precompute arrays; o: pitched index of coef
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= npd) return;
  const long long o = p % nq + (long long)pq * (p / nq);
  if (curv) {
    const double Jp = J[p];
    for (int d = 0; d < 3; ++d)
      for (int c = 0; c < 3; ++c) coef[(d * 3 + c) * np + o] = (T)(Jp * metric[(c * 3 + d) * npd + p]);
    coef[9 * np + o] = (T)(1.0 / Jp);
    coef[10 * np + o] = (T)lam[p];
    coef[11 * np + o] = (T)mu[p];
    coef[12 * np + o] = (T)(1.0 / (rho[p] * Jp));
  } else {
    coef[0 * np + o] = (T)lam[p];
    coef[1 * np + o] = (T)mu[p];
    coef[2 * np + o] = (T)(1.0 / rho[p]);
  }
}

}  // namespace

void launch_metrics(int nq, int nr, int ns, const double* x, double* metric, double* J,
                    void* stream) {
  dim3 blk(32, 4, 1), grd((nq + 31) / 32, (nr + 3) / 4, ns);
  metrics_kernel<<<grd, blk, 0, (cudaStream_t)stream>>>(nq, nr, ns, x, metric, J);
}

void launch_faces(int nq, int nr, int ns, const double* metric, const double* lam,
                  const double* mu, const double* rho, double* const face[6], void* stream) {
  FacePtrs fp;
  for (int s = 0; s < 6; ++s) fp.f[s] = face[s];
  const int mx = nq > nr ? nq : nr;
  const int my = nr > ns ? nr : ns;
  dim3 blk(32, 4, 1), grd((mx + 31) / 32, (my + 3) / 4, 6);
  faces_kernel<<<grd, blk, 0, (cudaStream_t)stream>>>(nq, nr, ns, metric, lam, mu, rho, fp);
}

template <typename T>
void launch_coef(int nq, int nr, int ns, int pq, bool curv, const double* metric, const double* J,
                 const double* lam, const double* mu, const double* rho, T* coef, void* stream) {
  const int blk = 256;
  const long long npd = (long long)nq * nr * ns, np = (long long)pq * nr * ns;
  const long long grd = (npd + blk - 1) / blk;
  coef_kernel<T><<<(unsigned)grd, blk, 0, (cudaStream_t)stream>>>(nq, npd, pq, np, curv ? 1 : 0, metric, J,
                                                                   lam, mu, rho, coef);
}

// Anelastic set-up, one thread per point (src/material.f90:69-74, 117-140):
// the quality factors from the relaxed shear speed, then the moduli that
// make the relaxed speeds the unrelaxed ones at the reference frequency.
struct AnelMat {
  double c, den[4], w[4];
};

__global__ void anelastic_material_kernel(long long n, AnelMat m, double* __restrict__ lam, double* __restrict__ mu,
                                          const double* __restrict__ rho, double* __restrict__ qsinv) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const double r = rho[p];
  const double qs = 1.0 / (m.c * sqrt(mu[p] / r));
  const double qp = 0.5 * qs;
  double val_S = 0.0, val_P = 0.0;
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const double denom_S = m.den[l] * (1.0 / qs) * 1.0;
    const double denom_P = m.den[l] * (1.0 / qp) * 1.0;
    val_S = val_S + m.w[l] / denom_S;
    val_P = val_P + m.w[l] / denom_P;
  }
  double vs = sqrt(mu[p] / r);
  double vp = sqrt((lam[p] + 2.0 * mu[p]) / r);
  const double mu_S = r * (vs * vs) / (1.0 - val_S);
  const double mu_P = r * (vp * vp) / (1.0 - val_P);
  vs = sqrt(mu_S / r);
  vp = sqrt(mu_P / r);
  const double mu_new = (vs * vs) * r;
  mu[p] = mu_new;
  lam[p] = (vp * vp) * r - 2.0 * mu_new;
  qsinv[p] = qs;
}

void launch_anelastic_material(long long n, double c, const double den[4], const double w[4], double* lam,
                               double* mu, const double* rho, double* qsinv, void* stream) {
  AnelMat m;
  m.c = c;
  for (int l = 0; l < 4; ++l) {
    m.den[l] = den[l];
    m.w[l] = w[l];
  }
  anelastic_material_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, m, lam, mu, rho,
                                                                                            qsinv);
}

// Manufactured-solution shapes (src/mms.f90:136-232), one thread per point,
// in FP64 from the dense grid and material: u_exact = T(t) S with
// S = sin(kx x) sin(ky y) sin(kz z) for the velocities and
// cos(kx x) cos(ky y) cos(kz z) for the stresses, T = cos(kt t); the operator
// shapes mp = A S_x + B S_y + C S_z of mms_forcing (src/mms.f90:104-122), so
// that the forcing f = A u_x + B u_y + C u_z - u_t is T(t) mp - T'(t) S; and
// the initial fields F = S (T(0) = 1).  Outputs are pitched (row pitch pq).
__global__ void mms_setup_kernel(long long npd, int nq, int pq, long long np, MmsWave w,
                                 const double* __restrict__ x, const double* __restrict__ lam,
                                 const double* __restrict__ mu, const double* __restrict__ rho, int fp64,
                                 void* ms, void* mp, void* F) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= npd) return;
  const long long o = p % nq + (long long)pq * (p / nq);
  const double X = x[p], Y = x[npd + p], Z = x[2 * npd + p];
  const double sx = sin(w.kx * X), sy = sin(w.ky * Y), sz = sin(w.kz * Z);
  const double cx = cos(w.kx * X), cy = cos(w.ky * Y), cz = cos(w.kz * Z);
  const double sv = sx * sy * sz, ss = cx * cy * cz;
  // space derivatives of the velocity and stress shapes
  const double vx = w.kx * cx * sy * sz, vy = w.ky * sx * cy * sz, vz = w.kz * sx * sy * cz;
  const double tx = -w.kx * sx * cy * cz, ty = -w.ky * cx * sy * cz, tz = -w.kz * cx * cy * sz;
  const double l = lam[p], m = mu[p], r = rho[p];
  double P[9];
  P[0] = (1.0 / r) * (tx + ty + tz);
  P[1] = P[0];
  P[2] = P[0];
  P[3] = (2.0 * m + l) * vx + l * vy + l * vz;
  P[4] = l * vx + (2.0 * m + l) * vy + l * vz;
  P[5] = l * vx + l * vy + (2.0 * m + l) * vz;
  P[6] = m * (vy + vx);
  P[7] = m * (vz + vx);
  P[8] = m * (vz + vy);
  if (fp64) {
    double* s = (double*)ms;
    double* q = (double*)mp;
    double* f = (double*)F;
    s[o] = sv;
    s[np + o] = ss;
    for (int c = 0; c < 9; ++c) {
      q[c * np + o] = P[c];
      f[c * np + o] = c < 3 ? sv : ss;
    }
  } else {
    float* s = (float*)ms;
    float* q = (float*)mp;
    float* f = (float*)F;
    s[o] = (float)sv;
    s[np + o] = (float)ss;
    for (int c = 0; c < 9; ++c) {
      q[c * np + o] = (float)P[c];
      f[c * np + o] = (float)(c < 3 ? sv : ss);
    }
  }
}

void launch_mms_setup(int nq, int nr, int ns, int pq, const MmsWave& w, const double* x, const double* lam,
                      const double* mu, const double* rho, bool fp64, void* ms, void* mp, void* F, void* stream) {
  const long long npd = (long long)nq * nr * ns, np = (long long)pq * nr * ns;
  mms_setup_kernel<<<(unsigned)((npd + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      npd, nq, pq, np, w, x, lam, mu, rho, fp64 ? 1 : 0, ms, mp, F);
}

// Sums over the points of one block, per field component, of
// (F - T S)^2 and (T S)^2 (acc[0..9) and acc[9..18), accumulated in FP64).
template <typename T>
__global__ void mms_norms_kernel(int nq, int nr, int ns, int pq, long long np, const T* __restrict__ F,
                                 const T* __restrict__ ms, double Tt, double* acc) {
  const long long npd = (long long)nq * nr * ns;
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double e[9], r[9];
  for (int c = 0; c < 9; ++c) e[c] = r[c] = 0.0;
  if (p < npd) {
    const long long o = p % nq + (long long)pq * (p / nq);
    const double sv = Tt * (double)ms[o], ss = Tt * (double)ms[np + o];
    for (int c = 0; c < 9; ++c) {
      const double u = c < 3 ? sv : ss;
      const double d = (double)F[c * np + o] - u;
      e[c] = d * d;
      r[c] = u * u;
    }
  }
  for (int c = 0; c < 9; ++c)
    for (int off = 16; off > 0; off >>= 1) {
      e[c] += __shfl_down_sync(0xffffffffu, e[c], off);
      r[c] += __shfl_down_sync(0xffffffffu, r[c], off);
    }
  if ((threadIdx.x & 31) == 0)
    for (int c = 0; c < 9; ++c) {
      atomicAdd(acc + c, e[c]);
      atomicAdd(acc + 9 + c, r[c]);
    }
}

template <typename T>
void launch_mms_norms(int nq, int nr, int ns, int pq, const T* F, const T* ms, double Tt, double* acc,
                      void* stream) {
  const long long npd = (long long)nq * nr * ns, np = (long long)pq * nr * ns;
  mms_norms_kernel<T><<<(unsigned)((npd + 255) / 256), 256, 0, (cudaStream_t)stream>>>(nq, nr, ns, pq, np, F, ms,
                                                                                       Tt, acc);
}
template void launch_mms_norms<double>(int, int, int, int, const double*, const double*, double, double*, void*);
template void launch_mms_norms<float>(int, int, int, int, const float*, const float*, double, double*, void*);

template void launch_coef<double>(int, int, int, int, bool, const double*, const double*, const double*,
                                  const double*, const double*, double*, void*);
template void launch_coef<float>(int, int, int, int, bool, const double*, const double*, const double*,
                                 const double*, const double*, float*, void*);

}  // namespace wql
