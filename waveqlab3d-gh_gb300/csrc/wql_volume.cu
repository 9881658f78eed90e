// Volume kernels: one RK stage of the elastic velocity-stress system on one
// block.  The stencil kernel does the bulk per grid point; small correction
// kernels add the PML, boundary/fault penalties and the plastic map:
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
#include "wql_stencil.cuh"

namespace wql {
namespace {

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

// SBP-6 derivative along one axis of the three velocities only (no flux).
template <typename T>
__device__ __forceinline__ void diff_v(const T* __restrict__ F, long long np, long long p, int i, int n, long long st,
                                       T r[3]) {
  r[0] = r[1] = r[2] = T(0);
  const int kind = sbp_kind(i, n);
  if (kind == 0) {
    const T cs[3] = {T(kC1), T(kC2), T(kC3)};
#pragma unroll
    for (int s = 1; s <= 3; ++s)
#pragma unroll
      for (int c = 0; c < 3; ++c) r[c] += cs[s - 1] * (F[c * np + p + s * st] - F[c * np + p - s * st]);
  } else if (kind < 0) {
    const int row = -kind - 1;
    const long long p0 = p - (long long)i * st;
    for (int col = 0; col < 9; ++col) {
      const T w = sbp_w<T>(row, col);
      if (w != T(0))
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] += w * F[c * np + p0 + col * st];
    }
  } else {
    const int row = kind - 1;
    const long long pn = p + (long long)(n - 1 - i) * st;
    for (int col = 0; col < 9; ++col) {
      const T w = -sbp_w<T>(row, col);
      if (w != T(0))
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] += w * F[c * np + pn - col * st];
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


// ---------------------------------------------------------------------------
// Upwind SBP-6 (fd 1, src/JU_xJU_yJU_z6.f90:2680-3706, 17675-17983): D+ on
// the velocities, D- on the fluxes.  Interior D+ weights on offsets -2..4
// and D- weights on offsets -4..2; the closure rows of both operators cover
// the same columns, so one load per column serves both.
template <typename T, bool CURV, int FD>
__device__ __forceinline__ void diff6_up(const T* __restrict__ F, const T* __restrict__ coef, long long np,
                                         long long p, int i, int n, long long st, int d, T r[6]) {
  constexpr int PHI = UpOp<FD>::PHI, NCOL = UpOp<FD>::NCOL;
  T t[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) r[c] = T(0);
  const int kind = up_kind<FD>(i, n);
  if (kind == 0) {
#pragma unroll
    for (int o = -PHI; o <= PHI; ++o) {
      load6<T, CURV>(F, coef, np, p + o * st, d, t);
      if (o >= -2)
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] += up_cf<T, FD>(o) * t[c];
      if (o <= 2)
#pragma unroll
        for (int c = 3; c < 6; ++c) r[c] -= up_cf<T, FD>(-o) * t[c];
    }
  } else {
    const long long base = kind < 0 ? p - (long long)i * st : p + (long long)(n - 1 - i) * st;
    for (int col = 0; col < NCOL; ++col) {
      T wv, wf;
      int off;
      upx_entry<T, FD>(kind, col, d, wv, wf, off);
      if (wv != T(0) || wf != T(0)) {
        load6<T, CURV>(F, coef, np, base + (kind < 0 ? col : -col) * st, d, t);
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] += wv * t[c];
#pragma unroll
        for (int c = 3; c < 6; ++c) r[c] += wf * t[c];
      }
    }
  }
}

// D+ of the three velocities only, along axis d.
template <typename T, int FD>
__device__ __forceinline__ void diff_v_up(const T* __restrict__ F, long long np, long long p, int i, int n,
                                          long long st, int d, T r[3]) {
  constexpr int PHI = UpOp<FD>::PHI, NCOL = UpOp<FD>::NCOL;
  r[0] = r[1] = r[2] = T(0);
  const int kind = up_kind<FD>(i, n);
  if (kind == 0) {
#pragma unroll
    for (int o = -2; o <= PHI; ++o)
#pragma unroll
      for (int c = 0; c < 3; ++c) r[c] += up_cf<T, FD>(o) * F[c * np + p + o * st];
  } else {
    const long long base = kind < 0 ? p - (long long)i * st : p + (long long)(n - 1 - i) * st;
    for (int col = 0; col < NCOL; ++col) {
      T wv, wf;
      int off;
      upx_entry<T, FD>(kind, col, d, wv, wf, off);
      if (wv != T(0))
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] += wv * F[c * np + base + (kind < 0 ? col : -col) * st];
    }
  }
}

// D- of the three fluxes J*metric_j(d)*sigma_{c,j} (PML split, as
// diff_pml_flux).
template <typename T, int FD>
__device__ void diff_pml_flux_up(const T* __restrict__ F, const T* __restrict__ coef, long long np, long long p,
                                 int i, int n, long long st, int d, int j, T r[3]) {
  constexpr int PHI = UpOp<FD>::PHI, NCOL = UpOp<FD>::NCOL;
  r[0] = r[1] = r[2] = T(0);
  const int kind = up_kind<FD>(i, n);
  auto acc = [&](long long q, T w) {
    const T a = coef[(d * 3 + j) * np + q];
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c] += w * (a * F[sig(c, j) * np + q]);
  };
  if (kind == 0) {
#pragma unroll
    for (int o = -PHI; o <= 2; ++o) acc(p + o * st, -up_cf<T, FD>(-o));
  } else {
    const long long base = kind < 0 ? p - (long long)i * st : p + (long long)(n - 1 - i) * st;
    for (int col = 0; col < NCOL; ++col) {
      T wv, wf;
      int off;
      upx_entry<T, FD>(kind, col, d, wv, wf, off);
      if (wf != T(0)) acc(base + (kind < 0 ? col : -col) * st, wf);
    }
  }
}

// ---- table upwind operators (fd 3), as the reference applies them: the
// near-boundary routine JJU_x<order>_upwind(_drp) at points of the boundary
// shell (its closure rows, and its interior case bp/bm on the axes where the
// point is interior), the interior routine JJU_x<order>_interior_upwind(_drp)
// (ip/im) at the other points (src/RHS_Interior.f90:40-125, 276-1512).
template <typename T>
__device__ __forceinline__ T ugw(const UpG& g, int idx) {
  return ((const T*)g.w)[idx];
}

// Whether point idx lies in the boundary shell: outside [lo, n-1-hi] on some
// axis, with lo and hi the closure rows R, or npml on a PML side if larger
// (the interior limits of the interior routines).
template <typename T>
__device__ __forceinline__ bool ug_shell(const VolumeArgs<T>& a, const int idx[3], const int nn[3]) {
  bool shell = false;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int lo = a.pml[2 * d] ? max(a.ug.R, a.npml) : a.ug.R;
    const int hi = a.pml[2 * d + 1] ? max(a.ug.R, a.npml) : a.ug.R;
    shell = shell || idx[d] < lo || idx[d] > nn[d] - 1 - hi;
  }
  return shell;
}

// Weights of the D+ (plus) or D- row at 0-based index i of n along axis d:
// calls f(offset from the point, weight) for each nonzero weight.
template <typename T, typename Fn>
__device__ __forceinline__ void ug_row(const UpG& g, bool shell, bool plus, int i, int n, int d, Fn&& f) {
  if (i >= g.R && i < n - g.R) {
    const int base = (shell ? 2 * kUgCol : 0) + (plus ? 0 : kUgCol);
    const int lo = plus ? g.plo : g.mlo, cnt = plus ? g.pn : g.mn;
    for (int k = 0; k < cnt; ++k) {
      const T w = ugw<T>(g, base + k);
      if (w != T(0)) f(lo + k, w);
    }
  } else if (i < g.R) {  // left row i, points 0..12
    const int base = 4 * kUgCol + (plus ? 0 : kUgRowBlock) + (d * kUgRows + i) * kUgCol;
    for (int t = 0; t < kUgCol; ++t) {
      const T w = ugw<T>(g, base + t);
      if (w != T(0)) f(t - i, w);
    }
  } else {  // right row k = n-1-i, points n-1-t
    const int k = n - 1 - i;
    const int base = 4 * kUgCol + (plus ? 2 : 3) * kUgRowBlock + (d * kUgRows + k) * kUgCol;
    for (int t = 0; t < kUgCol; ++t) {
      const T w = ugw<T>(g, base + t);
      if (w != T(0)) f(k - t, w);
    }
  }
}

// The six differenced quantities of load6 along axis d: D+ of the
// velocities, D- of the d-face momentum fluxes.
template <typename T, bool CURV>
__device__ void diff6_ug(const T* __restrict__ F, const T* __restrict__ coef, long long np, long long p, int i,
                         int n, long long st, int d, const UpG& g, bool shell, T r[6]) {
#pragma unroll
  for (int c = 0; c < 6; ++c) r[c] = T(0);
  ug_row<T>(g, shell, true, i, n, d, [&](int off, T w) {
    const long long q = p + off * st;
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c] += w * F[c * np + q];
  });
  ug_row<T>(g, shell, false, i, n, d, [&](int off, T w) {
    T t[6];
    load6<T, CURV>(F, coef, np, p + off * st, d, t);
#pragma unroll
    for (int c = 3; c < 6; ++c) r[c] += w * t[c];
  });
}

// D+ of the three velocities only, along axis d.
template <typename T>
__device__ void diff_v_ug(const T* __restrict__ F, long long np, long long p, int i, int n, long long st, int d,
                          const UpG& g, bool shell, T r[3]) {
  r[0] = r[1] = r[2] = T(0);
  ug_row<T>(g, shell, true, i, n, d, [&](int off, T w) {
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c] += w * F[c * np + p + off * st];
  });
}

// D- of the three fluxes J*metric_j(d)*sigma_{c,j} (the PML split).
template <typename T>
__device__ void diff_pml_flux_ug(const T* __restrict__ F, const T* __restrict__ coef, long long np, long long p,
                                 int i, int n, long long st, int d, int j, const UpG& g, bool shell, T r[3]) {
  r[0] = r[1] = r[2] = T(0);
  ug_row<T>(g, shell, false, i, n, d, [&](int off, T w) {
    const long long q = p + off * st;
    const T a = coef[(d * 3 + j) * np + q];
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c] += w * (a * F[sig(c, j) * np + q]);
  });
}

// Operator dispatch on the compile-time fd of a kernel.
template <typename T, bool CURV, int FD>
__device__ __forceinline__ void diff6_op(const T* __restrict__ F, const T* __restrict__ coef, long long np,
                                         long long p, int i, int n, long long st, int d, T r[6]) {
  if (FD) diff6_up<T, CURV, FD ? FD : 1>(F, coef, np, p, i, n, st, d, r);
  else diff6<T, CURV>(F, coef, np, p, i, n, st, d, r);
}



// ---------------------------------------------------------------------------
// Main stencil kernel (2.5-D tiled).  Computes, for every point of the block,
//   DF <- A*DF + L(F)      and      F_out <- F + B*dt*DF
// (scale_rates + set_rates + update_fields, src/fields.f90:49-171,
// src/JU_xJU_yJU_z6.f90:12-812 and 16141-16449, src/RHS_Interior.f90:133-274),
// with the Kahan-compensated update in FP32C mode.  Boundary penalties, PML
// terms and the plastic return map are applied afterwards by the correction
// kernels below (they are linear in DF, so the order of the sums changes only
// rounding).
//
// A CTA of TQ x TR threads owns a (q,r) tile and marches along s through a
// chunk of planes.  Per plane the tile plus a 3-point halo in q and r is
// staged into shared memory as the differenced quantities -- velocities and
// the q- and r-face momentum fluxes J*metric*sigma -- so each is formed once
// and read by up to 7 neighbours from shared memory.  Along s every thread
// keeps (v, s-face flux) of a 9-plane window in private shared-memory slots,
// enough for the 7-point central rows and for the one-sided closure rows,
// which read planes 0..8 (or n-9..n-1).  The last tile along q and r is
// shifted to end on the last point and owns its whole width, so every
// closure row lies inside one tile plus halo (needs TQ, TR >= 8).
template <typename T, int TQ, int TR>
struct Tile {
  static constexpr int HQ = TQ + 6, HR = TR + 6, NRING = 9;
  static constexpr int sgq_off = 3 * HR * HQ, sgr_off = sgq_off + 3 * TR * HQ, ring_off = sgr_off + 3 * HR * TQ;
  static constexpr size_t words = ring_off + NRING * 6 * TR * TQ;
  __device__ static T& sv(T* b, int c, int lr, int lq) { return b[(c * HR + lr) * HQ + lq]; }
  __device__ static T& sgq(T* b, int c, int ty, int lq) { return b[sgq_off + (c * TR + ty) * HQ + lq]; }
  __device__ static T& sgr(T* b, int c, int lr, int tx) { return b[sgr_off + (c * HR + lr) * TQ + tx]; }
  __device__ static T& ring(T* b, int slot, int c, int ty, int tx) {
    return b[ring_off + ((slot * 6 + c) * TR + ty) * TQ + tx];
  }
};

template <typename T, bool CURV, bool KAHAN, int TQ, int TR, int MINB>
__global__ void __launch_bounds__(TQ * TR, MINB) stencil_kernel_tiled(const __grid_constant__ VolumeArgs<T> a,
                                                                       int schunk) {
  using TL = Tile<T, TQ, TR>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nq = a.nq, nr = a.nr, ns = a.ns;
  const long long np = a.np;
  const long long sts = (long long)a.pq * nr;
  const TileSpan spq = tile_span(blockIdx.x, nq, TQ), spr = tile_span(blockIdx.y, nr, TR);
  const int q0 = spq.origin, r0 = spr.origin;
  const int q = q0 + tx, r = r0 + ty;
  const bool valid = q < nq && r < nr;
  const bool own = valid && q >= spq.own_lo && q < spq.own_hi && r >= spr.own_lo && r < spr.own_hi;
  const int s_begin = blockIdx.z * schunk;
  const int s_end = min(ns, s_begin + schunk);
  const T* __restrict__ F = a.Fin;
  const T* __restrict__ coef = a.coef;
  const int lq = tx + 3, lr = ty + 3;
  const int kq = sbp_kind(q, nq), kr = sbp_kind(r, nr);
  const long long col = q + (long long)a.pq * r;
  int lo = 0, hi = -1;  // planes held by the ring (uniform across the CTA)

  for (int s = s_begin; s < s_end; ++s) {
    const long long p = col + sts * s;
    // ---- ring: make planes [need_lo, need_hi] resident (private slots)
    const int ks = sbp_kind(s, ns);
    const int need_lo = ks < 0 ? 0 : (ks > 0 ? ns - 9 : s - 3);
    const int need_hi = ks < 0 ? 8 : (ks > 0 ? ns - 1 : s + 3);
    if (need_lo < lo || need_lo > hi + 1) {
      lo = need_lo;
      hi = need_lo - 1;
    }
    for (int pl = hi + 1; pl <= need_hi; ++pl) {
      if (valid) {
        T t6[6];
        load6<T, CURV>(F, coef, np, col + sts * pl, 2, t6);
        const int slot = pl % 9;
#pragma unroll
        for (int c = 0; c < 6; ++c) TL::ring(sm, slot, c, ty, tx) = t6[c];
      }
    }
    hi = need_hi;
    lo = max(lo, hi - 8);
    // ---- stage the plane's cross region into shared memory
    __syncthreads();
    auto stage = [&](int gq, int gr, int lq_, int lr_, bool wq, bool wr) {
      const long long pp = gq + (long long)a.pq * gr + sts * s;
      T f[9];
#pragma unroll
      for (int c = 0; c < 9; ++c) f[c] = F[c * np + pp];
#pragma unroll
      for (int c = 0; c < 3; ++c) TL::sv(sm, c, lr_, lq_) = f[c];
      if (wq) {
        if (CURV) {
          const T a0 = coef[0 * np + pp], a1 = coef[1 * np + pp], a2 = coef[2 * np + pp];
#pragma unroll
          for (int c = 0; c < 3; ++c)
            TL::sgq(sm, c, lr_ - 3, lq_) = a0 * f[sig(c, 0)] + a1 * f[sig(c, 1)] + a2 * f[sig(c, 2)];
        } else {
#pragma unroll
          for (int c = 0; c < 3; ++c) TL::sgq(sm, c, lr_ - 3, lq_) = f[sig(c, 0)];
        }
      }
      if (wr) {
        if (CURV) {
          const T a0 = coef[3 * np + pp], a1 = coef[4 * np + pp], a2 = coef[5 * np + pp];
#pragma unroll
          for (int c = 0; c < 3; ++c)
            TL::sgr(sm, c, lr_, lq_ - 3) = a0 * f[sig(c, 0)] + a1 * f[sig(c, 1)] + a2 * f[sig(c, 2)];
        } else {
#pragma unroll
          for (int c = 0; c < 3; ++c) TL::sgr(sm, c, lr_, lq_ - 3) = f[sig(c, 1)];
        }
      }
    };
    if (valid) stage(q, r, lq, lr, true, true);
    if (r < nr) {
      if (tx < 3 && q0 - 3 + tx >= 0) stage(q0 - 3 + tx, r, tx, lr, true, false);
      if (tx >= TQ - 3 && q0 + TQ + (tx - (TQ - 3)) < nq)
        stage(q0 + TQ + (tx - (TQ - 3)), r, TQ + 3 + (tx - (TQ - 3)), lr, true, false);
    }
    if (q < nq) {
      if (ty < 3 && r0 - 3 + ty >= 0) stage(q, r0 - 3 + ty, lq, ty, false, true);
      if (ty >= TR - 3 && r0 + TR + (ty - (TR - 3)) < nr)
        stage(q, r0 + TR + (ty - (TR - 3)), lq, TR + 3 + (ty - (TR - 3)), false, true);
    }
    __syncthreads();
    if (!own) continue;

    // ---- derivatives, consumed axis by axis
    T g[3][3], dv[3];
    const T Jinv = CURV ? coef[9 * np + p] : T(1);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      T o[6];
      const int kind = d == 0 ? kq : (d == 1 ? kr : ks);
      if (kind == 0) {
        const T c1 = T(kC1), c2 = T(kC2), c3 = T(kC3);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          T xp1, xm1, xp2, xm2, xp3, xm3;
          if (d == 0) {
            auto X = [&](int l) -> T { return c < 3 ? TL::sv(sm, c, lr, l) : TL::sgq(sm, c - 3, ty, l); };
            xp1 = X(lq + 1); xm1 = X(lq - 1); xp2 = X(lq + 2); xm2 = X(lq - 2); xp3 = X(lq + 3); xm3 = X(lq - 3);
          } else if (d == 1) {
            auto X = [&](int l) -> T { return c < 3 ? TL::sv(sm, c, l, lq) : TL::sgr(sm, c - 3, l, tx); };
            xp1 = X(lr + 1); xm1 = X(lr - 1); xp2 = X(lr + 2); xm2 = X(lr - 2); xp3 = X(lr + 3); xm3 = X(lr - 3);
          } else {
            xp1 = TL::ring(sm, (s + 1) % 9, c, ty, tx); xm1 = TL::ring(sm, (s + 8) % 9, c, ty, tx);
            xp2 = TL::ring(sm, (s + 2) % 9, c, ty, tx); xm2 = TL::ring(sm, (s + 7) % 9, c, ty, tx);
            xp3 = TL::ring(sm, (s + 3) % 9, c, ty, tx); xm3 = TL::ring(sm, (s + 6) % 9, c, ty, tx);
          }
          o[c] = c1 * (xp1 - xm1) + c2 * (xp2 - xm2) + c3 * (xp3 - xm3);
        }
      } else {
#pragma unroll
        for (int c = 0; c < 6; ++c) o[c] = T(0);
#pragma unroll 1
        for (int t = 0; t < 9; ++t) {
          T w;
          int off;
          row_entry<T>(kind, t, w, off);
#pragma unroll
          for (int c = 0; c < 6; ++c) {
            T x;
            if (d == 0) x = c < 3 ? TL::sv(sm, c, lr, lq + off) : TL::sgq(sm, c - 3, ty, lq + off);
            else if (d == 1) x = c < 3 ? TL::sv(sm, c, lr + off, lq) : TL::sgr(sm, c - 3, lr + off, tx);
            else x = TL::ring(sm, (s + off + 18) % 9, c, ty, tx);
            o[c] += w * x;
          }
        }
      }
      const T rh = a.rh[d];
      if (CURV) {
        T m[3];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) m[jj] = coef[(d * 3 + jj) * np + p] * Jinv;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          dv[c] = d == 0 ? rh * o[3 + c] : dv[c] + rh * o[3 + c];
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) g[c][jj] = d == 0 ? m[jj] * (rh * o[c]) : g[c][jj] + m[jj] * (rh * o[c]);
        }
      } else {
        const T sc = a.cart_metric[d] * rh;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          dv[c] = d == 0 ? sc * o[3 + c] : dv[c] + sc * o[3 + c];
          g[c][d] = sc * o[c];
        }
      }
    }
    T lam, mu, rinv;
    if (CURV) {
      lam = coef[10 * np + p];
      mu = coef[11 * np + p];
      rinv = coef[12 * np + p];
    } else {
      lam = coef[0 * np + p];
      mu = coef[1 * np + p];
      rinv = coef[2 * np + p];
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
#pragma unroll
    for (int c = 0; c < 9; ++c) {
      const T f0 = F[c * np + p];
      const T df = a.A * a.DF[c * np + p] + du[c];
      a.DF[c * np + p] = df;
      if (KAHAN) {
        const T y = a.Bdt * df - (T)comp_get(a.C, c * np + p);
        const T t = f0 + y;
        comp_put(a.C, c * np + p, (float)((t - f0) - y));
        a.Fout[c * np + p] = t;
      } else {
        a.Fout[c * np + p] = f0 + a.Bdt * df;
      }
    }
  }
}

// Per-point form of the same stencil kernel: every neighbour value is read
// through L1/L2 (kept for cross-checks of the tiled kernel).
// smode 1 restricts it to the 12 s-boundary planes (grid z = 12), the part
// the TMA kernel leaves out.
template <typename T, bool CURV, bool KAHAN, int FD = 0>
__global__ void __launch_bounds__(256) stencil_kernel_pointwise(const __grid_constant__ VolumeArgs<T> a, int smode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = smode ? (blockIdx.z < 6 ? (int)blockIdx.z : a.ns - 12 + (int)blockIdx.z) : (int)blockIdx.z;
  if (i >= a.nq || j >= a.nr) return;
  const long long np = a.np;
  const long long p = i + (long long)a.pq * (j + (long long)a.nr * k);
  T g[3][3], dv[3];
  const T Jinv = CURV ? a.coef[9 * np + p] : T(1);
  const int idx[3] = {i, j, k}, nn[3] = {a.nq, a.nr, a.ns};
  const long long st[3] = {1, a.pq, (long long)a.pq * a.nr};
#pragma unroll
  const bool shell = FD == 3 && ug_shell(a, idx, nn);
  for (int d = 0; d < 3; ++d) {
    T o[6];
    if (FD == 3) diff6_ug<T, CURV>(a.Fin, a.coef, np, p, idx[d], nn[d], st[d], d, a.ug, shell, o);
    else diff6_op<T, CURV, FD == 3 ? 0 : FD>(a.Fin, a.coef, np, p, idx[d], nn[d], st[d], d, o);
    const T rh = a.rh[d];
    if (CURV) {
      T m[3];
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) m[jj] = a.coef[(d * 3 + jj) * np + p] * Jinv;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        dv[c] = d == 0 ? rh * o[3 + c] : dv[c] + rh * o[3 + c];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) g[c][jj] = d == 0 ? m[jj] * (rh * o[c]) : g[c][jj] + m[jj] * (rh * o[c]);
      }
    } else {
      const T sc = a.cart_metric[d] * rh;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        dv[c] = d == 0 ? sc * o[3 + c] : dv[c] + sc * o[3 + c];
        g[c][d] = sc * o[c];
      }
    }
  }
  const T* coef = a.coef;
  const T lam = CURV ? coef[10 * np + p] : coef[0 * np + p];
  const T mu = CURV ? coef[11 * np + p] : coef[1 * np + p];
  const T rinv = CURV ? coef[12 * np + p] : coef[2 * np + p];
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
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    const T f0 = a.Fin[c * np + p];
    const T df = a.A * a.DF[c * np + p] + du[c];
    a.DF[c * np + p] = df;
    if (KAHAN) {
      const T y = a.Bdt * df - (T)comp_get(a.C, c * np + p);
      const T t = f0 + y;
      comp_put(a.C, c * np + p, (float)((t - f0) - y));
      a.Fout[c * np + p] = t;
    } else {
      a.Fout[c * np + p] = f0 + a.Bdt * df;
    }
  }
}

// ---------------------------------------------------------------------------
// PML kernel (src/RHS_Interior.f90:1782-2201, src/fields.f90:70-105,131-166):
// for every point inside one or more active slabs, the damping terms of the
// rates, DQ <- A*DQ + sources - (d+cfs)*Q (plus the face penalty on the
// slab's own boundary, src/RHS_Interior.f90:1560-1700) and Q <- Q + B*dt*DQ.
// One thread per point of the block; points outside every slab exit.
// The PML slab union of a block as up to six disjoint boxes: the q slabs
// over the whole (r, s) extent, the r slabs between them, the s slabs inside
// both; start[b] is the number of points in boxes before b.
struct PmlBoxes {
  int n;
  int lo[6][3], dim[6][3];
  long long start[7];
};

template <typename T>
PmlBoxes pml_boxes(const VolumeArgs<T>& a) {
  PmlBoxes B;
  B.n = 0;
  B.start[0] = 0;
  const int nq = a.nq, nr = a.nr, ns = a.ns, w = a.npml;
  const int qlo = a.pml[0] ? w : 0, qhi = a.pml[1] ? nq - w : nq;
  const int rlo = a.pml[2] ? w : 0, rhi = a.pml[3] ? nr - w : nr;
  const int slo = a.pml[4] ? w : 0, shi = a.pml[5] ? ns - w : ns;
  auto add = [&](int q0, int q1, int r0, int r1, int s0, int s1) {
    if (q1 <= q0 || r1 <= r0 || s1 <= s0) return;
    const int b = B.n++;
    B.lo[b][0] = q0; B.lo[b][1] = r0; B.lo[b][2] = s0;
    B.dim[b][0] = q1 - q0; B.dim[b][1] = r1 - r0; B.dim[b][2] = s1 - s0;
    B.start[b + 1] = B.start[b] + (long long)(q1 - q0) * (r1 - r0) * (s1 - s0);
  };
  add(0, qlo, 0, nr, 0, ns);
  add(qhi, nq, 0, nr, 0, ns);
  add(qlo, qhi, 0, rlo, 0, ns);
  add(qlo, qhi, rhi, nr, 0, ns);
  add(qlo, qhi, rlo, rhi, 0, slo);
  add(qlo, qhi, rlo, rhi, shi, ns);
  for (int b = B.n; b < 6; ++b) B.start[b + 1] = B.start[b];
  return B;
}

// FP32 fields: capped at 80 registers for three CTAs per SM (24 warps to
// hide the latency of its dependent loads; measured 0.39 -> 0.31 ms per
// correction launch on config 2 despite some spilling).
template <typename T, bool CURV, bool KAHAN, int FD>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) pml_kernel(const __grid_constant__ VolumeArgs<T> a,
                                                                           const __grid_constant__ PmlBoxes bx) {
  // one thread per point of the slab union, enumerated box by box (q
  // fastest within a box)
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int b = 0;
  while (b < bx.n && t >= bx.start[b + 1]) ++b;
  if (b >= bx.n) return;
  const long long l = t - bx.start[b];
  const int i = bx.lo[b][0] + (int)(l % bx.dim[b][0]);
  const int j = bx.lo[b][1] + (int)((l / bx.dim[b][0]) % bx.dim[b][1]);
  const int k = bx.lo[b][2] + (int)(l / ((long long)bx.dim[b][0] * bx.dim[b][1]));
  const int nq = a.nq, nr = a.nr, ns = a.ns, npml = a.npml;
  const int idx[3] = {i, j, k}, nn[3] = {nq, nr, ns};
  bool any = false;
#pragma unroll
  for (int side = 0; side < 6; ++side) {
    const int ax = side >> 1;
    if (a.pml[side] && ((side & 1) ? idx[ax] >= nn[ax] - npml : idx[ax] < npml)) any = true;
  }
  if (!any) return;
  const long long np = a.np;
  const long long p = i + (long long)a.pq * (j + (long long)nr * k);
  const long long st[3] = {1, a.pq, (long long)a.pq * nr};
  const T* __restrict__ F = a.Fin;
  const T* __restrict__ coef = a.coef;
  const bool shell = FD == 3 && ug_shell(a, idx, nn);
  // velocity gradient at the point: from the TMA stencil of this stage
  // (a.G), else formed here
  T g[3][3];
  const T Jinv = CURV ? coef[9 * np + p] : T(1);
  const bool have_g = a.G != nullptr;
  if (have_g) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) g[c][jj] = a.G[(c * 3 + jj) * np + p];
  }
  // every loop over axes and sides is unrolled so that the per-axis index,
  // extent and stride are compile-time selections (no local-memory arrays)
  if (!have_g) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      T o[3];
      if (FD == 3) diff_v_ug<T>(F, np, p, idx[d], nn[d], st[d], d, a.ug, shell, o);
      else if (FD) diff_v_up<T, FD == 3 ? 1 : (FD ? FD : 1)>(F, np, p, idx[d], nn[d], st[d], d, o);
      else diff_v<T>(F, np, p, idx[d], nn[d], st[d], o);
      const T rh = a.rh[d];
      for (int c = 0; c < 3; ++c) {
        if (CURV) {
          for (int jj = 0; jj < 3; ++jj) {
            const T m = coef[(d * 3 + jj) * np + p] * Jinv;
            g[c][jj] = d == 0 ? m * (rh * o[c]) : g[c][jj] + m * (rh * o[c]);
          }
        } else {
          g[c][d] = a.cart_metric[d] * rh * o[c];
        }
      }
    }
  }
  const T lam = CURV ? coef[10 * np + p] : coef[0 * np + p];
  const T mu = CURV ? coef[11 * np + p] : coef[1 * np + p];
  const T rinv = CURV ? coef[12 * np + p] : coef[2 * np + p];
  const T rhoinv = CURV ? rinv / Jinv : rinv;
  const T l2m = lam + T(2) * mu;
  const double d0 = a.pml_d0;  // 6/(2*1) * ln(1/1e-3), src/RHS_Interior.f90:1815
  const T cfs = T(1);
  T corr[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) corr[c] = T(0);
  // reference order of the layers: s-low, s-high, r-low, r-high, q-low, q-high
#pragma unroll
  for (int oi = 0; oi < 6; ++oi) {
    const int side = oi < 2 ? 4 + oi : (oi < 4 ? oi : oi - 4);
    if (!a.pml[side]) continue;
    const int axis = side >> 1;
    const bool hi = side & 1;
    const int ii = idx[axis], n = nn[axis];
    if (!(hi ? (ii >= n - npml) : (ii < npml))) continue;
    // damping profile in grid-index units (src/RHS_Interior.f90:1855,1973,2092),
    // in the field precision
    const int off = hi ? ii + 1 - (n - npml) : (axis == 2 ? ii + 1 - npml : ii - npml);
    const T damp = (T)d0 * (fabs((T)off / (T)npml));
    long long sp;
    if (axis == 0) sp = (hi ? ii - (n - npml) : ii) + (long long)npml * (j + (long long)nr * k);
    else if (axis == 1) sp = i + (long long)nq * ((hi ? ii - (n - npml) : ii) + (long long)npml * k);
    else sp = i + (long long)nq * (j + (long long)nr * (hi ? ii - (n - npml) : ii));
    const long long snp = a.slab_np[side];
    T* __restrict__ Q = a.Q[side];
    T* __restrict__ DQ = a.DQ[side];
    T qv[9];
    for (int c = 0; c < 9; ++c) qv[c] = Q[c * snp + sp];
    // per-axis split of the stress divergence along physical axis `axis`
    T sd[3];
    if (CURV) {
      T acc3[3] = {T(0), T(0), T(0)};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        T r3[3];
        if (FD == 3) diff_pml_flux_ug<T>(F, coef, np, p, idx[d], nn[d], st[d], d, axis, a.ug, shell, r3);
        else if (FD) diff_pml_flux_up<T, FD == 3 ? 1 : (FD ? FD : 1)>(F, coef, np, p, idx[d], nn[d], st[d], d, axis, r3);
        else diff_pml_flux<T>(F, coef, np, p, idx[d], nn[d], st[d], d, axis, r3);
        for (int c = 0; c < 3; ++c) acc3[c] += a.rh[d] * r3[c];
      }
      for (int c = 0; c < 3; ++c) sd[c] = acc3[c] * Jinv;
    } else {
      T o[6];
      if (FD == 3) diff6_ug<T, false>(F, coef, np, p, idx[axis], nn[axis], st[axis], axis, a.ug, shell, o);
      else diff6_op<T, false, FD == 3 ? 0 : FD>(F, coef, np, p, idx[axis], nn[axis], st[axis], axis, o);
      for (int c = 0; c < 3; ++c) sd[c] = a.cart_metric[axis] * a.rh[axis] * o[3 + c];
    }
    corr[0] -= damp * qv[0] * rhoinv;
    corr[1] -= damp * qv[1] * rhoinv;
    corr[2] -= damp * qv[2] * rhoinv;
    corr[3] -= damp * (l2m * qv[3] + lam * qv[4] + lam * qv[5]);
    corr[4] -= damp * (lam * qv[3] + l2m * qv[4] + lam * qv[5]);
    corr[5] -= damp * (lam * qv[3] + lam * qv[4] + l2m * qv[5]);
    corr[6] -= mu * damp * qv[6];
    corr[7] -= mu * damp * qv[7];
    corr[8] -= mu * damp * qv[8];
    T src[9];
    for (int c = 0; c < 9; ++c) src[c] = T(0);
    src[0] = sd[0];
    src[1] = sd[1];
    src[2] = sd[2];
    // velocity-gradient sources (src/RHS_Interior.f90:1890-1907, 2008-2025, 2125-2142)
    if (axis == 0) { src[3] = g[0][0]; src[6] = g[1][0]; src[7] = g[2][0]; }
    else if (axis == 1) { src[4] = g[1][1]; src[6] = g[0][1]; src[8] = g[2][1]; }
    else { src[5] = g[2][2]; src[7] = g[0][2]; src[8] = g[1][2]; }
    T dq[9];
    for (int c = 0; c < 9; ++c) dq[c] = a.A * DQ[c * snp + sp] + src[c] - (damp + cfs) * qv[c];
    const bool on_face = hi ? (ii == n - 1) : (ii == 0);
    if (on_face && a.bc[side] >= 1 && a.bc[side] <= 3) {
      T u[9], sat[9], ubc[9];
      for (int c = 0; c < 9; ++c) u[c] = F[c * np + p];
      const int na = axis == 0 ? nr : nq;
      const long long f = axis == 0 ? (j + (long long)nr * k) : (axis == 1 ? (i + (long long)nq * k) : (i + (long long)nq * j));
      const long long nf = (long long)na * (axis == 2 ? nr : ns);
      boundary_sat(u, a.face[side], nf, f, a.bc[side], hi, a.bc_form, sat, ubc);
      for (int c = 0; c < 9; ++c) dq[c] -= a.tau_h[axis] * (T)ubc[c];
    }
    for (int c = 0; c < 9; ++c) {
      DQ[c * snp + sp] = dq[c];
      Q[c * snp + sp] = qv[c] + a.Bdt * dq[c];
    }
  }
  add_correction<T, KAHAN>(a, p, corr);
}

// ---------------------------------------------------------------------------
// three CTAs per SM: 80 registers, no spills (four would cap it at 64 and
// spill)
#ifndef WQL_ANEL_MINB
#define WQL_ANEL_MINB 3
#endif
// Anelastic kernel (response = 'anelastic'; src/RHS_Interior.f90:2390-2509,
// the interior terms of src/JU_xJU_yJU_z6.f90:16316-16346, src/fields.f90:
// 61-68 and 122-129), one thread per point: the stress rates lose the sum
// of the point's four memory variables, each memory variable's rate is
//   Deta <- A*Deta + (relaxed strain-rate forcing - eta) / tau
// and eta <- eta + B*dt*Deta.  Inside a PML slab the strain rates lose the
// damped auxiliary fields (pml_damping_and_q, src/RHS_Interior.f90:
// 2287-2387), so this kernel runs before the PML kernel advances Q.  The
// velocity gradient comes from the TMA stencil (FP32C) or is formed here
// with the block's operator.
template <typename T, bool CURV, bool KAHAN, int FD>
__global__ void __launch_bounds__(256, WQL_ANEL_MINB) anelastic_kernel(const __grid_constant__ VolumeArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  const int nq = a.nq, nr = a.nr, ns = a.ns, npml = a.npml;
  if (i >= nq || j >= nr) return;
  const long long np = a.np;
  const long long p = i + (long long)a.pq * (j + (long long)nr * k);
  const int idx[3] = {i, j, k}, nn[3] = {nq, nr, ns};
  const long long st[3] = {1, a.pq, (long long)a.pq * nr};
  const T* __restrict__ F = a.Fin;
  const T* __restrict__ coef = a.coef;
  const T Jinv = CURV ? coef[9 * np + p] : T(1);
  T g[3][3];
  // the velocity gradient: from the TMA stencil of this stage (a.G), else
  // formed here
  if (a.G != nullptr) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) g[c][jj] = a.G[(c * 3 + jj) * np + p];
  }
  if (a.G == nullptr) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      T o[3];
      if (FD == 3) diff_v_ug<T>(F, np, p, idx[d], nn[d], st[d], d, a.ug, ug_shell(a, idx, nn), o);
      else if (FD) diff_v_up<T, FD == 3 ? 1 : (FD ? FD : 1)>(F, np, p, idx[d], nn[d], st[d], d, o);
      else diff_v<T>(F, np, p, idx[d], nn[d], st[d], o);
      const T rh = a.rh[d];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (CURV) {
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) {
            const T m = coef[(d * 3 + jj) * np + p] * Jinv;
            g[c][jj] = d == 0 ? m * (rh * o[c]) : g[c][jj] + m * (rh * o[c]);
          }
        } else {
          g[c][d] = a.cart_metric[d] * rh * o[c];
        }
      }
    }
  }
  // strain rates: exx, eyy, ezz, gxy, gxz, gyz and the trace
  T e[6];
  e[0] = g[0][0];
  e[1] = g[1][1];
  e[2] = g[2][2];
  e[3] = g[0][1] + g[1][0];
  e[4] = g[0][2] + g[2][0];
  e[5] = g[1][2] + g[2][1];
  bool in_pml = false;
#pragma unroll
  for (int side = 0; side < 6; ++side) {
    const int ax = side >> 1;
    if (a.pml[side] && ((side & 1) ? idx[ax] >= nn[ax] - npml : idx[ax] < npml)) in_pml = true;
  }
  if (in_pml) {
    // d * Q terms per axis (damping profile and slab indexing as the PML kernel)
    T dq[3][3] = {{T(0), T(0), T(0)}, {T(0), T(0), T(0)}, {T(0), T(0), T(0)}};
#pragma unroll
    for (int side = 0; side < 6; ++side) {
      if (!a.pml[side]) continue;
      const int axis = side >> 1;
      const bool hi = side & 1;
      const int ii = idx[axis], n = nn[axis];
      if (!(hi ? (ii >= n - npml) : (ii < npml))) continue;
      const int off = hi ? ii + 1 - (n - npml) : (axis == 2 ? ii + 1 - npml : ii - npml);
      const T damp = (T)a.pml_d0 * (fabs((T)off / (T)npml));
      long long sp;
      if (axis == 0) sp = (hi ? ii - (n - npml) : ii) + (long long)npml * (j + (long long)nr * k);
      else if (axis == 1) sp = i + (long long)nq * ((hi ? ii - (n - npml) : ii) + (long long)npml * k);
      else sp = i + (long long)nq * (j + (long long)nr * (hi ? ii - (n - npml) : ii));
      const long long snp = a.slab_np[side];
      const T* Q = a.Q[side];
      // Q components of the normal strain and the two shear strains of this axis
      const int cn = 3 + axis;
      const int c1 = axis == 0 ? 6 : (axis == 1 ? 6 : 7);
      const int c2 = axis == 0 ? 7 : 8;
      dq[axis][0] = damp * Q[cn * snp + sp];
      dq[axis][1] = damp * Q[c1 * snp + sp];
      dq[axis][2] = damp * Q[c2 * snp + sp];
    }
    e[0] = e[0] - dq[0][0];
    e[1] = e[1] - dq[1][0];
    e[2] = e[2] - dq[2][0];
    e[3] = e[3] - dq[0][1] - dq[1][1];  // gxy: Qx(7), Qy(7)
    e[4] = e[4] - dq[0][2] - dq[2][1];  // gxz: Qx(8), Qz(8)
    e[5] = e[5] - dq[1][2] - dq[2][2];  // gyz: Qy(9), Qz(9)
  }
  const T tr = e[0] + e[1] + e[2];
  const T lam = CURV ? coef[10 * np + p] : coef[0 * np + p];
  const T mu = CURV ? coef[11 * np + p] : coef[1 * np + p];
  const T qs = a.qsinv[p];
  const T qp = T(0.5) * qs;
  T corr[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) corr[c] = T(0);
  // the memory-variable streams do not overlap (restrict): a component's
  // loads need not wait for the previous component's stores
  T* __restrict__ eta = a.eta;
  T* __restrict__ deta = a.Deta;
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    T ev[1][4], dv[1][4];  // this component's four mechanisms
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      ev[0][m] = eta[(c * 4 + m) * np + p];
      dv[0][m] = deta[(c * 4 + m) * np + p];
    }
    corr[3 + c] = -(ev[0][0] + ev[0][1] + ev[0][2] + ev[0][3]);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const T w = (T)a.an_w[m];
      const T force = c < 3 ? (w * T(2) * mu * qs) * e[c] + (w * ((lam + T(2) * mu) * qp - T(2) * mu * qs)) * tr
                            : w * mu * qs * e[c];
      const long long q = (c * 4 + m) * np + p;
      const T de = a.A * dv[0][m] + (force - ev[0][m]) / (T)a.an_tau[m];
      deta[q] = de;
      eta[q] = ev[0][m] + a.Bdt * de;
    }
  }
  add_correction<T, KAHAN>(a, p, corr);
}

// ---------------------------------------------------------------------------
// With a manufactured solution the boundary penalty acts on the fields less
// the exact solution at the stage's time (u = F - switch*fu,
// src/BoundaryConditions.f90:86-92, 126).
template <typename T>
__device__ __forceinline__ void mms_deviation(const VolumeArgs<T>& a, long long p, T (&u)[9]) {
  if (!a.ms) return;
  const T sv = a.mms_T * a.ms[p], ss = a.mms_T * a.ms[a.np + p];
#pragma unroll
  for (int c = 0; c < 9; ++c) u[c] -= c < 3 ? sv : ss;
}

// Manufactured-solution forcing (mms_forcing, src/mms.f90:77-133, which the
// reference never calls): DF -= T(t) mp - T'(t) S at every point of the
// block, with the matching update of F_out.
template <typename T, bool KAHAN>
__global__ void __launch_bounds__(256) mms_kernel(const __grid_constant__ VolumeArgs<T> a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= a.nq || j >= a.nr) return;
  const long long np = a.np;
  const long long p = i + (long long)a.pq * (j + (long long)a.nr * k);
  const T sv = a.ms[p], ss = a.ms[np + p];
  T corr[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) corr[c] = -(a.mms_T * a.mp[c * np + p] - a.mms_Tp * (c < 3 ? sv : ss));
  add_correction<T, KAHAN>(a, p, corr);
}

// ---------------------------------------------------------------------------
// Face kernel: outer-boundary SAT (src/RHS_Interior.f90:1516-1703 with
// src/BoundaryConditions.f90:777-918 + structure(), or the weighted form of
// src/BoundaryConditions3.f90:777-903) and the fault SAT computed by the
// interface kernel (src/RHS_Interior.f90:1757-1772).  One thread per face
// point; a point on several faces is handled once, by its lowest side.
template <typename T, bool KAHAN>
__global__ void __launch_bounds__(256) face_kernel(const __grid_constant__ VolumeArgs<T> a) {
  const int nq = a.nq, nr = a.nr, ns = a.ns;
  const long long nfs[6] = {(long long)nr * ns, (long long)nr * ns, (long long)nq * ns, (long long)nq * ns,
                            (long long)nq * nr, (long long)nq * nr};
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int side = 0;
  while (side < 6 && t >= nfs[side]) {
    t -= nfs[side];
    ++side;
  }
  if (side >= 6) return;
  const int axis = side >> 1;
  int i, j, k;
  if (axis == 0) { i = (side & 1) ? nq - 1 : 0; j = (int)(t % nr); k = (int)(t / nr); }
  else if (axis == 1) { i = (int)(t % nq); j = (side & 1) ? nr - 1 : 0; k = (int)(t / nq); }
  else { i = (int)(t % nq); j = (int)(t / nq); k = (side & 1) ? ns - 1 : 0; }
  const int idx[3] = {i, j, k}, nn[3] = {nq, nr, ns};
  // owner: the lowest side containing the point
  for (int s2 = 0; s2 < side; ++s2) {
    const int ax2 = s2 >> 1;
    if (idx[ax2] == ((s2 & 1) ? nn[ax2] - 1 : 0)) return;
  }
  const long long np = a.np;
  const long long p = i + (long long)a.pq * (j + (long long)nr * k);
  T u[9], tot[9], corr[9];
  for (int c = 0; c < 9; ++c) u[c] = a.Fin[c * np + p];
  mms_deviation(a, p, u);
  const bool any = face_penalty(a, i, j, k, u, tot);
  for (int c = 0; c < 9; ++c) corr[c] = -tot[c];
  if (any) add_correction<T, KAHAN>(a, p, corr);
}

// ---------------------------------------------------------------------------
// Face pre-kernel (for the stencil variant without a face pass): the
// boundary and fault penalty tot of each face point (face_penalty, as in the
// face kernel) folded into the rates before the stencil kernel runs,
// DF <- DF - tot/A, or DF <- -tot on a stage with A = 0, so that the
// stencil's A*DF + du (or DF + du on face points when A = 0) carries it.
// One thread per face point, a point on several faces taken by its lowest
// side.
template <typename T>
__device__ __forceinline__ void face_pre_point(const VolumeArgs<T>& a, long long t) {
  const int nq = a.nq, nr = a.nr, ns = a.ns;
  const long long nfs[6] = {(long long)nr * ns, (long long)nr * ns, (long long)nq * ns, (long long)nq * ns,
                            (long long)nq * nr, (long long)nq * nr};
  int side = 0;
  while (side < 6 && t >= nfs[side]) {
    t -= nfs[side];
    ++side;
  }
  if (side >= 6) return;
  const int axis = side >> 1;
  const int w = axis == 0 ? nr : nq;
  const int c1 = (int)(t % w), c2 = (int)(t / w);
  int i, j, k;
  if (axis == 0) { i = (side & 1) ? nq - 1 : 0; j = c1; k = c2; }
  else if (axis == 1) { i = c1; j = (side & 1) ? nr - 1 : 0; k = c2; }
  else { i = c1; j = c2; k = (side & 1) ? ns - 1 : 0; }
  for (int s2 = 0; s2 < side; ++s2) {
    const int ax2 = s2 >> 1;
    const int ii = ax2 == 0 ? i : (ax2 == 1 ? j : k), n2 = ax2 == 0 ? nq : (ax2 == 1 ? nr : ns);
    if (ii == ((s2 & 1) ? n2 - 1 : 0)) return;
  }
  const long long np = a.np;
  const long long p = i + (long long)a.pq * (j + (long long)nr * k);
  T u[9], tot[9], df[9];
  // the rates are read together with the fields (not after the penalty is
  // formed), so the two loads' latencies overlap; a stage with A = 0
  // overwrites them without reading
  const bool keep = a.A != T(0);
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    u[c] = a.Fin[c * np + p];
    df[c] = keep ? a.DF[c * np + p] : T(0);
  }
  mms_deviation(a, p, u);
  if (!face_penalty(a, i, j, k, u, tot)) return;
#pragma unroll
  for (int c = 0; c < 9; ++c) a.DF[c * np + p] = keep ? df[c] - tot[c] / a.A : -tot[c];
}

template <typename T>
__global__ void __launch_bounds__(256) face_pre_kernel(const __grid_constant__ VolumeArgs<T> a) {
  face_pre_point(a, blockIdx.x * (long long)blockDim.x + threadIdx.x);
}

// Both blocks of a scenario in one launch: threads [0, n0) take block 0's
// face points, the rest block 1's (one launch of about twice the threads
// hides the latency of these sub-wave launches better than two).
template <typename T>
struct FacePair {
  VolumeArgs<T> a[2];
  long long n0;
};

template <typename T>
__global__ void __launch_bounds__(256) face_pre_kernel2(const __grid_constant__ FacePair<T> P) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < P.n0) face_pre_point(P.a[0], t);
  else face_pre_point(P.a[1], t - P.n0);
}

// ---------------------------------------------------------------------------
// Moment-tensor point source (set_moment_tensor / set_moment_tensor_smooth,
// src/moment_tensor.f90:1014-1078, 1400-1475): DF(4:9) -= (A(t) M) * delta
// on the source's box of points, with the matching update of F_out.
struct SourceArgs {
  int lo[3], dim[3];
  const double* delta;
  double am[6];
};

template <typename T, bool KAHAN>
__global__ void __launch_bounds__(256) source_kernel(const __grid_constant__ VolumeArgs<T> a,
                                                     const __grid_constant__ SourceArgs s) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n = (long long)s.dim[0] * s.dim[1] * s.dim[2];
  if (e >= n) return;
  const int i = s.lo[0] + (int)(e % s.dim[0]);
  const int j = s.lo[1] + (int)((e / s.dim[0]) % s.dim[1]);
  const int k = s.lo[2] + (int)(e / ((long long)s.dim[0] * s.dim[1]));
  const long long p = i + (long long)a.pq * (j + (long long)a.nr * k);
  const double d = s.delta[e];
  T corr[9];
#pragma unroll
  for (int c = 0; c < 3; ++c) corr[c] = T(0);
#pragma unroll
  for (int c = 0; c < 6; ++c) corr[3 + c] = (T)(-(s.am[c] * d));
  add_correction<T, KAHAN>(a, p, corr);
}

// ---------------------------------------------------------------------------
// Plastic return map after the last stage (update_fields_plastic,
// src/plastic.f90:11-151: plastic_flow2 :153-217 for plastic_model 'scec',
// plastic_flow :220-290 otherwise), on points outside the PML slabs,
// applied to the updated stresses.
// The grid covers the box outside the slabs, [lo, hi) per axis; the
// uniform constants come in the field type (pc: c cos(atan nu), sin(atan nu),
// exp(-dt/Tv); s0: the uniform initial stress), so no thread converts from
// FP64.
template <typename T>
struct PlasticBox {
  int lo[3], hi[3];
  T pc[3];
  T s0[6];
};

template <typename T, bool CURV, bool KAHAN>
__global__ void __launch_bounds__(256) plastic_kernel(const __grid_constant__ VolumeArgs<T> a,
                                                      const __grid_constant__ PlasticBox<T> box) {
  const int i = box.lo[0] + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = box.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = box.lo[2] + blockIdx.z;
  if (i >= box.hi[0] || j >= box.hi[1]) return;
  const long long np = a.np;
  const long long p = i + (long long)a.pq * (j + (long long)a.nr * k);
  T s0[6];
  if (!initial_stress_y<T>(a.preset, a.ycoord[p], s0))
    for (int c = 0; c < 6; ++c) s0[c] = box.s0[c];
  T sa[6];
  for (int c = 0; c < 6; ++c) sa[c] = a.Fout[(3 + c) * np + p] + s0[c];
  const T sigma = (sa[0] + sa[1] + sa[2]) / T(3);
  const T J2 = ((sa[0] - sa[1]) * (sa[0] - sa[1]) + (sa[1] - sa[2]) * (sa[1] - sa[2]) +
                (sa[2] - sa[0]) * (sa[2] - sa[0])) / T(6) +
               sa[3] * sa[3] + sa[4] * sa[4] + sa[5] * sa[5];
  const T tau = sqrt(J2);
  if (a.pl_flow) {
    // plastic_flow (src/plastic.f90:220-290): yield function Y = tau + mu*sigma;
    // above it the closed-form solution of eta*lambda = Y(s) for the plastic
    // strain rate, with shear modulus G and bulk modulus K of the point
    const T mu = (T)a.pl_mu, beta = (T)a.pl_beta, eta = (T)a.pl_eta, dt = (T)a.dt;
    const T Y = tau + mu * sigma;
    if (Y <= T(0)) {
      a.pl_lambda[p] = T(0);
      return;
    }
    const T* coef = a.coef;
    const T G = CURV ? coef[11 * np + p] : coef[1 * np + p];
    const T K = (CURV ? coef[10 * np + p] : coef[0 * np + p]) + T(2.0 / 3.0) * G;
    T sd[6];
    for (int c = 0; c < 6; ++c) sd[c] = sa[c] - sigma * (c < 3 ? T(1) : T(0));
    const T lambda = (tau + mu * sigma) / (eta + dt * (G + mu * beta * K));
    a.pl_lambda[p] = lambda;
    a.pl_gammap[p] = a.pl_gammap[p] + dt * lambda;
    const T tau1 = tau - dt * lambda * G;
    const T sigma1 = sigma - dt * lambda * beta * K;
    for (int c = 0; c < 6; ++c) {
      const T sdc = sd[c] * tau1 / (tau1 + dt * lambda * G);
      a.Fout[(3 + c) * np + p] = (sigma1 * (c < 3 ? T(1) : T(0)) + sdc) - s0[c];
      if (KAHAN) a.C[(3 + c) * np + p] = 0;  // bfloat16 zero
    }
    return;
  }
  // c cos(atan nu), sin(atan nu) and exp(-dt/Tv) are uniform: set on the host
  const T Ys = fmax(T(0), box.pc[0] - sigma * box.pc[1]);
  if (!(tau - Ys > T(0))) return;
  const T e = box.pc[2];
  const T rr = e + (T(1) - e) * Ys / tau;
  for (int c = 0; c < 6; ++c) {
    const T dlt = c < 3 ? T(1) : T(0);
    const T sd = sa[c] - sigma * dlt;
    a.Fout[(3 + c) * np + p] = (sigma * dlt + rr * sd) - s0[c];
    if (KAHAN) a.C[(3 + c) * np + p] = 0;  // bfloat16 zero
  }
}

}  // namespace

template <typename T, bool CURV, bool KAHAN, int TQ, int TR, int MINB>
void launch_tiled(const VolumeArgs<T>& a, cudaStream_t s) {
  const size_t smem = sizeof(T) * Tile<T, TQ, TR>::words;
  auto kern = stencil_kernel_tiled<T, CURV, KAHAN, TQ, TR, MINB>;
  static bool attr_done = false;
  if (!attr_done) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr_done = true;
  }
  const int schunk = a.schunk > 0 ? a.schunk : 16;
  dim3 blk(TQ, TR, 1), grd((a.nq + TQ - 1) / TQ, (a.nr + TR - 1) / TR, (a.ns + schunk - 1) / schunk);
  kern<<<grd, blk, smem, s>>>(a, schunk);
}

// Stencil-kernel variants (the tuning table): 1 per-point, 2 tiled 32x8 at
// 1 CTA/SM, 3 tiled 32x8 at 3 CTAs/SM in FP32, 4 tiled 64x8 at 1 CTA/SM,
// 5 TMA-pipelined (FP32), 6 accepted as 5; 0 picks the
// fastest measured on a 2 x 201^3 curvilinear block pair (TMA in FP32,
// tiled 32x8 in FP64).
//
// A tiled axis of n points with tiles of T keeps every closure row inside
// the tile that owns it plus a 3-point halo unless the shifted last tile
// starts at 4 or 5 (then it would own left closure rows whose stencil
// reaches point 0 from outside the halo); such sizes run per point.
// With the upwind pair (halo 4, closure rows reading points 0..9) only a
// last tile starting at 5 is excluded.
inline bool tiles_ok(int n, int T) { return n <= T + 3 || n >= T + 6; }
inline bool tiles_ok_up(int n, int T) { return n <= T + 4 || n >= T + 6; }

template <typename T>
int effective_variant(const VolumeArgs<T>& a) {
  constexpr bool f32 = sizeof(T) == 4;
  int v = a.kernel != 0 ? a.kernel : (f32 ? 5 : 2);
  if ((v == 5 || v == 6) && !f32) v = 2;
  if (a.fd) {
    // the order-6 upwind pair: the TMA kernel (compensated FP32) or per
    // point; order 5 per point
    if (a.fd != 1 || !(v == 5 || v == 6) || a.C == nullptr || !tiles_ok_up(a.nr, kTmaTR)) v = 1;
    return v;
  }
  if ((v == 5 || v == 6) && !tiles_ok(a.nr, kTmaTR)) v = 1;
  if ((v == 2 || v == 3) && !(tiles_ok(a.nq, 32) && tiles_ok(a.nr, 8))) v = 1;
  if (v == 4 && !(tiles_ok(a.nq, 64) && tiles_ok(a.nr, 8))) v = 1;
  return v;
}

// Whether the block's stencil runs as the TMA kernel.  Its penalties are
// folded into DF beforehand by the face pre-kernel (launch_pre); the other
// variants get them afterwards from the face kernel (launch_corrections).
template <typename T>
bool stencil_is_tma(const VolumeArgs<T>& a) {
  const int v = effective_variant(a);
  return v == 5 || v == 6;
}

template <typename T, bool CURV, bool KAHAN>
void launch_stencil(const VolumeArgs<T>& a, cudaStream_t s) {
  constexpr bool f32 = sizeof(T) == 4;
  const int v = effective_variant(a);
  switch (v) {
    case 1: {
      dim3 blk(32, 8, 1), grd((a.nq + 31) / 32, (a.nr + 7) / 8, a.ns);
      if (a.fd == 1) stencil_kernel_pointwise<T, CURV, KAHAN, 1><<<grd, blk, 0, s>>>(a, 0);
      else if (a.fd == 2) stencil_kernel_pointwise<T, CURV, KAHAN, 2><<<grd, blk, 0, s>>>(a, 0);
      else if (a.fd == 3) stencil_kernel_pointwise<T, CURV, KAHAN, 3><<<grd, blk, 0, s>>>(a, 0);
      else stencil_kernel_pointwise<T, CURV, KAHAN, 0><<<grd, blk, 0, s>>>(a, 0);
      return;
    }
    case 3: launch_tiled<T, CURV, KAHAN, 32, 8, f32 ? 3 : 1>(a, s); return;
    case 4: launch_tiled<T, CURV, KAHAN, 64, 8, 1>(a, s); return;
    case 5:
    case 6:
      if constexpr (f32) {
        launch_stencil_tma(a, CURV, KAHAN, s);
        return;
      }
      [[fallthrough]];
    default: launch_tiled<T, CURV, KAHAN, 32, 8, 1>(a, s); return;
  }
}

template <typename T, bool CURV, bool KAHAN>
int launch_corr(const VolumeArgs<T>& a, cudaStream_t s) {
  int n = 0;
  dim3 blk(32, 8, 1), grd((a.nq + 31) / 32, (a.nr + 7) / 8, a.ns);
  if (a.anel) {  // before the PML kernel: it reads Q of the stage's input
    if (a.fd == 1) anelastic_kernel<T, CURV, KAHAN, 1><<<grd, blk, 0, s>>>(a);
    else if (a.fd == 2) anelastic_kernel<T, CURV, KAHAN, 2><<<grd, blk, 0, s>>>(a);
    else if (a.fd == 3) anelastic_kernel<T, CURV, KAHAN, 3><<<grd, blk, 0, s>>>(a);
    else anelastic_kernel<T, CURV, KAHAN, 0><<<grd, blk, 0, s>>>(a);
    ++n;
  }
  if (a.npml > 0) {
    const PmlBoxes bx = pml_boxes(a);
    const unsigned nblk = (unsigned)((bx.start[bx.n] + 255) / 256);
    if (bx.start[bx.n] > 0) {
      if (a.fd == 1) pml_kernel<T, CURV, KAHAN, 1><<<nblk, 256, 0, s>>>(a, bx);
      else if (a.fd == 2) pml_kernel<T, CURV, KAHAN, 2><<<nblk, 256, 0, s>>>(a, bx);
      else if (a.fd == 3) pml_kernel<T, CURV, KAHAN, 3><<<nblk, 256, 0, s>>>(a, bx);
      else pml_kernel<T, CURV, KAHAN, 0><<<nblk, 256, 0, s>>>(a, bx);
    }
    ++n;
  }
  if (!stencil_is_tma(a)) {
    const long long nface = 2LL * ((long long)a.nr * a.ns + (long long)a.nq * a.ns + (long long)a.nq * a.nr);
    face_kernel<T, KAHAN><<<(unsigned)((nface + 255) / 256), 256, 0, s>>>(a);
    ++n;
  }
  if (a.mp) {
    mms_kernel<T, KAHAN><<<grd, blk, 0, s>>>(a);
    ++n;
  }
  if (a.plastic) {
    PlasticBox<T> box;
    const int nn[3] = {a.nq, a.nr, a.ns};
    for (int ax = 0; ax < 3; ++ax) {
      box.lo[ax] = a.pml[2 * ax] ? a.npml : 0;
      box.hi[ax] = a.pml[2 * ax + 1] ? nn[ax] - a.npml : nn[ax];
    }
    box.pc[0] = (T)a.pl_ccos;
    box.pc[1] = (T)a.pl_sin;
    box.pc[2] = (T)a.pl_decay;
    for (int c = 0; c < 6; ++c) box.s0[c] = (T)a.s0u[c];
    const int bq = box.hi[0] - box.lo[0], br = box.hi[1] - box.lo[1], bs = box.hi[2] - box.lo[2];
    if (bq > 0 && br > 0 && bs > 0) {
      dim3 pgrd((bq + 31) / 32, (br + 7) / 8, bs);
      plastic_kernel<T, CURV, KAHAN><<<pgrd, blk, 0, s>>>(a, box);
    }
    ++n;
  }
  return n;
}

template <typename T>
void launch_volume(const VolumeArgs<T>& a, bool curv, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const bool kahan = a.C != nullptr;
  if (curv) kahan ? launch_stencil<T, true, true>(a, s) : launch_stencil<T, true, false>(a, s);
  else kahan ? launch_stencil<T, false, true>(a, s) : launch_stencil<T, false, false>(a, s);
}

template <typename T>
int launch_pre(const VolumeArgs<T>& a, void* stream) {
  if (!stencil_is_tma(a)) return 0;
  const long long nface = 2LL * ((long long)a.nr * a.ns + (long long)a.nq * a.ns + (long long)a.nq * a.nr);
  face_pre_kernel<T><<<(unsigned)((nface + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a);
  return 1;
}

template <typename T>
int launch_pre2(const VolumeArgs<T>& a0, const VolumeArgs<T>& a1, void* stream) {
  FacePair<T> P;
  P.a[0] = a0;
  P.a[1] = a1;
  auto nface = [](const VolumeArgs<T>& a) {
    return 2LL * ((long long)a.nr * a.ns + (long long)a.nq * a.ns + (long long)a.nq * a.nr);
  };
  P.n0 = nface(a0);
  const long long n = P.n0 + nface(a1);
  face_pre_kernel2<T><<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(P);
  return 1;
}

template <typename T>
int launch_corrections(const VolumeArgs<T>& a0, bool curv, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  // the PML velocity gradient comes from the stencil only when that was the
  // TMA kernel (the only one that writes it)
  VolumeArgs<T> a = a0;
  if (!stencil_is_tma(a)) a.G = nullptr;
  const bool kahan = a.C != nullptr;
  if (curv) return kahan ? launch_corr<T, true, true>(a, s) : launch_corr<T, true, false>(a, s);
  return kahan ? launch_corr<T, false, true>(a, s) : launch_corr<T, false, false>(a, s);
}

template <typename T>
void launch_source(const VolumeArgs<T>& a, const int lo[3], const int dim[3], const double* delta,
                   const double am[6], void* stream) {
  SourceArgs s;
  for (int c = 0; c < 3; ++c) {
    s.lo[c] = lo[c];
    s.dim[c] = dim[c];
  }
  for (int c = 0; c < 6; ++c) s.am[c] = am[c];
  s.delta = delta;
  const long long n = (long long)dim[0] * dim[1] * dim[2];
  if (n <= 0) return;
  const unsigned g = (unsigned)((n + 255) / 256);
  if (a.C) source_kernel<T, true><<<g, 256, 0, (cudaStream_t)stream>>>(a, s);
  else source_kernel<T, false><<<g, 256, 0, (cudaStream_t)stream>>>(a, s);
}

template void launch_source<double>(const VolumeArgs<double>&, const int*, const int*, const double*,
                                    const double*, void*);
template void launch_source<float>(const VolumeArgs<float>&, const int*, const int*, const double*,
                                   const double*, void*);
template void launch_volume<double>(const VolumeArgs<double>&, bool, void*);
template void launch_volume<float>(const VolumeArgs<float>&, bool, void*);
template int launch_corrections<double>(const VolumeArgs<double>&, bool, void*);
template int launch_pre<double>(const VolumeArgs<double>&, void*);
template int launch_pre<float>(const VolumeArgs<float>&, void*);
template int launch_pre2<float>(const VolumeArgs<float>&, const VolumeArgs<float>&, void*);
template int launch_corrections<float>(const VolumeArgs<float>&, bool, void*);
template bool stencil_is_tma<float>(const VolumeArgs<float>&);
template bool stencil_is_tma<double>(const VolumeArgs<double>&);

}  // namespace wql
