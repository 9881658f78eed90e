// Device helpers shared by the stencil kernels: the SBP-6 closure weights in
// constant memory, the row lookup of the first-derivative operator, the
// stress-component map and the tile ownership rule of the tiled kernels.
// Included by each CUDA translation unit that differences fields (every
// unit gets its own constant-memory copy of the table).
#pragma once

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

}  // namespace
}  // namespace wql
