// Sixth-order SBP first-derivative operator used by every stencil in the
// hot path (src/JU_xJU_yJU_z6.f90:55-164 and :16200-16300 for the central
// rows; src/metrics.f90:29-160 for the same rows applied to grid
// coordinates).  Rows 1..6 are one-sided closures on points 1..9; the right
// boundary uses the negated mirror image; interior rows are the 7-point
// central stencil (0.75, -0.15, 1/60).
#pragma once

#ifdef __CUDACC__
#define WQL_HD __host__ __device__ __forceinline__
#else
#define WQL_HD inline
#endif

namespace wql {

// Dense closure table: SBP_L[row][col] is the weight of point col+1 in the
// derivative at point row+1 (1-based), for rows 1..6.
#define WQL_SBP_TABLE                                                                                  \
  {{-1.582533518939116, 2.033378678700676, -0.141512858744873, -0.450398306578272, 0.104488069284042, \
    0.036577936277544, 0.0, 0.0, 0.0},                                                                 \
   {-0.462059195631158, 0.0, 0.287258622978251, 0.258816087376832, -0.069112065532624,                 \
    -0.014903449191300, 0.0, 0.0, 0.0},                                                                \
   {0.071247104721830, -0.636451095137907, 0.0, 0.606235523609147, -0.022902190275815,                 \
    -0.018129342917256, 0.0, 0.0, 0.0},                                                                \
   {0.114713313798970, -0.290087484386815, -0.306681191361148, 0.0, 0.520262285050482,                 \
    -0.051642265516119, 0.013435342414630, 0.0, 0.0},                                                  \
   {-0.036210680656541, 0.105400944933782, 0.015764336127392, -0.707905442575989, 0.0,                 \
    0.769199413962647, -0.164529643265203, 0.018281071473911, 0.0},                                   \
   {-0.011398193015050, 0.020437334208704, 0.011220896474665, 0.063183694641876, -0.691649024426814,   \
    0.0, 0.739709139060752, -0.147941827812150, 0.016437980868017}}

constexpr double kC1 = 0.75, kC2 = -0.15, kC3 = 1.0 / 60.0;

// Row kind of 0-based index i on an axis of n points: -1..-6 left closure
// rows (row = -kind-1), +1..+6 right closure rows (row = kind-1), 0 central.
WQL_HD int sbp_kind(int i, int n) {
  if (i < 6) return -(i + 1);
  if (i >= n - 6) return (n - i);
  return 0;
}

}  // namespace wql
