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

// Sixth-order upwind SBP operators (fd_type 'upwind', order 6,
// src/JU_xJU_yJU_z6.f90:2680-3706 and :17675-17983): the velocities are
// differenced with the forward operator D+, the stress fluxes with the
// backward operator D-.  WQL_UP_TABLE[0] holds the left closure rows 1..6 of
// D+, [1] those of D- (dense, point col+1 of row+1, up to 10 points).  The
// right closure rows of D+ are the negated mirror images of the left rows of
// D-, and those of D- of D+.  Interior rows: D+ weights WQL_UP_CF on
// offsets -2..4; D- weights -WQL_UP_CF[2-o] on offsets o = -4..2.
#define WQL_UP_TABLE                                                                                          \
  {{{-1.593253459452621, 2.093702214477299, -0.275607596716317, -0.302855902188632, 0.023993033880123,        \
     0.054021710000147, 0.0, 0.0, 0.0, 0.0},                                                                  \
    {-0.460835552271137, -0.029551468764759, 0.393228064437077, 0.105980141988699, 0.030739159126096,         \
     -0.039560344515975, 0.0, 0.0, 0.0, 0.0},                                                                 \
    {0.096333139747688, -0.629259919521358, -0.306540940575249, 1.258766829227482, -0.589452745232692,        \
     0.197069524204597, -0.026915887850467, 0.0, 0.0, 0.0},                                                   \
    {0.0925965903611, -0.240558007429252, -0.243684445410829, -0.318292975073623, 0.946962507015985,          \
     -0.330443502642251, 0.106765523632994, -0.013345690454124, 0.0, 0.0},                                    \
    {-0.015609194255155, 0.033485250803205, 0.041897570295664, -0.450132219590077, -0.593528379527062,        \
     1.406282074938901, -0.550950133911491, 0.146920035709731, -0.018365004463716, 0.0},                      \
    {-0.0161631016574, 0.040531470682718, -0.00533856744421, -0.025427590054054, -0.357460227911152,          \
     -0.572337434946968, 1.313958528183954, -0.492734448068983, 0.131395852818395, -0.016424481602299}},      \
   {{-1.58018369620741, 2.039450367044345, -0.189297839436616, -0.366971721882124, 0.044953974933765,         \
     0.05204891554804, 0.0, 0.0, 0.0, 0.0},                                                                   \
    {-0.473094335557797, 0.029551468764759, 0.279404147185598, 0.215422101432619, -0.021790841692085,         \
     -0.029492540133095, 0.0, 0.0, 0.0, 0.0},                                                                 \
    {0.140255933237354, -0.88560840157053, 0.306540940575249, 0.491468255323896, -0.061405392278187,          \
     0.008748664712219, 0.0, 0.0, 0.0, 0.0},                                                                  \
    {0.076418487423426, -0.11834612889915, -0.624133691970994, 0.318292975073623, 0.327107204245208,          \
     0.020661154127888, 0.0, 0.0, 0.0, 0.0},                                                                  \
    {-0.008331008040049, -0.047235828122731, 0.402190050630647, -1.303115093827634, 0.593528379527062,        \
     0.399693508760138, -0.036730008927433, 0.0, 0.0, 0.0},                                                 \
    {-0.016775726857039, 0.054367610816546, -0.120254802392339, 0.406675342006739, -1.257688453771463,        \
     0.572337434946968, 0.394187558455186, -0.032848963204599, 0.0, 0.0}}}

// Interior weights of the order-6 D+ on offsets -2..4 (D- at offset o is
// -WQL_UP_CF[2-o]).
#define WQL_UP_CF {1.0 / 30.0, -2.0 / 5.0, -7.0 / 12.0, 4.0 / 3.0, -1.0 / 2.0, 2.0 / 15.0, -1.0 / 60.0}

// Upwind operators of order 5 (src/JU_xJU_yJU_z6.f90:2049-2677, 17364-17671):
// four closure rows per end reading up to 7 points, laid out as
// WQL_UP_TABLE; interior D+ weights WQL_UP5_CF on offsets -2..3, D- at
// offset o is -WQL_UP5_CF[2-o] (offsets -3..2).
#define WQL_UP5_TABLE                                                                                        \
  {{{-1.458167330677291, 1.874501992031873, -0.374501992031873, -0.041832669322709, 0.0, 0.0, 0.0},          \
    {-0.484392419175028, -0.073578595317726, 0.627090301003345, -0.0958751393534, 0.026755852842809, 0.0,     \
     0.0},                                                                                                    \
    {0.091627172195893, -0.604265402843602, -0.274881516587678, 1.033965244865719, -0.28436018957346,         \
     0.037914691943128, 0.0},                                                                                 \
    {0.030446549391069, -0.029769959404601, -0.44722598105548, -0.316644113667118, 0.974289580514208,         \
     -0.243572395128552, 0.032476319350474}},                                                                 \
   {{-1.410358565737052, 1.731075697211155, -0.231075697211155, -0.089641434262948, 0.0, 0.0, 0.0},          \
    {-0.524526198439242, 0.073578595317726, 0.426421404682274, 0.024526198439242, 0.0, 0.0, 0.0},             \
    {0.148499210110585, -0.888625592417062, 0.274881516587678, 0.522116903633491, -0.056872037914692, 0.0,     \
     0.0},                                                                                                    \
    {0.014208389715832, 0.11637347767253, -0.885656292286874, 0.316644113667118, 0.487144790257104,           \
     -0.04871447902571, 0.0}}}
#define WQL_UP5_CF {0.05, -0.5, -1.0 / 3.00, 1.0, -0.25, 1.0 / 30.0}
constexpr double kTau0Upwind5 = 720.0 / 251.0;  // src/block.f90:208-210

// Penalty weight tau0 of the upwind operators of order 6, as the reference
// sets it (src/block.f90:212-214).  It is 0.979 times 1/h11 of the
// operators' diagonal norm (h11 = 13613/43200).
constexpr double kTau0Upwind6 = 42300.0 / 13613.0;

// Closure rows of the s derivative in the TMA stencil, which keeps the
// velocities and s fluxes of nearby planes in a register window (central
// operator: planes s-3..s+3 for both; order-6 upwind pair: velocities of
// s-2..s+4, fluxes of s-4..s+2).  Closure row `row` (0..5) at the left end
// (plane s = row) or the right end (plane s = ns-1-row), column t:
// its weight on the velocities (flux = false) or fluxes (flux = true) --
// the central SBP-6 row, or for the upwind pair D+ on the velocities and D-
// on the fluxes (right rows: the negated mirror images, D- on the velocities
// and D+ on the fluxes) -- its plane offset from s, and its positions in
// the velocity and flux windows (outside 0..6: the plane is read from
// memory).
constexpr double s_close_w(int fd, bool right, bool flux, int row, int t) {
  constexpr double L[6][9] = WQL_SBP_TABLE;
  constexpr double U[2][6][10] = WQL_UP_TABLE;
  if (fd == 0) return t < 9 ? (right ? -L[row][t] : L[row][t]) : 0.0;
  const int op = right ? (flux ? 0 : 1) : (flux ? 1 : 0);
  return right ? -U[op][row][t] : U[op][row][t];
}
constexpr int s_close_off(bool right, int row, int t) { return right ? row - t : t - row; }
constexpr int s_close_vpos(int fd, bool right, int row, int t) { return s_close_off(right, row, t) + (fd ? 2 : 3); }
constexpr int s_close_fpos(int fd, bool right, int row, int t) { return s_close_off(right, row, t) + (fd ? 4 : 3); }

// Row kind of 0-based index i on an axis of n points: -1..-6 left closure
// rows (row = -kind-1), +1..+6 right closure rows (row = kind-1), 0 central.
WQL_HD int sbp_kind(int i, int n) {
  if (i < 6) return -(i + 1);
  if (i >= n - 6) return (n - i);
  return 0;
}

}  // namespace wql
