// Device-side data layout and kernel argument blocks (internal).
//
// HBM layout per block (nq x nr x ns points, q fastest, no ghost layers --
// the reference's 3-deep MPI halos, src/mpi3dcomm.f90:722-746, do not exist
// on one GPU).  Rows along q are padded to a pitch pq (a multiple of 16
// bytes) so every row starts on a TMA-legal address; np = pq*nr*ns:
//   F[2]  : 9 x np field components, ping-pong buffers (stage reads one and
//           writes the other, so neighbours never see a half-updated state)
//   DF    : 9 x np rates (RK 2N-storage register), updated in place
//   C     : 9 x np Kahan compensation of F, as bfloat16 (FP32-compensated
//           mode only; see comp_t)
//   coef  : curvilinear: 13 x np = J*metric (3 directions x 3 components),
//           1/J, lambda, mu, 1/(rho*J); Cartesian: 3 x np = lambda, mu, 1/rho
//   face  : per side 15 x nface (FP64): n(3), m(3), l(3), grad(3) of the
//           face-normal coordinate, lambda, mu, rho
//   Q/DQ  : PML auxiliary fields on slabs of npml layers per active side
//   G     : 9 x np velocity gradient hand-off (FP32C with PML or attenuation)
//   eta/Deta, qs : 24 x np memory variables and their rates, 1/Qs per point
//           (anelastic response only)
#pragma once
#include <cuda.h>

#include <cstddef>
#include <cstdint>
#ifdef __CUDACC__
#include <cuda_bf16.h>
#endif

#include "wql_presets.cuh"

namespace wql {

// Storage of the Kahan compensation term of the FP32 fields: the bits of a
// bfloat16.  The term is the rounding error of the last compensated update
// (at most half an FP32 unit in the last place of the field); kept to 8
// significant bits it still cancels all but 2^-9 of that error at the next
// update, so a field carries about 33 significant bits between stages,
// against 24 for FP32 alone, and the rates' own FP32 rounding stays the
// larger error.  The stencil moves 36 bytes per point less than with an
// FP32 term (232 instead of 268).
typedef unsigned short comp_t;

constexpr int kFaceWords = 15;
constexpr int kCurvCoef = 13;
constexpr int kCartCoef = 3;

// Boundary penalty selection for the outer faces.
enum BcForm : int { BC_CHARACTERISTIC = 0, BC_WEIGHTED = 1 };

// A table upwind operator (fd 3: the upwind operators of orders 2, 3, 4, 7,
// 8, 9 and the DRP variants of src/JU_xJU_yJU_z6.f90, tabulated in
// wql_upwind_tables.h) in device memory, in the field type: the interior
// weights ip[13] im[13] (the interior routine) and bp[13] bm[13] (the
// interior rows of the boundary shell), then the closure rows lp, lm, rp, rm,
// each [axis 3][row 8][point 13].  R closure rows per end; interior D+ on
// offsets plo .. plo+pn-1, D- on mlo .. mlo+mn-1.
struct UpG {
  const void* w;
  int R, plo, pn, mlo, mn;
};
constexpr int kUgCol = 13, kUgRows = 8, kUgRowBlock = 3 * kUgRows * kUgCol, kUgWords = 4 * kUgCol + 4 * kUgRowBlock;

template <typename T>
struct VolumeArgs {
  int nq, nr, ns;
  int pq;             // row pitch along q (nq rounded up to 16 bytes)
  long long np;       // pq * nr * ns, the component stride of F, DF, C, coef
  int block;          // 0: fault on the q = nq face; 1: fault on the q = 1 face
  T rh[3];            // 1/h per axis, h = 1/(n-1)
  const T* __restrict__ Fin;
  T* __restrict__ Fout;
  T* __restrict__ DF;
  comp_t* __restrict__ C;  // compensation (FP32C) or nullptr
  const T* __restrict__ coef;
  T cart_metric[3];   // q_x, r_y, s_z for Cartesian blocks
  // outer faces (side 0..5 = -q,+q,-r,+r,-s,+s)
  const double* face[6];
  int bc[6];          // 1 absorbing, 2 free surface, 3 clamped, else none
  int bc_form;
  T tau_h[3];         // tau0 / h per axis
  // fault SAT added on the fault face (9 x nr*ns), already scaled by tau0/h
  const T* __restrict__ fault_sat;
  // PML
  int pml[6];
  int npml;
  T* Q[6];
  T* DQ[6];
  long long slab_np[6];
  // velocity gradient g[c][j] (component c*3+j, stride np) of the PML points
  // (of every point with the anelastic response), written by the TMA stencil
  // kernel and read by the PML and anelastic kernels of the same stage;
  // nullptr where those kernels form it themselves
  T* G;
  int fd;             // difference operator: 0 SBP-6 central; upwind pair (D+ on v, D- on fluxes) of order 6 (1),
                      // of order 5 (2), or a table operator (3, ug)
  UpG ug;
  int kernel;         // stencil variant: 0 default, 1 per-point, 2..4 tiled
  int schunk;         // planes per CTA along s for the tiled kernel (0: default)
  // RK
  T A, Bdt;
  // plasticity on the last stage
  int plastic;
  int preset;          // initial-stress preset for the plastic update (PRE_NONE: s0u)
  double s0u[6];       // uniform initial stress
  const T* __restrict__ ycoord;  // depth coordinate for the initial stress
  double pl_c, pl_nu, pl_Tv, dt;
  double pl_ccos, pl_sin, pl_decay;  // c*cos(atan nu), sin(atan nu), exp(-dt/Tv)
  // plastic_flow (plastic_model other than 'scec', src/plastic.f90:220-290):
  // the block's internal friction mu, dilatancy beta and viscosity eta, and
  // per point the plastic strain rate lambda and plastic strain gammap
  int pl_flow;
  double pl_mu, pl_beta, pl_eta;
  T* pl_lambda;
  T* pl_gammap;
  // anelastic response (src/RHS_Interior.f90:2390-2509): memory variables
  // eta and their rates Deta (24 x np each, component c*4 + i for stress
  // component 4+c and mechanism i), 1/Qs per point (1/Qp = 1/(2 Qs)), the
  // relaxation times and weights; anel = 0 without
  int anel;
  T* eta;
  T* Deta;
  const T* qsinv;
  double an_tau[4], an_w[4];
  int* err;                      // device error word (pipeline wait timeouts)
  double pml_d0;                 // PML damping scale 3 ln(1000)
  const void* tma;               // host pointer to the block's StencilMaps (FP32 only)
  // manufactured solution (&mms_list use_mms): u_exact = T(t) S(x), where S
  // is sin*sin*sin for the velocities (ms[0..np)) and cos*cos*cos for the
  // stresses (ms[np..2np)); the forcing is T(t) mp - T'(t) S with mp the
  // 9 x np operator shapes.  nullptr without; mms_T and mms_Tp are T and T'
  // at the stage's time.
  const T* ms;
  const T* mp;
  T mms_T, mms_Tp;
};

struct InterfaceArgs {
  int nr, ns;
  long long np0, np1;       // component strides (pitched) of the two blocks
  int nq0;
  int pq0, pq1;             // row pitches along q
  int fp64;                 // fields are double (1) or float (0)
  const void* F0;           // block 0 fields (9 x np0)
  const void* F1;           // block 1 fields (9 x np1)
  const double* face0;      // block 0, side +q (15 x nf)
  const double* face1;      // block 1, side -q (15 x nf)
  const double* xij;        // 2 x 3 x nf fault-point coordinates per block copy
  double* S;                // 2 x 4 x nf
  double* DS;               // 2 x 4 x nf
  double* W;                // 2 x nf
  double* DW;               // 2 x nf
  double* trup;             // 2 x nf
  void* sat;                // 2 x 9 x nf (T), scaled by tau0/h of the block
  const double* pre;        // 2 x 5 x nf: static Tn, Tm, Tl, nucleation weight, rate-state a
  double ramp;              // nucleation ramp at this stage's time
  double lnV0h;             // ln(1/(2 V0)) of the rate-and-state law
  double rs_bL, rs_binv;    // b/L and 1/b of the aging law (uniform along the fault)
  double rs_tol;            // FP64 regula falsi: tolerance and iteration cap
  int rs_maxit;
  double tau_h[2];
  double A, Bdt, t;
  int stage;
  FaultParams fp;
  float* frame;             // 39 x nf or nullptr
  unsigned int* solver_fail;  // count of non-converged rate-and-state solves
  // FP32 fields: the Kahan compensation of both blocks, and whether the
  // fault algebra reads the compensated face values in FP64 (1) or works
  // on the FP32 fields in FP32 (0)
  const void* C0;
  const void* C1;
  int fault_comp;
  // manufactured solution: the two blocks' shapes (2 x np, field type) or
  // nullptr, and T(t) at the stage's time
  const void* ms0;
  const void* ms1;
  double mms_T;
};

// Frame record layout (floats per fault point, component-major):
// Uface 9, Vface 9, S 4, Uhat 6, Vhat 6, Svel 3, trup 1, state 1.
constexpr int kFrameWords = 39;
enum FrameOff : int {
  FR_UFACE = 0, FR_VFACE = 9, FR_S = 18, FR_UHAT = 22, FR_VHAT = 28, FR_SVEL = 34,
  FR_TRUP = 37, FR_STATE = 38, FR_END = 39
};
// offsets of streams 0..7 (+ end) in the order of wql_get_frames
constexpr int kFrameOff[9] = {FR_UFACE, FR_VFACE, FR_S, FR_UHAT, FR_VHAT, FR_SVEL, FR_TRUP, FR_STATE, FR_END};

// Kernel launchers (stream-ordered).
// Tensor maps of one block for the TMA stencil kernel (FP32 fields): the
// field box with halo and the lead-plane tile for each of the two field
// buffers, and the coefficient boxes.  Built once at set-up.
// Tile 32 (q) x 12 (r): twelve consumer warps and a two-deep ring of
// stages fill one SM's shared memory (measured faster than 32 x 8 tiles with
// three stages, 32 x 10 and 64 x 6 on 2 x 201^3 blocks).
constexpr int kTmaTQ = 32, kTmaTR = 12, kTmaStages = 2;
// Cartesian blocks whose q extent fills 40-wide tiles better (76 points: 2
// tiles of 40 use 95 % of their columns, 3 of 32 use 79 %) take this width;
// 15 consumer warps, the same 128-register cap.
constexpr int kTmaTQWide = 40;
struct StencilMaps {
  CUtensorMap fbox[2], flead[2];  // per field buffer
  CUtensorMap ca, cb, cc, cl;     // coefficients: q-halo rows, r-halo columns, tile, lead plane
  CUtensorMap df, ck;             // rates and compensation on the tile
  CUtensorMap flead2[2];          // upwind pair: the stress lead tile (else = flead)
  int cur;                        // which field buffer is the stage input
  int fd;                         // operator the boxes are shaped for (0 central, 1 upwind)
  int tq;                         // tile width along q the boxes are shaped for
  int ok;
};
// Fills m for a block (fd: 0 the central SBP-6 operator, 1 the upwind pair:
// r halo of 4 rows, velocity and stress lead tiles from different planes);
// returns 0 or a CUDA driver error code.
int make_stencil_maps(StencilMaps& m, void* const F[2], void* coef, void* DF, void* C, int nq, int nr, int ns, int pq,
                      bool curv, int fd, int tq);
// Tile width along q (kTmaTQ or kTmaTQWide) for a scenario whose blocks have
// nq0 and nq1 points along q.
int tma_tile_width(int nq0, int nq1, bool curv);
// Launches the TMA stencil kernel (every plane of the block).
void launch_stencil_tma(const VolumeArgs<float>& a, bool curv, bool kahan, void* stream);
// The same for both blocks of a scenario in one launch.
void launch_stencil_tma2(const VolumeArgs<float>& a0, const VolumeArgs<float>& a1, bool curv, bool kahan,
                         void* stream);
// Whether the block's stencil runs as the TMA kernel (the tuning and the
// block shape allow it).
template <typename T>
bool stencil_is_tma(const VolumeArgs<T>& a);

// One entry of the packed table of the batched TMA stencil launch: one block
// at one stage (its tensor maps for the stage's input buffer, its arguments)
// and the range of CTAs [cta0, cta0 + tq*tr*nchunk) that work on it.
struct TmaBatchDesc {
  CUtensorMap m[9];  // field box, lead fields, coefficient boxes (q, r, tile, lead), DF, C, stress lead
  VolumeArgs<float> a;
  int schunk, tq, tr, nchunk;
  long long cta0;
};
// Fills d for one block (a.tma must point at the block's StencilMaps) and
// returns the number of CTAs it needs.
long long fill_tma_desc(const VolumeArgs<float>& a, TmaBatchDesc& d);
// Whether a block can go through the TMA stencil (FP32, r extent that keeps
// the closure rows of the shifted last r tile inside the halo).
bool tma_eligible(const VolumeArgs<float>& a);
// One launch over nd table entries (all curvilinear or all Cartesian, all
// with or all without compensation).
void launch_stencil_tma_batch(const TmaBatchDesc* d_dev, int nd, long long total_ctas, bool curv, bool kahan,
                              void* stream);

// One stage on one block: launch_volume runs the stencil kernel (DF and the
// updated fields for every point); launch_corrections then adds the PML,
// boundary/fault penalty and plastic kernels and returns how many it issued.
template <typename T>
void launch_volume(const VolumeArgs<T>& a, bool curv, void* stream);
// Before the stencil kernel of a variant without its own face pass: the
// boundary and fault penalties folded into DF of the face points.  Returns
// the number of launches.
template <typename T>
int launch_pre(const VolumeArgs<T>& a, void* stream);
// The same for both blocks of a scenario whose stencils both run as the TMA
// kernel, in one launch.
template <typename T>
int launch_pre2(const VolumeArgs<T>& a0, const VolumeArgs<T>& a1, void* stream);
template <typename T>
int launch_corrections(const VolumeArgs<T>& a, bool curv, void* stream);
// One moment-tensor source: DF(4:9) -= am * delta on a box of points
// (0-based origin lo, extents dim, delta q fastest), F_out to match.
template <typename T>
void launch_source(const VolumeArgs<T>& a, const int lo[3], const int dim[3], const double* delta,
                   const double am[6], void* stream);
void launch_interface(const InterfaceArgs& a, void* stream);
void launch_metrics(int nq, int nr, int ns, const double* x, double* metric, double* J,
                    void* stream);
// Anelastic set-up on the dense FP64 material arrays (src/material.f90:
// 69-140): qsinv = 1/(c vs) from the relaxed moduli, then mu and lambda
// replaced by their unrelaxed values; den[l] = (2 pi fref)^2 tau_l^2 + 1.
void launch_anelastic_material(long long n, double c, const double den[4], const double w[4], double* lam,
                               double* mu, const double* rho, double* qsinv, void* stream);
void launch_faces(int nq, int nr, int ns, const double* metric, const double* lam,
                  const double* mu, const double* rho, double* const face[6], void* stream);
template <typename T>
void launch_coef(int nq, int nr, int ns, int pq, bool curv, const double* metric, const double* J,
                 const double* lam, const double* mu, const double* rho, T* coef, void* stream);
// Manufactured solution (&mms_list): wavenumbers kx, ky, kz = n pi of the
// space factors (src/mms.f90:136-150).  The set-up writes the shapes ms
// (2 x np), the forcing shapes mp (9 x np) and the initial fields F of one
// block in the field type; the norms kernel adds, per component, the sums
// of (F - T S)^2 and (T S)^2 into acc[0..18).
struct MmsWave {
  double kx, ky, kz;
};
void launch_mms_setup(int nq, int nr, int ns, int pq, const MmsWave& w, const double* x, const double* lam,
                      const double* mu, const double* rho, bool fp64, void* ms, void* mp, void* F, void* stream);
template <typename T>
void launch_mms_norms(int nq, int nr, int ns, int pq, const T* F, const T* ms, double Tt, double* acc,
                      void* stream);

#ifdef __CUDACC__
// The compensation term i of C, widened to FP32, and a new value rounded to
// the nearest bfloat16.
__device__ __forceinline__ float comp_get(const comp_t* C, long long i) {
  return __bfloat162float(__ushort_as_bfloat16(C[i]));
}
__device__ __forceinline__ void comp_put(comp_t* C, long long i, float v) {
  C[i] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
}
#endif

}  // namespace wql
