// C ABI implementation: scenario setup (init_domain) and the RK step driver
// (time_step_RK, src/time_step.f90:68-150) over the device kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <filesystem>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/wql.h"
#include "host/wql_grid.h"
#include "host/wql_input.h"
#include "wql_internal.h"
#include "wql_sbp.cuh"
#include "wql_upwind_tables.h"

using namespace wql;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) return fail(WQL_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Kennedy-Carpenter (5,4) 2N-storage coefficients (src/time_step.f90:53-62).
struct RK {
  double A[6], B[6], C[6];
  RK() {
    A[1] = 0.0;
    A[2] = -567301805773.0 / 1357537059087.0;
    A[3] = -2404267990393.0 / 2016746695238.0;
    A[4] = -3550918686646.0 / 2091501179385.0;
    A[5] = -1275806237668.0 / 842570457699.0;
    B[1] = 1432997174477.0 / 9575080441755.0;
    B[2] = 5161836677717.0 / 13612068292357.0;
    B[3] = 1720146321549.0 / 2090206949498.0;
    B[4] = 3134564353537.0 / 4481467310338.0;
    B[5] = 2277821191437.0 / 14882151754819.0;
    C[0] = 0.0;
    C[1] = 1432997174477.0 / 9575080441755.0;
    C[2] = 2526269341429.0 / 6820363962896.0;
    C[3] = 2006345519317.0 / 3224310063776.0;
    C[4] = 2802321613138.0 / 2924317926251.0;
    C[5] = 1.0;
  }
};

// Records per station ring: as many as fit in 16 MiB for the largest
// requested station list, 64 to 1024 (a ring that fills is copied out
// synchronously, so a short served request should not fill it).
int station_ring_cap(const Problem& P) {
  const size_t n = std::max({P.stations.size(), P.stationsU.size(), P.stationsV.size()}) / 3;
  const long long per = std::max<long long>(1, (long long)n * 3 * (long long)sizeof(double));
  return (int)std::max(64LL, std::min(1024LL, (16LL << 20) / per));
}

// Frames per fault-frame ring: as many as fit in 128 MiB, 4 to 64.
int frame_ring_cap(long long nf) {
  const long long frame_bytes = (long long)kFrameWords * nf * (long long)sizeof(float);
  return (int)std::max(4LL, std::min(64LL, (128LL << 20) / std::max(frame_bytes, 1LL)));
}

int preset_of(const std::string& pb) {
  if (pb == "TPV5" || pb == "LOH1" || pb == "OKLAHOMA") return PRE_TPV5;
  if (pb == "TPV26") return PRE_TPV26;
  if (pb == "TPV27") return PRE_TPV27;
  if (pb == "TPV28") return PRE_TPV28;
  if (pb == "TPV29") return PRE_TPV29;
  if (pb == "TPV30") return PRE_TPV30;
  if (pb == "TPV10") return PRE_TPV10;
  if (pb == "TPV101") return PRE_TPV101;
  if (pb == "TPV102") return PRE_TPV102;
  if (pb == "sw_param") return PRE_SW_PARAM;
  if (pb == "rs_param") return PRE_RS_PARAM;
  if (pb == "rate-weakening") return PRE_RATE_WEAKENING;
  return PRE_NONE;
}

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct wql_ctx {
  int device = 0;
};

struct wql_scn {
  // process-unique identity (an address can be reused by a later scenario)
  const long long uid = next_uid();
  static long long next_uid() {
    static std::atomic<long long> n{0};
    return ++n;
  }
  wql_ctx* ctx = nullptr;
  Problem P;
  wql_media media{};
  int prec = WQL_FP64;
  size_t esz = 8;
  cudaStream_t stream = nullptr;
  RK rk;
  double dt = 0, t = 0;
  int nt = 0, nstep = 0;
  bool curv = false;
  std::vector<DevBuf> allocs;
  long long device_bytes = 0;
  struct Block {
    int nq = 0, nr = 0, ns = 0;
    int pq = 0;         // row pitch along q: nq rounded up to 8 (FP32) or 2 (FP64) points
    long long npd = 0;  // nq * nr * ns (dense, the precompute arrays)
    long long np = 0;
    void* F[2] = {nullptr, nullptr};
    void* DF = nullptr;
    void* C = nullptr;
    void* coef = nullptr;
    double* face[6] = {};
    int bc[6] = {};
    int pml[6] = {};
    int npml = 0;
    void* Q[6] = {};
    void* DQ[6] = {};
    long long slab_np[6] = {};
    void* G = nullptr;  // velocity gradient hand-off (FP32C with PML or attenuation)
    void* eta = nullptr;   // anelastic memory variables (24 x np)
    void* Deta = nullptr;  // and their rates
    void* qs = nullptr;    // 1/Qs per point
    void* y = nullptr;
    void* pl_lambda = nullptr;  // plastic_flow: plastic strain rate and
    void* pl_gammap = nullptr;  // plastic strain per point
    void* ms = nullptr;    // manufactured-solution shapes (2 x np) and
    void* mp = nullptr;    // forcing shapes (9 x np), use_mms only
    double cart_metric[3] = {1, 1, 1};
    double tau_h[3] = {};
    StencilMaps maps{};  // TMA tensor maps (FP32 fields)
  } B[2];
  int cur = 0;
  // interface (two block copies)
  double *S = nullptr, *DS = nullptr, *W = nullptr, *DW = nullptr, *trup = nullptr, *xij = nullptr;
  double* pre = nullptr;  // 2 x 5 x nf time-independent interface data
  void* sat = nullptr;
  unsigned int* solver_fail = nullptr;
  int* err_dev = nullptr;  // kernel error word (bounded pipeline waits that ran out)
  FaultParams fp{};
  int bc_form = BC_CHARACTERISTIC;
  double rs_tol = 1.0e-12;  // FP64 regula falsi tolerance and iteration cap
  int rs_maxit = 5000;
  bool fault_comp = true;   // FP32C: fault algebra on the compensated face values in FP64
  // manufactured solution (&mms_list use_mms): T(t) = cos(kt t) and T'(t)
  // at the current stage's time, and an 18-double accumulator for the norms
  bool mms = false;
  double mms_kt = 0.0, mms_T = 1.0, mms_Tp = 0.0;
  double* mms_acc = nullptr;
  // a step advanced stage by stage (wql_stage): the next stage to run (1:
  // no step in progress) and the step's context
  int next_stage = 1;
  bool want_frame = false, want_station = false;
  double stage_t0 = 0.0;
  int stage_launches = 0;
  int kernel_variant = 0;  // stencil variant (0 default per precision)
  int fd = 0;              // 0: traditional SBP-6; 1: upwind order 6; 2: upwind order 5; 3: a table operator
  const UpwindTable* ut = nullptr;  // fd 3: the operator's table
  void* ug_dev = nullptr;           // fd 3: the table on the device, in the field type
  bool anel = false;       // response = 'anelastic'
  double an_tau[4] = {}, an_w[4] = {};
  int schunk = 0;          // planes per CTA along s (0: default)
  bool plastic = false;
  bool pl_flow = false;  // plastic_flow (the reference's default model) instead of scec
  double pl_c = 1.36, pl_nu = 0.1934, pl_Tv = 0.03;
  // fault frames: two device rings of frame_cap frames.  When the ring
  // being filled is full, its copy to pinned host memory is queued on the
  // stream and the other ring takes the next frames, so stepping never
  // waits on the copy; the pinned frames move to the host chunks when the
  // next ring fills or the frames are read.
  float* frame_ring[2] = {nullptr, nullptr};
  float* frame_dev = nullptr;  // the ring being filled
  int frame_cap = 0, frame_fill = 0, ring_cur = 0;
  float* frame_pin = nullptr;  // pinned staging of one ring (null: synchronous copies)
  int pin_frames = 0;          // frames in flight to frame_pin
  cudaEvent_t pin_done = nullptr;
  std::vector<std::vector<float>> frame_chunks;  // flushed frames, whole frames per chunk
  int nframes = 0;
  // seismogram stations per block (src/seismogram.f90): 1-based grid
  // indices, device point offsets, a device ring of velocity records
  // (same capacity as the frame ring) and the flushed host records
  struct Stations {
    std::vector<int> ijk;
    std::vector<double> xyz;       // requested positions of the stations found
    long long* idx_dev = nullptr;
    double* ring = nullptr;        // cap x n x 3
    std::vector<double> host;      // records x n x 4 (t, vx, vy, vz)
  } st[2];
  int st_cap = 0, st_fill = 0, st_records = 0;
  std::vector<double> st_times;    // times of the records still in the ring
  // moment-tensor point sources (src/moment_tensor.f90): per block, every
  // listed source's placement (found at set-up), then the applied ones with
  // their discrete delta on a box of grid points
  struct MTCand {
    bool found = false, in_box = false;
    int lo[3] = {0, 0, 0}, dim[3] = {0, 0, 0};  // delta box (0-based origin, extents)
    std::vector<double> delta;                  // box points, q fastest
  };
  struct MTSrc {
    MomentSource src;
    int lo[3], dim[3];
    double* delta = nullptr;  // device, box points
  };
  std::vector<MTCand> mt_cand[2][2];  // [block][0: unified list, 1: the block's own list]
  std::vector<MTSrc> mt[2];
  // optional per-launch timing (CUDA events on the scenario stream)
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<size_t, int>> ev_marks;  // (start event, kind 0 interface / 1 stencil / 2 corrections)
  int launches_last_step = 0;
  cudaEvent_t next_event() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }

  ~wql_scn() {
    if (stream) cudaStreamSynchronize(stream);  // no copy in flight to frame_pin
    if (frame_pin) cudaFreeHost(frame_pin);
    if (pin_done) cudaEventDestroy(pin_done);
    for (auto e : ev_pool) cudaEventDestroy(e);
    for (auto& a : allocs)
      if (a.p) cudaFree(a.p);
    if (stream) cudaStreamDestroy(stream);
  }

  int alloc(void** p, size_t bytes, bool zero = true) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
      *p = nullptr;
      return fail(WQL_E_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " +
                                 cudaGetErrorString(e));
    }
    allocs.push_back({*p, bytes});
    device_bytes += (long long)bytes;
    if (zero) {
      e = cudaMemsetAsync(*p, 0, bytes, stream);
      if (e != cudaSuccess) return fail(WQL_E_CUDA, cudaGetErrorString(e));
    }
    return WQL_OK;
  }
  void release(void* p) {
    for (auto& a : allocs)
      if (a.p == p) {
        cudaFree(a.p);
        device_bytes -= (long long)a.bytes;
        a.p = nullptr;
      }
  }
};

namespace {

template <typename T>
__global__ void fill_comp(T* F, long long np, int comp, T val) {
  long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p < np) F[comp * np + p] = val;
}


// Pitched rows (pq per row) <-> dense FP64 rows (nq per row), so that the
// host copy is one contiguous transfer (a 2-D copy of short rows runs at a
// fraction of the link's rate).
template <typename T>
__global__ void pitched_to_dense(const T* __restrict__ in, int pq, int nq, long long rows, double* __restrict__ out) {
  const long long n = (long long)nq * rows;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const long long row = t / nq;
    out[t] = (double)in[row * pq + (t - row * nq)];
  }
}
template <typename T>
__global__ void dense_to_pitched(const double* __restrict__ in, int pq, int nq, long long rows, T* __restrict__ out) {
  const long long n = (long long)pq * rows;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const long long row = t / pq;
    const int i = (int)(t - row * pq);
    out[t] = i < nq ? (T)in[row * nq + i] : T(0);
  }
}


// Dense (nq-pitched) FP64 array to a pq-pitched array of T.
template <typename T>
__global__ void pad_rows(const double* in, T* out, int nq, int pq, long long npd) {
  long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p < npd) out[p % nq + (long long)pq * (p / nq)] = (T)in[p];
}

// write_seismogram (src/seismogram.f90:460-474): velocities at the stations.
template <typename T>
__global__ void station_kernel(const T* __restrict__ F, long long np, const long long* __restrict__ idx, int n,
                               double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long p = idx[i];
#pragma unroll
  for (int c = 0; c < 3; ++c) out[i * 3 + c] = (double)F[c * np + p];
}

template <typename T>
__global__ void count_nonfinite(const T* a, long long n, unsigned int* cnt) {
  long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p < n && !isfinite((double)a[p])) atomicAdd(cnt, 1u);
}

// source_time (src/moment_tensor.f90:958-1011); false for an unknown type.
bool source_time(const std::string& type, double t, double t0, double w, double& A) {
  const double pi = 3.141592653589793;
  if (type == "gaussian") A = (w / std::sqrt(2.0 * pi)) * std::exp((-(w * w) * ((t - t0) * (t - t0))) / 2.0);
  else if (type == "LOH_discontinuity") A = (t / (w * w)) * std::exp(-t / w);
  else if (type == "Brune") A = (w * w) * t * std::exp(-w * t);
  else if (type == "Cos-Bell") A = t < t0 ? (1.0 - std::cos(2.0 * pi * t / t0)) / t0 : 0.0;
  else if (type == "cosine") A = (t >= 0.0 && t <= w) ? 1.0 - std::cos(2.0 * pi * t / w) : 0.0;
  else if (type == "LOH_moment_time_history") A = 1.0 - (1.0 + t / w) * std::exp(-t / w);
  else if (type == "sine_moment_time_history") A = t <= w ? t - w / (2.0 * pi) * std::sin(2.0 * pi * t / w) : w;
  else return false;
  return true;
}

// Discrete delta weight at index i of a source at grid index i0 offset by a
// cells (singular_source, src/moment_tensor.f90:1081-1265): 5 points for
// order 2, the 9-point tables (alpha 0/25/50/100) for order 4.
double point_delta(int i, int i0, double h, double a, int order, int alpha) {
  if (order == 2) {
    const double beta = (1.0 - 2.0 * a) / 4.0 + 0.25, gam = (2.0 * a - 1.0) / 16.0, gap = (2.0 * a + 1.0) / 16.0;
    switch (i - i0) {
      case -2: return (-gam) / h;
      case -1: return (beta + 3.0 * gam - gap) / h;
      case 0: return (1.0 - a - 2.0 * beta - 3.0 * gam + 3.0 * gap) / h;
      case 1: return (a + beta + gam - 3.0 * gap) / h;
      case 2: return gap / h;
      default: return 0.0;
    }
  }
  static const double w9[4][9] = {
      {-0.01171875, -0.03125, 0.046875, 0.28125, 0.4296875, 0.28125, 0.046875, -0.03125, -0.01171875},
      {-0.00246875, -0.02275, -0.014125, 0.16575, 0.4171875, 0.38675, 0.117875, -0.02975, -0.01846875},
      {-0.00728125, -0.028, 0.014875, 0.224, 0.4265625, 0.336, 0.081375, -0.032, -0.01553125},
      {-0.0095625, -0.02990625, 0.03053125, 0.25284375, 0.42890625, 0.30903125, 0.06384375, -0.03196875,
       -0.01371875}};
  const int row = alpha == 0 ? 0 : (alpha == 25 ? 1 : (alpha == 50 ? 2 : 3));
  const int o = i - i0;
  return (o < -4 || o > 4) ? 0.0 : w9[row][o + 4] / h;
}

// Placement of one listed source in a block and its time-independent
// delta: the nearest grid point of a position inside the block's coordinate
// range (Find_Coordinates_moment, src/seismogram.f90:652-727, last point on
// ties), the block test between the first and last point's coordinates
// (src/moment_tensor.f90:304-306), and the weights of set_moment_tensor
// (local spacing h/metric at each point, src/moment_tensor.f90:1014-1078)
// or set_moment_tensor_smooth (Gaussian of width 2h, :1400-1475; evaluated
// on the points within 28 cells, beyond which the weight is below 1e-42 of
// its peak).  metric_at(p, d) gives metric_d(d) (q_x, r_y, s_z) at point p.
template <typename MetricAt>
void place_source(const BlockGrid& G, const MomentSource& m, int order, int alpha1, bool mollify,
                  MetricAt metric_at, wql_scn::MTCand& C) {
  const int nq = G.nq, nr = G.nr, ns = G.ns;
  auto X = [&](int c, int i, int j, int k) {  // 0-based
    return G.x[c][(size_t)i + (size_t)nq * ((size_t)j + (size_t)nr * k)];
  };
  const double pos[3] = {m.x, m.y, m.z};
  double lo[3], hi[3];
  for (int c = 0; c < 3; ++c) {
    lo[c] = *std::min_element(G.x[c].begin(), G.x[c].end());
    hi[c] = *std::max_element(G.x[c].begin(), G.x[c].end());
  }
  C.found = lo[0] <= pos[0] && pos[0] <= hi[0] && lo[1] <= pos[1] && pos[1] <= hi[1] && lo[2] <= pos[2] && pos[2] <= hi[2];
  C.in_box = true;
  for (int c = 0; c < 3; ++c)
    if (!(X(c, 0, 0, 0) <= pos[c] && pos[c] <= X(c, nq - 1, nr - 1, ns - 1))) C.in_box = false;
  if (!C.found) return;
  int n0[3];
  nearest_grid_point(G, pos, n0);
  const int nn[3] = {nq, nr, ns};
  const int R = mollify ? 28 : (order == 2 ? 2 : 4);
  for (int c = 0; c < 3; ++c) {
    C.lo[c] = std::max(0, n0[c] - R);
    C.dim[c] = std::min(nn[c] - 1, n0[c] + R) - C.lo[c] + 1;
  }
  const double near[3] = {X(0, n0[0], n0[1], n0[2]), X(1, n0[0], n0[1], n0[2]), X(2, n0[0], n0[1], n0[2])};
  const double hq = 1.0 / (nq - 1), hr = 1.0 / (nr - 1), hs = 1.0 / (ns - 1);
  C.delta.assign((size_t)C.dim[0] * C.dim[1] * C.dim[2], 0.0);
  size_t e = 0;
  for (int n = C.lo[2]; n < C.lo[2] + C.dim[2]; ++n)
    for (int mm = C.lo[1]; mm < C.lo[1] + C.dim[1]; ++mm)
      for (int l = C.lo[0]; l < C.lo[0] + C.dim[0]; ++l, ++e) {
        if (mollify) {
          const double pi = 3.14159265359;
          const double hx = l == 0 ? X(0, 1, mm, n) - X(0, l, mm, n) : X(0, l, mm, n) - X(0, l - 1, mm, n);
          const double hy = mm == 0 ? X(1, l, 1, n) - X(1, l, mm, n) : X(1, l, mm, n) - X(1, l, mm - 1, n);
          const double hz = n == 0 ? X(2, l, mm, 1) - X(2, l, mm, n) : X(2, l, mm, n) - X(2, l, mm, n - 1);
          const double sx = 2.0 * hx, sy = 2.0 * hy, sz = 2.0 * hz;
          const double ex = (X(0, l, mm, n) - m.x) / sx, ey = (X(1, l, mm, n) - m.y) / sy, ez = (X(2, l, mm, n) - m.z) / sz;
          const double dx = std::exp(-0.5 * (ex * ex)) / (sx * std::sqrt(2.0 * pi));
          const double dy = std::exp(-0.5 * (ey * ey)) / (sy * std::sqrt(2.0 * pi));
          const double dz = std::exp(-0.5 * (ez * ez)) / (sz * std::sqrt(2.0 * pi));
          C.delta[e] = dx * dy * dz;
        } else {
          const size_t p = (size_t)l + (size_t)nq * ((size_t)mm + (size_t)nr * n);
          const double hx = hq / metric_at(p, 0), hy = hr / metric_at(p, 1), hz = hs / metric_at(p, 2);
          const double ax = (m.x - near[0]) / hx, ay = (m.y - near[1]) / hy, az = (m.z - near[2]) / hz;
          const double dx = point_delta(l, n0[0], hx, ax, order, alpha1);
          const double dy = point_delta(mm, n0[1], hy, ay, order, alpha1);
          const double dz = point_delta(n, n0[2], hz, az, order, alpha1);
          C.delta[e] = dx * dy * dz;
        }
      }
}

int setup_block(wql_scn* S, int b) {
  const BlockParams& bp = S->P.btp[b];
  auto& B = S->B[b];
  BlockGrid G;
  std::string err;
  SurfaceMods mods;
  {
    const long long nr = bp.nqrs[1], ns = bp.nqrs[2], nq = bp.nqrs[0];
    if (S->media.fault_offset) mods.fault_offset.assign(S->media.fault_offset, S->media.fault_offset + nr * ns);
    if (S->media.topo_offset[b]) mods.topo_offset.assign(S->media.topo_offset[b], S->media.topo_offset[b] + nq * ns);
  }
  if (make_block_grid(S->P, b, mods, G, err)) return fail(WQL_E_INPUT, err);
  B.nq = G.nq;
  B.nr = G.nr;
  B.ns = G.ns;
  // resident arrays (fields, rates, coefficients) use a row pitch of a
  // multiple of 16 bytes so that every row starts on a TMA-legal address;
  // FP32 rows round to 8 points (32 bytes) so that the bfloat16
  // compensation rows (2 bytes a point) are 16-byte multiples too
  const int per16 = S->esz == 4 ? 8 : 2;
  B.pq = (G.nq + per16 - 1) / per16 * per16;
  B.npd = (long long)G.nq * G.nr * G.ns;
  B.np = (long long)B.pq * G.nr * G.ns;
  const long long np = B.npd;  // dense count for the one-time precompute below
  // geometry on the device (FP64) for the one-time precompute
  double *x = nullptr, *metric = nullptr, *J = nullptr, *mat = nullptr;
  int rc;
  if ((rc = S->alloc((void**)&x, 3 * np * sizeof(double), false))) return rc;
  for (int c = 0; c < 3; ++c)
    CK(cudaMemcpyAsync(x + c * np, G.x[c].data(), np * sizeof(double), cudaMemcpyHostToDevice, S->stream));
  if ((rc = S->alloc((void**)&metric, 9 * np * sizeof(double), false))) return rc;
  if ((rc = S->alloc((void**)&J, np * sizeof(double), false))) return rc;
  launch_metrics(B.nq, B.nr, B.ns, x, metric, J, S->stream);
  CK(cudaGetLastError());
  // material: caller arrays (the reference's file media, src/material.f90:706-747)
  // or homogeneous from rho_s_p (src/material.f90:180-187)
  if ((rc = S->alloc((void**)&mat, 3 * np * sizeof(double), false))) return rc;
  const double* user[3] = {S->media.lam[b], S->media.mu[b], S->media.rho[b]};
  if (user[0] || user[1] || user[2]) {
    if (!(user[0] && user[1] && user[2])) return fail(WQL_E_INPUT, "lam, mu and rho must be given together");
    for (int c = 0; c < 3; ++c)
      CK(cudaMemcpyAsync(mat + c * np, user[c], np * sizeof(double), cudaMemcpyHostToDevice, S->stream));
    CK(cudaStreamSynchronize(S->stream));
  } else if (S->P.material_source == "file") {
    // init_material_from_file (src/material.f90:706-747): lambda, mu, rho
    // as raw FP64 arrays, q fastest, named by btp(i)%material_path
    std::vector<double> h;
    for (int c = 0; c < 3; ++c) {
      std::string e2;
      if (bp.material_path[c].empty()) return fail(WQL_E_INPUT, "material_source = 'file' needs btp%material_path");
      if (read_f64(resolve_path(S->P.base_dir, bp.material_path[c]), (size_t)np, h, e2)) return fail(WQL_E_INPUT, e2);
      CK(cudaMemcpyAsync(mat + c * np, h.data(), np * sizeof(double), cudaMemcpyHostToDevice, S->stream));
      CK(cudaStreamSynchronize(S->stream));
    }
  } else if (S->P.material_source != "hardcode") {
    return fail(WQL_E_INPUT, "material_source '" + S->P.material_source + "' needs the media arrays");
  } else {
    const double rho = bp.rho_s_p[0], cs = bp.rho_s_p[1], cp = bp.rho_s_p[2];
    const double lam = rho * (cp * cp - 2.0 * (cs * cs)), mu = rho * (cs * cs);
    std::vector<double> h(np);
    const double vals[3] = {lam, mu, rho};
    for (int c = 0; c < 3; ++c) {
      std::fill(h.begin(), h.end(), vals[c]);
      CK(cudaMemcpyAsync(mat + c * np, h.data(), np * sizeof(double), cudaMemcpyHostToDevice, S->stream));
      CK(cudaStreamSynchronize(S->stream));
    }
  }
  // anelastic response: Q and the unrelaxed moduli before anything reads
  // the material (src/block.f90:150-151)
  if (S->anel) {
    double* qsd = nullptr;
    if ((rc = S->alloc((void**)&qsd, np * sizeof(double), false))) return rc;
    const double wref = 2.0 * 3.141592653589793 * S->P.anel.fref;
    double den[4];
    for (int l = 0; l < 4; ++l) den[l] = (wref * wref) * (S->an_tau[l] * S->an_tau[l]) + 1.0;
    launch_anelastic_material(np, S->P.anel.c, den, S->an_w, mat, mat + np, mat + 2 * np, qsd, S->stream);
    CK(cudaGetLastError());
    if ((rc = S->alloc(&B.qs, B.np * S->esz))) return rc;
    if ((rc = S->alloc(&B.eta, 24 * B.np * S->esz))) return rc;
    if ((rc = S->alloc(&B.Deta, 24 * B.np * S->esz))) return rc;
    if (S->prec == WQL_FP64)
      pad_rows<double><<<(unsigned)((np + 255) / 256), 256, 0, S->stream>>>(qsd, (double*)B.qs, B.nq, B.pq, np);
    else
      pad_rows<float><<<(unsigned)((np + 255) / 256), 256, 0, S->stream>>>(qsd, (float*)B.qs, B.nq, B.pq, np);
    CK(cudaGetLastError());
  }
  // faces
  for (int s = 0; s < 6; ++s) {
    const int axis = s / 2;
    const long long nf = axis == 0 ? (long long)B.nr * B.ns : (axis == 1 ? (long long)B.nq * B.ns : (long long)B.nq * B.nr);
    if ((rc = S->alloc((void**)&B.face[s], kFaceWords * nf * sizeof(double), false))) return rc;
  }
  launch_faces(B.nq, B.nr, B.ns, metric, mat, mat + np, mat + 2 * np, B.face, S->stream);
  CK(cudaGetLastError());
  // coefficients
  const int ncoef = S->curv ? kCurvCoef : kCartCoef;
  if ((rc = S->alloc(&B.coef, ncoef * B.np * S->esz))) return rc;
  if (S->prec == WQL_FP64)
    launch_coef<double>(B.nq, B.nr, B.ns, B.pq, S->curv, metric, J, mat, mat + np, mat + 2 * np, (double*)B.coef,
                        S->stream);
  else
    launch_coef<float>(B.nq, B.nr, B.ns, B.pq, S->curv, metric, J, mat, mat + np, mat + 2 * np, (float*)B.coef,
                       S->stream);
  CK(cudaGetLastError());
  // Cartesian diagonal metric, taken at the block centre
  {
    const long long pc = (B.nq / 2) + (long long)B.nq * ((B.nr / 2) + (long long)B.nr * (B.ns / 2));
    const int diag[3] = {0, 4, 8};  // metricx(1), metricy(2), metricz(3)
    for (int d = 0; d < 3; ++d)
      CK(cudaMemcpyAsync(&B.cart_metric[d], metric + diag[d] * np + pc, sizeof(double),
                         cudaMemcpyDeviceToHost, S->stream));
  }
  // fields
  for (int i = 0; i < 2; ++i)
    if ((rc = S->alloc(&B.F[i], 9 * B.np * S->esz))) return rc;
  if ((rc = S->alloc(&B.DF, 9 * B.np * S->esz))) return rc;
  if (S->prec == WQL_FP32C) {
    if ((rc = S->alloc(&B.C, 9 * B.np * sizeof(comp_t)))) return rc;
    const int erc = make_stencil_maps(B.maps, B.F, B.coef, B.DF, B.C, B.nq, B.nr, B.ns, B.pq, S->curv, S->fd,
                                      tma_tile_width(S->P.btp[0].nqrs[0], S->P.btp[1].nqrs[0], S->curv));
    if (erc) return fail(WQL_E_CUDA, "cuTensorMapEncodeTiled failed for the stencil maps (error " + std::to_string(erc) + ")");
  }
  // boundary codes (src/BoundaryConditions.f90:15-48) and PML slabs (src/block.f90:163-178)
  B.bc[0] = bp.lqrs[0]; B.bc[1] = bp.rqrs[0];
  B.bc[2] = bp.lqrs[1]; B.bc[3] = bp.rqrs[1];
  B.bc[4] = bp.lqrs[2]; B.bc[5] = bp.rqrs[2];
  B.npml = 0;
  for (int s = 0; s < 6; ++s) {
    B.pml[s] = (s % 2 == 0) ? bp.pml_lqrs[s / 2] : bp.pml_rqrs[s / 2];
    if (B.pml[s]) B.npml = bp.npml;
  }
  if (B.npml > 0) {
    const int dims[3] = {B.nq, B.nr, B.ns};
    for (int s = 0; s < 6; ++s) {
      if (!B.pml[s]) continue;
      if (B.npml >= dims[s / 2]) return fail(WQL_E_INPUT, "npml exceeds the block size");
      long long slab = np / dims[s / 2] * B.npml;
      B.slab_np[s] = slab;
      if ((rc = S->alloc(&B.Q[s], 9 * slab * S->esz))) return rc;
      if ((rc = S->alloc(&B.DQ[s], 9 * slab * S->esz))) return rc;
    }
    if (S->prec == WQL_FP32C && !S->anel && (rc = S->alloc(&B.G, 9 * B.np * S->esz))) return rc;
  }
  // anelastic: the TMA stencil hands the velocity gradient of every point
  // to the anelastic kernel
  if (S->prec == WQL_FP32C && S->anel && (rc = S->alloc(&B.G, 9 * B.np * S->esz))) return rc;
  // src/block.f90:189-214
  const double tau0 = S->fd == 1 ? kTau0Upwind6
                      : (S->fd == 2 ? kTau0Upwind5 : (S->fd == 3 ? S->ut->tau0 : 1.0 / (0.315949074074074)));
  const int dims[3] = {B.nq, B.nr, B.ns};
  for (int d = 0; d < 3; ++d) B.tau_h[d] = tau0 / (1.0 / (double)(dims[d] - 1));
  // manufactured solution: shapes, forcing shapes and the initial fields
  if (S->mms) {
    if ((rc = S->alloc(&B.ms, 2 * B.np * S->esz))) return rc;
    if ((rc = S->alloc(&B.mp, 9 * B.np * S->esz))) return rc;
    const double pi = 3.141592653589793;
    const MmsWave w{S->P.mms_nx * pi, S->P.mms_ny * pi, S->P.mms_nz * pi};
    launch_mms_setup(B.nq, B.nr, B.ns, B.pq, w, x, mat, mat + np, mat + 2 * np, S->prec == WQL_FP64, B.ms, B.mp,
                     B.F[S->cur], S->stream);
    CK(cudaGetLastError());
  }
  // depth coordinate for the plastic update; plastic_flow's per-point
  // plastic strain rate and strain, zero at the start
  // (src/plastic_material.f90:38-44)
  if (S->pl_flow) {
    if ((rc = S->alloc(&B.pl_lambda, B.np * S->esz))) return rc;
    if ((rc = S->alloc(&B.pl_gammap, B.np * S->esz))) return rc;
  }
  if (S->plastic) {
    if ((rc = S->alloc(&B.y, B.np * S->esz))) return rc;
    if (S->prec == WQL_FP64)
      pad_rows<double><<<(unsigned)((np + 255) / 256), 256, 0, S->stream>>>(x + np, (double*)B.y, B.nq, B.pq, np);
    else
      pad_rows<float><<<(unsigned)((np + 255) / 256), 256, 0, S->stream>>>(x + np, (float*)B.y, B.nq, B.pq, np);
  }
  // seismogram stations: nearest grid points, as pitched offsets
  if (S->P.output_seismograms) {
    const std::vector<double>& req = !S->P.stations.empty() ? S->P.stations : (b == 0 ? S->P.stationsU : S->P.stationsV);
    auto& T = S->st[b];
    std::vector<int> which;
    find_station_points(G, req, T.ijk, &which);
    for (int w : which) T.xyz.insert(T.xyz.end(), req.begin() + 3 * w, req.begin() + 3 * w + 3);
    const int n = (int)T.ijk.size() / 3;
    if (n > 0) {
      std::vector<long long> off(n);
      for (int i = 0; i < n; ++i)
        off[i] = (T.ijk[3 * i] - 1) + (long long)B.pq * ((T.ijk[3 * i + 1] - 1) + (long long)B.nr * (T.ijk[3 * i + 2] - 1));
      if ((rc = S->alloc((void**)&T.idx_dev, n * sizeof(long long), false))) return rc;
      CK(cudaMemcpy(T.idx_dev, off.data(), n * sizeof(long long), cudaMemcpyHostToDevice));
      if ((rc = S->alloc((void**)&T.ring, (size_t)S->st_cap * n * 3 * sizeof(double)))) return rc;
    }
  }
  // interface coordinates of this block's fault face
  {
    const long long nf = (long long)B.nr * B.ns;
    std::vector<double> xi(3 * nf);
    const int iq = (b == 0) ? B.nq - 1 : 0;
    for (int k = 0; k < B.ns; ++k)
      for (int j = 0; j < B.nr; ++j) {
        const long long p = iq + (long long)B.nq * (j + (long long)B.nr * k);
        for (int c = 0; c < 3; ++c) xi[c * nf + j + (long long)B.nr * k] = G.x[c][p];
      }
    CK(cudaMemcpyAsync(S->xij + (long long)b * 3 * nf, xi.data(), 3 * nf * sizeof(double),
                       cudaMemcpyHostToDevice, S->stream));
    CK(cudaStreamSynchronize(S->stream));
  }
  // moment-tensor sources: placement and delta of every listed source
  if (S->P.use_moment_tensor) {
    const Problem& Pr = S->P;
    // q_x, r_y, s_z on the host (the discrete delta uses the local spacing
    // h/metric at each point of its support)
    std::vector<double> diag[3];
    if (!Pr.mollify_source) {
      const int di[3] = {0, 4, 8};
      for (int d = 0; d < 3; ++d) {
        diag[d].resize(np);
        CK(cudaMemcpy(diag[d].data(), metric + (size_t)di[d] * np, np * sizeof(double), cudaMemcpyDeviceToHost));
      }
    }
    auto metric_at = [&](size_t p, int d) { return diag[d][p]; };
    const std::vector<MomentSource>& own = b == 0 ? Pr.tensorsU : Pr.tensorsV;
    const std::vector<MomentSource>* lists[2] = {&Pr.tensors, &own};
    for (int li = 0; li < 2; ++li) {
      const auto& L = *lists[li];
      const int alpha1 = L.empty() ? 0 : L[0].alpha;
      S->mt_cand[b][li].resize(L.size());
      for (size_t i = 0; i < L.size(); ++i)
        place_source(G, L[i], Pr.mt_order, alpha1, Pr.mollify_source, metric_at, S->mt_cand[b][li][i]);
    }
  }
  CK(cudaStreamSynchronize(S->stream));
  S->release(x);
  S->release(metric);
  S->release(J);
  S->release(mat);
  return WQL_OK;
}

// Per fault point and block copy, the parts of the interface condition that
// do not change in time: the static prestress in the copy's (n, m, l) frame,
// the nucleation weight (prestress(t) = static + weight * ramp(t)) and the
// rate-and-state direct-effect parameter a(x).
int precompute_fault(wql_scn* S) {
  const long long nf = (long long)S->B[0].nr * S->B[0].ns;
  std::vector<double> pre(2 * 5 * nf, 0.0);
  for (int b = 0; b < 2; ++b) {
    auto& B = S->B[b];
    const int side = (b == 0) ? 1 : 0;
    std::vector<double> face(kFaceWords * nf), xi(3 * nf);
    CK(cudaMemcpy(face.data(), B.face[side], face.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(xi.data(), S->xij + (long long)b * 3 * nf, xi.size() * sizeof(double), cudaMemcpyDeviceToHost));
    double* P = pre.data() + (long long)b * 5 * nf;
    for (long long f = 0; f < nf; ++f) {
      double n[3], m[3], l[3], x[3];
      for (int c = 0; c < 3; ++c) {
        n[c] = face[(0 + c) * nf + f];
        m[c] = face[(3 + c) * nf + f];
        l[c] = face[(6 + c) * nf + f];
        x[c] = xi[c * nf + f];
      }
      prestress_static(S->fp, x, l, m, n, P[f], P[nf + f], P[2 * nf + f]);
      P[3 * nf + f] = nucleation_weight(S->fp, x, P[f]);
      P[4 * nf + f] = S->fp.coupling == CPL_RS ? rs_direct_a(S->fp, x) : 0.0;
    }
  }
  int rc;
  if ((rc = S->alloc((void**)&S->pre, pre.size() * sizeof(double), false))) return rc;
  CK(cudaMemcpy(S->pre, pre.data(), pre.size() * sizeof(double), cudaMemcpyHostToDevice));
  return WQL_OK;
}

// Init_Vel_State (src/Interface_Condition.f90:2722-2850) for each block copy.
int init_rate_state(wql_scn* S) {
  const long long nf = (long long)S->B[0].nr * S->B[0].ns;
  // 'rate-weakening' starts at rest with a uniform state 0.4367
  // (src/Interface_Condition.f90:2819-2843)
  const bool rw = S->fp.preset == PRE_RATE_WEAKENING;
  const double Vin = (S->fp.preset == PRE_RS_PARAM) ? S->fp.Vini : (rw ? 0.0 : 1.0e-12);
  std::vector<double> W(2 * nf);
  for (int b = 0; b < 2; ++b) {
    auto& B = S->B[b];
    const int side = (b == 0) ? 1 : 0;
    std::vector<double> face(kFaceWords * nf), xi(3 * nf);
    CK(cudaMemcpy(face.data(), B.face[side], face.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(xi.data(), S->xij + (long long)b * 3 * nf, xi.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (long long f = 0; f < nf; ++f) {
      double n[3], m[3], l[3], x[3];
      for (int c = 0; c < 3; ++c) {
        n[c] = face[(0 + c) * nf + f];
        m[c] = face[(3 + c) * nf + f];
        l[c] = face[(6 + c) * nf + f];
        x[c] = xi[c * nf + f];
      }
      if (rw) {
        W[b * nf + f] = 0.4367;
        continue;
      }
      double Tn, Tm, Tl;
      prestress(S->fp, x, 0.0, l, m, n, Tn, Tm, Tl);
      const RSParams r = rs_params(S->fp, x);
      const double sn = -Tn;
      const double theta =
          r.L0 / r.V0 * std::exp(((r.a * std::log(2.0 * std::sinh(Tl / (r.a * sn)))) - r.f0 - r.a * std::log(Vin / r.V0)) / r.b);
      W[b * nf + f] = r.f0 + r.b * std::log(r.V0 / r.L0 * theta);
    }
    // uniform initial slip velocity split across the fault: -/+ Vin/2 in z
    const double vz = (b == 0 ? -1.0 : 1.0) * std::fabs(0.5 * Vin);
    const long long np = B.np;
    for (int i = 0; i < 2; ++i) {
      if (S->prec == WQL_FP64)
        fill_comp<double><<<(unsigned)((np + 255) / 256), 256, 0, S->stream>>>((double*)B.F[i], np, 2, vz);
      else
        fill_comp<float><<<(unsigned)((np + 255) / 256), 256, 0, S->stream>>>((float*)B.F[i], np, 2, (float)vz);
    }
    CK(cudaGetLastError());
  }
  CK(cudaMemcpy(S->W, W.data(), W.size() * sizeof(double), cudaMemcpyHostToDevice));
  return WQL_OK;
}

int create(wql_ctx* ctx, Problem&& P, int precision, const wql_media* media, wql_scn** out) {
  if (!ctx || !out) return fail(WQL_E_INPUT, "null argument");
  if (precision != WQL_FP64 && precision != WQL_FP32C) return fail(WQL_E_INPUT, "unknown precision");
  std::unique_ptr<wql_scn> S(new wql_scn());
  S->ctx = ctx;
  S->P = std::move(P);
  if (media) S->media = *media;
  S->prec = precision;
  S->esz = precision == WQL_FP64 ? 8 : 4;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
  const Problem& Pr = S->P;
  // src/RHS_Interior.f90:31-125: the traditional SBP-6 operator, the upwind
  // operators of orders 2..9 or the upwind DRP operators of orders 3..7, 66
  // and 679 (the ones other than upwind 5 and 6 from wql_upwind_tables.h)
  if (Pr.fd_type == "upwind" && Pr.order == 6) S->fd = 1;
  else if (Pr.fd_type == "upwind" && Pr.order == 5) S->fd = 2;
  else if (Pr.fd_type != "traditional") {
    for (int k = 0; k < kUpwindTableCount; ++k)
      if (Pr.fd_type == kUpwindTable[k].fd_type && Pr.order == kUpwindTable[k].order) S->ut = &kUpwindTable[k];
    if (!S->ut)
      return fail(WQL_E_INPUT, "fd_type '" + Pr.fd_type + "' with order " + std::to_string(Pr.order) +
                                   " is not supported (traditional; upwind with order 2..9; upwind_drp with order "
                                   "3..7, 66 or 679)");
    S->fd = 3;
    // every row must fit in the block: the closure rows reach at most point
    // 13, the interior rows R points either side
    int reach = 2 * S->ut->R + 1;
    const double* rows[4] = {&S->ut->lp[0][0][0], &S->ut->lm[0][0][0], &S->ut->rp[0][0][0], &S->ut->rm[0][0][0]};
    for (const double* r : rows)
      for (int e = 0; e < kUgRowBlock; ++e)
        if (r[e] != 0.0) reach = std::max(reach, e % kUgCol + 1);
    for (int b = 0; b < 2; ++b)
      for (int d = 0; d < 3; ++d)
        if (Pr.btp[b].nqrs[d] < reach)
          return fail(WQL_E_INPUT, "fd_type '" + Pr.fd_type + "' with order " + std::to_string(Pr.order) +
                                       " needs at least " + std::to_string(reach) + " points per axis");
    std::vector<double> w(kUgWords, 0.0);
    std::copy(S->ut->ip, S->ut->ip + kUgCol, w.begin());
    std::copy(S->ut->im, S->ut->im + kUgCol, w.begin() + kUgCol);
    std::copy(S->ut->bp, S->ut->bp + kUgCol, w.begin() + 2 * kUgCol);
    std::copy(S->ut->bm, S->ut->bm + kUgCol, w.begin() + 3 * kUgCol);
    for (int q = 0; q < 4; ++q) std::copy(rows[q], rows[q] + kUgRowBlock, w.begin() + 4 * kUgCol + q * kUgRowBlock);
    int rc;
    if ((rc = S->alloc(&S->ug_dev, kUgWords * S->esz, false))) return rc;
    if (precision == WQL_FP64) {
      CK(cudaMemcpy(S->ug_dev, w.data(), kUgWords * sizeof(double), cudaMemcpyHostToDevice));
    } else {
      std::vector<float> wf(w.begin(), w.end());
      CK(cudaMemcpy(S->ug_dev, wf.data(), kUgWords * sizeof(float), cudaMemcpyHostToDevice));
    }
  }
  if (Pr.response == "anelastic") {
    // init_anelastic_properties (src/material.f90:85-115): relaxation times
    // and weights exist for weight_exp 0 and 0.6 only
    const double we = Pr.anel.weight_exp;
    const bool w0 = we < 0.01, w6 = we > 0.59 && we < 0.61;
    if (!w0 && !w6) return fail(WQL_E_INPUT, "anelastic weight_exp must be 0 or 0.6");
    const double pi = 3.141592653589793, FAC = 1.0;
    const double taumin = 1.0 / (2.0 * pi * 15.0) * 1.0 * FAC;
    const double taumax = 1.0 / (2.0 * pi * 0.08) * 200.0 * FAC;
    const double wa[4] = {1.6126, 0.6255, 0.6382, 1.5969}, wb[4] = {0.0336, 0.6873, 0.8767, 1.5202};
    for (int k = 1; k <= 4; ++k) {
      S->an_tau[k - 1] = std::exp(std::log(taumin) + (2.0 * k - 1.0) / 16.0 * (std::log(taumax) - std::log(taumin)));
      S->an_w[k - 1] = w0 ? wa[k - 1] : wb[k - 1];
    }
    S->anel = true;
  }
  if (Pr.use_moment_tensor) {
    if (Pr.mt_order != 2 && Pr.mt_order != 4) return fail(WQL_E_INPUT, "moment_list order must be 2 or 4");
    for (const auto* L : {&Pr.tensors, &Pr.tensorsU, &Pr.tensorsV}) {
      for (const auto& m : *L) {
        double A;
        if (!source_time(m.type, 0.0, m.t_init, m.duration, A))
          return fail(WQL_E_INPUT, "invalid source type '" + m.type + "' (src/moment_tensor.f90:970)");
      }
      if (Pr.mt_order == 4 && !L->empty()) {
        const int a = (*L)[0].alpha;
        if (a != 0 && a != 25 && a != 50 && a != 100)
          return fail(WQL_E_INPUT, "order-4 sources need alpha 0, 25, 50 or 100 (src/moment_tensor.f90:1129-1262)");
      }
    }
  }
  S->curv = Pr.type_of_mesh == "curvilinear";
  S->bc_form = Pr.bc_penalty == "weighted" ? BC_WEIGHTED : BC_CHARACTERISTIC;
  S->rs_tol = Pr.rs_tol;
  S->rs_maxit = Pr.rs_maxit;
  S->fault_comp = Pr.fp32c_fault == "compensated";
  S->mms = Pr.use_mms;
  if (S->mms) {
    // the manufactured solution is smooth across the fault: a locked
    // interface, an elastic medium, no PML and no point sources
    bool pml = false;
    for (int b = 0; b < 2; ++b)
      for (int d = 0; d < 3; ++d) pml = pml || Pr.btp[b].pml_lqrs[d] || Pr.btp[b].pml_rqrs[d];
    if (Pr.coupling != "locked" || Pr.response != "elastic" || pml || Pr.use_moment_tensor)
      return fail(WQL_E_INPUT, "use_mms needs coupling='locked', response='elastic', no PML and no sources");
    S->mms_kt = Pr.mms_nt * 3.141592653589793;
  }
  S->plastic = Pr.response == "plastic";
  S->pl_flow = S->plastic && Pr.plastic_model != "scec";
  // plastic_flow reads mu_beta_eta, which init_plastic_material sets only for
  // problem 'rate-weakening' (src/plastic_material.f90:38-42); elsewhere the
  // reference leaves it undefined
  if (S->pl_flow && Pr.problem != "rate-weakening")
    return fail(WQL_E_INPUT, "plastic_model '" + Pr.plastic_model +
                                 "' (plastic_flow) needs problem 'rate-weakening', the only one that sets mu_beta_eta");
  if (Pr.plast.set) {
    S->pl_c = Pr.plast.cohesion;
    S->pl_nu = Pr.plast.friction;
    S->pl_Tv = Pr.plast.Tv;
  } else if (Pr.problem == "TPV30") {
    S->pl_c = 1.18; S->pl_nu = 0.1680; S->pl_Tv = 0.05;  // src/plastic.f90:178-182
  }
  // coupling and friction preset
  FaultParams& fp = S->fp;
  std::memset(&fp, 0, sizeof(fp));
  const std::string& cp = Pr.coupling;
  if (cp == "locked") fp.coupling = CPL_LOCKED;
  else if (cp == "linear_friction") fp.coupling = CPL_LINEAR;
  else if (cp == "slip-weakening_friction") fp.coupling = CPL_SW;
  else if (cp == "rate-and-state_friction") fp.coupling = CPL_RS;
  else return fail(WQL_E_INPUT, "invalid coupling condition '" + cp + "'");
  fp.preset = preset_of(Pr.problem);
  if (fp.preset == PRE_TPV28 && Pr.tpv28_prestress == "benchmark") fp.preset = PRE_TPV28_BENCH;
  const bool sw_ok = fp.preset == PRE_TPV5 || fp.preset == PRE_TPV26 || fp.preset == PRE_TPV27 ||
                     fp.preset == PRE_TPV28 || fp.preset == PRE_TPV28_BENCH || fp.preset == PRE_TPV29 || fp.preset == PRE_TPV30 ||
                     fp.preset == PRE_TPV10 || fp.preset == PRE_SW_PARAM;
  const bool rs_ok = fp.preset == PRE_TPV101 || fp.preset == PRE_TPV102 || fp.preset == PRE_RS_PARAM ||
                     fp.preset == PRE_RATE_WEAKENING;
  if ((fp.coupling == CPL_SW && !sw_ok) || (fp.coupling == CPL_RS && !rs_ok))
    return fail(WQL_E_INPUT, "problem '" + Pr.problem + "' has no preset for coupling '" + cp + "'");
  const FrictionExt& fe = Pr.fric;
  fp.fs = fe.fs; fp.fd = fe.fd; fp.Dc = fe.Dc; fp.barrier_y = fe.barrier_y; fp.barrier_z = fe.barrier_z;
  fp.a = fe.a; fp.b = fe.b; fp.V0 = fe.V0; fp.f0 = fe.f0; fp.L = fe.L; fp.Vini = fe.Vini;
  for (int c = 0; c < 6; ++c) fp.s0[c] = fe.s0[c];
  fp.s0_profile = fe.stress_profile.empty() ? PRE_NONE : preset_of(fe.stress_profile);
  if (!fe.stress_profile.empty() && fp.s0_profile == PRE_NONE)
    return fail(WQL_E_INPUT, "unknown stress_profile '" + fe.stress_profile + "'");
  fp.nuc_amp = fe.nuc_amp; fp.nuc_radius = fe.nuc_radius;
  fp.nuc_y = fe.nuc_y; fp.nuc_z = fe.nuc_z; fp.nuc_rise = fe.nuc_rise;
  if (S->plastic && fp.preset != PRE_SW_PARAM && fp.preset != PRE_RS_PARAM) {
    double s0[6], x0[3] = {0, 0, 0};
    if (!initial_stress(fp.preset, x0, s0))
      return fail(WQL_E_INPUT, "problem '" + Pr.problem + "' has no initial stress tensor for plasticity");
  }
  // the two blocks share the fault face (src/domain.f90:243-244, 518-530)
  if (Pr.btp[0].nqrs[1] != Pr.btp[1].nqrs[1] || Pr.btp[0].nqrs[2] != Pr.btp[1].nqrs[2])
    return fail(WQL_E_INPUT, "the two blocks must share the fault face (equal nr, ns)");
  const long long nf = (long long)Pr.btp[0].nqrs[1] * Pr.btp[0].nqrs[2];
  int rc;
  if ((rc = S->alloc((void**)&S->xij, 2 * 3 * nf * sizeof(double)))) return rc;
  S->st_cap = station_ring_cap(Pr);
  for (int b = 0; b < 2; ++b)
    if ((rc = setup_block(S.get(), b))) return rc;
  // moment-tensor sources: the unified list goes to the preferred block when
  // the source lies in its box, else to the other block when it lies in
  // that one; per-block lists stay with their block; a source in no block is
  // not applied (the reference keeps it at grid index -1, where its discrete
  // delta still reaches the block's corner points 1..3 of each axis,
  // src/moment_tensor.f90:318-345 -- not reproduced here)
  if (Pr.use_moment_tensor) {
    auto take = [&](int b, const MomentSource& m, const wql_scn::MTCand& C) -> int {
      if (!C.found) return WQL_OK;
      wql_scn::MTSrc T;
      T.src = m;
      for (int c = 0; c < 3; ++c) {
        T.lo[c] = C.lo[c];
        T.dim[c] = C.dim[c];
      }
      int r2;
      if ((r2 = S->alloc((void**)&T.delta, C.delta.size() * sizeof(double), false))) return r2;
      CK(cudaMemcpy(T.delta, C.delta.data(), C.delta.size() * sizeof(double), cudaMemcpyHostToDevice));
      S->mt[b].push_back(T);
      return WQL_OK;
    };
    if (Pr.mt_unified) {
      const int pref = Pr.mt_block_preference == 2 ? 1 : 0;
      for (size_t i = 0; i < Pr.tensors.size(); ++i) {
        int b = -1;
        if (S->mt_cand[pref][0][i].in_box) b = pref;
        else if (S->mt_cand[1 - pref][0][i].in_box) b = 1 - pref;
        if (b >= 0 && (rc = take(b, Pr.tensors[i], S->mt_cand[b][0][i]))) return rc;
      }
    } else {
      for (int b = 0; b < 2; ++b) {
        const auto& L = b == 0 ? Pr.tensorsU : Pr.tensorsV;
        for (size_t i = 0; i < L.size(); ++i)
          if (S->mt_cand[b][1][i].in_box && (rc = take(b, L[i], S->mt_cand[b][1][i]))) return rc;
      }
    }
    for (int b = 0; b < 2; ++b)
      for (int li = 0; li < 2; ++li) S->mt_cand[b][li].clear();
  }
  if ((rc = S->alloc((void**)&S->S, 2 * 4 * nf * sizeof(double)))) return rc;
  if ((rc = S->alloc((void**)&S->DS, 2 * 4 * nf * sizeof(double)))) return rc;
  if ((rc = S->alloc((void**)&S->W, 2 * nf * sizeof(double)))) return rc;
  if ((rc = S->alloc((void**)&S->DW, 2 * nf * sizeof(double)))) return rc;
  if ((rc = S->alloc((void**)&S->trup, 2 * nf * sizeof(double), false))) return rc;
  {
    std::vector<double> t9(2 * nf, 1.0e9);  // src/iface.f90:41
    CK(cudaMemcpy(S->trup, t9.data(), t9.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  if ((rc = S->alloc(&S->sat, 2 * 9 * nf * S->esz))) return rc;
  if ((rc = S->alloc((void**)&S->solver_fail, sizeof(unsigned int)))) return rc;
  if ((rc = S->alloc((void**)&S->err_dev, sizeof(int)))) return rc;
  if (S->mms && (rc = S->alloc((void**)&S->mms_acc, 18 * sizeof(double)))) return rc;
  if (fp.coupling == CPL_SW || fp.coupling == CPL_RS)
    if ((rc = precompute_fault(S.get()))) return rc;
  if (fp.coupling == CPL_RS)
    if ((rc = init_rate_state(S.get()))) return rc;
  if (Pr.w_fault) {
    S->frame_cap = frame_ring_cap(nf);
    const size_t ring_bytes = (size_t)S->frame_cap * kFrameWords * nf * sizeof(float);
    for (int k = 0; k < 2; ++k)
      if ((rc = S->alloc((void**)&S->frame_ring[k], ring_bytes))) return rc;
    S->frame_dev = S->frame_ring[0];
    // pinned staging for the overlapped copies; without it every full ring
    // is copied synchronously
    if (cudaMallocHost((void**)&S->frame_pin, ring_bytes) != cudaSuccess ||
        cudaEventCreateWithFlags(&S->pin_done, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      if (S->frame_pin) cudaFreeHost(S->frame_pin);
      S->frame_pin = nullptr;
    }
  }
  // time step: src/domain.f90:222-235, src/block.f90:437-452
  double dtmin = 1e300;
  for (int b = 0; b < 2; ++b) {
    const BlockParams& bp = Pr.btp[b];
    double h = 1e300;
    for (int d = 0; d < 3; ++d) h = std::fmin(h, (bp.bqrs[d] - bp.aqrs[d]) / (double)(bp.nqrs[d] - 1));
    dtmin = std::fmin(dtmin, Pr.CFL * h / std::sqrt(bp.rho_s_p[1] * bp.rho_s_p[1] + bp.rho_s_p[2] * bp.rho_s_p[2]));
  }
  S->dt = dtmin;
  S->nt = (int)std::floor(Pr.t_final / dtmin);
  CK(cudaStreamSynchronize(S->stream));
  CK(cudaGetLastError());
  *out = S.release();
  return WQL_OK;
}

int flush_stations(wql_scn* S) {
  if (S->st_fill == 0) return WQL_OK;
  for (int b = 0; b < 2; ++b) {
    auto& T = S->st[b];
    const int n = (int)T.ijk.size() / 3;
    if (n == 0) continue;
    std::vector<double> tmp((size_t)S->st_fill * n * 3);
    CK(cudaMemcpyAsync(tmp.data(), T.ring, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost, S->stream));
    CK(cudaStreamSynchronize(S->stream));
    for (int r = 0; r < S->st_fill; ++r)
      for (int i = 0; i < n; ++i) {
        T.host.push_back(S->st_times[r]);
        for (int c = 0; c < 3; ++c) T.host.push_back(tmp[((size_t)r * n + i) * 3 + c]);
      }
  }
  S->st_fill = 0;
  S->st_times.clear();
  return WQL_OK;
}

// Appends the frames of the pinned staging buffer to the host chunks, after
// their copy has completed.
int drain_pinned(wql_scn* S) {
  if (S->pin_frames == 0) return WQL_OK;
  CK(cudaEventSynchronize(S->pin_done));
  const size_t words = (size_t)S->pin_frames * kFrameWords * S->B[0].nr * S->B[0].ns;
  S->frame_chunks.emplace_back(S->frame_pin, S->frame_pin + words);
  S->pin_frames = 0;
  return WQL_OK;
}

// Every frame to the host (before a read or the output files).
int flush_frames(wql_scn* S) {
  int rc = flush_stations(S);
  if (rc) return rc;
  if ((rc = drain_pinned(S))) return rc;
  if (S->frame_fill == 0) return WQL_OK;
  const long long nf = (long long)S->B[0].nr * S->B[0].ns;
  const size_t words = (size_t)S->frame_fill * kFrameWords * nf;
  S->frame_chunks.emplace_back(words);
  CK(cudaMemcpyAsync(S->frame_chunks.back().data(), S->frame_dev, words * sizeof(float), cudaMemcpyDeviceToHost,
                     S->stream));
  CK(cudaStreamSynchronize(S->stream));
  S->frame_fill = 0;
  return WQL_OK;
}

// The ring being filled is full: queue its copy to the pinned buffer (once
// the previous copy has been taken out of it) and switch rings.  Kernels
// that write the other ring later are queued after its own copy.
int rotate_frames(wql_scn* S) {
  if (!S->frame_pin) return flush_frames(S);
  int rc = drain_pinned(S);
  if (rc) return rc;
  const size_t words = (size_t)S->frame_fill * kFrameWords * S->B[0].nr * S->B[0].ns;
  CK(cudaMemcpyAsync(S->frame_pin, S->frame_dev, words * sizeof(float), cudaMemcpyDeviceToHost, S->stream));
  CK(cudaEventRecord(S->pin_done, S->stream));
  S->pin_frames = S->frame_fill;
  S->ring_cur ^= 1;
  S->frame_dev = S->frame_ring[S->ring_cur];
  S->frame_fill = 0;
  return WQL_OK;
}

template <typename T>
VolumeArgs<T> volume_args(wql_scn* S, int b, double A, double Bdt, bool last) {
  auto& B = S->B[b];
  VolumeArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.nq = B.nq; a.nr = B.nr; a.ns = B.ns; a.pq = B.pq; a.np = B.np; a.block = b;
  a.rh[0] = (T)(B.nq - 1); a.rh[1] = (T)(B.nr - 1); a.rh[2] = (T)(B.ns - 1);
  a.Fin = (const T*)B.F[S->cur];
  a.Fout = (T*)B.F[S->cur ^ 1];
  a.DF = (T*)B.DF;
  a.C = (comp_t*)B.C;
  a.coef = (const T*)B.coef;
  for (int d = 0; d < 3; ++d) {
    a.cart_metric[d] = (T)B.cart_metric[d];
    a.tau_h[d] = (T)B.tau_h[d];
  }
  for (int s = 0; s < 6; ++s) {
    a.face[s] = B.face[s];
    a.bc[s] = B.bc[s];
    a.pml[s] = B.pml[s];
    a.Q[s] = (T*)B.Q[s];
    a.DQ[s] = (T*)B.DQ[s];
    a.slab_np[s] = B.slab_np[s];
  }
  a.G = (T*)B.G;  // used only when the block's stencil is the TMA kernel
  a.bc_form = S->bc_form;
  a.kernel = S->kernel_variant;
  a.fd = S->fd;
  if (S->ut) a.ug = UpG{S->ug_dev, S->ut->R, S->ut->plo, S->ut->pn, S->ut->mlo, S->ut->mn};
  a.schunk = S->schunk;
  a.fault_sat = (const T*)S->sat + (long long)b * 9 * B.nr * B.ns;
  a.npml = B.npml;
  a.A = (T)A;
  a.Bdt = (T)Bdt;
  a.plastic = (S->plastic && last) ? 1 : 0;
  a.preset = S->fp.preset;
  if (S->fp.preset == PRE_SW_PARAM || S->fp.preset == PRE_RS_PARAM) a.preset = S->fp.s0_profile;
  for (int c = 0; c < 6; ++c) a.s0u[c] = S->fp.s0[c];
  a.ycoord = (const T*)B.y;
  a.pl_c = S->pl_c; a.pl_nu = S->pl_nu; a.pl_Tv = S->pl_Tv; a.dt = S->dt;
  a.pl_ccos = S->pl_c * std::cos(std::atan(S->pl_nu));
  a.pl_sin = std::sin(std::atan(S->pl_nu));
  a.pl_decay = std::exp(-S->dt / S->pl_Tv);
  a.pl_flow = S->pl_flow ? 1 : 0;
  a.pl_mu = S->P.btp[b].mu_beta_eta[0];
  a.pl_beta = S->P.btp[b].mu_beta_eta[1];
  a.pl_eta = S->P.btp[b].mu_beta_eta[2];
  a.pl_lambda = (T*)B.pl_lambda;
  a.pl_gammap = (T*)B.pl_gammap;
  a.err = S->err_dev;
  a.anel = S->anel ? 1 : 0;
  a.eta = (T*)B.eta;
  a.Deta = (T*)B.Deta;
  a.qsinv = (const T*)B.qs;
  for (int m = 0; m < 4; ++m) {
    a.an_tau[m] = S->an_tau[m];
    a.an_w[m] = S->an_w[m];
  }
  a.pml_d0 = 6.0 / (2.0 * 1.0) * std::log(1.0 / 1.0e-3);
  a.ms = (const T*)B.ms;
  a.mp = (const T*)B.mp;
  a.mms_T = (T)S->mms_T;
  a.mms_Tp = (T)S->mms_Tp;
  B.maps.cur = S->cur;
  a.tma = &B.maps;
  return a;
}

// One time step split into phases so that a batch can interleave the
// phases of many scenarios: per stage the interface kernel (and the stage-1
// station gather), per block the face pre-kernel, the stencil, then the
// sources and correction kernels.  run_step strings them together for one
// scenario.
struct StepCtx {
  bool want_frame = false, want_station = false;
  double t0 = 0.0;
  int launches = 0;
};

StepCtx step_begin(wql_scn* S) {
  StepCtx c;
  c.want_frame = S->frame_dev && (S->nstep % std::max(S->P.w_stride, 1) == 0);
  c.want_station = S->P.output_seismograms && (S->st[0].ijk.size() + S->st[1].ijk.size() > 0) &&
                   (S->nstep % std::max(S->P.w_stride, 1) == 0);
  c.t0 = S->t;
  return c;
}

double stage_A(const wql_scn* S, int stage) { return S->rk.A[stage]; }
double stage_Bdt(const wql_scn* S, int stage) { return S->rk.B[stage] * S->dt; }
double stage_time(const wql_scn* S, const StepCtx& c, int stage) { return c.t0 + S->rk.C[stage - 1] * S->dt; }

void mark_begin(wql_scn* S, int kind) {
  if (!S->profiling) return;
  S->ev_marks.push_back({S->ev_used, kind});
  cudaEventRecord(S->next_event(), S->stream);
}
void mark_end(wql_scn* S) {
  if (S->profiling) cudaEventRecord(S->next_event(), S->stream);
}

void stage_head(wql_scn* S, StepCtx& c, int stage) {
  const long long nf = (long long)S->B[0].nr * S->B[0].ns;
  const double ts = stage_time(S, c, stage);
  InterfaceArgs ia;
  std::memset(&ia, 0, sizeof(ia));
  ia.nr = S->B[0].nr; ia.ns = S->B[0].ns;
  ia.np0 = S->B[0].np; ia.np1 = S->B[1].np; ia.nq0 = S->B[0].nq;
  ia.pq0 = S->B[0].pq; ia.pq1 = S->B[1].pq;
  ia.fp64 = S->prec == WQL_FP64;
  ia.F0 = S->B[0].F[S->cur];
  ia.F1 = S->B[1].F[S->cur];
  ia.face0 = S->B[0].face[1];
  ia.face1 = S->B[1].face[0];
  ia.xij = S->xij;
  ia.S = S->S; ia.DS = S->DS; ia.W = S->W; ia.DW = S->DW; ia.trup = S->trup;
  ia.sat = S->sat;
  ia.tau_h[0] = S->B[0].tau_h[0];
  ia.tau_h[1] = S->B[1].tau_h[0];
  ia.A = stage_A(S, stage); ia.Bdt = stage_Bdt(S, stage); ia.t = ts; ia.stage = stage;
  ia.pre = S->pre;
  ia.ramp = nucleation_ramp(S->fp, ts);
  {
    const double x0[3] = {0.0, 0.0, 0.0};  // V0, b and L do not vary along the fault
    const RSParams r0 = rs_params(S->fp, x0, 0.0);
    ia.lnV0h = std::log(0.5 / r0.V0);
    ia.rs_bL = r0.b / r0.L0;
    ia.rs_binv = 1.0 / r0.b;
  }
  ia.rs_tol = S->rs_tol;
  ia.rs_maxit = S->rs_maxit;
  ia.C0 = S->B[0].C;
  ia.C1 = S->B[1].C;
  ia.fault_comp = S->fault_comp && S->B[0].C && S->B[1].C;
  if (S->mms) {
    // T(t) and T'(t) of the manufactured solution at this stage's time, for
    // the interface here and the block phases of the same stage
    S->mms_T = std::cos(S->mms_kt * ts);
    S->mms_Tp = -S->mms_kt * std::sin(S->mms_kt * ts);
    ia.ms0 = S->B[0].ms;
    ia.ms1 = S->B[1].ms;
    ia.mms_T = S->mms_T;
  }
  ia.fp = S->fp;
  ia.frame = (c.want_frame && stage == 1) ? S->frame_dev + (size_t)S->frame_fill * kFrameWords * nf : nullptr;
  ia.solver_fail = S->solver_fail;
  mark_begin(S, 0);
  launch_interface(ia, S->stream);
  c.launches += 1;
  mark_end(S);
  if (stage == 1 && c.want_station) {
    // stage-1 fields are the fields at t0 (write_output, src/time_step.f90:137)
    for (int b = 0; b < 2; ++b) {
      auto& T = S->st[b];
      const int n = (int)T.ijk.size() / 3;
      if (n == 0) continue;
      double* out = T.ring + (size_t)S->st_fill * n * 3;
      if (S->prec == WQL_FP64)
        station_kernel<double><<<(n + 127) / 128, 128, 0, S->stream>>>((const double*)S->B[b].F[S->cur], S->B[b].np, T.idx_dev, n, out);
      else
        station_kernel<float><<<(n + 127) / 128, 128, 0, S->stream>>>((const float*)S->B[b].F[S->cur], S->B[b].np, T.idx_dev, n, out);
      c.launches += 1;
    }
  }
}

void stage_block_pre(wql_scn* S, StepCtx& c, int stage, int b) {
  mark_begin(S, 2);
  if (S->prec == WQL_FP64) c.launches += launch_pre<double>(volume_args<double>(S, b, stage_A(S, stage), stage_Bdt(S, stage), stage == 5), S->stream);
  else c.launches += launch_pre<float>(volume_args<float>(S, b, stage_A(S, stage), stage_Bdt(S, stage), stage == 5), S->stream);
  mark_end(S);
}

void stage_block_stencil(wql_scn* S, StepCtx& c, int stage, int b) {
  mark_begin(S, 1);
  if (S->prec == WQL_FP64) launch_volume<double>(volume_args<double>(S, b, stage_A(S, stage), stage_Bdt(S, stage), stage == 5), S->curv, S->stream);
  else launch_volume<float>(volume_args<float>(S, b, stage_A(S, stage), stage_Bdt(S, stage), stage == 5), S->curv, S->stream);
  mark_end(S);
  c.launches += 1;
}

void stage_block_post(wql_scn* S, StepCtx& c, int stage, int b) {
  const double A = stage_A(S, stage), Bdt = stage_Bdt(S, stage), ts = stage_time(S, c, stage);
  mark_begin(S, 2);
  // moment-tensor sources (set_rates, src/domain.f90:926-952) at the stage time
  for (const auto& T : S->mt[b]) {
    double At = 0.0;
    source_time(T.src.type, ts, T.src.t_init, T.src.duration, At);
    double am[6];
    for (int k = 0; k < 6; ++k) am[k] = At * T.src.m[k];
    if (S->prec == WQL_FP64)
      launch_source<double>(volume_args<double>(S, b, A, Bdt, stage == 5), T.lo, T.dim, T.delta, am, S->stream);
    else
      launch_source<float>(volume_args<float>(S, b, A, Bdt, stage == 5), T.lo, T.dim, T.delta, am, S->stream);
    c.launches += 1;
  }
  if (S->prec == WQL_FP64) c.launches += launch_corrections<double>(volume_args<double>(S, b, A, Bdt, stage == 5), S->curv, S->stream);
  else c.launches += launch_corrections<float>(volume_args<float>(S, b, A, Bdt, stage == 5), S->curv, S->stream);
  mark_end(S);
}

int step_end(wql_scn* S, StepCtx& c) {
  CK(cudaGetLastError());
  S->launches_last_step = c.launches;
  S->t = c.t0 + S->rk.C[5] * S->dt;
  S->nstep += 1;
  if (c.want_station) {
    S->st_times.push_back(c.t0);
    S->st_fill += 1;
    S->st_records += 1;
    if (S->st_fill == S->st_cap) {
      const int rc = flush_stations(S);
      if (rc) return rc;
    }
  }
  if (c.want_frame) {
    S->frame_fill += 1;
    S->nframes += 1;
    if (S->frame_fill == S->frame_cap) return rotate_frames(S);
  }
  return WQL_OK;
}

int run_step(wql_scn* S);

}  // namespace

// Scenarios advanced together (continuous batching): per stage each member's
// interface and face pre-kernels run on the member's own stream, the stencil
// of every TMA-eligible block of every member is one launch from a packed
// table on the batch stream, and the members' source and correction kernels
// run on their own streams again.  Members join and leave between steps.
struct wql_batch {
  wql_ctx* ctx = nullptr;
  std::vector<wql_scn*> members;
  cudaStream_t stream = nullptr;
  cudaEvent_t joined = nullptr;
  std::vector<cudaEvent_t> ev;
  // Packed stencil tables of the current membership, built once per
  // membership (and tuning): every member's buffer index flips with every
  // stage, so a step starts in one of two phases, and the tables hold
  // [phase][stage][curvilinear] groups of descriptors in one device array.
  TmaBatchDesc* d_dev = nullptr;
  size_t d_cap = 0;
  struct Group {
    size_t off = 0;
    int nd = 0;
    long long total = 0;
    std::vector<size_t> who;  // members with a block in the group
  };
  Group groups[2][5][2];
  std::vector<long long> key_members;  // member uids
  std::vector<int> key_tuning;  // variant, schunk per member
  std::vector<int> cur0;        // members' buffer index when the tables were built
  bool built = false;
  ~wql_batch() {
    for (auto e : ev) cudaEventDestroy(e);
    if (joined) cudaEventDestroy(joined);
    if (d_dev) cudaFree(d_dev);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

bool batch_tma(const wql_scn* S) {
  return S->prec == WQL_FP32C && !S->fd && (S->kernel_variant == 0 || S->kernel_variant == 5 || S->kernel_variant == 6);
}

// (Re)builds the packed tables when the membership or a member's tuning
// changed, and returns the phase of this step.
int batch_tables(wql_batch* B, int* phase) {
  const size_t n = B->members.size();
  std::vector<int> tun;
  for (auto* S : B->members) {
    tun.push_back(S->kernel_variant);
    tun.push_back(S->schunk);
  }
  std::vector<long long> uids;
  for (auto* S : B->members) uids.push_back(S->uid);
  bool same = B->built && B->key_members == uids && B->key_tuning == tun;
  int p = 0;
  if (same && n) {
    p = B->members[0]->cur ^ B->cur0[0];
    for (size_t i = 0; i < n; ++i) same = same && ((B->members[i]->cur ^ B->cur0[i]) == p);
  }
  if (same) {
    *phase = p;
    return WQL_OK;
  }
  std::vector<TmaBatchDesc> h;
  B->cur0.assign(n, 0);
  for (size_t i = 0; i < n; ++i) B->cur0[i] = B->members[i]->cur;
  for (int ph = 0; ph < 2; ++ph)
    for (int stage = 1; stage <= 5; ++stage)
      for (int curv = 0; curv < 2; ++curv) {
        wql_batch::Group& g = B->groups[ph][stage - 1][curv];
        g = wql_batch::Group();
        g.off = h.size();
        for (size_t i = 0; i < n; ++i) {
          wql_scn* S = B->members[i];
          if (!batch_tma(S) || (int)S->curv != curv) continue;
          const int keep = S->cur;
          S->cur = B->cur0[i] ^ ph ^ ((stage - 1) & 1);
          bool any = false;
          for (int b = 0; b < 2; ++b) {
            VolumeArgs<float> a = volume_args<float>(S, b, stage_A(S, stage), stage_Bdt(S, stage), stage == 5);
            if (!tma_eligible(a)) continue;
            TmaBatchDesc d;
            const long long k = fill_tma_desc(a, d);
            d.cta0 = g.total;
            g.total += k;
            h.push_back(d);
            any = true;
          }
          S->cur = keep;
          if (any) g.who.push_back(i);
        }
        g.nd = (int)(h.size() - g.off);
      }
  if (h.size() > B->d_cap) {
    CK(cudaStreamSynchronize(B->stream));
    if (B->d_dev) cudaFree(B->d_dev);
    B->d_dev = nullptr;
    B->d_cap = h.size();
    CK(cudaMalloc(&B->d_dev, B->d_cap * sizeof(TmaBatchDesc)));
  }
  if (!h.empty()) {
    // the previous tables may still be in use by launches in flight
    CK(cudaStreamSynchronize(B->stream));
    CK(cudaMemcpy(B->d_dev, h.data(), h.size() * sizeof(TmaBatchDesc), cudaMemcpyHostToDevice));
  }
  B->key_members = uids;
  B->key_tuning = tun;
  B->built = true;
  *phase = 0;
  return WQL_OK;
}

int batch_step(wql_batch* B) {
  const size_t n = B->members.size();
  while (B->ev.size() < n) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    B->ev.push_back(e);
  }
  int phase = 0;
  int trc = batch_tables(B, &phase);
  if (trc) return trc;
  std::vector<StepCtx> c(n);
  for (size_t i = 0; i < n; ++i) c[i] = step_begin(B->members[i]);
  for (int stage = 1; stage <= 5; ++stage) {
    for (size_t i = 0; i < n; ++i) {
      wql_scn* S = B->members[i];
      stage_head(S, c[i], stage);
      for (int b = 0; b < 2; ++b) stage_block_pre(S, c[i], stage, b);
    }
    // the packed stencil launches: one group per mesh kind
    for (int curv = 0; curv < 2; ++curv) {
      const wql_batch::Group& g = B->groups[phase][stage - 1][curv];
      if (g.nd == 0) continue;
      for (size_t i : g.who) {
        CK(cudaEventRecord(B->ev[i], B->members[i]->stream));
        CK(cudaStreamWaitEvent(B->stream, B->ev[i], 0));
      }
      launch_stencil_tma_batch(B->d_dev + g.off, g.nd, g.total, curv == 1, true, B->stream);
      CK(cudaEventRecord(B->joined, B->stream));
      for (size_t i : g.who) {
        CK(cudaStreamWaitEvent(B->members[i]->stream, B->joined, 0));
        c[i].launches += 1;
      }
    }
    // blocks outside the packed launch: their own stencil launch
    for (size_t i = 0; i < n; ++i) {
      wql_scn* S = B->members[i];
      for (int b = 0; b < 2; ++b) {
        bool packed = false;
        if (batch_tma(S)) packed = tma_eligible(volume_args<float>(S, b, 0.0, 0.0, false));
        if (!packed) stage_block_stencil(S, c[i], stage, b);
      }
    }
    for (size_t i = 0; i < n; ++i) {
      wql_scn* S = B->members[i];
      for (int b = 0; b < 2; ++b) stage_block_post(S, c[i], stage, b);
      S->cur ^= 1;
    }
  }
  for (size_t i = 0; i < n; ++i) {
    const int rc = step_end(B->members[i], c[i]);
    if (rc) return rc;
  }
  // the batch stream ends after every member's step
  for (size_t i = 0; i < n; ++i) {
    CK(cudaEventRecord(B->ev[i], B->members[i]->stream));
    CK(cudaStreamWaitEvent(B->stream, B->ev[i], 0));
  }
  return WQL_OK;
}

// One RK stage of the current step (stages 1..5 in order).
void run_stage(wql_scn* S, StepCtx& c, int stage) {
  bool pair = false;  // both blocks through the TMA kernel: one stencil launch per stage
  if (S->prec == WQL_FP32C) {
    pair = true;
    for (int b = 0; b < 2; ++b) pair = pair && stencil_is_tma(volume_args<float>(S, b, 0.0, 0.0, false));
  }
  stage_head(S, c, stage);
  if (pair) {
    // both blocks' pre-kernels, the stencil launch, both blocks'
    // corrections (the blocks touch disjoint arrays)
    const double A = stage_A(S, stage), Bdt = stage_Bdt(S, stage);
    {
      const VolumeArgs<float> a0 = volume_args<float>(S, 0, A, Bdt, stage == 5);
      const VolumeArgs<float> a1 = volume_args<float>(S, 1, A, Bdt, stage == 5);
      mark_begin(S, 2);
      c.launches += launch_pre2<float>(a0, a1, S->stream);
      mark_end(S);
    }
    mark_begin(S, 1);
    launch_stencil_tma2(volume_args<float>(S, 0, A, Bdt, stage == 5), volume_args<float>(S, 1, A, Bdt, stage == 5),
                        S->curv, true, S->stream);
    mark_end(S);
    c.launches += 1;
    for (int b = 0; b < 2; ++b) stage_block_post(S, c, stage, b);
  } else {
    for (int b = 0; b < 2; ++b) {
      stage_block_pre(S, c, stage, b);
      stage_block_stencil(S, c, stage, b);
      stage_block_post(S, c, stage, b);
    }
  }
  S->cur ^= 1;
}

int run_step(wql_scn* S) {
  StepCtx c = step_begin(S);
  for (int stage = 1; stage <= 5; ++stage) run_stage(S, c, stage);
  return step_end(S, c);
}

}  // namespace

extern "C" {

int wql_last_error(char* buf, size_t n) {
  if (buf && n) {
    std::snprintf(buf, n, "%s", g_err.c_str());
  }
  return (int)g_err.size();
}

int wql_ctx_create(int device, wql_ctx** out) {
  if (!out) return fail(WQL_E_INPUT, "null argument");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(WQL_E_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (device < 0 || device >= ndev) return fail(WQL_E_INPUT, "device index out of range");
  CK(cudaSetDevice(device));
  wql_ctx* c = new wql_ctx();
  c->device = device;
  *out = c;
  return WQL_OK;
}

int wql_ctx_destroy(wql_ctx* ctx) {
  delete ctx;
  return WQL_OK;
}

int wql_scenario_create_from_text(wql_ctx* ctx, const char* in_text, const char* base_dir,
                                  int precision, wql_scn** out) {
  if (!in_text) return fail(WQL_E_INPUT, "null input text");
  Problem P;
  std::string err;
  if (parse_in_text(in_text, base_dir ? base_dir : "", P, err)) return fail(WQL_E_INPUT, err);
  return create(ctx, std::move(P), precision, nullptr, out);
}

int wql_scenario_create_ex(wql_ctx* ctx, const char* in_text, const char* base_dir, int precision,
                           const wql_media* media, wql_scn** out) {
  if (!in_text) return fail(WQL_E_INPUT, "null input text");
  Problem P;
  std::string err;
  if (parse_in_text(in_text, base_dir ? base_dir : "", P, err)) return fail(WQL_E_INPUT, err);
  return create(ctx, std::move(P), precision, media, out);
}

int wql_scenario_create_from_in(wql_ctx* ctx, const char* in_path, int precision, wql_scn** out) {
  if (!in_path) return fail(WQL_E_INPUT, "null path");
  Problem P;
  std::string err;
  if (parse_in_file(in_path, P, err)) return fail(WQL_E_INPUT, err);
  return create(ctx, std::move(P), precision, nullptr, out);
}

int wql_scenario_destroy(wql_scn* scn) {
  delete scn;
  return WQL_OK;
}

int wql_stage(wql_scn* scn, int stage) {
  if (!scn) return fail(WQL_E_INPUT, "null scenario");
  if (stage != scn->next_stage)
    return fail(WQL_E_STATE, "stage " + std::to_string(stage) + " requested, stage " +
                                 std::to_string(scn->next_stage) + " is next");
  CK(cudaSetDevice(scn->ctx->device));
  StepCtx c;
  if (stage == 1) {
    c = step_begin(scn);
  } else {
    c.want_frame = scn->want_frame;
    c.want_station = scn->want_station;
    c.t0 = scn->stage_t0;
    c.launches = scn->stage_launches;
  }
  run_stage(scn, c, stage);
  if (stage < 5) {
    scn->want_frame = c.want_frame;
    scn->want_station = c.want_station;
    scn->stage_t0 = c.t0;
    scn->stage_launches = c.launches;
    scn->next_stage = stage + 1;
    return WQL_OK;
  }
  scn->next_stage = 1;
  const int rc = step_end(scn, c);
  if (rc) return rc;
  return flush_frames(scn);
}

int wql_step(wql_scn* scn, int nsteps) {
  if (!scn) return fail(WQL_E_INPUT, "null scenario");
  if (nsteps < 0) return fail(WQL_E_INPUT, "negative step count");
  if (scn->next_stage != 1) return fail(WQL_E_STATE, "a step is in progress (wql_stage)");
  CK(cudaSetDevice(scn->ctx->device));
  for (int n = 0; n < nsteps; ++n) {
    int rc = run_step(scn);
    if (rc) return rc;
  }
  // no flush here: the frame and station rings are read out by the calls
  // that return them (wql_get_frames, wql_get_seismograms, the output
  // writer), so a caller stepping one step at a time never waits on the
  // device between steps
  return WQL_OK;
}

int wql_sync(wql_scn* scn, int check_nan) {
  if (!scn) return fail(WQL_E_INPUT, "null scenario");
  CK(cudaStreamSynchronize(scn->stream));
  CK(cudaGetLastError());
  unsigned int fails = 0;
  CK(cudaMemcpy(&fails, scn->solver_fail, sizeof(unsigned), cudaMemcpyDeviceToHost));
  int kerr = 0;
  CK(cudaMemcpy(&kerr, scn->err_dev, sizeof(int), cudaMemcpyDeviceToHost));
  if (kerr) return fail(WQL_E_CUDA, "stencil pipeline wait ran out of its iteration limit (code " + std::to_string(kerr) + ")");
  if (check_nan) {
    unsigned int* cnt = nullptr;
    CK(cudaMalloc(&cnt, sizeof(unsigned)));
    CK(cudaMemset(cnt, 0, sizeof(unsigned)));
    for (int b = 0; b < 2; ++b) {
      const long long n = 9 * scn->B[b].np;
      if (scn->prec == WQL_FP64)
        count_nonfinite<double><<<(unsigned)((n + 255) / 256), 256, 0, scn->stream>>>((const double*)scn->B[b].F[scn->cur], n, cnt);
      else
        count_nonfinite<float><<<(unsigned)((n + 255) / 256), 256, 0, scn->stream>>>((const float*)scn->B[b].F[scn->cur], n, cnt);
    }
    unsigned int h = 0;
    CK(cudaStreamSynchronize(scn->stream));
    CK(cudaMemcpy(&h, cnt, sizeof(unsigned), cudaMemcpyDeviceToHost));
    cudaFree(cnt);
    if (h) return fail(WQL_E_NAN, std::to_string(h) + " non-finite field values");
  }
  if (fails) return fail(WQL_E_SOLVER, std::to_string(fails) + " rate-and-state solves hit the 5000-iteration cap");
  return WQL_OK;
}

int wql_get_info(wql_scn* scn, wql_info* info) {
  if (!scn || !info) return fail(WQL_E_INPUT, "null argument");
  for (int b = 0; b < 2; ++b) {
    info->nq[b] = scn->B[b].nq;
    info->nr[b] = scn->B[b].nr;
    info->ns[b] = scn->B[b].ns;
  }
  info->dt = scn->dt;
  info->t = scn->t;
  info->nt = scn->nt;
  info->nstep = scn->nstep;
  info->precision = scn->prec;
  info->frames = scn->nframes;
  info->device_bytes = scn->device_bytes;
  return WQL_OK;
}

int wql_get_field(wql_scn* scn, int block, int comp, double* host_out) {
  if (!scn || !host_out || block < 0 || block > 1 || comp < 0 || comp > 10)
    return fail(WQL_E_INPUT, "bad argument");
  auto& B = scn->B[block];
  if (comp > 8 && !scn->pl_flow)
    return fail(WQL_E_STATE, "components 9 and 10 (plastic strain rate and strain) need plastic_flow");
  const void* src = comp == 9 ? B.pl_lambda : (comp == 10 ? B.pl_gammap : B.F[scn->cur]);
  const long long off = comp > 8 ? 0 : comp * B.np;
  CK(cudaStreamSynchronize(scn->stream));
  const long long rows = (long long)B.nr * B.ns;
  double* tmp = nullptr;
  CK(cudaMalloc(&tmp, B.npd * sizeof(double)));
  const unsigned grid = (unsigned)std::min<long long>((B.npd + 255) / 256, 4096);
  if (scn->prec == WQL_FP64)
    pitched_to_dense<double><<<grid, 256, 0, scn->stream>>>((const double*)src + off, B.pq, B.nq, rows, tmp);
  else
    pitched_to_dense<float><<<grid, 256, 0, scn->stream>>>((const float*)src + off, B.pq, B.nq, rows, tmp);
  cudaError_t e = cudaStreamSynchronize(scn->stream);
  if (e == cudaSuccess) e = cudaMemcpy(host_out, tmp, B.npd * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail(WQL_E_CUDA, cudaGetErrorString(e));
  return WQL_OK;
}

}  // extern "C"

namespace {

// Allocation-free field read: FP32 planes are widened through this fixed
// device array instead of a cudaMalloc'd temporary.  One s plane of pq*nr
// pitched points at a time; nothing in it needs to start at zero (each
// plane is written in full before it is copied out).
constexpr long long kPlaneScratchWords = 1LL << 20;  // 8 MiB of doubles
static __device__ __align__(256) double g_plane_scratch[kPlaneScratchWords];

__global__ void widen_plane(const float* __restrict__ src, double* __restrict__ dst, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (double)src[i];
}

// Device address of the scratch, resolved once per device with that device
// current.
int plane_scratch(int device, double** out) {
  static std::mutex mu;
  static double* addr[64] = {};
  if (device < 0 || device >= 64) return fail(WQL_E_INPUT, "device index out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_plane_scratch);
    if (e != cudaSuccess) return fail(WQL_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    addr[device] = (double*)p;
  }
  *out = addr[device];
  return WQL_OK;
}

}  // namespace

extern "C" {

int wql_get_field_noalloc(wql_scn* scn, int block, int comp, double* host_out) {
  if (!scn || !host_out || block < 0 || block > 1 || comp < 0 || comp > 8)
    return fail(WQL_E_INPUT, "bad argument");
  auto& B = scn->B[block];
  const int dev = scn->ctx->device;
  // the caller's current device is restored on every return
  struct DeviceGuard {
    int prev = -1;
    ~DeviceGuard() {
      if (prev >= 0) cudaSetDevice(prev);
    }
  } guard;
  CK(cudaGetDevice(&guard.prev));
  CK(cudaSetDevice(dev));
  CK(cudaStreamSynchronize(scn->stream));
  if (scn->prec == WQL_FP64) {
    // ordered on the scenario's stream only (no legacy-stream synchronisation)
    CK(cudaMemcpy2DAsync(host_out, B.nq * sizeof(double), (const double*)B.F[scn->cur] + comp * B.np,
                         B.pq * sizeof(double), B.nq * sizeof(double), (size_t)B.nr * B.ns, cudaMemcpyDeviceToHost,
                         scn->stream));
    CK(cudaStreamSynchronize(scn->stream));
    return WQL_OK;
  }
  const long long plane = (long long)B.pq * B.nr;
  if (plane > kPlaneScratchWords)
    return fail(WQL_E_INPUT, "wql_get_field_noalloc: a plane of " + std::to_string(plane) +
                                 " pitched points exceeds the " + std::to_string(kPlaneScratchWords) +
                                 "-point device scratch; use wql_get_field");
  double* scr = nullptr;
  int rc = plane_scratch(dev, &scr);
  if (rc) return rc;
  const float* src = (const float*)B.F[scn->cur] + comp * B.np;
  for (int k = 0; k < B.ns; ++k) {
    widen_plane<<<(unsigned)((plane + 255) / 256), 256, 0, scn->stream>>>(src + k * plane, scr, plane);
    CK(cudaMemcpy2DAsync(host_out + (size_t)k * B.nq * B.nr, B.nq * sizeof(double), scr, B.pq * sizeof(double),
                         B.nq * sizeof(double), B.nr, cudaMemcpyDeviceToHost, scn->stream));
  }
  CK(cudaStreamSynchronize(scn->stream));
  CK(cudaGetLastError());
  return WQL_OK;
}

int wql_set_field(wql_scn* scn, int block, int comp, const double* host_in) {
  if (!scn || !host_in || block < 0 || block > 1 || comp < 0 || comp > 8)
    return fail(WQL_E_INPUT, "bad argument");
  auto& B = scn->B[block];
  CK(cudaStreamSynchronize(scn->stream));
  const long long rows = (long long)B.nr * B.ns;
  double* tmp = nullptr;
  CK(cudaMalloc(&tmp, B.npd * sizeof(double)));
  cudaError_t e = cudaMemcpy(tmp, host_in, B.npd * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    const unsigned grid = (unsigned)std::min<long long>((B.np + 255) / 256, 4096);
    if (scn->prec == WQL_FP64)
      dense_to_pitched<double><<<grid, 256, 0, scn->stream>>>(tmp, B.pq, B.nq, rows, (double*)B.F[scn->cur] + comp * B.np);
    else
      dense_to_pitched<float><<<grid, 256, 0, scn->stream>>>(tmp, B.pq, B.nq, rows, (float*)B.F[scn->cur] + comp * B.np);
    // the new values carry no rounding error yet: clear their compensation
    if (B.C) e = cudaMemsetAsync((comp_t*)B.C + comp * B.np, 0, B.np * sizeof(comp_t), scn->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(scn->stream);
  }
  cudaFree(tmp);
  if (e != cudaSuccess) return fail(WQL_E_CUDA, cudaGetErrorString(e));
  return WQL_OK;
}

int wql_get_iface(wql_scn* scn, int copy, int what, double* host_out) {
  if (!scn || !host_out || copy < 0 || copy > 1 || what < 0 || what > 5) return fail(WQL_E_INPUT, "bad argument");
  const long long nf = (long long)scn->B[0].nr * scn->B[0].ns;
  const double* src;
  if (what < 4) src = scn->S + ((long long)copy * 4 + what) * nf;
  else if (what == 4) src = scn->W + (long long)copy * nf;
  else src = scn->trup + (long long)copy * nf;
  CK(cudaStreamSynchronize(scn->stream));
  CK(cudaMemcpy(host_out, src, nf * sizeof(double), cudaMemcpyDeviceToHost));
  return WQL_OK;
}

int wql_mms_norms(wql_scn* scn, int block, double* err2, double* ref2) {
  if (!scn || !err2 || !ref2 || block < 0 || block > 1) return fail(WQL_E_INPUT, "bad argument");
  if (!scn->mms) return fail(WQL_E_INPUT, "the scenario has no manufactured solution (&mms_list use_mms)");
  if (scn->next_stage != 1) return fail(WQL_E_INPUT, "a step is in progress (wql_stage)");
  const auto& B = scn->B[block];
  const double Tt = std::cos(scn->mms_kt * scn->t);
  double acc[18];
  CK(cudaMemsetAsync(scn->mms_acc, 0, sizeof(acc), scn->stream));
  if (scn->prec == WQL_FP64)
    launch_mms_norms<double>(B.nq, B.nr, B.ns, B.pq, (const double*)B.F[scn->cur], (const double*)B.ms, Tt,
                             scn->mms_acc, scn->stream);
  else
    launch_mms_norms<float>(B.nq, B.nr, B.ns, B.pq, (const float*)B.F[scn->cur], (const float*)B.ms, Tt,
                            scn->mms_acc, scn->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(acc, scn->mms_acc, sizeof(acc), cudaMemcpyDeviceToHost, scn->stream));
  CK(cudaStreamSynchronize(scn->stream));
  for (int c = 0; c < 9; ++c) {
    err2[c] = acc[c];
    ref2[c] = acc[9 + c];
  }
  return WQL_OK;
}

int wql_frame_count(wql_scn* scn, int* frames) {
  if (!scn || !frames) return fail(WQL_E_INPUT, "null argument");
  *frames = scn->nframes;
  return WQL_OK;
}

int wql_get_frames(wql_scn* scn, int what, float* host_out) {
  if (!scn || !host_out || what < 0 || what > 7) return fail(WQL_E_INPUT, "bad argument");
  int rc = flush_frames(scn);
  if (rc) return rc;
  const long long nf = (long long)scn->B[0].nr * scn->B[0].ns;
  const int off = kFrameOff[what], nc = kFrameOff[what + 1] - kFrameOff[what];
  int fr = 0;
  for (const auto& chunk : scn->frame_chunks)
    for (size_t k = 0; k < chunk.size(); k += (size_t)kFrameWords * nf, ++fr)
      std::memcpy(host_out + (size_t)fr * nc * nf, chunk.data() + k + (size_t)off * nf,
                  (size_t)nc * nf * sizeof(float));
  return WQL_OK;
}

int wql_station_count(wql_scn* scn, int block, int* nstations, int* nrecords) {
  if (!scn || block < 0 || block > 1 || !nstations) return fail(WQL_E_INPUT, "bad argument");
  *nstations = (int)scn->st[block].ijk.size() / 3;
  if (nrecords) *nrecords = scn->st_records;
  return WQL_OK;
}

int wql_station_index(wql_scn* scn, int block, int* ijk) {
  if (!scn || block < 0 || block > 1 || !ijk) return fail(WQL_E_INPUT, "bad argument");
  std::memcpy(ijk, scn->st[block].ijk.data(), scn->st[block].ijk.size() * sizeof(int));
  return WQL_OK;
}

int wql_get_seismograms(wql_scn* scn, int block, double* host_out) {
  if (!scn || block < 0 || block > 1 || !host_out) return fail(WQL_E_INPUT, "bad argument");
  const int rc = flush_stations(scn);
  if (rc) return rc;
  std::memcpy(host_out, scn->st[block].host.data(), scn->st[block].host.size() * sizeof(double));
  return WQL_OK;
}

// Output files in the reference's formats, so that its tools read them:
// the eight fault streams as raw float32 frames in <name>_interface.<ext>
// (init_fault_output / write_fault / write_hats, src/fault_output.f90:12-121,
// frame layout src/mpi3dio.f90:327-364), and one text file per station with
// one line (4f15.10) of t, vx, vy, vz per record (init_seismogram /
// write_seismogram, src/seismogram.f90:98-114, 368-384, 460-474) at
// <station_file_directory>/block<b>/<name>_<i>_<j>_<k>_block<b>.dat, or
// <name>_<x>_<y>_<z>.dat (f20.3 positions) with station_xyz_index.
namespace {

// Fortran Fw.d edit of one value (right-justified, w characters; asterisks
// when it does not fit).
std::string fortran_f(double v, int w, int d) {
  char buf[64];
  if (std::isnan(v)) std::snprintf(buf, sizeof(buf), "%*s", w, "NaN");
  else if (std::isinf(v)) std::snprintf(buf, sizeof(buf), "%*s", w, v > 0 ? "Infinity" : "-Infinity");
  else std::snprintf(buf, sizeof(buf), "%*.*f", w, d, v);
  std::string s(buf);
  if ((int)s.size() > w) s.assign(w, '*');
  return s;
}

std::string trimmed_f(double v, int w, int d) {  // trim(adjustl(...)) of an Fw.d edit
  std::string s = fortran_f(v, w, d);
  const size_t i = s.find_first_not_of(' ');
  return i == std::string::npos ? std::string() : s.substr(i);
}

}  // namespace

int wql_write_outputs(wql_scn* scn, const char* out_dir) {
  if (!scn || !out_dir) return fail(WQL_E_INPUT, "null argument");
  namespace fs = std::filesystem;
  const std::string name = scn->P.name;
  std::error_code ec;
  fs::create_directories(out_dir, ec);
  if (ec) return fail(WQL_E_INPUT, std::string("cannot create ") + out_dir + ": " + ec.message());
  int frames = 0, rc = wql_frame_count(scn, &frames);
  if (rc) return rc;
  if (frames > 0) {
    static const char* ext[8] = {"Uface", "Vface", "S", "Uhat", "Vhat", "Svel", "trup", "state"};
    const long long nf = (long long)scn->B[0].nr * scn->B[0].ns;
    for (int what = 0; what < 8; ++what) {
      const int nc = kFrameOff[what + 1] - kFrameOff[what];
      std::vector<float> buf((size_t)frames * nc * nf);
      if ((rc = wql_get_frames(scn, what, buf.data()))) return rc;
      const fs::path path = fs::path(out_dir) / (name + "_interface." + ext[what]);
      fs::create_directories(path.parent_path(), ec);  // the name may hold a directory part
      std::FILE* f = std::fopen(path.c_str(), "wb");
      if (!f) return fail(WQL_E_INPUT, "cannot write " + path.string());
      const size_t n = std::fwrite(buf.data(), sizeof(float), buf.size(), f);
      std::fclose(f);
      if (n != buf.size()) return fail(WQL_E_INPUT, "short write to " + path.string());
    }
  }
  if ((rc = flush_stations(scn))) return rc;
  const std::string sdir = scn->P.station_file_directory;
  for (int b = 0; b < 2; ++b) {
    const auto& T = scn->st[b];
    const int n = (int)T.ijk.size() / 3;
    if (n == 0) continue;
    const std::string bdir = "block" + std::to_string(b + 1);
    const fs::path dir = (sdir.empty() || sdir == ".") ? fs::path(out_dir) / bdir : fs::path(out_dir) / sdir / bdir;
    fs::create_directories(dir, ec);
    if (ec) return fail(WQL_E_INPUT, "cannot create " + dir.string() + ": " + ec.message());
    const size_t nrec = T.host.size() / (4 * (size_t)n);
    for (int i = 0; i < n; ++i) {
      std::string file;
      if (scn->P.station_xyz_index)
        file = name + "_" + trimmed_f(T.xyz[3 * i], 20, 3) + "_" + trimmed_f(T.xyz[3 * i + 1], 20, 3) + "_" +
               trimmed_f(T.xyz[3 * i + 2], 20, 3) + ".dat";
      else
        file = name + "_" + std::to_string(T.ijk[3 * i]) + "_" + std::to_string(T.ijk[3 * i + 1]) + "_" +
               std::to_string(T.ijk[3 * i + 2]) + "_block" + std::to_string(b + 1) + ".dat";
      const fs::path path = dir / file;
      fs::create_directories(path.parent_path(), ec);
      std::FILE* f = std::fopen(path.c_str(), "w");
      if (!f) return fail(WQL_E_INPUT, "cannot write " + path.string());
      for (size_t r = 0; r < nrec; ++r) {
        const double* rec = &T.host[(r * n + i) * 4];
        std::string line;
        for (int c = 0; c < 4; ++c) line += fortran_f(rec[c], 15, 10);
        line += '\n';
        std::fputs(line.c_str(), f);
      }
      std::fclose(f);
    }
  }
  return WQL_OK;
}

int wql_write_block_grids(const char* in_text, const char* base_dir, const char* out_dir) {
  if (!in_text || !out_dir) return fail(WQL_E_INPUT, "null argument");
  Problem P;
  std::string err;
  if (parse_in_text(in_text, base_dir ? base_dir : "", P, err)) return fail(WQL_E_INPUT, err);
  std::error_code ec;
  std::filesystem::create_directories(out_dir, ec);
  if (ec) return fail(WQL_E_INPUT, std::string("cannot create ") + out_dir + ": " + ec.message());
  if (write_block_grids(P, out_dir, err)) return fail(WQL_E_INPUT, err);
  return WQL_OK;
}

int wql_autotune(wql_scn* scn, int reps, int* variant, int* schunk) {
  if (!scn || reps <= 0) return fail(WQL_E_INPUT, "bad argument");
  CK(cudaSetDevice(scn->ctx->device));
  // results are kept per block shape, mesh and precision
  static std::mutex mu;
  static std::map<std::vector<int>, std::pair<int, int>> cache;
  std::vector<int> key = {scn->prec, (int)scn->curv, scn->fd};
  for (int b = 0; b < 2; ++b) {
    key.push_back(scn->B[b].nq);
    key.push_back(scn->B[b].nr);
    key.push_back(scn->B[b].ns);
  }
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      scn->kernel_variant = it->second.first;
      scn->schunk = it->second.second;
      if (variant) *variant = scn->kernel_variant;
      if (schunk) *schunk = scn->schunk;
      return WQL_OK;
    }
  }
  // candidates: the TMA kernel with several s chunk sizes (FP32C; on
  // Cartesian blocks that fill 40-wide tiles better, with both tile
  // widths), the tiled and per-point kernels (FP64)
  std::vector<std::pair<int, int>> cand;
  if (scn->prec == WQL_FP32C) {
    const bool wide = tma_tile_width(scn->B[0].nq, scn->B[1].nq, scn->curv) != kTmaTQ;
    for (int c : {0, 12, 14, 16, 24, 32, 48})
      if (c <= scn->B[0].ns) {
        cand.push_back({5, c});
        if (wide) cand.push_back({6, c});
      }
  } else {
    for (int c : {8, 16, 32}) cand.push_back({2, c});
    cand.push_back({1, 0});
  }
  // scratch rates, compensation and output so the scenario state is untouched
  void* scratch[2][3] = {};
  int rc = WQL_OK;
  for (int b = 0; b < 2 && !rc; ++b)
    for (int k = 0; k < 3 && !rc; ++k) {
      if (k == 1 && scn->prec != WQL_FP32C) continue;
      if (cudaMalloc(&scratch[b][k], 9 * scn->B[b].np * scn->esz) != cudaSuccess) rc = fail(WQL_E_OOM, "autotune scratch");
      else CK(cudaMemsetAsync(scratch[b][k], 0, 9 * scn->B[b].np * scn->esz, scn->stream));
    }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int keep_v = scn->kernel_variant, keep_c = scn->schunk;
  float best = 1e30f;
  std::pair<int, int> choice = {keep_v, keep_c};
  for (auto& c : cand) {
    if (rc) break;
    scn->kernel_variant = c.first;
    scn->schunk = c.second;
    auto run = [&]() {
      for (int b = 0; b < 2; ++b) {
        if (scn->prec == WQL_FP64) {
          VolumeArgs<double> a = volume_args<double>(scn, b, 0.5, 1e-4, false);
          a.DF = (double*)scratch[b][0];
          a.Fout = (double*)scratch[b][2];
          a.C = nullptr;
          launch_volume<double>(a, scn->curv, scn->stream);
        } else {
          VolumeArgs<float> a = volume_args<float>(scn, b, 0.5, 1e-4, false);
          a.DF = (float*)scratch[b][0];
          a.C = (comp_t*)scratch[b][1];
          a.Fout = (float*)scratch[b][2];
          if (c.first == 5 || c.first == 6) {
            // the TMA kernel reads DF and C through the block's tensor maps:
            // point them at the scratch arrays for the trial
            StencilMaps m = scn->B[b].maps;
            void* Fs[2] = {scn->B[b].F[0], scn->B[b].F[1]};
            if (make_stencil_maps(m, Fs, scn->B[b].coef, scratch[b][0], scratch[b][1], scn->B[b].nq, scn->B[b].nr,
                                  scn->B[b].ns, scn->B[b].pq, scn->curv, scn->fd,
                                  c.first == 6 ? kTmaTQ : tma_tile_width(scn->B[0].nq, scn->B[1].nq, scn->curv))) {
              rc = fail(WQL_E_CUDA, "autotune tensor maps");
              return;
            }
            m.cur = scn->cur;
            a.tma = &m;
            launch_volume<float>(a, scn->curv, scn->stream);
          } else {
            launch_volume<float>(a, scn->curv, scn->stream);
          }
        }
      }
    };
    run();  // warm-up
    cudaEventRecord(e0, scn->stream);
    for (int r = 0; r < reps; ++r) run();
    cudaEventRecord(e1, scn->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = fail(WQL_E_CUDA, "autotune trial failed");
      break;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      choice = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (int b = 0; b < 2; ++b)
    for (int k = 0; k < 3; ++k)
      if (scratch[b][k]) cudaFree(scratch[b][k]);
  if (rc) {
    scn->kernel_variant = keep_v;
    scn->schunk = keep_c;
    return rc;
  }
  CK(cudaGetLastError());
  scn->kernel_variant = choice.first;
  scn->schunk = choice.second;
  {
    std::lock_guard<std::mutex> lock(mu);
    cache[key] = choice;
  }
  if (variant) *variant = choice.first;
  if (schunk) *schunk = choice.second;
  return WQL_OK;
}

int wql_estimate_device_bytes(const char* in_text, const char* base_dir, int precision, long long* resident,
                              long long* peak) {
  if (!in_text || !resident || !peak) return fail(WQL_E_INPUT, "null argument");
  if (precision != WQL_FP64 && precision != WQL_FP32C) return fail(WQL_E_INPUT, "unknown precision");
  Problem P;
  std::string err;
  if (parse_in_text(in_text, base_dir ? base_dir : "", P, err)) return fail(WQL_E_INPUT, err);
  // the allocations of create() / setup_block(), rounded up as cudaMalloc does
  const long long esz = precision == WQL_FP64 ? 8 : 4;
  auto al = [](long long b) { return (b + 511) / 512 * 512; };
  long long res = 0, transient = 0;
  const long long nf = (long long)P.btp[0].nqrs[1] * P.btp[0].nqrs[2];
  for (int b = 0; b < 2; ++b) {
    const BlockParams& bp = P.btp[b];
    const long long nq = bp.nqrs[0], nr = bp.nqrs[1], ns = bp.nqrs[2];
    const long long per16 = esz == 4 ? 8 : 2, pq = (nq + per16 - 1) / per16 * per16;
    const long long npd = nq * nr * ns, np = pq * nr * ns;
    const bool curv = P.type_of_mesh == "curvilinear";
    res += 2 * al(9 * np * esz) + al(9 * np * esz) + al((curv ? kCurvCoef : kCartCoef) * np * esz);
    if (precision == WQL_FP32C) res += al(9 * np * (long long)sizeof(comp_t));
    const long long nfs[3] = {nr * ns, nq * ns, nq * nr};
    for (int s2 = 0; s2 < 6; ++s2) res += al(kFaceWords * nfs[s2 / 2] * 8);
    const int dims[3] = {(int)nq, (int)nr, (int)ns};
    for (int s2 = 0; s2 < 6; ++s2) {
      const bool pml = (s2 % 2 == 0) ? bp.pml_lqrs[s2 / 2] : bp.pml_rqrs[s2 / 2];
      if (pml && bp.npml > 0) res += 2 * al(9 * (npd / dims[s2 / 2]) * bp.npml * esz);
    }
    bool any_pml = false;
    for (int s2 = 0; s2 < 3; ++s2) any_pml = any_pml || bp.pml_lqrs[s2] || bp.pml_rqrs[s2];
    if (any_pml && bp.npml > 0 && precision == WQL_FP32C) res += al(9 * np * esz);
    if (P.response == "plastic") res += al(np * esz);
    if (P.response == "plastic" && P.plastic_model != "scec") res += 2 * al(np * esz);
    if (P.response == "anelastic") {
      res += 2 * al(24 * np * esz) + al(np * esz) + al(npd * 8);
      if (precision == WQL_FP32C && !(any_pml && bp.npml > 0)) res += al(9 * np * esz);
    }
    // set-up arrays of one block: x, metric, J, material (FP64)
    transient = std::max(transient, al(3 * npd * 8) + al(9 * npd * 8) + al(npd * 8) + al(3 * npd * 8));
  }
  res += al(6 * nf * 8) + 2 * al(8 * nf * 8) + 3 * al(2 * nf * 8) + al(18 * nf * esz) + al(10 * nf * 8) + 2 * 512;
  if (P.w_fault) res += 2 * al((long long)frame_ring_cap(nf) * kFrameWords * nf * 4);
  if (P.output_seismograms) {
    // station rings: each requested station is found in at most one block
    // (within half a cell of a grid point)
    const long long n = !P.stations.empty() ? (long long)P.stations.size() / 3
                                            : (long long)(P.stationsU.size() + P.stationsV.size()) / 3;
    res += al((long long)station_ring_cap(P) * n * 3 * 8) + al(n * 8);
  }
  *resident = res;
  *peak = res + transient;
  return WQL_OK;
}

int wql_batch_create(wql_ctx* ctx, wql_batch** out) {
  if (!ctx || !out) return fail(WQL_E_INPUT, "null argument");
  CK(cudaSetDevice(ctx->device));
  std::unique_ptr<wql_batch> B(new wql_batch());
  B->ctx = ctx;
  CK(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&B->joined, cudaEventDisableTiming));
  *out = B.release();
  return WQL_OK;
}

int wql_batch_destroy(wql_batch* b) {
  if (b) {
    cudaStreamSynchronize(b->stream);
    delete b;
  }
  return WQL_OK;
}

int wql_batch_add(wql_batch* b, wql_scn* scn) {
  if (!b || !scn) return fail(WQL_E_INPUT, "null argument");
  if (scn->ctx->device != b->ctx->device) return fail(WQL_E_INPUT, "scenario is on another device");
  for (auto* m : b->members)
    if (m == scn) return fail(WQL_E_STATE, "scenario is already in the batch");
  if (scn->next_stage != 1) return fail(WQL_E_STATE, "the scenario is in the middle of a step (wql_stage)");
  // the packed launch runs 32-wide tiles: a member set up with the wide
  // Cartesian tiles gets 32-wide tensor maps
  if (scn->prec == WQL_FP32C)
    for (int k = 0; k < 2; ++k) {
      auto& B = scn->B[k];
      if (B.maps.tq == kTmaTQ) continue;
      const int erc =
          make_stencil_maps(B.maps, B.F, B.coef, B.DF, B.C, B.nq, B.nr, B.ns, B.pq, scn->curv, scn->fd, kTmaTQ);
      if (erc) return fail(WQL_E_CUDA, "cuTensorMapEncodeTiled failed for the stencil maps (error " + std::to_string(erc) + ")");
    }
  b->members.push_back(scn);
  return WQL_OK;
}

int wql_batch_remove(wql_batch* b, wql_scn* scn) {
  if (!b || !scn) return fail(WQL_E_INPUT, "null argument");
  for (size_t i = 0; i < b->members.size(); ++i)
    if (b->members[i] == scn) {
      CK(cudaStreamSynchronize(b->stream));
      b->members.erase(b->members.begin() + i);
      return WQL_OK;
    }
  return fail(WQL_E_STATE, "scenario is not in the batch");
}

int wql_batch_step(wql_batch* b, int nsteps) {
  if (!b) return fail(WQL_E_INPUT, "null batch");
  if (nsteps < 0) return fail(WQL_E_INPUT, "negative step count");
  CK(cudaSetDevice(b->ctx->device));
  for (int k = 0; k < nsteps; ++k) {
    const int rc = batch_step(b);
    if (rc) return rc;
  }
  // as wql_step: the members' frames and station records are read out by
  // the calls that return them, so the call does not wait for the device
  return WQL_OK;
}

int wql_batch_stream(wql_batch* b, uintptr_t* stream) {
  if (!b || !stream) return fail(WQL_E_INPUT, "null argument");
  *stream = (uintptr_t)b->stream;
  return WQL_OK;
}

int wql_scenario_stream(wql_scn* scn, uintptr_t* stream) {
  if (!scn || !stream) return fail(WQL_E_INPUT, "null argument");
  *stream = (uintptr_t)scn->stream;
  return WQL_OK;
}

int wql_profile(wql_scn* scn, int enable) {
  if (!scn) return fail(WQL_E_INPUT, "null scenario");
  CK(cudaStreamSynchronize(scn->stream));
  scn->profiling = enable != 0;
  scn->ev_used = 0;
  scn->ev_marks.clear();
  return WQL_OK;
}

int wql_kernel_times(wql_scn* scn, int kind, double* ms, int* launches) {
  if (!scn || !ms || !launches) return fail(WQL_E_INPUT, "null argument");
  if (kind < 0 || kind > 2) return fail(WQL_E_INPUT, "kernel kind must be 0 (interface), 1 (stencil) or 2 (corrections)");
  CK(cudaStreamSynchronize(scn->stream));
  double t = 0.0;
  int n = 0;
  for (auto& m : scn->ev_marks) {
    if (m.second != kind) continue;
    float e = 0.0f;
    CK(cudaEventElapsedTime(&e, scn->ev_pool[m.first], scn->ev_pool[m.first + 1]));
    t += e;
    n += 1;
  }
  *ms = t;
  *launches = n;
  return WQL_OK;
}

int wql_set_tuning(wql_scn* scn, int kernel_variant, int schunk) {
  if (!scn || kernel_variant < 0 || kernel_variant > 6 || schunk < 0) return fail(WQL_E_INPUT, "bad tuning");
  if ((kernel_variant == 5 || kernel_variant == 6) && scn->prec == WQL_FP64)
    return fail(WQL_E_INPUT, "stencil variants 5 and 6 (TMA pipeline) are FP32-only");
  // 64x8 tiles of FP64 need 273 KiB of shared memory, more than a block may hold.
  if (kernel_variant == 4 && scn->prec == WQL_FP64)
    return fail(WQL_E_INPUT, "stencil variant 4 (64x8 tiles) is FP32-only");
  // variant 6 runs the TMA kernel on 32-wide tiles; the others keep (or
  // restore) the width chosen for the blocks at set-up
  if (scn->prec == WQL_FP32C) {
    CK(cudaStreamSynchronize(scn->stream));  // no launch in flight reads the old maps
    const int want = kernel_variant == 6 ? kTmaTQ : tma_tile_width(scn->B[0].nq, scn->B[1].nq, scn->curv);
    for (int k = 0; k < 2; ++k) {
      auto& B = scn->B[k];
      if (B.maps.tq == want) continue;
      const int erc =
          make_stencil_maps(B.maps, B.F, B.coef, B.DF, B.C, B.nq, B.nr, B.ns, B.pq, scn->curv, scn->fd, want);
      if (erc) return fail(WQL_E_CUDA, "cuTensorMapEncodeTiled failed for the stencil maps (error " + std::to_string(erc) + ")");
    }
  }
  scn->kernel_variant = kernel_variant;
  scn->schunk = schunk;
  return WQL_OK;
}

int wql_launches_per_step(wql_scn* scn, int* launches) {
  if (!scn || !launches) return fail(WQL_E_INPUT, "null argument");
  if (scn->launches_last_step == 0) return fail(WQL_E_STATE, "no step taken yet");
  *launches = scn->launches_last_step;
  return WQL_OK;
}

}  // extern "C"
