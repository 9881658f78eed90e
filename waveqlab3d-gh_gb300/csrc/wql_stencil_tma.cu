// TMA-pipelined stencil kernel for FP32 fields (the FP32-compensated mode):
// the same per-point update as the other stencil kernels,
//   DF <- A*DF + L(F),   F_out <- F + B*dt*DF   (Kahan-compensated),
// (scale_rates + set_rates + update_fields, src/fields.f90:49-171,
// src/JU_xJU_yJU_z6.f90:12-812 and 16141-16449, src/RHS_Interior.f90:133-274)
// on every plane of the block.
//
// The boundary and fault penalties of the face points (src/RHS_Interior.f90:
// 1516-1703, 1757-1772) are folded into DF beforehand by the face
// pre-kernel, so this kernel has no face-dependent work.
//
// A tile is 32 x 12 (q, r) points over a chunk of s planes; a CTA takes a
// tile (or, launched persistently, tiles in turn) and marches along its
// planes.  One
// producer thread streams each plane into shared memory with
// cp.async.bulk.tensor (TMA) through an NS-deep ring of stages guarded by
// mbarriers ("full" completes on the transaction bytes, "empty" when all
// consumer warps have read the stage):
//   main (plane s)   : the 9 field components on the tile plus a q halo of
//                      8 points each side (so every box starts on a 16-byte
//                      boundary and every q closure row of a tile is inside
//                      the box) and an r halo of 3 rows; J*metric_q on the
//                      q-extended rows, J*metric_r on the r-extended columns,
//                      the remaining 7 coefficients, the rates DF and the
//                      compensation C on the tile;
//   lead (plane s+3) : the 9 field components and J*metric_s on the tile.
// Each consumer thread keeps the velocities and the s-face momentum flux of
// planes s-3..s+3 of its point in registers (the first six read directly at
// the start of a chunk, then one pushed per step from the lead tile), so
// the s derivative of a central row needs no shared memory (lead planes
// outside 0..ns-1 load as zeros and are never used: the 12 s closure rows
// take the planes of their stencil that the window holds from it and read
// the at most three others from global memory); the q and r derivatives read the
// main box, the curvilinear q and r fluxes formed once per box point into
// the stage (one mbarrier phase among the consumer threads per step).  The r
// tiles follow the ownership rule of tile_span (the last
// tile is shifted to end on the last point), which keeps every r closure row
// inside tile + halo.  DF, F_out and C are stored directly from registers.
//
// Every mbarrier wait is bounded; a wait that runs out sets *err and the
// thread leaves its loop (the producer first waits, again bounded, for the
// copies it issued).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <utility>

#include "wql_internal.h"
#include "wql_stencil.cuh"

namespace wql {
namespace {

template <bool CURV, bool KAHAN, int FD, int TQ_ = kTmaTQ>
struct TmaTile {
  static constexpr int TQ = TQ_, TR = kTmaTR, NC = TQ * TR;
  // r halo: 3 rows for the central operator, 4 for the upwind pair
  static constexpr int HR = FD ? 4 : 3;
  static constexpr int BQ = TQ + 16, BR = TR + 2 * HR;  // field box: q from q0-8, r from r0-HR
  static constexpr int NCC = CURV ? 7 : 3;         // tile coefficients: 6..12 or lambda, mu, 1/rho
  static constexpr int F_BOX = 9 * BR * BQ;          // words the field box copy delivers
  static constexpr int F_W = (F_BOX + 31) / 32 * 32;  // its slot, padded to 128 bytes
  static constexpr int CA_W = CURV ? 3 * TR * BQ : 0;
  static constexpr int CB_W = CURV ? 3 * BR * TQ : 0;
  static constexpr int CC_W = NCC * NC;
  static constexpr int LF_W = 9 * NC;  // lead fields (FD 1: velocities of s+4, then stresses of s+2)
  static constexpr int LC_W = CURV ? 3 * NC : 0;
  static constexpr int DF_W = 9 * NC;            // rates of the main plane
  // compensation of the main plane: 9 x NC bfloat16 in a slot of whole
  // 128-byte lines
  static constexpr int CK_BOX = KAHAN ? 9 * NC * 2 : 0;  // bytes the copy delivers
  static constexpr int CK_W = (CK_BOX / 4 + 31) / 32 * 32;
  static constexpr int OFF_F = 0;
  static constexpr int OFF_CA = OFF_F + F_W;
  static constexpr int OFF_CB = OFF_CA + CA_W;
  static constexpr int OFF_CC = OFF_CB + CB_W;
  static constexpr int OFF_LF = OFF_CC + CC_W;
  static constexpr int OFF_LC = OFF_LF + LF_W;
  static constexpr int OFF_DF = OFF_LC + LC_W;
  static constexpr int OFF_CK = OFF_DF + DF_W;
  static constexpr int STAGE_W = OFF_CK + CK_W;
  static constexpr unsigned MAIN_BYTES = 4u * (F_BOX + CA_W + CB_W + CC_W + DF_W) + CK_BOX;
  static constexpr unsigned LEAD_BYTES = 4u * (LF_W + LC_W);
  // every sub-buffer starts on a 128-byte boundary
  static_assert(F_W % 32 == 0 && CA_W % 32 == 0 && CB_W % 32 == 0 && CC_W % 32 == 0 && LF_W % 32 == 0 &&
                    LC_W % 32 == 0 && DF_W % 32 == 0 && CK_W % 32 == 0,
                "stage sub-buffers must be multiples of 128 bytes");
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}

// One potentially blocking test of the phase with parity `parity`; the
// thread sleeps in hardware for at most about 0.5 ms before it returns false.
__device__ __forceinline__ bool mbar_try(uint64_t* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity), "r"(500000u)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase of parity `parity` to complete: at most 8192
// blocking tests (a few seconds).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity) {
  for (unsigned i = 0; i < 8192u; ++i)
    if (mbar_try(b, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// s derivative of the six differenced quantities on a closure row (planes
// 0..5 and ns-6..ns-1).  The s window already holds most of the planes a
// closure row reads (planes s-3..s+3 for the central operator; velocities of
// s-2..s+4 and fluxes of s-4..s+2 for the upwind pair); the at most three
// planes of a row outside it are read from global memory.  Each row is a
// separate instantiation (the weights, offsets and window positions are
// compile-time constants, so the window stays in registers); the columns are
// summed in the order of the operator table, zero weights skipped.
template <bool CURV, int FD, int ROW, bool RIGHT, int T>
__device__ __forceinline__ void s_close_col(const VolumeArgs<float>& a, long long p, const float (&qv)[7][6],
                                            float acc[6]) {
  constexpr float wv = (float)s_close_w(FD, RIGHT, false, ROW, T);
  constexpr float wf = (float)s_close_w(FD, RIGHT, true, ROW, T);
  constexpr int off = s_close_off(RIGHT, ROW, T);  // plane offset from s
  constexpr int iv = s_close_vpos(FD, RIGHT, ROW, T), iflux = s_close_fpos(FD, RIGHT, ROW, T);
  const long long np = a.np, pp = p + off * ((long long)a.pq * a.nr);
  const float* F = a.Fin;
  if constexpr (wv != 0.0f) {
    float x[3];
    if constexpr (iv >= 0 && iv <= 6) {
#pragma unroll
      for (int c = 0; c < 3; ++c) x[c] = qv[iv][c];
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) x[c] = F[c * np + pp];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[c] += wv * x[c];
  }
  if constexpr (wf != 0.0f) {
    float x[3];
    if constexpr (iflux >= 0 && iflux <= 6) {
#pragma unroll
      for (int c = 0; c < 3; ++c) x[c] = qv[iflux][3 + c];
    } else if constexpr (CURV) {
      const float a0 = a.coef[6 * np + pp], a1 = a.coef[7 * np + pp], a2 = a.coef[8 * np + pp];
#pragma unroll
      for (int c = 0; c < 3; ++c)
        x[c] = a0 * F[sig(c, 0) * np + pp] + a1 * F[sig(c, 1) * np + pp] + a2 * F[sig(c, 2) * np + pp];
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) x[c] = F[sig(c, 2) * np + pp];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[3 + c] += wf * x[c];
  }
}

template <bool CURV, int FD, int ROW, bool RIGHT, int... T>
__device__ __forceinline__ void s_close_row(const VolumeArgs<float>& a, long long p, const float (&qv)[7][6],
                                            float o[6], std::integer_sequence<int, T...>) {
  float acc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  (s_close_col<CURV, FD, ROW, RIGHT, T>(a, p, qv, acc), ...);
#pragma unroll
  for (int c = 0; c < 6; ++c) o[c] = acc[c];
}

// ks = sbp_kind(s, ns), nonzero: -1..-6 left rows 0..5, 1..6 right rows 0..5.
template <bool CURV, int FD>
__device__ __forceinline__ void s_closure(const VolumeArgs<float>& a, long long p, int ks, const float (&qv)[7][6],
                                          float o[6]) {
  using Cols = std::make_integer_sequence<int, FD ? 10 : 9>;
  switch (ks) {
    case -1: s_close_row<CURV, FD, 0, false>(a, p, qv, o, Cols{}); break;
    case -2: s_close_row<CURV, FD, 1, false>(a, p, qv, o, Cols{}); break;
    case -3: s_close_row<CURV, FD, 2, false>(a, p, qv, o, Cols{}); break;
    case -4: s_close_row<CURV, FD, 3, false>(a, p, qv, o, Cols{}); break;
    case -5: s_close_row<CURV, FD, 4, false>(a, p, qv, o, Cols{}); break;
    case -6: s_close_row<CURV, FD, 5, false>(a, p, qv, o, Cols{}); break;
    case 1: s_close_row<CURV, FD, 0, true>(a, p, qv, o, Cols{}); break;
    case 2: s_close_row<CURV, FD, 1, true>(a, p, qv, o, Cols{}); break;
    case 3: s_close_row<CURV, FD, 2, true>(a, p, qv, o, Cols{}); break;
    case 4: s_close_row<CURV, FD, 3, true>(a, p, qv, o, Cols{}); break;
    case 5: s_close_row<CURV, FD, 4, true>(a, p, qv, o, Cols{}); break;
    default: s_close_row<CURV, FD, 5, true>(a, p, qv, o, Cols{}); break;
  }
}

struct MapArgs {
  CUtensorMap fbox, flead, ca, cb, cc, cl, df, ck, flead2;
};

// The work of one CTA: tile (bx, by) of the block, s chunk bz.
// Ring positions continue from one tile to the next: tb counts the stages
// the CTA has used before this tile (the same count in every thread), so a
// persistent CTA keeps its mbarriers and the producer runs ahead into the
// next tile.  Returns false after a wait ran out (the error word is set).
template <bool CURV, bool KAHAN, int NS, int FD, int TQW = kTmaTQ>
__device__ __forceinline__ bool tma_body(const VolumeArgs<float>& a, const MapArgs& m, int schunk, int bx, int by,
                                         int bz, int& tb) {
  using TL = TmaTile<CURV, KAHAN, FD, TQW>;
  constexpr int TQ = TL::TQ, TR = TL::TR, NC = TL::NC, BQ = TL::BQ, BR = TL::BR, HR = TL::HR;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // 128-byte aligned start, derived from the shared array itself so the
  // compiler keeps every access in the shared address space
  float* sm = reinterpret_cast<float*>(smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u));
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + NS * TL::STAGE_W);
  uint64_t* empty = full + NS;
  uint64_t* fluxbar = empty + NS;  // consumer-only: fluxes of the step written

  const int tid = threadIdx.x;
  const int nq = a.nq, nr = a.nr, ns = a.ns;
  const int q0 = bx * TQ;
  const TileSpan spr = tile_span(by, nr, TR);
  const int r0 = spr.origin;
  const int s_begin = bz * schunk;
  const int s_end = min(ns, s_begin + schunk);
  const int nstep = s_end - s_begin;

  if (tid >= NC) {  // producer warp: one thread issues every copy
    if (tid == NC) {
      for (int t = 0; t < nstep; ++t) {
        const int T = tb + t;
        const int st = T % NS;
        if (T >= NS && !mbar_wait(&empty[st], ((T / NS) & 1) ^ 1)) {
          atomicExch(a.err, 1);
          tb = T;  // stages issued so far, for the final wait on copies in flight
          return false;
        }
        const int sp = s_begin + t;  // main plane
        mbar_expect_tx(&full[st], TL::LEAD_BYTES + TL::MAIN_BYTES);
        float* S = sm + st * TL::STAGE_W;
        if (FD) {  // velocities of plane s+4, stresses and J*metric_s of plane s+2
          tma_load_4d(S + TL::OFF_LF, &m.flead, &full[st], q0, r0, sp + 4, 0);
          tma_load_4d(S + TL::OFF_LF + 3 * NC, &m.flead2, &full[st], q0, r0, sp + 2, 3);
          if (CURV) tma_load_4d(S + TL::OFF_LC, &m.cl, &full[st], q0, r0, sp + 2, 6);
        } else {
          tma_load_4d(S + TL::OFF_LF, &m.flead, &full[st], q0, r0, sp + 3, 0);
          if (CURV) tma_load_4d(S + TL::OFF_LC, &m.cl, &full[st], q0, r0, sp + 3, 6);
        }
        tma_load_4d(S + TL::OFF_F, &m.fbox, &full[st], q0 - 8, r0 - HR, sp, 0);
        tma_load_4d(S + TL::OFF_DF, &m.df, &full[st], q0, r0, sp, 0);
        if (KAHAN) tma_load_4d(S + TL::OFF_CK, &m.ck, &full[st], q0, r0, sp, 0);
        if (CURV) {
          tma_load_4d(S + TL::OFF_CA, &m.ca, &full[st], q0 - 8, r0, sp, 0);
          tma_load_4d(S + TL::OFF_CB, &m.cb, &full[st], q0, r0 - HR, sp, 3);
          tma_load_4d(S + TL::OFF_CC, &m.cc, &full[st], q0, r0, sp, 6);
        } else {
          tma_load_4d(S + TL::OFF_CC, &m.cc, &full[st], q0, r0, sp, 0);
        }
      }
    }
    tb += nstep;
    return true;
  }

  // ---- consumers: one thread per (q, r) point of the tile
  const int tx = tid % TQ, ty = tid / TQ;
  const int q = q0 + tx, r = r0 + ty;
  const bool own = q < nq && r >= spr.own_lo && r < spr.own_hi;
  const int kq = sbp_kind(q, nq), kr = sbp_kind(r, nr);
  // PML points (every point with the anelastic response) hand their
  // velocity gradient to the correction kernels (a.G)
  const int npml = a.npml;
  const bool pml_qr = a.G != nullptr && ((a.pml[0] && q < npml) || (a.pml[1] && q >= nq - npml) ||
                                         (a.pml[2] && r < npml) || (a.pml[3] && r >= nr - npml));
  const long long np = a.np;
  const long long sts = (long long)a.pq * nr;
  const long long col = q + (long long)a.pq * r;
  const int lq = tx + 8, lr = ty + HR;
  const float c1 = float(kC1), c2 = float(kC2), c3 = float(kC3);
  const float cf[7] = WQL_UP_CF;

  // s window: velocities of planes s-3..s+3 and the s-face flux of the same
  // planes (central operator), or velocities of s-2..s+4 and fluxes of
  // s-4..s+2 (upwind pair: the planes D+ and D- read)
  float qv[7][6];
  // the window's first six entries straight from global memory, all loads
  // in flight at once; planes outside the block stay zero (only central
  // rows read the window)
#pragma unroll
  for (int i = 0; i < 7; ++i) {
#pragma unroll
    for (int c = 0; c < 6; ++c) qv[i][c] = 0.0f;
    const int plv = s_begin + (FD ? -2 : -3) + i, pl = s_begin + (FD ? -4 : -3) + i;
    const float* F = a.Fin;
    if (i < 6 && plv >= 0 && plv < ns && q < nq && r < nr) {
      const long long pp = col + sts * plv;
#pragma unroll
      for (int c = 0; c < 3; ++c) qv[i][c] = F[c * np + pp];
    }
    if (i < 6 && pl >= 0 && pl < ns && q < nq && r < nr) {
      const long long pp = col + sts * pl;
      if (CURV) {
        const float a0 = a.coef[6 * np + pp], a1 = a.coef[7 * np + pp], a2 = a.coef[8 * np + pp];
#pragma unroll
        for (int c = 0; c < 3; ++c)
          qv[i][3 + c] = a0 * F[sig(c, 0) * np + pp] + a1 * F[sig(c, 1) * np + pp] + a2 * F[sig(c, 2) * np + pp];
      } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) qv[i][3 + c] = F[sig(c, 2) * np + pp];
      }
    }
  }

  for (int t = 0; t < nstep; ++t) {
    const int T = tb + t;
    const int st = T % NS;
    const int s = s_begin + t;  // output plane
    const bool work = own;
    const int ks = sbp_kind(s, ns);
    const long long p = col + sts * s;
    if (!mbar_wait(&full[st], (T / NS) & 1)) {
      atomicExch(a.err, 2);
      return false;
    }
    const float* S = sm + st * TL::STAGE_W;
    // push the lead plane(s) into the s window
    {
      const float* LF = S + TL::OFF_LF;
      const int li = ty * TQ + tx;
      float f[9];
#pragma unroll
      for (int c = 0; c < 9; ++c) f[c] = LF[c * NC + li];
#pragma unroll
      for (int c = 0; c < 3; ++c) qv[6][c] = f[c];
      if (CURV) {
        const float* LC = S + TL::OFF_LC;
        const float a0 = LC[li], a1 = LC[NC + li], a2 = LC[2 * NC + li];
#pragma unroll
        for (int c = 0; c < 3; ++c) qv[6][3 + c] = a0 * f[sig(c, 0)] + a1 * f[sig(c, 1)] + a2 * f[sig(c, 2)];
      } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) qv[6][3 + c] = f[sig(c, 2)];
      }
    }

    // curvilinear: the q- and r-face momentum fluxes J*metric*sigma of the
    // main plane, formed once per box point and written over the
    // coefficients they come from (CA becomes the q flux on the q-extended
    // rows, CB the r flux on the r-extended columns); each position is
    // handled by one thread, which reads its coefficients first
    float* FB = const_cast<float*>(S) + TL::OFF_F;
    float* CA = const_cast<float*>(S) + TL::OFF_CA;
    float* CB = const_cast<float*>(S) + TL::OFF_CB;
    const float* CC = S + TL::OFF_CC;
    auto fb = [&](int c, int rr, int qq) -> float { return FB[(c * BR + rr) * BQ + qq]; };
    float mq[3] = {0.0f, 0.0f, 0.0f}, mr[3] = {0.0f, 0.0f, 0.0f};  // own J*metric_q, J*metric_r
    if (CURV) {
      auto qflux = [&](int row, int l, float m[3]) {
        float sg[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) sg[c] = fb(3 + c, row + HR, l);
#pragma unroll
        for (int j = 0; j < 3; ++j) m[j] = CA[(j * TR + row) * BQ + l];
#pragma unroll
        for (int c = 0; c < 3; ++c)
          CA[(c * TR + row) * BQ + l] = m[0] * sg[sig(c, 0) - 3] + m[1] * sg[sig(c, 1) - 3] + m[2] * sg[sig(c, 2) - 3];
      };
      auto rflux = [&](int l, int col_, float m[3]) {
        float sg[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) sg[c] = fb(3 + c, l, col_ + 8);
#pragma unroll
        for (int j = 0; j < 3; ++j) m[j] = CB[(j * BR + l) * TQ + col_];
#pragma unroll
        for (int c = 0; c < 3; ++c)
          CB[(c * BR + l) * TQ + col_] = m[0] * sg[sig(c, 0) - 3] + m[1] * sg[sig(c, 1) - 3] + m[2] * sg[sig(c, 2) - 3];
      };
      qflux(ty, lq, mq);
      rflux(lr, tx, mr);
      float tmp[3];
      if (tx < 16) qflux(ty, tx < 8 ? tx : tx + TQ, tmp);     // q halo: 8 columns each side
      if (ty < 2 * HR) rflux(ty < HR ? ty : ty + TR, tx, tmp);  // r halo: HR rows each side
      // a warp forms every q flux of its own row (the q derivative needs
      // only those: warp sync); the r fluxes of other rows come from other
      // warps: every consumer thread arrives here and waits (bounded) just
      // before the r derivative, so the q and s derivatives overlap the wait
      __syncwarp();
      mbar_arrive(fluxbar);
    }

    if (work) {
      // differenced quantities along q at box column l (row lr) and along r at box row l (column lq)
      auto qvals = [&](int l, float o[6]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) o[c] = fb(c, lr, l);
#pragma unroll
        for (int c = 0; c < 3; ++c) o[3 + c] = CURV ? CA[(c * TR + ty) * BQ + l] : fb(sig(c, 0), lr, l);
      };
      auto rvals = [&](int l, float o[6]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) o[c] = fb(c, l, lq);
#pragma unroll
        for (int c = 0; c < 3; ++c) o[3 + c] = CURV ? CB[(c * BR + l) * TQ + tx] : fb(sig(c, 1), l, lq);
      };
      float g[3][3], dv[3];
      const float Jinv = CURV ? CC[3 * NC + ty * TQ + tx] : 1.0f;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int d = k == 0 ? 0 : (k == 1 ? 2 : 1);  // q, s, then r
        if (CURV && k == 2 && !mbar_wait(fluxbar, T & 1)) {
          atomicExch(a.err, 3);
          return false;
        }
        float o[6];
        if (d == 2) {
          if (ks == 0 && FD) {
#pragma unroll
            for (int c = 0; c < 6; ++c) o[c] = 0.0f;
#pragma unroll
            for (int i = 0; i < 7; ++i) {
#pragma unroll
              for (int c = 0; c < 3; ++c) o[c] += cf[i] * qv[i][c];
#pragma unroll
              for (int c = 3; c < 6; ++c) o[c] -= cf[6 - i] * qv[i][c];
            }
          } else if (ks == 0) {
#pragma unroll
            for (int c = 0; c < 6; ++c)
              o[c] = c1 * (qv[4][c] - qv[2][c]) + c2 * (qv[5][c] - qv[1][c]) + c3 * (qv[6][c] - qv[0][c]);
          } else {
            float os[6];
            s_closure<CURV, FD>(a, p, ks, qv, os);
#pragma unroll
            for (int c = 0; c < 6; ++c) o[c] = os[c];
          }
        } else {
          const int kind = d == 0 ? kq : kr;
          const int l0 = d == 0 ? lq : lr;
          if (kind == 0 && FD) {
#pragma unroll
            for (int c = 0; c < 6; ++c) o[c] = 0.0f;
#pragma unroll
            for (int of = -4; of <= 4; ++of) {
              float x[6];
              if (d == 0) qvals(l0 + of, x);
              else rvals(l0 + of, x);
              if (of >= -2)
#pragma unroll
                for (int c = 0; c < 3; ++c) o[c] += cf[of + 2] * x[c];
              if (of <= 2)
#pragma unroll
                for (int c = 3; c < 6; ++c) o[c] -= cf[2 - of] * x[c];
            }
          } else if (kind == 0) {
            float xp[6], xm[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) o[c] = 0.0f;
#pragma unroll
            for (int k = 1; k <= 3; ++k) {
              if (d == 0) {
                qvals(l0 + k, xp);
                qvals(l0 - k, xm);
              } else {
                rvals(l0 + k, xp);
                rvals(l0 - k, xm);
              }
              const float ck = k == 1 ? c1 : (k == 2 ? c2 : c3);
#pragma unroll
              for (int c = 0; c < 6; ++c) o[c] += ck * (xp[c] - xm[c]);
            }
          } else {
#pragma unroll
            for (int c = 0; c < 6; ++c) o[c] = 0.0f;
#pragma unroll 1
            for (int e = 0; e < (FD ? 10 : 9); ++e) {
              float w, wf;
              int off;
              if (FD) {
                up_entry<float>(kind, e, w, wf, off);
              } else {
                row_entry<float>(kind, e, w, off);
                wf = w;
              }
              float x[6];
              if (d == 0) qvals(l0 + off, x);
              else rvals(l0 + off, x);
#pragma unroll
              for (int c = 0; c < 3; ++c) o[c] += w * x[c];
#pragma unroll
              for (int c = 3; c < 6; ++c) o[c] += wf * x[c];
            }
          }
        }
        const float rh = a.rh[d];
        if (CURV) {
          float mt[3];
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) {
            const float cj = d == 0 ? mq[jj] : (d == 1 ? mr[jj] : CC[jj * NC + ty * TQ + tx]);
            mt[jj] = cj * Jinv;
          }
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            dv[c] = k == 0 ? rh * o[3 + c] : dv[c] + rh * o[3 + c];
#pragma unroll
            for (int jj = 0; jj < 3; ++jj) g[c][jj] = k == 0 ? mt[jj] * (rh * o[c]) : g[c][jj] + mt[jj] * (rh * o[c]);
          }
        } else {
          const float sc = a.cart_metric[d] * rh;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            dv[c] = k == 0 ? sc * o[3 + c] : dv[c] + sc * o[3 + c];
            g[c][d] = sc * o[c];
          }
        }
      }
      if (a.G != nullptr && (a.anel || pml_qr || (a.pml[4] && s < npml) || (a.pml[5] && s >= ns - npml))) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) a.G[(c * 3 + jj) * np + p] = g[c][jj];
      }
      const int ci = ty * TQ + tx;
      const float lam = CURV ? CC[4 * NC + ci] : CC[0 * NC + ci];
      const float mu = CURV ? CC[5 * NC + ci] : CC[1 * NC + ci];
      const float rinv = CURV ? CC[6 * NC + ci] : CC[2 * NC + ci];
      const float l2m = lam + 2.0f * mu;
      float du[9];
      du[0] = rinv * dv[0];
      du[1] = rinv * dv[1];
      du[2] = rinv * dv[2];
      du[3] = l2m * g[0][0] + lam * (g[1][1] + g[2][2]);
      du[4] = l2m * g[1][1] + lam * (g[0][0] + g[2][2]);
      du[5] = l2m * g[2][2] + lam * (g[0][0] + g[1][1]);
      du[6] = mu * (g[0][1] + g[1][0]);
      du[7] = mu * (g[0][2] + g[2][0]);
      du[8] = mu * (g[1][2] + g[2][1]);
      // the face pre-kernel has folded the boundary and fault penalties
      // into DF of the face points: DF - tot/A, or -tot on the first stage
      // (A = 0, where DF holds nothing else)
      const bool face = q == 0 || q == nq - 1 || r == 0 || r == nr - 1 || s == 0 || s == ns - 1;
#pragma unroll
      for (int c = 0; c < 9; ++c) {
        const float f0 = fb(c, lr, lq);
        const float dfs = S[TL::OFF_DF + c * NC + ty * TQ + tx];
        const float df = a.A != 0.0f ? a.A * dfs + du[c] : (face ? dfs : 0.0f) + du[c];
        a.DF[c * np + p] = df;
        if (KAHAN) {
          const comp_t* CKs = reinterpret_cast<const comp_t*>(S + TL::OFF_CK);
          const float y = a.Bdt * df - comp_get(CKs, c * NC + ty * TQ + tx);
          const float tt = f0 + y;
          comp_put(a.C, c * np + p, (tt - f0) - y);
          a.Fout[c * np + p] = tt;
        } else {
          a.Fout[c * np + p] = f0 + a.Bdt * df;
        }
      }
    } else if (CURV && !mbar_wait(fluxbar, T & 1)) {  // the same phase for threads without a point
      atomicExch(a.err, 3);
      return false;
    }
    // order this thread's shared-memory writes (the fluxes) before the
    // producer's next bulk copy into the stage
    if (CURV) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncwarp();
    if ((tid & 31) == 0) mbar_arrive(&empty[st]);
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int c = 0; c < 6; ++c) qv[i][c] = qv[i + 1][c];
  }
  tb += nstep;
  return true;
}

// Shared-memory ring of a persistent CTA: NS stages then the mbarriers.
template <bool CURV, bool KAHAN, int NS, int FD, int TQW = kTmaTQ>
struct Ring {
  float* sm;
  uint64_t *full, *empty, *fluxbar;
  __device__ Ring() {
    using TL = TmaTile<CURV, KAHAN, FD, TQW>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    sm = reinterpret_cast<float*>(smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u));
    full = reinterpret_cast<uint64_t*>(sm + NS * TL::STAGE_W);
    empty = full + NS;
    fluxbar = empty + NS;
  }
  // one thread initialises the barriers once per CTA
  __device__ void init() {
    using TL = TmaTile<CURV, KAHAN, FD, TQW>;
    if (threadIdx.x == 0) {
      for (int i = 0; i < NS; ++i) {
        mbar_init(&full[i], 1);
        mbar_init(&empty[i], TL::NC / 32);
      }
      mbar_init(fluxbar, TL::NC);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
  }
  // the producer's copies of the last stages land before the CTA leaves
  // (tb = stages issued)
  __device__ void drain(int tb) {
    if (threadIdx.x == TmaTile<CURV, KAHAN, FD, TQW>::NC)
      for (int T = max(0, tb - NS); T < tb; ++T) mbar_wait(&full[T % NS], (T / NS) & 1);
  }
};

// Each CTA takes tiles w = blockIdx.x, blockIdx.x + gridDim.x, ... of the
// tq x tr x nchunk tiles of the block (q fastest, so neighbouring CTAs share
// halos in L2); with one CTA per tile that is one tile each.
template <bool CURV, bool KAHAN, int NS, int FD, int TQW>
__global__ void __launch_bounds__(TQW * kTmaTR + 32, 1)
    stencil_kernel_tma(const __grid_constant__ VolumeArgs<float> a, const __grid_constant__ MapArgs m, int schunk,
                       int tq, int tr, int ntile) {
  Ring<CURV, KAHAN, NS, FD, TQW> ring;
  ring.init();
  int tb = 0;
  for (int w = blockIdx.x; w < ntile; w += gridDim.x)
    if (!tma_body<CURV, KAHAN, NS, FD, TQW>(a, m, schunk, w % tq, (w / tq) % tr, w / (tq * tr), tb)) break;
  ring.drain(tb);
}

// One launch over many blocks (of one or many scenarios): CTA i works on the
// descriptor whose CTA range holds i, found by binary search in the packed
// table (descriptors sorted by cta0).
template <bool CURV, bool KAHAN, int NS>
__global__ void __launch_bounds__(kTmaTQ * kTmaTR + 32, 1)
    stencil_kernel_tma_batch(const TmaBatchDesc* __restrict__ d, int nd, long long total) {
  // the entry's arguments are copied to shared memory: read from there they
  // cost no registers across the plane loop (held in registers they spill)
  __shared__ VolumeArgs<float> sa;
  Ring<CURV, KAHAN, NS, 0> ring;
  const long long cta = blockIdx.x;
  int lo = 0, hi = nd - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (d[mid].cta0 <= cta) lo = mid;
    else hi = mid - 1;
  }
  const TmaBatchDesc& D = d[lo];
  {
    const int* src = reinterpret_cast<const int*>(&D.a);
    int* dst = reinterpret_cast<int*>(&sa);
    for (int i = threadIdx.x; i < (int)(sizeof(VolumeArgs<float>) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  }
  // the table was written by a host copy: order that write before the
  // tensor-map proxy reads the entry's maps (in the thread that issues copies)
  if (threadIdx.x == kTmaTQ * kTmaTR)
    for (int i = 0; i < 9; ++i)
      asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"(&D.m[i]) : "memory");
  ring.init();  // its barrier also publishes sa
  int tb = 0;
  const long long l = cta - D.cta0;
  tma_body<CURV, KAHAN, NS, 0>(sa, *reinterpret_cast<const MapArgs*>(&D.m), D.schunk, (int)(l % D.tq),
                            (int)((l / D.tq) % D.tr), (int)(l / ((long long)D.tq * D.tr)), tb);
  ring.drain(tb);
}

// Both blocks of a scenario in one launch: CTAs [0, ntile0) take block 0's
// tiles, the rest block 1's.  The arguments stay kernel parameters (two
// inlined copies of the tile code, each with its own constant offsets), so
// the block pair costs what two single launches cost minus one launch tail.
struct TwoBlocks {
  VolumeArgs<float> a[2];
  MapArgs m[2];
  int schunk[2], tq[2], tr[2];
  int ntile0;
};

template <bool CURV, bool KAHAN, int NS, int FD, int TQW>
__global__ void __launch_bounds__(TQW * kTmaTR + 32, 1)
    stencil_kernel_tma2(const __grid_constant__ TwoBlocks P) {
  Ring<CURV, KAHAN, NS, FD, TQW> ring;
  ring.init();
  int tb = 0;
  const int w = blockIdx.x;
  if (w < P.ntile0) {
    tma_body<CURV, KAHAN, NS, FD, TQW>(P.a[0], P.m[0], P.schunk[0], w % P.tq[0], (w / P.tq[0]) % P.tr[0],
                              w / (P.tq[0] * P.tr[0]), tb);
  } else {
    const int l = w - P.ntile0;
    tma_body<CURV, KAHAN, NS, FD, TQW>(P.a[1], P.m[1], P.schunk[1], l % P.tq[1], (l / P.tq[1]) % P.tr[1],
                              l / (P.tq[1] * P.tr[1]), tb);
  }
  ring.drain(tb);
}

// Planes per s chunk of a single-block launch: the tuned value, else 32.
int chunk_planes(const VolumeArgs<float>& a) {
  if (a.schunk > 0) return a.schunk;
  return 32;
}

int sm_count() {
  static int n[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 152;
  if (!n[dev] && cudaDeviceGetAttribute(&n[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) n[dev] = 152;
  return n[dev];
}

// Chunk length for a launch over both blocks with `tiles[b]` (q, r) tiles
// each: 32 planes while that gives at least 8 waves of one CTA per SM, else
// shorter chunks (down to 12 planes) for more CTAs.  Measured per launch
// (planes per chunk: ms): 2 x 201^3 curvilinear, 1666 CTAs at 32 planes,
// 16: 0.904, 24: 0.902, 32: 0.891; 2 x 401x201x201, 3094 CTAs at 32,
// 16: 1.829, 24: 1.782, 32: 1.765; 2 x 76x101x151 Cartesian upwind, 270 CTAs
// at 32, 12: 0.173, 16: 0.176, 24: 0.197, 32: 0.194.  Equal-length chunks
// (29 planes on 201) measured slower than 32 with a short last chunk.
int chunk_planes2(const VolumeArgs<float>* const a[2], const int tiles[2]) {
  if (a[0]->schunk > 0) return a[0]->schunk;
  const long long want = 8LL * sm_count();
  int c = 32;
  for (; c > 12; c -= 4) {
    long long ncta = 0;
    for (int b = 0; b < 2; ++b) ncta += (long long)tiles[b] * ((a[b]->ns + c - 1) / c);
    if (ncta >= want) break;
  }
  return c;
}

MapArgs stage_maps(const StencilMaps& sm) {
  MapArgs m;
  m.fbox = sm.fbox[sm.cur];
  m.flead = sm.flead[sm.cur];
  m.ca = sm.ca;
  m.cb = sm.cb;
  m.cc = sm.cc;
  m.cl = sm.cl;
  m.df = sm.df;
  m.ck = sm.ck;
  m.flead2 = sm.flead2[sm.cur];
  return m;
}

template <bool CURV, bool KAHAN, int FD, int TQW = kTmaTQ>
constexpr size_t tma_smem_bytes(int NS) {
  return sizeof(float) * (size_t)NS * TmaTile<CURV, KAHAN, FD, TQW>::STAGE_W + (2 * NS + 1) * sizeof(uint64_t) + 128;
}
static_assert(tma_smem_bytes<true, true, 0>(kTmaStages) <= 227 * 1024 &&
                  tma_smem_bytes<false, true, 0>(kTmaStages) <= 227 * 1024 &&
                  tma_smem_bytes<true, true, 1>(kTmaStages) <= 227 * 1024 &&
                  tma_smem_bytes<false, true, 1>(kTmaStages) <= 227 * 1024,
              "the stage ring must fit in the shared memory of one CTA");
static_assert(tma_smem_bytes<false, true, 0, kTmaTQWide>(kTmaStages) <= 227 * 1024 &&
                  tma_smem_bytes<false, true, 1, kTmaTQWide>(kTmaStages) <= 227 * 1024,
              "the wide Cartesian stage ring must fit in the shared memory of one CTA");

template <typename K>
size_t prepare(K kern, int NS, int stage_words) {
  const size_t smem = sizeof(float) * (size_t)NS * stage_words + (2 * NS + 1) * sizeof(uint64_t) + 128;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return smem;
}

// Grid: one CTA per tile.  The kernels also run persistently (fewer CTAs,
// each taking tiles in turn with its ring and barriers kept), but with the
// tiles statically interleaved that measured slower on 2 x 201^3 blocks
// (0.54 ms against 0.50 ms per launch): the chunks holding the s closure
// rows take longer, and the hardware's dynamic CTA scheduling balances them.
template <bool CURV, bool KAHAN, int NS, int FD, int TQW = kTmaTQ>
void launch_tma(const VolumeArgs<float>& a, const StencilMaps& sm, cudaStream_t s) {
  using TL = TmaTile<CURV, KAHAN, FD, TQW>;
  auto kern = stencil_kernel_tma<CURV, KAHAN, NS, FD, TQW>;
  static const size_t smem = prepare(kern, NS, TL::STAGE_W);
  const int tq = (a.nq + TL::TQ - 1) / TL::TQ, tr = (a.nr + TL::TR - 1) / TL::TR;
  const int schunk = chunk_planes(a);
  const int ntile = tq * tr * ((a.ns + schunk - 1) / schunk);
  kern<<<ntile, TL::NC + 32, smem, s>>>(a, stage_maps(sm), schunk, tq, tr, ntile);
}

template <bool CURV, bool KAHAN, int NS, int FD, int TQW = kTmaTQ>
void launch_tma2(const VolumeArgs<float>& a0, const VolumeArgs<float>& a1, cudaStream_t s) {
  using TL = TmaTile<CURV, KAHAN, FD, TQW>;
  auto kern = stencil_kernel_tma2<CURV, KAHAN, NS, FD, TQW>;
  static const size_t smem = prepare(kern, NS, TL::STAGE_W);
  TwoBlocks P;
  const VolumeArgs<float>* a[2] = {&a0, &a1};
  int ntile[2];
  int tiles[2];
  for (int b = 0; b < 2; ++b) {
    P.a[b] = *a[b];
    P.m[b] = stage_maps(*static_cast<const StencilMaps*>(a[b]->tma));
    P.tq[b] = (a[b]->nq + TL::TQ - 1) / TL::TQ;
    P.tr[b] = (a[b]->nr + TL::TR - 1) / TL::TR;
    tiles[b] = P.tq[b] * P.tr[b];
  }
  const int c = chunk_planes2(a, tiles);
  for (int b = 0; b < 2; ++b) {
    P.schunk[b] = a[b]->schunk > 0 ? a[b]->schunk : c;
    ntile[b] = tiles[b] * ((a[b]->ns + P.schunk[b] - 1) / P.schunk[b]);
  }
  P.ntile0 = ntile[0];
  kern<<<ntile[0] + ntile[1], TL::NC + 32, smem, s>>>(P);
}

template <bool CURV, bool KAHAN, int NS>
void launch_tma_batch(const TmaBatchDesc* d, int nd, long long total, cudaStream_t s) {
  using TL = TmaTile<CURV, KAHAN, 0>;
  auto kern = stencil_kernel_tma_batch<CURV, KAHAN, NS>;
  static const size_t smem = prepare(kern, NS, TL::STAGE_W);
  if (total <= 0) return;
  kern<<<(unsigned)total, TL::NC + 32, smem, s>>>(d, nd, total);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

// 4-D map over (q, r, s, component) of an FP32 array (bf16: of a bfloat16
// array) with row pitch pq.
int encode4(CUtensorMap* map, void* base, int nq, int nr, int ns, int ncomp, int pq, int bq, int br, int bc,
            bool bf16 = false) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return 1;
  const long long np = (long long)pq * nr * ns;
  const cuuint64_t es = bf16 ? 2 : 4;
  cuuint64_t dims[4] = {(cuuint64_t)nq, (cuuint64_t)nr, (cuuint64_t)ns, (cuuint64_t)ncomp};
  cuuint64_t strides[3] = {(cuuint64_t)pq * es, (cuuint64_t)pq * nr * es, (cuuint64_t)np * es};
  cuuint32_t box[4] = {(cuuint32_t)bq, (cuuint32_t)br, 1, (cuuint32_t)bc};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = fn(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims,
                  strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return (int)r;
}

}  // namespace

int make_stencil_maps(StencilMaps& m, void* const F[2], void* coef, void* DF, void* C, int nq, int nr, int ns, int pq,
                      bool curv, int fd, int tq) {
  const int TQ = (tq == kTmaTQWide && !curv) ? kTmaTQWide : kTmaTQ, TR = kTmaTR;
  const int hr = fd ? 4 : 3;  // r halo rows
  int rc = 0;
  m.ok = 0;
  m.cur = 0;
  m.fd = fd;
  m.tq = TQ;
  for (int i = 0; i < 2 && !rc; ++i) {
    rc = encode4(&m.fbox[i], F[i], nq, nr, ns, 9, pq, TQ + 16, TR + 2 * hr, 9);
    // lead tiles: all 9 components of one plane, or (upwind) the 3
    // velocities and, from another plane, the 6 stresses
    if (!rc) rc = encode4(&m.flead[i], F[i], nq, nr, ns, 9, pq, TQ, TR, fd ? 3 : 9);
    if (!rc && fd) rc = encode4(&m.flead2[i], F[i], nq, nr, ns, 9, pq, TQ, TR, 6);
    if (!fd) m.flead2[i] = m.flead[i];
  }
  if (!rc) rc = encode4(&m.df, DF, nq, nr, ns, 9, pq, TQ, TR, 9);
  // the compensation is bfloat16 (without one the map is never read)
  if (!rc) rc = encode4(&m.ck, C ? C : DF, nq, nr, ns, 9, pq, TQ, TR, 9, true);
  if (curv) {
    if (!rc) rc = encode4(&m.ca, coef, nq, nr, ns, kCurvCoef, pq, TQ + 16, TR, 3);
    if (!rc) rc = encode4(&m.cb, coef, nq, nr, ns, kCurvCoef, pq, TQ, TR + 2 * hr, 3);
    if (!rc) rc = encode4(&m.cc, coef, nq, nr, ns, kCurvCoef, pq, TQ, TR, 7);
    if (!rc) rc = encode4(&m.cl, coef, nq, nr, ns, kCurvCoef, pq, TQ, TR, 3);
  } else {
    if (!rc) rc = encode4(&m.cc, coef, nq, nr, ns, kCartCoef, pq, TQ, TR, 3);
    m.ca = m.cb = m.cl = m.cc;
  }
  m.ok = rc == 0;
  return rc;
}

long long fill_tma_desc(const VolumeArgs<float>& a, TmaBatchDesc& d) {
  static_assert(sizeof(MapArgs) == sizeof(d.m), "map set layout");
  const StencilMaps& sm = *static_cast<const StencilMaps*>(a.tma);
  const MapArgs m = stage_maps(sm);
  std::memcpy(d.m, &m, sizeof(m));
  d.a = a;
  d.schunk = chunk_planes(a);
  d.tq = (a.nq + kTmaTQ - 1) / kTmaTQ;
  d.tr = (a.nr + kTmaTR - 1) / kTmaTR;
  d.nchunk = (a.ns + d.schunk - 1) / d.schunk;
  d.cta0 = 0;
  return (long long)d.tq * d.tr * d.nchunk;
}

bool tma_eligible(const VolumeArgs<float>& a) {
  // the packed launch runs the central operator on 32-wide tiles; tile_span
  // keeps every r closure row inside tile + halo unless the shifted last
  // tile starts at 4 or 5
  return a.tma != nullptr && a.fd == 0 && static_cast<const StencilMaps*>(a.tma)->tq == kTmaTQ &&
         (a.nr <= kTmaTR + 3 || a.nr >= kTmaTR + 6);
}

int tma_tile_width(int nq0, int nq1, bool curv) {
  if (curv) return kTmaTQ;
  auto used = [&](int T) { return (double)(nq0 + nq1) / (double)(((nq0 + T - 1) / T + (nq1 + T - 1) / T) * T); };
  return used(kTmaTQWide) > used(kTmaTQ) + 0.02 ? kTmaTQWide : kTmaTQ;
}

void launch_stencil_tma_batch(const TmaBatchDesc* d, int nd, long long total, bool curv, bool kahan, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (curv) kahan ? launch_tma_batch<true, true, kTmaStages>(d, nd, total, s)
                  : launch_tma_batch<true, false, kTmaStages>(d, nd, total, s);
  else kahan ? launch_tma_batch<false, true, kTmaStages>(d, nd, total, s)
             : launch_tma_batch<false, false, kTmaStages>(d, nd, total, s);
}

// The upwind pair runs with the compensated update only (the FP32 mode
// always carries C); stencil_is_tma sends an uncompensated upwind block to
// the per-point kernel.
void launch_stencil_tma2(const VolumeArgs<float>& a0, const VolumeArgs<float>& a1, bool curv, bool kahan,
                         void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (!curv && kahan && static_cast<const StencilMaps*>(a0.tma)->tq == kTmaTQWide) {
    if (a0.fd) launch_tma2<false, true, kTmaStages, 1, kTmaTQWide>(a0, a1, s);
    else launch_tma2<false, true, kTmaStages, 0, kTmaTQWide>(a0, a1, s);
    return;
  }
  if (a0.fd) {
    if (curv) launch_tma2<true, true, kTmaStages, 1>(a0, a1, s);
    else launch_tma2<false, true, kTmaStages, 1>(a0, a1, s);
    return;
  }
  if (curv) kahan ? launch_tma2<true, true, kTmaStages, 0>(a0, a1, s) : launch_tma2<true, false, kTmaStages, 0>(a0, a1, s);
  else kahan ? launch_tma2<false, true, kTmaStages, 0>(a0, a1, s) : launch_tma2<false, false, kTmaStages, 0>(a0, a1, s);
}

void launch_stencil_tma(const VolumeArgs<float>& a, bool curv, bool kahan, void* stream) {
  const StencilMaps& sm = *static_cast<const StencilMaps*>(a.tma);
  cudaStream_t s = (cudaStream_t)stream;
  if (!curv && kahan && sm.tq == kTmaTQWide) {
    if (a.fd) launch_tma<false, true, kTmaStages, 1, kTmaTQWide>(a, sm, s);
    else launch_tma<false, true, kTmaStages, 0, kTmaTQWide>(a, sm, s);
    return;
  }
  if (a.fd) {
    if (curv) launch_tma<true, true, kTmaStages, 1>(a, sm, s);
    else launch_tma<false, true, kTmaStages, 1>(a, sm, s);
    return;
  }
  if (curv) kahan ? launch_tma<true, true, kTmaStages, 0>(a, sm, s) : launch_tma<true, false, kTmaStages, 0>(a, sm, s);
  else kahan ? launch_tma<false, true, kTmaStages, 0>(a, sm, s) : launch_tma<false, false, kTmaStages, 0>(a, sm, s);
}

}  // namespace wql
