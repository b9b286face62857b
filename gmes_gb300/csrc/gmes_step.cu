// One FDTD time step on the GPU: ghost-plane copies, the fused E and H
// half-step kernels over all material classes, and the point sources.
//
// Reference path replaced (GMES): FDTD.step (gmes/fdtd.py:1099-1122) with
// talk_with_*_neighbors (gmes/fdtd.py:811-1097), update_e?/h?
// (gmes/fdtd.py:673-809) and the per-point updaters of src/pw_*.hh.
//
// Index geometry.  With N = whole_field_size, every E component is updated
// on the N0 x N1 x N2 "cells" (i, j, k) (the last plane along each non-own
// axis is a ghost, src/pw_dummy.hh semantics via gmes/fdtd.py:365-470), and
// every H component on the same cells shifted by +1 along its two non-own
// axes (its first planes are the ghosts).  One thread owns one cell and
// updates the three components of its half-step there, so each kernel reads
// every neighbouring field value through L1/L2 and writes each updated value
// once.  For component c with own axis a and curl axes a1 = a+1, a2 = a+2
// (mod 3):
//   E_c at x:  D1 = H_{a2}[x + e_a + e_a1] - H_{a2}[x + e_a]
//              D2 = H_{a1}[x + e_a + e_a2] - H_{a1}[x + e_a]
//   H_c at x + e_a1 + e_a2:
//              D1 = E_{a2}[x + e_a1] - E_{a2}[x],  D2 = E_{a1}[x + e_a2] - E_{a1}[x]
// which is exactly the (in1, in2, d1, d2) binding of gmes/fdtd.py:673-809
// and the stencils of src/pw_dielectric.hh:118-371.
#include <cstring>

#include <type_traits>

#include "gmes_internal.cuh"

namespace gmes {
namespace {

// Threads per block of the cell kernels, single-grid and multi-grid:
// kCellThreads (16 cells along k by 8 rows).  Measured on GB300, Gcell/s at
// 128 / 256 / 512 threads (the same registers and resident warps per SM):
//   256^3 cube        FP64 17.34 / 16.70 / 14.97   FP32 33.66 / 33.42   df64 21.80 / 20.98
//   192^3 dispersive  FP64  9.81 /  9.36 /  8.70   FP32 20.26 / 19.85   df64 14.76 / 13.75
// GMES_CELL_THREADS overrides it (tuning builds).
//
// Resident blocks per SM the cell kernels' register budget targets (blocks
// of 128 threads).  Measured on GB300 with the warp-uniform plain path
// (256^3 cube, Gcell/s):
//   FP64  7 blocks (72 registers) 17.29   8 (64) 18.48   9 (56) 18.90
//   FP32  10 blocks (48) 34.31           11 (46) 39.40  12 (40) 39.42
//   df64  7 blocks 20.44                 8 (64) 22.33   9 (56) 22.60  10 (48) 24.19
//   (FP64 at 10 blocks 18.71; FP32 at 14 or 16 blocks, spilling, 35.7)
// FP32 is bound by the loads in flight, so extra resident warps pay most
// there; FP64 is bound by its pipe.  GMES_CELL_BLOCKS_F64 / _F32 / _DF
// override them (tuning builds).
#ifndef GMES_CELL_BLOCKS_F64
#define GMES_CELL_BLOCKS_F64 9
#endif
#ifndef GMES_CELL_BLOCKS_F32
#define GMES_CELL_BLOCKS_F32 12
#endif
#ifndef GMES_CELL_BLOCKS_DF
#define GMES_CELL_BLOCKS_DF 10
#endif
// The H half (GMES_CELL_BLOCKS_F64_H / _F32_H / _DF_H) and the E half of
// dispersive grids (the kernel with the Drude / Lorentz / DCP updates, _D)
// take their own budgets.  Measured on GB300, ms per half-step:
//   df64 H, 256^3 cube, 10 / 9 / 8 blocks: 0.3275 / 0.3403 / 0.3223 (8: 64
//     registers, no spills; at 10 the hot path spilled)
//   dispersive E, 192^3, blocks 12 or 10 (the E budget) / 9 / 8 / 7 / 6:
//     FP32 0.1937 / 0.1701 / 0.1812 / -      / -      (9: no spills)
//     df64 0.2733 / 0.2581 / 0.2693 / 0.2574 / 0.2751
//     FP64 0.4052 (9) / -   / 0.4041 / 0.4035 / 0.4107
//   (FP32 H at 10 blocks and FP64 H at 8 ran 1-2 % slower than their E
//   budgets.  Re-measured with these: 256^3 cube df64 E at 8 blocks 0.329
//   vs 0.316; FP32 E / H at 9 or 8 blocks 0.230 / 0.254 vs 0.203 / 0.205,
//   H alone at 9 0.254; FP64 E at 8 0.4485 vs 0.4435, H at 7 0.4638 vs
//   0.4428.)
#ifndef GMES_CELL_BLOCKS_F64_H
#define GMES_CELL_BLOCKS_F64_H GMES_CELL_BLOCKS_F64
#endif
#ifndef GMES_CELL_BLOCKS_F32_H
#define GMES_CELL_BLOCKS_F32_H GMES_CELL_BLOCKS_F32
#endif
#ifndef GMES_CELL_BLOCKS_DF_H
#define GMES_CELL_BLOCKS_DF_H 8
#endif
#ifndef GMES_CELL_BLOCKS_F64_D
#define GMES_CELL_BLOCKS_F64_D 7
#endif
#ifndef GMES_CELL_BLOCKS_F32_D
#define GMES_CELL_BLOCKS_F32_D 9
#endif
#ifndef GMES_CELL_BLOCKS_DF_D
#define GMES_CELL_BLOCKS_DF_D 9
#endif
constexpr int cell_blocks(int e, int h, int d, int side, bool disp) {
  return (side == 1 ? h : (disp ? d : e)) * 128 / kCellThreads;
}
template <class P, int SIDE, bool DISP>
struct CellMinBlocks {
  static constexpr int value = cell_blocks(GMES_CELL_BLOCKS_F64, GMES_CELL_BLOCKS_F64_H,
                                           GMES_CELL_BLOCKS_F64_D, SIDE, DISP);
};
template <int SIDE, bool DISP>
struct CellMinBlocks<PolF32, SIDE, DISP> {
  static constexpr int value = cell_blocks(GMES_CELL_BLOCKS_F32, GMES_CELL_BLOCKS_F32_H,
                                           GMES_CELL_BLOCKS_F32_D, SIDE, DISP);
};
template <int SIDE, bool DISP>
struct CellMinBlocks<PolDF, SIDE, DISP> {
  static constexpr int value = cell_blocks(GMES_CELL_BLOCKS_DF, GMES_CELL_BLOCKS_DF_H,
                                           GMES_CELL_BLOCKS_DF_D, SIDE, DISP);
};
// The multi-grid cell kernels carry a tile loop and a grid look-up on top of
// the cell body (GMES_MULTI_BLOCKS_F64 / _F32 / _DF override the budgets).
// Measured on GB300 (one 160^3 cube in a batch, descriptors as launch
// arguments, ms per step): FP32 at 8 / 10 / 12 blocks 0.203 / 0.174 / 0.187;
// FP64 at 7 / 8 / 9 blocks 0.304 / 0.302 / 0.292.  Re-measured with chunks
// replayed as CUDA graphs and the tile range from the host: FP32 at 10 / 12
// blocks 0.158 / 0.164; df64 at 9 / 10 / 12 blocks 0.224 / 0.236 / 0.246.
#ifndef GMES_MULTI_BLOCKS_F64
#define GMES_MULTI_BLOCKS_F64 9
#endif
#ifndef GMES_MULTI_BLOCKS_F32
#define GMES_MULTI_BLOCKS_F32 10
#endif
#ifndef GMES_MULTI_BLOCKS_DF
#define GMES_MULTI_BLOCKS_DF 9
#endif
// The H half (_H) and the E half of dispersive grids (_D) may take their
// own budgets; by default the precision's.  (FP64, 34 grids of the serving
// mix below 2^20 cells, 25 of them dispersive, ms per 64-step chunk: 141.5
// at 9 blocks; H at 8 / 7 blocks 143.6 / 146.5, dispersive E at 7 145.1.)
#ifndef GMES_MULTI_BLOCKS_F64_H
#define GMES_MULTI_BLOCKS_F64_H GMES_MULTI_BLOCKS_F64
#endif
#ifndef GMES_MULTI_BLOCKS_F32_H
#define GMES_MULTI_BLOCKS_F32_H GMES_MULTI_BLOCKS_F32
#endif
#ifndef GMES_MULTI_BLOCKS_DF_H
#define GMES_MULTI_BLOCKS_DF_H GMES_MULTI_BLOCKS_DF
#endif
#ifndef GMES_MULTI_BLOCKS_F64_D
#define GMES_MULTI_BLOCKS_F64_D GMES_MULTI_BLOCKS_F64
#endif
#ifndef GMES_MULTI_BLOCKS_F32_D
#define GMES_MULTI_BLOCKS_F32_D GMES_MULTI_BLOCKS_F32
#endif
#ifndef GMES_MULTI_BLOCKS_DF_D
#define GMES_MULTI_BLOCKS_DF_D GMES_MULTI_BLOCKS_DF
#endif
template <class P, int SIDE, bool DISP>
struct MultiMinBlocks {
  static constexpr int value = cell_blocks(GMES_MULTI_BLOCKS_F64, GMES_MULTI_BLOCKS_F64_H,
                                           GMES_MULTI_BLOCKS_F64_D, SIDE, DISP);
};
template <int SIDE, bool DISP>
struct MultiMinBlocks<PolF32, SIDE, DISP> {
  static constexpr int value = cell_blocks(GMES_MULTI_BLOCKS_F32, GMES_MULTI_BLOCKS_F32_H,
                                           GMES_MULTI_BLOCKS_F32_D, SIDE, DISP);
};
template <int SIDE, bool DISP>
struct MultiMinBlocks<PolDF, SIDE, DISP> {
  static constexpr int value = cell_blocks(GMES_MULTI_BLOCKS_DF, GMES_MULTI_BLOCKS_DF_H,
                                           GMES_MULTI_BLOCKS_DF_D, SIDE, DISP);
};
// Whether a batch of at most kParamJobs grids takes its descriptors from
// the argument bank (k_multi_cell_arg) or copies them to shared memory per
// block (k_multi_cell); GMES_MULTI_ARG_F64 / _F32 / _DF override it.
// Measured on GB300 (one 160^3 cube in a batch, ms per step, argument bank
// / shared memory, single-grid kernel): FP32 0.173 / 0.194 (0.148), df64
// 0.266 / 0.290 (0.220), FP64 0.289 / 0.279 (0.265).
#ifndef GMES_MULTI_ARG_F64
#define GMES_MULTI_ARG_F64 0
#endif
#ifndef GMES_MULTI_ARG_F32
#define GMES_MULTI_ARG_F32 1
#endif
#ifndef GMES_MULTI_ARG_DF
#define GMES_MULTI_ARG_DF 1
#endif
template <class P>
struct ArgDescs {
  static constexpr bool value = GMES_MULTI_ARG_F64 != 0;
};
template <>
struct ArgDescs<PolF32> {
  static constexpr bool value = GMES_MULTI_ARG_F32 != 0;
};
template <>
struct ArgDescs<PolDF> {
  static constexpr bool value = GMES_MULTI_ARG_DF != 0;
};

template <int C>
__device__ __forceinline__ int64_t stride_of(const GridDev& g, int axis) {
  return axis == 0 ? g.st[C][0] : (axis == 1 ? g.st[C][1] : 1);
}

// ---------------------------------------------------------------------------
// Per-point update, fast form: precomputed reciprocals, FMA contraction
// allowed (FP64, FP32) or float-float arithmetic (DF64).
//   side 0 (E): F += c1 D1 - c2 D2            (Dielectric E)
//   side 1 (H): F += c2 D2 - c1 D1            (Dielectric H)
// ---------------------------------------------------------------------------
// State values of a CPML (psi1, psi2) or UPML (d) point, loaded for all
// three components of a cell before any of them is computed.
template <class P>
struct Pre {
  typename P::R a, b;
};

template <class P, int C>
__device__ __forceinline__ Pre<P> prefetch_state(const GridDev& g, int64_t lin, const int x[3],
                                                 uint8_t id) {
  (void)x;
  Pre<P> r{P::zero(), P::zero()};
  const int kind = __ldg(&g.tab[C][id].kind);
  const typename P::T* aux = static_cast<const typename P::T*>(g.aux[C]);
  if (kind == GMES_KIND_CPML) {
    // loaded unconditionally: testing the profile first (to skip the loads
    // outside the slabs) adds a dependent lookup and measured slower
    r.a = P::ldw(aux + lin);
    r.b = P::ldw(aux + g.npts[C] + lin);
  } else if (kind == GMES_KIND_UPML) {
    r.a = P::ldw(aux + lin);
  }
  return r;
}

// Whether the CPML psi updates run behind a warp-wide vote.  Measured on
// GB300 (256^3 cube): FP64 13.58 -> 14.18 Gcell/s (19.0 -> 17.6 FP64
// instructions per cell) and FP32 31.2 -> 32.7; the float-float type runs
// slower with it (19.6 -> 18.3; with a __syncwarp opening each voted block
// and 16-cell rows, 21.05 -> 20.67).  Votes in front of the other kinds'
// blocks were slower in every precision.
// (The float-float type keeps plain branches in its own CPML block in
// update_fast.)
template <class P>
struct PsiVote {
  static constexpr bool value = true;
};

// Whether a profile entry has kappa == 1 (the default CPML grading,
// kappa_max = 1, and every point outside the slab).
__device__ __forceinline__ bool kappa_one(const Coef* q) {
  return __ldg(reinterpret_cast<const unsigned long long*>(&q[2].d)) == 0x3FF0000000000000ull;
}

// CPML point with kappa == 1 on its live axes, written as the dielectric
// update plus the psi terms:
//   E: F + cdt ((psi1 - psi2) + D1/d1 - D2/d2) = ((F + c1 D1) - c2 D2) + cdt psi1 - cdt psi2
// (c1 = cdt/d1, c2 = cdt/d2), so the dielectric and CPML points of a warp
// share the first two FMAs, and a psi block runs only in warps where some
// lane is inside that axis' slab.  The separate CPML form ran both forms in
// every warp that straddles a slab edge along the contiguous axis.  Points
// with kappa != 1 take the separate form.  A __syncwarp at the top of each
// voted psi block keeps it a branch: without it the compiler predicated
// the blocks and every warp with a CPML lane issued both.  Measured on
// GB300 (256^3 cube, 10-cell CPML), FP64 warp-instructions per cell and
// half-step (E side) and Gcell/s:
//   separate form, psi votes                 17.6   14.23
//   shared form, votes                       16.8   14.93
//   shared form, votes + __syncwarp          14.4   16.17
// 14.4 is what a warp-level count of the slabs predicts when each psi block
// issues only in warps that need it.  FP32 (32.7 -> 30.7 Gcell/s) and the
// float-float type (19.6 -> 18.5) run slower with the shared form, and
// slower with __syncwarp in their own psi votes, so both keep the
// separate form.
template <class P>
struct SharedCpml {
  static constexpr bool value = false;
};
template <>
struct SharedCpml<PolF64> {
  static constexpr bool value = true;
};

// The plain update of a point (a dielectric class, or a CPML point outside
// both of its slabs): E: (F + c1 D1) - c2 D2, H: (F + c2 D2) - c1 D1, with
// both multiply-adds fused explicitly, so that the per-point path, the
// uniform-tile path and the multi-grid kernels round identically.
__device__ __forceinline__ double plain_e(double F, double c1, double c2, double p1, double p2) {
  return __fma_rn(-c2, p2, __fma_rn(c1, p1, F));
}
__device__ __forceinline__ float plain_e(float F, float c1, float c2, float p1, float p2) {
  return __fmaf_rn(-c2, p2, __fmaf_rn(c1, p1, F));
}
__device__ __forceinline__ df plain_e(df F, df c1, df c2, df p1, df p2) {
  return df_fma(-c2, p2, df_fma(c1, p1, F));
}
// A curl difference a - b of neighbouring field values.  Float-float: the
// high words' difference exactly (two-sum), the low words' difference
// added once (11 FP32 operations against 20 for the fully compensated
// difference); its error is about 2^-48 of the operands, the precision the
// float-float values are stored to.
__device__ __forceinline__ double curl_diff(double a, double b) { return a - b; }
__device__ __forceinline__ float curl_diff(float a, float b) { return a - b; }
__device__ __forceinline__ df curl_diff(df a, df b) {
  df s = df_two_sum(a.hi, -b.hi);
  s.lo = __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo));
  return df_fast_two_sum(s.hi, s.lo);
}

template <bool E, class R>
__device__ __forceinline__ R plain_upd(R F, R c1, R c2, R p1, R p2) {
  return E ? plain_e(F, c1, c2, p1, p2) : plain_e(F, c2, c1, p2, p1);
}

// a b + c, fused explicitly, so that the CPML update rounds the same wherever
// it is inlined.
__device__ __forceinline__ double madd(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float madd(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ df madd(df a, df b, df c) { return df_fma(a, b, c); }

// Update of a CPML point in the separate form (src/pw_cpml.hh:115-132 E,
// 327-344 H): psi1 = b1 psi1 + (c1/d1) D1 and psi2 likewise where the point
// is inside that axis' slab (c != 0; elsewhere psi stays exactly 0), then
// F +/- cdt ((psi1 - psi2) + D1/(kappa1 d1) - D2/(kappa2 d2)); a point
// outside both slabs takes the dielectric form.  Per point in update_fast,
// and for warps of one class per component in cell_body_fast.
template <class P, int C>
__device__ __forceinline__ void cpml_separate(const GridDev& g, int64_t lin, const int x[3],
                                              typename P::R p1, typename P::R p2,
                                              typename P::R F, const ClassCoef& cc,
                                              Pre<P> pre) {
  using R = typename P::R;
  using T = typename P::T;
  constexpr int own = C % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  constexpr bool E = C < 3;
  T* fp = static_cast<T*>(g.f[C]) + lin;
  T* aux = static_cast<T*>(g.aux[C]);
  const int64_t np = g.npts[C];
  const int pm = __ldg(&cc.pml);
  const Coef* q1 = g.prof[pm][C][a1] + (int64_t)x[a1] * kProfStride;
  const Coef* q2 = g.prof[pm][C][a2] + (int64_t)x[a2] * kProfStride;
  const bool on1 = coef_nonzero(q1 + 1), on2 = coef_nonzero(q2 + 1);
  if (!on1 && !on2) {
    // outside both slabs kappa = 1 and psi = 0: the dielectric update
    const R c1 = P::cfg(&cc.c1), c2 = P::cfg(&cc.c2);
    P::st(fp, plain_upd<E>(F, c1, c2, p1, p2));
    return;
  }
  R psi1 = pre.a, psi2 = pre.b;
  if constexpr (PsiVote<P>::value) {
    // A warp-wide vote before each psi update: the compiler otherwise
    // predicates the short update blocks, and every warp of the shell then
    // issues their instructions whether or not a lane is in that slab.
    // Each lane still keeps its own value (psi changes only where on).
    const unsigned am = __activemask();
    if (__any_sync(am, on1)) {
      const R n1 = madd(P::cfg(q1 + 3), p1, P::cfg(q1) * psi1);
      if (on1) {
        psi1 = n1;
        P::st(aux + lin, psi1);
      }
    }
    if (__any_sync(am, on2)) {
      const R n2 = madd(P::cfg(q2 + 3), p2, P::cfg(q2) * psi2);
      if (on2) {
        psi2 = n2;
        P::st(aux + np + lin, psi2);
      }
    }
  } else {
    if (on1) {
      psi1 = madd(P::cfg(q1 + 3), p1, P::cfg(q1) * psi1);
      P::st(aux + lin, psi1);
    }
    if (on2) {
      psi2 = madd(P::cfg(q2 + 3), p2, P::cfg(q2) * psi2);
      P::st(aux + np + lin, psi2);
    }
  }
  const R X = madd(-P::cfg(q2 + 4), p2, madd(P::cfg(q1 + 4), p1, psi1 - psi2));
  const R cdt = P::cfg(&cc.cdt);
  P::st(fp, E ? madd(cdt, X, F) : madd(-cdt, X, F));
}

template <class P, int C, bool DISP>
__device__ __forceinline__ void update_fast(const GridDev& g, int64_t lin, const int x[3],
                                            typename P::R p1, typename P::R p2,
                                            typename P::R F, uint8_t id, Pre<P> pre) {
  using R = typename P::R;
  using T = typename P::T;
  constexpr int own = C % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  constexpr bool E = C < 3;
  const ClassCoef& cc = g.tab[C][id];
  const int kind = __ldg(&cc.kind);
  if (kind == GMES_KIND_DUMMY) return;
  T* fp = static_cast<T*>(g.f[C]) + lin;
  if constexpr (SharedCpml<P>::value) {
    if (kind == GMES_KIND_DIELECTRIC || kind == GMES_KIND_CPML) {
      const bool cp = kind == GMES_KIND_CPML;
      // dielectric lanes point their profile entries at valid memory (the
      // class's own coefficients) so that a warp-wide psi block may load
      // them; their results are never used
      const Coef* q1 = &cc.eps;
      const Coef* q2 = &cc.eps;
      bool on1 = false, on2 = false, scaled = false;
      if (cp) {
        const int pm = __ldg(&cc.pml);
        q1 = g.prof[pm][C][a1] + (int64_t)x[a1] * kProfStride;
        q2 = g.prof[pm][C][a2] + (int64_t)x[a2] * kProfStride;
        on1 = coef_nonzero(q1 + 1);
        on2 = coef_nonzero(q2 + 1);
        scaled = (on1 && !kappa_one(q1)) || (on2 && !kappa_one(q2));
      }
      if (!scaled) {
        const R c1 = P::cfg(&(cc.c1)), c2 = P::cfg(&(cc.c2));
        R t = plain_upd<E>(F, c1, c2, p1, p2);
        const unsigned am = __activemask();
        if (__any_sync(am, on1 || on2)) {
          T* aux = static_cast<T*>(g.aux[C]);
          const R cdt = P::cfg(&cc.cdt);
          if (__any_sync(am, on1)) {
            __syncwarp(am);  // keeps the block a branch
            const R n1 = P::cfg(q1) * pre.a + P::cfg(q1 + 3) * p1;
            if (on1) {
              P::st(aux + lin, n1);
              t = E ? t + cdt * n1 : t - cdt * n1;
            }
          }
          if (__any_sync(am, on2)) {
            __syncwarp(am);  // keeps the block a branch
            const R n2 = P::cfg(q2) * pre.b + P::cfg(q2 + 3) * p2;
            if (on2) {
              P::st(aux + g.npts[C] + lin, n2);
              t = E ? t - cdt * n2 : t + cdt * n2;
            }
          }
        }
        P::st(fp, t);
        return;
      }
    }
  }
  if (kind == GMES_KIND_DIELECTRIC) {
    const R c1 = P::cfg(&(cc.c1)), c2 = P::cfg(&(cc.c2));
    P::st(fp, plain_upd<E>(F, c1, c2, p1, p2));
    return;
  }
  T* aux = static_cast<T*>(g.aux[C]);
  const int64_t np = g.npts[C];
  if (kind == GMES_KIND_CPML) {
    if constexpr (!std::is_same<P, PolDF>::value) {
      cpml_separate<P, C>(g, lin, x, p1, p2, F, cc, pre);
    } else {
      // the float-float type keeps this block inline: in cpml_separate it
      // spilled more and ran 1.5 % slower (256^3 cube, 24.21 -> 23.84
      // Gcell/s); the arithmetic is cpml_separate's, term for term (its
      // warp-uniform CPML path takes cpml_separate)
      const Coef* q1 = g.prof[__ldg(&cc.pml)][C][a1] + (int64_t)x[a1] * kProfStride;
      const Coef* q2 = g.prof[__ldg(&cc.pml)][C][a2] + (int64_t)x[a2] * kProfStride;
      const bool on1 = coef_nonzero(q1 + 1), on2 = coef_nonzero(q2 + 1);
      if (!on1 && !on2) {
        P::st(fp, plain_upd<E>(F, P::cfg(&cc.c1), P::cfg(&cc.c2), p1, p2));
        return;
      }
      R psi1 = pre.a, psi2 = pre.b;
      if (on1) {
        psi1 = madd(P::cfg(q1 + 3), p1, P::cfg(q1) * psi1);
        P::st(aux + lin, psi1);
      }
      if (on2) {
        psi2 = madd(P::cfg(q2 + 3), p2, P::cfg(q2) * psi2);
        P::st(aux + np + lin, psi2);
      }
      const R X = madd(-P::cfg(q2 + 4), p2, madd(P::cfg(q1 + 4), p1, psi1 - psi2));
      const R cdt = P::cfg(&cc.cdt);
      P::st(fp, E ? madd(cdt, X, F) : madd(-cdt, X, F));
    }
    return;
  }
  const R r1 = P::cf(g.rdr[a1]);
  const R r2 = P::cf(g.rdr[a2]);
  if (kind == GMES_KIND_UPML) {
    const Coef* q1 = g.prof[cc.pml][C][a1] + (int64_t)x[a1] * kProfStride;
    const Coef* q2 = g.prof[cc.pml][C][a2] + (int64_t)x[a2] * kProfStride;
    const Coef* q3 = g.prof[cc.pml][C][own] + (int64_t)x[own] * kProfStride;
    T* sp = aux + lin;
    const R d_old = pre.a;
    const R curl = p1 * r1 - p2 * r2;
    const R d_new = E ? P::cfg(&(q1[0])) * d_old + P::cfg(&(q1[1])) * curl
                      : P::cfg(&(q1[0])) * d_old - P::cfg(&(q1[1])) * curl;
    P::st(sp, d_new);
    P::st(fp, P::cfg(&(q2[0])) * F +
                  P::cfg(&(q2[2])) * (P::cfg(&(q3[3])) * d_new - P::cfg(&(q3[4])) * d_old) *
                      P::cfg(&(cc.reps)));
    return;
  }
  if (kind == GMES_KIND_CONST) {
    P::st(fp, P::cfg(g.part ? &(cc.value_im) : &(cc.value)));
    return;
  }
  if constexpr (DISP && E) {
    const Coef* pool = g.pool[C] + (int64_t)id * kPoolStride;
    const R curl = p1 * r1 - p2 * r2;
    const R e_now = F;
    if (kind == GMES_KIND_DRUDE || kind == GMES_KIND_LORENTZ) {
      // src/pw_drude.hh:89-151, src/pw_lorentz.hh:96-157
      R sum = P::zero();
      for (int q = 0; q < cc.npole; ++q) {
        T* qn = aux + (int64_t)(2 * q) * np + lin;      // q_now
        T* qw = aux + (int64_t)(2 * q + 1) * np + lin;  // q_new
        const R q_old = P::ldw(qn);
        const R q_now = P::ldw(qw);
        const R q_new = P::cfg(&(pool[kPoolA + 3 * q])) * q_old +
                        P::cfg(&(pool[kPoolA + 3 * q + 1])) * q_now +
                        P::cfg(&(pool[kPoolA + 3 * q + 2])) * e_now;
        P::st(qn, q_now);
        P::st(qw, q_new);
        sum = sum + (q_new - q_now);
      }
      P::st(fp, P::cfg(&(pool[kPoolC])) * curl + P::cfg(&(pool[kPoolC + 1])) * sum +
                    P::cfg(&(pool[kPoolC + 2])) * e_now);
      return;
    }
    if (kind == GMES_KIND_DCP) {
      // src/pw_dcp.hh:105-225
      T* eo = aux + lin;
      const R e_old = P::ldw(eo);
      R sd = P::zero(), sc = P::zero();
      for (int q = 0; q < cc.npole; ++q) {
        const R qo = P::ldw(aux + (int64_t)(1 + 2 * q) * np + lin);
        const R qn = P::ldw(aux + (int64_t)(2 + 2 * q) * np + lin);
        const R a0 = P::cfg(&(pool[kPoolA + 3 * q])), a1c = P::cfg(&(pool[kPoolA + 3 * q + 1]));
        sd = sd + ((P::from_double(1.0) - a1c) * qn - a0 * qo);
      }
      const int cb = 1 + 2 * cc.npole;
      for (int q = 0; q < cc.ncp; ++q) {
        const R po = P::ldw(aux + (int64_t)(cb + 2 * q) * np + lin);
        const R pn = P::ldw(aux + (int64_t)(cb + 2 * q + 1) * np + lin);
        const R b0 = P::cfg(&(pool[kPoolB + 5 * q])), b1 = P::cfg(&(pool[kPoolB + 5 * q + 1]));
        sc = sc + ((P::from_double(1.0) - b1) * pn - b0 * po);
      }
      const R e_new = P::cfg(&(pool[kPoolC])) * curl + P::cfg(&(pool[kPoolC + 1])) * (sd + sc) +
                      P::cfg(&(pool[kPoolC + 2])) * e_old + P::cfg(&(pool[kPoolC + 3])) * e_now;
      const R esum = (e_old + P::from_double(2.0) * e_now) + e_new;
      for (int q = 0; q < cc.npole; ++q) {
        T* qop = aux + (int64_t)(1 + 2 * q) * np + lin;
        T* qnp = aux + (int64_t)(2 + 2 * q) * np + lin;
        const R qo = P::ldw(qop), qn = P::ldw(qnp);
        const R q_new = P::cfg(&(pool[kPoolA + 3 * q])) * qo + P::cfg(&(pool[kPoolA + 3 * q + 1])) * qn +
                        P::cfg(&(pool[kPoolA + 3 * q + 2])) * esum;
        P::st(qop, qn);
        P::st(qnp, q_new);
      }
      for (int q = 0; q < cc.ncp; ++q) {
        T* pop = aux + (int64_t)(cb + 2 * q) * np + lin;
        T* pnp = aux + (int64_t)(cb + 2 * q + 1) * np + lin;
        const R po = P::ldw(pop), pn = P::ldw(pnp);
        const Coef* b = pool + kPoolB + 5 * q;
        const R p_new = P::cfg(&(b[0])) * po + P::cfg(&(b[1])) * pn + P::cfg(&(b[2])) * e_old +
                        P::cfg(&(b[3])) * e_now + P::cfg(&(b[4])) * e_new;
        P::st(pop, pn);
        P::st(pnp, p_new);
      }
      P::st(eo, e_now);
      P::st(fp, e_new);
      return;
    }
    if (kind == GMES_KIND_DCP_PLRC) {
      // src/pw_dcp.hh:466-583: psi_dp[npole] real, psi_cp[ncp] complex (re, im)
      const int cb = cc.npole;
      R psum = P::zero(), csum = P::zero();
      for (int q = 0; q < cc.npole; ++q) psum = psum + P::ldw(aux + (int64_t)q * np + lin);
      for (int q = 0; q < cc.ncp; ++q)
        csum = csum + P::ldw(aux + (int64_t)(cb + 2 * q) * np + lin);
      const R e_new = (P::cfg(&(pool[kPoolC])) * curl + P::cfg(&(pool[kPoolC + 1])) * e_now) +
                      P::cfg(&(pool[kPoolC + 2])) * (psum + csum);
      for (int q = 0; q < cc.npole; ++q) {
        T* sp = aux + (int64_t)q * np + lin;
        const Coef* a = pool + kPoolA + 3 * q;
        P::st(sp, (P::cfg(a) * e_new + P::cfg(a + 1) * e_now) + P::cfg(a + 2) * P::ldw(sp));
      }
      for (int q = 0; q < cc.ncp; ++q) {
        T* pr_ = aux + (int64_t)(cb + 2 * q) * np + lin;
        T* pi_ = aux + (int64_t)(cb + 2 * q + 1) * np + lin;
        const R pr = P::ldw(pr_), pi = P::ldw(pi_);
        const Coef* b = pool + kPoolB + 6 * q;
        P::st(pr_, (P::cfg(b) * e_new + P::cfg(b + 2) * e_now) +
                       (P::cfg(b + 4) * pr - P::cfg(b + 5) * pi));
        P::st(pi_, (P::cfg(b + 1) * e_new + P::cfg(b + 3) * e_now) +
                       (P::cfg(b + 4) * pi + P::cfg(b + 5) * pr));
      }
      P::st(fp, e_new);
      return;
    }
  }
}

// ---------------------------------------------------------------------------
// Per-point update in the reference's exact operation order (FP64, no FMA,
// IEEE division): bit-for-bit the arithmetic of src/pw_*.hh.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ADD(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double SUB(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double MUL(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double DIV(double a, double b) { return __ddiv_rn(a, b); }

template <int C, bool DISP>
__device__ __forceinline__ void update_strict(const GridDev& g, int64_t lin, const int x[3],
                                              double D1, double D2, double F, uint8_t id) {
  constexpr int own = C % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  constexpr bool E = C < 3;
  const ClassCoef& cc = g.tab[C][id];
  const int kind = cc.kind;
  if (kind == GMES_KIND_DUMMY) return;
  double* fp = static_cast<double*>(g.f[C]) + lin;
  const double dt = g.dt, d1 = g.dr[a1], d2 = g.dr[a2], eps = cc.eps.d;
  if (kind == GMES_KIND_DIELECTRIC) {
    // E: e += dt/eps * (D1/d1 - D2/d2); H: h += dt/mu * (D2/d2 - D1/d1)
    const double X = E ? SUB(DIV(D1, d1), DIV(D2, d2)) : SUB(DIV(D2, d2), DIV(D1, d1));
    *fp = ADD(F, MUL(DIV(dt, eps), X));
    return;
  }
  double* aux = static_cast<double*>(g.aux[C]);
  const int64_t np = g.npts[C];
  if (kind == GMES_KIND_CPML) {
    // src/pw_cpml.hh:115-132 (E), 327-344 (H)
    const Coef* q1 = g.prof[cc.pml][C][a1] + (int64_t)x[a1] * kProfStride;
    const Coef* q2 = g.prof[cc.pml][C][a2] + (int64_t)x[a2] * kProfStride;
    double* s1 = aux + lin;
    double* s2 = aux + np + lin;
    const double psi1 = ADD(MUL(q1[0].d, *s1), DIV(MUL(q1[1].d, D1), d1));
    const double psi2 = ADD(MUL(q2[0].d, *s2), DIV(MUL(q2[1].d, D2), d2));
    *s1 = psi1;
    *s2 = psi2;
    const double X =
        SUB(ADD(SUB(DIV(DIV(D1, d1), q1[2].d), DIV(DIV(D2, d2), q2[2].d)), psi1), psi2);
    const double inc = MUL(DIV(dt, eps), X);
    *fp = E ? ADD(F, inc) : SUB(F, inc);
    return;
  }
  const double curl = SUB(DIV(D1, d1), DIV(D2, d2));
  if (kind == GMES_KIND_UPML) {
    // src/pw_upml.hh:113-128 (E), 317-332 (H)
    const Coef* q1 = g.prof[cc.pml][C][a1] + (int64_t)x[a1] * kProfStride;
    const Coef* q2 = g.prof[cc.pml][C][a2] + (int64_t)x[a2] * kProfStride;
    const Coef* q3 = g.prof[cc.pml][C][own] + (int64_t)x[own] * kProfStride;
    double* sp = aux + lin;
    const double dstore = *sp;
    const double dn = E ? ADD(MUL(q1[0].d, dstore), MUL(q1[1].d, curl))
                        : SUB(MUL(q1[0].d, dstore), MUL(q1[1].d, curl));
    *sp = dn;
    *fp = ADD(MUL(q2[0].d, F),
              DIV(MUL(q2[2].d, SUB(MUL(q3[3].d, dn), MUL(q3[4].d, dstore))), eps));
    return;
  }
  if (kind == GMES_KIND_CONST) {
    *fp = g.part ? cc.value_im.d : cc.value.d;
    return;
  }
  if constexpr (DISP && E) {
    const Coef* pool = g.pool[C] + (int64_t)id * kPoolStride;
    const double e_now = F;
    if (kind == GMES_KIND_DRUDE || kind == GMES_KIND_LORENTZ) {
      double sum = 0.0;
      for (int q = 0; q < cc.npole; ++q) {
        double* qn = aux + (int64_t)(2 * q) * np + lin;
        double* qw = aux + (int64_t)(2 * q + 1) * np + lin;
        const double q_old = *qn, q_now = *qw;
        const double q_new = ADD(ADD(MUL(pool[kPoolA + 3 * q].d, q_old),
                                     MUL(pool[kPoolA + 3 * q + 1].d, q_now)),
                                 MUL(pool[kPoolA + 3 * q + 2].d, e_now));
        *qn = q_now;
        *qw = q_new;
        sum = ADD(sum, SUB(q_new, q_now));
      }
      *fp = ADD(ADD(MUL(pool[kPoolC].d, curl), MUL(pool[kPoolC + 1].d, sum)),
                MUL(pool[kPoolC + 2].d, e_now));
      return;
    }
    if (kind == GMES_KIND_DCP) {
      double* eo = aux + lin;
      const double e_old = *eo;
      double sd = 0.0, sc = 0.0;
      for (int q = 0; q < cc.npole; ++q) {
        const double qo = aux[(int64_t)(1 + 2 * q) * np + lin];
        const double qn = aux[(int64_t)(2 + 2 * q) * np + lin];
        sd = ADD(sd, SUB(MUL(SUB(1.0, pool[kPoolA + 3 * q + 1].d), qn),
                         MUL(pool[kPoolA + 3 * q].d, qo)));
      }
      const int cb = 1 + 2 * cc.npole;
      for (int q = 0; q < cc.ncp; ++q) {
        const double po = aux[(int64_t)(cb + 2 * q) * np + lin];
        const double pn = aux[(int64_t)(cb + 2 * q + 1) * np + lin];
        sc = ADD(sc, SUB(MUL(SUB(1.0, pool[kPoolB + 5 * q + 1].d), pn),
                         MUL(pool[kPoolB + 5 * q].d, po)));
      }
      const double e_new =
          ADD(ADD(ADD(MUL(pool[kPoolC].d, curl), MUL(pool[kPoolC + 1].d, ADD(sd, sc))),
                  MUL(pool[kPoolC + 2].d, e_old)),
              MUL(pool[kPoolC + 3].d, e_now));
      const double esum = ADD(ADD(e_old, MUL(2.0, e_now)), e_new);
      for (int q = 0; q < cc.npole; ++q) {
        double* qop = aux + (int64_t)(1 + 2 * q) * np + lin;
        double* qnp = aux + (int64_t)(2 + 2 * q) * np + lin;
        const double qo = *qop, qn = *qnp;
        const double q_new = ADD(ADD(MUL(pool[kPoolA + 3 * q].d, qo),
                                     MUL(pool[kPoolA + 3 * q + 1].d, qn)),
                                 MUL(pool[kPoolA + 3 * q + 2].d, esum));
        *qop = qn;
        *qnp = q_new;
      }
      for (int q = 0; q < cc.ncp; ++q) {
        double* pop = aux + (int64_t)(cb + 2 * q) * np + lin;
        double* pnp = aux + (int64_t)(cb + 2 * q + 1) * np + lin;
        const double po = *pop, pn = *pnp;
        const Coef* b = pool + kPoolB + 5 * q;
        const double p_new =
            ADD(ADD(ADD(ADD(MUL(b[0].d, po), MUL(b[1].d, pn)), MUL(b[2].d, e_old)),
                    MUL(b[3].d, e_now)),
                MUL(b[4].d, e_new));
        *pop = pn;
        *pnp = p_new;
      }
      *eo = e_now;
      *fp = e_new;
      return;
    }
    if (kind == GMES_KIND_DCP_PLRC) {
      // src/pw_dcp.hh:466-583 in its operation order; psi_cp complex
      // products as (ac - bd, ad + bc)
      const int cb = cc.npole;
      double psum = 0.0, csum = 0.0;
      for (int q = 0; q < cc.npole; ++q) psum = ADD(psum, aux[(int64_t)q * np + lin]);
      for (int q = 0; q < cc.ncp; ++q) csum = ADD(csum, aux[(int64_t)(cb + 2 * q) * np + lin]);
      const double e_new = ADD(ADD(MUL(pool[kPoolC].d, curl), MUL(pool[kPoolC + 1].d, e_now)),
                               MUL(pool[kPoolC + 2].d, ADD(psum, csum)));
      for (int q = 0; q < cc.npole; ++q) {
        double* sp = aux + (int64_t)q * np + lin;
        const Coef* a = pool + kPoolA + 3 * q;
        *sp = ADD(ADD(MUL(a[0].d, e_new), MUL(a[1].d, e_now)), MUL(a[2].d, *sp));
      }
      for (int q = 0; q < cc.ncp; ++q) {
        double* pr_ = aux + (int64_t)(cb + 2 * q) * np + lin;
        double* pi_ = aux + (int64_t)(cb + 2 * q + 1) * np + lin;
        const double pr = *pr_, pi = *pi_;
        const Coef* b = pool + kPoolB + 6 * q;
        *pr_ = ADD(ADD(MUL(b[0].d, e_new), MUL(b[2].d, e_now)),
                   SUB(MUL(b[4].d, pr), MUL(b[5].d, pi)));
        *pi_ = ADD(ADD(MUL(b[1].d, e_new), MUL(b[3].d, e_now)),
                   ADD(MUL(b[4].d, pi), MUL(b[5].d, pr)));
      }
      *fp = e_new;
      return;
    }
  }
}

// ---------------------------------------------------------------------------
// The half-step kernel.  One thread per cell (i, j, k) of the N0 x N1 x N2
// update domain; the thread updates the three components of its half there.
// Every value the cell needs from DRAM -- the class ids, the component's own
// values and the nine neighbour values of the curls -- is loaded up front,
// before any store, so a thread waits for one memory latency instead of a
// chain of them; only state slots (PML, ADE) are loaded after the class is
// known.  Block = bx x by threads over (k, j) with bx = min(32, n2 rounded up
// to a power of two), so thin (2-D) grids still fill whole warps along j;
// grid.z walks i.
// ---------------------------------------------------------------------------
template <int MASK, int C>
__device__ __forceinline__ bool is_active(const GridDev& g) {
  if constexpr (MASK != 0)
    return (MASK >> C) & 1;
  else
    return (g.active >> C) & 1;
}

template <class P, int MASK, int C, class I>
__device__ __forceinline__ typename P::R ldf(const GridDev& g, I off) {
  if (!is_active<MASK, C>(g)) return P::zero();
  return P::ld(static_cast<const typename P::T*>(g.f[C]) + off);
}

template <int MASK, int C, class I>
__device__ __forceinline__ uint8_t ldc(const GridDev& g, I off) {
  if (!is_active<MASK, C>(g)) return 0;
  return __ldg(g.cls[C] + off);
}

template <class P, int MASK, int C, bool STRICT, bool DISP>
__device__ __forceinline__ void upd(const GridDev& g, int64_t lin, const int x[3],
                                    typename P::R p1, typename P::R p2, typename P::R F,
                                    uint8_t id, Pre<P> pre) {
  if (!is_active<MASK, C>(g)) return;
  if constexpr (STRICT)
    update_strict<C, DISP>(g, lin, x, p1, p2, F, id);
  else
    update_fast<P, C, DISP>(g, lin, x, p1, p2, F, id, pre);
}

template <class P, int MASK, int C, bool STRICT>
__device__ __forceinline__ Pre<P> pre_of(const GridDev& g, int64_t lin, const int x[3],
                                         uint8_t id) {
  if constexpr (STRICT) {
    return Pre<P>{P::zero(), P::zero()};
  } else {
    if (!is_active<MASK, C>(g)) return Pre<P>{P::zero(), P::zero()};
    return prefetch_state<P, C>(g, lin, x, id);
  }
}

// MASK: the active-component mask when known at compile time, 0 when read
// from the grid; I: offset type (int32_t for grids whose components hold
// fewer than 2^31 points, int64_t otherwise).
template <class P, int SIDE, bool STRICT, bool DISP, int MASK, class I>
__device__ __forceinline__ void cell_body(const GridDev& g, int i, int j, int k) {
  using R = typename P::R;
  const I s00 = (I)g.st[0][0], s01 = (I)g.st[0][1], s10 = (I)g.st[1][0], s11 = (I)g.st[1][1];
  const I s20 = (I)g.st[2][0], s21 = (I)g.st[2][1], s30 = (I)g.st[3][0], s31 = (I)g.st[3][1];
  const I s40 = (I)g.st[4][0], s41 = (I)g.st[4][1], s50 = (I)g.st[5][0], s51 = (I)g.st[5][1];
  const I ii = (I)i, jj = (I)j, kk = (I)k;
  const int xc[3] = {i, j, k};
  if constexpr (SIDE == 0) {
    // own points: Ex, Ey, Ez at (i, j, k)
    const I lx = ii * s00 + jj * s01 + kk;
    const I ly = ii * s10 + jj * s11 + kk;
    const I lz = ii * s20 + jj * s21 + kk;
    const uint8_t idx = ldc<MASK, 0>(g, lx), idy = ldc<MASK, 1>(g, ly), idz = ldc<MASK, 2>(g, lz);
    const R ex = ldf<P, MASK, 0>(g, lx), ey = ldf<P, MASK, 1>(g, ly), ez = ldf<P, MASK, 2>(g, lz);
    // neighbour H values
    const I hx = ii * s30 + jj * s31 + kk;         // Hx[i, j, k]
    const I hy = (ii + 1) * s40 + jj * s41 + kk;   // Hy[i+1, j, k]
    const I hz = (ii + 1) * s50 + jj * s51 + kk;   // Hz[i+1, j, k]
    const R hz_a = ldf<P, MASK, 5>(g, hz + s51);          // Hz[i+1, j+1, k]
    const R hz_b = ldf<P, MASK, 5>(g, hz);                // Hz[i+1, j,   k]
    const R hz_c = ldf<P, MASK, 5>(g, hz + s51 - s50);    // Hz[i,   j+1, k]
    const R hy_a = ldf<P, MASK, 4>(g, hy + 1);            // Hy[i+1, j, k+1]
    const R hy_b = ldf<P, MASK, 4>(g, hy);                // Hy[i+1, j, k]
    const R hy_c = ldf<P, MASK, 4>(g, hy + 1 - s40);      // Hy[i,   j, k+1]
    const R hx_a = ldf<P, MASK, 3>(g, hx + s31 + 1);      // Hx[i, j+1, k+1]
    const R hx_b = ldf<P, MASK, 3>(g, hx + s31);          // Hx[i, j+1, k]
    const R hx_c = ldf<P, MASK, 3>(g, hx + 1);            // Hx[i, j,   k+1]
    const Pre<P> px = pre_of<P, MASK, 0, STRICT>(g, lx, xc, idx);
    const Pre<P> py = pre_of<P, MASK, 1, STRICT>(g, ly, xc, idy);
    const Pre<P> pz = pre_of<P, MASK, 2, STRICT>(g, lz, xc, idz);
    upd<P, MASK, 0, STRICT, DISP>(g, lx, xc, hz_a - hz_b, hy_a - hy_b, ex, idx, px);
    upd<P, MASK, 1, STRICT, DISP>(g, ly, xc, hx_a - hx_b, hz_a - hz_c, ey, idy, py);
    upd<P, MASK, 2, STRICT, DISP>(g, lz, xc, hy_a - hy_c, hx_a - hx_c, ez, idz, pz);
  } else {
    // own points: Hx[i, j+1, k+1], Hy[i+1, j, k+1], Hz[i+1, j+1, k]
    const I lx = ii * s30 + (jj + 1) * s31 + kk + 1;
    const I ly = (ii + 1) * s40 + jj * s41 + kk + 1;
    const I lz = (ii + 1) * s50 + (jj + 1) * s51 + kk;
    const uint8_t idx = ldc<MASK, 3>(g, lx), idy = ldc<MASK, 4>(g, ly), idz = ldc<MASK, 5>(g, lz);
    const R hx = ldf<P, MASK, 3>(g, lx), hy = ldf<P, MASK, 4>(g, ly), hz = ldf<P, MASK, 5>(g, lz);
    const I ex = ii * s00 + jj * s01 + kk;
    const I ey = ii * s10 + jj * s11 + kk;
    const I ez = ii * s20 + jj * s21 + kk;
    const R ez_0 = ldf<P, MASK, 2>(g, ez);           // Ez[i, j, k]
    const R ez_j = ldf<P, MASK, 2>(g, ez + s21);     // Ez[i, j+1, k]
    const R ez_i = ldf<P, MASK, 2>(g, ez + s20);     // Ez[i+1, j, k]
    const R ey_0 = ldf<P, MASK, 1>(g, ey);           // Ey[i, j, k]
    const R ey_k = ldf<P, MASK, 1>(g, ey + 1);       // Ey[i, j, k+1]
    const R ey_i = ldf<P, MASK, 1>(g, ey + s10);     // Ey[i+1, j, k]
    const R ex_0 = ldf<P, MASK, 0>(g, ex);           // Ex[i, j, k]
    const R ex_k = ldf<P, MASK, 0>(g, ex + 1);       // Ex[i, j, k+1]
    const R ex_j = ldf<P, MASK, 0>(g, ex + s01);     // Ex[i, j+1, k]
    const int x3[3] = {i, j + 1, k + 1}, x4[3] = {i + 1, j, k + 1}, x5[3] = {i + 1, j + 1, k};
    const Pre<P> px = pre_of<P, MASK, 3, STRICT>(g, lx, x3, idx);
    const Pre<P> py = pre_of<P, MASK, 4, STRICT>(g, ly, x4, idy);
    const Pre<P> pz = pre_of<P, MASK, 5, STRICT>(g, lz, x5, idz);
    upd<P, MASK, 3, STRICT, DISP>(g, lx, x3, ez_j - ez_0, ey_k - ey_0, hx, idx, px);
    upd<P, MASK, 4, STRICT, DISP>(g, ly, x4, ex_k - ex_0, ez_i - ez_0, hy, idy, py);
    upd<P, MASK, 5, STRICT, DISP>(g, lz, x5, ey_i - ey_0, ex_j - ex_0, hz, idz, pz);
  }
}

// Whether a warp whose class triple is uniform, with DIELECTRIC or CPML
// classes (the CPML shell), takes those kinds' updates directly instead of
// the per-point kind dispatch.  Measured on GB300 (256^3 cube, Gcell/s, one
// box): FP32 39.78 -> 40.64; with it df64 ran 24.21 -> 23.01 and FP64 18.90
// -> 18.91, so only FP32 takes it (GMES_UNIFORM_CPML = 1 gives it every
// precision, 0 none).  Re-measured per half with the per-half register
// budgets (ms): df64 E 0.3185 -> 0.403, H 0.3245 -> 0.3200; FP64 E 0.4435
// -> 0.4697, H 0.4428 -> 0.4497; so the float-float type takes it on its H
// half too.  The CPML update it shares with the per-point path
// (cpml_separate) fuses every multiply-add explicitly: inlined in two places
// with implicit contraction, the two copies rounded differently and a grid
// batched with another warp layout lost bit-identity with its solo run.
template <class P, int SIDE>
struct UniformCpml {
#if defined(GMES_UNIFORM_CPML)
  static constexpr bool value = GMES_UNIFORM_CPML != 0;
#else
  static constexpr bool value = false;
#endif
};
template <int SIDE>
struct UniformCpml<PolF32, SIDE> {
#if defined(GMES_UNIFORM_CPML)
  static constexpr bool value = GMES_UNIFORM_CPML != 0;
#else
  static constexpr bool value = true;
#endif
};
template <int SIDE>
struct UniformCpml<PolDF, SIDE> {
#if defined(GMES_UNIFORM_CPML)
  static constexpr bool value = GMES_UNIFORM_CPML != 0;
#else
  static constexpr bool value = SIDE == 1;
#endif
};

// The psi pair (psi1, psi2) of a CPML point of component c.
template <class P>
__device__ __forceinline__ Pre<P> psi_pair(const GridDev& g, int c, int64_t lin) {
  const typename P::T* aux = static_cast<const typename P::T*>(g.aux[c]);
  return {P::ldw(aux + lin), P::ldw(aux + g.npts[c] + lin)};
}

// Whether a warp on the warp-uniform CPML path reads its classes'
// plain-form coefficients together with their kinds (one round trip to the
// class table instead of two).  Measured on GB300 (256^3 cube, ms per E / H
// half): df64 0.3143 / 0.3192 -> 0.3145 / 0.3135; FP32 0.2044 / 0.2070 ->
// 0.2269 / 0.2098 (three more live values at 40 registers), so the
// float-float type only (GMES_EARLY_COEF = 0 / 1 sets it for both).
template <class P>
struct EarlyCoef {
#if defined(GMES_EARLY_COEF)
  static constexpr bool value = GMES_EARLY_COEF != 0;
#else
  static constexpr bool value = std::is_same<P, PolDF>::value;
#endif
};

// The half-step update of one cell in the fast precisions.  Every field
// value and class id the cell reads is loaded first, so that no load waits
// for another.  Then a warp whose cells all carry the same class triple, each
// class of kind DIELECTRIC (one vote, __match_all_sync, and three
// warp-uniform kind look-ups), updates its three points with those classes'
// coefficients and nothing else (FP32 and the float-float H half also take
// warps of one DIELECTRIC or CPML class per component directly:
// UniformCpml); every other warp goes through the per-point path
// (update_fast), whose dielectric and CPML branches are the same
// arithmetic, so the paths agree bit for bit.  The offsets come from
// the three array-shape families (fst): an active component's strides are
// its family's.  Measured on GB300 (256^3 cube / 192^3 dispersive scene,
// Gcell/s, per-point path only -> with the warp-uniform path):
//   cube FP64 17.42 -> 18.60, FP32 34.17 -> 34.91, df64 21.89 -> 23.63;
//   dispersive FP64 9.85 -> 10.09, FP32 20.48 -> 22.36, df64 14.85 -> 15.04.
// A per-warp table of plain warps built at set-up (read with the field
// values, class maps read only by the other warps) ran slower: cube FP64
// 18.20, FP32 31.90, df64 22.95.  So did two cells per thread, (i, j, k) and
// (i + 1, j, k), with the loads of both issued before either update (twice
// the bytes in flight per warp, four shared neighbour loads): cube FP32
// 42.54 -> 30.1 / 29.7 / 34.3 / 31.1 Gcell/s at 6 / 7 / 8 / 10 blocks per SM
// (64 registers at 8), dispersive FP32 25.42 -> 22.35; df64 (5, 6 blocks)
// 26.74 -> 17.5 / 20.7, FP64 (6 blocks) 19.25 -> 16.99.
template <class P, int SIDE, bool DISP, int MASK, class I>
__device__ __forceinline__ void cell_body_fast(const GridDev& g, int i, int j, int k) {
  using R = typename P::R;
  using T = typename P::T;
  constexpr int c0 = 3 * SIDE;
  const I X0 = (I)g.fst[0][0], X1 = (I)g.fst[0][1];
  const I Y0 = (I)g.fst[1][0], Y1 = (I)g.fst[1][1];
  const I Z0 = (I)g.fst[2][0], Z1 = (I)g.fst[2][1];
  const I ii = (I)i, jj = (I)j, kk = (I)k;
  const I oX = ii * X0 + jj * X1 + kk;
  const I oY = ii * Y0 + jj * Y1 + kk;
  const I oZ = ii * Z0 + jj * Z1 + kk;
  // own points: E (i, j, k); Hx[i, j+1, k+1], Hy[i+1, j, k+1], Hz[i+1, j+1, k]
  const I l0 = SIDE == 0 ? oX : oX + X1 + 1;
  const I l1 = SIDE == 0 ? oY : oY + Y0 + 1;
  const I l2 = SIDE == 0 ? oZ : oZ + Z0 + Z1;
  const R f0 = ldf<P, MASK, c0>(g, l0), f1 = ldf<P, MASK, c0 + 1>(g, l1),
          f2 = ldf<P, MASK, c0 + 2>(g, l2);
  R d01, d02, d11, d12, d21, d22;  // (D1, D2) of each component
  if constexpr (SIDE == 0) {
    const R hz_a = ldf<P, MASK, 5>(g, oZ + Z0 + Z1);  // Hz[i+1, j+1, k]
    const R hz_b = ldf<P, MASK, 5>(g, oZ + Z0);       // Hz[i+1, j,   k]
    const R hz_c = ldf<P, MASK, 5>(g, oZ + Z1);       // Hz[i,   j+1, k]
    const R hy_a = ldf<P, MASK, 4>(g, oY + Y0 + 1);   // Hy[i+1, j, k+1]
    const R hy_b = ldf<P, MASK, 4>(g, oY + Y0);       // Hy[i+1, j, k]
    const R hy_c = ldf<P, MASK, 4>(g, oY + 1);        // Hy[i,   j, k+1]
    const R hx_a = ldf<P, MASK, 3>(g, oX + X1 + 1);   // Hx[i, j+1, k+1]
    const R hx_b = ldf<P, MASK, 3>(g, oX + X1);       // Hx[i, j+1, k]
    const R hx_c = ldf<P, MASK, 3>(g, oX + 1);        // Hx[i, j,   k+1]
    d01 = curl_diff(hz_a, hz_b); d02 = curl_diff(hy_a, hy_b);
    d11 = curl_diff(hx_a, hx_b); d12 = curl_diff(hz_a, hz_c);
    d21 = curl_diff(hy_a, hy_c); d22 = curl_diff(hx_a, hx_c);
  } else {
    const R ez_0 = ldf<P, MASK, 2>(g, oZ);       // Ez[i, j, k]
    const R ez_j = ldf<P, MASK, 2>(g, oZ + Z1);  // Ez[i, j+1, k]
    const R ez_i = ldf<P, MASK, 2>(g, oZ + Z0);  // Ez[i+1, j, k]
    const R ey_0 = ldf<P, MASK, 1>(g, oY);       // Ey[i, j, k]
    const R ey_k = ldf<P, MASK, 1>(g, oY + 1);   // Ey[i, j, k+1]
    const R ey_i = ldf<P, MASK, 1>(g, oY + Y0);  // Ey[i+1, j, k]
    const R ex_0 = ldf<P, MASK, 0>(g, oX);       // Ex[i, j, k]
    const R ex_k = ldf<P, MASK, 0>(g, oX + 1);   // Ex[i, j, k+1]
    const R ex_j = ldf<P, MASK, 0>(g, oX + X1);  // Ex[i, j+1, k]
    d01 = curl_diff(ez_j, ez_0); d02 = curl_diff(ey_k, ey_0);
    d11 = curl_diff(ex_k, ex_0); d12 = curl_diff(ez_i, ez_0);
    d21 = curl_diff(ey_i, ey_0); d22 = curl_diff(ex_j, ex_0);
  }
  const uint8_t id0 = ldc<MASK, c0>(g, l0), id1 = ldc<MASK, c0 + 1>(g, l1),
                id2 = ldc<MASK, c0 + 2>(g, l2);
  const uint32_t t = (uint32_t)id0 | (uint32_t)id1 << 8 | (uint32_t)id2 << 16;
  int same = 0;
  __match_all_sync(__activemask(), t, &same);
  const bool uniform = same && !g.pointwise;
  // the warp's kinds when its class triple is uniform (inactive components
  // count as dielectric: they are skipped)
  int ka = GMES_KIND_DIELECTRIC, kb = GMES_KIND_DIELECTRIC, kc = GMES_KIND_DIELECTRIC;
  bool fast;
  // plain-form coefficients of the warp's three classes, read with the kinds
  // (one round trip to the class table instead of two)
  R ca1 = P::zero(), ca2 = P::zero(), cb1 = P::zero(), cb2 = P::zero(), cc1 = P::zero(),
    cc2 = P::zero();
  if constexpr (UniformCpml<P, SIDE>::value) {
    if (uniform) {
      if (is_active<MASK, c0>(g)) {
        const ClassCoef& q = g.tab[c0][id0];
        ka = q.kind;
        if (EarlyCoef<P>::value) ca1 = P::cfg(&q.c1), ca2 = P::cfg(&q.c2);
      }
      if (is_active<MASK, c0 + 1>(g)) {
        const ClassCoef& q = g.tab[c0 + 1][id1];
        kb = q.kind;
        if (EarlyCoef<P>::value) cb1 = P::cfg(&q.c1), cb2 = P::cfg(&q.c2);
      }
      if (is_active<MASK, c0 + 2>(g)) {
        const ClassCoef& q = g.tab[c0 + 2][id2];
        kc = q.kind;
        if (EarlyCoef<P>::value) cc1 = P::cfg(&q.c1), cc2 = P::cfg(&q.c2);
      }
    }
    fast = uniform && ka == GMES_KIND_DIELECTRIC && kb == GMES_KIND_DIELECTRIC &&
           kc == GMES_KIND_DIELECTRIC;
  } else {
    fast = uniform &&
           (!is_active<MASK, c0>(g) || g.tab[c0][id0].kind == GMES_KIND_DIELECTRIC) &&
           (!is_active<MASK, c0 + 1>(g) || g.tab[c0 + 1][id1].kind == GMES_KIND_DIELECTRIC) &&
           (!is_active<MASK, c0 + 2>(g) || g.tab[c0 + 2][id2].kind == GMES_KIND_DIELECTRIC);
  }
  constexpr bool E = SIDE == 0;
  if (fast) {  // warp-uniform
    const ClassCoef& qa = g.tab[c0][id0];
    const ClassCoef& qb = g.tab[c0 + 1][id1];
    const ClassCoef& qc = g.tab[c0 + 2][id2];
    if (UniformCpml<P, SIDE>::value && EarlyCoef<P>::value) {
      if (is_active<MASK, c0>(g))
        P::st(static_cast<T*>(g.f[c0]) + l0, plain_upd<E>(f0, ca1, ca2, d01, d02));
      if (is_active<MASK, c0 + 1>(g))
        P::st(static_cast<T*>(g.f[c0 + 1]) + l1, plain_upd<E>(f1, cb1, cb2, d11, d12));
      if (is_active<MASK, c0 + 2>(g))
        P::st(static_cast<T*>(g.f[c0 + 2]) + l2, plain_upd<E>(f2, cc1, cc2, d21, d22));
      return;
    }
    if (is_active<MASK, c0>(g))
      P::st(static_cast<T*>(g.f[c0]) + l0,
            plain_upd<E>(f0, P::cfg(&qa.c1), P::cfg(&qa.c2), d01, d02));
    if (is_active<MASK, c0 + 1>(g))
      P::st(static_cast<T*>(g.f[c0 + 1]) + l1,
            plain_upd<E>(f1, P::cfg(&qb.c1), P::cfg(&qb.c2), d11, d12));
    if (is_active<MASK, c0 + 2>(g))
      P::st(static_cast<T*>(g.f[c0 + 2]) + l2,
            plain_upd<E>(f2, P::cfg(&qc.c1), P::cfg(&qc.c2), d21, d22));
    return;
  }
  if constexpr (UniformCpml<P, SIDE>::value) {
    const auto dc = [](int kd) {
      return kd == GMES_KIND_DIELECTRIC || kd == GMES_KIND_CPML;
    };
    if (uniform && dc(ka) && dc(kb) && dc(kc)) {
      // one class per component across the warp, each DIELECTRIC or CPML
      // (the CPML shell): those kinds' updates with the kinds known for the
      // whole warp, the psi values of the CPML components loaded first
      const int xa[3] = {i, SIDE == 0 ? j : j + 1, SIDE == 0 ? k : k + 1};
      const int xb[3] = {SIDE == 0 ? i : i + 1, j, SIDE == 0 ? k : k + 1};
      const int xq[3] = {SIDE == 0 ? i : i + 1, SIDE == 0 ? j : j + 1, k};
      Pre<P> pa{P::zero(), P::zero()}, pb = pa, pc = pa;
      if (ka == GMES_KIND_CPML) pa = psi_pair<P>(g, c0, l0);
      if (kb == GMES_KIND_CPML) pb = psi_pair<P>(g, c0 + 1, l1);
      if (kc == GMES_KIND_CPML) pc = psi_pair<P>(g, c0 + 2, l2);
      const ClassCoef& qa = g.tab[c0][id0];
      const ClassCoef& qb = g.tab[c0 + 1][id1];
      const ClassCoef& qc = g.tab[c0 + 2][id2];
      if (ka == GMES_KIND_CPML)
        cpml_separate<P, c0>(g, l0, xa, d01, d02, f0, qa, pa);
      else if (is_active<MASK, c0>(g))
        P::st(static_cast<T*>(g.f[c0]) + l0,
              plain_upd<E>(f0, P::cfg(&qa.c1), P::cfg(&qa.c2), d01, d02));
      if (kb == GMES_KIND_CPML)
        cpml_separate<P, c0 + 1>(g, l1, xb, d11, d12, f1, qb, pb);
      else if (is_active<MASK, c0 + 1>(g))
        P::st(static_cast<T*>(g.f[c0 + 1]) + l1,
              plain_upd<E>(f1, P::cfg(&qb.c1), P::cfg(&qb.c2), d11, d12));
      if (kc == GMES_KIND_CPML)
        cpml_separate<P, c0 + 2>(g, l2, xq, d21, d22, f2, qc, pc);
      else if (is_active<MASK, c0 + 2>(g))
        P::st(static_cast<T*>(g.f[c0 + 2]) + l2,
              plain_upd<E>(f2, P::cfg(&qc.c1), P::cfg(&qc.c2), d21, d22));
      return;
    }
  }
  if constexpr (SIDE == 0) {
    const int xc[3] = {i, j, k};
    const Pre<P> pa = pre_of<P, MASK, 0, false>(g, l0, xc, id0);
    const Pre<P> pb = pre_of<P, MASK, 1, false>(g, l1, xc, id1);
    const Pre<P> pc = pre_of<P, MASK, 2, false>(g, l2, xc, id2);
    upd<P, MASK, 0, false, DISP>(g, l0, xc, d01, d02, f0, id0, pa);
    upd<P, MASK, 1, false, DISP>(g, l1, xc, d11, d12, f1, id1, pb);
    upd<P, MASK, 2, false, DISP>(g, l2, xc, d21, d22, f2, id2, pc);
  } else {
    const int x3[3] = {i, j + 1, k + 1}, x4[3] = {i + 1, j, k + 1}, x5[3] = {i + 1, j + 1, k};
    const Pre<P> pa = pre_of<P, MASK, 3, false>(g, l0, x3, id0);
    const Pre<P> pb = pre_of<P, MASK, 4, false>(g, l1, x4, id1);
    const Pre<P> pc = pre_of<P, MASK, 5, false>(g, l2, x5, id2);
    upd<P, MASK, 3, false, false>(g, l0, x3, d01, d02, f0, id0, pa);
    upd<P, MASK, 4, false, false>(g, l1, x4, d11, d12, f1, id1, pb);
    upd<P, MASK, 5, false, false>(g, l2, x5, d21, d22, f2, id2, pc);
  }
}

template <class P, int SIDE, bool STRICT, bool DISP, int MASK, class I>
__global__ void __launch_bounds__(kCellThreads, CellMinBlocks<P, SIDE, DISP>::value)
    k_cell(const GridDev g, int bx_log2, int i0) {
  const int bx = 1 << bx_log2;
  const int tx = threadIdx.x & (bx - 1);
  const int ty = threadIdx.x >> bx_log2;
  const int k = blockIdx.x * bx + tx;
  const int j = blockIdx.y * (kCellThreads >> bx_log2) + ty;
  const int i = i0 + (int)blockIdx.z;
  if (k >= g.n[2] || j >= g.n[1] || i >= g.n[0]) return;
  if constexpr (STRICT)
    cell_body<P, SIDE, STRICT, DISP, MASK, I>(g, i, j, k);
  else
    cell_body_fast<P, SIDE, DISP, MASK, I>(g, i, j, k);
}

// Cells per block row along k (log2): a warp covers 16 cells of two rows
// (128 bytes per row in FP64 and df64, 64 in FP32).  (Measured with blocks
// of 256 threads.)  Against 32 cells of
// one row, a warp straddles a material or CPML edge along k in half as many
// places, so fewer warps run two kinds' code or a psi block for a few
// lanes.  Measured on GB300, Gcell/s, rows of 32 / 16 / 8 cells:
//   256^3 cube (dielectric + CPML)   FP64 16.17 / 16.81 / 15.99
//                                    FP32 32.99 / 33.74 / 29.36
//                                    df64 19.72 / 21.12 / 20.12
//   192^3 dispersive + UPML          FP64  8.06 /  9.42 /  9.69
//                                    FP32 19.34 / 20.08 / 18.47
//                                    df64 12.73 / 13.86 / 13.80
// (FP64 E half of the cube: 14.4 -> 13.7 FP64 warp-instructions per cell,
// what a warp-level count of the slabs predicts for both shapes.)  The row
// length is kRowLog2 (cell_tiling).

template <class P, bool STRICT, int MASK, class I>
void launch_cell(const GridDev& d, int side, bool disp, dim3 grid, int bx_log2, int i0,
                 cudaStream_t s) {
  if (side == 0) {
    if (disp)
      k_cell<P, 0, STRICT, true, MASK, I><<<grid, kCellThreads, 0, s>>>(d, bx_log2, i0);
    else
      k_cell<P, 0, STRICT, false, MASK, I><<<grid, kCellThreads, 0, s>>>(d, bx_log2, i0);
  } else {
    k_cell<P, 1, STRICT, false, MASK, I><<<grid, kCellThreads, 0, s>>>(d, bx_log2, i0);
  }
}

// Ghost planes of one half's components (gmes/fdtd.py:811-1097 with the
// single-domain cyclic communicator): E ghosts are the last planes along the
// non-own axes and receive plane 0; H ghosts are the first planes and
// receive the last plane.  A ghost point's source is found by mapping every
// ghost coordinate at once, so corners get the value the reference's two
// successive plane copies give them and no source is itself a ghost.
template <class T>
__device__ __forceinline__ void ghost_point(const GridDev& g, int side, int item, int64_t t) {
  const int c = side * 3 + item / 2;
  if (!(g.active & (1 << c))) return;
  const int own = c % 3;
  const int ga = (item & 1) ? (own + 2) % 3 : (own + 1) % 3;
  const int pa = (ga + 1) % 3, qa = (ga + 2) % 3;
  const int p_ = pa < qa ? pa : qa, q_ = pa < qa ? qa : pa;  // q_ is the faster axis
  const int64_t np = g.sh[c][p_] * g.sh[c][q_];
  if (t >= np) return;
  int64_t x[3];
  x[p_] = t / g.sh[c][q_];
  x[q_] = t - x[p_] * g.sh[c][q_];
  x[ga] = side == 0 ? g.sh[c][ga] - 1 : 0;
  int64_t s[3] = {x[0], x[1], x[2]};
  const int a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  for (int h = 0; h < 2; ++h) {
    const int ax = h == 0 ? a1 : a2;
    if (side == 0) {
      if (x[ax] == g.sh[c][ax] - 1) s[ax] = 0;
    } else {
      if (x[ax] == 0) s[ax] = g.sh[c][ax] - 1;
    }
  }
  T* f = static_cast<T*>(g.f[c]);
  const int64_t dst = x[0] * g.st[c][0] + x[1] * g.st[c][1] + x[2];
  const int64_t src = s[0] * g.st[c][0] + s[1] * g.st[c][1] + s[2];
  f[dst] = f[src];
}

template <class T>
__global__ void k_ghost(const GridDev g, int side, int64_t maxplane) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= maxplane) return;
  ghost_point<T>(g, side, blockIdx.y, t);
}

// The same for grids whose components hold fewer than 2^31 points: 32-bit
// index arithmetic (one unsigned division per point instead of a 64-bit
// one).  Same points, same copies.
template <class T>
__global__ void k_ghost32(const GridDev g, int side, unsigned maxplane) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= maxplane) return;
  const int item = blockIdx.y;
  const int c = side * 3 + item / 2;
  if (!(g.active & (1 << c))) return;
  const int own = c % 3;
  const int ga = (item & 1) ? (own + 2) % 3 : (own + 1) % 3;
  const int pa = (ga + 1) % 3, qa = (ga + 2) % 3;
  const int p_ = pa < qa ? pa : qa, q_ = pa < qa ? qa : pa;  // q_ is the faster axis
  const unsigned sh[3] = {(unsigned)g.sh[c][0], (unsigned)g.sh[c][1], (unsigned)g.sh[c][2]};
  if (t >= sh[p_] * sh[q_]) return;
  unsigned x[3];
  x[p_] = t / sh[q_];
  x[q_] = t - x[p_] * sh[q_];
  x[ga] = side == 0 ? sh[ga] - 1 : 0;
  unsigned s[3] = {x[0], x[1], x[2]};
  const int a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  if (side == 0) {
    if (x[a1] == sh[a1] - 1) s[a1] = 0;
    if (x[a2] == sh[a2] - 1) s[a2] = 0;
  } else {
    if (x[a1] == 0) s[a1] = sh[a1] - 1;
    if (x[a2] == 0) s[a2] = sh[a2] - 1;
  }
  const unsigned st0 = (unsigned)g.st[c][0], st1 = (unsigned)g.st[c][1];
  T* f = static_cast<T*>(g.f[c]);
  f[x[0] * st0 + x[1] * st1 + x[2]] = f[s[0] * st0 + s[1] * st1 + s[2]];
}

// Ghost planes of a complex grid (Bloch boundary, gmes/fdtd.py:811-1097):
// as ghost_point, but the value is multiplied by the phase factor of each
// ghost axis in the reference's copy order (own+1, then own+2).  The
// imaginary plane follows the real plane of every component.  Strict: the
// product in the fused form numpy's SIMD complex multiply uses,
// re = fma(pr, vr, -(pi vi)), im = fma(pr, vi, pi vr).
template <bool STRICT>
__device__ __forceinline__ void ghost_point_c(const GridDev& g, int side, int item, int64_t t) {
  const int c = side * 3 + item / 2;
  if (!(g.active & (1 << c))) return;
  const int own = c % 3;
  const int ga = (item & 1) ? (own + 2) % 3 : (own + 1) % 3;
  const int pa = (ga + 1) % 3, qa = (ga + 2) % 3;
  const int p_ = pa < qa ? pa : qa, q_ = pa < qa ? qa : pa;
  const int64_t np = g.sh[c][p_] * g.sh[c][q_];
  if (t >= np) return;
  int64_t x[3];
  x[p_] = t / g.sh[c][q_];
  x[q_] = t - x[p_] * g.sh[c][q_];
  x[ga] = side == 0 ? g.sh[c][ga] - 1 : 0;
  int64_t s[3] = {x[0], x[1], x[2]};
  bool ghost[2];
  const int axes[2] = {(own + 1) % 3, (own + 2) % 3};
  for (int h = 0; h < 2; ++h) {
    const int ax = axes[h];
    ghost[h] = side == 0 ? x[ax] == g.sh[c][ax] - 1 : x[ax] == 0;
    if (ghost[h]) s[ax] = side == 0 ? 0 : g.sh[c][ax] - 1;
  }
  double* fr = static_cast<double*>(g.f[c]);
  double* fi = fr + g.npts[c];
  const int64_t dst = x[0] * g.st[c][0] + x[1] * g.st[c][1] + x[2];
  const int64_t src = s[0] * g.st[c][0] + s[1] * g.st[c][1] + s[2];
  double vr = fr[src], vi = fi[src];
  for (int h = 0; h < 2; ++h) {
    if (!ghost[h]) continue;
    const double pr = g.phase[c][h][0], pi = g.phase[c][h][1];
    double nr, ni;
    if (STRICT) {
      nr = __fma_rn(pr, vr, -__dmul_rn(pi, vi));
      ni = __fma_rn(pr, vi, __dmul_rn(pi, vr));
    } else {
      nr = pr * vr - pi * vi;
      ni = pr * vi + pi * vr;
    }
    vr = nr;
    vi = ni;
  }
  fr[dst] = vr;
  fi[dst] = vi;
}

template <bool STRICT>
__global__ void k_ghost_c(const GridDev g, int side, int64_t maxplane) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= maxplane) return;
  ghost_point_c<STRICT>(g, side, blockIdx.y, t);
}

// Point sources of one half-step (gmes/pw_source.py:74-131), applied after
// that half's material update.  `v` has been computed on the host in FP64.
template <class P, bool STRICT>
__device__ __forceinline__ void source_point(const GridDev& g, int side, int64_t slot, int q) {
  const gmes_point_source ps = g.src[q];
  // the table is caller-provided device memory: skip entries that do not
  // name a point of an active component
  if (ps.comp < 0 || ps.comp > 5 || !(g.active & (1 << ps.comp))) return;
  if (ps.offset < 0 || ps.offset >= g.npts[ps.comp]) return;
  if ((ps.comp < 3) != (side == 0)) return;
  const double v = g.src_val[slot * g.nsrc + q];
  using T = typename P::T;
  T* f = static_cast<T*>(g.f[ps.comp]) + ps.offset;
  if (ps.mode == 0) {
    P::st(f, P::from_double(v));
  } else if constexpr (STRICT) {
    *reinterpret_cast<double*>(f) = __dsub_rn(*reinterpret_cast<double*>(f), v);
  } else {
    P::st(f, P::ldw(f) - P::from_double(v));
  }
}

// Point sources of one half-step (gmes/pw_source.py:74-131), applied after
// that half's material update.  The values were computed on the host in FP64.
template <class P, bool STRICT>
__global__ void k_sources(const GridDev g, int side, int64_t slot) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= g.nsrc) return;
  source_point<P, STRICT>(g, side, slot, q);
}

// TFSF consistency corrections of one half (gmes/pw_source.py:134-486):
// after the material update and the point sources, every face of a
// transparent point adds coef * (r0 A[s] + r1 A[s+1]) in face order, A the
// incident-field grid's Hy (E side) or Ex (H side).  Strict: the
// reference's operation order (coef is the signed dt/(eps d) * amp).
template <class P, bool STRICT>
__global__ void k_transparent(const GridDev g, int side) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= g.ntfsf) return;
  const gmes_transparent& t = g.tfsf[q];
  const int c = __ldg(&t.comp);
  if (c < 0 || c > 5 || !(g.active & (1 << c)) || (c < 3) != (side == 0)) return;
  const int64_t off = __ldg(&t.offset);
  if (off < 0 || off >= g.npts[c]) return;
  const int nf = __ldg(&t.nface);
  using T = typename P::T;
  using R = typename P::R;
  const T* A = static_cast<const T*>(g.tf_field[side]);
  const int64_t na = g.tf_npts[side];
  T* f = static_cast<T*>(g.f[c]) + off;
  if constexpr (STRICT) {
    double v = *reinterpret_cast<double*>(f);
    const double* a = reinterpret_cast<const double*>(A);
    for (int k = 0; k < nf && k < GMES_TFSF_MAX_FACES; ++k) {
      const int64_t sp = __ldg(&t.sample[k]);
      if (sp < 0 || sp + 1 >= na) continue;
      const double inc = __dadd_rn(__dmul_rn(__ldg(&t.r0[k]), a[sp]),
                                   __dmul_rn(__ldg(&t.r1[k]), a[sp + 1]));
      v = __dadd_rn(v, __dmul_rn(__ldg(&t.coef[k]), inc));
    }
    *reinterpret_cast<double*>(f) = v;
  } else {
    R v = P::ldw(f);
    for (int k = 0; k < nf && k < GMES_TFSF_MAX_FACES; ++k) {
      const int64_t sp = __ldg(&t.sample[k]);
      if (sp < 0 || sp + 1 >= na) continue;
      const R inc = P::from_double(__ldg(&t.r0[k])) * P::ldw(A + sp) +
                    P::from_double(__ldg(&t.r1[k])) * P::ldw(A + sp + 1);
      v = v + P::from_double(__ldg(&t.coef[k])) * inc;
    }
    P::st(f, v);
  }
}

// Probe recording of one half: the value of every probe of this half's
// components after its updates, sources and TFSF corrections.
template <class P>
__global__ void k_probes(const GridDev g, int side, int64_t slot) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= g.nprobe) return;
  const gmes_probe pr = g.probe[q];
  if (pr.comp < 0 || pr.comp > 5 || (pr.comp < 3) != (side == 0)) return;
  double v = 0.0;
  if ((g.active & (1 << pr.comp)) && pr.offset >= 0 && pr.offset < g.npts[pr.comp])
    v = to_double(P::ldw(static_cast<const typename P::T*>(g.f[pr.comp]) + pr.offset));
  g.probe_val[slot * g.nprobe + q] = v;
}

// ---------------------------------------------------------------------------
// Multi-grid ("batch") form: one launch per half-step advances every grid of
// a batch.  The per-grid views live in a caller-allocated workspace with
// prefix sums of each grid's blocks, ghost-plane points and sources; a block
// (or thread) finds its grid by binary search in the prefix array and runs
// exactly the per-grid code, so a grid's result does not depend on what else
// is in the batch.  Grids with steps[g] <= s sit out step s of the chunk.
// ---------------------------------------------------------------------------
template <class I>
__device__ __forceinline__ int find_job(const I* prefix, int njobs, I v) {
  int lo = 0, hi = njobs;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(prefix + mid) <= v)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

static_assert(sizeof(GridDev) % 16 == 0, "GridDev is copied as 16-byte words");

// The tile's grid descriptor is copied to shared memory when the block's
// job changes and read from there: read from global memory, its fields
// (pointers, strides, tables of six components) cost the batched FP32
// half-step ~70 extra global loads per cell and ran it 1.7x slower than
// the single-grid kernel, whose descriptor is a kernel parameter; from
// shared memory it runs 1.3x slower (measured on GB300, 160^3 cube).
template <class P, int SIDE, bool STRICT, bool DISP>
__global__ void __launch_bounds__(kBatchThreads, MultiMinBlocks<P, SIDE, DISP>::value)
    k_multi_cell(const BatchView v, int s, int64_t per) {
  __shared__ __align__(16) unsigned char desc[sizeof(GridDev)];
  const GridDev& g = *reinterpret_cast<const GridDev*>(desc);
  int cached = -1;
  // a persistent grid (fewer blocks than tiles) gives each block a
  // contiguous range of per tiles (ceil(tiles / blocks), from the host: a
  // 64-bit division here cost every thread tens of instructions), so that a
  // block mostly stays on one grid and copies its descriptor once
  const int64_t b0 = (int64_t)blockIdx.x * per;
  const int64_t b1 = b0 + per < v.tiles ? b0 + per : v.tiles;
  for (int64_t b = b0; b < b1; ++b) {
    const int job = find_job<int64_t>(v.tile_prefix, v.njobs, b);  // block-uniform
    if (s >= __ldg(v.steps + job)) continue;
    if (job != cached) {
      __syncthreads();  // the previous descriptor is no longer read
      const uint4* src = reinterpret_cast<const uint4*>(v.jobs + job);
      uint4* dst = reinterpret_cast<uint4*>(desc);
      for (int w = threadIdx.x; w < (int)(sizeof(GridDev) / 16); w += blockDim.x)
        dst[w] = __ldg(src + w);
      __syncthreads();
      cached = job;
    }
    const TileDiv& td = v.td[job];
    const int bxl = __ldg(&td.bxl);
    const int bx = 1 << bxl, by = kBatchThreads >> bxl;
    // a grid has fewer than 2^31 tiles: quotients by multiply and shift
    const unsigned local = (unsigned)(b - __ldg(v.tile_prefix + job));
    const unsigned plane = __ldg(&td.plane), nkb = __ldg(&td.nkb);
    const int i = (int)tile_quot(local, __ldg(&td.m_plane), __ldg(&td.s_plane));
    const unsigned rem = local - (unsigned)i * plane;
    const unsigned jq = tile_quot(rem, __ldg(&td.m_nkb), __ldg(&td.s_nkb));
    const int jb = (int)jq, kb = (int)(rem - jq * nkb);
    const int k = kb * bx + (threadIdx.x & (bx - 1));
    const int j = jb * by + (threadIdx.x >> bxl);
    // batched grids hold fewer than 2^31 points per component (checked when
    // the batch is prepared)
    if (k < g.n[2] && j < g.n[1]) {
      if constexpr (STRICT)
        cell_body<P, SIDE, STRICT, DISP, 0, int32_t>(g, i, j, k);
      else
        cell_body_fast<P, SIDE, DISP, 0, int32_t>(g, i, j, k);
    }
  }
}

// The same with the descriptors in the kernel's argument bank (batches of
// at most kParamJobs grids): no shared-memory copy and no barrier per tile.
template <class P, int SIDE, bool STRICT, bool DISP>
__global__ void __launch_bounds__(kBatchThreads, MultiMinBlocks<P, SIDE, DISP>::value)
    k_multi_cell_arg(const BatchView v, int s, int64_t per, const __grid_constant__ BatchDescs d) {
  const int64_t b0 = (int64_t)blockIdx.x * per;
  const int64_t b1 = b0 + per < v.tiles ? b0 + per : v.tiles;
  for (int64_t b = b0; b < b1; ++b) {
    const int job = find_job<int64_t>(v.tile_prefix, v.njobs, b);  // block-uniform
    if (s >= __ldg(v.steps + job)) continue;
    const GridDev& g = d.jobs[job];
    const TileDiv& td = v.td[job];
    const int bxl = __ldg(&td.bxl);
    const int bx = 1 << bxl, by = kBatchThreads >> bxl;
    // a grid has fewer than 2^31 tiles: quotients by multiply and shift
    const unsigned local = (unsigned)(b - __ldg(v.tile_prefix + job));
    const unsigned plane = __ldg(&td.plane), nkb = __ldg(&td.nkb);
    const int i = (int)tile_quot(local, __ldg(&td.m_plane), __ldg(&td.s_plane));
    const unsigned rem = local - (unsigned)i * plane;
    const unsigned jq = tile_quot(rem, __ldg(&td.m_nkb), __ldg(&td.s_nkb));
    const int jb = (int)jq, kb = (int)(rem - jq * nkb);
    const int k = kb * bx + (threadIdx.x & (bx - 1));
    const int j = jb * by + (threadIdx.x >> bxl);
    if (k < g.n[2] && j < g.n[1]) {
      if constexpr (STRICT)
        cell_body<P, SIDE, STRICT, DISP, 0, int32_t>(g, i, j, k);
      else
        cell_body_fast<P, SIDE, DISP, 0, int32_t>(g, i, j, k);
    }
  }
}

template <class T>
__global__ void k_multi_ghost(const BatchView v, int side, int s) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < v.ghosts;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int job = find_job<int64_t>(v.ghost_prefix, v.njobs, t);
    if (s >= __ldg(v.steps + job)) continue;
    const GridDev& g = v.jobs[job];
    const int64_t local = t - __ldg(v.ghost_prefix + job);
    const int64_t per = (__ldg(v.ghost_prefix + job + 1) - __ldg(v.ghost_prefix + job)) / 6;
    ghost_point<T>(g, side, (int)(local / per), local % per);
  }
}

template <class P, bool STRICT>
__global__ void k_multi_sources(const BatchView v, int side, int s) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < v.srcs; t += gridDim.x * blockDim.x) {
    const int job = find_job<int>(v.src_prefix, v.njobs, t);
    if (s >= __ldg(v.steps + job)) continue;
    source_point<P, STRICT>(v.jobs[job], side, 2 * (int64_t)s + side, t - __ldg(v.src_prefix + job));
  }
}

template <class P, bool STRICT>
cudaError_t run_steps(const Plan& p, int nsteps, int side_mask, int st0, cudaStream_t s);

// One half-step: ghost copy of the other half's components, the fused
// update of this half's components, this half's point sources, TFSF
// corrections and probes; after the E half, one full step of the TFSF
// incident-field grid (FDTD.step's _step_aux_fdtd, gmes/fdtd.py:1113).
// A complex grid runs every per-plane kernel on its real and imaginary
// planes; only the ghost copy couples them.
template <class P, bool STRICT>
void run_half(const Plan& p, int side, int st, cudaStream_t s) {
  using T = typename P::T;
  const GridDev& d = p.re;
  int64_t maxplane = 1;
  for (int c = 0; c < 6; ++c)
    for (int a = 0; a < 3; ++a)
      for (int b = a + 1; b < 3; ++b) {
        const int64_t v = d.sh[c][a] * d.sh[c][b];
        maxplane = v > maxplane ? v : maxplane;
      }
  const dim3 ggrid((unsigned)((maxplane + 255) / 256), 6);
  constexpr int kMaxY = 65535;
  if (p.cplx)
    k_ghost_c<STRICT><<<ggrid, 256, 0, s>>>(d, 1 - side, maxplane);
  else if (offsets_fit_i32(d))
    k_ghost32<T><<<ggrid, 256, 0, s>>>(d, 1 - side, (unsigned)maxplane);
  else
    k_ghost<T><<<ggrid, 256, 0, s>>>(d, 1 - side, maxplane);
  const CellTiling tl = cell_tiling(d.n);
  const int bx_log2 = tl.bx_log2, bx = tl.bx, by = tl.by;
  const int nplanes = p.cplx ? 2 : 1;
  for (int part = 0; part < nplanes; ++part) {
    const GridDev& v = part == 0 ? p.re : p.im;
    for (int i0 = 0; i0 < d.n[0]; i0 += kMaxY) {
      const dim3 grid((unsigned)((d.n[2] + bx - 1) / bx), (unsigned)((d.n[1] + by - 1) / by),
                      (unsigned)min(kMaxY, d.n[0] - i0));
      // Measured on GB300 (256^3 cube): 32-bit offsets run the FP64 step 7%
      // and the df64 step 6% faster than 64-bit ones (fewer registers and
      // spills), so every grid whose components hold fewer than 2^31 points
      // takes them; a compile-time active mask (all six components) ran ~35%
      // slower, so the mask stays a runtime value.
      if (offsets_fit_i32(d))
        launch_cell<P, STRICT, 0, int32_t>(v, side, p.disp, grid, bx_log2, i0, s);
      else
        launch_cell<P, STRICT, 0, int64_t>(v, side, p.disp, grid, bx_log2, i0, s);
    }
  }
  for (int part = 0; part < nplanes; ++part) {
    const GridDev& v = part == 0 ? p.re : p.im;
    if (v.nsrc > 0)
      k_sources<P, STRICT><<<(v.nsrc + 127) / 128, 128, 0, s>>>(v, side, 2 * (int64_t)st + side);
    if (v.ntfsf > 0) k_transparent<P, STRICT><<<(v.ntfsf + 127) / 128, 128, 0, s>>>(v, side);
    if (v.nprobe > 0) k_probes<P><<<(v.nprobe + 127) / 128, 128, 0, s>>>(v, side, st);
  }
  if (side == 0 && p.incident != nullptr) run_steps<P, STRICT>(*p.incident, 1, 3, st, s);
}

template <class P, bool STRICT>
cudaError_t run_steps(const Plan& p, int nsteps, int side_mask, int st0, cudaStream_t s) {
  for (int st = 0; st < nsteps; ++st) {
    if (side_mask & 1) run_half<P, STRICT>(p, 0, st0 + st, s);
    if (side_mask & 2) run_half<P, STRICT>(p, 1, st0 + st, s);
  }
  return cudaGetLastError();
}

cudaError_t dispatch_precision(const gmes_grid_desc& g, const Plan& p, int nsteps,
                               int side_mask, int st0, cudaStream_t s) {
  switch (g.precision) {
    case GMES_FP64:
      return run_steps<PolF64, false>(p, nsteps, side_mask, st0, s);
    case GMES_FP64_STRICT:
      return run_steps<PolF64, true>(p, nsteps, side_mask, st0, s);
    case GMES_FP32:
      return run_steps<PolF32, false>(p, nsteps, side_mask, st0, s);
    case GMES_DF64:
      return run_steps<PolDF, false>(p, nsteps, side_mask, st0, s);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace

template <class P, bool STRICT>
cudaError_t run_batch(const BatchView& v, const GridDev* host_jobs, bool disp, int nsteps,
                      int blocks, cudaStream_t st) {
  using T = typename P::T;
  const int cells = blocks > 0 ? blocks : (int)(v.tiles < (1 << 30) ? v.tiles : (1 << 30));
  const int64_t per = cells > 0 ? (v.tiles + cells - 1) / cells : 0;  // tiles per block
  const int gblocks = (int)((v.ghosts + 255) / 256 < 65535 * 16 ? (v.ghosts + 255) / 256 : 65535 * 16);
  const int sblocks = (v.srcs + 127) / 128;
  const bool arg = ArgDescs<P>::value && host_jobs != nullptr && v.njobs <= kParamJobs;
  static thread_local BatchDescs descs;
  if (arg) {
    std::memset(&descs, 0, sizeof(descs));
    for (int q = 0; q < v.njobs; ++q) descs.jobs[q] = host_jobs[q];
  }
  for (int s = 0; s < nsteps; ++s) {
    for (int side = 0; side < 2; ++side) {
      if (gblocks > 0) k_multi_ghost<T><<<gblocks, 256, 0, st>>>(v, 1 - side, s);
      if (cells > 0) {
        if (arg) {
          if (side == 0) {
            if (disp)
              k_multi_cell_arg<P, 0, STRICT, true><<<cells, kBatchThreads, 0, st>>>(v, s, per, descs);
            else
              k_multi_cell_arg<P, 0, STRICT, false><<<cells, kBatchThreads, 0, st>>>(v, s, per, descs);
          } else {
            k_multi_cell_arg<P, 1, STRICT, false><<<cells, kBatchThreads, 0, st>>>(v, s, per, descs);
          }
        } else if (side == 0) {
          if (disp)
            k_multi_cell<P, 0, STRICT, true><<<cells, kBatchThreads, 0, st>>>(v, s, per);
          else
            k_multi_cell<P, 0, STRICT, false><<<cells, kBatchThreads, 0, st>>>(v, s, per);
        } else {
          k_multi_cell<P, 1, STRICT, false><<<cells, kBatchThreads, 0, st>>>(v, s, per);
        }
      }
      if (sblocks > 0) k_multi_sources<P, STRICT><<<sblocks, 128, 0, st>>>(v, side, s);
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_batch(const BatchView& v, const GridDev* host_jobs, int precision, bool disp,
                         int nsteps, int blocks, cudaStream_t s) {
  switch (precision) {
    case GMES_FP64:
      return run_batch<PolF64, false>(v, host_jobs, disp, nsteps, blocks, s);
    case GMES_FP64_STRICT:
      return run_batch<PolF64, true>(v, host_jobs, disp, nsteps, blocks, s);
    case GMES_FP32:
      return run_batch<PolF32, false>(v, host_jobs, disp, nsteps, blocks, s);
    case GMES_DF64:
      return run_batch<PolDF, false>(v, host_jobs, disp, nsteps, blocks, s);
    default:
      return cudaErrorInvalidValue;
  }
}

// Non-finite guard (gmes_nonfinite): an infinity or NaN has an all-ones
// exponent; the test is on the bits, so no floating-point pipe is used.
__device__ __forceinline__ bool nonfinite(double v) {
  return ((__double_as_longlong(v) >> 52) & 0x7ff) == 0x7ff;
}
__device__ __forceinline__ bool nonfinite(float v) {
  return ((__float_as_uint(v) >> 23) & 0xff) == 0xff;
}
__device__ __forceinline__ bool nonfinite(float2 v) { return nonfinite(v.x); }  // hi word

template <class T>
__global__ void k_nonfinite(const GridDev g, int planes, int32_t* flag) {
  bool bad = false;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int c = 0; c < 6; ++c) {
    if (!((g.active >> c) & 1)) continue;
    const T* f = static_cast<const T*>(g.f[c]);
    const int64_t n = g.npts[c] * planes;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride)
      bad = bad || nonfinite(f[t]);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) *flag = 1;
}

cudaError_t launch_nonfinite(const gmes_grid_desc& g, const GridDev& d, int32_t* flag,
                             cudaStream_t s) {
  const int planes = (g.flags & GMES_FLAG_COMPLEX) ? 2 : 1;
  int64_t most = 1;
  for (int c = 0; c < 6; ++c) most = d.npts[c] * planes > most ? d.npts[c] * planes : most;
  const int blocks = (int)((most + 255) / 256 < 152 * 8 ? (most + 255) / 256 : 152 * 8);
  switch (g.precision) {
    case GMES_FP64:
    case GMES_FP64_STRICT:
      k_nonfinite<double><<<blocks, 256, 0, s>>>(d, planes, flag);
      break;
    case GMES_FP32:
      k_nonfinite<float><<<blocks, 256, 0, s>>>(d, planes, flag);
      break;
    case GMES_DF64:
      k_nonfinite<float2><<<blocks, 256, 0, s>>>(d, planes, flag);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_step(const gmes_grid_desc& g, const Plan& p, int nsteps, cudaStream_t s) {
  return dispatch_precision(g, p, nsteps, 3, 0, s);
}

cudaError_t launch_half(const gmes_grid_desc& g, const Plan& p, int side, int step,
                        cudaStream_t s) {
  return dispatch_precision(g, p, 1, side == 0 ? 1 : 2, step, s);
}

}  // namespace gmes
