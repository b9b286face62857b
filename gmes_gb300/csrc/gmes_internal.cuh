// Internal definitions shared by the engine's translation units:
// coefficient-block layout (host and device agree through the same
// functions), the kernel-side grid view, and the three arithmetic policies
// (FP64, FP32, float-float).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gmes_gb300.h"

namespace gmes {

// ---------------------------------------------------------------------------
// Coefficients.  Every coefficient is computed once in FP64 on the GPU and
// stored in three forms so no kernel converts on the hot path:
//   d  -- FP64 (GMES_FP64, GMES_FP64_STRICT)
//   hi -- FP32 round-to-nearest of d (GMES_FP32; high word of GMES_DF64)
//   lo -- FP32 of (d - hi)  (low word of GMES_DF64)
// ---------------------------------------------------------------------------
struct Coef {
  double d;
  float hi, lo;
};

// True unless the coefficient is +0 or -0 (bit test: no FP64 instruction).
__device__ __forceinline__ bool coef_nonzero(const Coef* c) {
  return (__ldg(reinterpret_cast<const unsigned long long*>(&c->d)) << 1) != 0ull;
}

__host__ __device__ inline Coef make_coef(double v) {
  Coef c;
  c.d = v;
  c.hi = static_cast<float>(v);
  c.lo = static_cast<float>(v - static_cast<double>(c.hi));
  return c;
}

// Per (component, class) entry of the class table.
struct ClassCoef {
  int32_t kind, pml, npole, ncp;
  int32_t pad[4];
  Coef eps;   // eps_inf (E) / mu_inf (H)
  Coef cdt;   // dt / eps
  Coef c1;    // dt / eps / d1   (d1, d2: cell sizes of the two curl axes)
  Coef c2;    // dt / eps / d2
  Coef reps;  // 1 / eps
  Coef value; // CONST (real part)
  Coef value_im; // CONST, imaginary part (complex grids)
};

// Dispersive coefficients of one class: a[p][3] (Drude/Lorentz poles or DCP
// Drude terms), b[q][5] (DCP-ADE critical points; DCP-PLRC: b0, b1, b2 as
// re/im pairs, 6 per point), c[4].
constexpr int kPoolA = 0;
constexpr int kPoolB = 3 * GMES_MAX_POLES;
constexpr int kPoolC = kPoolB + 6 * GMES_MAX_POLES;
constexpr int kPoolStride = kPoolC + 4;

// PML profile entry at one index along one axis (5 coefficients):
//   CPML: b, c, kappa, c / d, 1 / (kappa d)
//   UPML: c1 (= c3), c2, c4, c5, c6     (src/material.pyx:558-591)
constexpr int kProfStride = 5;

// Yee staggering, rows Ex..Hz (gmes/geometry.py:360-732).
__host__ __device__ inline double yee_offset(int c, int axis) {
  if (c < 3) return axis == c ? 0.5 : 0.0;
  return axis == c - 3 ? 0.0 : -0.5;
}

__host__ __device__ inline void comp_shape(const int32_t n[3], int32_t active, int c,
                                           int64_t sh[3]) {
  if (!(active & (1 << c))) {
    sh[0] = sh[1] = sh[2] = 1;
    return;
  }
  const int own = c % 3;
  for (int a = 0; a < 3; ++a) sh[a] = a == own ? n[a] : n[a] + 1;
}

__host__ __device__ inline int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

// ---------------------------------------------------------------------------
// Block tiling of the single-grid cell kernels.  A block of kCellThreads
// threads covers bx cells along k (bx = 2^bx_log2, at most 2^kRowLog2, the
// smallest power of two >= n2 below that) by kCellThreads / bx rows along j,
// at one i; blocks are numbered ((i * njb) + jb) * nkb + kb.  Warp w of a
// block covers its threads 32 w .. 32 w + 31.
// ---------------------------------------------------------------------------
#ifndef GMES_CELL_THREADS
#define GMES_CELL_THREADS 128
#endif
constexpr int kCellThreads = GMES_CELL_THREADS;
constexpr int kCellWarps = kCellThreads / 32;
#ifndef GMES_ROW_LOG2
#define GMES_ROW_LOG2 4
#endif
constexpr int kRowLog2 = GMES_ROW_LOG2;

struct CellTiling {
  int bx_log2, bx, by, nkb, njb;
  int64_t blocks;  // nkb * njb * n0
};

__host__ __device__ inline CellTiling cell_tiling(const int32_t n[3]) {
  CellTiling t;
  t.bx_log2 = 0;
  while (t.bx_log2 < kRowLog2 && (1 << t.bx_log2) < n[2]) ++t.bx_log2;
  t.bx = 1 << t.bx_log2;
  t.by = kCellThreads / t.bx;
  t.nkb = (n[2] + t.bx - 1) / t.bx;
  t.njb = (n[1] + t.by - 1) / t.by;
  t.blocks = (int64_t)t.nkb * t.njb * n[0];
  return t;
}

// Coefficient block layout (offsets in bytes from g.coef).
struct CoefLayout {
  int64_t raw_classes;  // gmes_class_desc[sum nclass] (host input staging)
  int64_t raw_params;   // double[nparam]
  int64_t raw_pmls;     // gmes_pml_desc[npml]
  int64_t class_tab[6]; // ClassCoef[nclass[c]]
  int64_t pool[6];      // Coef[nclass[c] * kPoolStride]
  int64_t prof[GMES_MAX_PML][6][3];  // Coef[shape[c][axis] * kProfStride]
  int64_t total;
};

__host__ __device__ inline CoefLayout coef_layout(const gmes_grid_desc& g) {
  CoefLayout L;
  int64_t off = 0;
  int64_t ncls = 0;
  for (int c = 0; c < 6; ++c) ncls += g.nclass[c];
  L.raw_classes = off;
  off = align256(off + ncls * (int64_t)sizeof(gmes_class_desc));
  L.raw_params = off;
  off = align256(off + (int64_t)g.nparam * 8);
  L.raw_pmls = off;
  off = align256(off + (int64_t)g.npml * (int64_t)sizeof(gmes_pml_desc));
  // Every component gets a full 256-entry class table: a class id without a
  // class (any u8 value) reads a zeroed entry, i.e. kind DUMMY -- no update.
  for (int c = 0; c < 6; ++c) {
    L.class_tab[c] = off;
    off = align256(off + (int64_t)GMES_MAX_CLASSES * (int64_t)sizeof(ClassCoef));
  }
  for (int c = 0; c < 6; ++c) {
    L.pool[c] = off;
    off = align256(off + (int64_t)g.nclass[c] * kPoolStride * (int64_t)sizeof(Coef));
  }
  for (int p = 0; p < GMES_MAX_PML; ++p)
    for (int c = 0; c < 6; ++c)
      for (int a = 0; a < 3; ++a) {
        L.prof[p][c][a] = off;
        if (p < g.npml) {
          int64_t sh[3];
          comp_shape(g.n, g.active, c, sh);
          off = align256(off + sh[a] * kProfStride * (int64_t)sizeof(Coef));
        }
      }
  L.total = align256(off);
  return L;
}

// ---------------------------------------------------------------------------
// Kernel-side view of a grid (passed by value as a kernel parameter).
// ---------------------------------------------------------------------------
struct GridDev {
  int32_t n[3];
  int32_t active;
  int32_t nsrc;
  int32_t pointwise;      // GMES_FLAG_POINTWISE: no warp-uniform plain updates
  int64_t sh[6][3];       // component shapes
  int64_t st[6][2];       // strides of axes 0 and 1 (axis 2 stride is 1)
  int64_t npts[6];        // points per component
  int32_t naux[6];        // state slots per point
  void* f[6];
  const uint8_t* cls[6];
  void* aux[6];
  const ClassCoef* tab[6];
  const Coef* pool[6];
  const Coef* prof[GMES_MAX_PML][6][3];
  const gmes_point_source* src;
  const double* src_val;
  double dr[3];
  double dt;
  Coef rdr[3];            // 1 / dr, computed on the host
  // TFSF plane-wave source: transparent points and the incident-field
  // arrays they sample (the aux grid's Hy for the E side, Ex for the H side)
  const gmes_transparent* tfsf;
  int32_t ntfsf;
  int32_t pad2;
  const void* tf_field[2];
  int64_t tf_npts[2];
  // probes: values recorded per step of a call
  const gmes_probe* probe;
  double* probe_val;
  int32_t nprobe;
  int32_t pad3;
  double phase[6][2][2];   // Bloch phase factors (complex grids)
  int32_t part;            // 0: real plane, 1: imaginary plane (complex grids)
  int32_t pad4;
  // strides of axes 0 and 1 of the three array shapes: X = Ex/Hx
  // (n0, n1+1, n2+1), Y = Ey/Hy (n0+1, n1, n2+1), Z = Ez/Hz (n0+1, n1+1, n2);
  // an active component's strides are its family's
  int64_t fst[3][2];
};

// Host-side launch plan of one grid: its real-plane view, the imaginary-
// plane view of a complex grid, and the TFSF incident-field grid's plan.
struct Plan {
  GridDev re, im;
  bool cplx, disp;
  const Plan* incident;
};

// ---------------------------------------------------------------------------
// Arithmetic policies.
// ---------------------------------------------------------------------------

// Float-float number: value = hi + lo with |lo| <= ulp(hi)/2.  Operations are
// the classical error-free transformations (Knuth two-sum, Dekker/FMA
// two-product) written with round-to-nearest intrinsics so the compiler can
// neither contract nor reassociate them.
struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ df df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df operator+(df a, df b) {
  df s = df_two_sum(a.hi, b.hi);
  const df t = df_two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = df_fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return df_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df operator-(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }

// a b + c in one pass: the product's high word and its exact error (FMA),
// the cross terms, then a two-sum with c's high word whose error absorbs the
// low-order terms (15 FP32 operations against 27 for a product followed by
// an accurate sum).  The low-order terms are added without their own error
// term, so a result that cancels most of c carries an absolute error of
// about 2^-48 |c|.
__device__ __forceinline__ df df_fma(df a, df b, df c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  df s = df_two_sum(p, c.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(e, c.lo));
  return df_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df operator*(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}

struct PolF64 {
  using T = double;
  using R = double;
  static __device__ __forceinline__ R ld(const T* p) { return __ldg(p); }
  static __device__ __forceinline__ R ldw(const T* p) { return *p; }
  static __device__ __forceinline__ void st(T* p, R v) { *p = v; }
  static __device__ __forceinline__ R cf(const Coef& c) { return c.d; }
  static __device__ __forceinline__ R cfg(const Coef* c) { return __ldg(&c->d); }
  static __device__ __forceinline__ R zero() { return 0.0; }
  static __device__ __forceinline__ R from_double(double v) { return v; }
};

struct PolF32 {
  using T = float;
  using R = float;
  static __device__ __forceinline__ R ld(const T* p) { return __ldg(p); }
  static __device__ __forceinline__ R ldw(const T* p) { return *p; }
  static __device__ __forceinline__ void st(T* p, R v) { *p = v; }
  static __device__ __forceinline__ R cf(const Coef& c) { return c.hi; }
  static __device__ __forceinline__ R cfg(const Coef* c) { return __ldg(&c->hi); }
  static __device__ __forceinline__ R zero() { return 0.f; }
  static __device__ __forceinline__ R from_double(double v) { return static_cast<float>(v); }
};

struct PolDF {
  using T = float2;
  using R = df;
  static __device__ __forceinline__ R ld(const T* p) {
    const float2 v = __ldg(p);
    return {v.x, v.y};
  }
  static __device__ __forceinline__ R ldw(const T* p) {
    const float2 v = *p;
    return {v.x, v.y};
  }
  static __device__ __forceinline__ void st(T* p, R v) { *p = make_float2(v.hi, v.lo); }
  static __device__ __forceinline__ R cf(const Coef& c) { return {c.hi, c.lo}; }
  static __device__ __forceinline__ R cfg(const Coef* c) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(&c->hi));
    return {v.x, v.y};
  }
  static __device__ __forceinline__ R zero() { return {0.f, 0.f}; }
  static __device__ __forceinline__ R from_double(double v) {
    const float h = static_cast<float>(v);
    return {h, static_cast<float>(v - static_cast<double>(h))};
  }
};

// FP64 value of an arithmetic-policy number (records, gradients).
__device__ __forceinline__ double to_double(double v) { return v; }
__device__ __forceinline__ double to_double(float v) { return (double)v; }
__device__ __forceinline__ double to_double(df v) { return (double)v.hi + (double)v.lo; }

// Threads per block of the multi-grid half-step kernel: the single-grid
// kernel's shape.
constexpr int kBatchThreads = kCellThreads;

// Kernel-side view of a batch workspace (gmes_batch_prepare).
// True when every component of the grid holds fewer than 2^31 points, so
// the cell kernels may index it with 32-bit offsets.
inline bool offsets_fit_i32(const GridDev& d) {
  for (int c = 0; c < 6; ++c)
    if (d.npts[c] >= (int64_t(1) << 31)) return false;
  return true;
}

// How a grid's tiles (blocks of the cell kernel) are numbered in the
// multi-grid kernels: tile t of the grid lies in plane i = t / plane, block
// row jb = (t - i plane) / nkb and block column kb = t - i plane - jb nkb.
// Each quotient is a product and a shift (tile_quot) with the multiplier
// and shift from tile_div_of, exact for t < 2^31.
struct TileDiv {
  int32_t bxl;              // log2 of the block's k extent
  uint32_t nkb;             // blocks per row along k
  uint32_t plane;           // blocks per plane (nkb x blocks along j)
  uint32_t m_nkb, m_plane;  // multipliers of / nkb and / plane
  int32_t s_nkb, s_plane;   // their shifts
  int32_t pad;
};

// n / d = (n m) >> s for 0 <= n < 2^31 and 1 <= d < 2^31, with l = ceil(log2
// d), m = ceil(2^(31+l) / d) (below 2^32) and s = 31 + l: n m / 2^s exceeds
// n / d by less than n / 2^s < 2^-l <= 1 / d, which never reaches the next
// integer.
inline void tile_div_of(uint32_t d, uint32_t& m, int32_t& s) {
  int l = 0;
  while ((uint64_t(1) << l) < d) ++l;
  const uint64_t p = uint64_t(1) << (31 + l);
  m = (uint32_t)((p + d - 1) / d);
  s = 31 + l;
}

__device__ __forceinline__ unsigned tile_quot(unsigned n, unsigned m, int s) {
  return (unsigned)(((unsigned long long)n * m) >> s);
}

struct BatchView {
  const GridDev* jobs;
  const int64_t* tile_prefix;   // [njobs + 1] blocks of each grid's half-step
  const TileDiv* td;            // per grid: tile numbering
  const int32_t* steps;         // per grid: steps to take in this chunk
  const int64_t* ghost_prefix;  // [njobs + 1] 6 x (largest ghost plane) per grid
  const int32_t* src_prefix;    // [njobs + 1] point sources
  int32_t njobs;
  int32_t srcs;
  int64_t tiles;
  int64_t ghosts;
};

// ---------------------------------------------------------------------------
// Differentiation (batched TMz forward + adjoint, gmes_adjoint.cu).
// ---------------------------------------------------------------------------
// Per design pixel: the Ez update coefficients dt/eps/dx, dt/eps/dy (built
// like a dielectric class's c1, c2) and -1/eps for the gradient.
struct DesignCoef {
  Coef c1, c2;
  double neg_reps;
  double eps;
};

// Number of arrays in the forward state and adjoint blocks.
constexpr int kTmzState = 7;    // Ez, Hx, Hy, psi_ez(x), psi_ez(y), psi_hx(y), psi_hy(x)
constexpr int kTmzAdjoint = 11; // lambda Ez, Hx, Hy, then 2 x the adjoints of the 4 psi

struct TmzDev {
  int32_t nx, ny, nb, nsrc;
  int64_t plane;            // nx * ny lattice points per array per design
  int32_t d0[2], dn[2];     // design box (lattice indices, extent)
  int32_t m0[2], mn[2];     // monitor box
  int32_t total_steps, hist_steps;
  void* f[kTmzState];       // [nb][nx][ny] each
  void* tmp[kTmzState];     // scratch copy of the state (blocked kernels), or null
  // Resolved update of every lattice point, shared by the batch (written by
  // launch_tmz_design): flags (kTmz* below) and the plain-form coefficients
  // c1, -c2 (Ez), -c1 (Hx), c2 (Hy) as [nx][ny] arrays of the precision's type.
  const uint32_t* pflags;
  const void* pcoef[4];
  void* l[3];
  void* phi[2][4];          // ping-pong buffers of the psi adjoints
  const DesignCoef* dc;     // [nb][nd]
  void* hist;               // [hist_steps][nb][nd]
  double* mon;              // [nb][total_steps][nm]
  double* grad;             // [nb][nd]
  const double* weight;     // [nb] or null
  const gmes_point_source* src;
  const double* src_val;    // [total_steps][2][nsrc]
};

// Flags of the resolved lattice map.  "Plain": the update is
// F + c1 D1 + c2 D2 with per-point coefficients (dielectric points, design
// pixels, CPML points outside both of their profiles); "psi": a CPML point
// inside a profile (keeps psi state); neither: the point is not updated.
// kTmzSrcE / kTmzSrcH: a point source of the E / H half sits on the point.
// For psi points, kTmzOn*: which of the point's profiles are on (Ez: along
// x and y; Hx: along y; Hy: along x) and the 2-bit fields at kTmzPml*: the
// class's profile set.
enum : uint32_t {
  kTmzPlainE = 1, kTmzPlainX = 2, kTmzPlainY = 4,
  kTmzPsiE = 8, kTmzPsiX = 16, kTmzPsiY = 32,
  kTmzDesign = 64, kTmzMonitor = 128,
  kTmzSrcE = 256, kTmzSrcH = 512,
  kTmzOnE1 = 1024, kTmzOnE2 = 2048, kTmzOnX = 4096, kTmzOnY = 8192
};
constexpr int kTmzPmlE = 16, kTmzPmlX = 18, kTmzPmlY = 20;  // bit offsets
static_assert(GMES_MAX_PML <= 4, "2-bit profile-set fields");

cudaError_t launch_tmz_design(int precision, const GridDev& g, const TmzDev& t,
                              const double* eps, cudaStream_t s);
cudaError_t launch_tmz_forward(int precision, const GridDev& g, const TmzDev& t, int step0,
                               int nsteps, int flags, int block_steps, cudaStream_t s);
cudaError_t launch_tmz_adjoint(int precision, const GridDev& g, const TmzDev& t, int step0,
                               int nsteps, int block_steps, cudaStream_t s);
cudaError_t launch_tmz_objective(const GridDev& g, const TmzDev& t, int nsteps, double* J,
                                 cudaStream_t s);

cudaError_t launch_points(const gmes_points& g, void* inplace, const void* in1, const void* in2,
                          double d1, double d2, double dt, cudaStream_t s);

// Host-side helpers implemented in gmes_capi.cu.
GridDev make_grid_dev(const gmes_grid_desc& g);

// Launchers implemented per precision in gmes_step.cu.
cudaError_t launch_step(const gmes_grid_desc& g, const Plan& p, int nsteps, cudaStream_t s);
cudaError_t launch_half(const gmes_grid_desc& g, const Plan& p, int side, int step,
                        cudaStream_t s);
// The descriptors of a batch of at most kParamJobs grids, passed by value
// to the multi-grid cell kernel (kernel arguments are limited to 32764
// bytes), so that a cell reads its grid's fields from the argument bank as
// the single-grid kernel does.
constexpr int kParamJobs = 20;
struct BatchDescs {
  GridDev jobs[kParamJobs];
};
static_assert(sizeof(BatchDescs) + 512 <= 32764, "batch descriptors exceed the argument space");

// host_jobs: host copies of the batch's descriptors (v.jobs), or NULL; with
// them a batch of at most kParamJobs grids may take the argument-bank kernel.
cudaError_t launch_batch(const BatchView& v, const GridDev* host_jobs, int precision, bool disp,
                         int nsteps, int blocks, cudaStream_t s);
cudaError_t launch_raster(const gmes_grid_desc& gd, const GridDev& d, int c,
                          const gmes_shape* shapes, int nshapes, const uint8_t* lut,
                          cudaStream_t s);
cudaError_t launch_build_coefficients(const gmes_grid_desc& g, const GridDev& d,
                                      cudaStream_t s);
cudaError_t launch_nonfinite(const gmes_grid_desc& g, const GridDev& d, int32_t* flag,
                             cudaStream_t s);

}  // namespace gmes
