// Differentiation: gradient of a monitor objective with respect to the
// permittivity of a design region, for a batch of TMz designs that share
// geometry, PML and sources and differ only in the design pixels.
//
// The reference has no adjoint; the forward map differentiated here is its
// TMz time step (gmes/fdtd.py:1099-1122) with the Dielectric and CPML
// updaters of src/pw_dielectric.hh:281-371 (Hx, Hy), src/pw_dielectric.hh:186-199
// (Ez), src/pw_cpml.hh:211-237, 319-397 and the point sources of
// gmes/pw_source.py:74-131.
//
// Lattice.  With N = (nx, ny, 1), the TMz fields live on one periodic
// nx x ny lattice per design:
//   E(i, j) = Ez[i, j, 0],  X(i, j) = Hx[i, j+1, 1],  Y(i, j) = Hy[i+1, j, 1]
// The reference's ghost planes (Ez[nx, :], Ez[:, ny], Hx[:, 0, :], Hy[0])
// only ever hold copies of these points (talk_with_*_neighbors,
// gmes/fdtd.py:811-1097), so the kernels read the periodic image directly
// (index nx-1 for -1, 0 for nx) and never store a ghost.  Then
//   E(i,j) += c1 (Y(i,j) - Y(i-1,j)) - c2 (X(i,j) - X(i,j-1))   (or its CPML form)
//   X(i,j) -= c1x (E(i,j+1) - E(i,j))
//   Y(i,j) += c2y (E(i+1,j) - E(i,j))
//
// Adjoint.  The objective is J_b = dt * sum_{n=1..N} sum_{m in monitor} E_n(m)^2.
// Reverse-mode through one step applies, in reverse order, the transposes
// of: H sources, H update, E sources, E update.  Every update is
// F' = F + (linear in the two curl differences and the psi state), so its
// transpose keeps lambda_F, adds the "curl weight" lambda_D = dF'/dD *
// lambda_F' to the neighbours the differences read, and runs the psi
// recursion backwards:  L = phi + (dF'/dpsi') lambda_F',
// lambda_D = (dpsi'/dD) L + (dF'/dD)|direct lambda_F',  phi <- b L.
// The psi adjoints are double-buffered so a thread can evaluate its
// neighbours' curl weights from the previous buffer while the owner writes
// the next one: one kernel per half, gather form, no atomics.
// The design enters only through c1, c2 of the design pixels:
//   dJ/deps_p = sum_n lambda_E'(p) * dE'/deps_p = -1/eps_p sum_n lambda_E'(p) inc_p(n)
// with inc_p(n) = c1 D1 - c2 D2 of forward step n, recorded when the step
// is recomputed from a checkpoint.
//
// Resolved map.  Every lattice point's update is resolved once per design
// set (k_tmz_map): most points (dielectric, design pixels, CPML outside
// both profiles) update as F + c1 D1 + c2 D2 with two coefficients that
// the kernels read from a small per-point map shared by the batch (L2
// resident) instead of following class map -> class table -> profile
// look-ups every step; CPML points inside a profile go through the
// per-point functions below.
//
// Two kernel forms.  The one-step kernels advance every lattice point by
// one half-step per launch.  The temporally blocked kernels (FP32) advance
// a tile of one design by up to kTbHalo steps per launch from a region of
// shared memory (see k_tmz_tb_fwd).  Both use the same map and per-point
// functions, and this file is compiled without implicit multiply-add
// contraction (every fused operation is an explicit fmadd), so the two
// forms give bit-identical fields, adjoints and gradients.
#include "gmes_internal.cuh"

namespace gmes {
namespace {

constexpr int kBX = 32, kBY = 8;

// a + b * c: one rounding in FP32 and FP64, the float-float operators for
// the df type.
template <class R>
__device__ __forceinline__ R fmadd(R a, R b, R c) {
  return a + b * c;
}
template <>
__device__ __forceinline__ float fmadd<float>(float a, float b, float c) {
  return __fmaf_rn(b, c, a);
}
template <>
__device__ __forceinline__ double fmadd<double>(double a, double b, double c) {
  return __fma_rn(b, c, a);
}

struct Lat {
  int i, j, b;
  int64_t base, lin;
};

__device__ __forceinline__ bool lattice_point(const TmzDev& t, Lat& p) {
  p.j = blockIdx.x * kBX + threadIdx.x;
  p.i = blockIdx.y * kBY + threadIdx.y;
  p.b = blockIdx.z;
  if (p.i >= t.nx || p.j >= t.ny) return false;
  p.base = (int64_t)p.b * t.plane;
  p.lin = (int64_t)p.i * t.ny + p.j;
  return true;
}

__device__ __forceinline__ int64_t design_index(const TmzDev& t, int i, int j) {
  const int di = i - t.d0[0], dj = j - t.d0[1];
  if (di < 0 || di >= t.dn[0] || dj < 0 || dj >= t.dn[1]) return -1;
  return (int64_t)di * t.dn[1] + dj;
}

__device__ __forceinline__ int64_t monitor_index(const TmzDev& t, int i, int j) {
  const int di = i - t.m0[0], dj = j - t.m0[1];
  if (di < 0 || di >= t.mn[0] || dj < 0 || dj >= t.mn[1]) return -1;
  return (int64_t)di * t.mn[1] + dj;
}

// Class entries of the three lattice components (template grid maps).
__device__ __forceinline__ const ClassCoef& class_e(const GridDev& g, int i, int j) {
  return g.tab[2][__ldg(g.cls[2] + (int64_t)i * g.st[2][0] + (int64_t)j * g.st[2][1])];
}
__device__ __forceinline__ const ClassCoef& class_x(const GridDev& g, int i, int j) {
  return g.tab[3][__ldg(g.cls[3] + (int64_t)i * g.st[3][0] + (int64_t)(j + 1) * g.st[3][1] + 1)];
}
__device__ __forceinline__ const ClassCoef& class_y(const GridDev& g, int i, int j) {
  return g.tab[4][__ldg(g.cls[4] + (int64_t)(i + 1) * g.st[4][0] + (int64_t)j * g.st[4][1] + 1)];
}

// CPML profile rows of one lattice point: q1 along the component's first
// curl axis, q2 along its second (Ez: x, y; Hx: y, z; Hy: z, x).
struct Prof {
  const Coef* q1;
  const Coef* q2;
};
__device__ __forceinline__ Prof prof_e(const GridDev& g, int pm, int i, int j) {
  return {g.prof[pm][2][0] + (int64_t)i * kProfStride, g.prof[pm][2][1] + (int64_t)j * kProfStride};
}
__device__ __forceinline__ Prof prof_x(const GridDev& g, int pm, int i, int j) {
  (void)i;
  return {g.prof[pm][3][1] + (int64_t)(j + 1) * kProfStride, g.prof[pm][3][2] + kProfStride};
}
__device__ __forceinline__ Prof prof_y(const GridDev& g, int pm, int i, int j) {
  (void)j;
  return {g.prof[pm][4][2] + kProfStride, g.prof[pm][4][0] + (int64_t)(i + 1) * kProfStride};
}

// ---------------------------------------------------------------------------
// CPML points inside a profile.
// ---------------------------------------------------------------------------
// Their updates are those of the reference's CPML updaters
// (src/pw_cpml.hh:211-237, 319-397) with psi:
//   Ez: psi1' = b1 psi1 + c1 D1 (where profile 1 is on), likewise psi2;
//       Ez' = Ez + cdt ((psi1' - psi2') + k1 D1 - k2 D2)
//   Hx: psi' = b psi + c D1 (on);  Hx' = Hx - cdt (psi' + k D1)
//   Hy: psi' = b psi + c D2 (on);  Hy' = Hy - cdt (-psi' - k D2)
// with b, c, k the profile row (entries 0, 3, 4) at the point's index along
// the profile's axis.  The map (k_tmz_map) holds the class's cdt in the
// point's coefficient slot, the profile set in the flags' pml fields and
// which profiles are on, so no class look-up is needed here.
template <class P>
__device__ __forceinline__ typename P::R e_cpml(const GridDev& g, unsigned fl, typename P::R cdt,
                                                int i, int j, typename P::R e, typename P::R D1,
                                                typename P::R D2, typename P::T* s1,
                                                typename P::T* s2) {
  using R = typename P::R;
  const int pm = (fl >> kTmzPmlE) & 3;
  const Coef* q1 = g.prof[pm][2][0] + (int64_t)i * kProfStride;
  const Coef* q2 = g.prof[pm][2][1] + (int64_t)j * kProfStride;
  R psi1 = P::ldw(s1), psi2 = P::ldw(s2);
  if (fl & kTmzOnE1) {
    psi1 = fmadd(P::cfg(q1) * psi1, P::cfg(q1 + 3), D1);
    P::st(s1, psi1);
  }
  if (fl & kTmzOnE2) {
    psi2 = fmadd(P::cfg(q2) * psi2, P::cfg(q2 + 3), D2);
    P::st(s2, psi2);
  }
  const R xv = fmadd(fmadd(psi1 - psi2, P::cfg(q1 + 4), D1), -P::cfg(q2 + 4), D2);
  return fmadd(e, cdt, xv);
}

template <class P>
__device__ __forceinline__ typename P::R x_cpml(const GridDev& g, unsigned fl, typename P::R cdt,
                                                int j, typename P::R x, typename P::R dx,
                                                typename P::T* s) {
  using R = typename P::R;
  const Coef* q = g.prof[(fl >> kTmzPmlX) & 3][3][1] + (int64_t)(j + 1) * kProfStride;
  R psi = P::ldw(s);
  if (fl & kTmzOnX) {
    psi = fmadd(P::cfg(q) * psi, P::cfg(q + 3), dx);
    P::st(s, psi);
  }
  return fmadd(x, -cdt, fmadd(psi, P::cfg(q + 4), dx));
}

template <class P>
__device__ __forceinline__ typename P::R y_cpml(const GridDev& g, unsigned fl, typename P::R cdt,
                                                int i, typename P::R y, typename P::R dy,
                                                typename P::T* s) {
  using R = typename P::R;
  const Coef* q = g.prof[(fl >> kTmzPmlY) & 3][4][0] + (int64_t)(i + 1) * kProfStride;
  R psi = P::ldw(s);
  if (fl & kTmzOnY) {
    psi = fmadd(P::cfg(q) * psi, P::cfg(q + 3), dy);
    P::st(s, psi);
  }
  return fmadd(y, -cdt, fmadd(-psi, -P::cfg(q + 4), dy));
}

// Their transposes.  Curl weight of an Hx point: lambda_D1 = dX'/dD1
// applied to its adjoint lx; phr: its psi adjoint before this step, OWN:
// the advanced one is written to *phw.
template <class P, bool OWN>
__device__ __forceinline__ typename P::R adjx_cpml(const GridDev& g, unsigned fl,
                                                   typename P::R cdt, int j, typename P::R lx,
                                                   const typename P::T* phr,
                                                   typename P::T* phw) {
  using R = typename P::R;
  const Coef* q = g.prof[(fl >> kTmzPmlX) & 3][3][1] + (int64_t)(j + 1) * kProfStride;
  const R direct = -(cdt * (P::cfg(q + 4) * lx));
  if (!(fl & kTmzOnX)) return direct;
  const R L = fmadd(P::ldw(phr), -cdt, lx);
  if (OWN) P::st(phw, P::cfg(q) * L);
  return fmadd(direct, P::cfg(q + 3), L);
}

// Curl weight of an Hy point: lambda_D2, D2 = E(i+1, j) - E(i, j).
template <class P, bool OWN>
__device__ __forceinline__ typename P::R adjy_cpml(const GridDev& g, unsigned fl,
                                                   typename P::R cdt, int i, typename P::R ly,
                                                   const typename P::T* phr,
                                                   typename P::T* phw) {
  using R = typename P::R;
  const Coef* q = g.prof[(fl >> kTmzPmlY) & 3][4][0] + (int64_t)(i + 1) * kProfStride;
  const R direct = cdt * (P::cfg(q + 4) * ly);
  if (!(fl & kTmzOnY)) return direct;
  const R L = fmadd(P::ldw(phr), cdt, ly);
  if (OWN) P::st(phw, P::cfg(q) * L);
  return fmadd(direct, P::cfg(q + 3), L);
}

// Curl weights (lambda_D1, lambda_D2) of an Ez point from its adjoint le;
// NEED1/NEED2: which weights the caller uses (both when OWN).
template <class P, bool OWN, bool NEED1, bool NEED2>
__device__ __forceinline__ void adje_cpml(const GridDev& g, unsigned fl, typename P::R cdt, int i,
                                          int j, typename P::R le, const typename P::T* phr0,
                                          typename P::T* phw0, const typename P::T* phr1,
                                          typename P::T* phw1, typename P::R& w1,
                                          typename P::R& w2) {
  using R = typename P::R;
  const int pm = (fl >> kTmzPmlE) & 3;
  w1 = P::zero();
  w2 = P::zero();
  if (NEED1 || OWN) {
    const Coef* q1 = g.prof[pm][2][0] + (int64_t)i * kProfStride;
    const R direct = cdt * (P::cfg(q1 + 4) * le);
    if (fl & kTmzOnE1) {
      const R L = fmadd(P::ldw(phr0), cdt, le);
      if (OWN) P::st(phw0, P::cfg(q1) * L);
      w1 = fmadd(direct, P::cfg(q1 + 3), L);
    } else {
      w1 = direct;
    }
  }
  if (NEED2 || OWN) {
    const Coef* q2 = g.prof[pm][2][1] + (int64_t)j * kProfStride;
    const R direct = -(cdt * (P::cfg(q2 + 4) * le));
    if (fl & kTmzOnE2) {
      const R L = fmadd(P::ldw(phr1), -cdt, le);
      if (OWN) P::st(phw1, P::cfg(q2) * L);
      w2 = fmadd(direct, P::cfg(q2 + 3), L);
    } else {
      w2 = direct;
    }
  }
}

// Objective seed of lattice point (i, j) of design b at reverse step n:
// dJ/dE_n = 2 dt w_b E_n on monitor points (*has), nothing elsewhere.
__device__ __forceinline__ double seed_of(const GridDev& g, const TmzDev& t, int b, int i, int j,
                                          int n, bool* has) {
  const int64_t m = monitor_index(t, i, j);
  *has = m >= 0;
  if (m < 0) return 0.0;
  const int64_t nm = (int64_t)t.mn[0] * t.mn[1];
  const double w = t.weight != nullptr ? t.weight[b] : 1.0;
  const double e = t.mon[((int64_t)b * t.total_steps + (n - 1)) * nm + m];
  return 2.0 * g.dt * w * e;
}

// ---------------------------------------------------------------------------
// The resolved lattice map.
// ---------------------------------------------------------------------------
// Whether a CPML point's profile is on along either curl axis.
__device__ __forceinline__ bool profile_on(const Prof& q) {
  return coef_nonzero(q.q1 + 1) || coef_nonzero(q.q2 + 1);
}

template <class P>
__device__ __forceinline__ const typename P::T* map_coef(const TmzDev& t, int k) {
  return static_cast<const typename P::T*>(t.pcoef[k]);
}

// Flags and plain-form coefficients of every lattice point, built once per
// design set from the class maps, class table and CPML profiles.  The
// coefficients are c1, c2 of a Dielectric class, or of a CPML class outside
// both profiles (whose update reduces to the dielectric form).  Design
// pixels take theirs from the per-design table.  CPML points inside a
// profile keep their class's cdt in the coefficient slot, and the flags
// name the profile set and which of the point's profiles are on.
template <class P>
__global__ void k_tmz_map(const GridDev g, const TmzDev t) {
  using R = typename P::R;
  using T = typename P::T;
  const int64_t ll = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ll >= t.plane) return;
  const int i = (int)(ll / t.ny), j = (int)(ll - (int64_t)i * t.ny);
  unsigned f = 0;
  R c1 = P::zero(), c2n = P::zero(), cxn = P::zero(), cy = P::zero();
  if (design_index(t, i, j) >= 0) {
    f |= kTmzPlainE | kTmzDesign;
  } else {
    const ClassCoef& cc = class_e(g, i, j);
    const int kind = __ldg(&cc.kind);
    const int pm = __ldg(&cc.pml);
    if (kind == GMES_KIND_CPML && profile_on(prof_e(g, pm, i, j))) {
      const Prof q = prof_e(g, pm, i, j);
      f |= kTmzPsiE | ((unsigned)pm << kTmzPmlE);
      if (coef_nonzero(q.q1 + 1)) f |= kTmzOnE1;
      if (coef_nonzero(q.q2 + 1)) f |= kTmzOnE2;
      c1 = P::cfg(&cc.cdt);
    } else if (kind == GMES_KIND_DIELECTRIC || kind == GMES_KIND_CPML) {
      f |= kTmzPlainE;
      c1 = P::cfg(&cc.c1);
      c2n = -P::cfg(&cc.c2);
    }
  }
  {
    const ClassCoef& cc = class_x(g, i, j);
    const int kind = __ldg(&cc.kind);
    const int pm = __ldg(&cc.pml);
    if (kind == GMES_KIND_CPML && profile_on(prof_x(g, pm, i, j))) {
      f |= kTmzPsiX | ((unsigned)pm << kTmzPmlX);
      if (coef_nonzero(prof_x(g, pm, i, j).q1 + 1)) f |= kTmzOnX;
      cxn = P::cfg(&cc.cdt);
    } else if (kind == GMES_KIND_DIELECTRIC || kind == GMES_KIND_CPML) {
      f |= kTmzPlainX;
      cxn = -P::cfg(&cc.c1);
    }
  }
  {
    const ClassCoef& cc = class_y(g, i, j);
    const int kind = __ldg(&cc.kind);
    const int pm = __ldg(&cc.pml);
    if (kind == GMES_KIND_CPML && profile_on(prof_y(g, pm, i, j))) {
      f |= kTmzPsiY | ((unsigned)pm << kTmzPmlY);
      if (coef_nonzero(prof_y(g, pm, i, j).q2 + 1)) f |= kTmzOnY;
      cy = P::cfg(&cc.cdt);
    } else if (kind == GMES_KIND_DIELECTRIC || kind == GMES_KIND_CPML) {
      f |= kTmzPlainY;
      cy = P::cfg(&cc.c2);
    }
  }
  if (monitor_index(t, i, j) >= 0) f |= kTmzMonitor;
  const_cast<uint32_t*>(t.pflags)[ll] = f;
  P::st(const_cast<T*>(map_coef<P>(t, 0)) + ll, c1);
  P::st(const_cast<T*>(map_coef<P>(t, 1)) + ll, c2n);
  P::st(const_cast<T*>(map_coef<P>(t, 2)) + ll, cxn);
  P::st(const_cast<T*>(map_coef<P>(t, 3)) + ll, cy);
}

// Marks the points that carry a point source of either half (after
// k_tmz_map, which clears those bits).
__global__ void k_tmz_map_sources(const TmzDev t) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= t.nsrc) return;
  const gmes_point_source s = t.src[k];
  if (s.comp < 2 || s.comp > 4 || s.offset < 0 || s.offset >= t.plane) return;
  atomicOr(const_cast<uint32_t*>(t.pflags) + s.offset, s.comp == 2 ? kTmzSrcE : kTmzSrcH);
}

// Plain-form Ez coefficients (c1, -c2) of lattice point (i, j) = ll of
// design b.
template <class P>
__device__ __forceinline__ void e_coef(const TmzDev& t, int b, int i, int j, int64_t ll,
                                       unsigned fl, typename P::R& c1, typename P::R& c2n) {
  c1 = P::ld(map_coef<P>(t, 0) + ll);
  c2n = P::ld(map_coef<P>(t, 1) + ll);
  if (fl & kTmzDesign) {
    const DesignCoef* dc = t.dc + (int64_t)b * t.dn[0] * t.dn[1] + design_index(t, i, j);
    c1 = P::cfg(&dc->c1);
    c2n = -P::cfg(&dc->c2);
  }
}

// Adjoint curl weights through the map: the plain form, the CPML form on
// points inside a profile, zero on points that are not updated.  ll:
// lattice offset; base: the design's offset.
template <class P, bool OWN>
__device__ __forceinline__ typename P::R weight_x(const GridDev& g, const TmzDev& t, int i, int j,
                                                  int64_t ll, int64_t base, int rb, int wb) {
  using T = typename P::T;
  const T* lx = static_cast<const T*>(t.l[1]) + base + ll;
  const typename P::R c = P::ld(map_coef<P>(t, 2) + ll);  // issued with the flags
  const unsigned fl = __ldg(t.pflags + ll);
  if (fl & kTmzPlainX) return c * P::ldw(lx);
  if (!(fl & kTmzPsiX)) return P::zero();
  return adjx_cpml<P, OWN>(g, fl, c, j, P::ldw(lx),
                           static_cast<const T*>(t.phi[rb][2]) + base + ll,
                           OWN ? static_cast<T*>(t.phi[wb][2]) + base + ll : nullptr);
}

template <class P, bool OWN>
__device__ __forceinline__ typename P::R weight_y(const GridDev& g, const TmzDev& t, int i, int j,
                                                  int64_t ll, int64_t base, int rb, int wb) {
  using T = typename P::T;
  const T* ly = static_cast<const T*>(t.l[2]) + base + ll;
  const typename P::R c = P::ld(map_coef<P>(t, 3) + ll);  // issued with the flags
  const unsigned fl = __ldg(t.pflags + ll);
  if (fl & kTmzPlainY) return c * P::ldw(ly);
  if (!(fl & kTmzPsiY)) return P::zero();
  return adjy_cpml<P, OWN>(g, fl, c, i, P::ldw(ly),
                           static_cast<const T*>(t.phi[rb][3]) + base + ll,
                           OWN ? static_cast<T*>(t.phi[wb][3]) + base + ll : nullptr);
}

template <class P, bool OWN, bool NEED1, bool NEED2>
__device__ __forceinline__ void weight_e(const GridDev& g, const TmzDev& t, int b, int i, int j,
                                         int64_t ll, int64_t base, int rb, int wb,
                                         typename P::R& w1, typename P::R& w2) {
  using R = typename P::R;
  using T = typename P::T;
  const T* le = static_cast<const T*>(t.l[0]) + base + ll;
  const unsigned fl = __ldg(t.pflags + ll);
  R c1, c2n;
  e_coef<P>(t, b, i, j, ll, fl, c1, c2n);
  if (fl & kTmzPlainE) {
    const R v = P::ldw(le);
    w1 = c1 * v;
    w2 = c2n * v;
    return;
  }
  if (!(fl & kTmzPsiE)) {
    w1 = w2 = P::zero();
    return;
  }
  adje_cpml<P, OWN, NEED1, NEED2>(g, fl, c1, i, j, P::ldw(le),
                                  static_cast<const T*>(t.phi[rb][0]) + base + ll,
                                  OWN ? static_cast<T*>(t.phi[wb][0]) + base + ll : nullptr,
                                  static_cast<const T*>(t.phi[rb][1]) + base + ll,
                                  OWN ? static_cast<T*>(t.phi[wb][1]) + base + ll : nullptr, w1,
                                  w2);
}

// ---------------------------------------------------------------------------
// One-step forward kernels.
// ---------------------------------------------------------------------------
template <class P>
__global__ void __launch_bounds__(kBX* kBY) k_tmz_fe(const GridDev g, const TmzDev t, int slot) {
  using R = typename P::R;
  using T = typename P::T;
  Lat p;
  if (!lattice_point(t, p)) return;
  const int im = p.i == 0 ? t.nx - 1 : p.i - 1, jm = p.j == 0 ? t.ny - 1 : p.j - 1;
  T* E = static_cast<T*>(t.f[0]) + p.base;
  const T* X = static_cast<const T*>(t.f[1]) + p.base;
  const T* Y = static_cast<const T*>(t.f[2]) + p.base;
  const unsigned fl = __ldg(t.pflags + p.lin);
  const R D1 = P::ld(Y + p.lin) - P::ld(Y + (int64_t)im * t.ny + p.j);
  const R D2 = P::ld(X + p.lin) - P::ld(X + (int64_t)p.i * t.ny + jm);
  const R e = P::ldw(E + p.lin);
  if (fl & kTmzPlainE) {
    R c1, c2n;
    e_coef<P>(t, p.b, p.i, p.j, p.lin, fl, c1, c2n);
    P::st(E + p.lin, fmadd(fmadd(e, c1, D1), c2n, D2));
    if ((fl & kTmzDesign) && slot >= 0) {
      const int64_t nd = (int64_t)t.dn[0] * t.dn[1];
      P::st(static_cast<T*>(t.hist) + ((int64_t)slot * t.nb + p.b) * nd +
                design_index(t, p.i, p.j),
            fmadd(c2n * D2, c1, D1));
    }
  } else if (fl & kTmzPsiE) {
    P::st(E + p.lin, e_cpml<P>(g, fl, P::ld(map_coef<P>(t, 0) + p.lin), p.i, p.j, e, D1, D2,
                               static_cast<T*>(t.f[3]) + p.base + p.lin,
                               static_cast<T*>(t.f[4]) + p.base + p.lin));
  }
}

template <class P>
__global__ void __launch_bounds__(kBX* kBY) k_tmz_fh(const GridDev g, const TmzDev t, int row) {
  using R = typename P::R;
  using T = typename P::T;
  Lat p;
  if (!lattice_point(t, p)) return;
  const int ip = p.i + 1 == t.nx ? 0 : p.i + 1, jp = p.j + 1 == t.ny ? 0 : p.j + 1;
  const T* E = static_cast<const T*>(t.f[0]) + p.base;
  T* X = static_cast<T*>(t.f[1]) + p.base;
  T* Y = static_cast<T*>(t.f[2]) + p.base;
  const unsigned fl = __ldg(t.pflags + p.lin);
  const R cxn = P::ld(map_coef<P>(t, 2) + p.lin), cy = P::ld(map_coef<P>(t, 3) + p.lin);
  const R e0 = P::ld(E + p.lin);
  const R dx = P::ld(E + (int64_t)p.i * t.ny + jp) - e0;  // D1 of Hx
  const R dy = P::ld(E + (int64_t)ip * t.ny + p.j) - e0;  // D2 of Hy
  if (fl & kTmzPlainX)
    P::st(X + p.lin, fmadd(P::ldw(X + p.lin), cxn, dx));
  else if (fl & kTmzPsiX)
    P::st(X + p.lin, x_cpml<P>(g, fl, cxn, p.j, P::ldw(X + p.lin), dx,
                               static_cast<T*>(t.f[5]) + p.base + p.lin));
  if (fl & kTmzPlainY)
    P::st(Y + p.lin, fmadd(P::ldw(Y + p.lin), cy, dy));
  else if (fl & kTmzPsiY)
    P::st(Y + p.lin, y_cpml<P>(g, fl, cy, p.i, P::ldw(Y + p.lin), dy,
                               static_cast<T*>(t.f[6]) + p.base + p.lin));
  if (row >= 0 && (fl & kTmzMonitor)) {
    const int64_t nm = (int64_t)t.mn[0] * t.mn[1];
    t.mon[((int64_t)p.b * t.total_steps + row) * nm + monitor_index(t, p.i, p.j)] = to_double(e0);
  }
}

// Point sources of one half (gmes/pw_source.py:74-131) for every design:
// comp 2/3/4 = E/X/Y lattice array, offset = i * ny + j.  Entries that do
// not name a lattice point of that half are skipped.
template <class P>
__global__ void k_tmz_src(const TmzDev t, int side, int n) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)t.nsrc * t.nb) return;
  const int b = (int)(q / t.nsrc), k = (int)(q - (int64_t)b * t.nsrc);
  const gmes_point_source s = t.src[k];
  if (s.comp < 2 || s.comp > 4 || (s.comp == 2) != (side == 0)) return;
  if (s.offset < 0 || s.offset >= t.plane) return;
  const double v = t.src_val[((int64_t)(n - 1) * 2 + side) * t.nsrc + k];
  using T = typename P::T;
  T* f = static_cast<T*>(t.f[s.comp - 2]) + (int64_t)b * t.plane + s.offset;
  if (s.mode == 0)
    P::st(f, P::from_double(v));
  else
    P::st(f, P::ldw(f) - P::from_double(v));
}

// ---------------------------------------------------------------------------
// One-step adjoint kernels.
// ---------------------------------------------------------------------------
// Transpose of the H half of step n, plus the objective's seed for the
// state after step n: lambda_E gathers the curl weights of its four H
// neighbours; the owner advances the Hx/Hy psi adjoints.
template <class P>
__global__ void __launch_bounds__(kBX* kBY)
    k_tmz_ah(const GridDev g, const TmzDev t, int n, int rb, int wb) {
  using R = typename P::R;
  using T = typename P::T;
  Lat p;
  if (!lattice_point(t, p)) return;
  const int im = p.i == 0 ? t.nx - 1 : p.i - 1, jm = p.j == 0 ? t.ny - 1 : p.j - 1;
  T* LE = static_cast<T*>(t.l[0]) + p.base + p.lin;
  R le = P::ldw(LE);
  if (__ldg(t.pflags + p.lin) & kTmzMonitor) {
    bool has;
    le = le + P::from_double(seed_of(g, t, p.b, p.i, p.j, n, &has));
  }
  const int64_t ljm = (int64_t)p.i * t.ny + jm, lim = (int64_t)im * t.ny + p.j;
  const R a = weight_x<P, false>(g, t, p.i, jm, ljm, p.base, rb, wb);
  const R bx = weight_x<P, true>(g, t, p.i, p.j, p.lin, p.base, rb, wb);
  const R c = weight_y<P, false>(g, t, im, p.j, lim, p.base, rb, wb);
  const R d = weight_y<P, true>(g, t, p.i, p.j, p.lin, p.base, rb, wb);
  P::st(LE, le + ((a - bx) + (c - d)));
}

// Transpose of the E half of step n: lambda_X, lambda_Y gather the curl
// weights of their two Ez neighbours; the owner advances the Ez psi
// adjoints and, in the design region, accumulates the gradient.
template <class P>
__global__ void __launch_bounds__(kBX* kBY)
    k_tmz_ae(const GridDev g, const TmzDev t, int slot, int rb, int wb) {
  using R = typename P::R;
  using T = typename P::T;
  Lat p;
  if (!lattice_point(t, p)) return;
  const int ip = p.i + 1 == t.nx ? 0 : p.i + 1, jp = p.j + 1 == t.ny ? 0 : p.j + 1;
  const int64_t ljp = (int64_t)p.i * t.ny + jp, lip = (int64_t)ip * t.ny + p.j;
  R w1, w2, u1, u2, v1, v2;
  weight_e<P, true, true, true>(g, t, p.b, p.i, p.j, p.lin, p.base, rb, wb, w1, w2);
  weight_e<P, false, false, true>(g, t, p.b, p.i, jp, ljp, p.base, rb, wb, u1, u2);
  weight_e<P, false, true, false>(g, t, p.b, ip, p.j, lip, p.base, rb, wb, v1, v2);
  T* LX = static_cast<T*>(t.l[1]) + p.base + p.lin;
  T* LY = static_cast<T*>(t.l[2]) + p.base + p.lin;
  P::st(LX, P::ldw(LX) + (w2 - u2));
  P::st(LY, P::ldw(LY) + (w1 - v1));
  if (__ldg(t.pflags + p.lin) & kTmzDesign) {
    const int64_t nd = (int64_t)t.dn[0] * t.dn[1];
    const int64_t dp = design_index(t, p.i, p.j);
    const int64_t k = (int64_t)p.b * nd + dp;
    const double le = to_double(P::ldw(static_cast<const T*>(t.l[0]) + p.base + p.lin));
    const double inc =
        to_double(P::ldw(static_cast<const T*>(t.hist) + ((int64_t)slot * t.nb + p.b) * nd + dp));
    t.grad[k] += le * inc * t.dc[k].neg_reps;
  }
}

// Transpose of a half's hard sources: the value written does not depend
// on the field before it, so its adjoint is zeroed.  Current sources add a
// constant and leave the adjoint unchanged.
template <class P>
__global__ void k_tmz_adj_src(const TmzDev t, int side) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)t.nsrc * t.nb) return;
  const int b = (int)(q / t.nsrc), k = (int)(q - (int64_t)b * t.nsrc);
  const gmes_point_source s = t.src[k];
  if (s.mode != 0 || s.comp < 2 || s.comp > 4 || (s.comp == 2) != (side == 0)) return;
  if (s.offset < 0 || s.offset >= t.plane) return;
  P::st(static_cast<typename P::T*>(t.l[s.comp - 2]) + (int64_t)b * t.plane + s.offset,
        P::zero());
}

// ---------------------------------------------------------------------------
// Temporally blocked kernels (FP32).
// ---------------------------------------------------------------------------
// A block owns a TI x TJ tile of one design's lattice and keeps the region
// of RI x RJ = (TI + 2 H) x (TJ + 2 H) points around it in shared memory
// (region point (a, c) is lattice point (ri0 + a, rj0 + c) taken periodically,
// so tiles at the lattice edge see its periodic images).  An E update reads
// its low-side neighbours (i-1, j-1) and an H update its high-side ones
// (i+1, j+1); updating every region point that has its neighbours in the
// region, each half-step leaves the values exact on the region shrunk by
// one more row and column on one side.  After s <= H steps the values are
// exact on [s, RI-1-s] (H fields) and [s, RI-s] (E), which contain the tile,
// so the tile is written back and the next launch reloads fresh halos.
// DRAM traffic per step falls from a read and write of every field per
// half-step to one read of the region and one write of the tile per H
// steps.  Sources, monitors, design increments and gradients are applied
// as in the one-step kernels: sources to every copy of their point in the
// region, records and gradients only from tile points.
//
// Each launch reads every region point's flags and plain-form
// coefficients from the resolved map once and keeps them in registers, so
// a sub-step of a plain point is a few shared-memory operations; CPML
// points inside a profile go through the per-point functions above.
//
// Threads: RJ = 64 columns x 8 rows; a thread owns column c of rows
// ty, ty + 8, ...; psi (and psi adjoint) values are loaded and stored only
// on CPML points inside a profile.
constexpr int kTbHalo = GMES_TMZ_MAX_BLOCK_STEPS;  // most steps per launch
constexpr int kTbRJ = 64;    // region columns (j)
constexpr int kTbRows = 8;   // thread rows
constexpr int kTbThreads = kTbRJ * kTbRows;

template <bool B>
struct PsiTag {
  static constexpr bool value = B;
};
constexpr int kTbRI = 32;    // region rows (i)
#ifndef GMES_TB_MIN_BLOCKS
#define GMES_TB_MIN_BLOCKS 2
#endif
constexpr int kTbMinBlocks = GMES_TB_MIN_BLOCKS;  // resident blocks per SM (register budget)

__device__ __forceinline__ int wrap_index(int v, int n) {
  if (v < 0) v += n;
  if (v >= n) v -= n;
  if (v >= 0 && v < n) return v;
  v %= n;  // regions wider than twice the lattice
  return v < 0 ? v + n : v;
}

template <int RI>
struct TbGeom {
  static constexpr int H = kTbHalo, RJ = kTbRJ, TI = RI - 2 * kTbHalo, TJ = kTbRJ - 2 * kTbHalo;
  static constexpr int NP = RI * kTbRJ, Q = RI / kTbRows;
  static_assert(RI % kTbRows == 0 && TI > 0, "region rows");
};

// Plain-form coefficients of one region point.
struct TbPoint {
  float c1, c2n;  // Ez: c1, -c2
  float cxn, cy;  // Hx: -c1, Hy: c2
};

// Flags and plain-form coefficients of lattice point (i, j) of design b,
// from the resolved map.
__device__ __forceinline__ unsigned tb_point(const TmzDev& t, int b, int i, int j, TbPoint& p) {
  using P = PolF32;
  const int64_t ll = (int64_t)i * t.ny + j;
  const unsigned f = __ldg(t.pflags + ll);
  e_coef<P>(t, b, i, j, ll, f, p.c1, p.c2n);
  p.cxn = __ldg(map_coef<P>(t, 2) + ll);
  p.cy = __ldg(map_coef<P>(t, 3) + ll);
  return f;
}

// Apply this half's sources of step n to every copy of their point in the
// region: the forward (ADJ false: hard sources set the value, current
// sources subtract theirs) or the adjoint (ADJ true: hard sources zero it).
template <bool ADJ>
__device__ __forceinline__ void tb_sources(const TmzDev& t, int side, int n, int ri0, int rj0,
                                           int RI, int RJ, float* fE, float* fX, float* fY) {
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  for (int k = tid; k < t.nsrc; k += kTbThreads) {
    const gmes_point_source s = t.src[k];
    if (s.comp < 2 || s.comp > 4 || (s.comp == 2) != (side == 0)) continue;
    if (s.offset < 0 || s.offset >= t.plane) continue;
    if (ADJ && s.mode != 0) continue;
    const int li = (int)(s.offset / t.ny), lj = (int)(s.offset - (int64_t)li * t.ny);
    float* f = s.comp == 2 ? fE : (s.comp == 3 ? fX : fY);
    const float v =
        ADJ ? 0.f
            : PolF32::from_double(t.src_val[((int64_t)(n - 1) * 2 + side) * t.nsrc + k]);
    for (int a = wrap_index(li - ri0, t.nx); a < RI; a += t.nx)
      for (int c = wrap_index(lj - rj0, t.ny); c < RJ; c += t.ny) {
        float* q = f + a * RJ + c;
        *q = (ADJ || s.mode == 0) ? v : *q - v;
      }
  }
}

// Forward steps n0+1 .. n0+nsub (nsub <= kTbHalo) of one tile, from the
// state in t.f to the state in t.tmp (the launch's other blocks still read
// t.f for their halos, so the result must not overwrite it).  slot0 >= 0:
// record the design increments of step n0+1+s at hist slot slot0+s;
// rec_mon: record monitor row n-1 of every step n.
template <int RI>
__global__ void __launch_bounds__(kTbThreads, kTbMinBlocks)
    k_tmz_tb_fwd(const GridDev g, const TmzDev t, int n0, int nsub, int slot0, int rec_mon) {
  using P = PolF32;
  using G = TbGeom<RI>;
  constexpr int H = G::H, RJ = G::RJ, TI = G::TI, TJ = G::TJ, NP = G::NP, Q = G::Q;
  extern __shared__ float4 tb_smem[];
  float* sE = reinterpret_cast<float*>(tb_smem);
  float* sX = sE + NP;
  float* sY = sX + NP;
  float* sS = sY + NP;  // psi of Ez (x, y), Hx, Hy: sS + k * NP
  const int c = threadIdx.x, ty = threadIdx.y, b = blockIdx.z;
  const int ri0 = (int)blockIdx.y * TI - H, rj0 = (int)blockIdx.x * TJ - H;
  const int j = wrap_index(rj0 + c, t.ny);
  const bool jtile = c >= H && c < H + TJ && rj0 + c < t.ny;
  const int64_t base = (int64_t)b * t.plane;
  int li[Q];
  TbPoint pt[Q];
  unsigned fl[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int a = ty + kTbRows * q, k = a * RJ + c;
    li[q] = wrap_index(ri0 + a, t.nx);
    fl[q] = tb_point(t, b, li[q], j, pt[q]);
    if (jtile && a >= H && a < H + TI && ri0 + a < t.nx) fl[q] |= 1u << 31;  // tile point
    const int64_t lin = base + (int64_t)li[q] * t.ny + j;
    sE[k] = __ldg(static_cast<const float*>(t.f[0]) + lin);
    sX[k] = __ldg(static_cast<const float*>(t.f[1]) + lin);
    sY[k] = __ldg(static_cast<const float*>(t.f[2]) + lin);
    if (fl[q] & kTmzPsiE) {
      sS[k] = __ldg(static_cast<const float*>(t.f[3]) + lin);
      sS[NP + k] = __ldg(static_cast<const float*>(t.f[4]) + lin);
    }
    if (fl[q] & kTmzPsiX) sS[2 * NP + k] = __ldg(static_cast<const float*>(t.f[5]) + lin);
    if (fl[q] & kTmzPsiY) sS[3 * NP + k] = __ldg(static_cast<const float*>(t.f[6]) + lin);
  }
  unsigned any = 0;
#pragma unroll
  for (int q = 0; q < Q; ++q) any |= fl[q];
  const bool src_e = __syncthreads_or(any & kTmzSrcE) != 0;  // also orders the loads
  const bool src_h = __syncthreads_or(any & kTmzSrcH) != 0;
  const int64_t nd = (int64_t)t.dn[0] * t.dn[1];
  const int64_t nm = (int64_t)t.mn[0] * t.mn[1];
  // Regions without CPML points inside a profile (most tiles) run a copy of
  // the sub-step loop without that code path: the choice is block-uniform,
  // and the arithmetic of every point is the same in both copies.
  const bool psi_any = __syncthreads_or(any & (kTmzPsiE | kTmzPsiX | kTmzPsiY)) != 0;
  auto steps = [&](auto tag) {
    constexpr bool PSI = decltype(tag)::value;
    for (int s = 0; s < nsub; ++s) {
      const int n = n0 + s + 1;
  #pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int a = ty + kTbRows * q, k = a * RJ + c;
        if (a >= 1 && c >= 1) {
          const float D1 = sY[k] - sY[k - RJ], D2 = sX[k] - sX[k - 1];
          if (fl[q] & kTmzPlainE) {
            sE[k] = fmadd(fmadd(sE[k], pt[q].c1, D1), pt[q].c2n, D2);
            if ((fl[q] & kTmzDesign) && (fl[q] >> 31) && slot0 >= 0)
              static_cast<float*>(t.hist)[((int64_t)(slot0 + s) * t.nb + b) * nd +
                                          design_index(t, li[q], j)] =
                  fmadd(pt[q].c2n * D2, pt[q].c1, D1);
          } else if (PSI && (fl[q] & kTmzPsiE)) {
            sE[k] = e_cpml<P>(g, fl[q], pt[q].c1, li[q], j, sE[k], D1, D2, sS + k, sS + NP + k);
          }
        }
      }
      __syncthreads();
      if (src_e) {
        tb_sources<false>(t, 0, n, ri0, rj0, RI, RJ, sE, sX, sY);
        __syncthreads();
      }
  #pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int a = ty + kTbRows * q, k = a * RJ + c;
        if (a < RI - 1 && c < RJ - 1) {
          const float e0 = sE[k];
          const float dx = sE[k + 1] - e0, dy = sE[k + RJ] - e0;
          if (fl[q] & kTmzPlainX)
            sX[k] = fmadd(sX[k], pt[q].cxn, dx);
          else if (PSI && (fl[q] & kTmzPsiX))
            sX[k] = x_cpml<P>(g, fl[q], pt[q].cxn, j, sX[k], dx, sS + 2 * NP + k);
          if (fl[q] & kTmzPlainY)
            sY[k] = fmadd(sY[k], pt[q].cy, dy);
          else if (PSI && (fl[q] & kTmzPsiY))
            sY[k] = y_cpml<P>(g, fl[q], pt[q].cy, li[q], sY[k], dy, sS + 3 * NP + k);
          if (rec_mon && (fl[q] & kTmzMonitor) && (fl[q] >> 31))
            t.mon[((int64_t)b * t.total_steps + (n - 1)) * nm + monitor_index(t, li[q], j)] =
                (double)e0;
        }
      }
      __syncthreads();
      if (src_h) {
        tb_sources<false>(t, 1, n, ri0, rj0, RI, RJ, sE, sX, sY);
        __syncthreads();
      }
    }
  };
  if (psi_any)
    steps(PsiTag<true>{});
  else
    steps(PsiTag<false>{});
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    if (!(fl[q] >> 31)) continue;
    const int k = (ty + kTbRows * q) * RJ + c;
    const int64_t lin = base + (int64_t)li[q] * t.ny + j;
    static_cast<float*>(t.tmp[0])[lin] = sE[k];
    static_cast<float*>(t.tmp[1])[lin] = sX[k];
    static_cast<float*>(t.tmp[2])[lin] = sY[k];
    if (fl[q] & kTmzPsiE) {
      static_cast<float*>(t.tmp[3])[lin] = sS[k];
      static_cast<float*>(t.tmp[4])[lin] = sS[NP + k];
    }
    if (fl[q] & kTmzPsiX) static_cast<float*>(t.tmp[5])[lin] = sS[2 * NP + k];
    if (fl[q] & kTmzPsiY) static_cast<float*>(t.tmp[6])[lin] = sS[3 * NP + k];
  }
}

// Adjoint steps n0 + nsub down to n0 + 1 of one tile (the transposes of
// k_tmz_ah / k_tmz_ae, same order), the field adjoints from t.l to
// t.tmp[0..2]; the gradient of step n uses hist slot n - step0 - 1.  The
// psi adjoints are read from buffer rb and written to the other one, so no
// block overwrites what another still reads (adjoint_blocked chooses rb so
// that a call leaves them where the one-step kernels' step-parity
// convention expects them).
template <int RI>
__global__ void __launch_bounds__(kTbThreads, kTbMinBlocks)
    k_tmz_tb_adj(const GridDev g, const TmzDev t, int n0, int nsub, int step0, int rb) {
  using P = PolF32;
  using G = TbGeom<RI>;
  constexpr int H = G::H, RJ = G::RJ, TI = G::TI, TJ = G::TJ, NP = G::NP, Q = G::Q;
  extern __shared__ float4 tb_smem[];
  float* sLE = reinterpret_cast<float*>(tb_smem);
  float* sLX = sLE + NP;
  float* sLY = sLX + NP;
  float* sP = sLY + NP;      // psi adjoints of Ez (x, y), Hx, Hy: sP + k * NP
  float* sW1 = sP + 4 * NP;  // curl weights of the H half: Hx
  float* sW2 = sW1 + NP;     //   and Hy
  float* sV1 = sW2 + NP;     // curl weights of the E half: Ez's first
  float* sV2 = sV1 + NP;     //   and its second
  const int c = threadIdx.x, ty = threadIdx.y, b = blockIdx.z;
  const int ri0 = (int)blockIdx.y * TI - H, rj0 = (int)blockIdx.x * TJ - H;
  const int j = wrap_index(rj0 + c, t.ny);
  const bool jtile = c >= H && c < H + TJ && rj0 + c < t.ny;
  const int64_t base = (int64_t)b * t.plane;
  const int wb = rb ^ 1;
  int li[Q];
  TbPoint pt[Q];
  unsigned fl[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int a = ty + kTbRows * q, k = a * RJ + c;
    li[q] = wrap_index(ri0 + a, t.nx);
    fl[q] = tb_point(t, b, li[q], j, pt[q]);
    if (jtile && a >= H && a < H + TI && ri0 + a < t.nx) fl[q] |= 1u << 31;  // tile point
    const int64_t lin = base + (int64_t)li[q] * t.ny + j;
    sLE[k] = static_cast<const float*>(t.l[0])[lin];
    sLX[k] = static_cast<const float*>(t.l[1])[lin];
    sLY[k] = static_cast<const float*>(t.l[2])[lin];
    if (fl[q] & kTmzPsiE) {
      sP[k] = static_cast<const float*>(t.phi[rb][0])[lin];
      sP[NP + k] = static_cast<const float*>(t.phi[rb][1])[lin];
    }
    if (fl[q] & kTmzPsiX) sP[2 * NP + k] = static_cast<const float*>(t.phi[rb][2])[lin];
    if (fl[q] & kTmzPsiY) sP[3 * NP + k] = static_cast<const float*>(t.phi[rb][3])[lin];
  }
  unsigned any = 0;
#pragma unroll
  for (int q = 0; q < Q; ++q) any |= fl[q];
  const bool src_e = __syncthreads_or(any & kTmzSrcE) != 0;  // also orders the loads
  const bool src_h = __syncthreads_or(any & kTmzSrcH) != 0;
  const int64_t nd = (int64_t)t.dn[0] * t.dn[1];
  // as in k_tmz_tb_fwd: a copy of the loop without the CPML path for
  // regions that have no CPML point inside a profile
  const bool psi_any = __syncthreads_or(any & (kTmzPsiE | kTmzPsiX | kTmzPsiY)) != 0;
  // Per step (n = n0 + s + 1, s from nsub - 1 down to 0), the transposes of
  // the one-step kernels in their order: H-side sources, the curl weights
  // of every Hx / Hy point (hw), lambda_E gathering them (eu), E-side
  // sources, the curl weights of every Ez point and the gradient (ew),
  // lambda_X / lambda_Y gathering those (xu).  A point's weights depend
  // only on its own adjoints, so ew runs in the same pass as eu and the
  // next step's hw in the same pass as xu (into other arrays than the
  // neighbours read): two barriers per step.  A block holding a source
  // point applies it between the two, with barriers around it.
  auto steps = [&](auto tag) {
    constexpr bool PSI = decltype(tag)::value;
    auto hw = [&](int q) {
      const int k = (ty + kTbRows * q) * RJ + c;
      sW1[k] = (fl[q] & kTmzPlainX) ? pt[q].cxn * sLX[k]
               : (PSI && (fl[q] & kTmzPsiX))
                   ? adjx_cpml<P, true>(g, fl[q], pt[q].cxn, j, sLX[k], sP + 2 * NP + k,
                                        sP + 2 * NP + k)
                   : 0.f;
      sW2[k] = (fl[q] & kTmzPlainY) ? pt[q].cy * sLY[k]
               : (PSI && (fl[q] & kTmzPsiY))
                   ? adjy_cpml<P, true>(g, fl[q], pt[q].cy, li[q], sLY[k], sP + 3 * NP + k,
                                        sP + 3 * NP + k)
                   : 0.f;
    };
    auto eu = [&](int q, int n) {
      const int a = ty + kTbRows * q, k = a * RJ + c;
      if (a >= 1 && c >= 1) {
        float le = sLE[k];
        if (fl[q] & kTmzMonitor) {
          bool has;
          le = le + P::from_double(seed_of(g, t, b, li[q], j, n, &has));
        }
        sLE[k] = le + ((sW1[k - 1] - sW1[k]) + (sW2[k - RJ] - sW2[k]));
      }
    };
    auto ew = [&](int q, int n) {
      const int k = (ty + kTbRows * q) * RJ + c;
      float w1, w2;
      if (fl[q] & kTmzPlainE) {
        const float le = sLE[k];
        w1 = pt[q].c1 * le;
        w2 = pt[q].c2n * le;
      } else {
        w1 = w2 = 0.f;
        if (PSI && (fl[q] & kTmzPsiE))
          adje_cpml<P, true, true, true>(g, fl[q], pt[q].c1, li[q], j, sLE[k], sP + k, sP + k,
                                         sP + NP + k, sP + NP + k, w1, w2);
      }
      sV1[k] = w1;
      sV2[k] = w2;
      if ((fl[q] & kTmzDesign) && (fl[q] >> 31)) {
        const int64_t kk = (int64_t)b * nd + design_index(t, li[q], j);
        const double le = (double)sLE[k];
        const double inc = (double)static_cast<const float*>(
            t.hist)[((int64_t)(n - step0 - 1) * t.nb + b) * nd + (kk - (int64_t)b * nd)];
        t.grad[kk] += le * inc * t.dc[kk].neg_reps;
      }
    };
    auto xu = [&](int q) {
      const int a = ty + kTbRows * q, k = a * RJ + c;
      if (a < RI - 1 && c < RJ - 1) {
        sLX[k] = sLX[k] + (sV2[k] - sV2[k + 1]);
        sLY[k] = sLY[k] + (sV1[k] - sV1[k + RJ]);
      }
    };
    if (src_h) {
      tb_sources<true>(t, 1, n0 + nsub, ri0, rj0, RI, RJ, sLE, sLX, sLY);
      __syncthreads();
    }
  #pragma unroll
    for (int q = 0; q < Q; ++q) hw(q);
    __syncthreads();
    for (int s = nsub - 1; s >= 0; --s) {
      const int n = n0 + s + 1;
  #pragma unroll
      for (int q = 0; q < Q; ++q) eu(q, n);
      if (src_e) {
        __syncthreads();
        tb_sources<true>(t, 0, n, ri0, rj0, RI, RJ, sLE, sLX, sLY);
        __syncthreads();
      }
  #pragma unroll
      for (int q = 0; q < Q; ++q) ew(q, n);
      __syncthreads();
  #pragma unroll
      for (int q = 0; q < Q; ++q) xu(q);
      if (s > 0) {
        if (src_h) {
          __syncthreads();
          tb_sources<true>(t, 1, n - 1, ri0, rj0, RI, RJ, sLE, sLX, sLY);
          __syncthreads();
        }
  #pragma unroll
        for (int q = 0; q < Q; ++q) hw(q);
      }
      __syncthreads();
    }
  };
  if (psi_any)
    steps(PsiTag<true>{});
  else
    steps(PsiTag<false>{});
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    if (!(fl[q] >> 31)) continue;
    const int k = (ty + kTbRows * q) * RJ + c;
    const int64_t lin = base + (int64_t)li[q] * t.ny + j;
    static_cast<float*>(t.tmp[0])[lin] = sLE[k];
    static_cast<float*>(t.tmp[1])[lin] = sLX[k];
    static_cast<float*>(t.tmp[2])[lin] = sLY[k];
    if (fl[q] & kTmzPsiE) {
      static_cast<float*>(t.phi[wb][0])[lin] = sP[k];
      static_cast<float*>(t.phi[wb][1])[lin] = sP[NP + k];
    }
    if (fl[q] & kTmzPsiX) static_cast<float*>(t.phi[wb][2])[lin] = sP[2 * NP + k];
    if (fl[q] & kTmzPsiY) static_cast<float*>(t.phi[wb][3])[lin] = sP[3 * NP + k];
  }
}

// Region of both blocked kernels: 32 x 64 points; forward 7 arrays (56 KB),
// adjoint 11 arrays (88 KB) of shared memory.  (Adjoint measured on GB300,
// 512^2 x 64 designs, 2000 steps: 9 arrays and four barriers per step
// 0.3168 s, 11 arrays and two barriers 0.3147 s, and with each design
// pixel's gradient summed in shared memory over a launch, 104 KB, 0.3266 s;
// a thread's own curl weights kept in registers from the pass that forms
// them to the pass that gathers them, four fewer shared-memory loads per
// point and step but spilling at 64 registers: 0.352 s, the E half's alone
// 0.328 s, against 0.316 s.)
constexpr int kTbFwdRI = kTbRI, kTbAdjRI = kTbRI;
constexpr size_t kTbFwdSmem = (size_t)7 * kTbFwdRI * kTbRJ * sizeof(float);
constexpr size_t kTbAdjSmem = (size_t)11 * kTbAdjRI * kTbRJ * sizeof(float);

template <int RI>
dim3 tb_grid(const TmzDev& t) {
  using G = TbGeom<RI>;
  return dim3((unsigned)((t.ny + G::TJ - 1) / G::TJ), (unsigned)((t.nx + G::TI - 1) / G::TI),
              (unsigned)t.nb);
}

// ---------------------------------------------------------------------------
// Setup and objective.
// ---------------------------------------------------------------------------
// Design coefficients in FP64, formed exactly as a dielectric class's
// (dt / eps, then / dx and / dy).
__global__ void k_tmz_design(const GridDev g, const TmzDev t, const double* eps) {
  const int64_t nd = (int64_t)t.dn[0] * t.dn[1];
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nd * t.nb) return;
  const double e = eps[k];
  const double cdt = g.dt / e;
  DesignCoef d;
  d.c1 = make_coef(cdt / g.dr[0]);
  d.c2 = make_coef(cdt / g.dr[1]);
  d.neg_reps = -1.0 / e;
  d.eps = e;
  const_cast<DesignCoef*>(t.dc)[k] = d;
}

// J[b] = dt * sum over the first nsteps monitor rows of E^2, one block per
// design, fixed summation order (deterministic).
__global__ void k_tmz_objective(const GridDev g, const TmzDev t, int nsteps, double* J) {
  __shared__ double part[256];
  const int b = blockIdx.x;
  const int64_t nm = (int64_t)t.mn[0] * t.mn[1];
  const int64_t count = (int64_t)nsteps * nm;
  const double* mon = t.mon + (int64_t)b * t.total_steps * nm;
  double s = 0.0;
  for (int64_t k = threadIdx.x; k < count; k += blockDim.x) s += mon[k] * mon[k];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) J[b] = g.dt * part[0];
}

dim3 lattice_grid(const TmzDev& t) {
  return dim3((unsigned)((t.ny + kBX - 1) / kBX), (unsigned)((t.nx + kBY - 1) / kBY),
              (unsigned)t.nb);
}

template <class P>
cudaError_t forward(const GridDev& g, const TmzDev& t, int step0, int nsteps, int flags,
                    cudaStream_t s) {
  const dim3 grid = lattice_grid(t), block(kBX, kBY);
  const int64_t nq = (int64_t)t.nsrc * t.nb;
  const unsigned sblocks = (unsigned)((nq + 127) / 128);
  for (int k = 0; k < nsteps; ++k) {
    const int n = step0 + k + 1;
    k_tmz_fe<P><<<grid, block, 0, s>>>(g, t, (flags & GMES_TMZ_RECORD_HIST) ? k : -1);
    if (nq > 0) k_tmz_src<P><<<sblocks, 128, 0, s>>>(t, 0, n);
    k_tmz_fh<P><<<grid, block, 0, s>>>(g, t, (flags & GMES_TMZ_RECORD_MONITOR) ? n - 1 : -1);
    if (nq > 0) k_tmz_src<P><<<sblocks, 128, 0, s>>>(t, 1, n);
  }
  return cudaGetLastError();
}

template <class P>
cudaError_t adjoint(const GridDev& g, const TmzDev& t, int step0, int nsteps, cudaStream_t s) {
  const dim3 grid = lattice_grid(t), block(kBX, kBY);
  const int64_t nq = (int64_t)t.nsrc * t.nb;
  const unsigned sblocks = (unsigned)((nq + 127) / 128);
  for (int k = nsteps - 1; k >= 0; --k) {
    const int n = step0 + k + 1;
    const int rb = n & 1, wb = rb ^ 1;
    if (nq > 0) k_tmz_adj_src<P><<<sblocks, 128, 0, s>>>(t, 1);
    k_tmz_ah<P><<<grid, block, 0, s>>>(g, t, n, rb, wb);
    if (nq > 0) k_tmz_adj_src<P><<<sblocks, 128, 0, s>>>(t, 0);
    k_tmz_ae<P><<<grid, block, 0, s>>>(g, t, k, rb, wb);
  }
  return cudaGetLastError();
}

// The blocked kernels read one copy of the state and write the other, so
// the launches alternate between the state and its scratch copy; with an
// odd number of launches the state is first copied to the scratch, so that
// the last launch writes the state.
void swap_fields(TmzDev& u) {  // forward: state <-> scratch
  for (int k = 0; k < kTmzState; ++k) {
    void* f = u.f[k];
    u.f[k] = u.tmp[k];
    u.tmp[k] = f;
  }
}

void swap_adjoints(TmzDev& u) {  // adjoint: field adjoints <-> scratch
  for (int k = 0; k < 3; ++k) {
    void* l = u.l[k];
    u.l[k] = u.tmp[k];
    u.tmp[k] = l;
  }
}

cudaError_t copy_state(void* const* dst, void* const* src, int n, int64_t bytes, cudaStream_t s) {
  for (int k = 0; k < n; ++k) {
    const cudaError_t e = cudaMemcpyAsync(dst[k], src[k], (size_t)bytes, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t forward_blocked(const GridDev& g, const TmzDev& t, int step0, int nsteps, int flags,
                            int per_launch, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_tmz_tb_fwd<kTbFwdRI>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kTbFwdSmem);
  if (e != cudaSuccess) return e;
  if (t.tmp[0] == nullptr) return cudaErrorInvalidValue;
  const dim3 grid = tb_grid<kTbFwdRI>(t), block(kTbRJ, kTbRows);
  const int launches = (nsteps + per_launch - 1) / per_launch;
  TmzDev u = t;
  if (launches % 2 == 1) {
    e = copy_state(t.tmp, t.f, kTmzState, (int64_t)t.nb * t.plane * (int64_t)sizeof(float), s);
    if (e != cudaSuccess) return e;
    swap_fields(u);
  }
  for (int k = 0; k < nsteps; k += per_launch) {
    const int m = nsteps - k < per_launch ? nsteps - k : per_launch;
    k_tmz_tb_fwd<kTbFwdRI><<<grid, block, kTbFwdSmem, s>>>(
        g, u, step0 + k, m, (flags & GMES_TMZ_RECORD_HIST) ? k : -1,
        (flags & GMES_TMZ_RECORD_MONITOR) ? 1 : 0);
    swap_fields(u);
  }
  return cudaGetLastError();
}

// Launches of the blocked adjoint for nsteps steps of at most per_launch
// each.  Each launch reads the psi adjoints from one buffer and writes the
// other; a call starts from the buffer the one-step kernels' step n0 + nsteps
// reads ((n0 + nsteps) & 1) and must end in the one step n0 + 1 writes
// (n0 & 1), so the number of launches has the parity of nsteps: the fewest
// launches of that parity, their step counts as even as possible.  (Odd
// step counts per launch, the earlier rule, capped launches at 3 steps
// against the forward's 4.)
int adj_launches(int nsteps, int per_launch) {
  int k = (nsteps + per_launch - 1) / per_launch;
  if ((k & 1) != (nsteps & 1)) ++k;
  return k < nsteps ? k : nsteps;
}

cudaError_t adjoint_blocked(const GridDev& g, const TmzDev& t, int step0, int nsteps,
                            int per_launch, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_tmz_tb_adj<kTbAdjRI>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kTbAdjSmem);
  if (e != cudaSuccess) return e;
  if (t.tmp[0] == nullptr) return cudaErrorInvalidValue;
  if (nsteps <= 0) return cudaSuccess;
  const dim3 grid = tb_grid<kTbAdjRI>(t), block(kTbRJ, kTbRows);
  const int launches = adj_launches(nsteps, per_launch);
  TmzDev u = t;
  if (launches % 2 == 1) {
    e = copy_state(t.tmp, t.l, 3, (int64_t)t.nb * t.plane * (int64_t)sizeof(float), s);
    if (e != cudaSuccess) return e;
    swap_adjoints(u);
  }
  int rb = (step0 + nsteps) & 1;
  int hi = nsteps;
  for (int q = 0; q < launches; ++q) {
    // launch q takes an even share of the steps left
    const int m = (hi + (launches - q) - 1) / (launches - q);
    k_tmz_tb_adj<kTbAdjRI><<<grid, block, kTbAdjSmem, s>>>(g, u, step0 + hi - m, m, step0, rb);
    swap_adjoints(u);
    rb ^= 1;
    hi -= m;
  }
  return cudaGetLastError();
}

// Steps per launch for a precision and the caller's request (0: default).
int steps_per_launch(int precision, int requested) {
  if (precision != GMES_FP32) return 1;
  if (requested <= 0) return kTbHalo;
  return requested < kTbHalo ? requested : kTbHalo;
}

}  // namespace

cudaError_t launch_tmz_design(int precision, const GridDev& g, const TmzDev& t,
                              const double* eps, cudaStream_t s) {
  const int64_t n = (int64_t)t.dn[0] * t.dn[1] * t.nb;
  if (n > 0) k_tmz_design<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, t, eps);
  const unsigned mblocks = (unsigned)((t.plane + 255) / 256);
  switch (precision) {
    case GMES_FP64:
      k_tmz_map<PolF64><<<mblocks, 256, 0, s>>>(g, t);
      break;
    case GMES_FP32:
      k_tmz_map<PolF32><<<mblocks, 256, 0, s>>>(g, t);
      break;
    case GMES_DF64:
      k_tmz_map<PolDF><<<mblocks, 256, 0, s>>>(g, t);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  if (t.nsrc > 0) k_tmz_map_sources<<<(t.nsrc + 127) / 128, 128, 0, s>>>(t);
  return cudaGetLastError();
}

cudaError_t launch_tmz_forward(int precision, const GridDev& g, const TmzDev& t, int step0,
                               int nsteps, int flags, int block_steps, cudaStream_t s) {
  const int per = steps_per_launch(precision, block_steps);
  switch (precision) {
    case GMES_FP64:
      return forward<PolF64>(g, t, step0, nsteps, flags, s);
    case GMES_FP32:
      if (per > 1) return forward_blocked(g, t, step0, nsteps, flags, per, s);
      return forward<PolF32>(g, t, step0, nsteps, flags, s);
    case GMES_DF64:
      return forward<PolDF>(g, t, step0, nsteps, flags, s);
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_tmz_adjoint(int precision, const GridDev& g, const TmzDev& t, int step0,
                               int nsteps, int block_steps, cudaStream_t s) {
  const int per = steps_per_launch(precision, block_steps);
  switch (precision) {
    case GMES_FP64:
      return adjoint<PolF64>(g, t, step0, nsteps, s);
    case GMES_FP32:
      if (per > 1) return adjoint_blocked(g, t, step0, nsteps, per, s);
      return adjoint<PolF32>(g, t, step0, nsteps, s);
    case GMES_DF64:
      return adjoint<PolDF>(g, t, step0, nsteps, s);
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_tmz_objective(const GridDev& g, const TmzDev& t, int nsteps, double* J,
                                 cudaStream_t s) {
  k_tmz_objective<<<(unsigned)t.nb, 256, 0, s>>>(g, t, nsteps, J);
  return cudaGetLastError();
}

}  // namespace gmes
