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
#include "gmes_internal.cuh"

namespace gmes {
namespace {

constexpr int kBX = 32, kBY = 8;

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
// Forward.
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
  const R e = P::ldw(E + p.lin);
  const R D1 = P::ld(Y + p.lin) - P::ld(Y + (int64_t)im * t.ny + p.j);
  const R D2 = P::ld(X + p.lin) - P::ld(X + (int64_t)p.i * t.ny + jm);
  const int64_t dp = design_index(t, p.i, p.j);
  if (dp >= 0) {
    const int64_t nd = (int64_t)t.dn[0] * t.dn[1];
    const DesignCoef* dc = t.dc + (int64_t)p.b * nd + dp;
    const R c1 = P::cfg(&dc->c1), c2 = P::cfg(&dc->c2);
    P::st(E + p.lin, (e + c1 * D1) - c2 * D2);
    if (slot >= 0)
      P::st(static_cast<T*>(t.hist) + ((int64_t)slot * t.nb + p.b) * nd + dp, c1 * D1 - c2 * D2);
    return;
  }
  const ClassCoef& cc = class_e(g, p.i, p.j);
  const int kind = __ldg(&cc.kind);
  if (kind == GMES_KIND_DIELECTRIC) {
    P::st(E + p.lin, (e + P::cfg(&cc.c1) * D1) - P::cfg(&cc.c2) * D2);
  } else if (kind == GMES_KIND_CPML) {
    const Prof q = prof_e(g, __ldg(&cc.pml), p.i, p.j);
    const bool on1 = coef_nonzero(q.q1 + 1), on2 = coef_nonzero(q.q2 + 1);
    if (!on1 && !on2) {
      P::st(E + p.lin, (e + P::cfg(&cc.c1) * D1) - P::cfg(&cc.c2) * D2);
      return;
    }
    T* s1 = static_cast<T*>(t.f[3]) + p.base + p.lin;
    T* s2 = static_cast<T*>(t.f[4]) + p.base + p.lin;
    R psi1 = P::ldw(s1), psi2 = P::ldw(s2);
    if (on1) {
      psi1 = P::cfg(q.q1) * psi1 + P::cfg(q.q1 + 3) * D1;
      P::st(s1, psi1);
    }
    if (on2) {
      psi2 = P::cfg(q.q2) * psi2 + P::cfg(q.q2 + 3) * D2;
      P::st(s2, psi2);
    }
    const R xv = ((psi1 - psi2) + P::cfg(q.q1 + 4) * D1) - P::cfg(q.q2 + 4) * D2;
    P::st(E + p.lin, e + P::cfg(&cc.cdt) * xv);
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
  const R e0 = P::ld(E + p.lin);
  const R dx = P::ld(E + (int64_t)p.i * t.ny + jp) - e0;  // D1 of Hx
  const R dy = P::ld(E + (int64_t)ip * t.ny + p.j) - e0;  // D2 of Hy
  {
    const ClassCoef& cc = class_x(g, p.i, p.j);
    const int kind = __ldg(&cc.kind);
    const R x = P::ldw(X + p.lin);
    if (kind == GMES_KIND_DIELECTRIC) {
      P::st(X + p.lin, x - P::cfg(&cc.c1) * dx);
    } else if (kind == GMES_KIND_CPML) {
      const Prof q = prof_x(g, __ldg(&cc.pml), p.i, p.j);
      const bool on1 = coef_nonzero(q.q1 + 1), on2 = coef_nonzero(q.q2 + 1);
      if (!on1 && !on2) {
        P::st(X + p.lin, x - P::cfg(&cc.c1) * dx);
      } else {
        T* s = static_cast<T*>(t.f[5]) + p.base + p.lin;
        R psi = P::ldw(s);
        if (on1) {
          psi = P::cfg(q.q1) * psi + P::cfg(q.q1 + 3) * dx;
          P::st(s, psi);
        }
        P::st(X + p.lin, x - P::cfg(&cc.cdt) * (psi + P::cfg(q.q1 + 4) * dx));
      }
    }
  }
  {
    const ClassCoef& cc = class_y(g, p.i, p.j);
    const int kind = __ldg(&cc.kind);
    const R y = P::ldw(Y + p.lin);
    if (kind == GMES_KIND_DIELECTRIC) {
      P::st(Y + p.lin, y + P::cfg(&cc.c2) * dy);
    } else if (kind == GMES_KIND_CPML) {
      const Prof q = prof_y(g, __ldg(&cc.pml), p.i, p.j);
      const bool on1 = coef_nonzero(q.q1 + 1), on2 = coef_nonzero(q.q2 + 1);
      if (!on1 && !on2) {
        P::st(Y + p.lin, y + P::cfg(&cc.c2) * dy);
      } else {
        T* s = static_cast<T*>(t.f[6]) + p.base + p.lin;
        R psi = P::ldw(s);
        if (on2) {
          psi = P::cfg(q.q2) * psi + P::cfg(q.q2 + 3) * dy;
          P::st(s, psi);
        }
        P::st(Y + p.lin, y - P::cfg(&cc.cdt) * ((-psi) - P::cfg(q.q2 + 4) * dy));
      }
    }
  }
  if (row >= 0) {
    const int64_t m = monitor_index(t, p.i, p.j);
    if (m >= 0) {
      const int64_t nm = (int64_t)t.mn[0] * t.mn[1];
      t.mon[((int64_t)p.b * t.total_steps + row) * nm + m] = to_double(e0);
    }
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
// Adjoint.
// ---------------------------------------------------------------------------
// Curl weight of the Hx point (i, j): lambda_D1 = dX'/dD1 applied to
// lambda_X, with D1 = E(i, j+1) - E(i, j).  OWN: also write the psi adjoint.
template <class P, bool OWN>
__device__ __forceinline__ typename P::R adj_x(const GridDev& g, const TmzDev& t, int64_t base,
                                               int i, int j, int rb, int wb) {
  using R = typename P::R;
  using T = typename P::T;
  const int64_t lin = (int64_t)i * t.ny + j;
  const ClassCoef& cc = class_x(g, i, j);
  const int kind = __ldg(&cc.kind);
  if (kind != GMES_KIND_DIELECTRIC && kind != GMES_KIND_CPML) return P::zero();
  const R lx = P::ldw(static_cast<const T*>(t.l[1]) + base + lin);
  if (kind == GMES_KIND_DIELECTRIC) return -(P::cfg(&cc.c1) * lx);
  const Prof q = prof_x(g, __ldg(&cc.pml), i, j);
  const bool on1 = coef_nonzero(q.q1 + 1), on2 = coef_nonzero(q.q2 + 1);
  if (!on1 && !on2) return -(P::cfg(&cc.c1) * lx);
  const R cdt = P::cfg(&cc.cdt);
  const R direct = -(cdt * (P::cfg(q.q1 + 4) * lx));
  if (!on1) return direct;
  const R L = P::ldw(static_cast<const T*>(t.phi[rb][2]) + base + lin) - cdt * lx;
  if (OWN) P::st(static_cast<T*>(t.phi[wb][2]) + base + lin, P::cfg(q.q1) * L);
  return P::cfg(q.q1 + 3) * L + direct;
}

// Curl weight of the Hy point (i, j): lambda_D2, D2 = E(i+1, j) - E(i, j).
template <class P, bool OWN>
__device__ __forceinline__ typename P::R adj_y(const GridDev& g, const TmzDev& t, int64_t base,
                                               int i, int j, int rb, int wb) {
  using R = typename P::R;
  using T = typename P::T;
  const int64_t lin = (int64_t)i * t.ny + j;
  const ClassCoef& cc = class_y(g, i, j);
  const int kind = __ldg(&cc.kind);
  if (kind != GMES_KIND_DIELECTRIC && kind != GMES_KIND_CPML) return P::zero();
  const R ly = P::ldw(static_cast<const T*>(t.l[2]) + base + lin);
  if (kind == GMES_KIND_DIELECTRIC) return P::cfg(&cc.c2) * ly;
  const Prof q = prof_y(g, __ldg(&cc.pml), i, j);
  const bool on1 = coef_nonzero(q.q1 + 1), on2 = coef_nonzero(q.q2 + 1);
  if (!on1 && !on2) return P::cfg(&cc.c2) * ly;
  const R cdt = P::cfg(&cc.cdt);
  const R direct = cdt * (P::cfg(q.q2 + 4) * ly);
  if (!on2) return direct;
  const R L = P::ldw(static_cast<const T*>(t.phi[rb][3]) + base + lin) + cdt * ly;
  if (OWN) P::st(static_cast<T*>(t.phi[wb][3]) + base + lin, P::cfg(q.q2) * L);
  return P::cfg(q.q2 + 3) * L + direct;
}

// Curl weights (lambda_D1, lambda_D2) of the Ez point (i, j) of design b.
template <class P, bool OWN, bool NEED1, bool NEED2>
__device__ __forceinline__ void adj_e(const GridDev& g, const TmzDev& t, int b, int64_t base,
                                      int i, int j, int rb, int wb, typename P::R& w1,
                                      typename P::R& w2) {
  using R = typename P::R;
  using T = typename P::T;
  const int64_t lin = (int64_t)i * t.ny + j;
  w1 = P::zero();
  w2 = P::zero();
  const int64_t dp = design_index(t, i, j);
  R c1, c2;
  if (dp >= 0) {
    const DesignCoef* dc = t.dc + (int64_t)b * t.dn[0] * t.dn[1] + dp;
    c1 = P::cfg(&dc->c1);
    c2 = P::cfg(&dc->c2);
  } else {
    const ClassCoef& cc = class_e(g, i, j);
    const int kind = __ldg(&cc.kind);
    if (kind != GMES_KIND_DIELECTRIC && kind != GMES_KIND_CPML) return;
    c1 = P::cfg(&cc.c1);
    c2 = P::cfg(&cc.c2);
    if (kind == GMES_KIND_CPML) {
      const Prof q = prof_e(g, __ldg(&cc.pml), i, j);
      const bool on1 = coef_nonzero(q.q1 + 1), on2 = coef_nonzero(q.q2 + 1);
      if (on1 || on2) {
        const R le = P::ldw(static_cast<const T*>(t.l[0]) + base + lin);
        const R cdt = P::cfg(&cc.cdt);
        if (NEED1 || OWN) {
          const R direct = cdt * (P::cfg(q.q1 + 4) * le);
          if (on1) {
            const R L = P::ldw(static_cast<const T*>(t.phi[rb][0]) + base + lin) + cdt * le;
            if (OWN) P::st(static_cast<T*>(t.phi[wb][0]) + base + lin, P::cfg(q.q1) * L);
            w1 = P::cfg(q.q1 + 3) * L + direct;
          } else {
            w1 = direct;
          }
        }
        if (NEED2 || OWN) {
          const R direct = -(cdt * (P::cfg(q.q2 + 4) * le));
          if (on2) {
            const R L = P::ldw(static_cast<const T*>(t.phi[rb][1]) + base + lin) - cdt * le;
            if (OWN) P::st(static_cast<T*>(t.phi[wb][1]) + base + lin, P::cfg(q.q2) * L);
            w2 = P::cfg(q.q2 + 3) * L + direct;
          } else {
            w2 = direct;
          }
        }
        return;
      }
    }
  }
  const R le = P::ldw(static_cast<const T*>(t.l[0]) + base + lin);
  if (NEED1 || OWN) w1 = c1 * le;
  if (NEED2 || OWN) w2 = -(c2 * le);
}

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
  const int64_t m = monitor_index(t, p.i, p.j);
  if (m >= 0) {
    const int64_t nm = (int64_t)t.mn[0] * t.mn[1];
    const double w = t.weight != nullptr ? t.weight[p.b] : 1.0;
    const double e = t.mon[((int64_t)p.b * t.total_steps + (n - 1)) * nm + m];
    le = le + P::from_double(2.0 * g.dt * w * e);
  }
  const R a = adj_x<P, false>(g, t, p.base, p.i, jm, rb, wb);
  const R bx = adj_x<P, true>(g, t, p.base, p.i, p.j, rb, wb);
  const R c = adj_y<P, false>(g, t, p.base, im, p.j, rb, wb);
  const R d = adj_y<P, true>(g, t, p.base, p.i, p.j, rb, wb);
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
  R w1, w2, u1, u2, v1, v2;
  adj_e<P, true, true, true>(g, t, p.b, p.base, p.i, p.j, rb, wb, w1, w2);
  adj_e<P, false, false, true>(g, t, p.b, p.base, p.i, jp, rb, wb, u1, u2);
  adj_e<P, false, true, false>(g, t, p.b, p.base, ip, p.j, rb, wb, v1, v2);
  T* LX = static_cast<T*>(t.l[1]) + p.base + p.lin;
  T* LY = static_cast<T*>(t.l[2]) + p.base + p.lin;
  P::st(LX, P::ldw(LX) + (w2 - u2));
  P::st(LY, P::ldw(LY) + (w1 - v1));
  const int64_t dp = design_index(t, p.i, p.j);
  if (dp >= 0) {
    const int64_t nd = (int64_t)t.dn[0] * t.dn[1];
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

}  // namespace

cudaError_t launch_tmz_design(const GridDev& g, const TmzDev& t, const double* eps,
                              cudaStream_t s) {
  const int64_t n = (int64_t)t.dn[0] * t.dn[1] * t.nb;
  if (n > 0) k_tmz_design<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, t, eps);
  return cudaGetLastError();
}

cudaError_t launch_tmz_forward(int precision, const GridDev& g, const TmzDev& t, int step0,
                               int nsteps, int flags, cudaStream_t s) {
  switch (precision) {
    case GMES_FP64:
      return forward<PolF64>(g, t, step0, nsteps, flags, s);
    case GMES_FP32:
      return forward<PolF32>(g, t, step0, nsteps, flags, s);
    case GMES_DF64:
      return forward<PolDF>(g, t, step0, nsteps, flags, s);
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_tmz_adjoint(int precision, const GridDev& g, const TmzDev& t, int step0,
                               int nsteps, cudaStream_t s) {
  switch (precision) {
    case GMES_FP64:
      return adjoint<PolF64>(g, t, step0, nsteps, s);
    case GMES_FP32:
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
