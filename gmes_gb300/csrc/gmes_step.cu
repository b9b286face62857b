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
#include "gmes_internal.cuh"

namespace gmes {
namespace {

constexpr int kThreads = 256;
constexpr int kIChunk = 16;  // cells per thread along i in k_march

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
template <class P, int C, bool DISP>
__device__ __forceinline__ void update_fast(const GridDev& g, int64_t lin, const int x[3],
                                            typename P::R p1, typename P::R p2) {
  using R = typename P::R;
  using T = typename P::T;
  constexpr int own = C % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  constexpr bool E = C < 3;
  const uint8_t id = g.cls[C][lin];
  const ClassCoef& cc = g.tab[C][id];
  const int kind = cc.kind;
  if (kind == GMES_KIND_DUMMY) return;
  T* fp = static_cast<T*>(g.f[C]) + lin;
  if (kind == GMES_KIND_DIELECTRIC) {
    const R F = P::ldw(fp);
    const R c1 = P::cf(cc.c1), c2 = P::cf(cc.c2);
    P::st(fp, E ? (F + c1 * p1) - c2 * p2 : (F + c2 * p2) - c1 * p1);
    return;
  }
  T* aux = static_cast<T*>(g.aux[C]);
  const int64_t np = g.npts[C];
  if (kind == GMES_KIND_CPML) {
    const Coef* q1 = g.prof[cc.pml][C][a1] + (int64_t)x[a1] * kProfStride;
    const Coef* q2 = g.prof[cc.pml][C][a2] + (int64_t)x[a2] * kProfStride;
    T* s1 = aux + lin;
    T* s2 = aux + np + lin;
    const R psi1 = P::cf(q1[0]) * P::ldw(s1) + P::cf(q1[3]) * p1;
    const R psi2 = P::cf(q2[0]) * P::ldw(s2) + P::cf(q2[3]) * p2;
    P::st(s1, psi1);
    P::st(s2, psi2);
    const R X = (P::cf(q1[4]) * p1 - P::cf(q2[4]) * p2) + (psi1 - psi2);
    const R F = P::ldw(fp);
    const R cdt = P::cf(cc.cdt);
    P::st(fp, E ? F + cdt * X : F - cdt * X);
    return;
  }
  const R r1 = P::cf(g.rdr[a1]);
  const R r2 = P::cf(g.rdr[a2]);
  if (kind == GMES_KIND_UPML) {
    const Coef* q1 = g.prof[cc.pml][C][a1] + (int64_t)x[a1] * kProfStride;
    const Coef* q2 = g.prof[cc.pml][C][a2] + (int64_t)x[a2] * kProfStride;
    const Coef* q3 = g.prof[cc.pml][C][own] + (int64_t)x[own] * kProfStride;
    T* sp = aux + lin;
    const R d_old = P::ldw(sp);
    const R curl = p1 * r1 - p2 * r2;
    const R d_new = E ? P::cf(q1[0]) * d_old + P::cf(q1[1]) * curl
                      : P::cf(q1[0]) * d_old - P::cf(q1[1]) * curl;
    P::st(sp, d_new);
    const R F = P::ldw(fp);
    P::st(fp, P::cf(q2[0]) * F +
                  P::cf(q2[2]) * (P::cf(q3[3]) * d_new - P::cf(q3[4]) * d_old) *
                      P::cf(cc.reps));
    return;
  }
  if (kind == GMES_KIND_CONST) {
    P::st(fp, P::cf(cc.value));
    return;
  }
  if constexpr (DISP && E) {
    const Coef* pool = g.pool[C] + (int64_t)id * kPoolStride;
    const R curl = p1 * r1 - p2 * r2;
    const R e_now = P::ldw(fp);
    if (kind == GMES_KIND_DRUDE || kind == GMES_KIND_LORENTZ) {
      // src/pw_drude.hh:89-151, src/pw_lorentz.hh:96-157
      R sum = P::zero();
      for (int q = 0; q < cc.npole; ++q) {
        T* qn = aux + (int64_t)(2 * q) * np + lin;      // q_now
        T* qw = aux + (int64_t)(2 * q + 1) * np + lin;  // q_new
        const R q_old = P::ldw(qn);
        const R q_now = P::ldw(qw);
        const R q_new = P::cf(pool[kPoolA + 3 * q]) * q_old +
                        P::cf(pool[kPoolA + 3 * q + 1]) * q_now +
                        P::cf(pool[kPoolA + 3 * q + 2]) * e_now;
        P::st(qn, q_now);
        P::st(qw, q_new);
        sum = sum + (q_new - q_now);
      }
      P::st(fp, P::cf(pool[kPoolC]) * curl + P::cf(pool[kPoolC + 1]) * sum +
                    P::cf(pool[kPoolC + 2]) * e_now);
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
        const R a0 = P::cf(pool[kPoolA + 3 * q]), a1c = P::cf(pool[kPoolA + 3 * q + 1]);
        sd = sd + ((P::from_double(1.0) - a1c) * qn - a0 * qo);
      }
      const int cb = 1 + 2 * cc.npole;
      for (int q = 0; q < cc.ncp; ++q) {
        const R po = P::ldw(aux + (int64_t)(cb + 2 * q) * np + lin);
        const R pn = P::ldw(aux + (int64_t)(cb + 2 * q + 1) * np + lin);
        const R b0 = P::cf(pool[kPoolB + 5 * q]), b1 = P::cf(pool[kPoolB + 5 * q + 1]);
        sc = sc + ((P::from_double(1.0) - b1) * pn - b0 * po);
      }
      const R e_new = P::cf(pool[kPoolC]) * curl + P::cf(pool[kPoolC + 1]) * (sd + sc) +
                      P::cf(pool[kPoolC + 2]) * e_old + P::cf(pool[kPoolC + 3]) * e_now;
      const R esum = (e_old + P::from_double(2.0) * e_now) + e_new;
      for (int q = 0; q < cc.npole; ++q) {
        T* qop = aux + (int64_t)(1 + 2 * q) * np + lin;
        T* qnp = aux + (int64_t)(2 + 2 * q) * np + lin;
        const R qo = P::ldw(qop), qn = P::ldw(qnp);
        const R q_new = P::cf(pool[kPoolA + 3 * q]) * qo + P::cf(pool[kPoolA + 3 * q + 1]) * qn +
                        P::cf(pool[kPoolA + 3 * q + 2]) * esum;
        P::st(qop, qn);
        P::st(qnp, q_new);
      }
      for (int q = 0; q < cc.ncp; ++q) {
        T* pop = aux + (int64_t)(cb + 2 * q) * np + lin;
        T* pnp = aux + (int64_t)(cb + 2 * q + 1) * np + lin;
        const R po = P::ldw(pop), pn = P::ldw(pnp);
        const Coef* b = pool + kPoolB + 5 * q;
        const R p_new = P::cf(b[0]) * po + P::cf(b[1]) * pn + P::cf(b[2]) * e_old +
                        P::cf(b[3]) * e_now + P::cf(b[4]) * e_new;
        P::st(pop, pn);
        P::st(pnp, p_new);
      }
      P::st(eo, e_now);
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
                                              double D1, double D2) {
  constexpr int own = C % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  constexpr bool E = C < 3;
  const uint8_t id = g.cls[C][lin];
  const ClassCoef& cc = g.tab[C][id];
  const int kind = cc.kind;
  if (kind == GMES_KIND_DUMMY) return;
  double* fp = static_cast<double*>(g.f[C]) + lin;
  const double dt = g.dt, d1 = g.dr[a1], d2 = g.dr[a2], eps = cc.eps.d;
  if (kind == GMES_KIND_DIELECTRIC) {
    // E: e += dt/eps * (D1/d1 - D2/d2); H: h += dt/mu * (D2/d2 - D1/d1)
    const double X = E ? SUB(DIV(D1, d1), DIV(D2, d2)) : SUB(DIV(D2, d2), DIV(D1, d1));
    *fp = ADD(*fp, MUL(DIV(dt, eps), X));
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
    *fp = E ? ADD(*fp, inc) : SUB(*fp, inc);
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
    *fp = ADD(MUL(q2[0].d, *fp),
              DIV(MUL(q2[2].d, SUB(MUL(q3[3].d, dn), MUL(q3[4].d, dstore))), eps));
    return;
  }
  if (kind == GMES_KIND_CONST) {
    *fp = cc.value.d;
    return;
  }
  if constexpr (DISP && E) {
    const Coef* pool = g.pool[C] + (int64_t)id * kPoolStride;
    const double e_now = *fp;
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
  }
}

// E component C at cell (i, j, k).
template <class P, int C, bool STRICT, bool DISP>
__device__ __forceinline__ void cell_e(const GridDev& g, int i, int j, int k) {
  using R = typename P::R;
  using T = typename P::T;
  constexpr int own = C, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  constexpr int in1 = 3 + a2, in2 = 3 + a1;
  const int x[3] = {i, j, k};
  const int64_t lin = (int64_t)i * g.st[C][0] + (int64_t)j * g.st[C][1] + k;
  R p1 = P::zero(), p2 = P::zero();
  if (g.active & (1 << in1)) {
    const T* h = static_cast<const T*>(g.f[in1]);
    const int64_t b = (int64_t)i * g.st[in1][0] + (int64_t)j * g.st[in1][1] + k +
                      stride_of<in1>(g, own);
    p1 = P::ld(h + b + stride_of<in1>(g, a1)) - P::ld(h + b);
  }
  if (g.active & (1 << in2)) {
    const T* h = static_cast<const T*>(g.f[in2]);
    const int64_t b = (int64_t)i * g.st[in2][0] + (int64_t)j * g.st[in2][1] + k +
                      stride_of<in2>(g, own);
    p2 = P::ld(h + b + stride_of<in2>(g, a2)) - P::ld(h + b);
  }
  if constexpr (STRICT)
    update_strict<C, DISP>(g, lin, x, p1, p2);
  else
    update_fast<P, C, DISP>(g, lin, x, p1, p2);
}

// H component C (3..5) at cell (i, j, k) = point (i, j, k) + e_a1 + e_a2.
template <class P, int C, bool STRICT, bool DISP>
__device__ __forceinline__ void cell_h(const GridDev& g, int i, int j, int k) {
  using R = typename P::R;
  using T = typename P::T;
  constexpr int own = C - 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  constexpr int in1 = a2, in2 = a1;
  int x[3] = {i, j, k};
  x[a1] += 1;
  x[a2] += 1;
  const int64_t lin = (int64_t)x[0] * g.st[C][0] + (int64_t)x[1] * g.st[C][1] + x[2];
  R p1 = P::zero(), p2 = P::zero();
  if (g.active & (1 << in1)) {
    const T* e = static_cast<const T*>(g.f[in1]);
    const int64_t b = (int64_t)i * g.st[in1][0] + (int64_t)j * g.st[in1][1] + k;
    p1 = P::ld(e + b + stride_of<in1>(g, a1)) - P::ld(e + b);
  }
  if (g.active & (1 << in2)) {
    const T* e = static_cast<const T*>(g.f[in2]);
    const int64_t b = (int64_t)i * g.st[in2][0] + (int64_t)j * g.st[in2][1] + k;
    p2 = P::ld(e + b + stride_of<in2>(g, a2)) - P::ld(e + b);
  }
  if constexpr (STRICT)
    update_strict<C, DISP>(g, lin, x, p1, p2);
  else
    update_fast<P, C, DISP>(g, lin, x, p1, p2);
}

template <class P, int SIDE, bool STRICT, bool DISP>
__global__ void __launch_bounds__(kThreads) k_half(const GridDev g, int i0) {
  // plane = n1 * n2 < 2^31 (checked by the host)
  const int plane = g.n[1] * g.n[2];
  const int t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= plane) return;
  const int j = t / g.n[2];
  const int k = t - j * g.n[2];
  const int i = i0 + (int)blockIdx.y;
  if (i >= g.n[0]) return;
  if constexpr (SIDE == 0) {
    if (g.active & 1) cell_e<P, 0, STRICT, DISP>(g, i, j, k);
    if (g.active & 2) cell_e<P, 1, STRICT, DISP>(g, i, j, k);
    if (g.active & 4) cell_e<P, 2, STRICT, DISP>(g, i, j, k);
  } else {
    if (g.active & 8) cell_h<P, 3, STRICT, DISP>(g, i, j, k);
    if (g.active & 16) cell_h<P, 4, STRICT, DISP>(g, i, j, k);
    if (g.active & 32) cell_h<P, 5, STRICT, DISP>(g, i, j, k);
  }
}

// Column-marching form of the half-step for grids with n2 >= 32: a block of
// 32 x 8 threads covers a (k, j) tile and every thread walks a run of
// `ichunk` cells along i.  The value of the previous i plane that the curl
// needs (Hz and Hy for the E half, Ez and Ey for the H half) is carried in
// registers, so each cell loads 7 neighbour values instead of 9 and no index
// is divided.  In-plane offsets are 32-bit; the i offset is 64-bit.
template <class P, int C>
__device__ __forceinline__ typename P::R ldc(const GridDev& g, int64_t off) {
  if (!(g.active & (1 << C))) return P::zero();
  return P::ld(static_cast<const typename P::T*>(g.f[C]) + off);
}

template <class P, int C, bool STRICT, bool DISP>
__device__ __forceinline__ void upd(const GridDev& g, int64_t lin, int x0, int x1, int x2,
                                    typename P::R p1, typename P::R p2) {
  if (!(g.active & (1 << C))) return;
  const int x[3] = {x0, x1, x2};
  if constexpr (STRICT)
    update_strict<C, DISP>(g, lin, x, p1, p2);
  else
    update_fast<P, C, DISP>(g, lin, x, p1, p2);
}

template <class P, int SIDE, bool STRICT, bool DISP>
__global__ void __launch_bounds__(256) k_march(const GridDev g, int ichunk) {
  using R = typename P::R;
  const int k = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int ibeg = blockIdx.z * ichunk;
  if (k >= g.n[2] || j >= g.n[1] || ibeg >= g.n[0]) return;
  const int iend = min(ibeg + ichunk, g.n[0]);
  // per-component strides (axis 2 stride is 1)
  const int64_t sx0 = g.st[0][0], sy0 = g.st[1][0], sz0 = g.st[2][0];
  const int64_t hx0 = g.st[3][0], hy0 = g.st[4][0], hz0 = g.st[5][0];
  const int sx1 = (int)g.st[0][1], sy1 = (int)g.st[1][1], sz1 = (int)g.st[2][1];
  const int hx1 = (int)g.st[3][1], hy1 = (int)g.st[4][1], hz1 = (int)g.st[5][1];
  if constexpr (SIDE == 0) {
    // E half.  Hz[i, j+1, k] and Hy[i, j, k+1] carried along i.
    R hz_prev = ldc<P, 5>(g, (int64_t)ibeg * hz0 + (j + 1) * hz1 + k);
    R hy_prev = ldc<P, 4>(g, (int64_t)ibeg * hy0 + j * hy1 + k + 1);
    for (int i = ibeg; i < iend; ++i) {
      const int64_t hzb = (int64_t)(i + 1) * hz0 + j * hz1 + k;  // Hz[i+1, j, k]
      const int64_t hyb = (int64_t)(i + 1) * hy0 + j * hy1 + k;  // Hy[i+1, j, k]
      const int64_t hxb = (int64_t)i * hx0 + j * hx1 + k;        // Hx[i, j, k]
      const R hz_a = ldc<P, 5>(g, hzb + hz1);                    // Hz[i+1, j+1, k]
      const R hz_b = ldc<P, 5>(g, hzb);
      const R hy_a = ldc<P, 4>(g, hyb + 1);                      // Hy[i+1, j, k+1]
      const R hy_b = ldc<P, 4>(g, hyb);
      const R hx_a = ldc<P, 3>(g, hxb + hx1 + 1);                // Hx[i, j+1, k+1]
      const R hx_b = ldc<P, 3>(g, hxb + hx1);                    // Hx[i, j+1, k]
      const R hx_c = ldc<P, 3>(g, hxb + 1);                      // Hx[i, j, k+1]
      upd<P, 0, STRICT, DISP>(g, (int64_t)i * sx0 + j * sx1 + k, i, j, k, hz_a - hz_b,
                              hy_a - hy_b);
      upd<P, 1, STRICT, DISP>(g, (int64_t)i * sy0 + j * sy1 + k, i, j, k, hx_a - hx_b,
                              hz_a - hz_prev);
      upd<P, 2, STRICT, DISP>(g, (int64_t)i * sz0 + j * sz1 + k, i, j, k, hy_a - hy_prev,
                              hx_a - hx_c);
      hz_prev = hz_a;
      hy_prev = hy_a;
    }
  } else {
    // H half.  Ez[i, j, k] and Ey[i, j, k] carried along i.
    R ez_cur = ldc<P, 2>(g, (int64_t)ibeg * sz0 + j * sz1 + k);
    R ey_cur = ldc<P, 1>(g, (int64_t)ibeg * sy0 + j * sy1 + k);
    for (int i = ibeg; i < iend; ++i) {
      const int64_t ezb = (int64_t)i * sz0 + j * sz1 + k;
      const int64_t eyb = (int64_t)i * sy0 + j * sy1 + k;
      const int64_t exb = (int64_t)i * sx0 + j * sx1 + k;
      const R ez_n = ldc<P, 2>(g, ezb + sz0);      // Ez[i+1, j, k]
      const R ez_j = ldc<P, 2>(g, ezb + sz1);      // Ez[i, j+1, k]
      const R ey_n = ldc<P, 1>(g, eyb + sy0);      // Ey[i+1, j, k]
      const R ey_k = ldc<P, 1>(g, eyb + 1);        // Ey[i, j, k+1]
      const R ex_0 = ldc<P, 0>(g, exb);            // Ex[i, j, k]
      const R ex_k = ldc<P, 0>(g, exb + 1);        // Ex[i, j, k+1]
      const R ex_j = ldc<P, 0>(g, exb + sx1);      // Ex[i, j+1, k]
      upd<P, 3, STRICT, DISP>(g, (int64_t)i * hx0 + (j + 1) * hx1 + k + 1, i, j + 1, k + 1,
                              ez_j - ez_cur, ey_k - ey_cur);
      upd<P, 4, STRICT, DISP>(g, (int64_t)(i + 1) * hy0 + j * hy1 + k + 1, i + 1, j, k + 1,
                              ex_k - ex_0, ez_n - ez_cur);
      upd<P, 5, STRICT, DISP>(g, (int64_t)(i + 1) * hz0 + (j + 1) * hz1 + k, i + 1, j + 1, k,
                              ey_n - ey_cur, ex_j - ex_0);
      ez_cur = ez_n;
      ey_cur = ey_n;
    }
  }
}

// Ghost planes of one half's components (gmes/fdtd.py:811-1097 with the
// single-domain cyclic communicator): E ghosts are the last planes along the
// non-own axes and receive plane 0; H ghosts are the first planes and
// receive the last plane.  A ghost point's source is found by mapping every
// ghost coordinate at once, so corners get the value the reference's two
// successive plane copies give them and no source is itself a ghost.
template <class T>
__global__ void k_ghost(const GridDev g, int side, int64_t maxplane) {
  const int item = blockIdx.y;  // component-in-side * 2 + which ghost axis
  const int c = side * 3 + item / 2;
  if (!(g.active & (1 << c))) return;
  const int own = c % 3;
  const int ga = (item & 1) ? (own + 2) % 3 : (own + 1) % 3;
  const int pa = (ga + 1) % 3, qa = (ga + 2) % 3;
  const int p_ = pa < qa ? pa : qa, q_ = pa < qa ? qa : pa;  // q_ is the faster axis
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t np = g.sh[c][p_] * g.sh[c][q_];
  if (t >= np || t >= maxplane) return;
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

// Point sources of one half-step (gmes/pw_source.py:74-131), applied after
// that half's material update.  `v` has been computed on the host in FP64.
template <class P, bool STRICT>
__global__ void k_sources(const GridDev g, int side, int64_t slot) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= g.nsrc) return;
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

// One half-step: ghost copy of the other half's components, the fused
// update of this half's components, this half's point sources.
template <class P, bool STRICT>
void run_half(const GridDev& d, int side, int st, cudaStream_t s, bool disp) {
  using T = typename P::T;
  const int64_t plane = (int64_t)d.n[1] * d.n[2];
  const unsigned bx = (unsigned)((plane + kThreads - 1) / kThreads);
  int64_t maxplane = 1;
  for (int c = 0; c < 6; ++c)
    for (int a = 0; a < 3; ++a)
      for (int b = a + 1; b < 3; ++b) {
        const int64_t v = d.sh[c][a] * d.sh[c][b];
        maxplane = v > maxplane ? v : maxplane;
      }
  const dim3 ggrid((unsigned)((maxplane + 255) / 256), 6);
  constexpr int kMaxY = 65535;
  k_ghost<T><<<ggrid, 256, 0, s>>>(d, 1 - side, maxplane);
  if (d.n[2] >= 32) {
    const dim3 grid((unsigned)((d.n[2] + 31) / 32), (unsigned)((d.n[1] + 7) / 8),
                    (unsigned)((d.n[0] + kIChunk - 1) / kIChunk));
    const dim3 block(32, 8);
    if (side == 0) {
      if (disp)
        k_march<P, 0, STRICT, true><<<grid, block, 0, s>>>(d, kIChunk);
      else
        k_march<P, 0, STRICT, false><<<grid, block, 0, s>>>(d, kIChunk);
    } else {
      k_march<P, 1, STRICT, false><<<grid, block, 0, s>>>(d, kIChunk);
    }
  } else {
    for (int i0 = 0; i0 < d.n[0]; i0 += kMaxY) {
      const dim3 grid(bx, (unsigned)min(kMaxY, d.n[0] - i0));
      if (side == 0) {
        if (disp)
          k_half<P, 0, STRICT, true><<<grid, kThreads, 0, s>>>(d, i0);
        else
          k_half<P, 0, STRICT, false><<<grid, kThreads, 0, s>>>(d, i0);
      } else {
        k_half<P, 1, STRICT, false><<<grid, kThreads, 0, s>>>(d, i0);
      }
    }
  }
  if (d.nsrc > 0)
    k_sources<P, STRICT><<<(d.nsrc + 127) / 128, 128, 0, s>>>(d, side, 2 * (int64_t)st + side);
}

template <class P, bool STRICT>
cudaError_t run_steps(const GridDev& d, int nsteps, int side_mask, int st0, cudaStream_t s,
                      bool disp) {
  for (int st = 0; st < nsteps; ++st) {
    if (side_mask & 1) run_half<P, STRICT>(d, 0, st0 + st, s, disp);
    if (side_mask & 2) run_half<P, STRICT>(d, 1, st0 + st, s, disp);
  }
  return cudaGetLastError();
}

template <class P, bool STRICT>
cudaError_t dispatch(const gmes_grid_desc& g, const GridDev& d, int nsteps, int side_mask,
                     int st0, cudaStream_t s) {
  const bool disp = (g.flags & GMES_FLAG_DISPERSIVE) != 0;
  return run_steps<P, STRICT>(d, nsteps, side_mask, st0, s, disp);
}

cudaError_t dispatch_precision(const gmes_grid_desc& g, const GridDev& d, int nsteps,
                               int side_mask, int st0, cudaStream_t s) {
  switch (g.precision) {
    case GMES_FP64:
      return dispatch<PolF64, false>(g, d, nsteps, side_mask, st0, s);
    case GMES_FP64_STRICT:
      return dispatch<PolF64, true>(g, d, nsteps, side_mask, st0, s);
    case GMES_FP32:
      return dispatch<PolF32, false>(g, d, nsteps, side_mask, st0, s);
    case GMES_DF64:
      return dispatch<PolDF, false>(g, d, nsteps, side_mask, st0, s);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_step(const gmes_grid_desc& g, const GridDev& d, int nsteps, cudaStream_t s) {
  return dispatch_precision(g, d, nsteps, 3, 0, s);
}

cudaError_t launch_half(const gmes_grid_desc& g, const GridDev& d, int side, int step,
                        cudaStream_t s) {
  return dispatch_precision(g, d, 1, side == 0 ? 1 : 2, step, s);
}

}  // namespace gmes
