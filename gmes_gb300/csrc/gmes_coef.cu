// Coefficient builder: every update coefficient of a grid, computed in FP64
// on the GPU from the physical parameters of the classes and PML layers.
//
// Formulas and operation order follow the reference's Cython material
// module so that FP64 results agree with it (exp/pow/sin/cos may differ in
// the last ulp from the host libm):
//   dielectric dt/eps               src/pw_dielectric.hh:118 (dt / eps_inf)
//   Drude a, c                      src/material.pyx:1546-1565
//   Lorentz a, c                    src/material.pyx:1727-1746
//   DCP-ADE a, b, c                 src/material.pyx:1074-1105
//   DCP-PLRC / RC a, b, c           src/material.pyx:1279-1370, 1474-1490
//   PML sigma/kappa grading         src/material.pyx:442-502
//   UPML c1..c6                     src/material.pyx:558-591
//   CPML a, b, c                    src/material.pyx:795-820
#include <cmath>

#include "gmes_internal.cuh"

namespace gmes {
namespace {

__device__ inline int axis1_of(int c) { return (c % 3 + 1) % 3; }
__device__ inline int axis2_of(int c) { return (c % 3 + 2) % 3; }

// Depth into a PML slab along `axis`, or -1 outside both slabs.
__device__ double pml_depth(const gmes_pml_desc& p, double w, int axis) {
  w -= p.center[axis];
  const double h = p.half_size[axis];
  if (w <= p.d - h) return fmin(fmax((h + w) / p.d, 0.0), 1.0);
  if (h - p.d <= w) return fmin(fmax((h - w) / p.d, 0.0), 1.0);
  return -1.0;
}

// Complex arithmetic of the reference's coefficient code (Python complex
// numbers, src/material.pyx:1227-1490): product (ar br - ai bi,
// ar bi + ai br) and Smith's quotient, the algorithm CPython's complex
// division uses.  This file is compiled without FMA contraction.
struct cplx {
  double r, i;
};
__device__ inline cplx cmul(cplx a, cplx b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
__device__ inline cplx cadd(cplx a, cplx b) { return {a.r + b.r, a.i + b.i}; }
__device__ inline cplx csub(cplx a, cplx b) { return {a.r - b.r, a.i - b.i}; }
__device__ inline cplx cdiv(cplx a, cplx b) {
  const double abr = b.r < 0 ? -b.r : b.r, abi = b.i < 0 ? -b.i : b.i;
  if (abr >= abi) {
    if (abr == 0.0) return {0.0, 0.0};
    const double ratio = b.i / b.r;
    const double den = b.r + b.i * ratio;
    return {(a.r + a.i * ratio) / den, (a.i - a.r * ratio) / den};
  }
  const double ratio = b.r / b.i;
  const double den = b.r * ratio + b.i;
  return {(a.r * ratio + a.i) / den, (a.i * ratio - a.r) / den};
}

// Python's sum() over floats (CPython 3.12 builtin sum): Neumaier
// compensated summation, the compensation added when the float run ends.
struct FloatSum {
  double f = 0.0, c = 0.0;
  int n = 0;
  __device__ void add(double x) {
    if (n++ == 0) {
      f = x;
      return;
    }
    const double t = f + x;
    if (fabs(f) >= fabs(x))
      c += (f - t) + x;
    else
      c += (x - t) + f;
    f = t;
  }
  __device__ double value() const { return (c != 0.0 && isfinite(c)) ? f + c : f; }
};

// PLRC / RC coefficients of one DCP class (src/material.pyx:1279-1370):
// a[p] = (dchi - dxi, dxi, exp(-gamma dt)) per Drude term,
// b[q] = (dchi - dxi, dxi, exp(-dt (gamma + i omega))) per critical point,
// c = (dt, eps - xi0 - cond, 1) / (eps - xi0 + chi0 + cond), where chi0 and
// xi0 are sum() over the Drude terms (floats) then the critical points
// (complex), real part.
__device__ void plrc_coefficients(const double* p, int npole, int ncp, double dt, Coef* pool) {
  const double eps_inf = p[0], sigma = p[1];
  const bool rc = p[2] != 0.0;
  const double* dp = p + 3;
  const double* cp = dp + 5 * npole;
  FloatSum chi_f, xi_f;
  for (int q = 0; q < npole; ++q) {
    const double omega = dp[5 * q], gamma = dp[5 * q + 1];
    const double e_m = dp[5 * q + 2], e_p = dp[5 * q + 3], th = dp[5 * q + 4];
    const double gdt = gamma * dt;
    const double w = omega / gamma;
    const double w2 = w * w;
    const double chi = w2 * ((e_m + gdt) - 1.0);
    const double k = 1.0 / (1.0 - e_p) + 1.0 / gdt;
    const double xi = chi * k + w2 * (gdt / 2.0 / th - 1.0);
    const double x = w * (1.0 - e_m);
    const double dchi = -(x * x);
    const double dxi = rc ? 0.0 : dchi * k;
    pool[kPoolA + 3 * q + 0] = make_coef(dchi - dxi);
    pool[kPoolA + 3 * q + 1] = make_coef(dxi);
    pool[kPoolA + 3 * q + 2] = make_coef(e_m);
    chi_f.add(chi);
    if (!rc) xi_f.add(xi);
  }
  double chi0 = chi_f.value(), xi0 = rc ? 0.0 : xi_f.value();
  for (int q = 0; q < ncp; ++q) {
    const double* c = cp + 9 * q;
    const double amp = c[0], omega = c[1], gamma = c[2];
    const cplx P = {c[3], c[4]}, Q = {c[5], c[6]}, R = {c[7], c[8]};
    const cplx go = {gamma, omega};
    const cplx dtgo = cmul({dt, 0.0}, go);
    const cplx one = {1.0, 0.0};
    const cplx omq = csub(one, Q);
    // 2j * amp * omega * exp(1j phi), left to right
    const cplx pre = cmul(cmul(cmul({0.0, 2.0}, {amp, 0.0}), {omega, 0.0}), P);
    const cplx chi = cdiv(cmul(pre, omq), go);
    // (1 - Q)**2 as CPython's integer power: 1 * ((1 - Q) * (1 - Q))
    const cplx dchi = cdiv(cmul(pre, cmul(one, cmul(omq, omq))), go);
    const cplx k = cadd(cdiv(one, csub(one, R)), cdiv(one, dtgo));
    const cplx xi = rc ? cplx{0.0, 0.0} : cmul(chi, k);
    const cplx dxi = rc ? cplx{0.0, 0.0} : cmul(dchi, k);
    const cplx b0 = csub(dchi, dxi);
    pool[kPoolB + 6 * q + 0] = make_coef(b0.r);
    pool[kPoolB + 6 * q + 1] = make_coef(b0.i);
    pool[kPoolB + 6 * q + 2] = make_coef(dxi.r);
    pool[kPoolB + 6 * q + 3] = make_coef(dxi.i);
    pool[kPoolB + 6 * q + 4] = make_coef(Q.r);
    pool[kPoolB + 6 * q + 5] = make_coef(Q.i);
    chi0 = chi0 + chi.r;
    xi0 = xi0 + xi.r;
  }
  const double cond = 0.5 * dt * sigma;
  const double denom = ((eps_inf - xi0) + chi0) + cond;
  pool[kPoolC + 0] = make_coef(dt / denom);
  pool[kPoolC + 1] = make_coef(((eps_inf - xi0) - cond) / denom);
  pool[kPoolC + 2] = make_coef(1.0 / denom);
  pool[kPoolC + 3] = make_coef(0.0);
}

__global__ void k_build_classes(gmes_grid_desc g, CoefLayout L) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  // map t -> (component, class)
  int c = 0, cls = t;
  while (c < 6 && cls >= g.nclass[c]) {
    cls -= g.nclass[c];
    ++c;
  }
  if (c >= 6) return;
  char* base = static_cast<char*>(g.coef);
  const gmes_class_desc* raw = reinterpret_cast<const gmes_class_desc*>(base + L.raw_classes);
  const double* prm = reinterpret_cast<const double*>(base + L.raw_params);
  const gmes_class_desc cd = raw[t];
  ClassCoef* tab = reinterpret_cast<ClassCoef*>(base + L.class_tab[c]);
  Coef* pool = reinterpret_cast<Coef*>(base + L.pool[c]) + (int64_t)cls * kPoolStride;

  const double dt = g.dt;
  const double d1 = g.dr[axis1_of(c)];
  const double d2 = g.dr[axis2_of(c)];
  ClassCoef cc;
  cc.kind = cd.kind;
  cc.pml = cd.pml;
  cc.npole = cd.npole;
  cc.ncp = cd.ncp;
  cc.pad[0] = cc.pad[1] = cc.pad[2] = cc.pad[3] = 0;
  cc.eps = make_coef(cd.eps);
  const double cdt = dt / cd.eps;
  cc.cdt = make_coef(cdt);
  cc.c1 = make_coef(cdt / d1);
  cc.c2 = make_coef(cdt / d2);
  cc.reps = make_coef(1.0 / cd.eps);
  cc.value = make_coef(cd.kind == GMES_KIND_CONST && cd.nparam > 0 ? prm[cd.param_off] : 0.0);
  cc.value_im =
      make_coef(cd.kind == GMES_KIND_CONST && cd.nparam > 1 ? prm[cd.param_off + 1] : 0.0);

  const double* p = prm + cd.param_off;
  if (cd.kind == GMES_KIND_DRUDE || cd.kind == GMES_KIND_LORENTZ) {
    const double eps_inf = p[0], sigma = p[1];
    for (int q = 0; q < cd.npole; ++q) {
      double a0, a1, a2;
      if (cd.kind == GMES_KIND_DRUDE) {
        const double omega = p[2 + 2 * q], gamma = p[3 + 2 * q];
        const double denom = dt * gamma + 2.0;
        const double x = dt * omega;
        a0 = (dt * gamma - 2.0) / denom;
        a1 = 4.0 / denom;
        a2 = 2.0 * (x * x) / denom;
      } else {
        const double amp = p[2 + 3 * q], omega = p[3 + 3 * q], gamma = p[4 + 3 * q];
        const double denom = dt * gamma + 2.0;
        const double x = dt * omega;
        a0 = (dt * gamma - 2.0) / denom;
        a1 = (4.0 - 2.0 * (x * x)) / denom;
        a2 = 2.0 * amp * (x * x) / denom;
      }
      pool[kPoolA + 3 * q + 0] = make_coef(a0);
      pool[kPoolA + 3 * q + 1] = make_coef(a1);
      pool[kPoolA + 3 * q + 2] = make_coef(a2);
    }
    const double denom = 2.0 * eps_inf + dt * sigma;
    pool[kPoolC + 0] = make_coef(2.0 * dt / denom);
    pool[kPoolC + 1] = make_coef(-2.0 / denom);
    pool[kPoolC + 2] = make_coef((2.0 * eps_inf - dt * sigma) / denom);
    pool[kPoolC + 3] = make_coef(0.0);
  } else if (cd.kind == GMES_KIND_DCP_PLRC) {
    plrc_coefficients(p, cd.npole, cd.ncp, dt, pool);
  } else if (cd.kind == GMES_KIND_DCP) {
    const double eps_inf = p[0], sigma = p[1];
    double sum_a2 = 0.0, sum_b2 = 0.0, sum_b3 = 0.0, sum_b4 = 0.0;
    for (int q = 0; q < cd.npole; ++q) {
      const double omega = p[2 + 2 * q], gamma = p[3 + 2 * q];
      const double denom = dt * gamma + 2.0;
      const double x = dt * omega;
      const double a2 = 0.5 * (x * x) / denom;
      pool[kPoolA + 3 * q + 0] = make_coef((dt * gamma - 2.0) / denom);
      pool[kPoolA + 3 * q + 1] = make_coef(4.0 / denom);
      pool[kPoolA + 3 * q + 2] = make_coef(a2);
      sum_a2 = sum_a2 + a2;
    }
    const double* cp = p + 2 + 2 * cd.npole;
    for (int q = 0; q < cd.ncp; ++q) {
      const double amp = cp[5 * q], cphi = cp[5 * q + 1], sphi = cp[5 * q + 2],
                   omega = cp[5 * q + 3], gamma = cp[5 * q + 4];
      const double gp = dt * gamma + 2.0, gm = dt * gamma - 2.0, wo = dt * omega;
      const double denom = gp * gp + wo * wo;
      const double b0 = -(gm * gm + wo * wo) / denom;
      const double b1 = 2.0 * (4.0 - (dt * dt) * (gamma * gamma + omega * omega)) / denom;
      const double b2 = 2.0 * dt * amp * omega *
                        (dt * cphi * omega + sphi * (2.0 - dt * gamma)) / denom;
      const double b3 =
          4.0 * (dt * dt) * amp * omega * (cphi * omega - sphi * gamma) / denom;
      const double b4 = 2.0 * dt * amp * omega *
                        (dt * cphi * omega - sphi * (2.0 + dt * gamma)) / denom;
      pool[kPoolB + 5 * q + 0] = make_coef(b0);
      pool[kPoolB + 5 * q + 1] = make_coef(b1);
      pool[kPoolB + 5 * q + 2] = make_coef(b2);
      pool[kPoolB + 5 * q + 3] = make_coef(b3);
      pool[kPoolB + 5 * q + 4] = make_coef(b4);
      sum_b2 = sum_b2 + b2;
      sum_b3 = sum_b3 + b3;
      sum_b4 = sum_b4 + b4;
    }
    const double denom = 0.5 * dt * sigma + sum_a2 + sum_b4 + eps_inf;
    pool[kPoolC + 0] = make_coef(dt / denom);
    pool[kPoolC + 1] = make_coef(1.0 / denom);
    pool[kPoolC + 2] = make_coef(-(sum_a2 + sum_b2) / denom);
    pool[kPoolC + 3] =
        make_coef(-(0.5 * dt * sigma + 2.0 * sum_a2 + sum_b3 - eps_inf) / denom);
  }
  tab[cls] = cc;
}

// One thread per (pml, component, axis, index along the axis).
__global__ void k_build_profiles(gmes_grid_desc g, CoefLayout L, int64_t maxn) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int item = blockIdx.y;  // pml * 18 + comp * 3 + axis
  const int pi = item / 18, c = (item / 3) % 6, axis = item % 3;
  if (pi >= g.npml || !(g.active & (1 << c))) return;
  int64_t sh[3];
  comp_shape(g.n, g.active, c, sh);
  if (t >= sh[axis] || t >= maxn) return;
  char* base = static_cast<char*>(g.coef);
  const gmes_pml_desc p = reinterpret_cast<const gmes_pml_desc*>(base + L.raw_pmls)[pi];
  Coef* out = reinterpret_cast<Coef*>(base + L.prof[pi][c][axis]) + t * kProfStride;

  // Yee coordinate (gmes/geometry.py:360-732)
  const double w = ((double)t + yee_offset(c, axis)) * g.dr[axis] - g.half[axis];
  const double depth = pml_depth(p, w, axis);
  double sigma = 0.0, kappa = 1.0, a = 0.0;
  if (depth >= 0.0) {
    const double r = pow(1.0 - depth, p.m);
    sigma = p.sigma_max[axis] * r;
    kappa = 1.0 + (p.kappa_max - 1.0) * r;
    a = p.a_max * pow(depth, p.m_a);
  }
  const double dt = g.dt;
  if (p.kind == GMES_KIND_CPML) {
    const double b = exp(-(sigma / kappa + a) * dt);
    const double den = (sigma + kappa * a) * kappa;
    const double cc = den != 0.0 ? sigma * (b - 1.0) / den : 0.0;
    out[0] = make_coef(b);
    out[1] = make_coef(cc);
    out[2] = make_coef(kappa);
    out[3] = make_coef(cc / g.dr[axis]);
    out[4] = make_coef(1.0 / (kappa * g.dr[axis]));
  } else {
    const double num = 2.0 * kappa - sigma * dt;
    const double den = 2.0 * kappa + sigma * dt;
    out[0] = make_coef(num / den);
    out[1] = make_coef(2.0 * dt / den);
    out[2] = make_coef(1.0 / den);
    out[3] = make_coef(den);
    out[4] = make_coef(num);
  }
}

}  // namespace

cudaError_t launch_build_coefficients(const gmes_grid_desc& g, const GridDev& d,
                                      cudaStream_t s) {
  (void)d;
  const CoefLayout L = coef_layout(g);
  int ncls = 0;
  for (int c = 0; c < 6; ++c) ncls += g.nclass[c];
  if (ncls > 0) {
    k_build_classes<<<(ncls + 127) / 128, 128, 0, s>>>(g, L);
  }
  if (g.npml > 0) {
    int64_t maxn = 1;
    for (int a = 0; a < 3; ++a) maxn = maxn > g.n[a] + 1 ? maxn : g.n[a] + 1;
    dim3 grid((unsigned)((maxn + 127) / 128), (unsigned)(g.npml * 18));
    k_build_profiles<<<grid, 128, 0, s>>>(g, L, maxn);
  }
  return cudaGetLastError();
}

}  // namespace gmes
