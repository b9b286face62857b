/*
 * gmes_oracle.c -- CPU oracle for the FDTD time step.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker; the product never calls it.
 *
 * A plain-C restatement of the reference (GMES) hot path, keeping its
 * structure as well as its arithmetic:
 *   - per field component, one updater per material class, each holding an
 *     array-of-structs list of points with per-point parameters and state
 *     (PwMaterial<T>::idx_list / param_list, src/pw_material.hh:49-117);
 *   - per-point CPML/UPML coefficients evaluated at each point's own Yee
 *     coordinate, as Cpml.get_pw_material_* does (src/material.pyx:822-954,
 *     593-729) with the grading of src/material.pyx:442-502, 795-820;
 *   - dispersive coefficients from src/material.pyx:1074-1105 (DCP),
 *     1546-1565 (Drude), 1727-1746 (Lorentz);
 *   - the update expressions of src/pw_dielectric.hh:118-371,
 *     src/pw_cpml.hh:115-447, src/pw_upml.hh:113-432,
 *     src/pw_drude.hh:89-151, src/pw_lorentz.hh:96-157,
 *     src/pw_dcp.hh:105-225, in the same operation order (compile with
 *     -ffp-contract=off so no multiply-add is fused);
 *   - the loop of FDTD.step (gmes/fdtd.py:1099-1122) with the serial
 *     periodic ghost copies of talk_with_*_neighbors (gmes/fdtd.py:811-1097)
 *     done as the reference's two successive plane copies;
 *   - OpenMP static scheduling above a point-count threshold
 *     (src/cpp23_support.hh:150-197, GMES_OPENMP_THRESHOLD default 8192).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

enum { K_DUMMY = 0, K_DIEL = 1, K_CPML = 2, K_UPML = 3, K_DRUDE = 4, K_LORENTZ = 5,
       K_DCP = 6, K_CONST = 7, K_DCP_PLRC = 8 };
#define MAXP 8
#define MAXCLS 256
#define MAXPML 4

typedef struct {
  int kind, pml, npole, ncp;
  double eps;
  double params[3 + 5 * MAXP + 9 * MAXP];
  int nparams;
  /* dispersive coefficients (per class, copied into every point by the reference) */
  double a[MAXP][3];
  double b[MAXP][5];
  double bc[MAXP][6]; /* DcpPlrc: b0, b1, b2 as (re, im) */
  double c[4];
} oclass;

typedef struct {
  int kind;
  double sigma_max[3], m, kappa_max, m_a, a_max, d, center[3], half_size[3];
} opml;

/* Per-point parameter structs (AoS), mirroring the reference's Param types. */
typedef struct { int64_t off; int idx[3]; double eps; } p_diel;
typedef struct { int64_t off; int idx[3]; double eps, b1, b2, c1, c2, k1, k2, psi1, psi2; } p_cpml;
typedef struct { int64_t off; int idx[3]; double eps, c1, c2, c3, c4, c5, c6, d; } p_upml;
typedef struct { int64_t off; int idx[3]; double st[1 + 4 * MAXP]; } p_ade;
typedef struct { int64_t off; int idx[3]; } p_plain;

typedef struct {
  int comp, cls, kind;
  int64_t count;
  void* pts;
} updater;

typedef struct oracle_s {
  int n[3];
  int active;
  double dr[3], half[3], dt;
  int64_t sh[6][3];
  double* f[6];
  oclass cls[6][MAXCLS];
  int ncls[6];
  opml pml[MAXPML];
  int npml;
  updater* upd[6];
  int nupd[6];
  int nsrc;
  int* src_comp;
  int* src_mode;
  int64_t* src_off;
  int64_t omp_threshold;
  /* TFSF: the incident-field oracle (a TEMz grid) and the transparent
     points, up to 4 faces each (gmes/pw_source.py:134-486) */
  struct oracle_s* incident;
  int ntfsf;
  int* tf_comp;
  int* tf_nface;
  int64_t* tf_off;
  double* tf_coef;  /* [ntfsf][4] */
  double* tf_r0;
  double* tf_r1;
  int64_t* tf_sample;
  /* complex grids: this oracle holds the real parts, `imag` the imaginary
     parts; the ghost copies multiply by the Bloch phases */
  struct oracle_s* imag;
  double phase[6][2][2];
} oracle;

static void comp_shape(const int n[3], int active, int c, int64_t sh[3]) {
  if (!(active & (1 << c))) { sh[0] = sh[1] = sh[2] = 1; return; }
  int own = c % 3;
  for (int a = 0; a < 3; ++a) sh[a] = a == own ? n[a] : n[a] + 1;
}

static double yee_offset(int c, int axis) {
  if (c < 3) return axis == c ? 0.5 : 0.0;
  return axis == c - 3 ? 0.0 : -0.5;
}

/* *_index_to_space (gmes/geometry.py:360-732): (idx + off) * dr - half,
   idx * dr - half when the offset is zero. */
static double coord(const oracle* o, int c, int axis, int idx) {
  double off = yee_offset(c, axis);
  if (off == 0.0) return (double)idx * o->dr[axis] - o->half[axis];
  return ((double)idx + off) * o->dr[axis] - o->half[axis];
}

/* ---- PML grading (src/material.pyx:474-502, 558-591, 795-820) ---------- */
static int pml_depth(const opml* p, double w, int axis, double* depth) {
  w -= p->center[axis];
  double h = p->half_size[axis];
  if (w <= p->d - h) { *depth = fmin(fmax((h + w) / p->d, 0), 1); return 1; }
  if (h - p->d <= w) { *depth = fmin(fmax((h - w) / p->d, 0), 1); return 1; }
  return 0;
}
static double pml_sigma(const opml* p, double w, int axis) {
  double depth;
  if (!pml_depth(p, w, axis, &depth)) return 0;
  return p->sigma_max[axis] * pow(1 - depth, p->m);
}
static double pml_kappa(const opml* p, double w, int axis) {
  double depth;
  if (!pml_depth(p, w, axis, &depth)) return 1;
  return 1 + (p->kappa_max - 1) * pow(1 - depth, p->m);
}
static double cpml_a(const opml* p, double w, int axis) {
  double depth;
  if (!pml_depth(p, w, axis, &depth)) return 0;
  return p->a_max * pow(depth, p->m_a);
}
static double cpml_b(const opml* p, double dt, double w, int axis) {
  double exponent = -(pml_sigma(p, w, axis) / pml_kappa(p, w, axis) + cpml_a(p, w, axis)) * dt;
  return exp(exponent);
}
static double cpml_c(const opml* p, double dt, double w, int axis) {
  double sigma = pml_sigma(p, w, axis);
  double kappa = pml_kappa(p, w, axis);
  double numerator = sigma * (cpml_b(p, dt, w, axis) - 1);
  double denominator = (sigma + kappa * cpml_a(p, w, axis)) * kappa;
  return denominator != 0 ? numerator / denominator : 0;
}
static double upml_c1(const opml* p, double dt, double w, int ax) {
  return (2 * pml_kappa(p, w, ax) - pml_sigma(p, w, ax) * dt) /
         (2 * pml_kappa(p, w, ax) + pml_sigma(p, w, ax) * dt);
}
static double upml_c2(const opml* p, double dt, double w, int ax) {
  return 2 * dt / (2 * pml_kappa(p, w, ax) + pml_sigma(p, w, ax) * dt);
}
static double upml_c4(const opml* p, double dt, double w, int ax) {
  return 1 / (2 * pml_kappa(p, w, ax) + pml_sigma(p, w, ax) * dt);
}
static double upml_c5(const opml* p, double dt, double w, int ax) {
  return 2 * pml_kappa(p, w, ax) + pml_sigma(p, w, ax) * dt;
}
static double upml_c6(const opml* p, double dt, double w, int ax) {
  return 2 * pml_kappa(p, w, ax) - pml_sigma(p, w, ax) * dt;
}

/* ---- Python complex arithmetic (src/material.pyx computes the DcpPlrc
   coefficients with Python complex numbers): product (ac - bd, ad + bc)
   and CPython's quotient (Smith's algorithm). */
typedef struct { double r, i; } cpx;
static cpx cmul(cpx a, cpx b) { cpx z = {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; return z; }
static cpx cadd(cpx a, cpx b) { cpx z = {a.r + b.r, a.i + b.i}; return z; }
static cpx csub(cpx a, cpx b) { cpx z = {a.r - b.r, a.i - b.i}; return z; }
static cpx cdiv(cpx a, cpx b) {
  const double abr = b.r < 0 ? -b.r : b.r, abi = b.i < 0 ? -b.i : b.i;
  cpx z = {0, 0};
  if (abr >= abi) {
    if (abr == 0.0) return z;
    const double ratio = b.i / b.r, den = b.r + b.i * ratio;
    z.r = (a.r + a.i * ratio) / den;
    z.i = (a.i - a.r * ratio) / den;
  } else {
    const double ratio = b.r / b.i, den = b.r * ratio + b.i;
    z.r = (a.r * ratio + a.i) / den;
    z.i = (a.i * ratio - a.r) / den;
  }
  return z;
}

/* Python's sum() over floats (CPython 3.12): Neumaier compensated
   summation, the compensation added when the float run ends. */
typedef struct { double f, c; int n; } fsum;
static void fsum_add(fsum* s, double x) {
  if (s->n++ == 0) { s->f = x; return; }
  const double t = s->f + x;
  if (fabs(s->f) >= fabs(x)) s->c += (s->f - t) + x; else s->c += (x - t) + s->f;
  s->f = t;
}
static double fsum_value(const fsum* s) { return (s->c != 0 && isfinite(s->c)) ? s->f + s->c : s->f; }

/* DcpPlrc / DcpRc coefficients (src/material.pyx:1279-1370, 1474-1490) from
   eps_inf, sigma, rc, per Drude term (omega, gamma, exp(-g dt), exp(g dt),
   tanh(g dt / 2)), per critical point (amp, omega, gamma, cos phi, sin phi,
   exp(-dt (g + i w)), exp(dt (g + i w))). */
static void init_plrc(oclass* k, double dt) {
  const double* p = k->params;
  const double eps_inf = p[0], sigma = p[1];
  const int rc = p[2] != 0.0;
  const double* dp = p + 3;
  const double* cp = dp + 5 * k->npole;
  fsum chi_f = {0, 0, 0}, xi_f = {0, 0, 0};
  for (int q = 0; q < k->npole; ++q) {
    const double omega = dp[5 * q], gamma = dp[5 * q + 1];
    const double e_m = dp[5 * q + 2], e_p = dp[5 * q + 3], th = dp[5 * q + 4];
    const double gdt = gamma * dt, w = omega / gamma, w2 = w * w;
    const double chi = w2 * ((e_m + gdt) - 1.0);
    const double kk = 1.0 / (1.0 - e_p) + 1.0 / gdt;
    const double xi = chi * kk + w2 * (gdt / 2.0 / th - 1.0);
    const double x = w * (1.0 - e_m);
    const double dchi = -(x * x);
    const double dxi = rc ? 0.0 : dchi * kk;
    k->a[q][0] = dchi - dxi;
    k->a[q][1] = dxi;
    k->a[q][2] = e_m;
    fsum_add(&chi_f, chi);
    if (!rc) fsum_add(&xi_f, xi);
  }
  double chi0 = fsum_value(&chi_f), xi0 = rc ? 0.0 : fsum_value(&xi_f);
  for (int q = 0; q < k->ncp; ++q) {
    const double* c = cp + 9 * q;
    const double amp = c[0], omega = c[1], gamma = c[2];
    const cpx P = {c[3], c[4]}, Q = {c[5], c[6]}, R = {c[7], c[8]};
    const cpx go = {gamma, omega}, one = {1.0, 0.0}, dtr = {dt, 0.0};
    const cpx dtgo = cmul(dtr, go);
    const cpx omq = csub(one, Q);
    const cpx two_j = {0.0, 2.0}, ampc = {amp, 0.0}, omc = {omega, 0.0};
    const cpx pre = cmul(cmul(cmul(two_j, ampc), omc), P);
    const cpx chi = cdiv(cmul(pre, omq), go);
    const cpx dchi = cdiv(cmul(pre, cmul(one, cmul(omq, omq))), go);
    const cpx kk = cadd(cdiv(one, csub(one, R)), cdiv(one, dtgo));
    const cpx zero = {0.0, 0.0};
    const cpx xi = rc ? zero : cmul(chi, kk);
    const cpx dxi = rc ? zero : cmul(dchi, kk);
    const cpx b0 = csub(dchi, dxi);
    k->bc[q][0] = b0.r; k->bc[q][1] = b0.i;
    k->bc[q][2] = dxi.r; k->bc[q][3] = dxi.i;
    k->bc[q][4] = Q.r; k->bc[q][5] = Q.i;
    chi0 = chi0 + chi.r;
    xi0 = xi0 + xi.r;
  }
  const double cond = 0.5 * dt * sigma;
  const double denom = ((eps_inf - xi0) + chi0) + cond;
  k->c[0] = dt / denom;
  k->c[1] = ((eps_inf - xi0) - cond) / denom;
  k->c[2] = 1 / denom;
}

/* ---- dispersive coefficients --------------------------------------------- */
static void init_dispersive(oclass* k, double dt) {
  if (k->kind == K_DCP_PLRC) { init_plrc(k, dt); return; }
  const double* p = k->params;
  if (k->kind == K_DRUDE || k->kind == K_LORENTZ) {
    double eps_inf = p[0], sigma = p[1];
    for (int q = 0; q < k->npole; ++q) {
      if (k->kind == K_DRUDE) {
        double omega = p[2 + 2 * q], gamma = p[3 + 2 * q];
        double denom = dt * gamma + 2.;
        double x = dt * omega;
        k->a[q][0] = (dt * gamma - 2) / denom;
        k->a[q][1] = 4 / denom;
        k->a[q][2] = 2 * (x * x) / denom;
      } else {
        double amp = p[2 + 3 * q], omega = p[3 + 3 * q], gamma = p[4 + 3 * q];
        double denom = dt * gamma + 2.;
        double x = dt * omega;
        k->a[q][0] = (dt * gamma - 2) / denom;
        k->a[q][1] = (4 - 2 * (x * x)) / denom;
        k->a[q][2] = 2 * amp * (x * x) / denom;
      }
    }
    double denom = 2. * eps_inf + dt * sigma;
    k->c[0] = 2 * dt / denom;
    k->c[1] = -2 / denom;
    k->c[2] = (2 * eps_inf - dt * sigma) / denom;
  } else if (k->kind == K_DCP) {
    double eps_inf = p[0], sigma = p[1];
    double sa2 = 0, sb2 = 0, sb3 = 0, sb4 = 0;
    for (int q = 0; q < k->npole; ++q) {
      double omega = p[2 + 2 * q], gamma = p[3 + 2 * q];
      double denom = dt * gamma + 2;
      double x = dt * omega;
      k->a[q][0] = (dt * gamma - 2) / denom;
      k->a[q][1] = 4 / denom;
      k->a[q][2] = 0.5 * (x * x) / denom;
      sa2 = sa2 + k->a[q][2];
    }
    const double* cp = p + 2 + 2 * k->npole;
    for (int q = 0; q < k->ncp; ++q) {
      /* per critical point: amp, cos(phi), sin(phi), omega, gamma */
      double amp = cp[5 * q], cphi = cp[5 * q + 1], sphi = cp[5 * q + 2];
      double omega = cp[5 * q + 3], gamma = cp[5 * q + 4];
      double gp = dt * gamma + 2, gm = dt * gamma - 2, wo = dt * omega;
      double denom = gp * gp + wo * wo;
      k->b[q][0] = -(gm * gm + wo * wo) / denom;
      k->b[q][1] = 2 * (4 - (dt * dt) * (gamma * gamma + omega * omega)) / denom;
      k->b[q][2] = 2 * dt * amp * omega * (dt * cphi * omega + sphi * (2 - dt * gamma)) / denom;
      k->b[q][3] = 4 * (dt * dt) * amp * omega * (cphi * omega - sphi * gamma) / denom;
      k->b[q][4] = 2 * dt * amp * omega * (dt * cphi * omega - sphi * (2 + dt * gamma)) / denom;
      sb2 = sb2 + k->b[q][2];
      sb3 = sb3 + k->b[q][3];
      sb4 = sb4 + k->b[q][4];
    }
    double denom = 0.5 * dt * sigma + sa2 + sb4 + eps_inf;
    k->c[0] = dt / denom;
    k->c[1] = 1 / denom;
    k->c[2] = -(sa2 + sb2) / denom;
    k->c[3] = -(0.5 * dt * sigma + 2 * sa2 + sb3 - eps_inf) / denom;
  }
}

/* ---- API ------------------------------------------------------------------ */
oracle* oracle_create(const int n[3], int active, const double dr[3], const double half[3],
                      double dt) {
  oracle* o = (oracle*)calloc(1, sizeof(oracle));
  if (!o) return NULL;
  for (int a = 0; a < 3; ++a) { o->n[a] = n[a]; o->dr[a] = dr[a]; o->half[a] = half[a]; }
  o->active = active;
  o->dt = dt;
  o->omp_threshold = 8192;
  const char* env = getenv("GMES_OPENMP_THRESHOLD");
  if (env && *env) o->omp_threshold = atoll(env);
  for (int c = 0; c < 6; ++c) {
    comp_shape(n, active, c, o->sh[c]);
    int64_t np = o->sh[c][0] * o->sh[c][1] * o->sh[c][2];
    o->f[c] = (double*)calloc((size_t)np, sizeof(double));
    if (!o->f[c]) return NULL;
  }
  return o;
}

int oracle_add_pml(oracle* o, int kind, const double sigma_max[3], double m, double kappa_max,
                   double m_a, double a_max, double d, const double center[3],
                   const double half_size[3]) {
  if (o->npml >= MAXPML) return -1;
  opml* p = &o->pml[o->npml];
  p->kind = kind;
  for (int a = 0; a < 3; ++a) {
    p->sigma_max[a] = sigma_max[a];
    p->center[a] = center[a];
    p->half_size[a] = half_size[a];
  }
  p->m = m; p->kappa_max = kappa_max; p->m_a = m_a; p->a_max = a_max; p->d = d;
  return o->npml++;
}

int oracle_add_class(oracle* o, int comp, int kind, double eps, int pml, int npole, int ncp,
                     const double* params, int nparams) {
  if (comp < 0 || comp > 5 || o->ncls[comp] >= MAXCLS || npole > MAXP || ncp > MAXP) return -1;
  if (nparams > (int)(sizeof(((oclass*)0)->params) / sizeof(double))) return -1;
  oclass* k = &o->cls[comp][o->ncls[comp]];
  memset(k, 0, sizeof(*k));
  k->kind = kind; k->eps = eps; k->pml = pml; k->npole = npole; k->ncp = ncp;
  k->nparams = nparams;
  for (int i = 0; i < nparams; ++i) k->params[i] = params[i];
  init_dispersive(k, o->dt);
  return o->ncls[comp]++;
}

/* Build the point lists of one component from its class map: points are
   visited in C order (np.ndindex order, gmes/fdtd.py:362), and each class's
   points are appended to its updater, as attach/merge do. */
int oracle_set_class_map(oracle* o, int c, const uint8_t* map) {
  const int64_t* sh = o->sh[c];
  int64_t np = sh[0] * sh[1] * sh[2];
  int64_t count[MAXCLS] = {0};
  for (int64_t t = 0; t < np; ++t) {
    if (map[t] >= o->ncls[c]) return -1;
    count[map[t]]++;
  }
  o->upd[c] = (updater*)calloc(MAXCLS, sizeof(updater));
  o->nupd[c] = 0;
  int slot[MAXCLS];
  for (int k = 0; k < o->ncls[c]; ++k) {
    slot[k] = -1;
    if (count[k] == 0 || o->cls[c][k].kind == K_DUMMY) continue;
    updater* u = &o->upd[c][o->nupd[c]];
    u->comp = c; u->cls = k; u->kind = o->cls[c][k].kind; u->count = 0;
    size_t sz;
    switch (u->kind) {
      case K_DIEL: sz = sizeof(p_diel); break;
      case K_CPML: sz = sizeof(p_cpml); break;
      case K_UPML: sz = sizeof(p_upml); break;
      case K_DRUDE: case K_LORENTZ: case K_DCP: case K_DCP_PLRC: sz = sizeof(p_ade); break;
      default: sz = sizeof(p_plain); break;
    }
    u->pts = calloc((size_t)count[k], sz);
    if (!u->pts) return -2;
    slot[k] = o->nupd[c]++;
  }
  const int own = c % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  for (int64_t t = 0; t < np; ++t) {
    int k = map[t];
    if (slot[k] < 0) continue;
    updater* u = &o->upd[c][slot[k]];
    const oclass* cl = &o->cls[c][k];
    int idx[3];
    idx[0] = (int)(t / (sh[1] * sh[2]));
    idx[1] = (int)((t / sh[2]) % sh[1]);
    idx[2] = (int)(t % sh[2]);
    double w[3];
    for (int a = 0; a < 3; ++a) w[a] = coord(o, c, a, idx[a]);
    switch (u->kind) {
      case K_DIEL: {
        p_diel* p = (p_diel*)u->pts + u->count;
        p->off = t; memcpy(p->idx, idx, sizeof(idx)); p->eps = cl->eps;
        break;
      }
      case K_CPML: {
        const opml* q = &o->pml[cl->pml];
        p_cpml* p = (p_cpml*)u->pts + u->count;
        p->off = t; memcpy(p->idx, idx, sizeof(idx)); p->eps = cl->eps;
        p->b1 = cpml_b(q, o->dt, w[a1], a1);
        p->b2 = cpml_b(q, o->dt, w[a2], a2);
        p->c1 = cpml_c(q, o->dt, w[a1], a1);
        p->c2 = cpml_c(q, o->dt, w[a2], a2);
        p->k1 = pml_kappa(q, w[a1], a1);
        p->k2 = pml_kappa(q, w[a2], a2);
        p->psi1 = p->psi2 = 0;
        break;
      }
      case K_UPML: {
        const opml* q = &o->pml[cl->pml];
        p_upml* p = (p_upml*)u->pts + u->count;
        p->off = t; memcpy(p->idx, idx, sizeof(idx)); p->eps = cl->eps;
        p->c1 = upml_c1(q, o->dt, w[a1], a1);
        p->c2 = upml_c2(q, o->dt, w[a1], a1);
        p->c3 = upml_c1(q, o->dt, w[a2], a2);
        p->c4 = upml_c4(q, o->dt, w[a2], a2);
        p->c5 = upml_c5(q, o->dt, w[own], own);
        p->c6 = upml_c6(q, o->dt, w[own], own);
        p->d = 0;
        break;
      }
      case K_DRUDE: case K_LORENTZ: case K_DCP: case K_DCP_PLRC: {
        p_ade* p = (p_ade*)u->pts + u->count;
        p->off = t; memcpy(p->idx, idx, sizeof(idx));
        break;
      }
      default: {
        p_plain* p = (p_plain*)u->pts + u->count;
        p->off = t; memcpy(p->idx, idx, sizeof(idx));
      }
    }
    u->count++;
  }
  return 0;
}

int oracle_set_sources(oracle* o, int n, const int* comp, const int* mode, const int64_t* off) {
  o->nsrc = n;
  o->src_comp = (int*)malloc(sizeof(int) * (n ? n : 1));
  o->src_mode = (int*)malloc(sizeof(int) * (n ? n : 1));
  o->src_off = (int64_t*)malloc(sizeof(int64_t) * (n ? n : 1));
  for (int i = 0; i < n; ++i) {
    o->src_comp[i] = comp[i]; o->src_mode[i] = mode[i]; o->src_off[i] = off[i];
  }
  return 0;
}

double* oracle_field(oracle* o, int c) { return o->f[c]; }

/* (b, c, kappa) [CPML] or (sigma, kappa, 0) [UPML] along one axis of one
   component, n = shape[axis] rows: lets the GPU run with the host libm's
   exact profile values. */
int oracle_pml_profile(const oracle* o, int pml, int c, int axis, double* out) {
  if (pml < 0 || pml >= o->npml) return -1;
  const opml* q = &o->pml[pml];
  for (int64_t i = 0; i < o->sh[c][axis]; ++i) {
    double w = coord(o, c, axis, (int)i);
    if (q->kind == K_CPML) {
      out[3 * i] = cpml_b(q, o->dt, w, axis);
      out[3 * i + 1] = cpml_c(q, o->dt, w, axis);
      out[3 * i + 2] = pml_kappa(q, w, axis);
    } else {
      out[3 * i] = pml_sigma(q, w, axis);
      out[3 * i + 1] = pml_kappa(q, w, axis);
      out[3 * i + 2] = 0;
    }
  }
  return 0;
}

/* ---- the updates ---------------------------------------------------------- */
#define AT(c, i, j, k) (o->f[c][((int64_t)(i) * o->sh[c][1] + (j)) * o->sh[c][2] + (k)])

/* The two curl differences of component c at point idx, as bound by
   FDTD.update_e?/h? (gmes/fdtd.py:673-809), reading inactive (collapsed)
   components as zero -- their (1,1,1) arrays are never written. */
static void diffs(const oracle* o, int c, const int x[3], double* D1, double* D2) {
  const int own = c % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  int in1, in2;
  int p[3] = {x[0], x[1], x[2]}, q[3];
  if (c < 3) {
    in1 = 3 + a2; in2 = 3 + a1;
    p[own] += 1;
    *D1 = *D2 = 0;
    if (o->active & (1 << in1)) {
      memcpy(q, p, sizeof(q)); q[a1] += 1;
      *D1 = AT(in1, q[0], q[1], q[2]) - AT(in1, p[0], p[1], p[2]);
    }
    if (o->active & (1 << in2)) {
      memcpy(q, p, sizeof(q)); q[a2] += 1;
      *D2 = AT(in2, q[0], q[1], q[2]) - AT(in2, p[0], p[1], p[2]);
    }
  } else {
    in1 = a2; in2 = a1;
    *D1 = *D2 = 0;
    if (o->active & (1 << in1)) {
      int u[3] = {x[0], x[1], x[2]}; u[a2] -= 1;
      int v[3] = {u[0], u[1], u[2]}; v[a1] -= 1;
      *D1 = AT(in1, u[0], u[1], u[2]) - AT(in1, v[0], v[1], v[2]);
    }
    if (o->active & (1 << in2)) {
      int u[3] = {x[0], x[1], x[2]}; u[a1] -= 1;
      int v[3] = {u[0], u[1], u[2]}; v[a2] -= 1;
      *D2 = AT(in2, u[0], u[1], u[2]) - AT(in2, v[0], v[1], v[2]);
    }
  }
}

static void run_updater(oracle* o, const updater* u) {
  const int c = u->comp;
  const int own = c % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  const double d1 = o->dr[a1], d2 = o->dr[a2], dt = o->dt;
  const int E = c < 3;
  const oclass* cl = &o->cls[c][u->cls];
  double* f = o->f[c];
  const int64_t count = u->count;
  switch (u->kind) {
    case K_DIEL: {
      p_diel* pts = (p_diel*)u->pts;
#pragma omp parallel for schedule(static) if (count >= o->omp_threshold)
      for (int64_t t = 0; t < count; ++t) {
        double D1, D2;
        diffs(o, c, pts[t].idx, &D1, &D2);
        if (E)
          f[pts[t].off] += dt / pts[t].eps * (D1 / d1 - D2 / d2);
        else
          f[pts[t].off] += dt / pts[t].eps * (D2 / d2 - D1 / d1);
      }
      break;
    }
    case K_CPML: {
      p_cpml* pts = (p_cpml*)u->pts;
#pragma omp parallel for schedule(static) if (count >= o->omp_threshold)
      for (int64_t t = 0; t < count; ++t) {
        p_cpml* p = &pts[t];
        double D1, D2;
        diffs(o, c, p->idx, &D1, &D2);
        p->psi1 = p->b1 * p->psi1 + p->c1 * D1 / d1;
        p->psi2 = p->b2 * p->psi2 + p->c2 * D2 / d2;
        double X = D1 / d1 / p->k1 - D2 / d2 / p->k2 + p->psi1 - p->psi2;
        if (E)
          f[p->off] += dt / p->eps * X;
        else
          f[p->off] -= dt / p->eps * X;
      }
      break;
    }
    case K_UPML: {
      p_upml* pts = (p_upml*)u->pts;
#pragma omp parallel for schedule(static) if (count >= o->omp_threshold)
      for (int64_t t = 0; t < count; ++t) {
        p_upml* p = &pts[t];
        double D1, D2;
        diffs(o, c, p->idx, &D1, &D2);
        const double dstore = p->d;
        if (E)
          p->d = p->c1 * p->d + p->c2 * (D1 / d1 - D2 / d2);
        else
          p->d = p->c1 * p->d - p->c2 * (D1 / d1 - D2 / d2);
        f[p->off] = p->c3 * f[p->off] + p->c4 * (p->c5 * p->d - p->c6 * dstore) / p->eps;
      }
      break;
    }
    case K_DRUDE:
    case K_LORENTZ: {
      p_ade* pts = (p_ade*)u->pts;
      const int P = cl->npole;
#pragma omp parallel for schedule(static) if (count >= o->omp_threshold)
      for (int64_t t = 0; t < count; ++t) {
        p_ade* p = &pts[t];
        double D1, D2;
        diffs(o, c, p->idx, &D1, &D2);
        double* q_now = p->st;      /* q_now[P] */
        double* q_new = p->st + P;  /* q_new[P] */
        const double e_now = f[p->off];
        double q_old[MAXP];
        for (int i = 0; i < P; ++i) q_old[i] = q_now[i];
        for (int i = 0; i < P; ++i) q_now[i] = q_new[i];
        for (int i = 0; i < P; ++i)
          q_new[i] = cl->a[i][0] * q_old[i] + cl->a[i][1] * q_now[i] + cl->a[i][2] * e_now;
        double sum = 0;
        for (int i = 0; i < P; ++i) sum += q_new[i] - q_now[i];
        f[p->off] = cl->c[0] * (D1 / d1 - D2 / d2) + cl->c[1] * sum + cl->c[2] * e_now;
      }
      break;
    }
    case K_DCP: {
      p_ade* pts = (p_ade*)u->pts;
      const int P = cl->npole, Q = cl->ncp;
#pragma omp parallel for schedule(static) if (count >= o->omp_threshold)
      for (int64_t t = 0; t < count; ++t) {
        p_ade* p = &pts[t];
        double D1, D2;
        diffs(o, c, p->idx, &D1, &D2);
        double* e_old = p->st;
        double* q_old = p->st + 1;
        double* q_now = p->st + 1 + P;
        double* p_old = p->st + 1 + 2 * P;
        double* p_now = p->st + 1 + 2 * P + Q;
        const double e_now = f[p->off];
        double dsum = 0, csum = 0;
        for (int i = 0; i < P; ++i) dsum += (1 - cl->a[i][1]) * q_now[i] - cl->a[i][0] * q_old[i];
        for (int i = 0; i < Q; ++i) csum += (1 - cl->b[i][1]) * p_now[i] - cl->b[i][0] * p_old[i];
        const double e_new = cl->c[0] * (D1 / d1 - D2 / d2) + cl->c[1] * (dsum + csum) +
                             cl->c[2] * *e_old + cl->c[3] * e_now;
        double q_new[MAXP], p_new[MAXP];
        for (int i = 0; i < P; ++i)
          q_new[i] = cl->a[i][0] * q_old[i] + cl->a[i][1] * q_now[i] +
                     cl->a[i][2] * (*e_old + 2.0 * e_now + e_new);
        for (int i = 0; i < P; ++i) { q_old[i] = q_now[i]; q_now[i] = q_new[i]; }
        for (int i = 0; i < Q; ++i)
          p_new[i] = cl->b[i][0] * p_old[i] + cl->b[i][1] * p_now[i] + cl->b[i][2] * *e_old +
                     cl->b[i][3] * e_now + cl->b[i][4] * e_new;
        for (int i = 0; i < Q; ++i) { p_old[i] = p_now[i]; p_now[i] = p_new[i]; }
        *e_old = e_now;
        f[p->off] = e_new;
      }
      break;
    }
    case K_DCP_PLRC: {
      /* src/pw_dcp.hh:466-583: e_new from the curl, e_now and the total
         accumulator, then psi_dp[P] (real) and psi_cp[Q] (complex) */
      p_ade* pts = (p_ade*)u->pts;
      const int P = cl->npole, Q = cl->ncp;
#pragma omp parallel for schedule(static) if (count >= o->omp_threshold)
      for (int64_t t = 0; t < count; ++t) {
        p_ade* p = &pts[t];
        double D1, D2;
        diffs(o, c, p->idx, &D1, &D2);
        double* psi_dp = p->st;
        double* psi_cp = p->st + P; /* (re, im) pairs */
        const double e_now = f[p->off];
        double sdp = 0, scp = 0;
        for (int i = 0; i < P; ++i) sdp += psi_dp[i];
        for (int i = 0; i < Q; ++i) scp += psi_cp[2 * i];
        const double e_new = cl->c[0] * (D1 / d1 - D2 / d2) + cl->c[1] * e_now +
                             cl->c[2] * (sdp + scp);
        for (int i = 0; i < P; ++i)
          psi_dp[i] = cl->a[i][0] * e_new + cl->a[i][1] * e_now + cl->a[i][2] * psi_dp[i];
        for (int i = 0; i < Q; ++i) {
          const double pr = psi_cp[2 * i], pi = psi_cp[2 * i + 1];
          const double* b = cl->bc[i];
          psi_cp[2 * i] = b[0] * e_new + b[2] * e_now + (b[4] * pr - b[5] * pi);
          psi_cp[2 * i + 1] = b[1] * e_new + b[3] * e_now + (b[4] * pi + b[5] * pr);
        }
        f[p->off] = e_new;
      }
      break;
    }
    case K_CONST: {
      p_plain* pts = (p_plain*)u->pts;
      for (int64_t t = 0; t < count; ++t) f[pts[t].off] = cl->params[0];
      break;
    }
    default:
      break;
  }
}

/* One ghost-plane copy: plane `dst` along `axis` of component c <- plane `src`. */
static void copy_plane(oracle* o, int c, int axis, int64_t dst, int64_t src) {
  const int64_t* sh = o->sh[c];
  const int p = (axis + 1) % 3, q = (axis + 2) % 3;
  for (int64_t u = 0; u < sh[p]; ++u)
    for (int64_t v = 0; v < sh[q]; ++v) {
      int64_t x[3], y[3];
      x[axis] = dst; x[p] = u; x[q] = v;
      y[axis] = src; y[p] = u; y[q] = v;
      AT(c, x[0], x[1], x[2]) = AT(c, y[0], y[1], y[2]);
    }
}

/* talk_with_{ex..hz}_neighbors in serial (gmes/fdtd.py:811-1097): E sends
   plane 0 to the last plane, first along own+1 then own+2 (Ex: y then z,
   Ey: z then x, Ez: x then y); H sends the last plane to plane 0, in the
   same axis order. */
static void chatter(oracle* o, int c) {
  if (!(o->active & (1 << c))) return;
  const int own = c % 3;
  const int ax[2] = {(own + 1) % 3, (own + 2) % 3};
  for (int h = 0; h < 2; ++h) {
    const int64_t last = o->sh[c][ax[h]] - 1;
    if (c < 3)
      copy_plane(o, c, ax[h], last, 0);
    else
      copy_plane(o, c, ax[h], 0, last);
  }
}

static void apply_sources(oracle* o, int side, const double* vals) {
  for (int q = 0; q < o->nsrc; ++q) {
    const int c = o->src_comp[q];
    if ((c < 3) != (side == 0)) continue;
    double* f = o->f[c] + o->src_off[q];
    if (o->src_mode[q] == 0)
      *f = vals[q];
    else
      *f -= vals[q];
  }
}

/* TFSF consistency corrections of one half, each point's faces in order:
   F -= / += dt/(eps d) * amp * (r0 A[s] + r1 A[s+1]) with A the incident
   grid's Hy (E side) or Ex (H side); coef holds the signed
   dt/(eps d) * amp (gmes/pw_source.py:196-486). */
static void apply_transparent(oracle* o, int side) {
  if (!o->incident) return;
  const double* A = o->incident->f[side == 0 ? 4 : 0];
  for (int q = 0; q < o->ntfsf; ++q) {
    const int c = o->tf_comp[q];
    if ((c < 3) != (side == 0)) continue;
    double* f = o->f[c] + o->tf_off[q];
    for (int k = 0; k < o->tf_nface[q]; ++k) {
      const int64_t sp = o->tf_sample[4 * q + k];
      const double inc = o->tf_r0[4 * q + k] * A[sp] + o->tf_r1[4 * q + k] * A[sp + 1];
      *f = *f + o->tf_coef[4 * q + k] * inc;
    }
  }
}

int oracle_set_tfsf(oracle* o, oracle* incident, int n, const int* comp, const int* nface,
                    const int64_t* off, const double* coef, const double* r0, const double* r1,
                    const int64_t* sample) {
  o->incident = incident;
  o->ntfsf = n;
  size_t m = (size_t)(n ? n : 1);
  o->tf_comp = (int*)malloc(m * sizeof(int));
  o->tf_nface = (int*)malloc(m * sizeof(int));
  o->tf_off = (int64_t*)malloc(m * sizeof(int64_t));
  o->tf_coef = (double*)malloc(4 * m * sizeof(double));
  o->tf_r0 = (double*)malloc(4 * m * sizeof(double));
  o->tf_r1 = (double*)malloc(4 * m * sizeof(double));
  o->tf_sample = (int64_t*)malloc(4 * m * sizeof(int64_t));
  if (!o->tf_comp || !o->tf_nface || !o->tf_off || !o->tf_coef || !o->tf_r0 || !o->tf_r1 ||
      !o->tf_sample)
    return -1;
  const int64_t na[2] = {incident->sh[4][0] * incident->sh[4][1] * incident->sh[4][2],
                         incident->sh[0][0] * incident->sh[0][1] * incident->sh[0][2]};
  for (int q = 0; q < n; ++q) {
    if (comp[q] < 0 || comp[q] > 5 || nface[q] < 1 || nface[q] > 4) return -2;
    o->tf_comp[q] = comp[q];
    o->tf_nface[q] = nface[q];
    o->tf_off[q] = off[q];
    for (int k = 0; k < 4; ++k) {
      o->tf_coef[4 * q + k] = coef[4 * q + k];
      o->tf_r0[4 * q + k] = r0[4 * q + k];
      o->tf_r1[4 * q + k] = r1[4 * q + k];
      o->tf_sample[4 * q + k] = sample[4 * q + k];
      if (k < nface[q] && (sample[4 * q + k] < 0 || sample[4 * q + k] + 1 >= na[comp[q] < 3 ? 0 : 1]))
        return -3;
    }
  }
  return 0;
}

/* src_vals: [nsteps][2][nsrc] (E value, H value per source); aux_vals the
   same for the incident-field grid (NULL without TFSF).  The incident grid
   takes its full step between the E and H halves, as FDTD.step calls
   _step_aux_fdtd (gmes/fdtd.py:1099-1122). */
int oracle_step_tfsf(oracle* o, int nsteps, const double* src_vals, const double* aux_vals) {
  if (o->incident && !aux_vals) return -1;
  for (int s = 0; s < nsteps; ++s) {
    for (int c = 3; c < 6; ++c) chatter(o, c);
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < o->nupd[c]; ++k) run_updater(o, &o->upd[c][k]);
    apply_sources(o, 0, src_vals + (int64_t)(2 * s) * o->nsrc);
    apply_transparent(o, 0);
    if (o->incident)
      oracle_step_tfsf(o->incident, 1, aux_vals + (int64_t)(2 * s) * o->incident->nsrc, NULL);
    for (int c = 0; c < 3; ++c) chatter(o, c);
    for (int c = 3; c < 6; ++c)
      for (int k = 0; k < o->nupd[c]; ++k) run_updater(o, &o->upd[c][k]);
    apply_sources(o, 1, src_vals + (int64_t)(2 * s + 1) * o->nsrc);
    apply_transparent(o, 1);
  }
  return 0;
}

int oracle_step(oracle* o, int nsteps, const double* src_vals) {
  return oracle_step_tfsf(o, nsteps, src_vals, NULL);
}

/* ---- complex fields (Bloch boundary) --------------------------------------
 * The update coefficients are real (src/pw_*.hh keep them double for T =
 * complex<double>), so the real and imaginary parts evolve independently
 * except in the ghost copies, which multiply the source plane by the Bloch
 * phase exp(1j k_a (x_dest - x_src)) (gmes/fdtd.py:811-1097), the two
 * curl axes in order.  The reference forms phase * plane with numpy's
 * complex multiply, which (SIMD build, x86-64 with AVX-512 where the golden
 * vectors were made) evaluates re = fma(pr, vr, -(pi vi)),
 * im = fma(pr, vi, pi vr); the same fused form is used here. */
static void chatter_complex(oracle* re, oracle* im, int c) {
  if (!(re->active & (1 << c))) return;
  const int own = c % 3;
  const int ax[2] = {(own + 1) % 3, (own + 2) % 3};
  const int64_t* sh = re->sh[c];
  for (int h = 0; h < 2; ++h) {
    const int axis = ax[h];
    const int64_t last = sh[axis] - 1;
    const int64_t dst = c < 3 ? last : 0, src = c < 3 ? 0 : last;
    const double pr = re->phase[c][h][0], pi = re->phase[c][h][1];
    const int p = (axis + 1) % 3, q = (axis + 2) % 3;
    for (int64_t u = 0; u < sh[p]; ++u)
      for (int64_t v = 0; v < sh[q]; ++v) {
        int64_t x[3], y[3];
        x[axis] = dst; x[p] = u; x[q] = v;
        y[axis] = src; y[p] = u; y[q] = v;
        const int64_t xo = (x[0] * sh[1] + x[1]) * sh[2] + x[2];
        const int64_t yo = (y[0] * sh[1] + y[1]) * sh[2] + y[2];
        const double vr = re->f[c][yo], vi = im->f[c][yo];
        re->f[c][xo] = fma(pr, vr, -(pi * vi));
        im->f[c][xo] = fma(pr, vi, pi * vr);
      }
  }
}

int oracle_set_complex(oracle* re, oracle* im, const double* phase) {
  re->imag = im;
  memcpy(re->phase, phase, sizeof(re->phase));
  return 0;
}

/* vals_re / vals_im: [nsteps][2][nsrc] real and imaginary source values;
   aux_re / aux_im the same for the TFSF incident-field grid (a complex
   pair itself), or NULL. */
int oracle_step_complex(oracle* re, int nsteps, const double* vals_re, const double* vals_im,
                        const double* aux_re, const double* aux_im) {
  oracle* im = re->imag;
  if (!im) return -1;
  if (re->incident && (!aux_re || !aux_im || !re->incident->imag)) return -1;
  for (int s = 0; s < nsteps; ++s) {
    for (int c = 3; c < 6; ++c) chatter_complex(re, im, c);
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < re->nupd[c]; ++k) {
        run_updater(re, &re->upd[c][k]);
        run_updater(im, &im->upd[c][k]);
      }
    apply_sources(re, 0, vals_re + (int64_t)(2 * s) * re->nsrc);
    apply_sources(im, 0, vals_im + (int64_t)(2 * s) * im->nsrc);
    apply_transparent(re, 0);
    apply_transparent(im, 0);
    if (re->incident) {
      const int64_t na = (int64_t)(2 * s) * re->incident->nsrc;
      oracle_step_complex(re->incident, 1, aux_re + na, aux_im + na, NULL, NULL);
    }
    for (int c = 0; c < 3; ++c) chatter_complex(re, im, c);
    for (int c = 3; c < 6; ++c)
      for (int k = 0; k < re->nupd[c]; ++k) {
        run_updater(re, &re->upd[c][k]);
        run_updater(im, &im->upd[c][k]);
      }
    apply_sources(re, 1, vals_re + (int64_t)(2 * s + 1) * re->nsrc);
    apply_sources(im, 1, vals_im + (int64_t)(2 * s + 1) * im->nsrc);
    apply_transparent(re, 1);
    apply_transparent(im, 1);
  }
  return 0;
}

/* ---- reset and per-point permittivity ------------------------------------ */

/* Zero every field and every per-point state (psi, d, ADE). */
int oracle_reset(oracle* o) {
  if (o->incident) oracle_reset(o->incident);
  for (int c = 0; c < 6; ++c) {
    memset(o->f[c], 0, sizeof(double) * (size_t)(o->sh[c][0] * o->sh[c][1] * o->sh[c][2]));
    for (int k = 0; k < o->nupd[c]; ++k) {
      updater* u = &o->upd[c][k];
      for (int64_t t = 0; t < u->count; ++t) {
        if (u->kind == K_CPML) { ((p_cpml*)u->pts)[t].psi1 = 0; ((p_cpml*)u->pts)[t].psi2 = 0; }
        else if (u->kind == K_UPML) ((p_upml*)u->pts)[t].d = 0;
        else if (u->kind == K_DRUDE || u->kind == K_LORENTZ || u->kind == K_DCP ||
                 u->kind == K_DCP_PLRC)
          memset(((p_ade*)u->pts)[t].st, 0, sizeof(((p_ade*)u->pts)[t].st));
      }
    }
  }
  return 0;
}

/* Give the dielectric points at offsets off[0..n) of component c their own
   permittivity (the reference keeps eps per point in DielectricElectricParam,
   src/pw_dielectric.hh:18-30).  Returns -1 if an offset is not a dielectric
   point of c. */
int oracle_set_eps(oracle* o, int c, int n, const int64_t* off, const double* eps) {
  for (int q = 0; q < n; ++q) {
    int found = 0;
    for (int k = 0; k < o->nupd[c] && !found; ++k) {
      updater* u = &o->upd[c][k];
      if (u->kind != K_DIEL) continue;
      p_diel* pts = (p_diel*)u->pts;
      for (int64_t t = 0; t < u->count; ++t)
        if (pts[t].off == off[q]) { pts[t].eps = eps[q]; found = 1; break; }
    }
    if (!found) return -1;
  }
  return 0;
}

/* ---- discrete adjoint (test infrastructure; the reference has none) ------- *
 * J = dt * sum_{n=1..N} sum_m F_{c_m}[off_m]^2 after each step n.  The
 * backward sweep applies the transpose of every operation of oracle_step in
 * reverse order, in scatter form on the full arrays: H sources, H updaters,
 * the E ghost-plane copies (plane by plane, last copy first), E sources,
 * E updaters (with the gradient of the design points), the H ghost copies.
 * Supported classes: Dielectric, CPML (and Dummy).  Serial. */
#define LAT(L, c, i, j, k) (L[c][((int64_t)(i) * o->sh[c][1] + (j)) * o->sh[c][2] + (k)])

static void scatter_diffs(const oracle* o, double** L, int c, const int x[3], double w1,
                          double w2) {
  const int own = c % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  if (c < 3) {
    const int in1 = 3 + a2, in2 = 3 + a1;
    int p[3] = {x[0], x[1], x[2]}, q[3];
    p[own] += 1;
    if (o->active & (1 << in1)) {
      memcpy(q, p, sizeof(q)); q[a1] += 1;
      LAT(L, in1, q[0], q[1], q[2]) += w1;
      LAT(L, in1, p[0], p[1], p[2]) -= w1;
    }
    if (o->active & (1 << in2)) {
      memcpy(q, p, sizeof(q)); q[a2] += 1;
      LAT(L, in2, q[0], q[1], q[2]) += w2;
      LAT(L, in2, p[0], p[1], p[2]) -= w2;
    }
  } else {
    const int in1 = a2, in2 = a1;
    if (o->active & (1 << in1)) {
      int u[3] = {x[0], x[1], x[2]}; u[a2] -= 1;
      int v[3] = {u[0], u[1], u[2]}; v[a1] -= 1;
      LAT(L, in1, u[0], u[1], u[2]) += w1;
      LAT(L, in1, v[0], v[1], v[2]) -= w1;
    }
    if (o->active & (1 << in2)) {
      int u[3] = {x[0], x[1], x[2]}; u[a1] -= 1;
      int v[3] = {u[0], u[1], u[2]}; v[a2] -= 1;
      LAT(L, in2, u[0], u[1], u[2]) += w2;
      LAT(L, in2, v[0], v[1], v[2]) -= w2;
    }
  }
}

/* Transpose of one updater; lpsi holds 2 psi adjoints per CPML point. */
static void adjoint_updater(const oracle* o, double** L, const updater* u, double* lpsi) {
  const int c = u->comp;
  const int own = c % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  const double d1 = o->dr[a1], d2 = o->dr[a2], dt = o->dt;
  const int E = c < 3;
  if (u->kind == K_DIEL) {
    const p_diel* pts = (const p_diel*)u->pts;
    for (int64_t t = 0; t < u->count; ++t) {
      const double lf = L[c][pts[t].off];
      const double s = dt / pts[t].eps;
      if (E)
        scatter_diffs(o, L, c, pts[t].idx, s / d1 * lf, -s / d2 * lf);
      else
        scatter_diffs(o, L, c, pts[t].idx, -s / d1 * lf, s / d2 * lf);
    }
  } else if (u->kind == K_CPML) {
    const p_cpml* pts = (const p_cpml*)u->pts;
    for (int64_t t = 0; t < u->count; ++t) {
      const p_cpml* p = &pts[t];
      const double lf = L[c][p->off];
      const double s = E ? dt / p->eps : -dt / p->eps;
      const double L1 = lpsi[2 * t] + s * lf;
      const double L2 = lpsi[2 * t + 1] - s * lf;
      const double w1 = p->c1 / d1 * L1 + s / (d1 * p->k1) * lf;
      const double w2 = p->c2 / d2 * L2 - s / (d2 * p->k2) * lf;
      lpsi[2 * t] = p->b1 * L1;
      lpsi[2 * t + 1] = p->b2 * L2;
      scatter_diffs(o, L, c, p->idx, w1, w2);
    }
  }
}

static void adjoint_copy_plane(const oracle* o, double** L, int c, int axis, int64_t dst,
                               int64_t src) {
  const int64_t* sh = o->sh[c];
  const int p = (axis + 1) % 3, q = (axis + 2) % 3;
  for (int64_t a = 0; a < sh[p]; ++a)
    for (int64_t b = 0; b < sh[q]; ++b) {
      int64_t x[3], y[3];
      x[axis] = dst; x[p] = a; x[q] = b;
      y[axis] = src; y[p] = a; y[q] = b;
      const double v = LAT(L, c, x[0], x[1], x[2]);
      LAT(L, c, x[0], x[1], x[2]) = 0;
      LAT(L, c, y[0], y[1], y[2]) += v;
    }
}

static void adjoint_chatter(const oracle* o, double** L, int c) {
  if (!(o->active & (1 << c))) return;
  const int own = c % 3;
  const int ax[2] = {(own + 1) % 3, (own + 2) % 3};
  for (int h = 1; h >= 0; --h) {
    const int64_t last = o->sh[c][ax[h]] - 1;
    if (c < 3)
      adjoint_copy_plane(o, L, c, ax[h], last, 0);
    else
      adjoint_copy_plane(o, L, c, ax[h], 0, last);
  }
}

static void adjoint_sources(const oracle* o, double** L, int side) {
  for (int q = 0; q < o->nsrc; ++q) {
    const int c = o->src_comp[q];
    if ((c < 3) != (side == 0) || o->src_mode[q] != 0) continue;
    L[c][o->src_off[q]] = 0;
  }
}

static const p_diel* find_diel(const oracle* o, int c, int64_t off) {
  for (int k = 0; k < o->nupd[c]; ++k) {
    const updater* u = &o->upd[c][k];
    if (u->kind != K_DIEL) continue;
    const p_diel* pts = (const p_diel*)u->pts;
    for (int64_t t = 0; t < u->count; ++t)
      if (pts[t].off == off) return &pts[t];
  }
  return NULL;
}

/* Runs nsteps forward from the current state, recording the monitor and
   the design points' curls, then (grad != NULL) the backward sweep.
   Returns 0, -1 for an unsupported class, -2 for a design point that is not
   a dielectric E point, -3 on allocation failure. */
int oracle_adjoint(oracle* o, int nsteps, const double* src_vals, int nmon, const int* mcomp,
                   const int64_t* moff, int ndes, const int* dcomp, const int64_t* doff,
                   double* J, double* grad) {
  if (o->incident) return -1;
  for (int c = 0; c < 6; ++c)
    for (int k = 0; k < o->nupd[c]; ++k)
      if (o->upd[c][k].kind != K_DIEL && o->upd[c][k].kind != K_CPML) return -1;
  const p_diel** dp = (const p_diel**)calloc((size_t)(ndes ? ndes : 1), sizeof(p_diel*));
  double* mon = (double*)calloc((size_t)nsteps * (nmon ? nmon : 1), sizeof(double));
  double* curl = (double*)calloc((size_t)nsteps * (ndes ? ndes : 1), sizeof(double));
  if (!dp || !mon || !curl) { free(dp); free(mon); free(curl); return -3; }
  for (int q = 0; q < ndes; ++q) {
    dp[q] = dcomp[q] < 3 ? find_diel(o, dcomp[q], doff[q]) : NULL;
    if (!dp[q]) { free(dp); free(mon); free(curl); return -2; }
  }
  double acc = 0;
  for (int s = 0; s < nsteps; ++s) {
    for (int c = 3; c < 6; ++c) chatter(o, c);
    for (int q = 0; q < ndes; ++q) {
      const int c = dcomp[q], own = c % 3;
      double D1, D2;
      diffs(o, c, dp[q]->idx, &D1, &D2);
      curl[(int64_t)s * ndes + q] = D1 / o->dr[(own + 1) % 3] - D2 / o->dr[(own + 2) % 3];
    }
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < o->nupd[c]; ++k) run_updater(o, &o->upd[c][k]);
    apply_sources(o, 0, src_vals + (int64_t)(2 * s) * o->nsrc);
    for (int c = 0; c < 3; ++c) chatter(o, c);
    for (int c = 3; c < 6; ++c)
      for (int k = 0; k < o->nupd[c]; ++k) run_updater(o, &o->upd[c][k]);
    apply_sources(o, 1, src_vals + (int64_t)(2 * s + 1) * o->nsrc);
    double js = 0;
    for (int m = 0; m < nmon; ++m) {
      const double v = o->f[mcomp[m]][moff[m]];
      mon[(int64_t)s * nmon + m] = v;
      js += v * v;
    }
    acc += js;
  }
  *J = o->dt * acc;
  if (grad == NULL) { free(dp); free(mon); free(curl); return 0; }

  double* L[6];
  double* lpsi[6][MAXCLS];
  int fail = 0;
  memset(lpsi, 0, sizeof(lpsi));
  for (int c = 0; c < 6; ++c) {
    L[c] = (double*)calloc((size_t)(o->sh[c][0] * o->sh[c][1] * o->sh[c][2]), sizeof(double));
    if (!L[c]) fail = 1;
    for (int k = 0; k < o->nupd[c]; ++k) {
      lpsi[c][k] = (double*)calloc((size_t)(2 * o->upd[c][k].count + 1), sizeof(double));
      if (!lpsi[c][k]) fail = 1;
    }
  }
  for (int q = 0; q < ndes; ++q) grad[q] = 0;
  for (int s = nsteps - 1; s >= 0 && !fail; --s) {
    for (int m = 0; m < nmon; ++m) L[mcomp[m]][moff[m]] += 2 * o->dt * mon[(int64_t)s * nmon + m];
    adjoint_sources(o, L, 1);
    for (int c = 3; c < 6; ++c)
      for (int k = 0; k < o->nupd[c]; ++k) adjoint_updater(o, L, &o->upd[c][k], lpsi[c][k]);
    for (int c = 2; c >= 0; --c) adjoint_chatter(o, L, c);
    adjoint_sources(o, L, 0);
    for (int q = 0; q < ndes; ++q) {
      const double eps = dp[q]->eps;
      grad[q] += L[dcomp[q]][doff[q]] * (-o->dt / (eps * eps)) * curl[(int64_t)s * ndes + q];
    }
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < o->nupd[c]; ++k) adjoint_updater(o, L, &o->upd[c][k], lpsi[c][k]);
    for (int c = 5; c >= 3; --c) adjoint_chatter(o, L, c);
  }
  for (int c = 0; c < 6; ++c) {
    free(L[c]);
    for (int k = 0; k < o->nupd[c]; ++k) free(lpsi[c][k]);
  }
  free(dp); free(mon); free(curl);
  return fail ? -3 : 0;
}

int oracle_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_destroy(oracle* o) {
  if (!o) return;
  for (int c = 0; c < 6; ++c) {
    free(o->f[c]);
    if (o->upd[c]) {
      for (int k = 0; k < o->nupd[c]; ++k) free(o->upd[c][k].pts);
      free(o->upd[c]);
    }
  }
  free(o->src_comp); free(o->src_mode); free(o->src_off);
  free(o->tf_comp); free(o->tf_nface); free(o->tf_off); free(o->tf_coef);
  free(o->tf_r0); free(o->tf_r1); free(o->tf_sample);
  free(o);
}
