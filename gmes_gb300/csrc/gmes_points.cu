// Point-list updaters: the reference's PwMaterial operator interface
// (src/pw_material.hh:49-117, update_all at :66-73) on the GPU.
//
// An updater object of the reference holds an array-of-structs list of
// attached points, each with its own parameters and state, and updates them
// in place on numpy arrays it borrows for the call.  Here the points of one
// updater are a structure of arrays in device memory: per point its index,
// its parameters and its state; one thread updates one point, in the
// reference's operation order (FP64, no contraction, IEEE division), the
// curl differences read through the reference's field_at() rule: an input
// array whose extent along the component's "collapsed" axis is 1 reads as
// its element 0 (src/cpp23_support.hh:52-74).
//
// Update expressions: src/pw_dielectric.hh:118-371, src/pw_cpml.hh:115-447,
// src/pw_upml.hh:113-432, src/pw_drude.hh:89-151, src/pw_lorentz.hh:96-157,
// src/pw_dcp.hh:105-225 (ADE) and 466-583 (PLRC), src/pw_const.hh.
#include "gmes_internal.cuh"

namespace gmes {
namespace {

__device__ __forceinline__ double ADD(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double SUB(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double MUL(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double DIV(double a, double b) { return __ddiv_rn(a, b); }

struct PointsDev {
  int32_t comp, kind, npoints, nparam, nstate, npole, ncp, plane;
  const int32_t* idx;    // [npoints][3]
  const double* param;   // [npoints][nparam]
  double* state;         // [npoints][nstate]
  int64_t sh[3][3];      // shapes of inplace, in1, in2
  double* f;             // inplace plane
  const double* in[2];   // in1, in2 planes
  double d1, d2, dt;
};

// field_at(): element 0 when the array is collapsed along `axis`; reads
// outside the array (the reference does not guard them) give 0.
__device__ __forceinline__ double read_at(const double* a, const int64_t sh[3], int axis, int i,
                                          int j, int k) {
  if (sh[axis] == 1) return a[0];
  if (i < 0 || j < 0 || k < 0 || i >= sh[0] || j >= sh[1] || k >= sh[2]) return 0.0;
  return a[((int64_t)i * sh[1] + j) * sh[2] + k];
}

__global__ void k_points(const PointsDev p) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= p.npoints) return;
  const int c = p.comp, own = c % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
  const bool E = c < 3;
  const int x[3] = {p.idx[3 * t], p.idx[3 * t + 1], p.idx[3 * t + 2]};
  // target element: field_at's collapsed axis of the component (own + 1);
  // src/pw_const.hh collapses only an array of one element
  double* fp;
  const bool collapsed = p.kind == GMES_KIND_CONST
                             ? (p.sh[0][0] == 1 && p.sh[0][1] == 1 && p.sh[0][2] == 1)
                             : p.sh[0][a1] == 1;
  if (collapsed) {
    fp = p.f;
  } else {
    // the host validates indices before the call; a caller that did not
    // gets out-of-range points skipped, never written
    for (int a = 0; a < 3; ++a)
      if (x[a] < 0 || x[a] >= p.sh[0][a]) return;
    fp = p.f + ((int64_t)x[0] * p.sh[0][1] + x[1]) * p.sh[0][2] + x[2];
  }
  // curl differences, bound as FDTD.update_e?/h? binds (in1, in2)
  const int ax1 = (a2 + 1) % 3, ax2 = (a1 + 1) % 3;  // collapsed axes of in1, in2
  double D1, D2;
  if (E) {
    int q[3] = {x[0], x[1], x[2]};
    q[own] += 1;
    int r[3] = {q[0], q[1], q[2]};
    r[a1] += 1;
    D1 = SUB(read_at(p.in[0], p.sh[1], ax1, r[0], r[1], r[2]),
             read_at(p.in[0], p.sh[1], ax1, q[0], q[1], q[2]));
    int s[3] = {q[0], q[1], q[2]};
    s[a2] += 1;
    D2 = SUB(read_at(p.in[1], p.sh[2], ax2, s[0], s[1], s[2]),
             read_at(p.in[1], p.sh[2], ax2, q[0], q[1], q[2]));
  } else {
    int u[3] = {x[0], x[1], x[2]};
    u[a2] -= 1;
    int v[3] = {u[0], u[1], u[2]};
    v[a1] -= 1;
    D1 = SUB(read_at(p.in[0], p.sh[1], ax1, u[0], u[1], u[2]),
             read_at(p.in[0], p.sh[1], ax1, v[0], v[1], v[2]));
    int w[3] = {x[0], x[1], x[2]};
    w[a1] -= 1;
    int z[3] = {w[0], w[1], w[2]};
    z[a2] -= 1;
    D2 = SUB(read_at(p.in[1], p.sh[2], ax2, w[0], w[1], w[2]),
             read_at(p.in[1], p.sh[2], ax2, z[0], z[1], z[2]));
  }
  const double* pr = p.param + (int64_t)t * p.nparam;
  double* st = p.state + (int64_t)t * p.nstate;
  const double d1 = p.d1, d2 = p.d2, dt = p.dt;
  const double F = *fp;
  switch (p.kind) {
    case GMES_KIND_DIELECTRIC: {  // pr: eps
      const double X = E ? SUB(DIV(D1, d1), DIV(D2, d2)) : SUB(DIV(D2, d2), DIV(D1, d1));
      *fp = ADD(F, MUL(DIV(dt, pr[0]), X));
      return;
    }
    case GMES_KIND_CPML: {  // pr: eps, b1, b2, c1, c2, kappa1, kappa2; st: psi1, psi2
      st[0] = ADD(MUL(pr[1], st[0]), DIV(MUL(pr[3], D1), d1));
      st[1] = ADD(MUL(pr[2], st[1]), DIV(MUL(pr[4], D2), d2));
      const double X =
          SUB(ADD(SUB(DIV(DIV(D1, d1), pr[5]), DIV(DIV(D2, d2), pr[6])), st[0]), st[1]);
      const double inc = MUL(DIV(dt, pr[0]), X);
      *fp = E ? ADD(F, inc) : SUB(F, inc);
      return;
    }
    case GMES_KIND_UPML: {  // pr: eps, c1..c6; st: d (E) or b (H)
      const double curl = SUB(DIV(D1, d1), DIV(D2, d2));
      const double old = st[0];
      st[0] = E ? ADD(MUL(pr[1], old), MUL(pr[2], curl)) : SUB(MUL(pr[1], old), MUL(pr[2], curl));
      *fp = ADD(MUL(pr[3], F), DIV(MUL(pr[4], SUB(MUL(pr[5], st[0]), MUL(pr[6], old))), pr[0]));
      return;
    }
    case GMES_KIND_CONST: {  // pr: value (this plane's part)
      *fp = pr[0];
      return;
    }
    default:
      break;
  }
  if (!E) return;
  const double curl = SUB(DIV(D1, d1), DIV(D2, d2));
  const int P = p.npole, Q = p.ncp;
  if (p.kind == GMES_KIND_DRUDE || p.kind == GMES_KIND_LORENTZ) {
    // pr: a[P][3], c[3]; st: q_now[P], q_new[P]
    const double* a = pr;
    const double* cc = pr + 3 * P;
    double sum = 0.0;
    for (int i = 0; i < P; ++i) {
      const double q_old = st[i], q_now = st[P + i];
      const double q_new = ADD(ADD(MUL(a[3 * i], q_old), MUL(a[3 * i + 1], q_now)),
                               MUL(a[3 * i + 2], F));
      st[i] = q_now;
      st[P + i] = q_new;
      sum = ADD(sum, SUB(q_new, q_now));
    }
    *fp = ADD(ADD(MUL(cc[0], curl), MUL(cc[1], sum)), MUL(cc[2], F));
    return;
  }
  if (p.kind == GMES_KIND_DCP) {
    // pr: a[P][3], b[Q][5], c[4]; st: e_old, q_old[P], q_now[P], p_old[Q], p_now[Q]
    const double* a = pr;
    const double* b = pr + 3 * P;
    const double* cc = b + 5 * Q;
    double* qo = st + 1;
    double* qn = st + 1 + P;
    double* po = st + 1 + 2 * P;
    double* pn = st + 1 + 2 * P + Q;
    const double e_old = st[0];
    double sd = 0.0, sc = 0.0;
    for (int i = 0; i < P; ++i)
      sd = ADD(sd, SUB(MUL(SUB(1.0, a[3 * i + 1]), qn[i]), MUL(a[3 * i], qo[i])));
    for (int i = 0; i < Q; ++i)
      sc = ADD(sc, SUB(MUL(SUB(1.0, b[5 * i + 1]), pn[i]), MUL(b[5 * i], po[i])));
    const double e_new = ADD(ADD(ADD(MUL(cc[0], curl), MUL(cc[1], ADD(sd, sc))),
                                 MUL(cc[2], e_old)), MUL(cc[3], F));
    const double esum = ADD(ADD(e_old, MUL(2.0, F)), e_new);
    for (int i = 0; i < P; ++i) {
      const double q_new = ADD(ADD(MUL(a[3 * i], qo[i]), MUL(a[3 * i + 1], qn[i])),
                               MUL(a[3 * i + 2], esum));
      qo[i] = qn[i];
      qn[i] = q_new;
    }
    for (int i = 0; i < Q; ++i) {
      const double* bb = b + 5 * i;
      const double p_new = ADD(ADD(ADD(ADD(MUL(bb[0], po[i]), MUL(bb[1], pn[i])), MUL(bb[2], e_old)),
                                   MUL(bb[3], F)), MUL(bb[4], e_new));
      po[i] = pn[i];
      pn[i] = p_new;
    }
    st[0] = F;
    *fp = e_new;
    return;
  }
  if (p.kind == GMES_KIND_DCP_PLRC) {
    // pr: a[P][3], b[Q][6] (b0, b1, b2 as re/im), c[3]; st: psi_dp[P], psi_cp[Q][2]
    const double* a = pr;
    const double* b = pr + 3 * P;
    const double* cc = b + 6 * Q;
    double sdp = 0.0, scp = 0.0;
    for (int i = 0; i < P; ++i) sdp = ADD(sdp, st[i]);
    for (int i = 0; i < Q; ++i) scp = ADD(scp, st[P + 2 * i]);
    const double e_new =
        ADD(ADD(MUL(cc[0], curl), MUL(cc[1], F)), MUL(cc[2], ADD(sdp, scp)));
    for (int i = 0; i < P; ++i)
      st[i] = ADD(ADD(MUL(a[3 * i], e_new), MUL(a[3 * i + 1], F)), MUL(a[3 * i + 2], st[i]));
    for (int i = 0; i < Q; ++i) {
      const double* bb = b + 6 * i;
      const double r = st[P + 2 * i], m = st[P + 2 * i + 1];
      st[P + 2 * i] = ADD(ADD(MUL(bb[0], e_new), MUL(bb[2], F)), SUB(MUL(bb[4], r), MUL(bb[5], m)));
      st[P + 2 * i + 1] =
          ADD(ADD(MUL(bb[1], e_new), MUL(bb[3], F)), ADD(MUL(bb[4], m), MUL(bb[5], r)));
    }
    *fp = e_new;
  }
}

}  // namespace

cudaError_t launch_points(const gmes_points& g, void* inplace, const void* in1, const void* in2,
                          double d1, double d2, double dt, cudaStream_t s) {
  const int planes = g.cmplx ? 2 : 1;
  for (int part = 0; part < planes; ++part) {
    PointsDev p;
    p.comp = g.comp;
    p.kind = g.kind;
    p.npoints = g.npoints;
    p.nparam = g.nparam;
    p.nstate = g.nstate;
    p.npole = g.npole;
    p.ncp = g.ncp;
    p.plane = part;
    p.idx = g.idx;
    p.param = g.param + (int64_t)part * g.npoints * g.nparam;
    p.state = g.state + (int64_t)part * g.npoints * g.nstate;
    int64_t n[3];
    for (int a = 0; a < 3; ++a) {
      for (int b = 0; b < 3; ++b) p.sh[a][b] = g.shape[a][b];
      n[a] = g.shape[a][0] * g.shape[a][1] * g.shape[a][2];
    }
    p.f = static_cast<double*>(inplace) + part * n[0];
    p.in[0] = static_cast<const double*>(in1) + part * n[1];
    p.in[1] = static_cast<const double*>(in2) + part * n[2];
    p.d1 = d1;
    p.d2 = d2;
    p.dt = dt;
    if (g.npoints > 0) k_points<<<(g.npoints + 127) / 128, 128, 0, s>>>(p);
  }
  return cudaGetLastError();
}

}  // namespace gmes
