// extern "C" entry points of libgmes_gb300.so: argument validation, the
// coefficient-block layout, host<->device staging and error reporting.
// Status codes follow the reference binding's exception classes
// (src/pw_material.i:23-33): ValueError, IndexError, RuntimeError.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "gmes_internal.cuh"

namespace gmes {
namespace {

thread_local std::string g_last_error;

gmes_status fail(gmes_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return st;
}

gmes_status cuda_fail(cudaError_t e, const char* what) {
  return fail(GMES_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

int elem_size(int32_t precision) {
  switch (precision) {
    case GMES_FP64:
    case GMES_FP64_STRICT:
    case GMES_DF64:
      return 8;
    case GMES_FP32:
      return 4;
    default:
      return 0;
  }
}

// Validate everything that can be checked without touching device memory.
gmes_status check_desc(const gmes_grid_desc* g, bool need_buffers) {
  if (g == nullptr) return fail(GMES_ERR_VALUE, "grid descriptor is NULL");
  if (g->abi_version != GMES_ABI_VERSION)
    return fail(GMES_ERR_VALUE, "ABI version mismatch: descriptor %d, library %d",
                g->abi_version, GMES_ABI_VERSION);
  if (elem_size(g->precision) == 0)
    return fail(GMES_ERR_VALUE, "unknown precision %d", g->precision);
  for (int a = 0; a < 3; ++a) {
    if (g->n[a] < 1) return fail(GMES_ERR_VALUE, "grid size n[%d] = %d must be >= 1", a, g->n[a]);
    if (!(g->dr[a] > 0) || !std::isfinite(g->dr[a]))
      return fail(GMES_ERR_VALUE, "cell size dr[%d] must be positive and finite", a);
  }
  if (!(g->dt > 0) || !std::isfinite(g->dt)) return fail(GMES_ERR_VALUE, "dt must be positive");
  if ((g->active & ~63) != 0 || (g->active & 7) == 0 || (g->active & 56) == 0)
    return fail(GMES_ERR_VALUE, "active mask 0x%x must name at least one E and one H component",
                g->active);
  if (g->npml < 0 || g->npml > GMES_MAX_PML)
    return fail(GMES_ERR_VALUE, "npml = %d outside [0, %d]", g->npml, GMES_MAX_PML);
  if (g->nsrc < 0 || g->nparam < 0 || g->src_steps < 0)
    return fail(GMES_ERR_VALUE, "negative nsrc / nparam / src_steps");
  for (int c = 0; c < 6; ++c) {
    const bool act = (g->active >> c) & 1;
    if (g->nclass[c] < 0 || g->nclass[c] > GMES_MAX_CLASSES)
      return fail(GMES_ERR_VALUE, "nclass[%d] = %d outside [0, %d]", c, g->nclass[c],
                  GMES_MAX_CLASSES);
    if (act && g->nclass[c] < 1)
      return fail(GMES_ERR_VALUE, "active component %d has no classes", c);
    if (g->naux[c] < 0 || g->naux[c] > 1 + 4 * GMES_MAX_POLES)
      return fail(GMES_ERR_VALUE, "naux[%d] = %d out of range", c, g->naux[c]);
    if (need_buffers) {
      if (g->field[c] == nullptr) return fail(GMES_ERR_VALUE, "field[%d] is NULL", c);
      if (act && g->cls[c] == nullptr) return fail(GMES_ERR_VALUE, "cls[%d] is NULL", c);
      if (act && g->naux[c] > 0 && g->aux[c] == nullptr)
        return fail(GMES_ERR_VALUE, "aux[%d] is NULL but naux[%d] = %d", c, c, g->naux[c]);
    }
  }
  if (need_buffers && g->coef == nullptr) return fail(GMES_ERR_VALUE, "coef is NULL");
  if (need_buffers && g->nsrc > 0 && (g->src == nullptr || g->src_val == nullptr))
    return fail(GMES_ERR_VALUE, "nsrc > 0 but src or src_val is NULL");
  if ((g->flags & GMES_FLAG_COMPLEX) && g->precision != GMES_FP64 &&
      g->precision != GMES_FP64_STRICT)
    return fail(GMES_ERR_VALUE, "complex grids support fp64 and fp64_strict only");
  if (g->ntfsf < 0) return fail(GMES_ERR_VALUE, "ntfsf = %d must be >= 0", g->ntfsf);
  if (g->nprobe < 0 || g->probe_steps < 0)
    return fail(GMES_ERR_VALUE, "negative nprobe / probe_steps");
  if (need_buffers && g->nprobe > 0 && (g->probe == nullptr || g->probe_val == nullptr))
    return fail(GMES_ERR_VALUE, "nprobe > 0 but probe or probe_val is NULL");
  if (need_buffers && g->ntfsf > 0) {
    const gmes_grid_desc* a = g->incident;
    if (g->tfsf == nullptr || a == nullptr)
      return fail(GMES_ERR_VALUE, "ntfsf > 0 but tfsf or the incident-field grid is NULL");
    if (a->abi_version != GMES_ABI_VERSION || a->precision != g->precision || a->dt != g->dt)
      return fail(GMES_ERR_VALUE, "the incident-field grid must share precision and dt");
    if ((a->active & ((1 << GMES_EX) | (1 << GMES_HY))) != ((1 << GMES_EX) | (1 << GMES_HY)) ||
        a->incident != nullptr || a->ntfsf != 0)
      return fail(GMES_ERR_VALUE, "the incident-field grid must be a plain Ex/Hy grid");
    if ((a->flags & GMES_FLAG_COMPLEX) != (g->flags & GMES_FLAG_COMPLEX))
      return fail(GMES_ERR_VALUE, "the incident-field grid must be complex iff the grid is");
  }
  return GMES_OK;
}

// The incident-field grid's own checks (without recursion into TFSF).
gmes_status check_aux(const gmes_grid_desc* g) {
  if (g->ntfsf == 0 || g->incident == nullptr) return GMES_OK;
  gmes_status st = check_desc(g->incident, true);
  if (st != GMES_OK) return fail(st, "incident-field grid: %s", g_last_error.c_str());
  return GMES_OK;
}

}  // namespace

GridDev make_grid_dev(const gmes_grid_desc& g) {
  GridDev d;
  std::memset(&d, 0, sizeof(d));
  for (int a = 0; a < 3; ++a) {
    d.n[a] = g.n[a];
    d.dr[a] = g.dr[a];
    d.rdr[a] = make_coef(1.0 / g.dr[a]);
  }
  d.dt = g.dt;
  d.active = g.active;
  d.nsrc = g.nsrc;
  d.pointwise = (g.flags & GMES_FLAG_POINTWISE) ? 1 : 0;
  const CoefLayout L = coef_layout(g);
  char* base = static_cast<char*>(g.coef);
  for (int c = 0; c < 6; ++c) {
    int64_t sh[3];
    comp_shape(g.n, g.active, c, sh);
    for (int a = 0; a < 3; ++a) d.sh[c][a] = sh[a];
    d.st[c][0] = sh[1] * sh[2];
    d.st[c][1] = sh[2];
    d.npts[c] = sh[0] * sh[1] * sh[2];
    d.naux[c] = g.naux[c];
    d.f[c] = g.field[c];
    d.cls[c] = g.cls[c];
    d.aux[c] = g.aux[c];
    d.tab[c] = reinterpret_cast<const ClassCoef*>(base + L.class_tab[c]);
    d.pool[c] = reinterpret_cast<const Coef*>(base + L.pool[c]);
    for (int p = 0; p < GMES_MAX_PML; ++p)
      for (int a = 0; a < 3; ++a)
        d.prof[p][c][a] = reinterpret_cast<const Coef*>(base + L.prof[p][c][a]);
  }
  const int64_t n1 = g.n[1], n2 = g.n[2];
  d.fst[0][0] = (n1 + 1) * (n2 + 1);
  d.fst[0][1] = n2 + 1;
  d.fst[1][0] = n1 * (n2 + 1);
  d.fst[1][1] = n2 + 1;
  d.fst[2][0] = (n1 + 1) * n2;
  d.fst[2][1] = n2;
  d.src = g.src;
  d.src_val = g.src_val;
  std::memcpy(d.phase, g.bloch_phase, sizeof(d.phase));
  if (g.nprobe > 0) {
    d.probe = g.probe;
    d.probe_val = g.probe_val;
    d.nprobe = g.nprobe;
  }
  if (g.ntfsf > 0 && g.incident != nullptr) {
    d.tfsf = g.tfsf;
    d.ntfsf = g.ntfsf;
    d.tf_field[0] = g.incident->field[GMES_HY];
    d.tf_field[1] = g.incident->field[GMES_EX];
    for (int k = 0; k < 2; ++k) {
      int64_t sh[3];
      comp_shape(g.incident->n, g.incident->active, k == 0 ? GMES_HY : GMES_EX, sh);
      d.tf_npts[k] = sh[0] * sh[1] * sh[2];
    }
  }
  return d;
}

// Tile numbering of a grid with blocks of 2^l cells along k.
TileDiv tile_div(int l, const int32_t n[3]) {
  TileDiv t;
  std::memset(&t, 0, sizeof(t));
  const int64_t bx = int64_t(1) << l, by = kBatchThreads / bx;
  t.bxl = l;
  t.nkb = (uint32_t)((n[2] + bx - 1) / bx);
  t.plane = t.nkb * (uint32_t)((n[1] + by - 1) / by);
  tile_div_of(t.nkb, t.m_nkb, t.s_nkb);
  tile_div_of(t.plane, t.m_plane, t.s_plane);
  return t;
}

struct BatchLayout {
  int64_t jobs, tile_prefix, td, steps, ghost_prefix, src_prefix, total;
};

BatchLayout batch_layout(int32_t njobs) {
  BatchLayout L;
  int64_t off = 0;
  L.jobs = off;
  off = align256(off + (int64_t)njobs * (int64_t)sizeof(GridDev));
  L.tile_prefix = off;
  off = align256(off + (int64_t)(njobs + 1) * 8);
  L.td = off;
  off = align256(off + (int64_t)njobs * (int64_t)sizeof(TileDiv));
  L.steps = off;
  off = align256(off + (int64_t)njobs * 4);
  L.ghost_prefix = off;
  off = align256(off + (int64_t)(njobs + 1) * 8);
  L.src_prefix = off;
  off = align256(off + (int64_t)(njobs + 1) * 4);
  L.total = off;
  return L;
}

BatchView batch_view(const gmes_batch& b) {
  const BatchLayout L = batch_layout(b.njobs);
  char* w = static_cast<char*>(b.workspace);
  BatchView v;
  v.jobs = reinterpret_cast<const GridDev*>(w + L.jobs);
  v.tile_prefix = reinterpret_cast<const int64_t*>(w + L.tile_prefix);
  v.td = reinterpret_cast<const TileDiv*>(w + L.td);
  v.steps = reinterpret_cast<const int32_t*>(w + L.steps);
  v.ghost_prefix = reinterpret_cast<const int64_t*>(w + L.ghost_prefix);
  v.src_prefix = reinterpret_cast<const int32_t*>(w + L.src_prefix);
  v.njobs = b.njobs;
  v.srcs = b.srcs;
  v.tiles = b.tiles;
  v.ghosts = b.ghosts;
  return v;
}

// Host copies of the descriptors of the last kHostBatches prepared batches,
// keyed by workspace address: gmes_batch_step passes them to the multi-grid
// cell kernel as launch arguments (batches of at most kParamJobs grids).
// A workspace prepared again replaces its entry.
constexpr int kHostBatches = 64;
struct HostBatch {
  const void* workspace = nullptr;
  std::vector<GridDev> jobs;
};
std::mutex g_host_batch_mutex;
HostBatch g_host_batches[kHostBatches];
int g_host_batch_next = 0;

void remember_batch(const void* ws, const GridDev* jobs, int njobs) {
  std::lock_guard<std::mutex> lock(g_host_batch_mutex);
  HostBatch* slot = nullptr;
  for (auto& h : g_host_batches)
    if (h.workspace == ws) slot = &h;
  if (slot == nullptr) slot = &g_host_batches[g_host_batch_next++ % kHostBatches];
  slot->workspace = ws;
  slot->jobs.assign(jobs, jobs + njobs);
}

// The remembered descriptors of the batch in `ws` (empty if unknown or of
// another size).
std::vector<GridDev> recall_batch(const void* ws, int njobs) {
  std::lock_guard<std::mutex> lock(g_host_batch_mutex);
  for (const auto& h : g_host_batches)
    if (h.workspace == ws && (int)h.jobs.size() == njobs) return h.jobs;
  return {};
}

int64_t max_ghost_plane(const GridDev& d) {
  int64_t m = 1;
  for (int c = 0; c < 6; ++c)
    for (int a = 0; a < 3; ++a)
      for (int b = a + 1; b < 3; ++b) m = d.sh[c][a] * d.sh[c][b] > m ? d.sh[c][a] * d.sh[c][b] : m;
  return m;
}

// The imaginary-plane view of a complex grid: every per-plane pointer moved
// past its real plane.
GridDev make_im_view(const GridDev& re, const gmes_grid_desc& g) {
  GridDev d = re;
  d.part = 1;
  const int64_t es = elem_size(g.precision);
  for (int c = 0; c < 6; ++c) {
    d.f[c] = static_cast<char*>(re.f[c]) + re.npts[c] * es;
    if (re.aux[c] != nullptr)
      d.aux[c] = static_cast<char*>(re.aux[c]) + (int64_t)re.naux[c] * re.npts[c] * es;
  }
  if (re.src_val != nullptr) d.src_val = re.src_val + (int64_t)g.src_steps * 2 * g.nsrc;
  for (int k = 0; k < 2; ++k)
    if (re.tf_field[k] != nullptr)
      d.tf_field[k] = static_cast<const char*>(re.tf_field[k]) + re.tf_npts[k] * es;
  if (re.probe_val != nullptr) d.probe_val = re.probe_val + (int64_t)g.probe_steps * g.nprobe;
  return d;
}

// Launch plan of a grid and (in *inc) of its TFSF incident-field grid.
Plan make_plan(const gmes_grid_desc& g, Plan* inc) {
  Plan p;
  p.re = make_grid_dev(g);
  p.cplx = (g.flags & GMES_FLAG_COMPLEX) != 0;
  p.disp = (g.flags & GMES_FLAG_DISPERSIVE) != 0;
  p.im = p.cplx ? make_im_view(p.re, g) : p.re;
  p.incident = nullptr;
  if (g.ntfsf > 0 && g.incident != nullptr && inc != nullptr) {
    *inc = make_plan(*g.incident, nullptr);
    p.incident = inc;
  }
  return p;
}

}  // namespace gmes

using namespace gmes;

extern "C" {

int gmes_abi_version(void) { return GMES_ABI_VERSION; }

const char* gmes_last_error(void) { return g_last_error.c_str(); }

int gmes_elem_size(int32_t precision) { return elem_size(precision); }

gmes_status gmes_field_shape(const gmes_grid_desc* g, int32_t comp, int64_t shape[3]) {
  if (g == nullptr || shape == nullptr) return fail(GMES_ERR_VALUE, "NULL argument");
  if (comp < 0 || comp > 5) return fail(GMES_ERR_INDEX, "component %d outside [0, 5]", comp);
  comp_shape(g->n, g->active, comp, shape);
  return GMES_OK;
}

gmes_status gmes_grid_sizes(const gmes_grid_desc* g, int64_t sizes[21]) {
  gmes_status st = check_desc(g, false);
  if (st != GMES_OK) return st;
  if (sizes == nullptr) return fail(GMES_ERR_VALUE, "sizes is NULL");
  const int es = elem_size(g->precision);
  const int parts = (g->flags & GMES_FLAG_COMPLEX) ? 2 : 1;
  for (int c = 0; c < 6; ++c) {
    int64_t sh[3];
    comp_shape(g->n, g->active, c, sh);
    const int64_t np = sh[0] * sh[1] * sh[2];
    const bool act = (g->active >> c) & 1;
    sizes[c] = np * es * parts;
    sizes[6 + c] = act ? np : 0;
    sizes[12 + c] = act ? np * es * g->naux[c] * parts : 0;
  }
  sizes[18] = coef_layout(*g).total;
  sizes[19] = (int64_t)g->nsrc * (int64_t)sizeof(gmes_point_source);
  sizes[20] = 2 * (int64_t)g->nsrc * (int64_t)sizeof(double) * parts;
  return GMES_OK;
}

gmes_status gmes_build_coefficients(const gmes_grid_desc* g, const gmes_class_desc* classes,
                                    const double* params, const gmes_pml_desc* pmls,
                                    void* stream) {
  gmes_status st = check_desc(g, true);
  if (st != GMES_OK) return st;
  int ncls = 0;
  for (int c = 0; c < 6; ++c) ncls += g->nclass[c];
  if (ncls > 0 && classes == nullptr) return fail(GMES_ERR_VALUE, "classes is NULL");
  if (g->nparam > 0 && params == nullptr) return fail(GMES_ERR_VALUE, "params is NULL");
  if (g->npml > 0 && pmls == nullptr) return fail(GMES_ERR_VALUE, "pmls is NULL");
  // validate the class table against the pool and the PML list
  int k = 0;
  bool disp = false;
  for (int c = 0; c < 6; ++c) {
    for (int i = 0; i < g->nclass[c]; ++i, ++k) {
      const gmes_class_desc& cd = classes[k];
      if (cd.kind < GMES_KIND_DUMMY || cd.kind > GMES_KIND_DCP_PLRC)
        return fail(GMES_ERR_VALUE, "component %d class %d: unknown kind %d", c, i, cd.kind);
      if ((cd.kind == GMES_KIND_CPML || cd.kind == GMES_KIND_UPML) &&
          (cd.pml < 0 || cd.pml >= g->npml))
        return fail(GMES_ERR_INDEX, "component %d class %d: pml index %d out of range", c, i,
                    cd.pml);
      if ((cd.kind == GMES_KIND_CPML || cd.kind == GMES_KIND_UPML) &&
          pmls[cd.pml].kind != cd.kind)
        return fail(GMES_ERR_VALUE, "component %d class %d: PML kind mismatch", c, i);
      if (cd.param_off < 0 || cd.nparam < 0 || cd.param_off + cd.nparam > g->nparam)
        return fail(GMES_ERR_INDEX, "component %d class %d: parameters outside the pool", c, i);
      if (cd.npole < 0 || cd.npole > GMES_MAX_POLES || cd.ncp < 0 || cd.ncp > GMES_MAX_POLES)
        return fail(GMES_ERR_VALUE, "component %d class %d: at most %d poles", c, i,
                    GMES_MAX_POLES);
      if (!(cd.eps > 0) && cd.kind != GMES_KIND_DUMMY && cd.kind != GMES_KIND_CONST)
        return fail(GMES_ERR_VALUE, "component %d class %d: eps/mu must be positive", c, i);
      int need = 0, naux = 0;
      switch (cd.kind) {
        case GMES_KIND_CONST: need = 1; break;
        case GMES_KIND_DRUDE: need = 2 + 2 * cd.npole; naux = 2 * cd.npole; break;
        case GMES_KIND_LORENTZ: need = 2 + 3 * cd.npole; naux = 2 * cd.npole; break;
        case GMES_KIND_DCP: need = 2 + 2 * cd.npole + 5 * cd.ncp;
          naux = 1 + 2 * cd.npole + 2 * cd.ncp; break;
        case GMES_KIND_DCP_PLRC: need = 3 + 5 * cd.npole + 9 * cd.ncp;
          naux = cd.npole + 2 * cd.ncp; break;
        case GMES_KIND_CPML: naux = 2; break;
        case GMES_KIND_UPML: naux = 1; break;
        default: break;
      }
      const bool dispk = cd.kind == GMES_KIND_DRUDE || cd.kind == GMES_KIND_LORENTZ ||
                         cd.kind == GMES_KIND_DCP || cd.kind == GMES_KIND_DCP_PLRC;
      if (dispk && c >= 3)
        return fail(GMES_ERR_VALUE, "component %d class %d: dispersive kinds are E-only", c, i);
      disp = disp || dispk;
      if (cd.nparam < need)
        return fail(GMES_ERR_VALUE, "component %d class %d: %d parameters, kind needs %d", c,
                    i, cd.nparam, need);
      if (naux > g->naux[c])
        return fail(GMES_ERR_VALUE, "component %d class %d needs %d state slots, naux = %d", c,
                    i, naux, g->naux[c]);
    }
  }
  if (disp && !(g->flags & GMES_FLAG_DISPERSIVE))
    return fail(GMES_ERR_VALUE, "dispersive classes present but GMES_FLAG_DISPERSIVE unset");
  const CoefLayout L = coef_layout(*g);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(g->coef);
  cudaError_t e = cudaSuccess;
  if (ncls > 0)
    e = cudaMemcpyAsync(base + L.raw_classes, classes, ncls * sizeof(gmes_class_desc),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && g->nparam > 0)
    e = cudaMemcpyAsync(base + L.raw_params, params, g->nparam * sizeof(double),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && g->npml > 0)
    e = cudaMemcpyAsync(base + L.raw_pmls, pmls, g->npml * sizeof(gmes_pml_desc),
                        cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "staging coefficient inputs");
  for (int c = 0; c < 6 && e == cudaSuccess; ++c)
    e = cudaMemsetAsync(base + L.class_tab[c], 0, GMES_MAX_CLASSES * sizeof(ClassCoef), s);
  if (e != cudaSuccess) return cuda_fail(e, "clearing class tables");
  const GridDev d = make_grid_dev(*g);
  e = launch_build_coefficients(*g, d, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "building coefficients");
  return GMES_OK;
}

gmes_status gmes_set_pml_profile(const gmes_grid_desc* g, int32_t pml, int32_t comp,
                                 int32_t axis, const double* values, void* stream) {
  gmes_status st = check_desc(g, true);
  if (st != GMES_OK) return st;
  if (pml < 0 || pml >= g->npml) return fail(GMES_ERR_INDEX, "pml %d out of range", pml);
  if (comp < 0 || comp > 5 || axis < 0 || axis > 2)
    return fail(GMES_ERR_INDEX, "component %d / axis %d out of range", comp, axis);
  if (!((g->active >> comp) & 1)) return fail(GMES_ERR_VALUE, "component %d inactive", comp);
  if (values == nullptr) return fail(GMES_ERR_VALUE, "values is NULL");
  const CoefLayout L = coef_layout(*g);
  int64_t sh[3];
  comp_shape(g->n, g->active, comp, sh);
  // The kind of this PML is read back from the staged inputs.
  gmes_pml_desc pd;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(g->coef);
  cudaError_t e = cudaMemcpyAsync(&pd, base + L.raw_pmls + pml * sizeof(gmes_pml_desc),
                                  sizeof(pd), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "reading PML descriptor");
  std::vector<Coef> rows(sh[axis] * kProfStride);
  const double dr = g->dr[axis], dt = g->dt;
  for (int64_t n = 0; n < sh[axis]; ++n) {
    const double* v = values + 3 * n;
    Coef* out = rows.data() + n * kProfStride;
    if (pd.kind == GMES_KIND_CPML) {
      const double b = v[0], c = v[1], kappa = v[2];
      out[0] = make_coef(b);
      out[1] = make_coef(c);
      out[2] = make_coef(kappa);
      out[3] = make_coef(c / dr);
      out[4] = make_coef(1.0 / (kappa * dr));
    } else {
      const double sigma = v[0], kappa = v[1];
      const double num = 2 * kappa - sigma * dt, den = 2 * kappa + sigma * dt;
      out[0] = make_coef(num / den);
      out[1] = make_coef(2 * dt / den);
      out[2] = make_coef(1 / den);
      out[3] = make_coef(den);
      out[4] = make_coef(num);
    }
  }
  e = cudaMemcpyAsync(base + L.prof[pml][comp][axis], rows.data(), rows.size() * sizeof(Coef),
                      cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "uploading PML profile");
  return GMES_OK;
}

gmes_status gmes_get_pml_profile(const gmes_grid_desc* g, int32_t pml, int32_t comp,
                                 int32_t axis, double* out, void* stream) {
  gmes_status st = check_desc(g, true);
  if (st != GMES_OK) return st;
  if (pml < 0 || pml >= g->npml) return fail(GMES_ERR_INDEX, "pml %d out of range", pml);
  if (comp < 0 || comp > 5 || axis < 0 || axis > 2)
    return fail(GMES_ERR_INDEX, "component %d / axis %d out of range", comp, axis);
  if (!((g->active >> comp) & 1)) return fail(GMES_ERR_VALUE, "component %d inactive", comp);
  if (out == nullptr) return fail(GMES_ERR_VALUE, "out is NULL");
  const CoefLayout L = coef_layout(*g);
  int64_t sh[3];
  comp_shape(g->n, g->active, comp, sh);
  std::vector<Coef> rows(sh[axis] * kProfStride);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(rows.data(), static_cast<char*>(g->coef) + L.prof[pml][comp][axis],
                                  rows.size() * sizeof(Coef), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "reading PML profile");
  for (size_t i = 0; i < rows.size(); ++i) out[i] = rows[i].d;
  return GMES_OK;
}

gmes_status gmes_reset(const gmes_grid_desc* g, void* stream) {
  gmes_status st = check_desc(g, true);
  if (st != GMES_OK) return st;
  int64_t sizes[21];
  gmes_grid_sizes(g, sizes);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  for (int c = 0; c < 6; ++c) {
    cudaError_t e = cudaMemsetAsync(g->field[c], 0, sizes[c], s);
    if (e == cudaSuccess && sizes[12 + c] > 0) e = cudaMemsetAsync(g->aux[c], 0, sizes[12 + c], s);
    if (e != cudaSuccess) return cuda_fail(e, "zeroing buffers");
  }
  return GMES_OK;
}

gmes_status gmes_step(const gmes_grid_desc* g, int32_t nsteps, void* stream) {
  gmes_status st = check_desc(g, true);
  if (st != GMES_OK) return st;
  if (nsteps < 0) return fail(GMES_ERR_VALUE, "nsteps = %d must be >= 0", nsteps);
  if (g->nsrc > 0 && nsteps > g->src_steps)
    return fail(GMES_ERR_VALUE, "nsteps = %d exceeds the source-value capacity %d", nsteps,
                g->src_steps);
  if (g->nprobe > 0 && nsteps > g->probe_steps)
    return fail(GMES_ERR_VALUE, "nsteps = %d exceeds the probe buffer capacity %d", nsteps,
                g->probe_steps);
  st = check_aux(g);
  if (st != GMES_OK) return st;
  if (g->ntfsf > 0 && g->incident->nsrc > 0 && nsteps > g->incident->src_steps)
    return fail(GMES_ERR_VALUE, "nsteps = %d exceeds the incident grid's source capacity %d",
                nsteps, g->incident->src_steps);
  if (nsteps == 0) return GMES_OK;
  Plan inc;
  const Plan p = make_plan(*g, &inc);
  cudaError_t e = launch_step(*g, p, nsteps, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching step kernels");
  return GMES_OK;
}

gmes_status gmes_half_step(const gmes_grid_desc* g, int32_t side, int32_t step, void* stream) {
  gmes_status st = check_desc(g, true);
  if (st != GMES_OK) return st;
  if (side != 0 && side != 1) return fail(GMES_ERR_VALUE, "side = %d must be 0 (E) or 1 (H)", side);
  if (step < 0 || (g->nsrc > 0 && step >= g->src_steps))
    return fail(GMES_ERR_INDEX, "step %d outside the source-value buffer (%d steps)", step,
                g->src_steps);
  if (g->nprobe > 0 && step >= g->probe_steps)
    return fail(GMES_ERR_INDEX, "step %d outside the probe buffer (%d steps)", step,
                g->probe_steps);
  st = check_aux(g);
  if (st != GMES_OK) return st;
  if (g->ntfsf > 0 && g->incident->nsrc > 0 && step >= g->incident->src_steps)
    return fail(GMES_ERR_INDEX, "step %d outside the incident grid's source-value buffer", step);
  Plan inc;
  const Plan p = make_plan(*g, &inc);
  cudaError_t e = launch_half(*g, p, side, step, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching half-step kernels");
  return GMES_OK;
}

int64_t gmes_batch_workspace_size(int32_t njobs) {
  if (njobs < 1) return 0;
  return batch_layout(njobs).total;
}

gmes_status gmes_batch_prepare(const gmes_grid_desc* const* grids, int32_t njobs,
                               void* workspace, int64_t workspace_bytes, int32_t bx_cap,
                               gmes_batch* out, void* stream) {
  if (grids == nullptr || out == nullptr || workspace == nullptr)
    return fail(GMES_ERR_VALUE, "NULL argument");
  if (njobs < 1) return fail(GMES_ERR_VALUE, "njobs = %d must be >= 1", njobs);
  if (bx_cap < 0 || bx_cap > 5) return fail(GMES_ERR_VALUE, "bx_cap = %d outside [0, 5]", bx_cap);
  if (bx_cap == 0) bx_cap = 4;  // 16-cell rows, as the single-grid kernel
  const BatchLayout L = batch_layout(njobs);
  if (workspace_bytes < L.total)
    return fail(GMES_ERR_VALUE, "workspace of %lld bytes, %lld needed",
                (long long)workspace_bytes, (long long)L.total);
  std::vector<char> host(L.total, 0);
  GridDev* jobs = reinterpret_cast<GridDev*>(host.data() + L.jobs);
  int64_t* tp = reinterpret_cast<int64_t*>(host.data() + L.tile_prefix);
  TileDiv* td = reinterpret_cast<TileDiv*>(host.data() + L.td);
  int32_t* steps = reinterpret_cast<int32_t*>(host.data() + L.steps);
  int64_t* gp = reinterpret_cast<int64_t*>(host.data() + L.ghost_prefix);
  int32_t* sp = reinterpret_cast<int32_t*>(host.data() + L.src_prefix);
  int32_t precision = -1;
  bool disp = false;
  tp[0] = 0;
  gp[0] = 0;
  sp[0] = 0;
  for (int q = 0; q < njobs; ++q) {
    const gmes_grid_desc* g = grids[q];
    gmes_status st = check_desc(g, true);
    if (st != GMES_OK) return fail(st, "grid %d: %s", q, g_last_error.c_str());
    if (g->ntfsf > 0) return fail(GMES_ERR_VALUE, "grid %d has a TFSF source: not batchable", q);
    if (g->nprobe > 0) return fail(GMES_ERR_VALUE, "grid %d has probes: not batchable", q);
    if (g->flags & GMES_FLAG_COMPLEX)
      return fail(GMES_ERR_VALUE, "grid %d is complex: not batchable", q);
    if (precision < 0) precision = g->precision;
    if (g->precision != precision)
      return fail(GMES_ERR_VALUE, "grid %d: all grids of a batch must share one precision", q);
    disp = disp || (g->flags & GMES_FLAG_DISPERSIVE);
    jobs[q] = make_grid_dev(*g);
    if (!offsets_fit_i32(jobs[q]))
      return fail(GMES_ERR_VALUE,
                  "grid %d has a component of 2^31 or more points: step it alone, not in a batch",
                  q);
    int l = 0;
    while (l < bx_cap && (1 << l) < g->n[2]) ++l;
    td[q] = tile_div(l, g->n);
    const int64_t tiles = (int64_t)td[q].plane * g->n[0];
    tp[q + 1] = tp[q] + tiles;
    gp[q + 1] = gp[q] + 6 * max_ghost_plane(jobs[q]);
    sp[q + 1] = sp[q] + g->nsrc;
    steps[q] = 0;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(workspace, host.data(), L.total, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "uploading the batch workspace");
  out->njobs = njobs;
  out->precision = precision;
  out->dispersive = disp ? 1 : 0;
  out->srcs = sp[njobs];
  out->tiles = tp[njobs];
  out->ghosts = gp[njobs];
  out->workspace = workspace;
  out->workspace_bytes = workspace_bytes;
  remember_batch(workspace, jobs, njobs);
  return GMES_OK;
}

gmes_status gmes_batch_set_steps(const gmes_batch* b, const int32_t* steps, void* stream) {
  if (b == nullptr || steps == nullptr || b->workspace == nullptr)
    return fail(GMES_ERR_VALUE, "NULL argument");
  for (int q = 0; q < b->njobs; ++q)
    if (steps[q] < 0) return fail(GMES_ERR_VALUE, "steps[%d] = %d < 0", q, steps[q]);
  const BatchLayout L = batch_layout(b->njobs);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(static_cast<char*>(b->workspace) + L.steps, steps,
                                  b->njobs * sizeof(int32_t), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "uploading batch steps");
  return GMES_OK;
}

gmes_status gmes_batch_step(const gmes_batch* b, int32_t nsteps, int32_t blocks, void* stream) {
  if (b == nullptr || b->workspace == nullptr) return fail(GMES_ERR_VALUE, "NULL argument");
  if (nsteps < 0 || blocks < 0) return fail(GMES_ERR_VALUE, "negative nsteps or blocks");
  if (b->njobs < 1) return fail(GMES_ERR_VALUE, "empty batch");
  if (nsteps == 0) return GMES_OK;
  const std::vector<GridDev> host =
      b->njobs <= kParamJobs ? recall_batch(b->workspace, b->njobs) : std::vector<GridDev>();
  cudaError_t e = launch_batch(batch_view(*b), host.empty() ? nullptr : host.data(),
                               b->precision, b->dispersive != 0, nsteps, blocks,
                               static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching batch kernels");
  return GMES_OK;
}

static gmes_status capture(cudaStream_t s, void** exec_out,
                           const std::function<gmes_status()>& body) {
  if (s == nullptr) return fail(GMES_ERR_VALUE, "graph capture needs a non-default stream");
  if (exec_out == nullptr) return fail(GMES_ERR_VALUE, "graph_exec is NULL");
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "beginning stream capture");
  gmes_status st = body();
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(s, &graph);
  if (st != GMES_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  if (e != cudaSuccess) return cuda_fail(e, "ending stream capture");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "instantiating graph");
  *exec_out = exec;
  return GMES_OK;
}

gmes_status gmes_graph_capture_step(const gmes_grid_desc* g, int32_t nsteps, void* stream,
                                    void** graph_exec) {
  return capture(static_cast<cudaStream_t>(stream), graph_exec,
                 [&]() { return gmes_step(g, nsteps, stream); });
}

gmes_status gmes_graph_capture_batch(const gmes_batch* b, int32_t nsteps, int32_t blocks,
                                     void* stream, void** graph_exec) {
  return capture(static_cast<cudaStream_t>(stream), graph_exec,
                 [&]() { return gmes_batch_step(b, nsteps, blocks, stream); });
}

gmes_status gmes_graph_launch(void* graph_exec, void* stream) {
  if (graph_exec == nullptr) return fail(GMES_ERR_VALUE, "graph_exec is NULL");
  cudaError_t e = cudaGraphLaunch(static_cast<cudaGraphExec_t>(graph_exec),
                                  static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching graph");
  return GMES_OK;
}

gmes_status gmes_graph_destroy(void* graph_exec) {
  if (graph_exec == nullptr) return GMES_OK;
  cudaError_t e = cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(graph_exec));
  if (e != cudaSuccess) return cuda_fail(e, "destroying graph");
  return GMES_OK;
}

gmes_status gmes_copy_async(void* dst, const void* src, int64_t bytes, void* stream) {
  if (bytes < 0) return fail(GMES_ERR_VALUE, "negative copy size");
  if (bytes == 0) return GMES_OK;
  if (dst == nullptr || src == nullptr) return fail(GMES_ERR_VALUE, "copy pointer is NULL");
  cudaError_t e = cudaMemcpyAsync(dst, src, static_cast<size_t>(bytes), cudaMemcpyDefault,
                                  static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "copying");
  return GMES_OK;
}

gmes_status gmes_rasterize(const gmes_grid_desc* g, int32_t comp, const gmes_shape* shapes,
                           int32_t nshapes, const uint8_t* lut, void* stream) {
  gmes_status st = check_desc(g, true);
  if (st != GMES_OK) return st;
  if (comp < 0 || comp > 5) return fail(GMES_ERR_INDEX, "component %d outside [0, 5]", comp);
  if (!((g->active >> comp) & 1)) return fail(GMES_ERR_VALUE, "component %d inactive", comp);
  if (shapes == nullptr || lut == nullptr) return fail(GMES_ERR_VALUE, "NULL shapes or lut");
  if (nshapes < 1 || nshapes > 255)
    return fail(GMES_ERR_VALUE, "nshapes = %d outside [1, 255]", nshapes);
  const GridDev d = make_grid_dev(*g);
  cudaError_t e = launch_raster(*g, d, comp, shapes, nshapes, lut,
                                static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching the rasteriser");
  return GMES_OK;
}

gmes_status gmes_nonfinite(const gmes_grid_desc* g, int32_t* flag, void* stream) {
  gmes_status st = check_desc(g, true);
  if (st != GMES_OK) return st;
  if (flag == nullptr) return fail(GMES_ERR_VALUE, "flag is NULL");
  const GridDev d = make_grid_dev(*g);
  cudaError_t e = launch_nonfinite(*g, d, flag, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching the non-finite check");
  return GMES_OK;
}

gmes_status gmes_read_field(const gmes_grid_desc* g, int32_t comp, double* host_out,
                            void* stream) {
  gmes_status st = check_desc(g, true);
  if (st != GMES_OK) return st;
  if (comp < 0 || comp > 5) return fail(GMES_ERR_INDEX, "component %d outside [0, 5]", comp);
  if (host_out == nullptr) return fail(GMES_ERR_VALUE, "host_out is NULL");
  int64_t sh[3];
  comp_shape(g->n, g->active, comp, sh);
  const int64_t np = sh[0] * sh[1] * sh[2] * ((g->flags & GMES_FLAG_COMPLEX) ? 2 : 1);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (g->precision == GMES_FP64 || g->precision == GMES_FP64_STRICT) {
    e = cudaMemcpyAsync(host_out, g->field[comp], np * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  } else if (g->precision == GMES_FP32) {
    std::vector<float> tmp(np);
    e = cudaMemcpyAsync(tmp.data(), g->field[comp], np * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (int64_t i = 0; e == cudaSuccess && i < np; ++i) host_out[i] = tmp[i];
  } else {
    std::vector<float> tmp(2 * np);
    e = cudaMemcpyAsync(tmp.data(), g->field[comp], np * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (int64_t i = 0; e == cudaSuccess && i < np; ++i)
      host_out[i] = (double)tmp[2 * i] + (double)tmp[2 * i + 1];
  }
  if (e != cudaSuccess) return cuda_fail(e, "reading field");
  return GMES_OK;
}

gmes_status gmes_write_field(const gmes_grid_desc* g, int32_t comp, const double* host_in,
                             void* stream) {
  gmes_status st = check_desc(g, true);
  if (st != GMES_OK) return st;
  if (comp < 0 || comp > 5) return fail(GMES_ERR_INDEX, "component %d outside [0, 5]", comp);
  if (host_in == nullptr) return fail(GMES_ERR_VALUE, "host_in is NULL");
  int64_t sh[3];
  comp_shape(g->n, g->active, comp, sh);
  const int64_t np = sh[0] * sh[1] * sh[2] * ((g->flags & GMES_FLAG_COMPLEX) ? 2 : 1);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (g->precision == GMES_FP64 || g->precision == GMES_FP64_STRICT) {
    e = cudaMemcpyAsync(g->field[comp], host_in, np * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  } else if (g->precision == GMES_FP32) {
    std::vector<float> tmp(np);
    for (int64_t i = 0; i < np; ++i) tmp[i] = (float)host_in[i];
    e = cudaMemcpyAsync(g->field[comp], tmp.data(), np * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  } else {
    std::vector<float> tmp(2 * np);
    for (int64_t i = 0; i < np; ++i) {
      const float h = (float)host_in[i];
      tmp[2 * i] = h;
      tmp[2 * i + 1] = (float)(host_in[i] - (double)h);
    }
    e = cudaMemcpyAsync(g->field[comp], tmp.data(), np * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e != cudaSuccess) return cuda_fail(e, "writing field");
  return GMES_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Differentiation: batched TMz forward / adjoint (gmes_adjoint.cu).
// ---------------------------------------------------------------------------
namespace gmes {
namespace {

constexpr int32_t kTmzActive = (1 << GMES_EZ) | (1 << GMES_HX) | (1 << GMES_HY);

struct TmzLayout {
  int64_t array;  // bytes of one [nb][nx][ny] array, 256-aligned
  int64_t state, adjoint, design, hist, monitor, grad, scratch;
  // the design buffer: per-pixel coefficients, then the lattice map's
  // flags and its four coefficient arrays
  int64_t design_coef, map_flags, map_coef;
};

// Whether the FP32 forward and adjoint run the temporally blocked kernels,
// which need the scratch copy of the state.
bool tmz_blocked(const gmes_grid_desc& g, const gmes_tmz_batch& b) {
  return g.precision == GMES_FP32 && b.block_steps != 1;
}

TmzLayout tmz_layout(const gmes_grid_desc& g, const gmes_tmz_batch& b) {
  TmzLayout L;
  const int64_t es = elem_size(g.precision);
  const int64_t plane = (int64_t)g.n[0] * g.n[1];
  const int64_t nd = (int64_t)b.design_n[0] * b.design_n[1];
  const int64_t nm = (int64_t)b.monitor_n[0] * b.monitor_n[1];
  L.array = align256((int64_t)b.nbatch * plane * es);
  L.state = kTmzState * L.array;
  L.adjoint = kTmzAdjoint * L.array;
  L.design_coef = align256((int64_t)b.nbatch * nd * (int64_t)sizeof(DesignCoef));
  L.map_flags = align256(plane * 4);
  L.map_coef = align256(plane * es);
  L.design = L.design_coef + L.map_flags + 4 * L.map_coef;
  L.hist = align256((int64_t)b.hist_steps * b.nbatch * nd * es);
  L.monitor = align256((int64_t)b.nbatch * b.total_steps * nm * 8);
  L.grad = align256((int64_t)b.nbatch * nd * 8);
  L.scratch = tmz_blocked(g, b) ? L.state : 0;
  return L;
}

gmes_status check_tmz(const gmes_grid_desc* g, const gmes_tmz_batch* b, bool need_buffers) {
  gmes_status st = check_desc(g, need_buffers);
  if (st != GMES_OK) return st;
  if (b == nullptr) return fail(GMES_ERR_VALUE, "batch descriptor is NULL");
  if (g->active != kTmzActive || g->n[2] != 1)
    return fail(GMES_ERR_VALUE, "the adjoint path needs a TMz grid (Ez, Hx, Hy; n[2] = 1)");
  if (g->precision == GMES_FP64_STRICT)
    return fail(GMES_ERR_VALUE, "fp64_strict has no adjoint path; use fp64");
  if (g->flags & GMES_FLAG_COMPLEX)
    return fail(GMES_ERR_VALUE, "the adjoint path needs a real grid");
  if (b->nbatch < 1 || b->nbatch > 65535)
    return fail(GMES_ERR_VALUE, "nbatch = %d outside [1, 65535]", b->nbatch);
  const int32_t nn[2] = {g->n[0], g->n[1]};
  for (int a = 0; a < 2; ++a) {
    if (b->design_n[a] < 1 || b->design_lo[a] < 0 || b->design_lo[a] + b->design_n[a] > nn[a])
      return fail(GMES_ERR_INDEX, "design box outside the %d x %d lattice", nn[0], nn[1]);
    if (b->monitor_n[a] < 1 || b->monitor_lo[a] < 0 || b->monitor_lo[a] + b->monitor_n[a] > nn[a])
      return fail(GMES_ERR_INDEX, "monitor box outside the %d x %d lattice", nn[0], nn[1]);
  }
  if (b->nsrc < 0 || b->total_steps < 1 || b->hist_steps < 0)
    return fail(GMES_ERR_VALUE, "negative nsrc / hist_steps or total_steps < 1");
  if (b->block_steps < 0 || b->block_steps > GMES_TMZ_MAX_BLOCK_STEPS)
    return fail(GMES_ERR_VALUE, "block_steps = %d outside [0, %d]", b->block_steps,
                GMES_TMZ_MAX_BLOCK_STEPS);
  if (need_buffers) {
    if (!b->state || !b->adjoint || !b->design || !b->monitor || !b->grad)
      return fail(GMES_ERR_VALUE, "a batch buffer is NULL");
    if (b->hist_steps > 0 && !b->hist) return fail(GMES_ERR_VALUE, "hist is NULL");
    if (tmz_blocked(*g, *b) && !b->scratch)
      return fail(GMES_ERR_VALUE, "scratch is NULL (needed by the FP32 blocked kernels)");
    if (b->nsrc > 0 && (!b->src || !b->src_val))
      return fail(GMES_ERR_VALUE, "nsrc > 0 but src or src_val is NULL");
  }
  return GMES_OK;
}

TmzDev make_tmz_dev(const gmes_grid_desc& g, const gmes_tmz_batch& b) {
  const TmzLayout L = tmz_layout(g, b);
  TmzDev t;
  std::memset(&t, 0, sizeof(t));
  t.nx = g.n[0];
  t.ny = g.n[1];
  t.nb = b.nbatch;
  t.nsrc = b.nsrc;
  t.plane = (int64_t)g.n[0] * g.n[1];
  for (int a = 0; a < 2; ++a) {
    t.d0[a] = b.design_lo[a];
    t.dn[a] = b.design_n[a];
    t.m0[a] = b.monitor_lo[a];
    t.mn[a] = b.monitor_n[a];
  }
  t.total_steps = b.total_steps;
  t.hist_steps = b.hist_steps;
  char* s = static_cast<char*>(b.state);
  for (int k = 0; k < kTmzState; ++k) t.f[k] = s + k * L.array;
  if (tmz_blocked(g, b))
    for (int k = 0; k < kTmzState; ++k) t.tmp[k] = static_cast<char*>(b.scratch) + k * L.array;
  char* a = static_cast<char*>(b.adjoint);
  for (int k = 0; k < 3; ++k) t.l[k] = a + k * L.array;
  for (int r = 0; r < 2; ++r)
    for (int k = 0; k < 4; ++k) t.phi[r][k] = a + (3 + 4 * r + k) * L.array;
  t.dc = static_cast<const DesignCoef*>(b.design);
  const char* map = static_cast<const char*>(b.design) + L.design_coef;
  t.pflags = reinterpret_cast<const uint32_t*>(map);
  for (int k = 0; k < 4; ++k) t.pcoef[k] = map + L.map_flags + k * L.map_coef;
  t.hist = b.hist;
  t.mon = b.monitor;
  t.grad = b.grad;
  t.weight = b.weight;
  t.src = b.src;
  t.src_val = b.src_val;
  return t;
}

}  // namespace
}  // namespace gmes

extern "C" {

gmes_status gmes_tmz_sizes(const gmes_grid_desc* g, const gmes_tmz_batch* b, int64_t sizes[7]) {
  gmes_status st = check_tmz(g, b, false);
  if (st != GMES_OK) return st;
  if (sizes == nullptr) return fail(GMES_ERR_VALUE, "sizes is NULL");
  const TmzLayout L = tmz_layout(*g, *b);
  sizes[0] = L.state;
  sizes[1] = L.adjoint;
  sizes[2] = L.design;
  sizes[3] = L.hist;
  sizes[4] = L.monitor;
  sizes[5] = L.grad;
  sizes[6] = L.scratch;
  return GMES_OK;
}

gmes_status gmes_tmz_check(const gmes_grid_desc* g, const gmes_tmz_batch* b) {
  gmes_status st = check_tmz(g, b, true);
  if (st != GMES_OK) return st;
  const CoefLayout CL = coef_layout(*g);
  const char* base = static_cast<const char*>(g->coef);
  int kinds[3][GMES_MAX_CLASSES];
  for (int c = 2; c < 5; ++c) {
    std::vector<ClassCoef> tab(g->nclass[c]);
    cudaError_t e = cudaMemcpy(tab.data(), base + CL.class_tab[c],
                               tab.size() * sizeof(ClassCoef), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "reading the class table");
    for (int k = 0; k < GMES_MAX_CLASSES; ++k) kinds[c - 2][k] = GMES_KIND_DUMMY;
    for (int k = 0; k < g->nclass[c]; ++k) {
      const int kind = tab[k].kind;
      if (kind != GMES_KIND_DUMMY && kind != GMES_KIND_DIELECTRIC && kind != GMES_KIND_CPML)
        return fail(GMES_ERR_VALUE,
                    "component %d class %d has kind %d; the adjoint path supports "
                    "DIELECTRIC, CPML and DUMMY", c, k, kind);
      kinds[c - 2][k] = kind;
    }
  }
  // the design box's Ez points must be dielectric
  const int64_t sez1 = g->n[2];                 // Ez shape (n0+1, n1+1, 1)
  const int64_t sez0 = (int64_t)(g->n[1] + 1) * sez1;
  std::vector<uint8_t> ids((size_t)b->design_n[0] * b->design_n[1]);
  cudaError_t e = cudaMemcpy2D(ids.data(), (size_t)b->design_n[1],
                               g->cls[2] + b->design_lo[0] * sez0 + b->design_lo[1] * sez1,
                               (size_t)sez0, (size_t)b->design_n[1], (size_t)b->design_n[0],
                               cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "reading the Ez class map");
  for (size_t k = 0; k < ids.size(); ++k)
    if (kinds[0][ids[k]] != GMES_KIND_DIELECTRIC)
      return fail(GMES_ERR_VALUE, "design point %zu is not on a dielectric Ez point", k);
  return GMES_OK;
}

gmes_status gmes_tmz_set_design(const gmes_grid_desc* g, const gmes_tmz_batch* b,
                                const double* eps, void* stream) {
  gmes_status st = check_tmz(g, b, true);
  if (st != GMES_OK) return st;
  if (eps == nullptr) return fail(GMES_ERR_VALUE, "eps is NULL");
  cudaError_t e = launch_tmz_design(g->precision, make_grid_dev(*g), make_tmz_dev(*g, *b), eps,
                                    static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching the design kernel");
  return GMES_OK;
}

gmes_status gmes_tmz_reset(const gmes_grid_desc* g, const gmes_tmz_batch* b, int32_t what,
                           void* stream) {
  gmes_status st = check_tmz(g, b, true);
  if (st != GMES_OK) return st;
  const TmzLayout L = tmz_layout(*g, *b);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
  if (what & 1) e = cudaMemsetAsync(b->state, 0, (size_t)L.state, s);
  if (e == cudaSuccess && (what & 2)) e = cudaMemsetAsync(b->adjoint, 0, (size_t)L.adjoint, s);
  if (e == cudaSuccess && (what & 2))
    e = cudaMemsetAsync(b->grad, 0, (size_t)b->nbatch * b->design_n[0] * b->design_n[1] * 8, s);
  if (e != cudaSuccess) return cuda_fail(e, "clearing the batch");
  return GMES_OK;
}

gmes_status gmes_tmz_forward(const gmes_grid_desc* g, const gmes_tmz_batch* b, int32_t step0,
                             int32_t nsteps, int32_t flags, void* stream) {
  gmes_status st = check_tmz(g, b, true);
  if (st != GMES_OK) return st;
  if (step0 < 0 || nsteps < 0 || (int64_t)step0 + nsteps > b->total_steps)
    return fail(GMES_ERR_INDEX, "steps %d..%d outside 1..%d", step0 + 1, step0 + nsteps,
                b->total_steps);
  if ((flags & ~3) != 0) return fail(GMES_ERR_VALUE, "unknown flags 0x%x", flags);
  if ((flags & GMES_TMZ_RECORD_HIST) && nsteps > b->hist_steps)
    return fail(GMES_ERR_VALUE, "%d steps exceed the hist capacity %d", nsteps, b->hist_steps);
  cudaError_t e = launch_tmz_forward(g->precision, make_grid_dev(*g), make_tmz_dev(*g, *b),
                                     step0, nsteps, flags, b->block_steps,
                                     static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching the forward kernels");
  return GMES_OK;
}

gmes_status gmes_tmz_objective(const gmes_grid_desc* g, const gmes_tmz_batch* b,
                               int32_t nsteps, double* J, void* stream) {
  gmes_status st = check_tmz(g, b, true);
  if (st != GMES_OK) return st;
  if (J == nullptr) return fail(GMES_ERR_VALUE, "J is NULL");
  if (nsteps < 0 || nsteps > b->total_steps)
    return fail(GMES_ERR_INDEX, "nsteps = %d outside [0, %d]", nsteps, b->total_steps);
  cudaError_t e = launch_tmz_objective(make_grid_dev(*g), make_tmz_dev(*g, *b), nsteps, J,
                                       static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching the objective kernel");
  return GMES_OK;
}

gmes_status gmes_tmz_adjoint(const gmes_grid_desc* g, const gmes_tmz_batch* b, int32_t step0,
                             int32_t nsteps, void* stream) {
  gmes_status st = check_tmz(g, b, true);
  if (st != GMES_OK) return st;
  if (step0 < 0 || nsteps < 0 || (int64_t)step0 + nsteps > b->total_steps)
    return fail(GMES_ERR_INDEX, "steps %d..%d outside 1..%d", step0 + 1, step0 + nsteps,
                b->total_steps);
  if (nsteps > b->hist_steps)
    return fail(GMES_ERR_VALUE, "%d steps exceed the hist capacity %d", nsteps, b->hist_steps);
  cudaError_t e = launch_tmz_adjoint(g->precision, make_grid_dev(*g), make_tmz_dev(*g, *b),
                                     step0, nsteps, b->block_steps,
                                     static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching the adjoint kernels");
  return GMES_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Point-list updaters (gmes_points.cu).
// ---------------------------------------------------------------------------
extern "C" gmes_status gmes_points_update(const gmes_points* p, void* inplace, const void* in1,
                                          const void* in2, double d1, double d2, double dt,
                                          void* stream) {
  if (p == nullptr || inplace == nullptr || in1 == nullptr || in2 == nullptr)
    return fail(GMES_ERR_VALUE, "NULL argument");
  if (p->comp < 0 || p->comp > 5) return fail(GMES_ERR_INDEX, "component %d outside [0, 5]", p->comp);
  if (p->kind < GMES_KIND_DUMMY || p->kind > GMES_KIND_DCP_PLRC)
    return fail(GMES_ERR_VALUE, "unknown kind %d", p->kind);
  if (p->npoints < 0 || p->nparam < 0 || p->nstate < 0 || p->npole < 0 || p->ncp < 0 ||
      p->npole > GMES_MAX_POLES || p->ncp > GMES_MAX_POLES)
    return fail(GMES_ERR_VALUE, "bad point-list sizes");
  int need = 0, nstate = 0;
  switch (p->kind) {
    case GMES_KIND_DIELECTRIC: need = 1; break;
    case GMES_KIND_CPML: need = 7; nstate = 2; break;
    case GMES_KIND_UPML: need = 7; nstate = 1; break;
    case GMES_KIND_DRUDE:
    case GMES_KIND_LORENTZ: need = 3 * p->npole + 3; nstate = 2 * p->npole; break;
    case GMES_KIND_DCP: need = 3 * p->npole + 5 * p->ncp + 4; nstate = 1 + 2 * p->npole + 2 * p->ncp; break;
    case GMES_KIND_DCP_PLRC: need = 3 * p->npole + 6 * p->ncp + 3; nstate = p->npole + 2 * p->ncp; break;
    case GMES_KIND_CONST: need = 1; break;
    default: break;
  }
  if (p->nparam < need || p->nstate < nstate)
    return fail(GMES_ERR_VALUE, "kind %d needs %d parameters and %d state slots per point",
                p->kind, need, nstate);
  if (p->npoints > 0 && (p->idx == nullptr || (p->nparam > 0 && p->param == nullptr) ||
                         (p->nstate > 0 && p->state == nullptr)))
    return fail(GMES_ERR_VALUE, "NULL point arrays");
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      if (p->shape[a][b] < 1) return fail(GMES_ERR_VALUE, "array extents must be >= 1");
  if (p->kind == GMES_KIND_DUMMY || p->npoints == 0) return GMES_OK;
  cudaError_t e = launch_points(*p, inplace, in1, in2, d1, d2, dt, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "launching the point-list kernel");
  return GMES_OK;
}

// ---------------------------------------------------------------------------
// gmes_batch_step_noalloc: the batch tables in a fixed device array.
// ---------------------------------------------------------------------------
namespace gmes {
namespace {

constexpr int64_t kNoAllocBytes = 192 * 1024;  // >= batch_layout(GMES_NOALLOC_MAX_GRIDS).total
static_assert(GMES_NOALLOC_MAX_GRIDS * (sizeof(GridDev) + sizeof(TileDiv)) + 8192 <= kNoAllocBytes,
              "fixed batch table too small for GMES_NOALLOC_MAX_GRIDS grids");

// The batch tables of gmes_batch_step_noalloc.  Host code never touches this
// symbol directly: its device address comes from cudaGetSymbolAddress.
__device__ __align__(256) char g_noalloc_tables[kNoAllocBytes];

// The tables reach the device as launch arguments of k_noalloc_fill, one
// piece of at most kTableChunk bytes per launch (a launch copies its
// arguments when it is enqueued), so no host buffer has to outlive the call
// and nothing waits for earlier work on the stream.
constexpr int kTableChunk = 24 * 1024;
struct TableChunk {
  int64_t offset;  // byte offset into the fixed array
  int32_t words;   // 16-byte words in data
  int32_t pad;
  uint4 data[kTableChunk / 16];
};
static_assert(sizeof(TableChunk) <= 32000, "kernel arguments are limited to 32764 bytes");
static_assert(kNoAllocBytes % 16 == 0 && kTableChunk % 256 == 0, "16-byte words");

__global__ void k_noalloc_fill(char* dst, const __grid_constant__ TableChunk c) {
  uint4* out = reinterpret_cast<uint4*>(dst + c.offset);
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < c.words; w += gridDim.x * blockDim.x)
    out[w] = c.data[w];
}

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[kMaxDevices] = {};          // per device, looked up on first use
alignas(256) char g_noalloc_image[kNoAllocBytes];  // host image, guarded by the mutex
TableChunk g_noalloc_chunk;                        // launch argument, guarded by the mutex

}  // namespace
}  // namespace gmes

extern "C" gmes_status gmes_batch_step_noalloc(const gmes_grid_desc* const* grids,
                                               const int32_t* steps, int32_t njobs,
                                               int32_t nsteps, int32_t bx_cap, void* stream) {
  if (grids == nullptr || steps == nullptr) return fail(GMES_ERR_VALUE, "NULL argument");
  if (njobs < 1 || njobs > GMES_NOALLOC_MAX_GRIDS)
    return fail(GMES_ERR_VALUE, "njobs = %d outside [1, %d] (the fixed table's capacity)",
                njobs, GMES_NOALLOC_MAX_GRIDS);
  if (nsteps < 0) return fail(GMES_ERR_VALUE, "nsteps = %d must be >= 0", nsteps);
  if (bx_cap < 0 || bx_cap > 5) return fail(GMES_ERR_VALUE, "bx_cap = %d outside [0, 5]", bx_cap);
  if (bx_cap == 0) bx_cap = 4;  // 16-cell rows, as the single-grid kernel
  const BatchLayout L = batch_layout(njobs);
  if (L.total > kNoAllocBytes)
    return fail(GMES_ERR_RUNTIME, "batch tables of %lld bytes exceed the fixed %lld",
                (long long)L.total, (long long)kNoAllocBytes);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(GMES_ERR_RUNTIME, "device %d unsupported", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_addr[dev] == nullptr) {
    void* addr = nullptr;
    e = cudaGetSymbolAddress(&addr, g_noalloc_tables);
    if (e != cudaSuccess) return cuda_fail(e, "looking up the fixed batch table");
    g_noalloc_addr[dev] = addr;
  }
  char* img = g_noalloc_image;
  std::memset(img, 0, (size_t)L.total);
  GridDev* jobs = reinterpret_cast<GridDev*>(img + L.jobs);
  int64_t* tp = reinterpret_cast<int64_t*>(img + L.tile_prefix);
  TileDiv* td = reinterpret_cast<TileDiv*>(img + L.td);
  int32_t* stp = reinterpret_cast<int32_t*>(img + L.steps);
  int64_t* gp = reinterpret_cast<int64_t*>(img + L.ghost_prefix);
  int32_t* sp = reinterpret_cast<int32_t*>(img + L.src_prefix);
  int32_t precision = -1;
  bool disp = false;
  for (int q = 0; q < njobs; ++q) {
    const gmes_grid_desc* g = grids[q];
    gmes_status st = check_desc(g, true);
    if (st != GMES_OK) return fail(st, "grid %d: %s", q, g_last_error.c_str());
    if (g->ntfsf > 0) return fail(GMES_ERR_VALUE, "grid %d has a TFSF source: not batchable", q);
    if (g->nprobe > 0) return fail(GMES_ERR_VALUE, "grid %d has probes: not batchable", q);
    if (g->flags & GMES_FLAG_COMPLEX)
      return fail(GMES_ERR_VALUE, "grid %d is complex: not batchable", q);
    if (precision < 0) precision = g->precision;
    if (g->precision != precision)
      return fail(GMES_ERR_VALUE, "grid %d: all grids must share one precision", q);
    if (steps[q] < 0 || steps[q] > nsteps)
      return fail(GMES_ERR_VALUE, "steps[%d] = %d outside [0, nsteps]", q, steps[q]);
    if (g->nsrc > 0 && steps[q] > g->src_steps)
      return fail(GMES_ERR_VALUE, "steps[%d] exceeds the grid's source-value capacity", q);
    disp = disp || (g->flags & GMES_FLAG_DISPERSIVE);
    jobs[q] = make_grid_dev(*g);
    if (!offsets_fit_i32(jobs[q]))
      return fail(GMES_ERR_VALUE,
                  "grid %d has a component of 2^31 or more points: step it alone, not in a batch",
                  q);
    int l = 0;
    while (l < bx_cap && (1 << l) < g->n[2]) ++l;
    td[q] = tile_div(l, g->n);
    const int64_t tiles = (int64_t)td[q].plane * g->n[0];
    tp[q + 1] = tp[q] + tiles;
    gp[q + 1] = gp[q] + 6 * max_ghost_plane(jobs[q]);
    sp[q + 1] = sp[q] + g->nsrc;
    stp[q] = steps[q];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* dst = static_cast<char*>(g_noalloc_addr[dev]);
  for (int64_t off = 0; off < L.total; off += kTableChunk) {
    TableChunk& c = g_noalloc_chunk;
    const int64_t bytes = L.total - off < kTableChunk ? L.total - off : kTableChunk;
    c.offset = off;
    c.words = (int32_t)(bytes / 16);
    c.pad = 0;
    std::memcpy(c.data, img + off, (size_t)bytes);
    k_noalloc_fill<<<8, 256, 0, s>>>(dst, c);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "uploading the fixed batch table");
  }
  gmes_batch b;
  b.njobs = njobs;
  b.precision = precision;
  b.dispersive = disp ? 1 : 0;
  b.srcs = sp[njobs];
  b.tiles = tp[njobs];
  b.ghosts = gp[njobs];
  b.workspace = g_noalloc_addr[dev];
  b.workspace_bytes = kNoAllocBytes;
  if (nsteps == 0) return GMES_OK;
  e = launch_batch(batch_view(b), jobs, precision, disp, nsteps, 0, s);
  if (e != cudaSuccess) return cuda_fail(e, "launching batch kernels");
  return GMES_OK;
}
