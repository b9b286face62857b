/*
 * gmes_gb300 -- C ABI of the GB300 FDTD time-stepping engine.
 *
 * This library replaces the hot path of the GMES electromagnetic solver:
 * one FDTD time step, i.e. the ghost-plane copies
 * (gmes/fdtd.py:811-1097), the per-component material updates dispatched
 * by FDTD.update_ex ... update_hz (gmes/fdtd.py:673-809) to the C++
 * per-point updaters PwMaterial<T>::update_all (src/pw_material.hh:66-73,
 * src/pw_dielectric.hh, src/pw_cpml.hh, src/pw_upml.hh, src/pw_drude.hh,
 * src/pw_lorentz.hh, src/pw_dcp.hh), and the point-source updates
 * (gmes/pw_source.py:74-131), in the order of FDTD.step()
 * (gmes/fdtd.py:1099-1122).
 *
 * The reference binds one C++ object per (material, component) through
 * SWIG (src/pw_material.i); each object owns an array-of-structs list of
 * points with their parameters and state.  Here a grid is described once by
 *   - a u8 class map per field component (same array shape as the field),
 *   - a table of update classes with their physical parameters,
 *   - the PML layers' grading parameters,
 * and the engine computes every update coefficient from those parameters
 * in FP64 on the GPU (gmes_build_coefficients).
 *
 * Conventions
 *   - All functions return a gmes_status; 0 is success.  The message of the
 *     last failure on the calling thread is returned by gmes_last_error().
 *     The status classes mirror the exception mapping of the reference's
 *     binding (src/pw_material.i:23-33): bad argument -> ValueError,
 *     out of range -> IndexError, everything else -> RuntimeError.
 *   - Every buffer in gmes_grid_desc is DEVICE memory allocated by the
 *     caller (gmes_grid_sizes() gives the sizes).  The library itself
 *     allocates no device memory: host inputs are staged through a region
 *     of the caller's coefficient block.
 *   - Arrays are C-ordered (k fastest), exactly the reference's numpy
 *     layout (gmes/geometry.py:276-358).
 *   - Work is enqueued on the caller's stream (cudaStream_t passed as
 *     void*; NULL = legacy default stream).  Calls on one grid must not
 *     overlap on the device.
 */
#ifndef GMES_GB300_H_
#define GMES_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GMES_ABI_VERSION 6
#define GMES_MAX_CLASSES 256 /* class ids are u8 */
#define GMES_MAX_PML 4       /* PML materials per grid */
#define GMES_MAX_POLES 8     /* Drude/Lorentz poles, DCP terms per class */

typedef enum {
  GMES_OK = 0,
  GMES_ERR_VALUE = 1,   /* invalid argument (reference: std::invalid_argument) */
  GMES_ERR_INDEX = 2,   /* index out of range (reference: std::out_of_range) */
  GMES_ERR_RUNTIME = 3, /* any other failure */
  GMES_ERR_CUDA = 4     /* a CUDA call failed; the message has the CUDA error */
} gmes_status;

typedef enum {
  GMES_FP64 = 0,        /* IEEE FP64 storage and arithmetic, FMA-contracted */
  GMES_FP32 = 1,        /* FP32 storage and arithmetic, FP64-derived coefficients */
  GMES_DF64 = 2,        /* float-float pairs (48-bit significand), FP32 pipes */
  GMES_FP64_STRICT = 3  /* FP64 in the reference's exact operation order, no FMA */
} gmes_precision;

/* Update kinds (one per reference updater family). */
typedef enum {
  GMES_KIND_DUMMY = 0,      /* src/pw_dummy.hh: no update */
  GMES_KIND_DIELECTRIC = 1, /* src/pw_dielectric.hh */
  GMES_KIND_CPML = 2,       /* src/pw_cpml.hh */
  GMES_KIND_UPML = 3,       /* src/pw_upml.hh */
  GMES_KIND_DRUDE = 4,      /* src/pw_drude.hh (E side; H side is DIELECTRIC) */
  GMES_KIND_LORENTZ = 5,    /* src/pw_lorentz.hh */
  GMES_KIND_DCP = 6,        /* src/pw_dcp.hh, DcpAde* (ADE form) */
  GMES_KIND_CONST = 7,      /* src/pw_const.hh */
  GMES_KIND_DCP_PLRC = 8    /* src/pw_dcp.hh:406-746, DcpPlrc* (PLRC / RC forms) */
} gmes_kind;

/* gmes_grid_desc.flags */
#define GMES_FLAG_DISPERSIVE 1 /* some E class is DRUDE, LORENTZ or DCP */
/* Complex fields (the reference's Cmplx updaters with a Bloch boundary,
   src/pw_material.i:387, gmes/fdtd.py:811-1097).  Every field, state,
   source-value and probe buffer holds its real plane followed by its
   imaginary plane (twice gmes_grid_sizes' real size); the update
   coefficients are real, so the two planes are updated independently and
   couple only through the Bloch phases of the ghost copies.  FP64 and
   FP64_STRICT only. */
#define GMES_FLAG_COMPLEX 2
/* Every warp of the cell kernels takes the per-point path.  By default a
   warp whose points all carry the same dielectric class per component
   updates them without the per-point kind look-ups and branches; the
   arithmetic is the same, so the fields are bit-identical either way (a
   switch for tests and measurements).  No counterpart in the reference. */
#define GMES_FLAG_POINTWISE 4

/* Field components: bit c of gmes_grid_desc.active. */
enum { GMES_EX = 0, GMES_EY = 1, GMES_EZ = 2, GMES_HX = 3, GMES_HY = 4, GMES_HZ = 5 };

/*
 * One update class of one component, with physical parameters
 * (replaces the per-point <Model>ElectricParam / MagneticParam structs,
 * src/pw_material.i:215-348).  Parameters live in a double pool:
 *   DIELECTRIC, CPML, UPML, DUMMY: none
 *   CONST:   value (complex grids: value, imaginary part)
 *   DRUDE:   eps_inf, sigma, then (omega, gamma) per pole   (src/material.pyx:1546-1565)
 *   LORENTZ: eps_inf, sigma, then (amp, omega, gamma) per pole (src/material.pyx:1727-1746)
 *   DCP:     eps_inf, sigma, (omega, gamma) per Drude term,
 *            (amp, cos phi, sin phi, omega, gamma) per critical point
 *            (src/material.pyx:1074-1105; the phase enters only through
 *            cos/sin, supplied by the caller's libm)
 *   DCP_PLRC: eps_inf, sigma, rc (1: the RC form, DcpRc), then per Drude
 *            term (omega, gamma, exp(-gamma dt), exp(gamma dt),
 *            tanh(gamma dt / 2)), per critical point (amp, omega, gamma,
 *            cos phi, sin phi, re/im of exp(-dt (gamma + i omega)), re/im of
 *            exp(dt (gamma + i omega))) (src/material.pyx:1227-1490; the
 *            caller's libm supplies every transcendental value, the GPU does
 *            the complex arithmetic)
 */
typedef struct {
  int32_t kind;      /* gmes_kind */
  int32_t pml;       /* index into the PML list for CPML/UPML, else -1 */
  int32_t npole;     /* Drude/Lorentz poles, or DCP Drude terms */
  int32_t ncp;       /* DCP critical points */
  int32_t param_off; /* first parameter in the parameter pool */
  int32_t nparam;
  double eps;        /* eps_inf (E) or mu_inf (H) the update divides by */
} gmes_class_desc;

/* Grading of one PML material (src/material.pyx:442-502, 558-591, 795-820). */
typedef struct {
  int32_t kind;         /* GMES_KIND_CPML or GMES_KIND_UPML */
  int32_t pad;
  double sigma_max[3];  /* sigma_max_ratio * sigma_opt, per axis */
  double m;             /* grading order of sigma and kappa */
  double kappa_max;
  double m_a;           /* CPML only: grading order of a */
  double a_max;         /* CPML only */
  double d;             /* slab thickness */
  double center[3];
  double half_size[3];  /* +inf on an axis whose half size is below d */
} gmes_pml_desc;

/*
 * One point of a total-field/scattered-field (TFSF) plane-wave source: the
 * consistency corrections of the reference's Transparent{E,H}? sources
 * (gmes/pw_source.py:134-486) at a point of the TFSF box faces.  After the
 * material update and the point sources of its half, face f adds
 *     field += coef[f] * (r0[f] * A[sample[f]] + r1[f] * A[sample[f] + 1])
 * in face order, where A is the incident-field grid's Hy array for an E
 * point and its Ex array for an H point; coef[f] is the signed
 * dt / (eps_or_mu * d) * amp of that face (gmes/source.py:616-665).
 */
#define GMES_TFSF_MAX_FACES 4
typedef struct {
  int32_t comp;     /* field component of the point */
  int32_t nface;    /* 1 .. GMES_TFSF_MAX_FACES */
  int64_t offset;   /* linear index into the component's array */
  double coef[GMES_TFSF_MAX_FACES];
  double r0[GMES_TFSF_MAX_FACES];
  double r1[GMES_TFSF_MAX_FACES];
  int64_t sample[GMES_TFSF_MAX_FACES];
} gmes_transparent;

/* One probe point (the reference's Probe, gmes/file_io.py:9-48). */
typedef struct {
  int32_t comp;   /* field component 0..5 */
  int32_t pad;
  int64_t offset; /* linear index into the component's array */
} gmes_probe;

/* One point source, resolved to one Yee point (gmes/pw_source.py:74-131). */
typedef struct {
  int32_t comp;   /* field component 0..5 */
  int32_t mode;   /* 0: field = value (hard); 1: field -= value (current) */
  int64_t offset; /* linear C-order index into the component's array */
} gmes_point_source;

/*
 * The grid: shape, step sizes and the caller-allocated device buffers.
 * Sizes in bytes of each buffer are given by gmes_grid_sizes().
 */
typedef struct gmes_grid_desc {
  int32_t abi_version;   /* GMES_ABI_VERSION */
  int32_t precision;     /* gmes_precision */
  int32_t n[3];          /* Cartesian.whole_field_size */
  int32_t active;        /* bit c set: component c is updated */
  int32_t naux[6];       /* state slots per point of component c (see below) */
  int32_t nclass[6];     /* number of classes of component c */
  int32_t npml;
  int32_t nsrc;
  int32_t nparam;        /* doubles in the class parameter pool */
  int32_t src_steps;     /* capacity of src_val in steps */
  int32_t flags;         /* GMES_FLAG_* */
  int32_t reserved;
  double dr[3];          /* dx, dy, dz */
  double half[3];        /* Cartesian.half_size (origin of the Yee coordinates) */
  double dt;
  /* device buffers */
  void* field[6];        /* element type by precision: double, float, float2 */
  uint8_t* cls[6];       /* class map of each active component */
  void* aux[6];          /* naux[c] slots x (points of c), same element type */
  void* coef;            /* coefficient block, written by gmes_build_coefficients */
  gmes_point_source* src;/* nsrc point sources */
  double* src_val;       /* source values, [step][source] (see gmes_step) */
  /* TFSF plane-wave source (optional): the 1-D incident-field grid (a TEMz
     grid, Ex and Hy, same precision and dt) is advanced one full step
     between this grid's E and H halves, as FDTD.step does with the
     aux_fdtd of TotalFieldScatteredField (gmes/fdtd.py:1099-1122,
     gmes/source.py:422-425); ntfsf transparent points correct the fields
     on the TFSF box faces.  Grids with a TFSF source cannot be batched. */
  int32_t ntfsf;
  int32_t reserved2;
  gmes_transparent* tfsf;
  const struct gmes_grid_desc* incident;
  /* Probes (optional): after each half's updates and sources, step s of a
     gmes_step call writes the value of every probe of that half's
     components to probe_val[s * nprobe + q] (FP64), as FDTD.step writes
     its E and H recorders (gmes/fdtd.py:1107-1122). */
  int32_t nprobe;
  int32_t probe_steps;   /* capacity of probe_val in steps */
  gmes_probe* probe;
  double* probe_val;
  /* Complex grids: the ghost plane along the h-th curl axis (h = 0: own+1,
     h = 1: own+2) of component c receives bloch_phase[c][h] = (re, im)
     times its source plane, the two axes in that order (corners get both
     factors); the reference's exp(1j k_a (x_dest - x_src)). */
  double bloch_phase[6][2][2];
} gmes_grid_desc;
/*
 * State slots (naux) per kind, the same state the reference keeps inside
 * each point's parameter struct:
 *   CPML 2 (psi1, psi2); UPML 1 (d or b); DRUDE/LORENTZ 2 per pole
 *   (q_now, q_new); DCP 1 + 2 per Drude term + 2 per critical point
 *   (e_old, q_old/q_now, p_old/p_now).  naux[c] is the maximum over the
 *   classes of component c.
 */

/* Element size in bytes of a field or state value at this precision. */
int gmes_elem_size(int32_t precision);

/* Array shape of component c (1,1,1 when inactive). */
gmes_status gmes_field_shape(const gmes_grid_desc* g, int32_t comp, int64_t shape[3]);

/*
 * Bytes of each device buffer the caller must allocate:
 *   sizes[0..5]   field[c]        sizes[6..11]  cls[c]
 *   sizes[12..17] aux[c]          sizes[18]     coef
 *   sizes[19]     src             sizes[20]     src_val for one step
 * (complex grids: field, aux and src_val sizes include both planes)
 */
gmes_status gmes_grid_sizes(const gmes_grid_desc* g, int64_t sizes[21]);

/*
 * Compute every update coefficient in FP64 on the GPU from the class
 * table, the parameter pool and the PML list, and write the coefficient
 * block g->coef (replaces Material.init / get_pw_material_* coefficient
 * assembly, src/material.pyx).  Host arrays: classes[6][nclass[c]]
 * (component-major, concatenated), params (the pool), pmls[npml].
 * Synchronous on `stream`.
 */
gmes_status gmes_build_coefficients(const gmes_grid_desc* g, const gmes_class_desc* classes,
                                    const double* params, const gmes_pml_desc* pmls,
                                    void* stream);

/*
 * Optional: overwrite the PML profile of (pml, comp, axis) with host values,
 * for bit-exact comparisons with a CPU implementation whose exp/pow differ
 * in the last ulp.  values: n = shape[axis] rows of 3 doubles, CPML
 * (b, c, kappa) or UPML (sigma, kappa, unused); the derived coefficients
 * are recomputed on the GPU from them.  Synchronous on `stream`.
 */
gmes_status gmes_set_pml_profile(const gmes_grid_desc* g, int32_t pml, int32_t comp,
                                 int32_t axis, const double* values, void* stream);

/*
 * Read back the FP64 profile of (pml, comp, axis) as computed on the GPU:
 * shape[axis] rows of 5 doubles, CPML (b, c, kappa, c/d, 1/(kappa d)) or
 * UPML (c1, c2, c4, c5, c6).  Synchronous on `stream`.
 */
gmes_status gmes_get_pml_profile(const gmes_grid_desc* g, int32_t pml, int32_t comp,
                                 int32_t axis, double* out, void* stream);

/*
 * Non-finite guard: sets *flag (an int32 in DEVICE memory) to 1 when any
 * field value of the grid (both planes of a complex grid) is an infinity or
 * a NaN, as a simulation past its stability limit produces; it never clears
 * the flag.  The reference has no device state to watch: a failure in its
 * binding surfaces to the caller as an exception and leaves everything else
 * untouched (src/cpp23_support.hh:155-173, src/pw_material.i:23-33).  A
 * server reads the flag between chunks and fails that job alone.
 * Asynchronous on `stream`.
 */
gmes_status gmes_nonfinite(const gmes_grid_desc* g, int32_t* flag, void* stream);

/* Zero every field and state buffer (FDTD.init's zero fields). */
gmes_status gmes_reset(const gmes_grid_desc* g, void* stream);

/*
 * Advance `nsteps` full time steps starting at step index `step0`
 * (FDTD.step(), gmes/fdtd.py:1099-1122): H ghost copy, E update, E
 * sources, E ghost copy, H update, H sources.  Source values are read from
 * g->src_val: for step s (0-based within this call) the E value of source
 * q is src_val[(2*s) * nsrc + q] and the H value src_val[(2*s+1) * nsrc + q].
 */
gmes_status gmes_step(const gmes_grid_desc* g, int32_t nsteps, void* stream);

/*
 * One half of step `step` (0-based index into src_val, < src_steps when
 * there are sources): side 0 = H ghost copy, E update, E sources; side 1 =
 * E ghost copy, H update, H sources.  gmes_step(g, n) is n pairs of these.
 */
gmes_status gmes_half_step(const gmes_grid_desc* g, int32_t side, int32_t step, void* stream);

/*
 * Batches: several grids (jobs) advanced together, one launch per kernel
 * kind per half-step for the whole batch (the serving path).  The caller
 * allocates a device workspace of gmes_batch_workspace_size(njobs) bytes;
 * gmes_batch_prepare() writes the per-grid views and work prefix sums into
 * it and fills *out.  All grids of a batch share one precision and must not
 * be stepped through any other call while the batch runs.  No reference
 * counterpart: the reference runs one simulation per process.
 */
typedef struct {
  int32_t njobs;
  int32_t precision;
  int32_t dispersive;    /* some grid has GMES_FLAG_DISPERSIVE */
  int32_t srcs;          /* point sources over all grids */
  int64_t tiles;         /* blocks of one half-step over all grids */
  int64_t ghosts;        /* ghost-copy work items over all grids */
  void* workspace;       /* device */
  int64_t workspace_bytes;
} gmes_batch;

int64_t gmes_batch_workspace_size(int32_t njobs);

/* bx_cap: log2 of the largest block extent along k (0..5; 0 = default 4). */
gmes_status gmes_batch_prepare(const gmes_grid_desc* const* grids, int32_t njobs,
                               void* workspace, int64_t workspace_bytes, int32_t bx_cap,
                               gmes_batch* out, void* stream);

/*
 * Steps each grid takes in the next chunk: host array of njobs, copied in
 * stream order (it must stay valid until the stream reaches the copy).
 */
gmes_status gmes_batch_set_steps(const gmes_batch* b, const int32_t* steps, void* stream);

/*
 * Advance a chunk of nsteps steps: grid g takes steps 0 .. steps[g]-1 of
 * the chunk, reading its source values from its own src_val at those step
 * slots.  blocks: grid size of the persistent update kernel (0 = one block
 * per tile).
 */
gmes_status gmes_batch_step(const gmes_batch* b, int32_t nsteps, int32_t blocks, void* stream);
/* (For batches of at most 20 grids the cell kernel takes the grids'
   descriptors as launch arguments: gmes_batch_prepare keeps a host copy of
   the last 64 prepared batches' descriptors, keyed by workspace address.
   Results are the same either way.) */

/*
 * Batch step that allocates nothing.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory: a process whose memory
 * pool already owns the GPU's free memory and forbids further cudaMalloc
 * (a serving host, or a plugin inside a framework that controls
 * allocation), and latency-sensitive loops that must not pay the implicit
 * device synchronisation a cudaMalloc can cost.  Instead of a caller
 * workspace, the batch tables live in one fixed array in the library's
 * device memory, sized for at most GMES_NOALLOC_MAX_GRIDS grids; every GPU
 * that loads the library keeps that array until the process exits.  The
 * call rebuilds the tables for `grids` (same rules as gmes_batch_prepare),
 * then advances grid g by steps[g] of the nsteps steps (same as
 * gmes_batch_set_steps + gmes_batch_step), reading each grid's staged
 * source values.  The tables reach that array as the launch arguments of
 * small copy kernels enqueued on `stream`, so the call does not wait for
 * earlier work on the stream and no host buffer outlives it.
 *   - The first call on a device also looks up that array's device address
 *     (with the device current); make that first call before any stream
 *     capture.
 *   - All calls share the one array: calls that overlap on the GPU (other
 *     streams, other threads) race and corrupt each other's tables.
 *     Calls on one stream are ordered.
 *   - More than GMES_NOALLOC_MAX_GRIDS grids is rejected with
 *     GMES_ERR_VALUE.
 *   - On success no host or device memory is allocated or freed.
 */
#define GMES_NOALLOC_MAX_GRIDS 64
gmes_status gmes_batch_step_noalloc(const gmes_grid_desc* const* grids, const int32_t* steps,
                                    int32_t njobs, int32_t nsteps, int32_t bx_cap,
                                    void* stream);

/*
 * CUDA graphs of whole chunks (stream capture of gmes_step / gmes_batch_step
 * on a non-default stream).  The graph bakes in the descriptors' device
 * pointers: replay it only while the same buffers are alive.
 */
gmes_status gmes_graph_capture_step(const gmes_grid_desc* g, int32_t nsteps, void* stream,
                                    void** graph_exec);
gmes_status gmes_graph_capture_batch(const gmes_batch* b, int32_t nsteps, int32_t blocks,
                                     void* stream, void** graph_exec);
gmes_status gmes_graph_launch(void* graph_exec, void* stream);
gmes_status gmes_graph_destroy(void* graph_exec);

/*
 * Asynchronous copy of `bytes` bytes between host and device memory on
 * `stream` (direction from the pointers; pinned host memory makes it truly
 * asynchronous).  Used to stage a chunk's source values ahead of its launch
 * (the per-step host inputs of gmes/pw_source.py:80) without a runtime call
 * from the host language.  bytes == 0 is a no-op; a negative size or a NULL
 * pointer with bytes > 0 is GMES_ERR_VALUE.
 */
gmes_status gmes_copy_async(void* dst, const void* src, int64_t bytes, void* stream);

/*
 * Material-map builder on the GPU (replaces the per-point Python loop of
 * FDTD.init_material_*, gmes/fdtd.py:353-477, and the geometry tree lookups
 * of src/pygeom.pyx:300-454).  Every point of component `comp` takes the
 * LAST shape of the list that contains it (shape 0 when none of shapes
 * 1.. does: find_object, src/pygeom.pyx:143-156); for a compound owner
 * (a PML) the "underneath" shape is the last earlier shape containing the
 * point.  The class id written is lut[owner * (nshapes + 1) + under + 1]
 * (under = -1 for a non-compound owner); ghost planes get class 0.
 * shapes and lut are DEVICE arrays.  Inclusion tests use the reference's
 * FP64 arithmetic (src/pygeom.pyx:538-1148) without multiply-add fusion.
 */
enum { GMES_SHAPE_ALL = 0, GMES_SHAPE_SPHERE = 1, GMES_SHAPE_BLOCK = 2,
       GMES_SHAPE_ELLIPSOID = 3, GMES_SHAPE_CONE = 4, GMES_SHAPE_SHELL = 5 };

typedef struct {
  int32_t type;         /* GMES_SHAPE_* */
  int32_t compound;     /* 1: the shape's material takes eps/mu from underneath */
  int32_t nbox;         /* SHELL: slab boxes in box_lo/box_hi */
  int32_t pad;
  double lo[3], hi[3];  /* bounding box (inclusive); a point outside is not inside */
  double center[3];
  double m[9];          /* BLOCK/ELLIPSOID: projection onto the edge axes, row-major */
  double p[3];          /* SPHERE: radius; BLOCK: half sizes; ELLIPSOID: 2 / sizes;
                           CONE: radius, radius2, height */
  double axis[3];       /* CONE: unit axis */
  double box_lo[6][3];  /* SHELL slabs */
  double box_hi[6][3];
} gmes_shape;

gmes_status gmes_rasterize(const gmes_grid_desc* g, int32_t comp, const gmes_shape* shapes,
                           int32_t nshapes, const uint8_t* lut, void* stream);

/* Copy a component between host and device memory (numpy <-> GPU). */
gmes_status gmes_read_field(const gmes_grid_desc* g, int32_t comp, double* host_out,
                            void* stream);
gmes_status gmes_write_field(const gmes_grid_desc* g, int32_t comp, const double* host_in,
                             void* stream);

/*
 * Differentiation (no counterpart in the reference, which has no adjoint).
 *
 * A batch of TMz designs shares one grid (geometry, CPML, sources: a
 * gmes_grid_desc with active = Ez|Hx|Hy, n[2] = 1, built as usual) and
 * differs only in the permittivity of a rectangular design box of Ez
 * points.  The forward kernels advance the batch and record the Ez values
 * of a monitor box after every step; gmes_tmz_objective gives
 *     J_b = dt * sum_{n=1..N} sum_{monitor} Ez_n^2;
 * gmes_tmz_adjoint runs the time-reversed (transposed) step and
 * accumulates dJ_b/deps into grad.  Steps are numbered 1..total_steps;
 * step n takes the state after n-1 steps to the state after n steps.
 *
 * Fields live on a periodic nx x ny lattice per design, without the
 * reference's ghost planes: Ez[i,j,0], Hx[i,j+1,1], Hy[i+1,j,1] of the grid
 * arrays are lattice point (i, j) of arrays 0, 1, 2.  Supported classes
 * of Ez, Hx, Hy: DIELECTRIC, CPML, DUMMY (gmes_tmz_check rejects others);
 * the design box must lie on DIELECTRIC Ez points.
 */
#define GMES_TMZ_RECORD_MONITOR 1 /* forward: write the monitor rows of these steps */
#define GMES_TMZ_RECORD_HIST 2    /* forward: write the design increments (slot = step - step0 - 1) */
#define GMES_TMZ_MAX_BLOCK_STEPS 4 /* most steps one launch of the FP32 kernels advances */

typedef struct {
  int32_t nbatch;        /* designs */
  int32_t design_lo[2];  /* lattice (i, j) of the design box's first point */
  int32_t design_n[2];   /* design box extent */
  int32_t monitor_lo[2];
  int32_t monitor_n[2];
  int32_t nsrc;          /* point sources: comp 2 (Ez), 3 (Hx), 4 (Hy); offset = i * ny + j */
  int32_t total_steps;   /* rows of monitor and src_val */
  int32_t hist_steps;    /* capacity of hist in steps (one checkpoint segment) */
  int32_t block_steps;   /* FP32: steps per launch, 0 = GMES_TMZ_MAX_BLOCK_STEPS (temporally
                            blocked kernels), 1 = one step per launch; the results are
                            bit-identical for every value.  Other precisions: one step. */
  /* device buffers (sizes from gmes_tmz_sizes) */
  void* state;           /* 7 arrays [nbatch][nx][ny]: Ez, Hx, Hy and the 4 CPML psi */
  void* adjoint;         /* 11 arrays: adjoints of Ez, Hx, Hy and 2 x 4 psi adjoints */
  void* design;          /* per-pixel coefficients and each lattice point's resolved update,
                            written by gmes_tmz_set_design */
  void* hist;            /* [hist_steps][nbatch][design points] Ez increments */
  double* monitor;       /* [nbatch][total_steps][monitor points] */
  double* grad;          /* [nbatch][design points] dJ_b / deps */
  const double* weight;  /* [nbatch] seed scale of each J_b (dL/dJ_b), or NULL for 1 */
  const gmes_point_source* src;
  const double* src_val; /* [total_steps][2][nsrc]: E-half and H-half values */
  void* scratch;         /* second copy of the state for the temporally blocked kernels,
                            which read one copy and write the other (size 0 and unused
                            when every launch takes one step) */
} gmes_tmz_batch;

/* Bytes of state, adjoint, design, hist, monitor, grad, scratch. */
gmes_status gmes_tmz_sizes(const gmes_grid_desc* g, const gmes_tmz_batch* b, int64_t sizes[7]);
/* Validate the classes of Ez/Hx/Hy and the design box against the grid's
   coefficient block and class maps (synchronous: copies them to the host). */
gmes_status gmes_tmz_check(const gmes_grid_desc* g, const gmes_tmz_batch* b);
/* Design coefficients from eps (device, [nbatch][design points], > 0), and
   the resolved update of every lattice point (flags and coefficients). */
gmes_status gmes_tmz_set_design(const gmes_grid_desc* g, const gmes_tmz_batch* b,
                                const double* eps, void* stream);
/* Zero the state (what & 1) and/or the adjoint and grad (what & 2). */
gmes_status gmes_tmz_reset(const gmes_grid_desc* g, const gmes_tmz_batch* b, int32_t what,
                           void* stream);
/* Steps step0+1 .. step0+nsteps forward; flags GMES_TMZ_RECORD_*. */
gmes_status gmes_tmz_forward(const gmes_grid_desc* g, const gmes_tmz_batch* b, int32_t step0,
                             int32_t nsteps, int32_t flags, void* stream);
/* J[b] (device, nbatch doubles) from the first nsteps monitor rows. */
gmes_status gmes_tmz_objective(const gmes_grid_desc* g, const gmes_tmz_batch* b,
                               int32_t nsteps, double* J, void* stream);
/* Steps step0+nsteps down to step0+1 backward, seeding each with its
   monitor row; needs the hist of the same steps (a forward call with
   GMES_TMZ_RECORD_HIST from the state after step0). */
gmes_status gmes_tmz_adjoint(const gmes_grid_desc* g, const gmes_tmz_batch* b, int32_t step0,
                             int32_t nsteps, void* stream);

/*
 * Point-list updaters: the reference's PwMaterial operator objects
 * (<Model><Comp><Real|Cmplx>.update_all, src/pw_material.hh:66-73,
 * src/pw_material.i:138-389).  One call updates the attached points of one
 * updater in place, in the reference's operation order (FP64), reading the
 * two curl inputs with its field_at() collapsed-axis rule.  All pointers are
 * device memory; complex updaters (cmplx = 1) take planar arrays (real plane
 * then imaginary plane) and two planes of param and state.
 * Per-point param layouts (doubles) and state slots:
 *   DIELECTRIC: eps                                  state: -
 *   CPML:  eps, b1, b2, c1, c2, kappa1, kappa2       state: psi1, psi2
 *   UPML:  eps, c1, c2, c3, c4, c5, c6               state: d (E) / b (H)
 *   DRUDE, LORENTZ: a[npole][3], c[3]                state: q_now[npole], q_new[npole]
 *   DCP:   a[npole][3], b[ncp][5], c[4]              state: e_old, q_old, q_now, p_old, p_now
 *   DCP_PLRC: a[npole][3], b[ncp][6] (re/im of b0, b1, b2), c[3]
 *                                                    state: psi_dp[npole], psi_cp[ncp][2]
 *   CONST: value                                     state: -
 * Points outside the target array are skipped (the reference raises
 * IndexError before any write; its Python binding checks, as this
 * package's binding does).
 */
typedef struct {
  int32_t comp;          /* field component 0..5 of the target */
  int32_t kind;          /* gmes_kind */
  int32_t npoints;
  int32_t nparam;        /* doubles per point */
  int32_t nstate;        /* state slots per point */
  int32_t npole, ncp;
  int32_t cmplx;
  const int32_t* idx;    /* [npoints][3] */
  const double* param;   /* [planes][npoints][nparam] */
  double* state;         /* [planes][npoints][nstate] */
  int64_t shape[3][3];   /* shapes of the target and the two inputs */
} gmes_points;

gmes_status gmes_points_update(const gmes_points* p, void* inplace, const void* in1,
                               const void* in2, double d1, double d2, double dt, void* stream);

/* Message of the last failed call on this thread ("" if none). */
const char* gmes_last_error(void);

/* GMES_ABI_VERSION of the loaded library. */
int gmes_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GMES_GB300_H_ */
