"""Gradients of a monitor objective with respect to a permittivity design region.

GMES has no adjoint; this module differentiates its TMz time step
(gmes/fdtd.py:1099-1122 with the Dielectric/CPML updaters and point
sources) for a batch of designs that share one scene:

* ``DesignRegion`` -- a rectangle of Ez points whose permittivities are the
  design variables (one value per point);
* ``TMzAdjoint`` -- the batched forward (``forward``), the objective
  ``J_b = dt * sum_{n=1..N} sum_{monitor} Ez_n^2`` and its gradient by the
  hand-written time-reversed kernels (``backward``).  The adjoint needs the
  forward Ez increments on the design points of every step.  Where the
  buffer for all N steps fits (the default when it takes at most a quarter
  of the free device memory), the forward records them and the backward is
  the adjoint sweep alone; otherwise the forward keeps checkpoints of the
  full state every ``segment`` steps (default ceil(sqrt(N))) and the
  backward recomputes each segment's increments before its adjoint steps;
* ``TMzAdjoint.objective(eps)`` -- the same behind ``torch.autograd``.

All work runs in the CUDA library (include/gmes_gb300.h, gmes_tmz_*);
torch provides the device buffers and the autograd hook.
"""

import ctypes as C
import math

import numpy as np

from . import _native as N
from .engine import GridEngine, _torch
from .scene import source_offsets, source_values


class DesignRegion:
    """A rectangle of Ez points of a TMz grid, given in space units.

    ``center`` and ``size`` are (x, y[, z]); z is ignored.  The region is the
    ``round(size / dr)`` Ez points per axis starting at the Ez point nearest
    to ``center - size / 2`` (Ez point (i, j) sits at (i dx - half_x,
    j dy - half_y), gmes/geometry.py:548-566).
    """

    def __init__(self, center, size):
        self.center = tuple(float(v) for v in center)[:2]
        self.size = tuple(float(v) for v in size)[:2]

    def box(self, space):
        """((i0, j0), (n0, n1)) in Ez lattice indices."""
        lo, n = [], []
        for a in range(2):
            dr = space.dr[a]
            cnt = int(round(self.size[a] / dr))
            start = int(round((self.center[a] - self.size[a] / 2 + space.half_size[a]) / dr))
            lo.append(start)
            n.append(max(cnt, 1))
        return tuple(lo), tuple(n)


def _lattice_sources(scene, nsteps):
    """Point sources on the TMz lattice: (comp, mode, i * ny + j) rows and their values.

    Sources on a ghost point of the reference's arrays are dropped: their
    value is overwritten by the next ghost copy before any update reads it.
    """
    nx, ny = scene.n[0], scene.n[1]
    rows, keep = [], []
    for q, (c, mode, off) in enumerate(source_offsets(scene)):
        i, j, k = np.unravel_index(off, scene.shape(c))
        if c == 2 and i < nx and j < ny:
            rows.append((2, mode, int(i) * ny + int(j)))
        elif c == 3 and k == 1 and j >= 1:
            rows.append((3, mode, int(i) * ny + int(j) - 1))
        elif c == 4 and k == 1 and i >= 1:
            rows.append((4, mode, (int(i) - 1) * ny + int(j)))
        else:
            continue
        keep.append(q)
    vals = source_values(scene, scene.dt, 0.0, nsteps)[:, :, keep]
    return rows, np.ascontiguousarray(vals)


class TMzAdjoint:
    """Batched TMz forward and adjoint over one scene.

    ``space``, ``geom_list``, ``src_list``, ``courant_ratio``, ``dt`` are
    those of ``TMzFDTD``.  Ez, Hx and Hy may use Dielectric and Cpml
    materials; the design region must lie on dielectric Ez points.
    ``precision``: "fp32" (FP32 fields and adjoint, FP64-derived
    coefficients, FP64 gradient accumulation), "fp64" or "df64".
    ``block_steps``: FP32 steps per kernel launch (0: the most the
    temporally blocked kernels take, 1: one step per launch); every value
    gives bit-identical fields and gradients.
    ``keep_history``: True records the design increments of all ``nsteps``
    steps in the forward (nsteps x batch x design points x element bytes)
    and skips the backward recompute; False uses √N checkpoints; None
    chooses False when ``segment`` is given, else True when that buffer
    takes at most a quarter of the free device memory.  Both give
    bit-identical J and gradients.
    """

    def __init__(self, space, geom_list, src_list, design, monitor, nsteps, batch=1,
                 precision="fp32", segment=None, courant_ratio=0.99, dt=None, device=None,
                 block_steps=0, keep_history=None):
        from .fdtd import TMzFDTD
        torch = _torch()
        if precision not in ("fp32", "fp64", "df64"):
            raise ValueError("precision must be fp32, fp64 or df64")
        sim = TMzFDTD(space=space, geom_list=geom_list, src_list=src_list,
                      courant_ratio=courant_ratio, dt=dt, verbose=False, precision=precision)
        self.scene = sim.compile()
        self.dt = self.scene.dt
        self.nsteps = int(nsteps)
        if self.nsteps < 1:
            raise ValueError("nsteps must be >= 1")
        self.batch = int(batch)
        self.precision = precision
        self.segment = int(segment) if segment else int(math.ceil(math.sqrt(self.nsteps)))
        self.segment = max(1, min(self.segment, self.nsteps))
        self.grid = GridEngine(self.scene, precision=precision, device=device, use_graphs=False)
        self.device = self.grid.device
        self.lib = self.grid.lib
        (d0, dn) = design.box(space)
        (m0, mn) = monitor.box(space)
        self.design_box = (d0, dn)
        self.monitor_box = (m0, mn)
        self.shape = dn
        rows, vals = _lattice_sources(self.scene, self.nsteps)
        b = N.TmzBatchC()
        b.nbatch = self.batch
        for a in range(2):
            b.design_lo[a], b.design_n[a] = d0[a], dn[a]
            b.monitor_lo[a], b.monitor_n[a] = m0[a], mn[a]
        b.nsrc = len(rows)
        b.total_steps = self.nsteps
        b.block_steps = int(block_steps)
        sizes = (C.c_int64 * 7)()
        if keep_history is None and segment:
            keep_history = False  # a segment length asks for checkpoints
        if keep_history is None:
            b.hist_steps = self.nsteps
            N.check(self.lib.gmes_tmz_sizes(C.byref(self.grid.desc), C.byref(b), sizes))
            free, _ = torch.cuda.mem_get_info(self.device)
            keep_history = sizes[3] <= free // 4
        self.keep_history = bool(keep_history)
        b.hist_steps = self.nsteps if self.keep_history else self.segment
        N.check(self.lib.gmes_tmz_sizes(C.byref(self.grid.desc), C.byref(b), sizes))
        self.sizes = list(sizes)
        dev = self.device

        def buf(n):
            return torch.zeros(max(int(n), 256), dtype=torch.uint8, device=dev)

        self.state = buf(sizes[0])
        self.adjoint = buf(sizes[1])
        self.design = buf(sizes[2])
        self.hist = buf(sizes[3])
        self.monitor = buf(sizes[4])
        self.grad = buf(sizes[5])
        self.scratch = buf(sizes[6]) if sizes[6] > 0 else None
        nd, nb = dn[0] * dn[1], self.batch
        self.eps = torch.ones((nb, nd), dtype=torch.float64, device=dev)
        self.weight = torch.ones(nb, dtype=torch.float64, device=dev)
        self.J = torch.zeros(nb, dtype=torch.float64, device=dev)
        if rows:
            arr = (N.PointSourceC * len(rows))(*[N.PointSourceC(c, m, o) for c, m, o in rows])
            self.src = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(dev)
            self.src_val = torch.from_numpy(vals).to(dev)
            b.src = self.src.data_ptr()
            b.src_val = self.src_val.data_ptr()
        else:
            self.src = self.src_val = None
        b.state = self.state.data_ptr()
        b.adjoint = self.adjoint.data_ptr()
        b.design = self.design.data_ptr()
        b.hist = self.hist.data_ptr()
        b.monitor = self.monitor.data_ptr()
        b.grad = self.grad.data_ptr()
        b.scratch = self.scratch.data_ptr() if self.scratch is not None else None
        b.weight = self.weight.data_ptr()
        self.desc = b
        self.checkpoints = None  # (segments, state bytes), allocated by the first forward
        self.grid.synchronize()
        N.check(self.lib.gmes_tmz_check(C.byref(self.grid.desc), C.byref(b)))
        self._version = 0
        self._have_checkpoints = False

    # -- helpers -------------------------------------------------------------
    def _call(self, name, *args):
        N.check(getattr(self.lib, name)(C.byref(self.grid.desc), C.byref(self.desc), *args))

    def _segments(self):
        for s0 in range(0, self.nsteps, self.segment):
            yield s0 // self.segment, s0, min(self.segment, self.nsteps - s0)

    def lattice(self, k):
        """State array k (0 Ez, 1 Hx, 2 Hy, 3..6 psi) as a (batch, nx, ny) float64 tensor."""
        return self._array(self.state, k)

    def adjoint_field(self, k):
        """Adjoint array k (0 Ez, 1 Hx, 2 Hy) as a (batch, nx, ny) float64 tensor."""
        return self._array(self.adjoint, k)

    def _array(self, block, k):
        torch = _torch()
        nx, ny = self.scene.n[0], self.scene.n[1]
        per = self.batch * nx * ny
        es = 8 if self.precision in ("fp64", "df64") else 4
        stride = ((per * es + 255) // 256) * 256
        raw = block[k * stride:k * stride + per * es]
        self.grid.synchronize()
        if self.precision == "fp64":
            return raw.view(torch.float64).view(self.batch, nx, ny).clone()
        if self.precision == "fp32":
            return raw.view(torch.float32).view(self.batch, nx, ny).double()
        v = raw.view(torch.float32).view(self.batch, nx, ny, 2)
        return v[..., 0].double() + v[..., 1].double()

    def monitor_values(self):
        """(batch, nsteps, monitor points) float64: Ez at the monitor after each step."""
        nm = self.monitor_box[1][0] * self.monitor_box[1][1]
        torch = _torch()
        self.grid.synchronize()
        n = self.batch * self.nsteps * nm
        return self.monitor[:n * 8].view(torch.float64).view(self.batch, self.nsteps, nm).clone()

    # -- forward / backward ----------------------------------------------------
    def _set_design(self, eps):
        torch = _torch()
        e = torch.as_tensor(eps, dtype=torch.float64, device=self.device)
        nd = self.shape[0] * self.shape[1]
        e = e.reshape(self.batch, nd)
        if not bool(torch.isfinite(e).all()) or not bool((e > 0).all()):
            raise ValueError("design permittivities must be positive and finite")
        self.eps.copy_(e)

    def forward(self, eps, checkpoints=True):
        """J (batch,) float64 device tensor for design permittivities eps (batch, n0, n1).

        ``checkpoints``: keep what the backward needs (the design increments
        of every step, or the √N checkpoints).
        """
        self._set_design(eps)
        torch = _torch()
        if self.keep_history:
            g = self.grid
            g._enter()
            st = C.c_void_p(g.stream)
            flags = N.TMZ_RECORD_MONITOR | (N.TMZ_RECORD_HIST if checkpoints else 0)
            self._call("gmes_tmz_set_design", C.c_void_p(self.eps.data_ptr()), st)
            self._call("gmes_tmz_reset", 1, st)
            self._call("gmes_tmz_forward", 0, self.nsteps, flags, st)
            self._call("gmes_tmz_objective", self.nsteps, C.c_void_p(self.J.data_ptr()), st)
            g._leave()
            self._version += 1
            self._have_checkpoints = bool(checkpoints)
            return self.J.clone()
        if checkpoints and self.checkpoints is None:
            nseg = (self.nsteps + self.segment - 1) // self.segment
            self.checkpoints = torch.empty((nseg, self.state.numel()), dtype=torch.uint8,
                                           device=self.device)
        g = self.grid
        g._enter()
        st = C.c_void_p(g.stream)
        self._call("gmes_tmz_set_design", C.c_void_p(self.eps.data_ptr()), st)
        self._call("gmes_tmz_reset", 1, st)
        with torch.cuda.stream(g.torch_stream):
            for seg, s0, k in self._segments():
                if checkpoints:
                    self.checkpoints[seg, :self.state.numel()].copy_(self.state)
                self._call("gmes_tmz_forward", s0, k, N.TMZ_RECORD_MONITOR, st)
            self._call("gmes_tmz_objective", self.nsteps, C.c_void_p(self.J.data_ptr()), st)
        g._leave()
        self._version += 1
        self._have_checkpoints = bool(checkpoints)
        return self.J.clone()

    def backward(self, weight=None):
        """dL/deps (batch, n0, n1) float64 for L = sum_b weight_b J_b of the last forward."""
        if not self._have_checkpoints:
            raise RuntimeError("backward needs a forward run with checkpoints")
        torch = _torch()
        g = self.grid
        if weight is None:
            self.weight.fill_(1.0)
        else:
            self.weight.copy_(torch.as_tensor(weight, dtype=torch.float64,
                                              device=self.device).reshape(self.batch))
        g._enter()
        st = C.c_void_p(g.stream)
        with torch.cuda.stream(g.torch_stream):
            self._call("gmes_tmz_reset", 2, st)
            if self.keep_history:
                # the forward recorded every step's increments (slot = step - 1)
                self._call("gmes_tmz_adjoint", 0, self.nsteps, st)
            for seg, s0, k in ([] if self.keep_history else reversed(list(self._segments()))):
                self.state.copy_(self.checkpoints[seg, :self.state.numel()])
                self._call("gmes_tmz_forward", s0, k, N.TMZ_RECORD_HIST, st)
                self._call("gmes_tmz_adjoint", s0, k, st)
        g._leave()
        nd = self.shape[0] * self.shape[1]
        return self.grad[:self.batch * nd * 8].view(torch.float64).view(
            self.batch, *self.shape).clone()

    def objective(self, eps):
        """J (batch,) as a differentiable function of eps (batch, n0, n1)."""
        return _Objective.apply(eps, self)


def _objective_class():
    torch = _torch()

    class Objective(torch.autograd.Function):
        """J = TMzAdjoint.forward(eps); dJ/deps by the adjoint kernels."""

        @staticmethod
        def forward(ctx, eps, problem):
            J = problem.forward(eps.detach())
            ctx.problem = problem
            ctx.version = problem._version
            ctx.dtype = eps.dtype
            return J

        @staticmethod
        def backward(ctx, gJ):
            p = ctx.problem
            if p._version != ctx.version:
                raise RuntimeError("a later forward call overwrote this forward's checkpoints; "
                                   "call backward before the next forward")
            return p.backward(gJ).to(ctx.dtype), None

    return Objective


class _LazyObjective:
    _cls = None

    def apply(self, *args):
        if _LazyObjective._cls is None:
            _LazyObjective._cls = _objective_class()
        return _LazyObjective._cls.apply(*args)


_Objective = _LazyObjective()

__all__ = ["DesignRegion", "TMzAdjoint"]
