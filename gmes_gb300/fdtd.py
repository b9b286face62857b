"""FDTD simulation classes (interface of the reference's gmes/fdtd.py).

``FDTD(space, geom_list, src_list, courant_ratio=0.99, dt=None, bloch=None,
verbose=True)``, ``init()``, ``step()``, ``step_until_n()``,
``step_until_t()``, ``step_while_zero()`` and the 2-D / 1-D subclasses keep
the reference's signatures and time bookkeeping (gmes/fdtd.py:24-1215,
1470-1593).  The fields live on the GPU; ``sim.ex`` ... ``sim.hz`` are
``FieldView`` objects that read back to numpy on access and write through
to the device on item assignment.  Extra keyword: ``precision`` ("fp64",
"fp64_strict", "fp32", "df64").
"""

from copy import deepcopy
from datetime import datetime
from math import sqrt

import numpy as np

from .constant import Ex, Ey, Ez, Hx, Hy, Hz, COMPONENTS
from .geometry import DefaultMedium, GeomBoxTree, in_range
from .scene import compile_scene


class TimeStep:
    """Current time-step n and time t = n * dt (gmes/fdtd.py:24-50)."""

    def __init__(self, dt, n=0.0, t=0.0):
        self.n = float(n)
        self.t = float(t)
        self.dt = float(dt)

    def half_step_up(self):
        self.n += 0.5
        self.t = self.n * self.dt


def _numpy_binop(name):
    def op(self, other, *rest):
        return getattr(np.asarray(self), name)(other, *rest)
    return op


class FieldView:
    """Numpy-compatible view of one field component held on the GPU.

    Reading (``np.asarray(view)``, indexing, reductions, arithmetic) copies
    the current device values to the host; item assignment writes to the
    device.  ``view.tensor()`` gives the device tensor without a copy.
    """

    def __init__(self, sim, comp):
        self._sim = sim
        self._c = comp.index

    def numpy(self):
        return self._sim._engine.read(self._c)

    def tensor(self):
        return self._sim._engine.read_tensor(self._c)

    def __array__(self, dtype=None, copy=None):
        a = self.numpy()
        return a if dtype is None else a.astype(dtype)

    @property
    def shape(self):
        return self._sim._scene.shape(self._c)

    @property
    def ndim(self):
        return 3

    @property
    def dtype(self):
        return np.dtype(np.complex128 if self._sim.cmplx else np.float64)

    @property
    def size(self):
        return int(np.prod(self.shape))

    def __len__(self):
        return self.shape[0]

    def __getitem__(self, key):
        return self.numpy()[key]

    def __setitem__(self, key, value):
        self._sim._engine.write(self._c, key, value)

    def __getattr__(self, name):
        return getattr(self.numpy(), name)

    def __repr__(self):
        return f"FieldView({self.numpy()!r})"

    __abs__ = lambda self: abs(self.numpy())
    __neg__ = lambda self: -self.numpy()
    __add__ = _numpy_binop("__add__")
    __radd__ = _numpy_binop("__radd__")
    __sub__ = _numpy_binop("__sub__")
    __rsub__ = _numpy_binop("__rsub__")
    __mul__ = _numpy_binop("__mul__")
    __rmul__ = _numpy_binop("__rmul__")
    __truediv__ = _numpy_binop("__truediv__")
    __pow__ = _numpy_binop("__pow__")
    __eq__ = _numpy_binop("__eq__")
    __ne__ = _numpy_binop("__ne__")
    __lt__ = _numpy_binop("__lt__")
    __le__ = _numpy_binop("__le__")
    __gt__ = _numpy_binop("__gt__")
    __ge__ = _numpy_binop("__ge__")


class _PwSummary:
    """Introspection stand-in for one reference updater object (name, idx_size)."""

    def __init__(self, name, count):
        self._name = name
        self._count = count

    def name(self):
        return self._name

    def idx_size(self):
        return self._count


class FDTD:
    """Three-dimensional FDTD simulation (gmes/fdtd.py:53-1467)."""

    def __init__(self, space=None, geom_list=None, src_list=None, courant_ratio=0.99,
                 dt=None, bloch=None, verbose=True, precision="fp64"):
        self._init_field_compnt()
        self.verbose = bool(verbose)
        self.space = space
        self.dx, self.dy, self.dz = self.space.dr
        self.precision = precision
        if bloch is None:
            self.cmplx = False
            self.bloch = None
        else:
            # complex fields; the ghost copies carry the Bloch phase
            # (gmes/fdtd.py:179-208, 811-1097)
            self.cmplx = True
            self.bloch = np.array(bloch, np.double)
        default_medium = next(i for i in geom_list if isinstance(i, DefaultMedium))
        dt_limit = self._dt_limit(space, default_medium.material.eps_inf,
                                  default_medium.material.mu_inf)
        if dt is None:
            self.courant_ratio = float(courant_ratio)
            time_step_size = self.courant_ratio * dt_limit
        else:
            time_step_size = float(dt)
            self.courant_ratio = time_step_size / dt_limit
        self.space.dt = time_step_size
        self.time_step = TimeStep(time_step_size)
        if self.verbose:
            self.space.display_info()
            print("dt:", time_step_size)
            print("courant ratio:", self.courant_ratio)
            if self.cmplx:
                # the numerical Bloch wave vector (Taflove & Hagness eq. 4.14a)
                ds = np.array(self.space.dr)
                mat = default_medium.material
                S = 1 / sqrt(mat.eps_inf * mat.mu_inf) * time_step_size / ds
                print("Bloch wave vector is", self.bloch)
                print("numerical Bloch wave vector is",
                      2 * sqrt(mat.eps_inf) / ds * np.arcsin(np.sin(self.bloch * S * ds / 2) / S))
        self.geom_list = geom_list
        for go in self.geom_list:
            go.init(self.space)
        self.geom_tree = GeomBoxTree(self.geom_list)
        self.src_list = [] if src_list is None else src_list
        for so in self.src_list:
            so.init(self.geom_tree, self.space, self.cmplx)
        self.pw_material = {}
        self.pw_source = {}
        self.e_recorder = []
        self.h_recorder = []
        self._engine = None
        self._scene = None
        self._probes_set = 0

    def _init_field_compnt(self):
        self.e_field_compnt = (Ex, Ey, Ez)
        self.h_field_compnt = (Hx, Hy, Hz)

    def _dt_limit(self, space, eps_inf, mu_inf):
        """Courant bound over the axes the active components use (gmes/fdtd.py:294-321)."""
        ds = {Ex: (1, 2), Ey: (2, 0), Ez: (0, 1), Hx: (1, 2), Hy: (2, 0), Hz: (0, 1)}
        e_ds = set()
        for i in self.e_field_compnt:
            e_ds.update(ds[i])
        h_ds = set()
        for i in self.h_field_compnt:
            h_ds.update(ds[i])
        non_inf = e_ds.intersection(h_ds)
        dr = np.array(space.dr, np.double)
        for i in range(3):
            if i not in non_inf:
                dr[i] = np.inf
        c = 1 / sqrt(eps_inf * mu_inf)
        return 1 / c / sqrt(sum(dr ** -2))

    # -- setup -------------------------------------------------------------
    def compile(self):
        """Compile the scene (class maps, class table, sources) without a GPU."""
        if self._scene is None:
            self._scene = compile_scene(self.space, self.geom_list, self.e_field_compnt,
                                        self.h_field_compnt, self.src_list, self.geom_tree,
                                        self.time_step.dt, bloch=self.bloch)
        return self._scene

    def init(self):
        """Map materials and sources onto the grid and allocate the GPU state."""
        from .engine import GridEngine
        st = datetime.now()
        self.compile()
        self._engine = GridEngine(self._scene, precision=self.precision)
        self.field = {}
        for comp in COMPONENTS:
            view = FieldView(self, comp)
            self.field[comp] = view
            setattr(self, comp.str(), view)
        self._fill_introspection()
        if self.verbose:
            print("Elapsed time:", datetime.now() - st)

    def _fill_introspection(self):
        from .material import KIND_NAMES
        side = {True: "Electric", False: "Magnetic"}
        for comp in self.e_field_compnt + self.h_field_compnt:
            c = comp.index
            out = {}
            per_kind = {}
            for cls_id, count in self._engine.class_counts(c).items():
                kind = self._scene.classes[c][cls_id].kind
                per_kind[kind] = per_kind.get(kind, 0) + count
            for kind, count in per_kind.items():
                name = KIND_NAMES[kind] + side[c < 3]
                out[name] = _PwSummary(name, count)
            self.pw_material[comp] = out
            self.pw_source[comp] = {
                "PointSource" + side[c < 3]: _PwSummary(
                    "PointSource" + side[c < 3],
                    sum(1 for s in self._scene.sources if s.comp.index == c))}
            if self._scene.tfsf is not None:
                n = sum(1 for q in self._scene.tfsf[1] if q[0] == c)
                if n:
                    name = "Transparent" + side[c < 3]
                    self.pw_source[comp][name] = _PwSummary(name, n)

    @property
    def engine(self):
        return self._engine

    @property
    def scene(self):
        return self._scene

    # -- time stepping ----------------------------------------------------
    def _advance(self, nsteps):
        if self._engine is None:
            raise RuntimeError("call init() before stepping")
        if nsteps <= 0:
            return
        n0 = self.time_step.n
        probes = self.e_recorder + self.h_recorder
        if probes:
            if self._engine.probes is None or self._probes_set != len(probes):
                self._engine.set_probes([(p.c, p.offset) for p in probes])
                self._probes_set = len(probes)

            def flush(done, k):
                vals = self._engine.probe_values(k)
                for s in range(k):
                    n = n0 + (done + s)
                    for q, p in enumerate(probes):
                        p.write(n + (0.5 if p.c < 3 else 1.0), vals[s, q])
                for p in probes:
                    p.f.flush()
            self._engine.step(nsteps, n0=n0, on_chunk=flush)
        else:
            self._engine.step(nsteps, n0=n0)
        for _ in range(nsteps):
            self.time_step.half_step_up()
            self.time_step.half_step_up()

    def step(self):
        """One full time step (gmes/fdtd.py:1099-1122)."""
        self._advance(1)

    def _steps_until(self, pred):
        """Number of steps the reference's while-loop would take (same float arithmetic)."""
        ts = TimeStep(self.time_step.dt, self.time_step.n, self.time_step.t)
        k = 0
        while pred(ts):
            ts.half_step_up()
            ts.half_step_up()
            k += 1
        return k

    def step_until_n(self, n=0, modulus=np.inf):
        st = datetime.now()
        k = self._steps_until(lambda ts: ts.n < n)
        self._advance(k)
        if self.verbose:
            print("Elapsed time:", datetime.now() - st)

    def step_until_t(self, t=0, modulus=np.inf):
        st = datetime.now()
        sn = self.time_step.n
        k = self._steps_until(lambda ts: ts.t < t)
        self._advance(k)
        if self.verbose:
            print("Elapsed time:", datetime.now() - st, "(%d timesteps)" % (self.time_step.n - sn))

    def step_while_zero(self, component, point, modulus=np.inf):
        idx = self.space.space_to_index(component, *point)
        if not in_range(idx, self.field[component].shape, component):
            raise ValueError("observation point is outside the simulation domain")
        c = component.index
        while True:
            self.step()
            if float(self._engine.read_tensor(c)[idx].item()) != 0:
                break

    # -- probes and output -------------------------------------------------
    def set_probe(self, p, prefix=None):
        """Record the field at point ``p`` every step into text files (gmes/fdtd.py:607-671)."""
        postfix = {Ex: "_ex.dat", Ey: "_ey.dat", Ez: "_ez.dat", Hx: "_hx.dat",
                   Hy: "_hy.dat", Hz: "_hz.dat"}
        for comp in self.e_field_compnt + self.h_field_compnt:
            idx = self.space.space_to_index(comp, *p)
            if in_range(idx, self.field[comp].shape, comp):
                rec = _Probe(self, comp, idx, (prefix or "") + postfix[comp])
                rec.write_header(self.space.index_to_space(comp, *idx), self.time_step.dt)
                rec.f.flush()
                (self.e_recorder if comp.index < 3 else self.h_recorder).append(rec)

    def write_field(self, comp, low=None, high=None, prefix=None, postfix=None):
        """Save the field window [low, high] of ``comp`` as .npy."""
        data = self.field[comp].numpy()
        if low is not None and high is not None:
            lo = self.space.space_to_index(comp, *low)
            hi = self.space.space_to_index(comp, *high)
            sl = tuple(slice(max(0, lo[a]), min(data.shape[a], hi[a] + 1)) for a in range(3))
            data = data[sl]
        name = (prefix or "") + comp.str() + "_t=" + str(self.time_step.t) + (postfix or "")
        np.save(name + ".npy", data)
        return data

    def __deepcopy__(self, memo=None):
        """Independent copy with the same fields AND the PML/ADE state."""
        memo = {} if memo is None else memo
        new = self.__class__(space=deepcopy(self.space, memo),
                             geom_list=deepcopy(self.geom_list, memo),
                             src_list=deepcopy(self.src_list, memo),
                             courant_ratio=self.courant_ratio, dt=self.time_step.dt,
                             bloch=deepcopy(self.bloch, memo),
                             verbose=self.verbose, precision=self.precision)
        memo[id(self)] = new
        if self._engine is not None:
            new.init()
            pairs = [(new._engine, self._engine)]
            if self._engine.incident is not None:
                pairs.append((new._engine.incident, self._engine.incident))
            for dst, src in pairs:
                for c in range(6):
                    dst.fields[c].copy_(src.fields[c])
                    if src.aux[c] is not None:
                        dst.aux[c].copy_(src.aux[c])
        new.time_step = deepcopy(self.time_step, memo)
        return new


class _Probe:
    """Per-step field recorder writing the reference's text format
    (gmes/file_io.py:9-48): a header, then "n value" per step.  Values come
    from the engine's device probe buffer, one read per chunk of steps."""

    def __init__(self, sim, comp, idx, filename):
        self.sim, self.c, self.idx = sim, comp.index, tuple(int(i) for i in idx)
        sh = sim._scene.shape(self.c) if sim._scene is not None else sim.field[comp].shape
        self.offset = int(np.ravel_multi_index(self.idx, sh))
        self.f = open(filename, "w")

    def write_header(self, loc, dt):
        self.f.write("# location=" + str(loc) + "\n")
        self.f.write("# dt=" + str(dt) + "\n")

    def write(self, n, value):
        v = np.complex128(value) if np.iscomplexobj(value) else np.float64(value)
        self.f.write(str(n) + " " + str(v) + "\n")

    def close(self):
        if not self.f.closed:
            self.f.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _mode(name, e, h, doc):
    def _init_field_compnt(self):
        self.e_field_compnt = e
        self.h_field_compnt = h
    return type(name, (FDTD,), {"_init_field_compnt": _init_field_compnt, "__doc__": doc})


TExFDTD = _mode("TExFDTD", (Ey, Ez), (Hx,), "2-D TE mode with respect to x.")
TEyFDTD = _mode("TEyFDTD", (Ex, Ez), (Hy,), "2-D TE mode with respect to y.")
TEzFDTD = _mode("TEzFDTD", (Ex, Ey), (Hz,), "2-D TE mode with respect to z.")
TMxFDTD = _mode("TMxFDTD", (Ex,), (Hy, Hz), "2-D TM mode with respect to x.")
TMyFDTD = _mode("TMyFDTD", (Ey,), (Hz, Hx), "2-D TM mode with respect to y.")
TMzFDTD = _mode("TMzFDTD", (Ez,), (Hx, Hy), "2-D TM mode with respect to z.")
TEMxFDTD = _mode("TEMxFDTD", (Ey,), (Hz,), "1-D, y-polarised, x-directed.")
TEMyFDTD = _mode("TEMyFDTD", (Ez,), (Hx,), "1-D, z-polarised, y-directed.")
TEMzFDTD = _mode("TEMzFDTD", (Ex,), (Hy,), "1-D, x-polarised, z-directed.")

__all__ = ["TimeStep", "FDTD", "TExFDTD", "TEyFDTD", "TEzFDTD", "TMxFDTD", "TMyFDTD",
           "TMzFDTD", "TEMxFDTD", "TEMyFDTD", "TEMzFDTD", "FieldView"]
