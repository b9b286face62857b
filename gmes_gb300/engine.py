"""One grid on the GPU: device buffers (torch tensors) + the C ABI.

PyTorch only supplies device memory and the stream; all computation runs in
the engine's own kernels (libgmes_gb300.so).  The buffers are sized by
``gmes_grid_sizes`` and described to the library by a ``GridDescC``.
"""

import ctypes as C

import numpy as np

from . import _native as N
from .scene import class_arrays, source_offsets, source_values

_TORCH = None


def _torch():
    global _TORCH
    if _TORCH is None:
        import torch
        _TORCH = torch
    return _TORCH


def require_cuda():
    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError("gmes_gb300 needs a CUDA GPU: no CUDA device is visible")


class GridEngine:
    """Device state of one FDTD grid.

    ``precision``: "fp64" (default), "fp64_strict", "fp32" or "df64".
    ``src_chunk``: steps of source values staged per ``gmes_step`` call.
    """

    def __init__(self, scene, precision="fp64", device=None, src_chunk=256, use_graphs=True):
        require_cuda()
        torch = _torch()
        self.lib = N.load()
        self.use_graphs = bool(use_graphs)
        self._graphs = {}
        self.scene = scene
        self.precision = precision
        self.prec = N.PRECISIONS[precision]
        self.device = torch.device(device if device is not None else "cuda")
        self.src_chunk = int(src_chunk)
        d = N.GridDescC()
        d.abi_version = N.ABI_VERSION
        d.precision = self.prec
        for a in range(3):
            d.n[a] = scene.n[a]
            d.dr[a] = scene.dr[a]
            d.half[a] = scene.half[a]
        d.dt = scene.dt
        d.active = scene.active_mask
        for c in range(6):
            d.naux[c] = scene.naux(c)
            d.nclass[c] = len(scene.classes[c])
        rows, pool, pmls = class_arrays(scene)
        d.npml = len(pmls)
        d.nsrc = len(scene.sources)
        d.nparam = len(pool)
        d.src_steps = self.src_chunk
        d.flags = N.FLAG_DISPERSIVE if scene.dispersive else 0
        self.cmplx = bool(scene.cmplx)
        if self.cmplx:
            if self.prec not in (N.FP64, N.FP64_STRICT):
                raise ValueError("complex (Bloch) fields need precision fp64 or fp64_strict")
            d.flags |= N.FLAG_COMPLEX
            for c in range(6):
                for h in range(2):
                    d.bloch_phase[c][h][0] = float(scene.bloch_phase[c, h, 0])
                    d.bloch_phase[c][h][1] = float(scene.bloch_phase[c, h, 1])
        sizes = (C.c_int64 * 21)()
        N.check(self.lib.gmes_grid_sizes(C.byref(d), sizes))
        self.sizes = list(sizes)
        dev = self.device
        self.fields = []
        self.aux = []
        self.cls = []
        for c in range(6):
            shape = scene.shape(c)
            if self.cmplx:
                t = torch.zeros((2,) + shape, dtype=torch.float64, device=dev)  # re, im planes
            elif self.prec in (N.FP64, N.FP64_STRICT):
                t = torch.zeros(shape, dtype=torch.float64, device=dev)
            elif self.prec == N.FP32:
                t = torch.zeros(shape, dtype=torch.float32, device=dev)
            else:
                t = torch.zeros(shape + (2,), dtype=torch.float32, device=dev)
            self.fields.append(t)
            d.field[c] = t.data_ptr()
            na = d.naux[c] if (scene.active_mask >> c) & 1 else 0
            if na:
                a = torch.zeros(self.sizes[12 + c], dtype=torch.uint8, device=dev)
                d.aux[c] = a.data_ptr()
            else:
                a = None
            self.aux.append(a)
            if (scene.active_mask >> c) & 1:
                if scene.cls[c] is not None or not scene.device_raster:
                    m = torch.from_numpy(scene.host_cls(c)).to(dev)
                else:
                    m = torch.zeros(shape, dtype=torch.uint8, device=dev)  # rasterised below
                d.cls[c] = m.data_ptr()
            else:
                m = None
            self.cls.append(m)
        self.coef = torch.zeros(max(self.sizes[18], 256), dtype=torch.uint8, device=dev)
        d.coef = self.coef.data_ptr()
        srcs = source_offsets(scene)
        if srcs:
            arr = (N.PointSourceC * len(srcs))(*[N.PointSourceC(c, m, o) for c, m, o in srcs])
            host = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8)
            self.src = host.to(dev)
            lead = (2,) if self.cmplx else ()
            self.src_val = torch.zeros(lead + (self.src_chunk, 2, len(srcs)), dtype=torch.float64,
                                       device=dev)
            self.src_host = torch.zeros(self.src_val.shape, dtype=torch.float64).pin_memory()
            self._src_host_np = self.src_host.numpy()  # shares the pinned memory
            d.src = self.src.data_ptr()
            d.src_val = self.src_val.data_ptr()
        else:
            self.src = self.src_val = self.src_host = self._src_host_np = None
        # TFSF: the incident-field grid (advanced inside this grid's step) and
        # the transparent points
        self.incident = None
        self.tfsf = None
        if scene.tfsf is not None:
            aux_scene, points = scene.tfsf
            self.incident = GridEngine(aux_scene, precision=precision, device=device,
                                       src_chunk=src_chunk, use_graphs=False)
            arr = (N.TransparentC * max(1, len(points)))()
            for q, (c, off, faces) in enumerate(points):
                t = arr[q]
                t.comp, t.nface, t.offset = c, len(faces), off
                for k, (cf, a, b, sp) in enumerate(faces):
                    t.coef[k], t.r0[k], t.r1[k], t.sample[k] = cf, a, b, sp
            self.tfsf = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(dev)
            d.ntfsf = len(points)
            d.tfsf = self.tfsf.data_ptr()
            d.incident = C.pointer(self.incident.desc)
        self.probes = None
        self.probe_val = None
        self.desc = d
        # events reused on every call: the pinned staging buffer's last copy,
        # and the two directions of ordering against the caller's stream
        self._staged = torch.cuda.Event()
        self._ev_in = torch.cuda.Event()
        self._ev_out = torch.cuda.Event()
        self._dev_index = dev.index if dev.index is not None else torch.cuda.current_device()
        self._rows, self._pool, self._pmls = rows, pool, pmls
        # The engine works on its own (non-default) stream so that chunks of
        # steps can be captured as CUDA graphs; it orders itself against the
        # caller's current stream on entry and exit of every call.
        self._stream = torch.cuda.Stream(device=dev)
        self._enter()
        self.build_coefficients()
        self.rasterized = False
        if scene.device_raster and any(scene.cls[c] is None for c in range(6)
                                       if (scene.active_mask >> c) & 1):
            self._rasterize()
        self._leave()

    def __del__(self):
        graphs = getattr(self, "_graphs", {})
        for h in graphs.values():
            try:
                self.lib.gmes_graph_destroy(h)
            except Exception:
                pass
        graphs.clear()

    # -- streams -----------------------------------------------------------
    @property
    def stream(self):
        """The engine's CUDA stream handle (cudaStream_t as an int)."""
        return self._stream.cuda_stream

    @property
    def torch_stream(self):
        return self._stream

    def _enter(self):
        cur = _torch().cuda.current_stream(self._dev_index)
        if cur.cuda_stream != self._stream.cuda_stream:
            self._ev_in.record(cur)
            self._stream.wait_event(self._ev_in)

    def _leave(self):
        cur = _torch().cuda.current_stream(self._dev_index)
        if cur.cuda_stream != self._stream.cuda_stream:
            self._ev_out.record(self._stream)
            cur.wait_event(self._ev_out)

    # -- setup -------------------------------------------------------------
    def build_coefficients(self):
        rows, pool, pmls = self._rows, self._pool, self._pmls
        crow = (N.ClassDescC * max(1, len(rows)))()
        for i, r in enumerate(rows):
            crow[i] = N.ClassDescC(r["kind"], r["pml"], r["npole"], r["ncp"], r["param_off"],
                                   r["nparam"], r["eps"])
        cpool = (C.c_double * max(1, len(pool)))(*pool)
        cpml = (N.PmlDescC * max(1, len(pmls)))()
        for i, p in enumerate(pmls):
            q = cpml[i]
            q.kind = p["kind"]
            for a in range(3):
                q.sigma_max[a] = p["sigma_max"][a]
                q.center[a] = p["center"][a]
                q.half_size[a] = p["half_size"][a]
            q.m, q.kappa_max, q.m_a, q.a_max, q.d = (p["m"], p["kappa_max"], p["m_a"],
                                                      p["a_max"], p["d"])
        N.check(self.lib.gmes_build_coefficients(C.byref(self.desc), crow, cpool, cpml,
                                                 C.c_void_p(self.stream)))

    def _rasterize(self):
        """Build the class maps of the components not given on the host (on the GPU)."""
        torch = _torch()
        scene = self.scene
        recs = scene.shapes
        arr = (N.ShapeC * len(recs))()
        for q, r in enumerate(recs):
            sh = arr[q]
            sh.type = r["type"]
            sh.compound = r["compound"]
            sh.nbox = r.get("nbox", 0)
            for a in range(3):
                sh.lo[a] = r["lo"][a]
                sh.hi[a] = r["hi"][a]
                sh.center[a] = r.get("center", [0.0] * 3)[a]
                sh.p[a] = r.get("p", [0.0] * 3)[a]
                sh.axis[a] = r.get("axis", [0.0] * 3)[a]
            for t, v in enumerate(r.get("m", [0.0] * 9)):
                sh.m[t] = v
            for b, (lo, hi) in enumerate(zip(r.get("box_lo", []), r.get("box_hi", []))):
                for a in range(3):
                    sh.box_lo[b][a] = lo[a]
                    sh.box_hi[b][a] = hi[a]
        with torch.cuda.stream(self._stream):
            shapes = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(self.device)
            for c in range(6):
                if not (scene.active_mask >> c) & 1 or scene.cls[c] is not None:
                    continue
                lut = torch.from_numpy(np.ascontiguousarray(scene.lut[c])).to(self.device)
                N.check(self.lib.gmes_rasterize(C.byref(self.desc), c,
                                                C.c_void_p(shapes.data_ptr()), len(recs),
                                                C.c_void_p(lut.data_ptr()),
                                                C.c_void_p(self.stream)))
                self._raster_keep = (shapes, lut)
            self._stream.synchronize()
        self.rasterized = True

    def class_counts(self, c):
        """Points per class of component ``c``, counted on the GPU."""
        m = self.cls[c]
        if m is None:
            return {}
        self._leave()
        cnt = _torch().bincount(m.view(-1).long(), minlength=len(self.scene.classes[c]))
        return {i: int(v) for i, v in enumerate(cnt.tolist()) if v}

    def set_pml_profile(self, pml, comp, axis, values):
        self._enter()
        v = np.ascontiguousarray(values, dtype=np.float64)
        N.check(self.lib.gmes_set_pml_profile(
            C.byref(self.desc), pml, comp, axis,
            v.ctypes.data_as(C.POINTER(C.c_double)), C.c_void_p(self.stream)))

    def get_pml_profile(self, pml, comp, axis):
        """FP64 profile rows (n, 5) of (pml, comp, axis) as computed on the GPU."""
        n = self.scene.shape(comp)[axis]
        out = np.zeros((n, 5), np.float64)
        N.check(self.lib.gmes_get_pml_profile(
            C.byref(self.desc), pml, comp, axis, out.ctypes.data_as(C.POINTER(C.c_double)),
            C.c_void_p(self.stream)))
        return out

    def reset(self):
        self._enter()
        N.check(self.lib.gmes_reset(C.byref(self.desc), C.c_void_p(self.stream)))
        if self.incident is not None:
            N.check(self.lib.gmes_reset(C.byref(self.incident.desc), C.c_void_p(self.stream)))
        self._leave()

    # -- probes ------------------------------------------------------------
    def set_probes(self, points):
        """Record the value of every (component, flat offset) point after each
        half-step (per step, into a device buffer read by ``probe_values``)."""
        torch = _torch()
        points = list(points)
        d = self.desc
        if not points:
            d.nprobe, d.probe, d.probe_val = 0, None, None
            self.probes = self.probe_val = None
        else:
            arr = (N.ProbeC * len(points))(*[N.ProbeC(c, 0, o) for c, o in points])
            self.probes = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(
                self.device)
            lead = (2,) if self.cmplx else ()
            self.probe_val = torch.zeros(lead + (self.src_chunk, len(points)),
                                         dtype=torch.float64, device=self.device)
            d.nprobe = len(points)
            d.probe_steps = self.src_chunk
            d.probe = self.probes.data_ptr()
            d.probe_val = self.probe_val.data_ptr()
        # captured graphs hold the old descriptor
        for h in self._graphs.values():
            self.lib.gmes_graph_destroy(h)
        self._graphs.clear()

    def probe_values(self, k):
        """(k, nprobe) float64 numpy: the probes of the last k recorded steps of a chunk."""
        self._stream.synchronize()
        if self.cmplx:
            v = self.probe_val[:, :k].cpu().numpy()
            return v[0] + 1j * v[1]
        return self.probe_val[:k].cpu().numpy()

    # -- stepping ----------------------------------------------------------
    def _graph(self, nsteps):
        h = self._graphs.get(nsteps)
        if h is None:
            out = C.c_void_p()
            N.check(self.lib.gmes_graph_capture_step(C.byref(self.desc), int(nsteps),
                                                     C.c_void_p(self.stream), C.byref(out)))
            h = self._graphs[nsteps] = out.value
        return h

    def _launch(self, nsteps):
        if self.use_graphs:
            N.check(self.lib.gmes_graph_launch(C.c_void_p(self._graph(nsteps)),
                                               C.c_void_p(self.stream)))
        else:
            N.check(self.lib.gmes_step(C.byref(self.desc), int(nsteps), C.c_void_p(self.stream)))

    def _stage(self, vals, k, stream=None):
        stream = stream if stream is not None else self._stream
        # the pinned staging buffer may still be read by the previous
        # chunk's asynchronous copy
        self._staged.synchronize()
        vals = np.asarray(vals)
        host = self._src_host_np
        if self.cmplx:
            host[0, :k] = vals.real
            host[1, :k] = vals.imag
        else:
            host[:k] = vals
        # rows of (2, nsrc) float64 per step; a complex grid has a real and
        # an imaginary plane of src_chunk rows each
        row = host.shape[-1] * host.shape[-2] * 8
        plane = self.src_chunk * row
        for q in range(2 if self.cmplx else 1):
            N.check(self.lib.gmes_copy_async(C.c_void_p(self.src_val.data_ptr() + q * plane),
                                             C.c_void_p(self.src_host.data_ptr() + q * plane),
                                             k * row, C.c_void_p(stream.cuda_stream)))
        self._staged.record(stream)

    def _stage_incident(self, n0, k):
        """Stage the incident-field grid's source values on this grid's stream."""
        inc = self.incident
        if inc is not None and inc.src is not None:
            inc._stage(source_values(inc.scene, inc.scene.dt, n0, k), k, self._stream)

    def step(self, nsteps, n0=0.0, src_values=None, on_chunk=None):
        """Advance ``nsteps`` steps; the first E half-step is at n0 + 1/2.

        Steps run in chunks of up to ``src_chunk``: the source values of a
        chunk are staged, then the chunk runs as one CUDA graph (or as plain
        launches with ``use_graphs=False``).  ``src_values`` (nsteps, 2, nsrc)
        overrides the host evaluation of the source-time functions.
        """
        nsteps = int(nsteps)
        self._enter()
        done = 0
        while done < nsteps:
            k = min(self.src_chunk, nsteps - done)
            if self.src is not None:
                vals = (src_values[done:done + k] if src_values is not None else
                        source_values(self.scene, self.scene.dt, n0 + done, k))
                self._stage(vals, k)
            self._stage_incident(n0 + done, k)
            self._launch(k)
            if on_chunk is not None:
                on_chunk(done, k)
            done += k
        self._leave()

    def half_step(self, side, slot=0):
        """Enqueue one half-step (0: E, 1: H) reading staged source slot ``slot``."""
        N.check(self.lib.gmes_half_step(C.byref(self.desc), int(side), int(slot),
                                        C.c_void_p(self.stream)))

    def stage_sources(self, n0, nsteps):
        """Stage the source values of ``nsteps`` steps from time step n0 (<= src_chunk)."""
        if nsteps > self.src_chunk:
            raise ValueError("more steps than the staging buffer holds")
        self._enter()
        self._stage_incident(n0, nsteps)
        if self.src is None:
            return
        self._stage(source_values(self.scene, self.scene.dt, n0, nsteps), nsteps)

    def launch_raw(self, nsteps):
        """Enqueue ``nsteps`` steps with the source values already staged."""
        self._launch(int(nsteps))

    # -- field access ------------------------------------------------------
    def tensor(self, c):
        """The raw device tensor of component ``c`` (precision-dependent layout)."""
        return self.fields[c]

    def read(self, c):
        """Component ``c`` as a float64 (complex128 for complex grids) numpy array."""
        t = self.fields[c]
        if self.cmplx:
            a = t.cpu().numpy()
            return a[0] + 1j * a[1]
        if self.prec == N.DF64:
            return (t[..., 0].double() + t[..., 1].double()).cpu().numpy()
        return t.double().cpu().numpy()

    def read_tensor(self, c):
        """Component ``c`` as a float64 (complex128) device tensor."""
        t = self.fields[c]
        if self.cmplx:
            return _torch().complex(t[0], t[1])
        if self.prec == N.DF64:
            return t[..., 0].double() + t[..., 1].double()
        return t.double()

    def write(self, c, key, value):
        torch = _torch()
        t = self.fields[c]
        if self.cmplx:
            v = torch.as_tensor(np.asarray(value, np.complex128), device=self.device)
            t[0][key] = v.real
            t[1][key] = v.imag
            return
        if self.prec == N.DF64:
            v = torch.as_tensor(value, dtype=torch.float64, device=self.device)
            hi = v.float()
            lo = (v - hi.double()).float()
            t[key + (0,) if isinstance(key, tuple) else (key, Ellipsis, 0)] = hi
            t[key + (1,) if isinstance(key, tuple) else (key, Ellipsis, 1)] = lo
        else:
            t[key] = torch.as_tensor(value, dtype=t.dtype, device=self.device)

    def write_all(self, c, array):
        torch = _torch()
        t = self.fields[c]
        if self.cmplx:
            a = np.asarray(array, np.complex128)
            t[0].copy_(torch.as_tensor(np.ascontiguousarray(a.real), device=self.device))
            t[1].copy_(torch.as_tensor(np.ascontiguousarray(a.imag), device=self.device))
            return
        a = torch.as_tensor(np.ascontiguousarray(array, dtype=np.float64), device=self.device)
        if self.prec == N.DF64:
            hi = a.float()
            t[..., 0] = hi
            t[..., 1] = (a - hi.double()).float()
        else:
            t.copy_(a.to(t.dtype))

    def aux_tensor(self, c):
        """State slots of component ``c`` as a (naux, *shape[, 2]) tensor view."""
        a = self.aux[c]
        if a is None:
            return None
        torch = _torch()
        shape = self.scene.shape(c)
        na = self.desc.naux[c]
        if self.cmplx:
            return a.view(torch.float64).view((2, na) + shape)
        if self.prec in (N.FP64, N.FP64_STRICT):
            return a.view(torch.float64).view((na,) + shape)
        if self.prec == N.FP32:
            return a.view(torch.float32).view((na,) + shape)
        return a.view(torch.float32).view((na,) + shape + (2,))

    def check_finite(self, flag_ptr, stream=None):
        """Enqueue the non-finite guard (gmes_nonfinite): sets the int32 at
        device address ``flag_ptr`` to 1 when any field value is an infinity
        or a NaN.  On ``stream`` (a cudaStream_t handle) or the engine's."""
        st = self.stream if stream is None else stream
        N.check(self.lib.gmes_nonfinite(C.byref(self.desc), C.c_void_p(flag_ptr),
                                        C.c_void_p(st)))

    def synchronize(self):
        self._stream.synchronize()
