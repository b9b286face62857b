"""Advance several grids together: the multi-grid kernels of the C ABI.

A ``Batch`` holds a set of ``GridEngine`` objects of one precision.  Each
chunk of steps runs as ONE launch per kernel kind per half-step for the
whole batch (``gmes_batch_step``), captured as a CUDA graph per chunk
length.  Each grid takes its own number of steps in a chunk, so grids of
different sizes and step counts share the device without waiting for one
another; a grid's arithmetic is the same as when it runs alone.
"""

import ctypes as C

import numpy as np

from . import _native as N
from .engine import _torch
from .scene import source_values


class Batch:
    """A fixed set of grids stepped together.

    ``bx_cap`` (0..5) caps the block's extent along k at 2**bx_cap;
    ``blocks`` is the grid size of the persistent update kernel (0: one
    block per tile).  Both are launch-shape knobs the autotuner sets.
    """

    def __init__(self, engines, bx_cap=0, blocks=0, use_graphs=True, stream=None):
        torch = _torch()
        if not engines:
            raise ValueError("a batch needs at least one grid")
        prec = {e.prec for e in engines}
        if len(prec) != 1:
            raise ValueError("all grids of a batch must share one precision")
        self.engines = list(engines)
        self.lib = N.load()
        self.device = engines[0].device
        self.stream = stream or torch.cuda.Stream(device=self.device)
        self.blocks = int(blocks)
        self.bx_cap = int(bx_cap)
        self.use_graphs = bool(use_graphs)
        self._graphs = {}
        n = len(self.engines)
        ws = int(self.lib.gmes_batch_workspace_size(n))
        self.workspace = torch.empty(ws, dtype=torch.uint8, device=self.device)
        # descriptors must outlive the batch: they are referenced by pointer
        self._descs = (C.POINTER(N.GridDescC) * n)(*[C.pointer(e.desc) for e in self.engines])
        self.b = N.BatchC()
        cur = torch.cuda.current_stream(self.device)
        self.stream.wait_stream(cur)
        for e in self.engines:
            self.stream.wait_stream(e.torch_stream)
        N.check(self.lib.gmes_batch_prepare(self._descs, n, C.c_void_p(self.workspace.data_ptr()),
                                            ws, self.bx_cap, C.byref(self.b),
                                            C.c_void_p(self.stream.cuda_stream)))
        self._steps = (C.c_int32 * n)()
        self._staged = []

    def __del__(self):
        for h in getattr(self, "_graphs", {}).values():
            try:
                self.lib.gmes_graph_destroy(h)
            except Exception:
                pass

    @property
    def tiles(self):
        return int(self.b.tiles)

    def _graph(self, nsteps):
        key = (nsteps, self.blocks)
        h = self._graphs.get(key)
        if h is None:
            out = C.c_void_p()
            N.check(self.lib.gmes_graph_capture_batch(C.byref(self.b), int(nsteps), self.blocks,
                                                      C.c_void_p(self.stream.cuda_stream),
                                                      C.byref(out)))
            h = self._graphs[key] = out.value
        return h

    def stage(self, steps, n0s):
        """Stage the source values of every grid for its next ``steps[i]`` steps."""
        torch = _torch()
        for ev in self._staged:
            ev.synchronize()
        self._staged = []
        with torch.cuda.stream(self.stream):
            for e, k, n0 in zip(self.engines, steps, n0s):
                if e.src is None or k <= 0:
                    continue
                if k > e.src_chunk:
                    raise ValueError("chunk longer than a grid's source staging buffer")
                vals = source_values(e.scene, e.scene.dt, n0, k)
                e.src_host[:k].copy_(torch.from_numpy(vals))
                e.src_val[:k].copy_(e.src_host[:k], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.stream)
            self._staged.append(ev)

    @property
    def launches_per_step(self):
        """Kernel launches of one batched step: per half-step the ghost copy
        (when a grid has ghost planes), the cell update and the sources (when
        a grid has any)."""
        return 2 * (int(self.b.ghosts > 0) + 1 + int(self.b.srcs > 0))

    def run(self, steps, n0s=None):
        """Advance grid i by steps[i] steps (one chunk; max(steps) <= every src_chunk).

        ``n0s[i]`` is grid i's current time step (for its source values).
        Work is enqueued on ``self.stream``; call ``synchronize()`` to wait.
        Returns the number of kernels it launched.
        """
        steps = [int(s) for s in steps]
        if len(steps) != len(self.engines):
            raise ValueError("one step count per grid")
        k = max(steps) if steps else 0
        if k == 0:
            return 0
        self.stage(steps, n0s if n0s is not None else [0.0] * len(steps))
        for i, s in enumerate(steps):
            self._steps[i] = s
        N.check(self.lib.gmes_batch_set_steps(C.byref(self.b), self._steps,
                                              C.c_void_p(self.stream.cuda_stream)))
        if self.use_graphs:
            N.check(self.lib.gmes_graph_launch(C.c_void_p(self._graph(k)),
                                               C.c_void_p(self.stream.cuda_stream)))
        else:
            N.check(self.lib.gmes_batch_step(C.byref(self.b), k, self.blocks,
                                             C.c_void_p(self.stream.cuda_stream)))
        return k * self.launches_per_step

    def synchronize(self):
        self.stream.synchronize()
        torch = _torch()
        for e in self.engines:
            e.torch_stream.wait_stream(self.stream)
        torch.cuda.current_stream(self.device).wait_stream(self.stream)
