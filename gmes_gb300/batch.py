"""Advance several grids together: the multi-grid kernels of the C ABI.

A ``Batch`` holds a set of ``GridEngine`` objects of one precision.  Each
chunk of steps runs as ONE launch per kernel kind per half-step for the
small grids of the batch (``gmes_batch_step``), captured as a CUDA graph
per chunk length; grids of ``solo_cells`` cells or more fill the GPU on
their own and run their single-grid kernels (their own chunk graph),
where the multi-grid kernel's per-block job look-up and descriptor loads
would only slow them, spread over a few side streams so that one grid's
last partial wave of blocks overlaps the next grid's and the multi-grid
chunk.  Each grid takes its own number of
steps in a chunk, so grids of different sizes and step counts share the
device without waiting for one another; a grid's arithmetic is the same as
when it runs alone.
"""

import ctypes as C

import numpy as np

from . import _native as N
from .engine import _torch
from .scene import source_values


# Grids of at least this many cells run their own single-grid kernels in a
# batch.  Measured on GB300 (64-job FP64 serving mix, 2-D 128^2-1024^2 and
# 3-D 64^3-160^3): the multi-grid kernel alone ran the mix at 8.47 Gcell/s
# against 8.74 one grid at a time.  The 34 grids of that mix below 2^20
# cells (25 dispersive), ms per 64-step chunk with the threshold at 2^20 /
# 2^19 / 2^18 / 2^17 cells: FP64 138.7 / 122.1 / 119.8 / 121.0, FP32 111.6
# / 78.4 / 72.8 / 73.6 -- a grid of 2^18 cells (64^3) fills the GPU's
# resident blocks once over, and the multi-grid kernel runs its cells up to
# 1.3x slower than the single-grid kernel (and a batch with one dispersive
# grid runs the dispersive E kernel for all of them).  With the solo grids
# on 4 side streams (below), ms per chunk at 2^18 / 2^17 / 2^16 / 2^14
# cells: FP64 101.3 / 99.8 / 99.9 / 99.9, FP32 61.1 / 59.3 / 59.3 / 59.2;
# the multi-grid kernel stays for grids below 2^17 cells (2-D up to ~360^2,
# 3-D up to ~50^3), where one launch serves many grids.
SOLO_CELLS = 1 << 17

# Side streams for the solo grids of a batch.
SOLO_STREAMS = 4


class Batch:
    """A fixed set of grids stepped together.

    ``bx_cap`` (0..5) caps the block's extent along k at 2**bx_cap;
    ``blocks`` is the grid size of the persistent update kernel (0: one
    block per tile).  Both are launch-shape knobs the autotuner sets.
    ``solo_cells``: grids with at least this many cells run their own
    single-grid kernels (0: every grid through the multi-grid kernel).
    ``solo_streams``: side streams the solo grids' chunks are spread over,
    so that one grid's last partial wave of blocks overlaps the next grid's
    (1: all on the batch's stream, one after another).
    """

    def __init__(self, engines, bx_cap=0, blocks=0, use_graphs=True, stream=None,
                 solo_cells=SOLO_CELLS, solo_streams=SOLO_STREAMS):
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
        solo_cells = int(solo_cells)
        self.solo = [i for i, e in enumerate(self.engines)
                     if solo_cells > 0 and e.scene.cells >= solo_cells]
        self.multi = [i for i in range(len(self.engines)) if i not in self.solo]
        ns = max(1, min(int(solo_streams), len(self.solo)))
        self._side = ([torch.cuda.Stream(device=self.device) for _ in range(ns)]
                      if ns > 1 else [])
        for i in self.solo:
            # the multi-grid kernel's conditions, so that a grid is batchable
            # or not whatever its size
            d = self.engines[i].desc
            if d.ntfsf > 0:
                raise ValueError(f"grid {i} has a TFSF source: not batchable")
            if d.nprobe > 0:
                raise ValueError(f"grid {i} has probes: not batchable")
            if self.engines[i].cmplx:
                raise ValueError(f"grid {i} is complex: not batchable")
        cur = torch.cuda.current_stream(self.device)
        self.stream.wait_stream(cur)
        for e in self.engines:
            self.stream.wait_stream(e.torch_stream)
        self.b = None
        n = len(self.multi)
        if n:
            ws = int(self.lib.gmes_batch_workspace_size(n))
            self.workspace = torch.empty(ws, dtype=torch.uint8, device=self.device)
            # descriptors must outlive the batch: they are referenced by pointer
            self._descs = (C.POINTER(N.GridDescC) * n)(
                *[C.pointer(self.engines[i].desc) for i in self.multi])
            self.b = N.BatchC()
            N.check(self.lib.gmes_batch_prepare(
                self._descs, n, C.c_void_p(self.workspace.data_ptr()), ws, self.bx_cap,
                C.byref(self.b), C.c_void_p(self.stream.cuda_stream)))
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
        """Tiles of the multi-grid kernel (0 when every grid runs solo)."""
        return int(self.b.tiles) if self.b is not None else 0

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

    def _multi_launches_per_step(self):
        """Launches of one multi-grid step: per half-step the ghost copy (when
        a grid has ghost planes), the cell update and the sources (when a grid
        has any)."""
        if self.b is None:
            return 0
        return 2 * (int(self.b.ghosts > 0) + 1 + int(self.b.srcs > 0))

    def _solo_launches_per_step(self, i):
        """Launches of one single-grid step: per half-step the ghost copy, the
        cell update and the sources (when the grid has any)."""
        return 2 * (2 + int(self.engines[i].desc.nsrc > 0))

    @property
    def launches_per_step(self):
        """Kernel launches of one step of every grid of the batch."""
        return self._multi_launches_per_step() + sum(self._solo_launches_per_step(i)
                                                     for i in self.solo)

    def run(self, steps, n0s=None):
        """Advance grid i by steps[i] steps (one chunk; max(steps) <= every src_chunk).

        ``n0s[i]`` is grid i's current time step (for its source values).
        Work is enqueued on ``self.stream`` (the solo grids' on side streams
        that start after the staging and that ``self.stream`` waits for);
        call ``synchronize()`` to wait.
        Returns the number of kernels it launched.
        """
        steps = [int(s) for s in steps]
        if len(steps) != len(self.engines):
            raise ValueError("one step count per grid")
        k = max(steps) if steps else 0
        if k == 0:
            return 0
        self.stage(steps, n0s if n0s is not None else [0.0] * len(steps))
        st = C.c_void_p(self.stream.cuda_stream)
        launched = 0
        run_solo = [i for i in self.solo if steps[i] > 0]
        side = self._side if len(run_solo) > 1 else []
        # the side streams start once the source values are staged, and run
        # alongside the multi-grid chunk; the batch's stream waits for them
        for ss in side:
            ss.wait_stream(self.stream)
        km = max((steps[i] for i in self.multi), default=0)
        if km > 0:
            for q, i in enumerate(self.multi):
                self._steps[q] = steps[i]
            N.check(self.lib.gmes_batch_set_steps(C.byref(self.b), self._steps, st))
            if self.use_graphs:
                N.check(self.lib.gmes_graph_launch(C.c_void_p(self._graph(km)), st))
            else:
                N.check(self.lib.gmes_batch_step(C.byref(self.b), km, self.blocks, st))
            launched += km * self._multi_launches_per_step()
        for n, i in enumerate(run_solo):
            s = steps[i]
            e = self.engines[i]
            sst = C.c_void_p(side[n % len(side)].cuda_stream) if side else st
            # the chunk length every grid shares is replayed as the grid's
            # own graph; a shorter last chunk runs as plain launches
            if self.use_graphs and s == k:
                N.check(self.lib.gmes_graph_launch(C.c_void_p(e._graph(s)), sst))
            else:
                N.check(self.lib.gmes_step(C.byref(e.desc), s, sst))
            launched += s * self._solo_launches_per_step(i)
        for ss in side:
            self.stream.wait_stream(ss)
        return launched

    def synchronize(self):
        self.stream.synchronize()
        torch = _torch()
        for e in self.engines:
            e.torch_stream.wait_stream(self.stream)
        torch.cuda.current_stream(self.device).wait_stream(self.stream)
