"""Continuous-batching server for FDTD jobs.

Jobs (a scene plus a step count) arrive over time.  The server keeps a
resident set of grids on the GPU and advances all of them together in
chunks of steps (``Batch``: one launch per kernel kind per half-step,
replayed as a CUDA graph).  Between chunks it

* retires the grids that finished (their fields are read back if asked);
* admits waiting jobs in arrival order while the GPU has the memory for
  them (the grid's buffer sizes from ``gmes_grid_sizes`` against
  ``torch.cuda.mem_get_info`` minus a reserve, and an optional budget) and
  a slot is free;
* compiles the next jobs' scenes on the host while the chunk runs;
* fails, alone, every resident job whose fields went non-finite during the
  chunk (a device check after each chunk, ``gmes_nonfinite``), and every
  job cancelled with ``cancel(jid)``, queued or resident.

A job's arithmetic does not depend on which other grids share its chunks,
so its result is the same alone and in the mix.  Latency of a job =
completion time - arrival time; the report gives p50 / p99 and the
aggregate cell-updates per second.  Failures surface to the caller as the
job's ``error`` text and touch no other job, as the reference's binding
turns a failed update into an exception for its caller
(src/cpp23_support.hh:155-173, src/pw_material.i:23-33).
"""

import time
from dataclasses import dataclass, field

import numpy as np

from .batch import SOLO_STREAMS, Batch
from .engine import GridEngine, _torch


# Resident cells beyond which a waiting job is held back.  Measured on
# GB300 (512-job FP64 Poisson mix at 3 jobs/s, both servers arrival-bound at
# 7.2 Gcell/s): with no limit the batched server's p99 latency was 12.8 s
# against 5.8 s for the same jobs one at a time in arrival order.
FILL_CELLS = 1 << 22


@dataclass(order=True)
class Job:
    """One simulation request.

    ``build`` returns an un-initialised FDTD object (the scene); ``nsteps``
    the number of full steps to run; ``arrival`` seconds after the server
    starts.  ``keep_fields`` reads the six fields back when the job ends.
    """

    arrival: float
    jid: int
    build: object = field(compare=False)
    nsteps: int = field(compare=False)
    keep_fields: bool = field(default=False, compare=False)
    # filled by the server
    scene: object = field(default=None, compare=False, repr=False)
    engine: object = field(default=None, compare=False, repr=False)
    done: int = field(default=0, compare=False)
    t_admit: float = field(default=None, compare=False)
    t_finish: float = field(default=None, compare=False)
    fields: list = field(default=None, compare=False, repr=False)
    error: str = field(default=None, compare=False)

    @property
    def cells(self):
        return self.scene.cells if self.scene is not None else 0


class Server:
    """Resident-set FDTD server on one GPU.

    ``precision``: engine precision of every job.  ``chunk``: steps per
    chunk (<= 256).  ``max_slots``: resident grids at most.
    ``memory_budget``: bytes the resident grids may use (default: free
    memory at start minus ``reserve``).  ``tuner``: an ``autotune.Tuner``
    choosing the batch launch shape, or None for the defaults.
    ``fill_cells``: a waiting job is admitted only while the resident grids
    hold fewer cells than this with it (one job is always admitted; 0: no
    limit).  A few million cells fill the GPU, so beyond that more resident
    grids only share it: every job's latency grows and throughput does not.
    ``guard``: check every resident grid for non-finite field values after
    each chunk and fail the jobs that have them.
    """

    def __init__(self, precision="fp64", chunk=64, max_slots=64, memory_budget=None,
                 reserve=2 << 30, tuner=None, use_graphs=True, device=None,
                 fill_cells=FILL_CELLS, guard=True):
        torch = _torch()
        self.precision = precision
        self.chunk = int(chunk)
        if not 1 <= self.chunk <= 256:
            raise ValueError("chunk must be in [1, 256]")
        self.max_slots = int(max_slots)
        self.device = torch.device(device if device is not None else "cuda")
        free, _total = torch.cuda.mem_get_info(self.device)
        self.memory_budget = int(memory_budget if memory_budget is not None
                                 else max(0, free - reserve))
        self.reserve = int(reserve)
        self.tuner = tuner
        self.use_graphs = use_graphs
        self.stream = torch.cuda.Stream(device=self.device)
        self.resident = []
        self.finished = []
        self.failed = []
        self.used_bytes = 0
        self._batch = None
        self._batch_key = None
        self.chunks = 0
        self.launches = 0
        self.fill_cells = int(fill_cells)
        self.resident_cells = 0
        self.max_resident = 0
        self.guard = bool(guard)
        self._flags = torch.zeros(self.max_slots, dtype=torch.int32, device=self.device)
        self._flags_host = torch.zeros(self.max_slots, dtype=torch.int32).pin_memory()
        self._cancel = set()

    # -- failures ------------------------------------------------------------
    def cancel(self, jid):
        """Cancel job ``jid``: a queued job never starts, a resident one stops
        at the end of its current chunk; either is reported as failed with
        the error "cancelled".  Safe to call from another thread or from the
        ``on_chunk`` callback of ``run``."""
        self._cancel.add(jid)

    def _fail(self, job, now, error):
        """Take a job out of service with ``error``, freeing what it holds."""
        job.error = error
        job.t_finish = now
        if job.engine is not None:
            job.engine = None
            self.used_bytes -= job.bytes
            self.resident_cells -= job.cells
        self.failed.append(job)

    def _apply_cancellations(self, pending, waiting, now):
        """Remove cancelled jobs from the arrival list, the queue and the
        resident set (between chunks)."""
        if not self._cancel:
            return
        hit = self._cancel
        for lst in (pending, waiting):
            for job in [j for j in lst if j.jid in hit]:
                lst.remove(job)
                self._fail(job, now, "cancelled")
        for job in [j for j in self.resident if j.jid in hit]:
            self.resident.remove(job)
            self._fail(job, now, "cancelled")
        self._cancel = set()

    def _enqueue_guard(self, jobs):
        """After a chunk: the non-finite check of every resident grid, its
        flags copied to pinned host memory on the server's stream."""
        n = len(jobs)
        with _torch().cuda.stream(self.stream):
            self._flags[:n].zero_()
            base = self._flags.data_ptr()
            for q, job in enumerate(jobs):
                job.engine.check_finite(base + 4 * q, self.stream.cuda_stream)
            self._flags_host[:n].copy_(self._flags[:n], non_blocking=True)

    def _diverged(self, jobs):
        """The jobs whose check found a non-finite value (after the chunk's
        synchronisation)."""
        return [j for j, f in zip(jobs, self._flags_host[:len(jobs)].tolist()) if f]

    # -- admission ---------------------------------------------------------
    @staticmethod
    def job_bytes(scene, precision):
        """Device bytes a grid needs (fields, maps, state, coefficients)."""
        from . import _native as N
        import ctypes as C
        lib = N.load()
        d = N.GridDescC()
        d.abi_version = N.ABI_VERSION
        d.precision = N.PRECISIONS[precision]
        for a in range(3):
            d.n[a] = scene.n[a]
            d.dr[a] = scene.dr[a]
        d.dt = scene.dt
        d.active = scene.active_mask
        for c in range(6):
            d.naux[c] = scene.naux(c)
            d.nclass[c] = len(scene.classes[c])
        d.npml = len(scene.pmls)
        d.nsrc = len(scene.sources)
        d.nparam = sum(len(x.params) for c in range(6) for x in scene.classes[c])
        sizes = (C.c_int64 * 21)()
        N.check(lib.gmes_grid_sizes(C.byref(d), sizes))
        return int(sum(sizes)) + 256 * 1024

    def _fits(self, nbytes):
        torch = _torch()
        if self.used_bytes + nbytes > self.memory_budget:
            return False
        free, _ = torch.cuda.mem_get_info(self.device)
        return nbytes + self.reserve <= free + 0  # caching allocator may hold freed blocks

    def _compile(self, job):
        if job.scene is None and job.error is None:
            try:
                sim = job.build()
                job.scene = sim.compile()
            except Exception as exc:  # a bad job fails alone
                job.error = f"{type(exc).__name__}: {exc}"

    def _admit(self, job, now):
        self._compile(job)
        if job.error is not None:
            return "failed"
        need = self.job_bytes(job.scene, self.precision)
        if len(self.resident) >= self.max_slots or not self._fits(need):
            return "wait"
        if (self.resident and self.fill_cells > 0
                and self.resident_cells + job.cells > self.fill_cells):
            return "wait"
        try:
            job.engine = GridEngine(job.scene, precision=self.precision, device=self.device,
                                    src_chunk=max(self.chunk, 1), use_graphs=False)
        except Exception as exc:
            job.error = f"{type(exc).__name__}: {exc}"
            return "failed"
        job.bytes = need
        self.used_bytes += need
        self.resident_cells += job.cells
        job.t_admit = now
        self.resident.append(job)
        self.max_resident = max(self.max_resident, len(self.resident))
        return "admitted"

    def _retire(self, job, now):
        job.t_finish = now
        if job.keep_fields:
            job.fields = [job.engine.read(c) for c in range(6)]
        job.engine = None
        self.used_bytes -= job.bytes
        self.resident_cells -= job.cells
        self.finished.append(job)

    # -- the loop ----------------------------------------------------------
    def _batch_for(self, jobs):
        shape = self.tuner.choice(jobs) if self.tuner is not None else (0, 0)
        key = (tuple(j.jid for j in jobs), shape)
        if self._batch is None or self._batch_key != key:
            self._batch = Batch([j.engine for j in jobs], bx_cap=shape[0], blocks=shape[1],
                                use_graphs=self.use_graphs, stream=self.stream)
            self._batch_key = key
        return self._batch

    def run(self, jobs, realtime=True, on_chunk=None):
        """Serve ``jobs`` (arrival times relative to the start); return the report.

        With ``realtime`` the server waits for arrivals on the wall clock;
        otherwise a job is available as soon as the clock reaches its
        arrival or the server is idle.  ``on_chunk(server)`` is called after
        every chunk (for example to cancel jobs).
        """
        torch = _torch()
        pending = sorted(jobs)
        waiting = []
        t0 = time.perf_counter()
        cell_updates = 0
        while pending or waiting or self.resident:
            now = time.perf_counter() - t0
            self._apply_cancellations(pending, waiting, now)
            while pending and (pending[0].arrival <= now or
                               (not realtime and not self.resident and not waiting)):
                waiting.append(pending.pop(0))
            # admission in arrival order; a job that does not fit blocks the
            # ones behind it (no overtaking) unless nothing is resident
            while waiting:
                st = self._admit(waiting[0], now)
                if st == "wait":
                    break
                job = waiting.pop(0)
                if st == "failed":
                    job.t_finish = now
                    self.failed.append(job)
            if not self.resident:
                if waiting and not self.resident:
                    job = waiting.pop(0)
                    job.error = job.error or "does not fit in the memory budget"
                    job.t_finish = now
                    self.failed.append(job)
                    continue
                if pending and realtime:
                    time.sleep(max(0.0, min(0.01, pending[0].arrival - now)))
                continue
            batch = self._batch_for(self.resident)
            steps = [min(self.chunk, j.nsteps - j.done) for j in self.resident]
            n0s = [float(j.done) for j in self.resident]
            if self.tuner is not None:
                self.tuner.observe_start(batch)
            self.launches += batch.run(steps, n0s)
            if self.tuner is not None:
                self.tuner.observe_stop(batch)
            if self.guard:
                self._enqueue_guard(self.resident)
                self.launches += len(self.resident)
            # host work overlaps the chunk: compile the next arrivals' scenes
            for job in waiting[:4]:
                self._compile(job)
            batch.synchronize()
            if self.tuner is not None:
                self.tuner.observe_end(batch, sum(s * j.cells for s, j in zip(steps, self.resident)))
            self.chunks += 1
            now = time.perf_counter() - t0
            bad = set(id(j) for j in self._diverged(self.resident)) if self.guard else set()
            still = []
            for j, s in zip(self.resident, steps):
                j.done += s
                cell_updates += s * j.cells
                if id(j) in bad:
                    self._fail(j, now, f"non-finite field values (Inf or NaN) by step {j.done}: "
                                       "the simulation diverged, e.g. a time step above the "
                                       "Courant stability limit")
                elif j.done >= j.nsteps:
                    self._retire(j, now)
                else:
                    still.append(j)
            self.resident = still
            if on_chunk is not None:
                on_chunk(self)
        torch.cuda.synchronize(self.device)
        wall = time.perf_counter() - t0
        return self.report(wall, cell_updates)

    def report(self, wall, cell_updates):
        lat = np.array([j.t_finish - j.arrival for j in self.finished], float)
        return {
            "jobs": len(self.finished), "failed": len(self.failed), "wall_s": wall,
            "cell_updates": int(cell_updates),
            "gcells_per_s": cell_updates / wall / 1e9 if wall > 0 else 0.0,
            "latency_p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "chunks": self.chunks, "launches": self.launches,
            "max_resident": self.max_resident,
        }


def run_one_at_a_time(jobs, precision="fp64", device=None, realtime=False):
    """The same jobs, each run alone with the plain single-grid kernels, in
    arrival order.  With ``realtime`` a job starts no earlier than its
    arrival (as in ``Server.run``), so throughput and latencies compare
    with the batched server on the same arrival process.  ``job_s`` holds
    each job's own wall time (scene, set-up and steps), in arrival order."""
    torch = _torch()
    t0 = time.perf_counter()
    cell_updates = 0
    lat = []
    job_s = []
    for job in sorted(jobs):
        if realtime:
            wait = job.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
        tj = time.perf_counter()
        sim = job.build()
        scene = sim.compile()
        eng = GridEngine(scene, precision=precision, device=device, use_graphs=False)
        eng.step(job.nsteps)
        eng.synchronize()
        cell_updates += job.nsteps * scene.cells
        if job.keep_fields:
            job.fields = [eng.read(c) for c in range(6)]
        del eng
        job_s.append(time.perf_counter() - tj)
        lat.append(time.perf_counter() - t0 - job.arrival)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    lat = np.array(lat, float)
    return {"wall_s": wall, "cell_updates": cell_updates,
            "gcells_per_s": cell_updates / wall / 1e9,
            "latency_p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "job_s": job_s}


def saturation_copies(cells, min_cells=1 << 21, max_copies=128, min_copies=SOLO_STREAMS):
    """Copies of a grid of ``cells`` cells that ``saturated_step_seconds``
    steps together: enough for ``min_cells`` cells, at most ``max_copies``,
    and at least ``min_copies`` (one per side stream of the batch)."""
    return int(max(min_copies, 1, min(max_copies, -(-min_cells // max(int(cells), 1)))))


def saturated_step_seconds(scene, precision="fp64", min_cells=1 << 21, max_copies=128,
                           steps=24, device=None, min_copies=SOLO_STREAMS):
    """Seconds per step of one grid when copies of it fill the GPU.

    ``copies`` = max(min_copies, min(max_copies, ceil(min_cells / cells)))
    grids of ``scene`` (at least one per side stream of the batch, so that a
    large grid's last partial wave of blocks overlaps another copy's, as it
    overlaps other grids in a mix)
    advance together through ``Batch`` (one multi-grid launch per kernel
    kind and half-step; a grid of SOLO_CELLS cells or more runs its own
    single-grid kernels, which fill the GPU by themselves and run its cells
    faster than the multi-grid kernel); the device time
    of ``steps`` steps (CUDA events, after a warm-up chunk) divided by
    copies x steps is the grid's step time at a saturated GPU -- the least
    time any batching of it can give.  Returns (seconds, copies).
    """
    torch = _torch()
    cells = scene.cells
    copies = saturation_copies(cells, min_cells, max_copies, min_copies)
    engines = [GridEngine(scene, precision=precision, device=device, src_chunk=steps)
               for _ in range(copies)]
    batch = Batch(engines)
    batch.run([steps] * copies, [0.0] * copies)  # warm-up: loads kernels, captures graphs
    batch.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(batch.stream)
    batch.run([steps] * copies, [float(steps)] * copies)
    t1.record(batch.stream)
    batch.synchronize()
    sec = t0.elapsed_time(t1) / 1e3 / (copies * steps)
    del batch, engines
    return sec, copies


def batching_bound(jobs, job_s, precision="fp64", device=None, cache=None):
    """The largest speed-up over one-at-a-time any batching can give on ``jobs``.

    ``job_s``: each job's one-at-a-time wall time (``run_one_at_a_time``),
    in arrival order.  Every job's least GPU time is its steps x its
    saturated step time (``saturated_step_seconds``); the bound is the
    summed one-at-a-time time over the summed least time.  ``cache`` (a
    dict) reuses measurements of identical grids.
    """
    cache = {} if cache is None else cache
    least = 0.0
    per_job = []
    for job in sorted(jobs):
        scene = job.build().compile()
        key = (tuple(scene.n), scene.cells, len(scene.classes[0]), scene.dispersive,
               tuple(len(scene.classes[c]) for c in range(6)), repr(scene.dt))
        if key not in cache:
            cache[key] = saturated_step_seconds(scene, precision, device=device)
        sec, copies = cache[key]
        least += sec * job.nsteps
        per_job.append((scene.cells, job.nsteps, sec, copies))
    total = float(sum(job_s))
    return {"bound": total / least if least > 0 else None, "one_at_a_time_s": total,
            "saturated_s": least, "per_job": per_job}
