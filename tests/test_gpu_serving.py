"""Batched multi-grid stepping and the continuous-batching server.

The contract: a grid's result does not depend on the other grids it is
batched with, nor on the launch shape -- bit for bit equal to running it
alone with the single-grid kernels, in every precision.
"""
import numpy as np
import pytest

import gmes_gb300 as G
from gmes_gb300 import workloads as W
from gmes_gb300.autotune import Tuner
from gmes_gb300.batch import Batch
from gmes_gb300.engine import GridEngine
from gmes_gb300.serving import Job, Server, run_one_at_a_time
from cases import CASES

pytestmark = pytest.mark.gpu

PULSE = G.Bandpass(freq=1.0, fwidth=1.0)


def mix():
    """Grids of different dimensionality, size, materials, boundaries and sources."""
    return [
        (lambda: CASES["drude2d"](G)[0], 70),
        (lambda: CASES["tez_upml_currents"](G)[0], 45),
        (lambda: CASES["dispersive3d"](G)[0], 33),
        (lambda: W.cube(n=40, nobj=4, pml_cells=5, src_time=PULSE)[0], 61),
        (lambda: CASES["air2d"](G)[0], 90),
        (lambda: CASES["tmx_cpml_hard"](G)[0], 20),
    ]


def alone(build, nsteps, precision):
    eng = GridEngine(build().compile(), precision=precision, use_graphs=False)
    eng.step(nsteps)
    eng.synchronize()
    return [eng.read(c) for c in range(6)]


@pytest.mark.parametrize("precision", ["fp64", "df64", "fp32", "fp64_strict"])
@pytest.mark.parametrize("shape", [(0, 0), (3, 0), (5, 4 * 152)])
def test_batch_equals_alone(precision, shape):
    jobs = mix()
    engines = [GridEngine(b().compile(), precision=precision, src_chunk=32) for b, _ in jobs]
    batch = Batch(engines, bx_cap=shape[0], blocks=shape[1])
    done = [0] * len(jobs)
    while any(d < n for d, (_, n) in zip(done, jobs)):
        steps = [min(32, n - d) for d, (_, n) in zip(done, jobs)]
        batch.run(steps, [float(d) for d in done])
        done = [d + s for d, s in zip(done, steps)]
    batch.synchronize()
    for (b, n), eng in zip(jobs, engines):
        ref = alone(b, n, precision)
        for c in range(6):
            assert np.array_equal(eng.read(c), ref[c]), (precision, shape, c)


@pytest.mark.parametrize("precision", ["fp64", "df64", "fp32"])
@pytest.mark.parametrize("solo_cells", [8000, 1])
def test_batch_with_solo_grids_equals_alone(precision, solo_cells):
    """Grids above the size threshold run their single-grid kernels inside the
    batch (as a graph for a full chunk, as plain launches for a shorter last
    one); every grid still matches its run alone bit for bit."""
    jobs = mix()
    engines = [GridEngine(b().compile(), precision=precision, src_chunk=32) for b, _ in jobs]
    batch = Batch(engines, solo_cells=solo_cells)
    assert batch.solo and (solo_cells == 1) == (not batch.multi)
    done = [0] * len(jobs)
    launched = 0
    while any(d < n for d, (_, n) in zip(done, jobs)):
        steps = [min(32, n - d) for d, (_, n) in zip(done, jobs)]
        launched += batch.run(steps, [float(d) for d in done])
        done = [d + s for d, s in zip(done, steps)]
    batch.synchronize()
    assert launched > 0
    for (b, n), eng in zip(jobs, engines):
        ref = alone(b, n, precision)
        for c in range(6):
            assert np.array_equal(eng.read(c), ref[c]), (precision, solo_cells, c)


def test_graph_chunks_equal_plain_launches():
    b, n = mix()[3]
    e1 = GridEngine(b().compile(), use_graphs=True, src_chunk=16)
    e1.step(n)
    e1.synchronize()
    ref = alone(b, n, "fp64")
    for c in range(6):
        assert np.array_equal(e1.read(c), ref[c])


def test_server_results_same_alone_and_in_mix():
    builds = mix()
    jobs = [Job(arrival=0.002 * i, jid=i, build=b, nsteps=n, keep_fields=True)
            for i, (b, n) in enumerate(builds)]
    server = Server(precision="fp64", chunk=16, max_slots=4, tuner=Tuner())
    rep = server.run(jobs, realtime=False)
    assert rep["jobs"] == len(jobs) and rep["failed"] == 0
    assert rep["latency_p99_s"] >= rep["latency_p50_s"] > 0
    for job in server.finished:
        b, n = builds[job.jid]
        ref = alone(b, n, "fp64")
        for c in range(6):
            assert np.array_equal(job.fields[c], ref[c]), (job.jid, c)


def test_server_admission_respects_memory_budget_and_survives_bad_jobs():
    def bad():
        raise ValueError("broken scene")
    builds = mix()[:3]
    jobs = [Job(arrival=0.0, jid=i, build=b, nsteps=n) for i, (b, n) in enumerate(builds)]
    jobs.append(Job(arrival=0.0, jid=99, build=bad, nsteps=10))
    one = Server.job_bytes(builds[2][0]().compile(), "fp64")
    server = Server(precision="fp64", chunk=16, memory_budget=one + 1024)
    rep = server.run(jobs, realtime=False)
    assert rep["jobs"] == 3 and rep["failed"] == 1
    assert server.failed[0].jid == 99 and "broken scene" in server.failed[0].error
    assert server.used_bytes == 0


@pytest.mark.parametrize("fill_cells,most", [(1, 1), (9000, 3), (0, 6)])
def test_server_fill_limit(fill_cells, most):
    """Jobs wait while the resident grids hold ``fill_cells`` cells (one is
    always admitted); results do not depend on it."""
    builds = mix()
    jobs = [Job(arrival=0.0, jid=i, build=b, nsteps=n, keep_fields=True)
            for i, (b, n) in enumerate(builds)]
    server = Server(precision="fp64", chunk=16, fill_cells=fill_cells)
    rep = server.run(jobs, realtime=False)
    assert rep["jobs"] == len(jobs) and rep["failed"] == 0
    assert 1 <= rep["max_resident"] <= most
    if fill_cells == 0:
        assert rep["max_resident"] == len(jobs)
    assert server.resident_cells == 0
    for job in server.finished:
        b, n = builds[job.jid]
        ref = alone(b, n, "fp64")
        for c in range(6):
            assert np.array_equal(job.fields[c], ref[c]), (fill_cells, job.jid, c)


def test_one_at_a_time_baseline_runs():
    builds = mix()[:2]
    jobs = [Job(arrival=0.0, jid=i, build=b, nsteps=n) for i, (b, n) in enumerate(builds)]
    rep = run_one_at_a_time(jobs)
    assert rep["cell_updates"] > 0 and rep["gcells_per_s"] > 0
    assert rep["latency_p99_s"] >= rep["latency_p50_s"] > 0


def unstable():
    """A TMz grid stepped at 1.5 times the Courant limit: its fields grow
    until they overflow to Inf (no fault: IEEE arithmetic)."""
    space = G.Cartesian(size=(3, 3, 0), resolution=10)
    geom = [G.DefaultMedium(material=G.Dielectric()), G.Shell(material=G.Cpml(), thickness=0.5)]
    src = [G.PointSource(src_time=G.Bandpass(freq=0.8, fwidth=1.0), center=(0, 0, 0),
                         component=G.Ez)]
    return G.TMzFDTD(space, geom, src, courant_ratio=1.5, verbose=False)


def test_server_fails_a_diverging_job_alone():
    builds = mix()[:4]
    jobs = [Job(arrival=0.0, jid=i, build=b, nsteps=n, keep_fields=True)
            for i, (b, n) in enumerate(builds)]
    jobs.append(Job(arrival=0.0, jid=77, build=unstable, nsteps=1500))
    server = Server(precision="fp64", chunk=16, fill_cells=0)
    rep = server.run(jobs, realtime=False)
    assert rep["jobs"] == len(builds) and rep["failed"] == 1
    bad = server.failed[0]
    assert bad.jid == 77 and "non-finite" in bad.error and bad.done < 1500
    assert server.used_bytes == 0 and server.resident_cells == 0
    for job in server.finished:
        b, n = builds[job.jid]
        ref = alone(b, n, "fp64")
        for c in range(6):
            assert np.array_equal(job.fields[c], ref[c]), (job.jid, c)


def test_server_cancels_a_resident_job():
    builds = mix()[:3]
    jobs = [Job(arrival=0.0, jid=i, build=b, nsteps=n, keep_fields=True)
            for i, (b, n) in enumerate(builds)]
    jobs.append(Job(arrival=0.0, jid=5, build=builds[0][0], nsteps=5000))
    server = Server(precision="fp64", chunk=16, fill_cells=0)

    def on_chunk(srv):
        if srv.chunks == 2:
            srv.cancel(5)
    rep = server.run(jobs, realtime=False, on_chunk=on_chunk)
    assert rep["jobs"] == 3 and rep["failed"] == 1
    assert server.failed[0].jid == 5 and server.failed[0].error == "cancelled"
    assert server.failed[0].done == 32
    for job in server.finished:
        b, n = builds[job.jid]
        ref = alone(b, n, "fp64")
        for c in range(6):
            assert np.array_equal(job.fields[c], ref[c]), (job.jid, c)
