"""Admission of the continuous-batching server on the host: arrival order,
the slot and memory limits, the fill limit on resident cells, and the
bookkeeping of retirement.  No GPU: the grid engine and the memory query
are replaced."""
import types

import pytest

pytest.importorskip("torch")

from gmes_gb300 import serving as S  # noqa: E402


class _Engine:
    def __init__(self, scene, **kw):
        self.scene = scene

    def read(self, c):
        return None


def _server(monkeypatch, fill_cells, max_slots=64, budget=1 << 40):
    monkeypatch.setattr(S, "GridEngine", _Engine)
    monkeypatch.setattr(S.Server, "job_bytes", staticmethod(lambda scene, prec: scene.cells))
    srv = object.__new__(S.Server)
    srv.precision, srv.chunk, srv.max_slots = "fp64", 64, max_slots
    srv.device, srv.memory_budget, srv.reserve = None, budget, 0
    srv.resident, srv.finished, srv.failed = [], [], []
    srv.used_bytes, srv.fill_cells, srv.resident_cells, srv.max_resident = 0, fill_cells, 0, 0
    srv._fits = lambda nbytes: srv.used_bytes + nbytes <= srv.memory_budget
    return srv


def _job(jid, cells):
    scene = types.SimpleNamespace(cells=cells)
    return S.Job(arrival=0.0, jid=jid, build=lambda: None, nsteps=10, scene=scene)


def test_fill_limit_holds_back_jobs_until_cells_retire(monkeypatch):
    srv = _server(monkeypatch, fill_cells=1000)
    a, b, c = _job(0, 600), _job(1, 300), _job(2, 200)
    assert srv._admit(a, 0.0) == "admitted"
    assert srv._admit(b, 0.0) == "admitted"          # 900 <= 1000
    assert srv._admit(c, 0.0) == "wait"              # 1100 > 1000
    assert srv.resident_cells == 900 and srv.max_resident == 2
    srv.resident.remove(a)
    srv._retire(a, 1.0)
    assert srv.resident_cells == 300 and srv.used_bytes == 300
    assert srv._admit(c, 1.0) == "admitted"
    assert srv.resident_cells == 500


def test_a_job_larger_than_the_fill_limit_runs_alone(monkeypatch):
    srv = _server(monkeypatch, fill_cells=1000)
    big, small = _job(0, 5000), _job(1, 10)
    assert srv._admit(big, 0.0) == "admitted"        # nothing resident: always admitted
    assert srv._admit(small, 0.0) == "wait"
    assert srv.max_resident == 1


def test_no_fill_limit_and_the_other_limits(monkeypatch):
    srv = _server(monkeypatch, fill_cells=0, max_slots=2, budget=1000)
    jobs = [_job(i, 400) for i in range(3)]
    assert srv._admit(jobs[0], 0.0) == "admitted"
    assert srv._admit(jobs[1], 0.0) == "admitted"
    assert srv._admit(jobs[2], 0.0) == "wait"        # slots (and memory: 1200 > 1000)
    srv.max_slots = 3
    assert srv._admit(jobs[2], 0.0) == "wait"        # memory
    srv.memory_budget = 1200
    assert srv._admit(jobs[2], 0.0) == "admitted"
    assert srv.resident_cells == 1200 and srv.max_resident == 3


def test_cancel_removes_queued_and_resident_jobs(monkeypatch):
    srv = _server(monkeypatch, fill_cells=0)
    srv._cancel = set()
    a, b, c, d = _job(0, 100), _job(1, 200), _job(2, 300), _job(3, 400)
    assert srv._admit(a, 0.0) == "admitted" and srv._admit(b, 0.0) == "admitted"
    pending, waiting = [d], [c]
    srv.cancel(1)   # resident
    srv.cancel(2)   # queued
    srv.cancel(3)   # not yet arrived
    srv.cancel(42)  # unknown: ignored
    srv._apply_cancellations(pending, waiting, 2.0)
    assert pending == [] and waiting == [] and srv.resident == [a]
    assert sorted(j.jid for j in srv.failed) == [1, 2, 3]
    assert all(j.error == "cancelled" and j.t_finish == 2.0 for j in srv.failed)
    assert srv.used_bytes == 100 and srv.resident_cells == 100
    assert b.engine is None
    srv._apply_cancellations(pending, waiting, 3.0)  # nothing left to cancel
    assert len(srv.failed) == 3


def test_failed_resident_job_frees_its_share(monkeypatch):
    srv = _server(monkeypatch, fill_cells=0)
    a, b = _job(0, 100), _job(1, 250)
    srv._admit(a, 0.0)
    srv._admit(b, 0.0)
    srv.resident.remove(b)
    srv._fail(b, 1.5, "non-finite field values")
    assert srv.used_bytes == 100 and srv.resident_cells == 100
    assert srv.failed == [b] and b.t_finish == 1.5 and b.engine is None


def test_saturation_copies():
    """Copies the batching bound steps together per grid: enough for 2^21
    cells, at most 128, at least one per side stream of the batch."""
    from gmes_gb300.batch import SOLO_STREAMS
    assert S.saturation_copies(1 << 14) == 128              # capped
    assert S.saturation_copies(1 << 16) == 32               # 2^21 / 2^16
    assert S.saturation_copies(100_000) == 21               # rounded up
    assert S.saturation_copies(1 << 20) == max(2, SOLO_STREAMS)
    assert S.saturation_copies(4096 ** 2) == SOLO_STREAMS   # large grid: one per side stream
    assert S.saturation_copies(4096 ** 2, min_copies=1) == 1
