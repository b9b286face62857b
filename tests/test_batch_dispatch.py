"""How a Batch chunk is dispatched, on the host: the small grids' step
counts go to the multi-grid kernel in their order, each large (solo) grid
replays its own chunk graph when it runs the full chunk and plain launches
otherwise, solo grids spread over the side streams, which start after the
staging and join the batch's stream at the end, and the launch count adds
up.  No GPU: the library and the streams are recorders."""
import ctypes as C
import types

import pytest

pytest.importorskip("torch")

from gmes_gb300 import _native as N  # noqa: E402
from gmes_gb300.batch import Batch  # noqa: E402


class _Lib:
    def __init__(self):
        self.calls = []
        self.streams = []  # stream of each solo launch

    def gmes_batch_set_steps(self, b, steps, stream):
        self.calls.append(("set_steps", list(steps)))
        return 0

    def gmes_graph_launch(self, h, stream):
        self.calls.append(("graph", h.value))
        self.streams.append(stream.value)
        return 0

    def gmes_batch_step(self, b, k, blocks, stream):
        self.calls.append(("batch_step", k))
        return 0

    def gmes_step(self, desc, k, stream):
        self.calls.append(("step", k))
        self.streams.append(stream.value)
        return 0


def _engine(cells, nsrc, handle):
    d = N.GridDescC()
    d.nsrc = nsrc
    return types.SimpleNamespace(scene=types.SimpleNamespace(cells=cells), desc=d,
                                 _graph=lambda k, h=handle: h + k)


class _Stream:
    def __init__(self, handle, batch):
        self.cuda_stream, self.batch = handle, batch

    def wait_stream(self, other):
        self.batch.lib.calls.append(("wait", self.cuda_stream, other.cuda_stream))


def _batch(engines, solo, use_graphs=True):
    b = object.__new__(Batch)
    b.engines, b.solo = engines, solo
    b.multi = [i for i in range(len(engines)) if i not in solo]
    b.lib, b.use_graphs, b.blocks = _Lib(), use_graphs, 0
    b.stream = _Stream(7, b)
    b._side = []
    b.b = N.BatchC()
    b.b.ghosts, b.b.srcs = 10, 1
    b._steps = (C.c_int32 * len(b.multi))()
    b._graph = lambda k: 5000 + k
    b.stage = lambda steps, n0s: None
    return b


@pytest.mark.parametrize("use_graphs", [True, False])
def test_chunk_dispatch_and_launch_count(use_graphs):
    engines = [_engine(2 << 20, 1, 1000), _engine(3 << 20, 0, 2000),
               _engine(4000, 1, 0), _engine(900, 0, 0)]
    b = _batch(engines, solo=[0, 1], use_graphs=use_graphs)
    n = b.run([32, 10, 32, 5])
    calls = b.lib.calls
    assert calls[0] == ("set_steps", [32, 5])
    if use_graphs:
        assert calls[1:] == [("graph", 5032), ("graph", 1032), ("step", 10)]
    else:
        assert calls[1:] == [("batch_step", 32), ("step", 32), ("step", 10)]
    multi = 2 * (1 + 1 + 1)                   # ghost, cell, sources per half-step
    solo0, solo1 = 2 * (2 + 1), 2 * (2 + 0)   # ghost + cell (+ sources)
    assert n == 32 * multi + 32 * solo0 + 10 * solo1
    assert b.launches_per_step == multi + solo0 + solo1


def test_all_solo_and_idle_chunks():
    engines = [_engine(2 << 20, 0, 1000), _engine(2 << 20, 0, 2000)]
    b = _batch(engines, solo=[0, 1])
    b.b, b.multi = None, []
    assert b.tiles == 0
    assert b.run([0, 0]) == 0 and b.lib.calls == []
    assert b.run([7, 0]) == 7 * 4
    assert b.lib.calls == [("graph", 1007)]


def test_solo_grids_on_side_streams():
    engines = [_engine(2 << 20, 0, 1000), _engine(2 << 20, 0, 2000), _engine(2 << 20, 0, 3000),
               _engine(4000, 1, 0)]
    b = _batch(engines, solo=[0, 1, 2])
    b._side = [_Stream(8, b), _Stream(9, b)]
    b.run([16, 16, 16, 16])
    calls = b.lib.calls
    # the side streams wait for the staging before the multi-grid chunk is enqueued
    assert calls[:3] == [("wait", 8, 7), ("wait", 9, 7), ("set_steps", [16])]
    assert calls[3] == ("graph", 5016)
    assert calls[4:7] == [("graph", 1016), ("graph", 2016), ("graph", 3016)]
    assert b.lib.streams == [7, 8, 9, 8]  # the multi-grid chunk, then the solo grids
    assert calls[7:] == [("wait", 7, 8), ("wait", 7, 9)]
    # one solo grid left: it runs on the batch's stream, no side streams
    b.lib = _Lib()
    b.run([0, 5, 0, 0])
    assert b.lib.calls == [("graph", 2005)] and b.lib.streams == [7]
