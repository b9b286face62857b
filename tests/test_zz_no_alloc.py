"""The batch step that allocates nothing, against the workspace batch step.

gmes_batch_step_noalloc serves callers that may not allocate device memory
(their memory pool owns the GPU, or a cudaMalloc's implicit synchronisation
is not allowed in their loop): it keeps the batch tables in a fixed array
inside the library instead of a caller workspace.  This test runs two
identical sets of grids, one through gmes_batch_prepare / gmes_batch_set_steps
/ gmes_batch_step with a workspace, the other through
gmes_batch_step_noalloc, both through the C ABI, and requires the same
fields (the batch kernels are deterministic, so the tolerance is exact
equality) after each of three calls in a row (the third with a narrower
block shape, which changes only how the cells are split into blocks).  The
device's free memory is the same before and after a call once the kernels
are loaded.  It builds everything it needs itself, so it passes alone in a
fresh process as well as after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

import gmes_gb300 as G
from gmes_gb300 import _native as N
from gmes_gb300 import workloads as W
from gmes_gb300.engine import GridEngine
from cases import CASES

pytestmark = pytest.mark.gpu

PULSE = G.Bandpass(freq=1.0, fwidth=1.0)


def grids():
    return [CASES["drude2d"](G)[0], W.cube(n=36, nobj=3, pml_cells=4, src_time=PULSE)[0],
            CASES["tez_upml_currents"](G)[0]]


def stage(engines, steps, n0s):
    for e, k, n0 in zip(engines, steps, n0s):
        if k:
            e.stage_sources(n0, k)
    for e in engines:
        e.synchronize()


def test_noalloc_batch_matches_workspace_batch():
    import torch
    lib = N.load()
    a = [GridEngine(s.compile(), src_chunk=32) for s in grids()]
    b = [GridEngine(s.compile(), src_chunk=32) for s in grids()]
    n = len(a)
    stream = torch.cuda.Stream()
    ws_bytes = int(lib.gmes_batch_workspace_size(n))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    desc_a = (C.POINTER(N.GridDescC) * n)(*[C.pointer(e.desc) for e in a])
    desc_b = (C.POINTER(N.GridDescC) * n)(*[C.pointer(e.desc) for e in b])
    batch = N.BatchC()
    torch.cuda.synchronize()
    N.check(lib.gmes_batch_prepare(desc_a, n, C.c_void_p(ws.data_ptr()), ws_bytes, 0,
                                   C.byref(batch), C.c_void_p(stream.cuda_stream)))
    done = [0] * n
    for call, (steps, bx_cap) in enumerate((([13, 7, 20], 0), ([5, 12, 9], 0),
                                            ([8, 3, 11], 3))):
        k = max(steps)
        stage(a, steps, done)
        stage(b, steps, done)
        st = (C.c_int32 * n)(*steps)
        N.check(lib.gmes_batch_set_steps(C.byref(batch), st, C.c_void_p(stream.cuda_stream)))
        N.check(lib.gmes_batch_step(C.byref(batch), k, 0, C.c_void_p(stream.cuda_stream)))
        stream.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        N.check(lib.gmes_batch_step_noalloc(desc_b, st, n, k, bx_cap,
                                            C.c_void_p(stream.cuda_stream)))
        stream.synchronize()
        if call > 0:  # the first call also loads the kernels
            assert torch.cuda.mem_get_info()[0] == free0, call
        done = [d + s for d, s in zip(done, steps)]
        for q in range(n):
            for c in range(6):
                fa, fb = a[q].read(c), b[q].read(c)
                assert np.isfinite(fa).all()
                assert np.array_equal(fa, fb), (call, q, c)
        assert any(np.abs(a[q].read(c)).max() > 0 for q in range(n) for c in range(6))


def test_noalloc_rejects_more_grids_than_its_table_holds():
    lib = N.load()
    e = GridEngine(grids()[0].compile())
    n = N.NOALLOC_MAX_GRIDS + 1
    descs = (C.POINTER(N.GridDescC) * n)(*([C.pointer(e.desc)] * n))
    steps = (C.c_int32 * n)(*([1] * n))
    with pytest.raises(ValueError, match="capacity"):
        N.check(lib.gmes_batch_step_noalloc(descs, steps, n, 1, 0, None))


def test_noalloc_rejects_steps_beyond_the_staged_source_values():
    lib = N.load()
    e = GridEngine(grids()[0].compile(), src_chunk=8)
    assert e.desc.nsrc > 0
    descs = (C.POINTER(N.GridDescC) * 1)(C.pointer(e.desc))
    steps = (C.c_int32 * 1)(9)
    with pytest.raises(ValueError, match="source-value capacity"):
        N.check(lib.gmes_batch_step_noalloc(descs, steps, 1, 9, 0, None))
