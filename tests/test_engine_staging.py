"""The per-step source staging of GridEngine on the host: the values land in
the pinned buffer in the layout the kernels read (slot s of the chunk =
row s, a complex grid's imaginary plane src_chunk rows after the real one),
and the copies the library is asked for cover exactly the staged rows.
No GPU: the library call and the CUDA event are replaced by recorders."""
import ctypes as C
import types

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gmes_gb300.engine import GridEngine  # noqa: E402


class _Lib:
    def __init__(self):
        self.copies = []

    def gmes_copy_async(self, dst, src, nbytes, stream):
        self.copies.append((dst.value, src.value, nbytes, stream.value))
        return 0


class _Event:
    def __init__(self):
        self.recorded = []

    def synchronize(self):
        pass

    def record(self, stream):
        self.recorded.append(stream)


def _engine(cmplx, chunk, nsrc):
    e = object.__new__(GridEngine)
    lead = (2,) if cmplx else ()
    e.cmplx = cmplx
    e.src_chunk = chunk
    e.src_val = torch.zeros(lead + (chunk, 2, nsrc), dtype=torch.float64)
    e.src_host = torch.zeros(e.src_val.shape, dtype=torch.float64)
    e._src_host_np = e.src_host.numpy()
    e.lib = _Lib()
    e._staged = _Event()
    e._stream = types.SimpleNamespace(cuda_stream=1234)
    return e


@pytest.mark.parametrize("cmplx", [False, True])
@pytest.mark.parametrize("k", [1, 5, 8])
def test_stage_layout_and_copies(cmplx, k):
    chunk, nsrc = 8, 3
    e = _engine(cmplx, chunk, nsrc)
    rng = np.random.default_rng(k)
    vals = rng.standard_normal((k, 2, nsrc))
    if cmplx:
        vals = vals + 1j * rng.standard_normal((k, 2, nsrc))
    e._stage(vals, k)
    host = e.src_host.numpy()
    if cmplx:
        assert np.array_equal(host[0, :k], vals.real) and np.array_equal(host[1, :k], vals.imag)
    else:
        assert np.array_equal(host[:k], vals)
    row = 2 * nsrc * 8
    planes = 2 if cmplx else 1
    assert len(e.lib.copies) == planes
    for q, (dst, src, nbytes, stream) in enumerate(e.lib.copies):
        assert dst == e.src_val.data_ptr() + q * chunk * row
        assert src == e.src_host.data_ptr() + q * chunk * row
        assert nbytes == k * row and stream == 1234
        # the copied bytes are exactly the staged rows of that plane
        flat = e.src_host.view(-1).numpy()
        first = (src - e.src_host.data_ptr()) // 8
        staged = (vals.imag if q else vals.real) if cmplx else vals
        assert np.array_equal(flat[first:first + nbytes // 8], staged.reshape(-1))
    assert e._staged.recorded == [e._stream]
