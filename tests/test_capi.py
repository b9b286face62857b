"""The C ABI library: loads, exports what include/gmes_gb300.h declares, and
validates descriptors on the host (no GPU needed for these calls)."""
import ctypes as C
import re
from pathlib import Path

import pytest

from gmes_gb300 import _native as N

HEADER = Path(__file__).resolve().parents[1] / "include" / "gmes_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gmes_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    lib = N.load()
    names = declared_functions()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), f"{name} declared in gmes_gb300.h but not exported"
    assert sorted(N.EXPORTS) == names


def test_abi_version_and_elem_sizes():
    lib = N.load()
    assert lib.gmes_abi_version() == N.ABI_VERSION
    assert [lib.gmes_elem_size(p) for p in (N.FP64, N.FP32, N.DF64, N.FP64_STRICT)] == [8, 4, 8, 8]
    assert lib.gmes_elem_size(9) == 0


def _desc(**kw):
    d = N.GridDescC()
    d.abi_version = N.ABI_VERSION
    d.precision = kw.get("precision", N.FP64)
    for a in range(3):
        d.n[a] = kw.get("n", (4, 5, 6))[a]
        d.dr[a] = 0.1
    d.dt = 0.05
    d.active = kw.get("active", 63)
    for c in range(6):
        d.nclass[c] = 2
        d.naux[c] = 2
    d.npml = kw.get("npml", 1)
    return d


def test_grid_sizes_match_reference_shapes():
    lib = N.load()
    d = _desc()
    sizes = (C.c_int64 * 21)()
    N.check(lib.gmes_grid_sizes(C.byref(d), sizes))
    shapes = [(4, 6, 7), (5, 5, 7), (5, 6, 6), (4, 6, 7), (5, 5, 7), (5, 6, 6)]
    for c, sh in enumerate(shapes):
        np_ = sh[0] * sh[1] * sh[2]
        assert sizes[c] == 8 * np_
        assert sizes[6 + c] == np_
        assert sizes[12 + c] == 2 * 8 * np_
        s = (C.c_int64 * 3)()
        N.check(lib.gmes_field_shape(C.byref(d), c, s))
        assert tuple(s) == sh
    assert sizes[18] > 0 and sizes[18] % 256 == 0


def test_inactive_components_are_one_point():
    lib = N.load()
    d = _desc(active=0b110100)  # TMz: Ez, Hx, Hy
    s = (C.c_int64 * 3)()
    N.check(lib.gmes_field_shape(C.byref(d), 0, s))
    assert tuple(s) == (1, 1, 1)
    N.check(lib.gmes_field_shape(C.byref(d), 2, s))
    assert tuple(s) == (5, 6, 6)


@pytest.mark.parametrize("field,value,exc", [
    ("abi_version", 99, ValueError),
    ("precision", 7, ValueError),
    ("active", 0b000111, ValueError),
    ("npml", 9, ValueError),
])
def test_descriptor_validation(field, value, exc):
    lib = N.load()
    d = _desc()
    setattr(d, field, value)
    sizes = (C.c_int64 * 21)()
    with pytest.raises(exc):
        N.check(lib.gmes_grid_sizes(C.byref(d), sizes))
    assert lib.gmes_last_error()


def test_bad_component_index():
    lib = N.load()
    d = _desc()
    s = (C.c_int64 * 3)()
    with pytest.raises(IndexError):
        N.check(lib.gmes_field_shape(C.byref(d), 6, s))


def test_step_rejects_null_buffers_without_touching_the_gpu():
    lib = N.load()
    d = _desc()
    with pytest.raises(ValueError, match="NULL"):
        N.check(lib.gmes_step(C.byref(d), 1, None))


def _tmz(**kw):
    b = N.TmzBatchC()
    b.nbatch = kw.get("nbatch", 2)
    lo, n = kw.get("design", ((2, 3), (4, 5)))
    for a in range(2):
        b.design_lo[a], b.design_n[a] = lo[a], n[a]
        b.monitor_lo[a], b.monitor_n[a] = 1, 2
    b.nsrc = 0
    b.total_steps = 10
    b.hist_steps = 4
    return b


def test_tmz_sizes_and_validation():
    lib = N.load()
    d = _desc(n=(16, 12, 1), active=(1 << 2) | (1 << 3) | (1 << 4))
    sizes = (C.c_int64 * 7)()
    N.check(lib.gmes_tmz_sizes(C.byref(d), C.byref(_tmz()), sizes))
    arr = ((2 * 16 * 12 * 8 + 255) // 256) * 256
    assert sizes[0] == 7 * arr and sizes[1] == 11 * arr
    up = lambda v: ((v + 255) // 256) * 256
    # DesignCoef = 48 bytes per pixel, then the lattice map: flags + 4 coefficient arrays
    assert sizes[2] == up(2 * 20 * 48) + up(16 * 12 * 4) + 4 * up(16 * 12 * 8)
    assert sizes[3] == ((4 * 2 * 20 * 8 + 255) // 256) * 256
    assert sizes[4] == ((2 * 10 * 4 * 8 + 255) // 256) * 256
    assert sizes[6] == 0                                     # FP64: one step per launch
    d32 = _desc(n=(16, 12, 1), active=(1 << 2) | (1 << 3) | (1 << 4))
    d32.precision = N.FP32
    N.check(lib.gmes_tmz_sizes(C.byref(d32), C.byref(_tmz()), sizes))
    arr32 = ((2 * 16 * 12 * 4 + 255) // 256) * 256
    assert sizes[0] == 7 * arr32 and sizes[6] == 7 * arr32  # blocked kernels: scratch state
    one = _tmz()
    one.block_steps = 1
    N.check(lib.gmes_tmz_sizes(C.byref(d32), C.byref(one), sizes))
    assert sizes[6] == 0
    bad = _tmz()
    bad.block_steps = 5
    with pytest.raises(ValueError):
        N.check(lib.gmes_tmz_sizes(C.byref(d32), C.byref(bad), sizes))
    with pytest.raises(IndexError):
        N.check(lib.gmes_tmz_sizes(C.byref(d), C.byref(_tmz(design=((14, 3), (4, 5)))), sizes))
    with pytest.raises(ValueError):
        N.check(lib.gmes_tmz_sizes(C.byref(_desc(n=(16, 12, 1))), C.byref(_tmz()), sizes))
    d.precision = N.FP64_STRICT
    with pytest.raises(ValueError):
        N.check(lib.gmes_tmz_sizes(C.byref(d), C.byref(_tmz()), sizes))


def test_copy_async_validates_before_any_copy():
    lib = N.load()
    buf = (C.c_char * 16)()
    ok, err_value = 0, 1  # GMES_OK, GMES_ERR_VALUE
    assert lib.gmes_copy_async(None, None, 0, None) == ok  # nothing to copy
    assert lib.gmes_copy_async(buf, buf, -1, None) == err_value
    assert b"negative" in lib.gmes_last_error()
    assert lib.gmes_copy_async(None, buf, 8, None) == err_value
    assert lib.gmes_copy_async(buf, None, 8, None) == err_value
    assert b"NULL" in lib.gmes_last_error()
