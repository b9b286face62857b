"""ctypes binding of ``libgmes_gb300.so`` (include/gmes_gb300.h).

The structures below mirror the header field for field.  Loading fails
loudly when the library is missing: the package has no CPU fallback.
"""

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
# GMES_GB300_LIB selects another build of the library (e.g. one compiled
# with different tuning macros); the default is the in-tree build.
LIB_PATH = Path(os.environ["GMES_GB300_LIB"]) if os.environ.get("GMES_GB300_LIB") else \
    PKG / "libgmes_gb300.so"

ABI_VERSION = 6
MAX_CLASSES = 256
MAX_PML = 4
MAX_POLES = 8

FP64, FP32, DF64, FP64_STRICT = 0, 1, 2, 3
PRECISIONS = {"fp64": FP64, "fp32": FP32, "df64": DF64, "fp64_strict": FP64_STRICT}
FLAG_DISPERSIVE = 1
FLAG_POINTWISE = 4
FLAG_COMPLEX = 2

EXPORTS = [
    "gmes_abi_version", "gmes_last_error", "gmes_elem_size", "gmes_field_shape",
    "gmes_grid_sizes", "gmes_build_coefficients", "gmes_set_pml_profile",
    "gmes_get_pml_profile", "gmes_reset",
    "gmes_step", "gmes_half_step", "gmes_read_field", "gmes_write_field",
    "gmes_batch_workspace_size", "gmes_batch_prepare", "gmes_batch_set_steps", "gmes_batch_step",
    "gmes_graph_capture_step", "gmes_graph_capture_batch", "gmes_graph_launch",
    "gmes_graph_destroy", "gmes_rasterize", "gmes_batch_step_noalloc",
    "gmes_tmz_sizes", "gmes_tmz_check", "gmes_tmz_set_design", "gmes_tmz_reset",
    "gmes_tmz_forward", "gmes_tmz_objective", "gmes_tmz_adjoint", "gmes_points_update",
    "gmes_copy_async", "gmes_nonfinite",
]
NOALLOC_MAX_GRIDS = 64


class ClassDescC(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pml", C.c_int32), ("npole", C.c_int32),
                ("ncp", C.c_int32), ("param_off", C.c_int32), ("nparam", C.c_int32),
                ("eps", C.c_double)]


class PmlDescC(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad", C.c_int32), ("sigma_max", C.c_double * 3),
                ("m", C.c_double), ("kappa_max", C.c_double), ("m_a", C.c_double),
                ("a_max", C.c_double), ("d", C.c_double), ("center", C.c_double * 3),
                ("half_size", C.c_double * 3)]


class PointSourceC(C.Structure):
    _fields_ = [("comp", C.c_int32), ("mode", C.c_int32), ("offset", C.c_int64)]


TFSF_MAX_FACES = 4


class TransparentC(C.Structure):
    _fields_ = [("comp", C.c_int32), ("nface", C.c_int32), ("offset", C.c_int64),
                ("coef", C.c_double * TFSF_MAX_FACES), ("r0", C.c_double * TFSF_MAX_FACES),
                ("r1", C.c_double * TFSF_MAX_FACES), ("sample", C.c_int64 * TFSF_MAX_FACES)]


class ProbeC(C.Structure):
    _fields_ = [("comp", C.c_int32), ("pad", C.c_int32), ("offset", C.c_int64)]


class GridDescC(C.Structure):
    pass


GridDescC._fields_ = [
    ("abi_version", C.c_int32), ("precision", C.c_int32), ("n", C.c_int32 * 3),
    ("active", C.c_int32), ("naux", C.c_int32 * 6), ("nclass", C.c_int32 * 6),
    ("npml", C.c_int32), ("nsrc", C.c_int32), ("nparam", C.c_int32),
    ("src_steps", C.c_int32), ("flags", C.c_int32), ("reserved", C.c_int32),
    ("dr", C.c_double * 3), ("half", C.c_double * 3), ("dt", C.c_double),
    ("field", C.c_void_p * 6), ("cls", C.c_void_p * 6), ("aux", C.c_void_p * 6),
    ("coef", C.c_void_p), ("src", C.c_void_p), ("src_val", C.c_void_p),
    ("ntfsf", C.c_int32), ("reserved2", C.c_int32), ("tfsf", C.c_void_p),
    ("incident", C.POINTER(GridDescC)),
    ("nprobe", C.c_int32), ("probe_steps", C.c_int32), ("probe", C.c_void_p),
    ("probe_val", C.c_void_p), ("bloch_phase", ((C.c_double * 2) * 2) * 6),
]


class ShapeC(C.Structure):
    _fields_ = [("type", C.c_int32), ("compound", C.c_int32), ("nbox", C.c_int32),
                ("pad", C.c_int32), ("lo", C.c_double * 3), ("hi", C.c_double * 3),
                ("center", C.c_double * 3), ("m", C.c_double * 9), ("p", C.c_double * 3),
                ("axis", C.c_double * 3), ("box_lo", (C.c_double * 3) * 6),
                ("box_hi", (C.c_double * 3) * 6)]


SHAPE_ALL, SHAPE_SPHERE, SHAPE_BLOCK, SHAPE_ELLIPSOID, SHAPE_CONE, SHAPE_SHELL = range(6)


class BatchC(C.Structure):
    _fields_ = [("njobs", C.c_int32), ("precision", C.c_int32), ("dispersive", C.c_int32),
                ("srcs", C.c_int32), ("tiles", C.c_int64), ("ghosts", C.c_int64),
                ("workspace", C.c_void_p), ("workspace_bytes", C.c_int64)]


TMZ_RECORD_MONITOR, TMZ_RECORD_HIST = 1, 2


class TmzBatchC(C.Structure):
    _fields_ = [("nbatch", C.c_int32), ("design_lo", C.c_int32 * 2), ("design_n", C.c_int32 * 2),
                ("monitor_lo", C.c_int32 * 2), ("monitor_n", C.c_int32 * 2),
                ("nsrc", C.c_int32), ("total_steps", C.c_int32), ("hist_steps", C.c_int32),
                ("block_steps", C.c_int32),
                ("state", C.c_void_p), ("adjoint", C.c_void_p), ("design", C.c_void_p),
                ("hist", C.c_void_p), ("monitor", C.c_void_p), ("grad", C.c_void_p),
                ("weight", C.c_void_p), ("src", C.c_void_p), ("src_val", C.c_void_p),
                ("scratch", C.c_void_p)]


class PointsC(C.Structure):
    _fields_ = [("comp", C.c_int32), ("kind", C.c_int32), ("npoints", C.c_int32),
                ("nparam", C.c_int32), ("nstate", C.c_int32), ("npole", C.c_int32),
                ("ncp", C.c_int32), ("cmplx", C.c_int32), ("idx", C.c_void_p),
                ("param", C.c_void_p), ("state", C.c_void_p),
                ("shape", (C.c_int64 * 3) * 3)]


class GmesError(RuntimeError):
    """Base of the errors raised for a failed engine call."""


_STATUS_EXC = {1: ValueError, 2: IndexError, 3: RuntimeError, 4: RuntimeError}

_lib = None


def load():
    """The loaded engine library (built on first use when nvcc is present)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if os.environ.get("GMES_GB300_LIB"):
            raise RuntimeError(f"GMES_GB300_LIB={LIB_PATH} does not exist")
        from . import build as _build
        _build.build()
    lib = C.CDLL(str(LIB_PATH))
    P = C.POINTER
    lib.gmes_abi_version.restype = C.c_int
    lib.gmes_last_error.restype = C.c_char_p
    lib.gmes_elem_size.restype = C.c_int
    lib.gmes_elem_size.argtypes = [C.c_int32]
    lib.gmes_field_shape.argtypes = [P(GridDescC), C.c_int32, P(C.c_int64)]
    lib.gmes_grid_sizes.argtypes = [P(GridDescC), P(C.c_int64)]
    lib.gmes_build_coefficients.argtypes = [P(GridDescC), P(ClassDescC), P(C.c_double),
                                            P(PmlDescC), C.c_void_p]
    lib.gmes_set_pml_profile.argtypes = [P(GridDescC), C.c_int32, C.c_int32, C.c_int32,
                                         P(C.c_double), C.c_void_p]
    lib.gmes_get_pml_profile.argtypes = [P(GridDescC), C.c_int32, C.c_int32, C.c_int32,
                                         P(C.c_double), C.c_void_p]
    lib.gmes_reset.argtypes = [P(GridDescC), C.c_void_p]
    lib.gmes_step.argtypes = [P(GridDescC), C.c_int32, C.c_void_p]
    lib.gmes_half_step.argtypes = [P(GridDescC), C.c_int32, C.c_int32, C.c_void_p]
    lib.gmes_read_field.argtypes = [P(GridDescC), C.c_int32, P(C.c_double), C.c_void_p]
    lib.gmes_write_field.argtypes = [P(GridDescC), C.c_int32, P(C.c_double), C.c_void_p]
    lib.gmes_batch_workspace_size.restype = C.c_int64
    lib.gmes_batch_workspace_size.argtypes = [C.c_int32]
    lib.gmes_batch_prepare.argtypes = [P(P(GridDescC)), C.c_int32, C.c_void_p, C.c_int64,
                                       C.c_int32, P(BatchC), C.c_void_p]
    lib.gmes_batch_set_steps.argtypes = [P(BatchC), P(C.c_int32), C.c_void_p]
    lib.gmes_batch_step.argtypes = [P(BatchC), C.c_int32, C.c_int32, C.c_void_p]
    lib.gmes_graph_capture_step.argtypes = [P(GridDescC), C.c_int32, C.c_void_p,
                                            P(C.c_void_p)]
    lib.gmes_graph_capture_batch.argtypes = [P(BatchC), C.c_int32, C.c_int32, C.c_void_p,
                                             P(C.c_void_p)]
    lib.gmes_graph_launch.argtypes = [C.c_void_p, C.c_void_p]
    lib.gmes_batch_step_noalloc.argtypes = [P(P(GridDescC)), P(C.c_int32), C.c_int32,
                                            C.c_int32, C.c_int32, C.c_void_p]
    lib.gmes_rasterize.argtypes = [P(GridDescC), C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                   C.c_void_p]
    lib.gmes_graph_destroy.argtypes = [C.c_void_p]
    lib.gmes_copy_async.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    lib.gmes_nonfinite.argtypes = [P(GridDescC), C.c_void_p, C.c_void_p]
    G, B = P(GridDescC), P(TmzBatchC)
    lib.gmes_tmz_sizes.argtypes = [G, B, P(C.c_int64)]
    lib.gmes_tmz_check.argtypes = [G, B]
    lib.gmes_tmz_set_design.argtypes = [G, B, C.c_void_p, C.c_void_p]
    lib.gmes_tmz_reset.argtypes = [G, B, C.c_int32, C.c_void_p]
    lib.gmes_tmz_forward.argtypes = [G, B, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]
    lib.gmes_tmz_objective.argtypes = [G, B, C.c_int32, C.c_void_p, C.c_void_p]
    lib.gmes_tmz_adjoint.argtypes = [G, B, C.c_int32, C.c_int32, C.c_void_p]
    lib.gmes_points_update.argtypes = [P(PointsC), C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_double, C.c_double, C.c_double, C.c_void_p]
    for name in EXPORTS:
        if name not in ("gmes_abi_version", "gmes_last_error", "gmes_elem_size",
                        "gmes_batch_workspace_size"):
            getattr(lib, name).restype = C.c_int
    if lib.gmes_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{LIB_PATH}: ABI {lib.gmes_abi_version()}, expected {ABI_VERSION}")
    _lib = lib
    return lib


def check(status):
    """Raise the Python exception matching a non-zero gmes_status."""
    if status == 0:
        return
    msg = load().gmes_last_error().decode(errors="replace")
    raise _STATUS_EXC.get(status, RuntimeError)(msg)
