"""Python driver of the CPU oracle (oracle/gmes_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.  The oracle
consumes the same compiled ``Scene`` as the CUDA engine and restates the
reference's per-point update loop on the CPU (see the C file's header for
the reference lines it follows).  Its fidelity is pinned against vectors
produced by the reference itself (tests/golden/).
"""

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "gmes_oracle.c"
BUILD = HERE / "_build"
LIB = BUILD / "libgmes_oracle.so"
CFLAGS = ["-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
          "-Wno-unknown-pragmas"]

_lib = None


def build():
    """Compile the oracle with gcc (no FMA contraction: the reference's operation order)."""
    BUILD.mkdir(exist_ok=True)
    if LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run(["gcc", *CFLAGS, str(SRC), "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = C.CDLL(str(LIB))
    P = C.POINTER
    lib.oracle_create.restype = C.c_void_p
    lib.oracle_create.argtypes = [P(C.c_int), C.c_int, P(C.c_double), P(C.c_double), C.c_double]
    lib.oracle_add_pml.restype = C.c_int
    lib.oracle_add_pml.argtypes = [C.c_void_p, C.c_int, P(C.c_double), C.c_double, C.c_double,
                                   C.c_double, C.c_double, C.c_double, P(C.c_double),
                                   P(C.c_double)]
    lib.oracle_add_class.restype = C.c_int
    lib.oracle_add_class.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                     C.c_int, P(C.c_double), C.c_int]
    lib.oracle_set_class_map.restype = C.c_int
    lib.oracle_set_class_map.argtypes = [C.c_void_p, C.c_int, P(C.c_uint8)]
    lib.oracle_set_sources.restype = C.c_int
    lib.oracle_set_sources.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_int),
                                       P(C.c_int64)]
    lib.oracle_field.restype = P(C.c_double)
    lib.oracle_field.argtypes = [C.c_void_p, C.c_int]
    lib.oracle_pml_profile.restype = C.c_int
    lib.oracle_pml_profile.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, P(C.c_double)]
    lib.oracle_step.restype = C.c_int
    lib.oracle_step.argtypes = [C.c_void_p, C.c_int, P(C.c_double)]
    lib.oracle_step_tfsf.restype = C.c_int
    lib.oracle_step_tfsf.argtypes = [C.c_void_p, C.c_int, P(C.c_double), P(C.c_double)]
    lib.oracle_set_tfsf.restype = C.c_int
    lib.oracle_set_tfsf.argtypes = [C.c_void_p, C.c_void_p, C.c_int, P(C.c_int), P(C.c_int),
                                    P(C.c_int64), P(C.c_double), P(C.c_double), P(C.c_double),
                                    P(C.c_int64)]
    lib.oracle_threads.restype = C.c_int
    lib.oracle_reset.restype = C.c_int
    lib.oracle_reset.argtypes = [C.c_void_p]
    lib.oracle_set_eps.restype = C.c_int
    lib.oracle_set_eps.argtypes = [C.c_void_p, C.c_int, C.c_int, P(C.c_int64), P(C.c_double)]
    lib.oracle_adjoint.restype = C.c_int
    lib.oracle_adjoint.argtypes = [C.c_void_p, C.c_int, P(C.c_double), C.c_int, P(C.c_int),
                                   P(C.c_int64), C.c_int, P(C.c_int), P(C.c_int64),
                                   P(C.c_double), P(C.c_double)]
    lib.oracle_destroy.argtypes = [C.c_void_p]
    lib.oracle_set_complex.restype = C.c_int
    lib.oracle_set_complex.argtypes = [C.c_void_p, C.c_void_p, P(C.c_double)]
    lib.oracle_step_complex.restype = C.c_int
    lib.oracle_step_complex.argtypes = [C.c_void_p, C.c_int, P(C.c_double), P(C.c_double),
                                        P(C.c_double), P(C.c_double)]
    _lib = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """CPU FDTD run of a compiled Scene (FP64, reference operation order).

    A complex (Bloch) scene runs as two C oracles, real and imaginary parts,
    coupled by the phase-shifted ghost copies (oracle_step_complex)."""

    def __init__(self, scene):
        self.lib = load()
        self.scene = scene
        self.cmplx = bool(getattr(scene, "cmplx", False))
        self.incident = Oracle(scene.tfsf[0]) if scene.tfsf is not None else None
        self.h = self._make(self.incident.h if self.incident is not None else None)
        self.h_im = None
        if self.cmplx:
            self.h_im = self._make(self.incident.h_im if self.incident is not None else None)
            ph = np.ascontiguousarray(scene.bloch_phase, np.float64)
            self.lib.oracle_set_complex(self.h, self.h_im, _dp(ph))
        self.n = 0.0

    def _make(self, incident_handle):
        """One C oracle with the scene's classes, maps, sources and TFSF table."""
        from gmes_gb300.scene import class_arrays, source_offsets
        scene = self.scene
        n = (C.c_int * 3)(*scene.n)
        dr = (C.c_double * 3)(*scene.dr)
        half = (C.c_double * 3)(*scene.half)
        h = self.lib.oracle_create(n, scene.active_mask, dr, half, scene.dt)
        if not h:
            raise MemoryError("oracle allocation failed")
        rows, pool, pmls = class_arrays(scene)
        for p in pmls:
            r = self.lib.oracle_add_pml(
                h, p["kind"], (C.c_double * 3)(*p["sigma_max"]), p["m"], p["kappa_max"],
                p["m_a"], p["a_max"], p["d"], (C.c_double * 3)(*p["center"]),
                (C.c_double * 3)(*p["half_size"]))
            if r < 0:
                raise ValueError("too many PML materials")
        pool = np.asarray(pool, np.float64) if pool else np.zeros(1)
        k = 0
        for c in range(6):
            for _ in scene.classes[c]:
                r = rows[k]
                prm = np.ascontiguousarray(pool[r["param_off"]:r["param_off"] + r["nparam"]])
                if self.lib.oracle_add_class(h, c, r["kind"], r["eps"], r["pml"], r["npole"],
                                             r["ncp"], _dp(prm), r["nparam"]) < 0:
                    raise ValueError("bad class")
                k += 1
        for c in range(6):
            if (scene.active_mask >> c) & 1:
                m = np.ascontiguousarray(scene.host_cls(c), np.uint8)
                if self.lib.oracle_set_class_map(h, c,
                                                 m.ctypes.data_as(C.POINTER(C.c_uint8))) != 0:
                    raise ValueError("bad class map")
        srcs = source_offsets(scene)
        comp = (C.c_int * max(1, len(srcs)))(*[s[0] for s in srcs])
        mode = (C.c_int * max(1, len(srcs)))(*[s[1] for s in srcs])
        off = (C.c_int64 * max(1, len(srcs)))(*[s[2] for s in srcs])
        self.lib.oracle_set_sources(h, len(srcs), comp, mode, off)
        if scene.tfsf is not None:
            points = scene.tfsf[1]
            n = len(points)
            tc = np.zeros(n, np.int32)
            nf = np.zeros(n, np.int32)
            to = np.zeros(n, np.int64)
            coef = np.zeros((n, 4))
            r0 = np.zeros((n, 4))
            r1 = np.zeros((n, 4))
            smp = np.zeros((n, 4), np.int64)
            for q, (c, o_, faces) in enumerate(points):
                tc[q], nf[q], to[q] = c, len(faces), o_
                for k, (cf, a, b, sp) in enumerate(faces):
                    coef[q, k], r0[q, k], r1[q, k], smp[q, k] = cf, a, b, sp
            ip = C.POINTER(C.c_int)
            lp = C.POINTER(C.c_int64)
            r = self.lib.oracle_set_tfsf(h, incident_handle, n, tc.ctypes.data_as(ip),
                                         nf.ctypes.data_as(ip), to.ctypes.data_as(lp),
                                         _dp(coef), _dp(r0), _dp(r1), smp.ctypes.data_as(lp))
            if r != 0:
                raise ValueError("bad TFSF table")
        return h

    def __del__(self):
        for name in ("h", "h_im"):
            if getattr(self, name, None):
                self.lib.oracle_destroy(getattr(self, name))
                setattr(self, name, None)

    def step(self, nsteps, src_values=None):
        from gmes_gb300.scene import source_values
        if src_values is None:
            src_values = source_values(self.scene, self.scene.dt, self.n, nsteps)

        def arr(a):
            a = np.ascontiguousarray(a, np.float64)
            return a if a.size else np.zeros(1)

        aux = None
        if self.incident is not None:
            aux = source_values(self.incident.scene, self.scene.dt, self.n, nsteps)
        if self.cmplx:
            sv = np.asarray(src_values, np.complex128)
            vr, vi = arr(sv.real), arr(sv.imag)
            if aux is not None:
                av = np.asarray(aux, np.complex128)
                ar, ai = arr(av.real), arr(av.imag)
                r = self.lib.oracle_step_complex(self.h, int(nsteps), _dp(vr), _dp(vi), _dp(ar),
                                                 _dp(ai))
            else:
                r = self.lib.oracle_step_complex(self.h, int(nsteps), _dp(vr), _dp(vi), None,
                                                 None)
            if r != 0:
                raise RuntimeError("complex oracle step failed")
            if self.incident is not None:
                self.incident.n += nsteps
        elif self.incident is not None:
            v, a = arr(src_values), arr(aux)
            self.lib.oracle_step_tfsf(self.h, int(nsteps), _dp(v), _dp(a))
            self.incident.n += nsteps
        else:
            v = arr(src_values)
            self.lib.oracle_step(self.h, int(nsteps), _dp(v))
        self.n += nsteps

    def field(self, c):
        sh = self.scene.shape(c)
        re = np.ctypeslib.as_array(self.lib.oracle_field(self.h, c), shape=sh).copy()
        if not self.cmplx:
            return re
        im = np.ctypeslib.as_array(self.lib.oracle_field(self.h_im, c), shape=sh)
        return re + 1j * im

    def fields(self):
        return [self.field(c) for c in range(6)]

    def pml_profile(self, pml, c, axis):
        n = self.scene.shape(c)[axis]
        out = np.zeros((n, 3), np.float64)
        if self.lib.oracle_pml_profile(self.h, pml, c, axis, _dp(out)) != 0:
            raise IndexError("bad pml index")
        return out

    def reset(self):
        """Zero the fields and every per-point state; time returns to 0."""
        self.lib.oracle_reset(self.h)
        if self.h_im:
            self.lib.oracle_reset(self.h_im)
        self.n = 0.0
        if self.incident is not None:
            self.incident.n = 0.0

    def set_eps(self, c, points, eps):
        """Per-point permittivity of dielectric points (c, index tuples) of component c."""
        sh = self.scene.shape(c)
        off = np.ascontiguousarray([np.ravel_multi_index(tuple(p), sh) for p in points],
                                   np.int64)
        e = np.ascontiguousarray(eps, np.float64).reshape(-1)
        if self.lib.oracle_set_eps(self.h, c, len(off), off.ctypes.data_as(C.POINTER(C.c_int64)),
                                   _dp(e)) != 0:
            raise ValueError("a point is not a dielectric point of this component")

    def adjoint(self, nsteps, monitor, design, gradient=True):
        """(J, dJ/deps) of J = dt * sum_n sum_monitor F^2 over nsteps steps from the current state.

        ``monitor`` and ``design``: lists of (component, index tuple); the
        gradient is with respect to the permittivity of each design point.
        """
        from gmes_gb300.scene import source_values
        vals = np.ascontiguousarray(source_values(self.scene, self.scene.dt, self.n, nsteps))
        if vals.size == 0:
            vals = np.zeros(1)

        def flat(pts):
            comp = np.ascontiguousarray([c for c, _ in pts], np.int32)
            off = np.ascontiguousarray(
                [np.ravel_multi_index(tuple(i), self.scene.shape(c)) for c, i in pts], np.int64)
            return comp, off

        mc, mo = flat(monitor)
        dc, do = flat(design)
        J = C.c_double()
        grad = np.zeros(max(1, len(design)), np.float64)
        r = self.lib.oracle_adjoint(
            self.h, int(nsteps), _dp(vals), len(mc), mc.ctypes.data_as(C.POINTER(C.c_int)),
            mo.ctypes.data_as(C.POINTER(C.c_int64)), len(dc),
            dc.ctypes.data_as(C.POINTER(C.c_int)), do.ctypes.data_as(C.POINTER(C.c_int64)),
            C.byref(J), _dp(grad) if gradient else None)
        if r == -1:
            raise ValueError("the adjoint supports Dielectric and CPML classes only")
        if r == -2:
            raise ValueError("a design point is not a dielectric E point")
        if r != 0:
            raise MemoryError("oracle adjoint allocation failed")
        self.n += nsteps
        return J.value, grad[:len(design)]

    @staticmethod
    def threads():
        return load().oracle_threads()
