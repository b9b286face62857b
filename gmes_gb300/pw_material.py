"""Point-wise material updaters with the interface of the reference's
``gmes.pw_material`` module (SWIG bindings of src/pw_*.hh,
src/pw_material.i:138-389), computed on the GPU.

Each updater class ``<Model><Comp><Real|Cmplx>`` (``DielectricExReal``,
``CpmlHyCmplx``, ...) keeps the reference's methods:

* ``attach(idx, param)`` -- copy ``param`` and attach it at index ``idx``;
* ``merge(other)`` -- append another updater's points;
* ``update_all(inplace, in1, in2, d1, d2, dt, n)`` -- update the attached
  points of ``inplace`` in place (numpy arrays, float64 or complex128,
  C-contiguous; a float64 CUDA tensor is used without a copy);
* ``idx_size()``, ``name()``, ``get_eps_inf(idx)`` / ``get_mu_inf(idx)``.

Parameter structs ``<Model><Electric|Magnetic>Param<Real|Cmplx>`` have the
reference's fields and ``set()`` helpers.  Errors follow the reference's
binding: a bad argument raises ValueError, an attached index outside the
target array IndexError("field index is out of bounds") before any write,
a read-only or wrongly typed array TypeError.

The points of an updater live on the GPU as a structure of arrays (index,
parameters, state); one ``gmes_points_update`` call runs one thread per
point in the reference's FP64 operation order.
"""

import copy
import ctypes as C

import numpy as np

from . import _native as N
from .material import (KIND_CONST, KIND_CPML, KIND_DCP, KIND_DCP_PLRC, KIND_DIELECTRIC,
                       KIND_DRUDE, KIND_DUMMY, KIND_LORENTZ, KIND_UPML)


# ---------------------------------------------------------------------------
# Parameter structs
# ---------------------------------------------------------------------------
class PwMaterialParam:
    """Base of the parameter structs (value-initialised: every field 0)."""

    _fields = ()

    def __init__(self):
        for f in self._fields:
            setattr(self, f, 0.0)


def _param(name, base_field, fields=(), setter=None, lists=()):
    def __init__(self):
        PwMaterialParam.__init__(self)
        for f in lists:
            setattr(self, f, [])
    ns = {"_fields": (base_field,) + tuple(fields), "__init__": __init__}
    if setter is not None:
        ns["set"] = setter
    return type(name, (PwMaterialParam,), ns)


def _rows(a, width, what, dtype=np.float64):
    a = np.asarray(a, dtype)
    if a.ndim != 2 or a.shape[1] != width:
        raise ValueError(what)
    return [list(r) for r in a]


def _vec(c, length, what):
    c = np.asarray(c, np.float64)
    if c.ndim != 1 or c.shape[0] != length:
        raise ValueError(what)
    return list(c)


def _set_ac(kind):
    msg = f"{kind} coefficients require shapes (n, 3) and (3,)"
    state = ("q_now", "q_new") if kind == "Drude" else ("l_now", "l_new")

    def set(self, a, c):
        self.a = _rows(a, 3, msg)
        self.c = _vec(c, 3, msg)
        for f in state:
            setattr(self, f, [0.0] * len(self.a))
    return set


def _set_dcp_ade(self, a, b, c):
    msg = "DcpAde coefficients require shapes (n, 3), (n, 5), and (4,)"
    self.a = _rows(a, 3, msg)
    self.b = _rows(b, 5, msg)
    self.c = _vec(c, 4, msg)
    self.q_old = [0.0] * len(self.a)
    self.q_now = [0.0] * len(self.a)
    self.p_old = [0.0] * len(self.b)
    self.p_now = [0.0] * len(self.b)


def _set_dcp_plrc(self, a, b, c):
    msg = "DcpPlrc coefficients require shapes (n, 3), (n, 3), and (3,)"
    self.a = _rows(a, 3, msg)
    self.b = _rows(b, 3, msg, np.complex128)
    self.c = _vec(c, 3, msg)
    self.psi_dp_re = [0.0] * len(self.a)
    self.psi_dp_im = [0.0] * len(self.a)
    self.psi_cp_re = [0j] * len(self.b)
    self.psi_cp_im = [0j] * len(self.b)


_PARAM_SPECS = {
    # model: (electric fields, magnetic fields, electric setter, electric lists)
    "Dummy": ((), (), None, ()),
    "Const": (("value",), ("value",), None, ()),
    "Dielectric": ((), (), None, ()),
    "Upml": (("c1", "c2", "c3", "c4", "c5", "c6", "d"),
             ("c1", "c2", "c3", "c4", "c5", "c6", "b"), None, ()),
    "Cpml": (("b1", "b2", "c1", "c2", "kappa1", "kappa2", "psi1", "psi2"),
             ("b1", "b2", "c1", "c2", "kappa1", "kappa2", "psi1", "psi2"), None, ()),
    "Drude": ((), (), _set_ac("Drude"), ("a", "c", "q_now", "q_new")),
    "Lorentz": ((), (), _set_ac("Lorentz"), ("a", "c", "l_now", "l_new")),
    "DcpAde": (("e_old",), (), _set_dcp_ade, ("a", "b", "c", "q_old", "q_now", "p_old", "p_now")),
    "DcpPlrc": ((), (), _set_dcp_plrc,
                ("a", "b", "c", "psi_dp_re", "psi_dp_im", "psi_cp_re", "psi_cp_im")),
}

_KINDS = {
    "Dummy": KIND_DUMMY, "Const": KIND_CONST, "Dielectric": KIND_DIELECTRIC, "Upml": KIND_UPML,
    "Cpml": KIND_CPML, "Drude": KIND_DRUDE, "Lorentz": KIND_LORENTZ, "DcpAde": KIND_DCP,
    "DcpPlrc": KIND_DCP_PLRC,
}
_DISPERSIVE = ("Drude", "Lorentz", "DcpAde", "DcpPlrc")
_COMPS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")

_g = globals()
for _sfx in ("Real", "Cmplx"):
    _g["ElectricParam" + _sfx] = _param("ElectricParam" + _sfx, "eps_inf")
    _g["MagneticParam" + _sfx] = _param("MagneticParam" + _sfx, "mu_inf")
    for _model, (_ef, _mf, _setter, _lists) in _PARAM_SPECS.items():
        _g[_model + "ElectricParam" + _sfx] = _param(_model + "ElectricParam" + _sfx, "eps_inf",
                                                     _ef, _setter, _lists)
        _g[_model + "MagneticParam" + _sfx] = _param(_model + "MagneticParam" + _sfx, "mu_inf",
                                                     _mf)


# ---------------------------------------------------------------------------
# Updaters
# ---------------------------------------------------------------------------
def _three(idx):
    try:
        t = tuple(int(v) for v in idx)
    except TypeError:
        raise ValueError("the field index must have exactly three values") from None
    if len(t) != 3:
        raise ValueError("the field index must have exactly three values")
    return t


class PwMaterial:
    """One reference updater object: a list of points with parameters."""

    model = "Dummy"
    comp = 0
    cmplx = False

    def __init__(self):
        self._idx = []
        self._param = []
        self._dev = None

    # -- reference interface --------------------------------------------
    def name(self):
        """The reference's updater tag (src/pw_*.hh ``tag``)."""
        if self.comp < 3:
            return self.model + "Electric"
        return ("Dcp" if self.model == "DcpAde" else self.model) + "Magnetic"

    def idx_size(self):
        return len(self._idx)

    def attach(self, idx, param):
        """Attach a copy of ``param`` at ``idx`` (the param is copied by value)."""
        idx = _three(idx)
        want = self._param_type()
        if not isinstance(param, want):
            raise TypeError(f"{type(self).__name__}.attach needs a {want.__name__}")
        self._sync_state()
        self._idx.append(idx)
        self._param.append(copy.deepcopy(param))
        self._dev = None
        return self

    def merge(self, other):
        if type(other) is not type(self):
            raise TypeError("merge needs an updater of the same type")
        self._sync_state()
        other._sync_state()
        self._idx.extend(other._idx)
        self._param.extend(copy.deepcopy(other._param))
        self._dev = None
        return self

    def _value_at(self, idx, field):
        idx = _three(idx)
        self._sync_state()
        for i, p in zip(self._idx, self._param):
            if i == idx:
                return getattr(p, field)
        return 0

    def update_all(self, inplace, in1, in2, d1, d2, dt, n):
        """Update every attached point of ``inplace`` (gmes/fdtd.py:673-809 binding)."""
        arrays = [self._check_array(a, i == 0) for i, a in enumerate((inplace, in1, in2))]
        shape = arrays[0][1]
        for idx in self._idx:
            for a in range(3):
                if not 0 <= idx[a] < shape[a]:
                    raise IndexError("field index is out of bounds")
        if not self._idx or self.model == "Dummy":
            return
        self._run(arrays, float(d1), float(d2), float(dt))

    # -- internals --------------------------------------------------------
    def _param_type(self):
        side = "Electric" if self.comp < 3 else "Magnetic"
        return _g[self.model + side + "Param" + ("Cmplx" if self.cmplx else "Real")]

    def _check_array(self, a, target):
        try:
            import torch
        except ImportError:  # pragma: no cover
            torch = None
        if torch is not None and isinstance(a, torch.Tensor):
            if self.cmplx or a.dtype != torch.float64 or not a.is_cuda or a.dim() != 3 or \
                    not a.is_contiguous():
                raise TypeError("tensors must be contiguous 3-D float64 CUDA tensors")
            return ("tensor", tuple(a.shape), a)
        if not isinstance(a, np.ndarray):
            raise TypeError("array must be a numpy.ndarray")
        want = np.complex128 if self.cmplx else np.float64
        if a.dtype != want:
            raise TypeError(f"array must have dtype {np.dtype(want).name}")
        if a.ndim != 3:
            raise TypeError("array must have 3 dimensions")
        if not a.flags.c_contiguous:
            raise TypeError("array must be contiguous")
        if target and not a.flags.writeable:
            raise TypeError("array must be writeable")
        return ("numpy", a.shape, a)

    def _layout(self):
        """(kind, npole, ncp, per-point params [planes][n][k], state [planes][n][s])."""
        m = self.model
        planes = 2 if self.cmplx else 1
        n = len(self._param)
        E = self.comp < 3
        if m in _DISPERSIVE and not E:
            m = "Dielectric"
        eps = [(p.eps_inf if E else p.mu_inf) for p in self._param]
        npole = ncp = 0
        if m == "Dielectric":
            par = [[[e] for e in eps]] * planes
            st = [[[] for _ in range(n)]] * planes
        elif m == "Const":
            vals = [complex(p.value) for p in self._param]
            par = [[[v.real] for v in vals], [[v.imag] for v in vals]][:planes]
            st = [[[] for _ in range(n)]] * planes
        elif m == "Cpml":
            par = [[[e, p.b1, p.b2, p.c1, p.c2, p.kappa1, p.kappa2]
                    for e, p in zip(eps, self._param)]] * planes
            psi = [(complex(p.psi1), complex(p.psi2)) for p in self._param]
            st = [[[a.real, b.real] for a, b in psi], [[a.imag, b.imag] for a, b in psi]][:planes]
        elif m == "Upml":
            par = [[[e, p.c1, p.c2, p.c3, p.c4, p.c5, p.c6] for e, p in zip(eps, self._param)]] \
                * planes
            s0 = [complex(p.d if E else p.b) for p in self._param]
            st = [[[v.real] for v in s0], [[v.imag] for v in s0]][:planes]
        else:
            npole = len(self._param[0].a)
            if m in ("DcpAde", "DcpPlrc"):
                ncp = len(self._param[0].b)
            for p in self._param:
                if len(p.a) != npole or (m in ("DcpAde", "DcpPlrc") and len(p.b) != ncp):
                    raise ValueError("all points of an updater must have the same number of poles")
            if npole > N.MAX_POLES or ncp > N.MAX_POLES:
                raise ValueError(f"at most {N.MAX_POLES} poles")
            par_rows, st_re, st_im = [], [], []
            for p in self._param:
                row = [v for r in p.a for v in r]
                if m in ("Drude", "Lorentz"):
                    row += list(p.c)
                    now, new = ("q_now", "q_new") if m == "Drude" else ("l_now", "l_new")
                    s = [complex(v) for v in getattr(p, now)] + [complex(v) for v in getattr(p, new)]
                elif m == "DcpAde":
                    row += [v for r in p.b for v in r] + list(p.c)
                    e_old = complex(getattr(p, "e_old", 0.0))
                    s = ([e_old] + [complex(v) for v in p.q_old] + [complex(v) for v in p.q_now]
                         + [complex(v) for v in p.p_old] + [complex(v) for v in p.p_now])
                else:  # DcpPlrc
                    for r in p.b:
                        for v in r:
                            row += [complex(v).real, complex(v).imag]
                    row += list(p.c)
                    s_re = [float(v) for v in p.psi_dp_re]
                    s_im = [float(v) for v in p.psi_dp_im]
                    for v in p.psi_cp_re:
                        s_re += [complex(v).real, complex(v).imag]
                    for v in p.psi_cp_im:
                        s_im += [complex(v).real, complex(v).imag]
                    par_rows.append(row)
                    st_re.append(s_re)
                    st_im.append(s_im)
                    continue
                par_rows.append(row)
                st_re.append([v.real for v in s])
                st_im.append([v.imag for v in s])
            par = [par_rows] * planes
            st = [st_re, st_im][:planes]
        return m, npole, ncp, par, st

    def _build(self):
        import torch
        m, npole, ncp, par, st = self._layout()
        dev = torch.device("cuda")
        n = len(self._idx)
        nparam = len(par[0][0]) if n and par[0][0] else 0
        nstate = len(st[0][0]) if n and st[0][0] else 0
        d = {
            "model": m, "npole": npole, "ncp": ncp, "nparam": nparam, "nstate": nstate,
            "idx": torch.tensor(self._idx, dtype=torch.int32, device=dev).reshape(-1),
            "param": torch.tensor(np.asarray(par, np.float64).reshape(-1), device=dev)
            if nparam else torch.zeros(1, dtype=torch.float64, device=dev),
            "state": torch.tensor(np.asarray(st, np.float64).reshape(-1), device=dev)
            if nstate else torch.zeros(1, dtype=torch.float64, device=dev),
        }
        self._dev = d
        return d

    def _sync_state(self):
        """Copy the device state back into the stored parameter copies."""
        d = self._dev
        if d is None or not d["nstate"]:
            return
        planes = 2 if self.cmplx else 1
        n = len(self._idx)
        s = d["state"].cpu().numpy().reshape(planes, n, d["nstate"])
        m, P, Q = d["model"], d["npole"], d["ncp"]
        E = self.comp < 3
        for t, p in enumerate(self._param):
            re = s[0, t]
            im = s[1, t] if planes == 2 else np.zeros_like(re)
            z = (re + 1j * im) if self.cmplx else re
            if m == "Cpml":
                p.psi1, p.psi2 = z[0], z[1]
            elif m == "Upml":
                if E:
                    p.d = z[0]
                else:
                    p.b = z[0]
            elif m in ("Drude", "Lorentz"):
                now, new = ("q_now", "q_new") if m == "Drude" else ("l_now", "l_new")
                setattr(p, now, list(z[:P]))
                setattr(p, new, list(z[P:2 * P]))
            elif m == "DcpAde":
                p.e_old = z[0]
                p.q_old, p.q_now = list(z[1:1 + P]), list(z[1 + P:1 + 2 * P])
                p.p_old = list(z[1 + 2 * P:1 + 2 * P + Q])
                p.p_now = list(z[1 + 2 * P + Q:1 + 2 * P + 2 * Q])
            elif m == "DcpPlrc":
                p.psi_dp_re = list(re[:P])
                p.psi_cp_re = [re[P + 2 * i] + 1j * re[P + 2 * i + 1] for i in range(Q)]
                if planes == 2:
                    p.psi_dp_im = list(im[:P])
                    p.psi_cp_im = [im[P + 2 * i] + 1j * im[P + 2 * i + 1] for i in range(Q)]

    def _run(self, arrays, d1, d2, dt):
        import torch
        from .engine import require_cuda
        require_cuda()
        lib = N.load()
        d = self._dev or self._build()
        dev = torch.device("cuda")
        bufs = []
        for kind, shape, a in arrays:
            if kind == "tensor":
                bufs.append(a)
            elif self.cmplx:
                bufs.append(torch.from_numpy(np.stack((a.real, a.imag))).to(dev))
            else:
                bufs.append(torch.from_numpy(a).to(dev))
        g = N.PointsC()
        g.comp = self.comp
        g.kind = _KINDS[d["model"]]
        g.npoints = len(self._idx)
        g.nparam = d["nparam"]
        g.nstate = d["nstate"]
        g.npole, g.ncp = d["npole"], d["ncp"]
        g.cmplx = 1 if self.cmplx else 0
        g.idx = d["idx"].data_ptr()
        g.param = d["param"].data_ptr()
        g.state = d["state"].data_ptr()
        for k, (_, shape, _) in enumerate(arrays):
            for a in range(3):
                g.shape[k][a] = int(shape[a])
        stream = torch.cuda.current_stream().cuda_stream
        N.check(lib.gmes_points_update(C.byref(g), C.c_void_p(bufs[0].data_ptr()),
                                       C.c_void_p(bufs[1].data_ptr()),
                                       C.c_void_p(bufs[2].data_ptr()), d1, d2, dt,
                                       C.c_void_p(stream)))
        kind, _, target = arrays[0]
        if kind == "numpy":
            out = bufs[0].cpu().numpy()
            if self.cmplx:
                target[...] = out[0] + 1j * out[1]
            else:
                target[...] = out


class MaterialElectric(PwMaterial):
    def get_eps_inf(self, idx):
        return self._value_at(idx, "eps_inf")


class MaterialMagnetic(PwMaterial):
    def get_mu_inf(self, idx):
        return self._value_at(idx, "mu_inf")


for _sfx, _cx in (("Real", False), ("Cmplx", True)):
    for _model in _PARAM_SPECS:
        for _c, _cn in enumerate(_COMPS):
            _base = MaterialElectric if _c < 3 else MaterialMagnetic
            _name = _model + _cn + _sfx
            _g[_name] = type(_name, (_base,), {"model": _model, "comp": _c, "cmplx": _cx})


def openmp_enabled():
    """The reference's OpenMP probe; the GPU engine has no OpenMP path."""
    return False


def openmp_max_threads():
    return 1


def openmp_cell_threshold():
    return 8192


__all__ = [n for n in list(_g) if n.endswith(("Real", "Cmplx"))] + [
    "PwMaterial", "PwMaterialParam", "MaterialElectric", "MaterialMagnetic",
    "openmp_enabled", "openmp_max_threads", "openmp_cell_threshold"]
