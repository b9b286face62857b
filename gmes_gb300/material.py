"""Material models.

Interface mirror of the reference's ``gmes.material`` (src/material.pyx):
same class names, constructor arguments, defaults and ``init()``
coefficient formulas.  What differs is what a material hands to the engine:
instead of one C++ updater object per Yee point
(``get_pw_material_e?/h?``, src/material.pyx:39-133 and siblings), each
material describes one *class* per field component (``engine_class``):
a kind id plus the physical parameters.  ``FDTD.init`` numbers the distinct
classes, writes a u8 class map per component, and the CUDA engine computes
the update coefficients from those parameters in FP64 on the GPU.

The host-side ``init()`` coefficients (``a``, ``b``, ``c``, ``sigma_max``)
are kept because user code and the CPU oracle read them.
"""

from cmath import exp as cexp
from math import cos, exp, sin, sqrt, tanh

import numpy as np

from . import constant as const

# Update kinds understood by the CUDA engine (include/gmes_gb300.h).
KIND_DUMMY = 0
KIND_DIELECTRIC = 1
KIND_CPML = 2
KIND_UPML = 3
KIND_DRUDE = 4
KIND_LORENTZ = 5
KIND_DCP = 6
KIND_CONST = 7
KIND_DCP_PLRC = 8

KIND_NAMES = {
    KIND_DUMMY: "Dummy", KIND_DIELECTRIC: "Dielectric", KIND_CPML: "Cpml",
    KIND_UPML: "Upml", KIND_DRUDE: "Drude", KIND_LORENTZ: "Lorentz",
    KIND_DCP: "DcpAde", KIND_CONST: "Const", KIND_DCP_PLRC: "DcpPlrc",
}


class ClassDesc:
    """One update class of one field component.

    ``eps`` is eps_inf for an electric component and mu_inf for a magnetic
    one: the value the reference stores in the point's parameter struct
    (the underneath medium's value for a PML).  ``params`` holds the
    kind-specific physical parameters as a flat tuple of floats;
    ``pml`` is the PML material object for KIND_CPML / KIND_UPML.
    """

    __slots__ = ("kind", "eps", "params", "pml", "ndrude", "ncp")

    def __init__(self, kind, eps=1.0, params=(), pml=None, ndrude=0, ncp=0):
        self.kind = int(kind)
        self.eps = float(eps)
        self.params = tuple(float(p) for p in params)
        self.pml = pml
        self.ndrude = int(ndrude)
        self.ncp = int(ncp)

    def key(self):
        return (self.kind, self.eps, self.params, id(self.pml), self.ndrude, self.ncp)

    def __repr__(self):
        return f"ClassDesc({KIND_NAMES[self.kind]}, eps={self.eps}, params={self.params})"


_PW_COMPS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


class Material:
    """Base of the material types (src/pygeom.pyx:19-112).

    ``get_pw_material_e?/h?(idx, coords, underneath=None, cmplx=False)``
    return the reference's point-wise updater for one point (a
    ``gmes_gb300.pw_material`` object, run on the GPU), with the point's
    parameters filled as src/material.pyx does.
    """

    compound = False
    pw_model = None

    def __init__(self, eps_inf=1, mu_inf=1):
        self.eps_inf = float(eps_inf)
        self.mu_inf = float(mu_inf)

    def init(self, space, param=None):
        pass

    def display_info(self, indent=0):
        print(" " * indent, type(self).__name__, "eps_inf:", self.eps_inf,
              "mu_inf:", self.mu_inf)

    def _own(self, comp, underneath):
        src = self if underneath is None else underneath
        return src.eps_inf if comp.index < 3 else src.mu_inf

    def engine_class(self, comp, underneath=None):
        raise NotImplementedError(f"{type(self).__name__} is not supported by the GPU engine")

    # -- point-wise updaters (src/material.pyx get_pw_material_*) -----------
    def _pw(self, c, idx, coords, underneath, cmplx):
        from . import pw_material as pm
        if self.pw_model is None:
            raise NotImplementedError(f"{type(self).__name__} has no point-wise updater")
        sfx = "Cmplx" if cmplx else "Real"
        upd = getattr(pm, self.pw_model + _PW_COMPS[c] + sfx)()
        param = getattr(pm, self.pw_model + ("Electric" if c < 3 else "Magnetic") + "Param"
                        + sfx)()
        src = self if underneath is None else underneath
        if c < 3:
            param.eps_inf = src.eps_inf
        else:
            param.mu_inf = src.mu_inf
        self._fill_pw(param, c, coords)
        upd.attach(idx, param)
        return upd

    def _fill_pw(self, param, c, coords):
        pass

    def get_pw_material_ex(self, idx, coords, underneath=None, cmplx=False):
        return self._pw(0, idx, coords, underneath, cmplx)

    def get_pw_material_ey(self, idx, coords, underneath=None, cmplx=False):
        return self._pw(1, idx, coords, underneath, cmplx)

    def get_pw_material_ez(self, idx, coords, underneath=None, cmplx=False):
        return self._pw(2, idx, coords, underneath, cmplx)

    def get_pw_material_hx(self, idx, coords, underneath=None, cmplx=False):
        return self._pw(3, idx, coords, underneath, cmplx)

    def get_pw_material_hy(self, idx, coords, underneath=None, cmplx=False):
        return self._pw(4, idx, coords, underneath, cmplx)

    def get_pw_material_hz(self, idx, coords, underneath=None, cmplx=False):
        return self._pw(5, idx, coords, underneath, cmplx)


class Dummy(Material):
    """No update: the point is only refreshed by the ghost-plane copy (src/pw_dummy.hh)."""

    pw_model = "Dummy"

    def engine_class(self, comp, underneath=None):
        return ClassDesc(KIND_DUMMY, self._own(comp, underneath))


class Const(Material):
    """Writes a constant value at every step (src/pw_const.hh)."""

    pw_model = "Const"

    def __init__(self, value=0, eps_inf=1, mu_inf=1):
        super().__init__(eps_inf, mu_inf)
        self.value = complex(value) if isinstance(value, complex) else float(value)

    def engine_class(self, comp, underneath=None):
        if isinstance(self.value, complex):
            # the imaginary part is written on the imaginary plane of complex grids
            return ClassDesc(KIND_CONST, self._own(comp, underneath),
                             (self.value.real, self.value.imag))
        return ClassDesc(KIND_CONST, self._own(comp, underneath), (self.value,))

    def _fill_pw(self, param, c, coords):
        param.value = self.value


class Dielectric(Material):
    """Non-dispersive isotropic medium (src/material.pyx:281-420, src/pw_dielectric.hh)."""

    pw_model = "Dielectric"

    def engine_class(self, comp, underneath=None):
        return ClassDesc(KIND_DIELECTRIC, self._own(comp, underneath))


class Pml(Material):
    """Base of the absorbing layers (src/material.pyx:423-502).

    A PML is a ``Compound`` material: the eps_inf/mu_inf of its update come
    from the medium underneath it.
    """

    compound = True

    def __init__(self, eps_inf, mu_inf):
        super().__init__(eps_inf, mu_inf)
        self.initialized = False

    def init(self, space, param=None):
        if param is None:
            raise ValueError("a PML material must be placed with a Shell")
        self.center = np.array(param[0], np.double)
        self.half_size = np.array(param[1], np.double)
        self.d = param[2]
        for i in range(3):
            if self.half_size[i] < self.d:
                self.half_size[i] = np.inf
        self.dt = space.dt
        self.dw = np.array(space.dr, np.double)
        self.sigma_max = self.sigma_max_ratio * self.get_sigma_opt()
        self.initialized = True

    def get_sigma_opt(self):
        eta = sqrt(self.mu_inf / self.eps_inf)
        return 0.8 * (self.m + 1) / (eta * self.dw)

    def _depth(self, w, component):
        """Normalised depth into the slab, or None outside it (src/material.pyx:474-502)."""
        w -= self.center[component]
        half_size = self.half_size[component]
        if w <= self.d - half_size:
            return min(max((half_size + w) / self.d, 0), 1)
        if half_size - self.d <= w:
            return min(max((half_size - w) / self.d, 0), 1)
        return None

    def sigma(self, w, component):
        depth = self._depth(w, component)
        if depth is None:
            return 0
        return self.sigma_max[component] * (1 - depth) ** self.m

    def kappa(self, w, component):
        depth = self._depth(w, component)
        if depth is None:
            return 1
        return 1 + (self.kappa_max - 1) * (1 - depth) ** self.m

    def pml_params(self):
        """Parameters of the on-GPU profile builder (``gmes_pml_desc``)."""
        raise NotImplementedError


class Upml(Pml):
    """Uniaxial PML (src/material.pyx:505-729, src/pw_upml.hh)."""

    def __init__(self, eps_inf=1, mu_inf=1, m=3.6, kappa_max=4.6, sigma_max_ratio=.745):
        super().__init__(eps_inf, mu_inf)
        self.m = float(m)
        self.kappa_max = float(kappa_max)
        self.sigma_max_ratio = float(sigma_max_ratio)

    def _sk(self, w, component):
        return self.sigma(w, component), self.kappa(w, component)

    def c1(self, w, component):
        s, k = self._sk(w, component)
        return (2 * k - s * self.dt) / (2 * k + s * self.dt)

    def c2(self, w, component):
        s, k = self._sk(w, component)
        return 2 * self.dt / (2 * k + s * self.dt)

    c3 = c1

    def c4(self, w, component):
        s, k = self._sk(w, component)
        return 1 / (2 * k + s * self.dt)

    def c5(self, w, component):
        s, k = self._sk(w, component)
        return 2 * k + s * self.dt

    def c6(self, w, component):
        s, k = self._sk(w, component)
        return 2 * k - s * self.dt

    pw_model = "Upml"

    def _fill_pw(self, param, c, coords):
        own, a1, a2 = c % 3, (c % 3 + 1) % 3, (c % 3 + 2) % 3
        param.c1 = self.c1(coords[a1], a1)
        param.c2 = self.c2(coords[a1], a1)
        param.c3 = self.c3(coords[a2], a2)
        param.c4 = self.c4(coords[a2], a2)
        param.c5 = self.c5(coords[own], own)
        param.c6 = self.c6(coords[own], own)

    def engine_class(self, comp, underneath=None):
        return ClassDesc(KIND_UPML, self._own(comp, underneath), pml=self)


class Cpml(Pml):
    """Complex-frequency-shifted PML (src/material.pyx:732-954, src/pw_cpml.hh)."""

    def __init__(self, eps_inf=1, mu_inf=1, m=3.4, kappa_max=1, m_a=4.8, a_max=0.8,
                 sigma_max_ratio=0.65):
        super().__init__(eps_inf, mu_inf)
        self.m = float(m)
        self.kappa_max = float(kappa_max)
        self.m_a = float(m_a)
        self.a_max = float(a_max)
        self.sigma_max_ratio = float(sigma_max_ratio)

    def a(self, w, component):
        depth = self._depth(w, component)
        if depth is None:
            return 0
        return self.a_max * depth ** self.m_a

    def b(self, w, component):
        exponent = -(self.sigma(w, component) / self.kappa(w, component)
                     + self.a(w, component)) * self.dt
        return exp(exponent)

    def c(self, w, component):
        sigma = self.sigma(w, component)
        kappa = self.kappa(w, component)
        numerator = sigma * (self.b(w, component) - 1)
        denominator = (sigma + kappa * self.a(w, component)) * kappa
        return numerator / denominator if denominator else 0

    pw_model = "Cpml"

    def _fill_pw(self, param, c, coords):
        a1, a2 = (c % 3 + 1) % 3, (c % 3 + 2) % 3
        param.b1 = self.b(coords[a1], a1)
        param.b2 = self.b(coords[a2], a2)
        param.c1 = self.c(coords[a1], a1)
        param.c2 = self.c(coords[a2], a2)
        param.kappa1 = self.kappa(coords[a1], a1)
        param.kappa2 = self.kappa(coords[a2], a2)

    def engine_class(self, comp, underneath=None):
        return ClassDesc(KIND_CPML, self._own(comp, underneath), pml=self)


class DrudePole:
    def __init__(self, omega, gamma):
        self.omega = float(omega)
        self.gamma = float(gamma)


class LorentzPole:
    def __init__(self, amp, omega, gamma):
        self.amp = float(amp)
        self.omega = float(omega)
        self.gamma = float(gamma)


class CriticalPoint:
    def __init__(self, amp, phi, omega, gamma):
        self.amp = float(amp)
        self.phi = float(phi)
        self.omega = float(omega)
        self.gamma = float(gamma)


class Drude(Dielectric):
    """Drude ADE medium (src/material.pyx:1500-1660, src/pw_drude.hh)."""

    pw_model = "Drude"

    def _fill_pw(self, param, c, coords):
        if c < 3:
            param.set(self.a, self.c)

    def __init__(self, eps_inf=1, mu_inf=1, sigma=0, dps=()):
        super().__init__(eps_inf, mu_inf)
        self.sigma = float(sigma)
        self.dps = tuple(dps)
        self.initialized = False

    def init(self, space, param=None):
        self.dt = space.dt
        self.a = np.empty((len(self.dps), 3), np.double)
        for i, pole in enumerate(self.dps):
            denom = self.dt * pole.gamma + 2.
            self.a[i, 0] = (self.dt * pole.gamma - 2) / denom
            self.a[i, 1] = 4 / denom
            self.a[i, 2] = 2 * (self.dt * pole.omega) ** 2 / denom
        self.c = np.empty(3, np.double)
        denom = 2. * self.eps_inf + self.dt * self.sigma
        self.c[0] = 2 * self.dt / denom
        self.c[1] = -2 / denom
        self.c[2] = (2 * self.eps_inf - self.dt * self.sigma) / denom
        self.initialized = True

    def engine_class(self, comp, underneath=None):
        if comp.index >= 3:
            return ClassDesc(KIND_DIELECTRIC, self._own(comp, underneath))
        params = [self.eps_inf, self.sigma]
        for p in self.dps:
            params += [p.omega, p.gamma]
        return ClassDesc(KIND_DRUDE, self._own(comp, underneath), params,
                         ndrude=len(self.dps))


class Lorentz(Dielectric):
    """Lorentz ADE medium (src/material.pyx:1663-1858, src/pw_lorentz.hh)."""

    pw_model = "Lorentz"

    def _fill_pw(self, param, c, coords):
        if c < 3:
            param.set(self.a, self.c)

    def __init__(self, eps_inf=1, mu_inf=1, sigma=0, lps=()):
        super().__init__(eps_inf, mu_inf)
        self.sigma = float(sigma)
        self.lps = tuple(lps)
        self.initialized = False

    def init(self, space, param=None):
        self.dt = space.dt
        self.a = np.empty((len(self.lps), 3), np.double)
        for i, pole in enumerate(self.lps):
            denom = self.dt * pole.gamma + 2.
            self.a[i, 0] = (self.dt * pole.gamma - 2) / denom
            self.a[i, 1] = (4 - 2 * (self.dt * pole.omega) ** 2) / denom
            self.a[i, 2] = 2 * pole.amp * (self.dt * pole.omega) ** 2 / denom
        self.c = np.empty(3, np.double)
        denom = 2. * self.eps_inf + self.dt * self.sigma
        self.c[0] = 2 * self.dt / denom
        self.c[1] = -2 / denom
        self.c[2] = (2 * self.eps_inf - self.dt * self.sigma) / denom
        self.initialized = True

    def engine_class(self, comp, underneath=None):
        if comp.index >= 3:
            return ClassDesc(KIND_DIELECTRIC, self._own(comp, underneath))
        params = [self.eps_inf, self.sigma]
        for p in self.lps:
            params += [p.amp, p.omega, p.gamma]
        return ClassDesc(KIND_LORENTZ, self._own(comp, underneath), params,
                         ndrude=len(self.lps))


class DcpAde(Dielectric):
    """Drude-critical-points medium, ADE form (src/material.pyx:1029-1176, src/pw_dcp.hh:44-400)."""

    pw_model = "DcpAde"

    def _fill_pw(self, param, c, coords):
        if c < 3:
            param.set(self.a, self.b, self.c)

    def __init__(self, eps_inf=1, mu_inf=1, sigma=0, dps=(), cps=()):
        super().__init__(eps_inf, mu_inf)
        self.sigma = float(sigma)
        self.dps = tuple(dps)
        self.cps = tuple(cps)
        self.initialized = False

    def init(self, space, param=None):
        dt = self.dt = space.dt
        self.a = np.empty((len(self.dps), 3), np.double)
        for i, pole in enumerate(self.dps):
            denom = float(dt * pole.gamma + 2)
            self.a[i, 0] = (dt * pole.gamma - 2) / denom
            self.a[i, 1] = 4 / denom
            self.a[i, 2] = 0.5 * (dt * pole.omega) ** 2 / denom
        self.b = np.empty((len(self.cps), 5), np.double)
        for i, p in enumerate(self.cps):
            denom = (dt * p.gamma + 2) ** 2 + (dt * p.omega) ** 2
            self.b[i, 0] = -((dt * p.gamma - 2) ** 2 + (dt * p.omega) ** 2) / denom
            self.b[i, 1] = 2 * (4 - dt ** 2 * (p.gamma ** 2 + p.omega ** 2)) / denom
            self.b[i, 2] = 2 * dt * p.amp * p.omega * (
                dt * cos(p.phi) * p.omega + sin(p.phi) * (2 - dt * p.gamma)) / denom
            self.b[i, 3] = 4 * dt ** 2 * p.amp * p.omega * (
                cos(p.phi) * p.omega - sin(p.phi) * p.gamma) / denom
            self.b[i, 4] = 2 * dt * p.amp * p.omega * (
                dt * cos(p.phi) * p.omega - sin(p.phi) * (2 + dt * p.gamma)) / denom
        self.c = np.empty(4, np.double)
        denom = 0.5 * dt * self.sigma + sum(self.a[:, 2]) + sum(self.b[:, 4]) + self.eps_inf
        self.c[0] = dt / denom
        self.c[1] = 1 / denom
        self.c[2] = -(sum(self.a[:, 2]) + sum(self.b[:, 2])) / denom
        self.c[3] = -(0.5 * dt * self.sigma + 2 * sum(self.a[:, 2]) + sum(self.b[:, 3])
                      - self.eps_inf) / denom
        self.initialized = True

    def engine_class(self, comp, underneath=None):
        if comp.index >= 3:
            return ClassDesc(KIND_DIELECTRIC, self._own(comp, underneath))
        params = [self.eps_inf, self.sigma]
        for p in self.dps:
            params += [p.omega, p.gamma]
        # cos/sin of the phase are taken on the host (libm, as
        # src/material.pyx:1090-1093 does) so the GPU coefficient arithmetic
        # is pure IEEE +,-,*,/
        for p in self.cps:
            params += [p.amp, cos(p.phi), sin(p.phi), p.omega, p.gamma]
        return ClassDesc(KIND_DCP, self._own(comp, underneath), params,
                         ndrude=len(self.dps), ncp=len(self.cps))


class _Unsupported(Dielectric):
    reason = "not supported by the GPU engine"

    def __init__(self, *args, **kwargs):
        eps_inf = kwargs.get("eps_inf", args[0] if args else 1)
        mu_inf = kwargs.get("mu_inf", args[1] if len(args) > 1 else 1)
        super().__init__(eps_inf, mu_inf)

    def engine_class(self, comp, underneath=None):
        raise NotImplementedError(f"{type(self).__name__}: {self.reason}")


class DcpPlrc(Dielectric):
    """Drude-critical-points medium, piecewise-linear recursive convolution
    (src/material.pyx:1227-1471, src/pw_dcp.hh:406-746).

    ``init()`` keeps the reference's host coefficients a, b, c; the engine
    recomputes them in FP64 on the GPU from the physical parameters and the
    transcendental values taken here with the host libm.
    """

    pw_model = "DcpPlrc"

    def _fill_pw(self, param, c, coords):
        if c < 3:
            param.set(self.a, self.b, self.c)

    rc = False

    def __init__(self, eps_inf=1, mu_inf=1, sigma=0, dps=(), cps=()):
        super().__init__(eps_inf, mu_inf)
        self.sigma = float(sigma)
        self.dps = tuple(dps)
        self.cps = tuple(cps)
        self.initialized = False

    def init(self, space, param=None):
        self.dt = space.dt
        self.a = np.empty((len(self.dps), 3), np.double)
        for i, pole in enumerate(self.dps):
            self.a[i, 0] = self.delta_chi_dp_0(pole) - self.delta_xi_dp_0(pole)
            self.a[i, 1] = self.delta_xi_dp_0(pole)
            self.a[i, 2] = exp(-pole.gamma * self.dt)
        self.b = np.empty((len(self.cps), 3), complex)
        for i, pnt in enumerate(self.cps):
            self.b[i, 0] = self.delta_chi_cp_0(pnt) - self.delta_xi_cp_0(pnt)
            self.b[i, 1] = self.delta_xi_cp_0(pnt)
            self.b[i, 2] = cexp(-self.dt * (pnt.gamma + 1j * pnt.omega))
        chi_0 = (sum([self.chi_dp_0(p) for p in self.dps] +
                     [self.chi_cp_0(p) for p in self.cps]) + 0j).real
        xi_0 = (sum([self.xi_dp_0(p) for p in self.dps] +
                    [self.xi_cp_0(p) for p in self.cps]) + 0j).real
        self.c = np.empty(3, np.double)
        conductivity = 0.5 * self.dt * self.sigma
        denom = self.eps_inf - xi_0 + chi_0 + conductivity
        self.c[0] = self.dt / denom
        self.c[1] = (self.eps_inf - xi_0 - conductivity) / denom
        self.c[2] = 1 / denom
        self.initialized = True

    # the susceptibility terms of src/material.pyx:1313-1356
    def chi_dp_0(self, dp):
        gdt = dp.gamma * self.dt
        return (dp.omega / dp.gamma) ** 2 * (exp(-gdt) + gdt - 1)

    def xi_dp_0(self, dp):
        gdt = dp.gamma * self.dt
        return (self.chi_dp_0(dp) * (1 / (1 - exp(gdt)) + 1 / gdt)
                + (dp.omega / dp.gamma) ** 2 * (gdt / 2 / tanh(gdt / 2) - 1))

    def delta_chi_dp_0(self, dp):
        gdt = dp.gamma * self.dt
        return -(dp.omega / dp.gamma * (1 - exp(-gdt))) ** 2

    def delta_xi_dp_0(self, dp):
        gdt = dp.gamma * self.dt
        return self.delta_chi_dp_0(dp) * (1 / (1 - exp(gdt)) + 1 / gdt)

    def chi_cp_0(self, cp):
        go = cp.gamma + 1j * cp.omega
        return 2j * cp.amp * cp.omega * cexp(1j * cp.phi) * (1 - cexp(-self.dt * go)) / go

    def xi_cp_0(self, cp):
        dtgo = self.dt * (cp.gamma + 1j * cp.omega)
        return self.chi_cp_0(cp) * (1 / (1 - cexp(dtgo)) + 1 / dtgo)

    def delta_chi_cp_0(self, cp):
        go = cp.gamma + 1j * cp.omega
        return 2j * cp.amp * cp.omega * cexp(1j * cp.phi) * (1 - cexp(-self.dt * go)) ** 2 / go

    def delta_xi_cp_0(self, cp):
        dtgo = self.dt * (cp.gamma + 1j * cp.omega)
        return self.delta_chi_cp_0(cp) * (1 / (1 - cexp(dtgo)) + 1 / dtgo)

    def engine_class(self, comp, underneath=None):
        if comp.index >= 3:
            return ClassDesc(KIND_DIELECTRIC, self._own(comp, underneath))
        dt = self.dt
        params = [self.eps_inf, self.sigma, 1.0 if self.rc else 0.0]
        for p in self.dps:
            gdt = p.gamma * dt
            params += [p.omega, p.gamma, exp(-gdt), exp(gdt), tanh(gdt / 2)]
        for p in self.cps:
            go = p.gamma + 1j * p.omega
            ph = cexp(1j * p.phi)
            q = cexp(-dt * go)
            r = cexp(dt * go)
            params += [p.amp, p.omega, p.gamma, ph.real, ph.imag, q.real, q.imag,
                       r.real, r.imag]
        return ClassDesc(KIND_DCP_PLRC, self._own(comp, underneath), params,
                         ndrude=len(self.dps), ncp=len(self.cps))


class DcpRc(DcpPlrc):
    """Drude-critical-points medium, recursive convolution (src/material.pyx:1474-1490):
    the PLRC updater with the xi terms set to zero."""

    rc = True

    def xi_dp_0(self, dp):
        return 0

    def xi_cp_0(self, cp):
        return 0j

    def delta_xi_dp_0(self, dp):
        return 0

    def delta_xi_cp_0(self, cp):
        return 0j


class Dm2(_Unsupported):
    reason = "the two-level density-matrix medium is not implemented"


__all__ = [
    "Material", "Dummy", "Const", "Dielectric", "Pml", "Upml", "Cpml",
    "DrudePole", "LorentzPole", "CriticalPoint", "Drude", "Lorentz", "DcpAde",
    "DcpPlrc", "DcpRc", "Dm2",
]
