"""Sources.

Interface mirror of the reference's ``gmes.source`` (gmes/source.py:44-368):
the source-time functions are evaluated on the host in FP64, one scalar
per half-step (as gmes/pw_source.py:74-87 does per point), and the engine
applies the values on the GPU after the material update of the component.
"""

from cmath import exp as cexp
from math import exp, pi, sin

import numpy as np

from . import constant as const
from .geometry import in_range


class SrcTime:
    """Time-dependent part of a source."""

    cmplx = False

    def init(self, cmplx):
        self.cmplx = bool(cmplx)

    def oscillator(self, time):
        raise NotImplementedError

    def display_info(self, indent=0):
        print(" " * indent, type(self).__name__)


class Continuous(SrcTime):
    """CW source with a Hann-window turn-on and turn-off (gmes/source.py:87-135)."""

    def __init__(self, freq, phase=0, start=0, end=np.inf, width=None):
        self.freq = float(freq)
        self.phase = float(phase)
        self.start = float(start)
        self.end = float(end)
        self.width = 5 / self.freq if width is None else float(width)

    def oscillator(self, time):
        ts = time - self.start
        te = self.end - time
        if ts < 0 or te < 0:
            return 0
        rise = sin(0.5 * pi * ts / self.width) ** 2 if ts < self.width else 1
        fall = sin(0.5 * pi * te / self.width) ** 2 if te < self.width else 1
        env = rise * fall
        osc = env * cexp(2j * pi * self.freq * time + 1j * self.phase)
        return osc if self.cmplx else osc.real


class Bandpass(SrcTime):
    """Gaussian-envelope pulse (gmes/source.py:138-182).

    ``Bandpass(freq, fwidth)`` is the reference's Gaussian pulse source:
    width 1/fwidth, peak at s*width, cutoff at 2*s*width.
    """

    def __init__(self, freq, fwidth, s=10, phase=0):
        self.freq = float(freq)
        self.phase = float(phase)
        self.fwidth = float(fwidth)
        self.width = 1 / self.fwidth
        self.peak_time = self.width * s
        self.cutoff = 2 * self.width * s
        while exp(-0.5 * (self.cutoff / self.width) ** 2) == 0:
            self.cutoff *= 0.9

    def oscillator(self, time):
        tt = time - self.peak_time
        if abs(tt) > self.cutoff:
            return 0
        cfactor = 1.0 / (-2j * pi * self.freq)
        osc = (cfactor * exp(-0.5 * (tt / self.width) ** 2)
               * cexp(2j * pi * self.freq * time + 1j * self.phase))
        return osc if self.cmplx else osc.real


class DifferentiatedGaussian(SrcTime):
    """-2((t-t0)/tw) exp(-((t-t0)/tw)^2) (gmes/source.py:185-213)."""

    def __init__(self, tw, t0):
        self.tw = float(tw)
        self.t0 = float(t0)

    def oscillator(self, time):
        exponent = -(((time - self.t0) / self.tw) ** 2)
        osc = -2 * (time - self.t0) / self.tw * cexp(exponent)
        return osc if self.cmplx else osc.real


class Src:
    """Space-dependent part of a source."""

    def init(self, geom_tree, space, cmplx):
        raise NotImplementedError

    def step(self):
        pass

    def display_info(self, indent=0):
        print(" " * indent, type(self).__name__)


class PointSourceSpec:
    """A point source resolved to one Yee point of one component.

    ``mode`` 0 = hard source (field := amp * f(t)), 1 = current source
    (field -= dt * amp * f(t) / eps_or_mu), gmes/pw_source.py:74-131.
    """

    __slots__ = ("comp", "idx", "mode", "amp", "eps", "src_time")

    def __init__(self, comp, idx, mode, amp, eps, src_time):
        self.comp = comp
        self.idx = tuple(int(v) for v in idx)
        self.mode = int(mode)
        self.amp = float(amp)
        self.eps = float(eps)
        self.src_time = src_time

    def value(self, dt, n):
        """The scalar the engine applies at half-step ``n`` (time dt * n)."""
        src_t = self.amp * self.src_time.oscillator(dt * n)
        if self.mode == 0:
            return src_t
        return dt * src_t / self.eps


class PointSource(Src):
    """Point source at the Yee point nearest ``center`` (gmes/source.py:216-368)."""

    def __init__(self, src_time, center, component, amp=1, filename=None):
        self.center = np.array(center, np.double)
        self.comp = component
        self.src_time = src_time
        self.amp = float(amp)
        self.filename = str(filename) if filename else None

    def init(self, geom_tree, space, cmplx):
        self.geom_tree = geom_tree
        self.src_time.init(cmplx)

    def display_info(self, indent=0):
        print(" " * indent, "point source:", "center:", self.center,
              "component:", self.comp.str(), "amp:", self.amp)

    def resolve(self, comp, shape, space, geom_tree):
        """``PointSourceSpec`` for field component ``comp`` or None."""
        field_of = {const.Ex: const.Ex, const.Jx: const.Ex, const.Ey: const.Ey,
                    const.Jy: const.Ey, const.Ez: const.Ez, const.Jz: const.Ez,
                    const.Hx: const.Hx, const.Mx: const.Hx, const.Hy: const.Hy,
                    const.My: const.Hy, const.Hz: const.Hz, const.Mz: const.Hz}
        if field_of.get(self.comp) is not comp:
            return None
        idx = space.space_to_index(comp, *self.center)
        if not in_range(idx, shape, comp):
            return None
        coords = space.index_to_space(comp, *idx)
        mat, _under = geom_tree.material_of_point(coords)
        current = issubclass(self.comp, (const.ElectricCurrent, const.MagneticCurrent))
        eps = mat.eps_inf if comp.index < 3 else mat.mu_inf
        return PointSourceSpec(comp, idx, 1 if current else 0, self.amp, eps, self.src_time)


class TotalFieldScatteredField(Src):
    """Plane wave launched through the faces of a box (gmes/source.py:370-1522).

    ``center``, ``size``: the total-field box; ``direction``: propagation
    direction; ``polarization``: E-field direction; ``amp``: amplitude.  The
    incident wave is carried by a 1-D TEMz grid with a cell size matched to
    the numerical dispersion (``gmes_gb300.tfsf``), stepped on the GPU
    between the E and H halves of every step.
    """

    def __init__(self, src_time, center, size, direction, polarization, amp=1):
        if not isinstance(src_time, SrcTime):
            raise TypeError("src_time must be an instance of SrcTime.")
        self.src_time = src_time
        self.k = np.array(direction, np.double) / np.linalg.norm(direction)
        self.center = np.array(center, np.double)
        if not np.isfinite(self.center).all():
            raise ValueError("center must contain only finite values")
        self.size = np.array(size, np.double)
        if not np.isfinite(self.size).all():
            raise ValueError("size must contain only finite values")
        self.half_size = 0.5 * self.size
        self.e_direction = np.array(polarization, np.double) / np.linalg.norm(polarization)
        self.h_direction = np.cross(self.k, self.e_direction)
        self.amp = float(amp)
        self.aux_fdtd = None

    def init(self, geom_tree, space, cmplx):
        from .tfsf import incident_grid
        self.geom_tree = geom_tree
        self.src_time.init(cmplx)
        self.aux_fdtd = incident_grid(self, space, geom_tree, cmplx)

    def display_info(self, indent=0):
        print(" " * indent, "plane-wave source:")
        print(" " * indent, "propagation direction:", self.k)
        print(" " * indent, "center:", self.center)
        print(" " * indent, "source plane size:", self.size)
        print(" " * indent, "polarization direction:", self.e_direction)
        print(" " * indent, "amplitude:", self.amp)
        self.src_time.display_info(4)

    def mode_function(self, x, y, z):
        return 1.0


class GaussianBeam(Src):
    def __init__(self, *args, **kwargs):
        raise NotImplementedError("GaussianBeam is not implemented")


__all__ = [
    "SrcTime", "Continuous", "Bandpass", "DifferentiatedGaussian", "Src",
    "PointSource", "TotalFieldScatteredField", "GaussianBeam",
]
