"""Field-component and direction tags, and physical constants.

Mirrors the interface of the reference's ``gmes.constant`` module
(src/constant.hh:11-47 for the constants, src/constant.i:48-218 for the
Python class tree).  Components and directions are *classes*, not
instances: user code compares them with ``is`` and ``issubclass`` and reads
their integer ``tag`` (src/constant.hh:52-259).  The tags are part of the
interface because the reference uses them as message tags.
"""

from math import atan, sqrt

pi = 4 * atan(1)
h = 6.6260695729e-34
hbar = h / (2 * pi)
c0 = 299792458.0
mu0 = 4 * pi * 1e-7
eps0 = 1 / (c0 * c0 * mu0)
Z0 = sqrt(mu0 / eps0)

YOTTA = 1e24
ZETTA = 1e21
EXA = 1e18
PETA = 1e15
TERA = 1e12
GIGA = 1e9
MEGA = 1e6
KILO = 1e3
MILLI = 1e-3
MICRO = 1e-6
NANO = 1e-9
PICO = 1e-12
FEMTO = 1e-15
ATTO = 1e-18
ZEPTO = 1e-21
YOCTO = 1e-24

inf = float("inf")


class Component:
    """Base of every field-component tag class."""

    tag = 0

    def __init__(self):
        raise RuntimeError("Component should be used as a class.")


def _named(name, base, tag, label, index=None, vector=None):
    attrs = {"tag": tag, "str": classmethod(lambda cls, _l=label: _l)}
    if index is not None:
        attrs["index"] = index
    if vector is not None:
        attrs["vector"] = vector
    return type(name, (base,), attrs)


class Electric(Component):
    tag = 1


class Magnetic(Component):
    tag = 2


class ElectricCurrent(Component):
    tag = 9


class MagneticCurrent(Component):
    tag = 13


# ``index`` is this package's own addition: the component number used by
# the engine's C ABI (Ex..Hz = 0..5).  Currents map to the field they drive.
Ex = _named("Ex", Electric, 3, "ex", 0)
Ey = _named("Ey", Electric, 4, "ey", 1)
Ez = _named("Ez", Electric, 5, "ez", 2)
Hx = _named("Hx", Magnetic, 6, "hx", 3)
Hy = _named("Hy", Magnetic, 7, "hy", 4)
Hz = _named("Hz", Magnetic, 8, "hz", 5)
Jx = _named("Jx", ElectricCurrent, 10, "jx", 0)
Jy = _named("Jy", ElectricCurrent, 11, "jy", 1)
Jz = _named("Jz", ElectricCurrent, 12, "jz", 2)
Mx = _named("Mx", MagneticCurrent, 14, "mx", 3)
My = _named("My", MagneticCurrent, 15, "my", 4)
Mz = _named("Mz", MagneticCurrent, 16, "mz", 5)


class Directional:
    """Base of every direction tag class."""

    tag = 17

    def __init__(self):
        raise RuntimeError("Directional should be used as a class.")


X = _named("X", Directional, 18, "x", 0)
Y = _named("Y", Directional, 19, "y", 1)
Z = _named("Z", Directional, 20, "z", 2)
PlusX = _named("PlusX", X, 21, "+x", 0, (1.0, 0.0, 0.0))
MinusX = _named("MinusX", X, 22, "-x", 0, (-1.0, 0.0, 0.0))
PlusY = _named("PlusY", Y, 23, "+y", 1, (0.0, 1.0, 0.0))
MinusY = _named("MinusY", Y, 24, "-y", 1, (0.0, -1.0, 0.0))
PlusZ = _named("PlusZ", Z, 25, "+z", 2, (0.0, 0.0, 1.0))
MinusZ = _named("MinusZ", Z, 26, "-z", 2, (0.0, 0.0, -1.0))

E_COMPONENTS = (Ex, Ey, Ez)
H_COMPONENTS = (Hx, Hy, Hz)
COMPONENTS = E_COMPONENTS + H_COMPONENTS

__all__ = [
    "pi", "h", "hbar", "c0", "mu0", "eps0", "Z0",
    "YOTTA", "ZETTA", "EXA", "PETA", "TERA", "GIGA", "MEGA", "KILO", "MILLI",
    "MICRO", "NANO", "PICO", "FEMTO", "ATTO", "ZEPTO", "YOCTO", "inf",
    "Component", "Electric", "Magnetic", "ElectricCurrent", "MagneticCurrent",
    "Ex", "Ey", "Ez", "Hx", "Hy", "Hz", "Jx", "Jy", "Jz", "Mx", "My", "Mz",
    "Directional", "X", "Y", "Z", "PlusX", "MinusX", "PlusY", "MinusY",
    "PlusZ", "MinusZ",
]
