"""gmes_gb300: a GB300-native FDTD time-stepping engine with GMES's Python API.

``from gmes_gb300 import *`` gives the same names as ``from gmes import *``
(gmes/__init__.py): Cartesian, the geometry primitives, the material
models, the sources, the component/direction tags and the FDTD classes.
The time stepping runs in hand-written CUDA kernels for sm_103a
(libgmes_gb300.so, C ABI in include/gmes_gb300.h); the host side is Python.
"""

from . import constant
from .constant import *
from .geometry import (AuxiCartComm, Block, Cartesian, Cone, Cylinder, DefaultMedium,
                       Ellipsoid, GeomBox, GeomBoxTree, Shell, Sphere, in_range)
from .material import (Const, CriticalPoint, DcpAde, DcpPlrc, DcpRc, Dielectric, Dm2,
                       Drude, DrudePole, Dummy, Lorentz, LorentzPole, Material, Cpml, Upml)
from .source import (Bandpass, Continuous, DifferentiatedGaussian, GaussianBeam, PointSource,
                     TotalFieldScatteredField)
from .fdtd import (FDTD, TEMxFDTD, TEMyFDTD, TEMzFDTD, TExFDTD, TEyFDTD, TEzFDTD, TimeStep,
                   TMxFDTD, TMyFDTD, TMzFDTD)

__version__ = "0.1.0"
