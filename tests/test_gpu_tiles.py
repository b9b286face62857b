"""The cell kernels' warp-uniform plain path against their per-point path.

A warp of a half-step kernel whose points all carry the same dielectric
class per component skips the per-point kind look-ups and branches.  Its
arithmetic is the per-point path's, term for term, so the fields must be
bit-identical with GMES_FLAG_POINTWISE set (every warp per point).  Scenes:
3-D dielectric objects in a CPML shell (kappa = 1 and kappa > 1), the
dispersive scene (Drude, Lorentz, DCP in a UPML shell, TFSF), two TMz
scenes and a complex Bloch scene, in every precision the scene supports.
"""
import numpy as np
import pytest

import gmes_gb300 as G
from gmes_gb300 import _native as N
from gmes_gb300 import workloads as W
from cases import CASES

pytestmark = pytest.mark.gpu

PULSE = G.Bandpass(freq=1.0, fwidth=1.0)


def _at(sim, precision):
    sim.precision = precision
    return sim


SCENES = {
    "cube45": lambda p: W.cube(n=45, nobj=6, pml_cells=5, precision=p, src_time=PULSE)[0],
    "cube45_kappa4": lambda p: W.cube(n=45, nobj=6, pml_cells=5, precision=p, src_time=PULSE,
                                      kappa_max=4.0)[0],
    "disp40": lambda p: W.dispersive(n=40, pml_cells=6, precision=p, res=10,
                                     src_time=PULSE)[0],
    "drude2d": lambda p: _at(CASES["drude2d"](G)[0], p),
    "air2d": lambda p: W.air2d(precision=p)[0],
    "bloch48": lambda p: _bloch48(p),
}
CASES_RUN = [("cube45", "fp64"), ("cube45", "fp32"), ("cube45", "df64"),
             ("cube45_kappa4", "fp64"), ("cube45_kappa4", "fp32"), ("cube45_kappa4", "df64"),
             ("disp40", "fp64"), ("disp40", "fp32"),
             ("disp40", "df64"), ("drude2d", "fp64"), ("air2d", "fp64"), ("air2d", "fp32"),
             ("bloch48", "fp64")]


def _bloch48(precision):
    """Complex fields with a Bloch vector (as the bloch3d golden scene) on a
    48^3 grid, so that whole 16-cell rows lie inside the PML-free interior."""
    space = G.Cartesian(size=(4.8, 4.8, 4.8), resolution=10)
    geometry = [G.DefaultMedium(material=G.Dielectric()),
                G.Sphere(material=G.Drude(eps_inf=1, dps=(G.DrudePole(omega=3.0, gamma=0.3),)),
                         center=(0.2, 0.1, 0), radius=0.9),
                G.Block(material=G.Dielectric(eps_inf=2.5), center=(-1.0, 0, 0.6),
                        size=(0.9, 2.4, 0.9)),
                G.Shell(material=G.Cpml(), thickness=0.3)]
    sources = [G.PointSource(src_time=G.Bandpass(freq=1.0, fwidth=1.0, s=3), center=(0, 0, 0),
                             component=G.Ex)]
    return G.FDTD(space, geometry, sources, bloch=(0.4, 0.2, 0.1), verbose=False,
                  precision=precision)


@pytest.mark.parametrize("name,precision", CASES_RUN)
def test_uniform_warps_bit_identical_to_point_path(name, precision):
    a = SCENES[name](precision)
    b = SCENES[name](precision)
    a.init()
    b.init()
    b.engine.desc.flags |= N.FLAG_POINTWISE  # before any step captures a graph
    a.step_until_n(70)
    b.step_until_n(70)
    nonzero = False
    for comp in G.constant.COMPONENTS:
        fa, fb = np.asarray(a.field[comp].numpy()), np.asarray(b.field[comp].numpy())
        assert np.isfinite(fa).all()
        assert np.array_equal(fa, fb), comp
        nonzero = nonzero or np.abs(fa).max() > 0
    assert nonzero
