"""The GPU material-map builder against the host rasteriser.

The host path (numpy, tests/test_oracle_golden.py pins it against the
reference's own per-point material mapping) and the GPU kernel must give
identical u8 class maps, point for point.
"""
import numpy as np
import pytest

import gmes_gb300 as G
from gmes_gb300 import workloads as W
from gmes_gb300.engine import GridEngine
from cases import CASES

pytestmark = pytest.mark.gpu


def scenes():
    out = [(name, lambda f=f: f(G)[0]) for name, f in CASES.items()]
    out.append(("cube96", lambda: W.cube(n=96)[0]))
    out.append(("disp64", lambda: W.dispersive(n=64, res=10)[0]))
    for q, (_, b, _) in enumerate(W.serving_jobs(6, seed=3, size_scale=0.3)):
        out.append((f"serving{q}", b))
    out.append(("rotated", rotated_shapes))
    return out


def rotated_shapes():
    geom = [G.DefaultMedium(material=G.Dielectric()),
            G.Block(material=G.Dielectric(eps_inf=3), center=(0.1, -0.2, 0.05),
                    e1=(1, 1, 0), e2=(-1, 1, 0.3), e3=(0, 0, 1), size=(0.6, 0.4, 0.8)),
            G.Ellipsoid(material=G.Dielectric(eps_inf=5), center=(-0.3, 0.2, 0),
                        e1=(1, 0.5, 0), size=(0.5, 0.3, 0.9)),
            G.Cone(material=G.Dielectric(eps_inf=7), center=(0.3, 0.3, -0.2), radius=0.3,
                   radius2=0.05, axis=(0.2, 1, 0.4), height=0.7),
            G.Cylinder(material=G.Dielectric(eps_inf=2), center=(0, 0, 0.4), radius=0.2,
                       axis=(1, 0, 0), height=1.2),
            G.Shell(material=G.Cpml(), thickness=0.25)]
    space = G.Cartesian(size=(1.6, 1.4, 1.2), resolution=20)
    return G.FDTD(space, geom, [], verbose=False)


@pytest.mark.parametrize("name,build", scenes(), ids=[n for n, _ in scenes()])
def test_device_class_maps_equal_host(name, build):
    sim = build()
    scene = sim.compile()
    assert scene.device_raster
    eng = GridEngine(scene)
    assert eng.rasterized
    for comp in scene.active:
        c = comp.index
        dev = eng.cls[c].cpu().numpy()
        host = scene.host_cls(c)
        assert dev.shape == host.shape
        assert np.array_equal(dev, host), (name, comp.__name__, int((dev != host).sum()))
