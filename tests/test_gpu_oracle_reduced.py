"""The benchmark scenes' generators at reduced size, pinned to the CPU oracle.

The full-size 256^3 and 192^3 runs are checked against the GPU's own
reference-order FP64 mode (test_gpu_march.py); here the same generators
build a 96^3 dielectric + CPML cube (object radii scaled with the grid) and
a 64^3 dispersive scene (Drude, Lorentz, DCP-ADE spheres in a UPML shell,
TFSF plane wave), small enough for the oracle -- the C restatement of the
reference's per-point loops, bit-exact with the reference on the golden
scenes -- and run a few hundred steps through the pulse peak.  Tolerances
(relative L2 per component): fp64 1e-12, df64 1e-11 (two floats carry 48-49
significand bits), fp32 5e-3.
"""
import numpy as np
import pytest

import gmes_gb300 as G
from gmes_gb300 import workloads as W
from conftest import rel_l2
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "df64": 1e-11, "fp32": 5e-3}
# peaks at t = 10: step ~175 of the cube (dt 0.057), ~385 of the dispersive
# scene (dt 0.026)
PULSE = G.Bandpass(freq=0.5, fwidth=1.0)
SCENES = {
    "cube96": (lambda p: W.cube(n=96, precision=p, src_time=PULSE)[0], 300),
    "dispersive64": (lambda p: W.dispersive(n=64, precision=p, src_time=PULSE)[0], 500),
}

_ref = {}


def oracle_fields(name):
    if name not in _ref:
        build, steps = SCENES[name]
        orc = Oracle(build("fp64").compile())
        orc.step(steps)
        _ref[name] = orc.fields()
    return _ref[name]


@pytest.mark.parametrize("precision", ["fp64", "df64", "fp32"])
@pytest.mark.parametrize("name", list(SCENES))
def test_reduced_benchmark_scene_against_oracle(name, precision):
    build, steps = SCENES[name]
    sim = build(precision)
    sim.init()
    sim.step_until_n(steps)
    ref = oracle_fields(name)
    assert max(float(np.abs(r).max()) for r in ref) > 1e-6
    for c, comp in enumerate(G.constant.COMPONENTS):
        f = sim.field[comp].numpy()
        assert np.isfinite(f).all()
        err = rel_l2(f, ref[c])
        assert err <= TOL[precision], (name, precision, comp.__name__, err)
