"""Device probes: FDTD.set_probe records through the engine's per-step device
buffer and writes the reference's text files (gmes/file_io.py:9-48).  The
files are compared with the reference's own recordings (tests/golden/
probe_*.dat, made by tests/golden/make_golden.py --probes)."""
import os

import numpy as np
import pytest

import gmes_gb300 as G
from cases import CASES
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
POINT = (0.2, 0.1, 0.0)


def record(name, precision, tmp_path, chunk=None):
    sim, nsteps = CASES[name](G)
    sim.precision = precision
    sim.init()
    if chunk:
        sim.engine.src_chunk = chunk
    if precision == "fp64_strict":
        engines = [(sim.engine, sim.scene)]
        if sim.engine.incident is not None:
            engines.append((sim.engine.incident, sim.scene.tfsf[0]))
        for eng, scene in engines:
            orc = Oracle(scene)
            for p in range(len(scene.pmls)):
                for comp in scene.active:
                    for axis in range(3):
                        eng.set_pml_profile(p, comp.index, axis,
                                            orc.pml_profile(p, comp.index, axis))
    prefix = str(tmp_path / "p")
    sim.set_probe(POINT, prefix)
    sim.step_until_n(nsteps)
    out = {}
    for rec in sim.e_recorder + sim.h_recorder:
        rec.close()
    for comp in ("ez", "hx", "hy"):
        out[comp] = (tmp_path / f"p_{comp}.dat").read_text()
    return out


def golden(name, comp):
    with open(os.path.join(GOLDEN, f"probe_{name}_{comp}.dat")) as f:
        return f.read()


@pytest.mark.parametrize("name", ["tmz_regression", "tfsf2d"])
def test_strict_probe_files_equal_reference(name, tmp_path):
    got = record(name, "fp64_strict", tmp_path)
    for comp, text in got.items():
        assert text == golden(name, comp), (name, comp)


def test_fast_probe_values_and_chunking(tmp_path):
    ref = {c: golden("tfsf2d", c) for c in ("ez", "hx", "hy")}
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    got = record("tfsf2d", "fp64", tmp_path / "a")
    got7 = record("tfsf2d", "fp64", tmp_path / "b", chunk=7)  # chunks of 7 steps
    for comp in ref:
        r = np.loadtxt(ref[comp].splitlines())
        g = np.loadtxt(got[comp].splitlines())
        assert got[comp].splitlines()[:2] == ref[comp].splitlines()[:2]
        assert np.array_equal(g[:, 0], r[:, 0])
        assert np.abs(g[:, 1] - r[:, 1]).max() <= 1e-12 * np.abs(r[:, 1]).max()
        assert got7[comp] == got[comp]
