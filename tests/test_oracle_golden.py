"""The CPU oracle against vectors produced by the reference itself.

tests/golden/*.npz were generated by tests/golden/make_golden.py, which runs
the reference GMES package on the scenes of tests/golden/cases.py.  The
oracle is fed by this package's scene compiler (vectorised rasterisation,
class maps) and must reproduce the reference BIT FOR BIT: same per-point
coefficients, same operation order, same ghost copies.
"""
import numpy as np
import pytest

import gmes_gb300 as G
from cases import CASES, COMP_NAMES, ORACLE_CASES, SUMMARY_ONLY
from conftest import checksum, load_golden
from oracle.oracle import Oracle


ALL_CASES = {**CASES, **ORACLE_CASES}


@pytest.mark.parametrize("name", list(ALL_CASES))
def test_oracle_matches_reference_bitwise(name):
    gold, meta = load_golden(name)
    sim, nsteps = ALL_CASES[name](G)
    assert nsteps == meta["steps"]
    scene = sim.compile()
    orc = Oracle(scene)
    orc.step(nsteps)
    for c, cn in enumerate(COMP_NAMES):
        f = orc.field(c)
        assert list(f.shape) == meta["shapes"][cn]
        if cn in gold:
            assert np.array_equal(f, gold[cn]), f"{name}.{cn} differs from the reference"
        else:
            assert checksum(f) == pytest.approx(meta["checksums"][cn], rel=1e-14, abs=0)
        # a golden scene must be physically stable, or agreement means nothing
        assert np.max(np.abs(f)) < 10.0, f"{name}.{cn} diverges"


def test_reference_known_answers():
    """tests/test_fdtd.py:74-79 and examples/VERIFICATION.md:7 of the reference."""
    sim, n = CASES["tmz_regression"](G)
    orc = Oracle(sim.compile())
    orc.step(n)
    ez = orc.field(2)
    assert ez.shape == (11, 11, 1)
    assert ez[5, 5, 0] == pytest.approx(-0.9996801161298625, abs=1e-15)
    assert np.sum(np.abs(ez) ** 2) == pytest.approx(1.5780099423691636, rel=1e-14)
    gold, _ = load_golden("air2d")
    assert float(np.max(np.abs(gold["ez"]))) == 0.999382775451675


def test_time_bookkeeping_matches_reference():
    """step count and final time of step_until_t(10) for air2d (286 steps)."""
    for name in CASES:
        _, meta = load_golden(name)
        ts = G.TimeStep(meta["dt"])
        for _ in range(meta["steps"]):
            ts.half_step_up()
            ts.half_step_up()
        assert ts.n == meta["n"] and ts.t == meta["t"]
    sim, _ = CASES["air2d"](G)
    k = sim._steps_until(lambda ts: ts.t < 10)
    assert k == 286


def test_updater_point_counts_match_reference():
    """Points per material updater equal the reference's idx_size() (benchmarks/field_updates.py:73-96)."""
    from gmes_gb300.material import KIND_NAMES
    for name in CASES:
        _, meta = load_golden(name)
        sim, _ = CASES[name](G)
        scene = sim.compile()
        for comp in scene.active:
            want = {}
            for tname, count in meta["updaters"][comp.__name__].items():
                suffix = "Cmplx" if tname.endswith("Cmplx") else "Real"
                kind = tname[:-len(comp.__name__) - len(suffix)]
                want[kind] = want.get(kind, 0) + count
            got = {}
            for cid, count in scene.counts(comp.index).items():
                k = KIND_NAMES[scene.classes[comp.index][cid].kind]
                got[k] = got.get(k, 0) + count
            # the reference's Drude/Lorentz/DcpAde H updaters are plain dielectric here
            for k in ("Drude", "Lorentz", "DcpAde", "DcpPlrc"):
                if comp.index >= 3 and k in want:
                    want["Dielectric"] = want.get("Dielectric", 0) + want.pop(k)
            assert got == want, (name, comp.__name__)
