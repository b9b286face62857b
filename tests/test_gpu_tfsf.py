"""TFSF plane-wave source on the GPU beyond the golden-vector parity of
test_gpu_parity.py: the incident-field grid's state travels with deepcopy,
the source counts match the reference's objects, and TFSF grids are refused
by the batch path."""
import ctypes as C
from copy import deepcopy

import numpy as np
import pytest

import gmes_gb300 as G
from cases import CASES

pytestmark = pytest.mark.gpu


def test_deepcopy_carries_the_incident_grid():
    sim, n = CASES["tfsf2d"](G)
    sim.init()
    for _ in range(40):
        sim.step()
    twin = deepcopy(sim)
    for _ in range(30):
        sim.step()
        twin.step()
    for comp in (G.Ez, G.Hx, G.Hy):
        assert np.array_equal(np.asarray(sim.field[comp]), np.asarray(twin.field[comp]))


def test_transparent_counts_match_reference_objects():
    sim, _ = CASES["tfsf2d"](G)
    sim.init()
    # the reference builds 42 TransparentEz / Hx / Hy points for this box
    for comp in (G.Ez, G.Hx, G.Hy):
        objs = [v for k, v in sim.pw_source[comp].items() if k.startswith("Transparent")]
        assert len(objs) == 1 and objs[0].idx_size() == 42


def test_tfsf_grid_is_not_batchable():
    from gmes_gb300 import _native as N
    from gmes_gb300.batch import Batch
    sim, _ = CASES["tfsf2d"](G)
    sim.init()
    with pytest.raises(ValueError):
        Batch([sim.engine])
