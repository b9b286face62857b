"""The CPU FP64 adjoint of the oracle against central finite differences of
the oracle's own forward run (no GPU).  This pins the double-precision CPU
adjoint that the GPU adjoint kernels are checked against."""
import numpy as np
import pytest

from gmes_gb300 import Bandpass, workloads as W
from gmes_gb300.fdtd import TMzFDTD
from oracle.oracle import Oracle


def small_problem(hard):
    st = Bandpass(freq=1.0, fwidth=1.0, s=3)
    space, geom, src, design, monitor, eps, nsteps = W.design2d(
        n=40, res=10, pml_cells=6, design_px=4, monitor_px=2, nsteps=120, batch=1, hard=hard,
        src_time=st, background=[((0.0, 1.2, 0.0), (1.0, 0.6, 1.0), 4.0)])
    scene = TMzFDTD(space, geom, src, verbose=False).compile()
    (d0, dn), (m0, mn) = design.box(space), monitor.box(space)
    dpts = [(2, (d0[0] + a, d0[1] + b, 0)) for a in range(dn[0]) for b in range(dn[1])]
    mpts = [(2, (m0[0] + a, m0[1] + b, 0)) for a in range(mn[0]) for b in range(mn[1])]
    return scene, dpts, mpts, eps[0].reshape(-1), nsteps


@pytest.mark.parametrize("hard", [False, True])
def test_cpu_adjoint_matches_central_differences(hard):
    scene, dpts, mpts, e, nsteps = small_problem(hard)
    o = Oracle(scene)
    o.set_eps(2, [p for _, p in dpts], e)
    J, g = o.adjoint(nsteps, mpts, dpts)
    assert J > 0 and np.all(np.isfinite(g)) and np.any(g != 0)

    def J_of(ev):
        o.reset()
        o.set_eps(2, [p for _, p in dpts], ev)
        return o.adjoint(nsteps, mpts, dpts, gradient=False)[0]

    h = 1e-4
    for q in range(len(e)):
        ep, em = e.copy(), e.copy()
        ep[q] += h
        em[q] -= h
        fd = (J_of(ep) - J_of(em)) / (2 * h)
        # FP64 central difference: truncation ~h^2, well below 1e-6 here
        assert abs(g[q] - fd) <= 1e-6 * abs(fd) + 1e-12 * np.abs(g).max(), (q, g[q], fd)


def test_cpu_adjoint_rejects_unsupported_points():
    scene, dpts, mpts, e, nsteps = small_problem(False)
    o = Oracle(scene)
    with pytest.raises(ValueError):
        o.set_eps(2, [(0, 0, 0)], [2.0])     # a CPML point, not dielectric
    with pytest.raises(ValueError):
        o.adjoint(2, mpts, [(3, (1, 1, 1))])  # design on an H component
