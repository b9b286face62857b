"""Host-side figures of the bench line that need no GPU: the kernel-launch
count claimed for the differentiation workload, which follows the
library's chunking of the temporally blocked kernels, and the algorithmic
bytes per half-step behind the roofline fraction."""
import types

import pytest


def _prob(nsteps, segment, keep):
    return types.SimpleNamespace(nsteps=nsteps, segment=segment, keep_history=keep)


def _adj_chunks(k, per):
    # the library's adjoint launches: the fewest of at most ``per`` steps
    # whose count has the parity of k (the psi-adjoint buffers alternate per
    # launch and must end where the step-parity convention puts them)
    n = -(-k // per)
    while n % 2 != k % 2:
        n += 1
    return min(n, k)


@pytest.mark.parametrize("nsteps,segment", [(2000, 45), (160, 7), (37, 37), (1, 1)])
def test_design_launch_count(nsteps, segment):
    import bench
    per = 4
    segs = [min(segment, nsteps - s0) for s0 in range(0, nsteps, segment)]
    fwd = sum(-(-k // per) for k in segs)
    # √N checkpoints: forward and recompute per segment, then the adjoint
    assert bench.design_launches(_prob(nsteps, segment, False), "fp32", 0) == \
        2 * fwd + sum(_adj_chunks(k, per) for k in segs)
    # recorded history: one forward and one adjoint over all steps
    assert bench.design_launches(_prob(nsteps, segment, True), "fp32", 0) == \
        -(-nsteps // per) + _adj_chunks(nsteps, per)
    # one step per launch: E, E sources, H, H sources per step of each pass
    assert bench.design_launches(_prob(nsteps, segment, True), "fp64", 0) == 8 * nsteps
    assert bench.design_launches(_prob(nsteps, segment, False), "fp32", 1) == 12 * nsteps


def test_adjoint_chunks_of_the_default_workload():
    # 2000 steps: 500 launches of 4; a 45-step segment: 13 launches (odd)
    assert _adj_chunks(2000, 4) == 500
    assert _adj_chunks(45, 4) == 13 and _adj_chunks(2, 4) == 2 and _adj_chunks(1, 4) == 1


@pytest.mark.parametrize("precision,es", [("fp64", 8), ("fp32", 4), ("df64", 8)])
def test_half_bytes_of_a_cube(precision, es):
    """E half: every E value read and written, every H value read, one class
    id per E point, and psi1 / psi2 read and written at every CPML point;
    the H half likewise with the roles swapped."""
    import bench
    from gmes_gb300 import workloads as W
    sim, _ = W.cube(n=12, nobj=2, pml_cells=3, precision="fp64")
    scene = sim.compile()
    e_b, h_b = bench.half_bytes(scene, precision)
    for side, got in ((0, e_b), (1, h_b)):
        own = [c for c in range(6) if (c < 3) == (side == 0)]
        other = [c for c in range(6) if c not in own]
        want = 0
        for c in own:
            n = 1
            for v in scene.shape(c):
                n *= v
            cpml = sum(cnt for cid, cnt in scene.counts(c).items()
                       if scene.classes[c][cid].kind == 2)  # GMES_KIND_CPML
            want += 2 * es * n + n + 2 * 2 * es * cpml
        for c in other:
            n = 1
            for v in scene.shape(c):
                n *= v
            want += es * n
        assert got == want, (side, got, want)
