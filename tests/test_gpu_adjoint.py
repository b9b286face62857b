"""Differentiation on the GPU: the batched TMz forward against the oracle
and the general engine, the adjoint gradient against the CPU FP64 adjoint
and central finite differences, checkpoint and batch invariance, and the
torch.autograd entry point.

Tolerances: fp64 forward <= 1e-12 relative (as the time step itself);
fp64 adjoint vs the CPU adjoint <= 1e-9 relative (different summation
order over a few hundred steps); adjoint vs central differences <= 1e-4
relative per pixel (the target; measured ~1e-8 in fp64 and ~4e-6 in fp32
at the full 512^2 / 2000-step size); df64 vs fp64 <= 1e-9; fp32 vs fp64
gradient <= 1e-5 of the largest component (measured 1.8e-7), the stated
error of the FP32 mode.
"""
import numpy as np
import pytest

from gmes_gb300 import Bandpass, Block, Dielectric, workloads as W
from gmes_gb300.fdtd import TMzFDTD
from conftest import rel_l2
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

BACKGROUND = [((0.0, 1.2, 0.0), (1.0, 0.6, 1.0), 4.0)]


def problem(hard=False, batch=1, n=48, nsteps=160, design_px=6, seed=0):
    st = Bandpass(freq=1.0, fwidth=1.0, s=3)
    return W.design2d(n=n, res=10, pml_cells=6, design_px=design_px, monitor_px=3,
                      nsteps=nsteps, batch=batch, hard=hard, src_time=st, seed=seed,
                      background=BACKGROUND)


def make(precision="fp64", batch=1, hard=False, segment=None, keep_history=None, **kw):
    from gmes_gb300.adjoint import TMzAdjoint
    space, geom, src, design, monitor, eps, nsteps = problem(hard=hard, batch=batch, **kw)
    prob = TMzAdjoint(space, geom, src, design, monitor, nsteps, batch=batch,
                      precision=precision, segment=segment, keep_history=keep_history)
    return prob, eps, (space, geom, src, design, monitor, nsteps)


def oracle_run(prob, eps_b, gradient=True):
    (d0, dn), (m0, mn) = prob.design_box, prob.monitor_box
    dpts = [(2, (d0[0] + a, d0[1] + b, 0)) for a in range(dn[0]) for b in range(dn[1])]
    mpts = [(2, (m0[0] + a, m0[1] + b, 0)) for a in range(mn[0]) for b in range(mn[1])]
    o = Oracle(prob.scene)
    o.set_eps(2, [p for _, p in dpts], np.asarray(eps_b).reshape(-1))
    J, g = o.adjoint(prob.nsteps, mpts, dpts, gradient=gradient)
    return o, J, g.reshape(dn)


@pytest.mark.parametrize("hard", [False, True])
def test_forward_matches_oracle(hard):
    prob, eps, _ = make("fp64", hard=hard)
    J = prob.forward(eps).cpu().numpy()
    o, Jo, _ = oracle_run(prob, eps[0], gradient=False)
    assert abs(J[0] - Jo) <= 1e-12 * abs(Jo)
    nx, ny = prob.scene.n[0], prob.scene.n[1]
    ez, hx, hy = (prob.lattice(k)[0].cpu().numpy() for k in range(3))
    assert rel_l2(ez, o.field(2)[:nx, :ny, 0]) <= 1e-12
    assert rel_l2(hx, o.field(3)[:, 1:, 1]) <= 1e-12
    assert rel_l2(hy, o.field(4)[1:, :, 1]) <= 1e-12


def test_forward_matches_engine_with_pixel_blocks():
    """The design pixels as per-pixel Blocks of the general engine: same fields."""
    prob, eps, (space, geom, src, design, monitor, nsteps) = make("fp64")
    prob.forward(eps)
    (d0, dn) = prob.design_box
    dx, dy = space.dr[0], space.dr[1]
    blocks = []
    for a in range(dn[0]):
        for b in range(dn[1]):
            x = (d0[0] + a) * dx - space.half_size[0]
            y = (d0[1] + b) * dy - space.half_size[1]
            blocks.append(Block(material=Dielectric(eps_inf=float(eps[0, a, b])),
                                center=(x, y, 0.0), size=(0.5 * dx, 0.5 * dy, 1.0)))
    sim = TMzFDTD(space, geom[:-1] + blocks + geom[-1:], src, verbose=False, precision="fp64")
    sim.init()
    for _ in range(nsteps):
        sim.step()
    nx, ny = prob.scene.n[0], prob.scene.n[1]
    assert rel_l2(prob.lattice(0)[0].cpu().numpy(), np.asarray(sim.ez)[:nx, :ny, 0]) <= 1e-12


@pytest.mark.parametrize("hard", [False, True])
def test_adjoint_matches_cpu_adjoint(hard):
    prob, eps, _ = make("fp64", hard=hard)
    J = prob.forward(eps).cpu().numpy()
    g = prob.backward().cpu().numpy()[0]
    _, Jo, go = oracle_run(prob, eps[0])
    assert abs(J[0] - Jo) <= 1e-12 * abs(Jo)
    assert np.abs(g - go).max() <= 1e-9 * np.abs(go).max()


def test_adjoint_matches_central_differences():
    """16 random pixels, +-h perturbations run as one batch of 32 designs."""
    prob, eps, _ = make("fp64")
    prob.forward(eps)
    g = prob.backward().cpu().numpy()[0]
    rng = np.random.default_rng(7)
    nd = eps.shape[1] * eps.shape[2]
    pix = rng.choice(nd, size=16, replace=False)
    h = 1e-4
    fd_prob, _, _ = make("fp64", batch=32)
    batch = np.repeat(eps, 32, axis=0).reshape(32, -1)
    for q, p in enumerate(pix):
        batch[2 * q, p] += h
        batch[2 * q + 1, p] -= h
    J = fd_prob.forward(batch.reshape(32, *eps.shape[1:]), checkpoints=False).cpu().numpy()
    fd = (J[0::2] - J[1::2]) / (2 * h)
    ga = g.reshape(-1)[pix]
    rel = np.abs(ga - fd) / np.abs(fd)
    print("adjoint vs central differences, max relative error", rel.max())
    assert rel.max() <= 1e-4


@pytest.mark.parametrize("precision", ["fp64", "fp32", "df64"])
def test_recorded_history_equals_checkpoint_recompute(precision):
    """The forward that records every step's design increments (no backward
    recompute) and the √N-checkpoint forward give the same J and gradient,
    bit for bit; the default picks the recorded history when it fits."""
    a, eps, _ = make(precision, batch=2, keep_history=True)
    b, _, _ = make(precision, batch=2, keep_history=False)
    assert a.keep_history and not b.keep_history
    assert make(precision)[0].keep_history  # a small problem: fits
    assert not make(precision, segment=9)[0].keep_history
    Ja, Jb = a.forward(eps).cpu().numpy(), b.forward(eps).cpu().numpy()
    assert np.array_equal(Ja, Jb)
    ga, gb = a.backward().cpu().numpy(), b.backward().cpu().numpy()
    assert np.abs(ga).max() > 0
    assert np.array_equal(ga, gb)
    # a second forward / backward on the same problem reuses its buffers
    a.forward(eps[::-1].copy())
    assert not np.array_equal(a.backward().cpu().numpy(), ga)


def test_checkpoint_segments_do_not_change_the_gradient():
    grads = []
    for seg in (1, 7, None, 160):
        prob, eps, _ = make("fp64", segment=seg)
        prob.forward(eps)
        grads.append(prob.backward().cpu().numpy())
    for g in grads[1:]:
        assert np.array_equal(g, grads[0])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_designs_are_independent_in_a_batch(precision):
    prob3, eps3, _ = make(precision, batch=3, seed=3)
    J3 = prob3.forward(eps3).cpu().numpy()
    g3 = prob3.backward().cpu().numpy()
    prob1, _, _ = make(precision, batch=1)
    J1 = prob1.forward(eps3[1:2]).cpu().numpy()
    g1 = prob1.backward().cpu().numpy()
    assert J1[0] == J3[1]
    assert np.array_equal(g1[0], g3[1])


@pytest.mark.parametrize("n,nsteps,segment,hard", [(48, 160, 7, False), (48, 37, None, True),
                                                   (130, 161, 9, False)])
def test_blocked_fp32_kernels_match_one_step_kernels(n, nsteps, segment, hard):
    """The temporally blocked FP32 kernels (2..4 steps per launch) against
    the one-step kernels: monitor objective, fields and gradients
    bit-identical.  The 48^2 lattice is smaller than a block's region (its
    periodic images repeat inside it); 130^2 has partial edge tiles; the
    step counts are not multiples of the steps per launch or the segment."""
    from gmes_gb300.adjoint import TMzAdjoint
    space, geom, src, design, monitor, eps, ns = problem(hard=hard, batch=2, n=n, nsteps=nsteps,
                                                         seed=4)
    out = {}
    for bs in (1, 2, 3, 4):
        prob = TMzAdjoint(space, geom, src, design, monitor, ns, batch=2, precision="fp32",
                          segment=segment, block_steps=bs)
        J = prob.forward(eps).cpu().numpy()
        fields = [prob.lattice(k).cpu().numpy() for k in range(3)]
        g = prob.backward().cpu().numpy()
        out[bs] = (J, fields, g)
    J1, f1, g1 = out[1]
    assert np.all(np.isfinite(g1)) and np.abs(g1).max() > 0
    for bs in (2, 3, 4):
        J, f, g = out[bs]
        assert np.array_equal(J, J1), bs
        for a, b in zip(f, f1):
            assert np.array_equal(a, b), bs
        assert np.array_equal(g, g1), bs


def test_block_steps_out_of_range():
    from gmes_gb300.adjoint import TMzAdjoint
    space, geom, src, design, monitor, eps, ns = problem()
    with pytest.raises(ValueError):
        TMzAdjoint(space, geom, src, design, monitor, ns, precision="fp32", block_steps=5)


@pytest.mark.parametrize("precision,tol", [("df64", 1e-9), ("fp32", 1e-5)])
def test_reduced_precision_gradient_error(precision, tol):
    ref, eps, _ = make("fp64")
    ref.forward(eps)
    g64 = ref.backward().cpu().numpy()
    prob, _, _ = make(precision)
    prob.forward(eps)
    g = prob.backward().cpu().numpy()
    err = np.abs(g - g64).max() / np.abs(g64).max()
    print(precision, "gradient error vs fp64 (max abs / max)", err)
    assert err <= tol


def test_autograd_function_and_weights():
    torch = pytest.importorskip("torch")
    prob, eps, _ = make("fp64", batch=2, seed=5)
    w = torch.tensor([0.25, -1.5], dtype=torch.float64, device="cuda")
    x = torch.tensor(eps, dtype=torch.float64, device="cuda", requires_grad=True)
    J = prob.objective(x)
    (w * J).sum().backward()
    prob.forward(eps)
    g = prob.backward(w)
    assert torch.equal(x.grad, g)
    # a later forward invalidates the earlier graph's checkpoints
    J1 = prob.objective(x)
    prob.forward(eps)
    with pytest.raises(RuntimeError):
        J1.sum().backward()


def test_rejects_bad_inputs():
    from gmes_gb300.adjoint import DesignRegion, TMzAdjoint
    prob, eps, (space, geom, src, design, monitor, nsteps) = make("fp64")
    with pytest.raises(ValueError):
        prob.forward(-eps)
    with pytest.raises(ValueError):
        TMzAdjoint(space, geom, src, DesignRegion((-2.1, 0.0), (0.4, 0.4)), monitor, 10)
    with pytest.raises(IndexError):
        TMzAdjoint(space, geom, src, DesignRegion((0.0, 0.0), (40.0, 0.4)), monitor, 10)


def test_full_size_gradient_against_central_differences():
    """The 512^2 / 64x64-pixel / 2000-step scene: fp32 and fp64 adjoints
    against FP64 central differences on 16 random pixels of one design."""
    from gmes_gb300.adjoint import TMzAdjoint
    torch = pytest.importorskip("torch")
    space, geom, src, design, monitor, eps, nsteps = W.design2d(batch=2)
    rng = np.random.default_rng(11)
    pix = rng.choice(64 * 64, size=16, replace=False)
    h = 1e-3
    fd_prob = TMzAdjoint(space, geom, src, design, monitor, nsteps, batch=32, precision="fp64")
    batch = np.repeat(eps[:1], 32, axis=0).reshape(32, -1)
    for q, p in enumerate(pix):
        batch[2 * q, p] += h
        batch[2 * q + 1, p] -= h
    J = fd_prob.forward(batch.reshape(32, 64, 64), checkpoints=False).cpu().numpy()
    fd = (J[0::2] - J[1::2]) / (2 * h)
    del fd_prob
    torch.cuda.empty_cache()
    for precision, tol in (("fp64", 1e-4), ("fp32", 1e-4)):
        prob = TMzAdjoint(space, geom, src, design, monitor, nsteps, batch=2,
                          precision=precision)
        Jp = prob.forward(eps).cpu().numpy()
        g = prob.backward().cpu().numpy()[0].reshape(-1)[pix]
        rel = np.abs(g - fd) / np.abs(fd)
        print(precision, "J", Jp, "max relative error vs central differences", rel.max(),
              "median", np.median(rel))
        assert np.all(np.isfinite(Jp)) and Jp.min() > 0
        assert rel.max() <= tol
        del prob
        torch.cuda.empty_cache()
