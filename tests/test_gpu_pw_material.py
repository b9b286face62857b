"""Point-wise updaters on the GPU against the reference's own updater
objects: every model x component x Real/Cmplx, three update_all calls with
the state carried between them, compared bit for bit with
tests/golden/pw_updaters.npz (made by tests/golden/make_golden.py --pw)."""
import os

import numpy as np
import pytest

import gmes_gb300 as G
from cases import PW_COMPS, PW_MODELS, pw_inputs, pw_run, pw_updater

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "pw_updaters.npz"))


@pytest.mark.parametrize("cmplx", [False, True])
@pytest.mark.parametrize("model", PW_MODELS)
def test_updaters_match_reference_bitwise(model, cmplx):
    for comp in PW_COMPS:
        key = f"{model}_{comp}_{'C' if cmplx else 'R'}"
        got = pw_run(G, model, comp, cmplx)
        want = GOLD[key]
        assert got.shape == want.shape
        assert np.array_equal(got, want), (key, np.abs(got - want).max())


def test_state_survives_attach_after_update():
    """Attaching a point after updates keeps the earlier points' state."""
    a = pw_updater(G, "Cpml", "ex", False)
    b = pw_updater(G, "Cpml", "ex", False)
    target_a = pw_inputs("Cpml", "ex", False, 0)[0]
    target_b = target_a.copy()
    for step in range(3):
        _, in1, in2 = pw_inputs("Cpml", "ex", False, step)
        a.update_all(target_a, in1, in2, 0.4, 0.3, 0.35, step)
        b.update_all(target_b, in1, in2, 0.4, 0.3, 0.35, step)
        if step == 0:
            extra = G.Dielectric(eps_inf=3.0).get_pw_material_ex((0, 0, 0), (0, 0, 0))
            # a different type cannot be merged; re-attach the same points' copy
            b.attach((3, 3, 3), b._param[0])
    assert np.array_equal(target_a[:3, :3, :3], target_b[:3, :3, :3])


def test_cuda_tensor_target_without_copy():
    torch = pytest.importorskip("torch")
    upd = pw_updater(G, "Drude", "ez", False)
    ref = pw_updater(G, "Drude", "ez", False)
    t_np = pw_inputs("Drude", "ez", False, 0)[0]
    t_cu = torch.from_numpy(t_np.copy()).cuda()
    for step in range(3):
        _, in1, in2 = pw_inputs("Drude", "ez", False, step)
        ref.update_all(t_np, in1, in2, 0.4, 0.3, 0.35, step)
        upd.update_all(t_cu, torch.from_numpy(in1).cuda(), torch.from_numpy(in2).cuda(),
                       0.4, 0.3, 0.35, step)
    torch.cuda.synchronize()
    assert np.array_equal(t_cu.cpu().numpy(), t_np)
