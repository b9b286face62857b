"""The point-wise updater interface (the reference's gmes.pw_material): the
argument checks and error classes of its binding (src/pw_material.i:23-51,
numpy.i), which run on the host before any GPU work.  The numerics are in
tests/test_gpu_pw_material.py."""
import numpy as np
import pytest

import gmes_gb300 as G
from gmes_gb300 import pw_material as pm
from cases import PW_COMPS, PW_MODELS, pw_material, pw_updater


def test_every_reference_class_exists():
    for sfx in ("Real", "Cmplx"):
        for model in PW_MODELS:
            if model == "DcpRc":
                continue
            for comp in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
                assert hasattr(pm, model + comp + sfx)
            assert hasattr(pm, model + "ElectricParam" + sfx)
            assert hasattr(pm, model + "MagneticParam" + sfx)


def test_names_sizes_and_merge():
    upd = pw_updater(G, "Cpml", "hy", False)
    assert upd.idx_size() == 3 and upd.name() == "CpmlMagnetic"
    assert pw_updater(G, "DcpAde", "hx", False).name() == "DcpMagnetic"
    assert pw_updater(G, "DcpRc", "ez", True).name() == "DcpPlrcElectric"
    assert type(pw_updater(G, "DcpRc", "ez", True)).__name__ == "DcpPlrcEzCmplx"
    with pytest.raises(TypeError):
        upd.merge(pw_updater(G, "Cpml", "hx", False))


def test_get_eps_inf_and_index_arity():
    m = pw_material(G, "Dielectric")
    upd = m.get_pw_material_ex((1, 1, 1), (0, 0, 0))
    for idx in np.ndindex(3, 3, 3):
        assert upd.get_eps_inf(idx) == (m.eps_inf if idx == (1, 1, 1) else 0)
    for bad in ((1, 1), (1, 1, 1, 1)):
        with pytest.raises(ValueError, match="exactly three values"):
            upd.get_eps_inf(bad)
    assert m.get_pw_material_hz((1, 1, 1), (0, 0, 0)).get_mu_inf((1, 1, 1)) == m.mu_inf


@pytest.mark.parametrize("shape,bad", [((3, 3, 3), (-1, 1, 1)), ((3, 3, 3), (3, 1, 1)),
                                       ((3, 3, 3), (1, -1, 1)), ((3, 3, 3), (1, 3, 1)),
                                       ((3, 3, 3), (1, 1, 3)), ((1, 1, 1), (1, 0, 0)),
                                       ((1, 1, 1), (0, 0, -1))])
def test_out_of_bounds_index_raises_before_any_write(shape, bad):
    for cmplx in (False, True):
        upd = pw_material(G, "Const").get_pw_material_ex(bad, (0, 0, 0), cmplx=cmplx)
        fields = [np.zeros(shape, complex if cmplx else float) for _ in range(3)]
        with pytest.raises(IndexError, match="out of bounds"):
            upd.update_all(*fields, 1, 1, 1, 0)
        assert not fields[0].any()


def test_array_checks():
    for comp in PW_COMPS:
        upd = pw_updater(G, "Dielectric", comp, False)
        fields = [np.zeros((4, 4, 4)) for _ in range(3)]
        fields[0].flags.writeable = False
        with pytest.raises(TypeError, match="must be writeable"):
            upd.update_all(*fields, 1, 1, 1, 0)
    upd = pw_updater(G, "Dielectric", "ex", False)
    with pytest.raises(TypeError):
        upd.update_all(np.zeros((4, 4, 4), complex), np.zeros((4, 4, 4)), np.zeros((4, 4, 4)),
                       1, 1, 1, 0)
    with pytest.raises(TypeError):
        upd.update_all(np.zeros((4, 4)), np.zeros((4, 4, 4)), np.zeros((4, 4, 4)), 1, 1, 1, 0)
    with pytest.raises(TypeError):
        upd.update_all(np.zeros((4, 4, 4))[:, ::2], np.zeros((4, 4, 4)), np.zeros((4, 4, 4)),
                       1, 1, 1, 0)


def test_coefficient_shapes_are_checked():
    for cls in (pm.DrudeElectricParamReal, pm.LorentzElectricParamCmplx):
        cls().set(np.zeros((1, 3)), np.zeros(3))
        for a, c in ((np.zeros((1, 2)), np.zeros(3)), (np.zeros((1, 3)), np.zeros(4))):
            with pytest.raises(ValueError):
                cls().set(a, c)
    pm.DcpAdeElectricParamReal().set(np.zeros((1, 3)), np.zeros((1, 5)), np.zeros(4))
    with pytest.raises(ValueError):
        pm.DcpAdeElectricParamReal().set(np.zeros((1, 3)), np.zeros((1, 4)), np.zeros(4))
    pm.DcpPlrcElectricParamCmplx().set(np.zeros((1, 3)), np.zeros((1, 3), complex), np.zeros(3))
    with pytest.raises(ValueError):
        pm.DcpPlrcElectricParamCmplx().set(np.zeros((1, 3)), np.zeros((1, 3), complex),
                                           np.zeros(2))


def test_attach_copies_the_parameter_by_value():
    p = pm.DielectricElectricParamReal()
    p.eps_inf = 2.0
    upd = pm.DielectricExReal().attach((1, 1, 1), p)
    p.eps_inf = 5.0
    assert upd.get_eps_inf((1, 1, 1)) == 2.0
    with pytest.raises(TypeError):
        pm.DielectricExReal().attach((1, 1, 1), pm.CpmlElectricParamReal())
