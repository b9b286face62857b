"""Total-field / scattered-field plane-wave source: host-side setup.

The reference (gmes/source.py:370-1522, gmes/pw_source.py:134-486) launches
a plane wave through the faces of a box: a 1-D TEMz FDTD ("incident-field
grid") carries the incident wave with a cell size matched to the 3-D
numerical dispersion, and every E/H point on a face of the box gets a
consistency correction ``F += sign * dt/(eps d) * amp * incident`` after its
material update, the incident value interpolated from the 1-D grid at the
point's projected distance along the beam axis.

This module computes, once, what those per-point Python objects hold: the
incident-field grid's geometry and the table of transparent points
(component, offset, and per face the signed coefficient, interpolation
weights and sample offset).  The CUDA engine applies the corrections and
steps the incident-field grid between the E and H halves.

The face table below restates the rules of the reference's 24
``_get_pw_source_<comp>_<face>`` methods: which faces a component has,
the cosine that scales its amplitude, which component's index function
spans the face (with an index shift for the H components), which
neighbouring point is projected onto the beam axis, and the sign.
"""

from math import floor, inf, pi, sin, sqrt

import numpy as np

from . import constant as const

MINUS, PLUS = 0, 1

# comp -> list of (cosine source "e"|"h", cosine axis, [faces]) in the
# reference's order; a face is (axis, side, index comp, index shift,
# sample comp, sample offset, sign).
_E, _H = "e", "h"
FACES = {
    const.Ex: [(_H, 2, [(1, MINUS, const.Ex, (0, 0, 0), const.Hz, (1, 0, 0), -1),
                        (1, PLUS, const.Ex, (0, 0, 0), const.Hz, (1, 1, 0), +1)]),
               (_H, 1, [(2, MINUS, const.Ex, (0, 0, 0), const.Hy, (1, 0, 0), +1),
                        (2, PLUS, const.Ex, (0, 0, 0), const.Hy, (1, 0, 1), -1)])],
    const.Ey: [(_H, 0, [(2, MINUS, const.Ey, (0, 0, 0), const.Hx, (0, 1, 0), -1),
                        (2, PLUS, const.Ey, (0, 0, 0), const.Hx, (0, 1, 1), +1)]),
               (_H, 2, [(0, MINUS, const.Ey, (0, 0, 0), const.Hz, (0, 1, 0), +1),
                        (0, PLUS, const.Ey, (0, 0, 0), const.Hz, (1, 1, 0), -1)])],
    const.Ez: [(_H, 1, [(0, MINUS, const.Ez, (0, 0, 0), const.Hy, (0, 0, 1), -1),
                        (0, PLUS, const.Ez, (0, 0, 0), const.Hy, (1, 0, 1), +1)]),
               (_H, 0, [(1, MINUS, const.Ez, (0, 0, 0), const.Hx, (0, 0, 1), +1),
                        (1, PLUS, const.Ez, (0, 0, 0), const.Hx, (0, 1, 1), -1)])],
    const.Hx: [(_E, 2, [(1, MINUS, const.Ez, (0, 0, 1), const.Ez, (0, 0, -1), +1),
                        (1, PLUS, const.Ez, (0, 1, 1), const.Ez, (0, -1, -1), -1)]),
               (_E, 1, [(2, MINUS, const.Ey, (0, 1, 0), const.Ey, (0, -1, -1), -1),
                        (2, PLUS, const.Ey, (0, 1, 1), const.Ey, (0, -1, 0), +1)])],
    const.Hy: [(_E, 0, [(2, MINUS, const.Ex, (1, 0, 0), const.Ex, (-1, 0, 0), +1),
                        (2, PLUS, const.Ex, (1, 0, 1), const.Ex, (-1, 0, -1), -1)]),
               (_E, 2, [(0, MINUS, const.Ez, (0, 0, 1), const.Ez, (0, 0, -1), -1),
                        (0, PLUS, const.Ez, (1, 0, 1), const.Ez, (-1, 0, -1), +1)])],
    const.Hz: [(_E, 1, [(0, MINUS, const.Ey, (0, 1, 0), const.Ey, (0, -1, 0), +1),
                        (0, PLUS, const.Ey, (1, 1, 0), const.Ey, (-1, -1, 0), -1)]),
               (_E, 0, [(1, MINUS, const.Ex, (1, 0, 0), const.Ex, (0, -1, 0), -1),
                        (1, PLUS, const.Ex, (1, 1, 0), const.Ex, (-1, -1, 0), +1)])],
}


def _bisect(f, a, b, args):
    """Root of f in [a, b] by bisection (scipy.optimize.bisect's stopping rule).

    The reference calls scipy.optimize.bisect with its defaults
    (xtol=2e-12, rtol=8.88e-16, maxiter=100); this uses scipy when it is
    importable and otherwise the same halving with the same tolerances.
    """
    try:
        from scipy.optimize import bisect
        return bisect(f, a, b, args)
    except ImportError:
        pass
    xtol, rtol = 2e-12, 4 * np.finfo(float).eps
    fa, fb = f(a, *args), f(b, *args)
    if fa * fb > 0:
        raise ValueError("f(a) and f(b) must have different signs")
    if fa == 0:
        return a
    if fb == 0:
        return b
    dm = b - a
    for _ in range(100):
        dm *= 0.5
        xm = a + dm
        fm = f(xm, *args)
        if fm * fa >= 0:
            a = xm
        if fm == 0 or abs(dm) < xtol + rtol * abs(xm):
            return xm
    raise RuntimeError("bisection did not converge")


def dispersion_3d(zeta, v, omega, ds, dt, k):
    """Numerical dispersion of the 3-D Yee grid (Taflove & Hagness eq. 5.65)."""
    lhs = (sin(0.5 * dt * omega) / v / dt) ** 2
    rhs = sum((np.sin(0.5 * zeta * np.array(ds) * k) / ds) ** 2)
    return lhs - rhs


def dispersion_1d(ds, zeta, v, omega, dt, k):
    """1-D cell size matching the 3-D numerical wave number (eq. 5.67)."""
    lhs = sin(0.5 * omega * dt) / v / dt
    rhs = 0.5 * k * zeta if ds == 0 else sin(0.5 * k * zeta * ds) / ds
    return lhs - rhs


def incident_grid(src, space, geom_tree, cmplx=False):
    """The TEMz incident-field simulation of a TFSF source (gmes/source.py:579-651)."""
    from copy import deepcopy
    from .fdtd import TEMzFDTD
    from .geometry import Cartesian, DefaultMedium, Shell
    from .material import Cpml
    from .source import PointSource
    with np.errstate(invalid="ignore"):
        default = geom_tree.object_of_point((inf, inf, inf))[0]
        material = geom_tree.material_of_point((inf, inf, inf))[0]
    eps_inf, mu_inf = default.material.eps_inf, default.material.mu_inf
    v = 1 / sqrt(eps_inf * mu_inf)
    ds = tuple(space.dr)
    dt = space.dt
    omega = 2 * pi * src.src_time.freq
    zeta = _bisect(dispersion_3d, 0, 2, (v, omega, ds, dt, omega * src.k / v))
    delta = _bisect(dispersion_1d, 0, 2 * max(ds), (zeta, v, omega, dt, omega / v))
    pml = 50 * delta
    verts = []
    for x in (0.5 * src.size[0], -0.5 * src.size[0]):
        for y in (0.5 * src.size[1], -0.5 * src.size[1]):
            for z in (0.5 * src.size[2], -0.5 * src.size[2]):
                verts.append(src.center + (x, y, z))
    max_dist = max(abs(float(np.dot(src.k, p - src.center))) for p in verts)
    length = 2 * (max_dist + pml + 2 * delta)
    aux_space = Cartesian(size=(0, 0, length), resolution=1 / delta, parallel=False)
    geom = (DefaultMedium(material=material), Shell(material=Cpml(), thickness=pml))
    sources = (PointSource(src_time=deepcopy(src.src_time), component=const.Ex,
                           center=(0, 0, -max_dist - delta)),)
    return TEMzFDTD(aux_space, list(geom), list(sources), dt=space.dt,
                    bloch=(0, 0, 0) if cmplx else None, verbose=False)


def _coords(space, comp, axis, idx):
    """Space coordinates of indices ``idx`` of ``comp`` along ``axis``
    (the arithmetic of the scalar index_to_space methods)."""
    from .geometry import YEE_OFFSET
    off = YEE_OFFSET[comp.index][axis]
    idx = np.asarray(idx, np.intp)
    if off == 0:
        return idx * space.dr[axis] - space.half_size[axis]
    return (idx + off) * space.dr[axis] - space.half_size[axis]


def _axis_ok(comp, shape, axis, idx):
    """in_range() of gmes/geometry.py:751-812, one axis at a time."""
    c = comp.index
    own = c % 3
    if c < 3:
        hi = shape[axis] if axis == own else shape[axis] - 1
        lo = 0
    else:
        hi = shape[axis]
        lo = 0 if axis == own else 1
    return (idx >= lo) & (idx < hi)


def transparent_points(src, comp, shape, space, geom_list, aux_space, aux_shapes):
    """Transparent points of component ``comp``: {flat offset: [(coef, r0, r1, sample), ...]}.

    Faces are listed in the reference's merge order (TransparentParam.merge,
    gmes/pw_source.py:134-150); ``sample`` is the flat offset into the
    incident grid's Hy (E points) or Ex (H points) array.  Each face is a
    box of points handled with array operations: its materials come from
    the same rasteriser as the class maps.
    """
    from .geometry import rasterize
    out = {}
    c = comp.index
    e_side = c < 3
    aux_comp = const.Hy if e_side else const.Ex
    aux_shape = aux_shapes[aux_comp.index]
    for cos_src, cos_axis, faces in FACES[comp]:
        vec = src.h_direction if cos_src == _H else src.e_direction
        unit = np.zeros(3)
        unit[cos_axis] = 1
        cosine = float(np.dot(vec, unit))
        if cosine == 0:
            continue
        for axis, side, idx_comp, shift, samp_comp, samp_off, sign in faces:
            if not 2 * space.half_size[axis] > space.dr[axis]:
                continue
            flip = np.ones(3)
            flip[axis] = -1
            if side == MINUS:
                low = src.center - src.half_size
                high = src.center + src.half_size * flip
            else:
                low = src.center - src.half_size * flip
                high = src.center + src.half_size
            lo = np.array(space.space_to_index(idx_comp, *low)) + shift
            hi = np.array(space.space_to_index(idx_comp, *high)) + 1 + shift
            rng = []
            for a in range(3):
                r = np.arange(lo[a], max(lo[a], hi[a]), dtype=np.intp)
                rng.append(r[_axis_ok(comp, shape, a, r)])
            if any(len(r) == 0 for r in rng):
                continue
            # materials of the points (material or, under a Compound, the one beneath)
            owner, under = rasterize(geom_list, [_coords(space, comp, a, rng[a])
                                                 for a in range(3)])
            pick = np.where(under >= 0, under, owner).ravel()
            vals = np.array([(g.material.eps_inf if e_side else g.material.mu_inf)
                             for g in geom_list])
            eps = vals[pick]
            d = space.dr[axis]
            amp = cosine * src.amp * 1.0
            coef = space.dt / (eps * d) * amp
            if sign < 0:
                coef = -coef
            # projected distance of the neighbouring sample point along k
            sx, sy, sz = (_coords(space, samp_comp, a, rng[a] + samp_off[a]) for a in range(3))
            P = np.stack(np.broadcast_arrays(sx[:, None, None], sy[None, :, None],
                                             sz[None, None, :]), axis=-1).reshape(-1, 3)
            diff = P - src.center
            z = np.array([np.dot(src.k, q) for q in diff])
            exact = np.array([aux_space.spc_to_exact_hy_idx(0, 0, v) if e_side else
                              aux_space.spc_to_exact_ex_idx(0, 0, v) for v in z])
            i0 = np.floor(exact).astype(np.intp)
            r1 = exact[:, 2] - np.floor(exact[:, 2])
            r0 = 1 - r1
            ok = ((i0 >= 0) & (i0 < np.array(aux_shape))).all(axis=1) & (i0[:, 2] + 1 <
                                                                        aux_shape[2])
            if not ok.all():
                raise ValueError("TFSF sample point outside the incident-field grid")
            flat_s = np.ravel_multi_index(i0.T, aux_shape)
            I, J, K = np.meshgrid(rng[0], rng[1], rng[2], indexing="ij")
            offs = ((I * shape[1] + J) * shape[2] + K).ravel()
            for q in range(len(offs)):
                faces_of = out.setdefault(int(offs[q]), {})
                faces_of[(axis, side)] = (float(coef[q]), float(r0[q]), float(r1[q]),
                                          int(flat_s[q]))
    return {off: list(f.values()) for off, f in out.items()}


def dt_over(space, eps, d):
    """dt / (eps * d), the reference's grouping."""
    return space.dt / (eps * d)
