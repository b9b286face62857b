"""Compile a GMES scene into the engine's grid description.

Replaces the reference's per-point material mapping (FDTD.init_material_*,
gmes/fdtd.py:353-503: one Python iteration, one tree lookup and one new C++
object per Yee point) by array operations: every component's points are
rasterised at once (``geometry.rasterize``), each distinct
(material, underneath material) pair becomes one update *class*, and the
result is a u8 class map per component plus a class table.  The Dummy edge
rule of gmes/fdtd.py:365,386,407,428,449,470 is applied on the map.

The compiled ``Scene`` is plain numpy: the CUDA engine and the CPU oracle
consume the same object.
"""

import numpy as np

from . import constant as const
from .geometry import rasterize
from .material import (KIND_CPML, KIND_DCP, KIND_DRUDE, KIND_DUMMY, KIND_LORENTZ,
                       KIND_UPML, ClassDesc, Cpml)

MAX_CLASSES = 256


def naux_of(desc):
    """State slots one point of this class needs (include/gmes_gb300.h)."""
    if desc.kind == KIND_CPML:
        return 2
    if desc.kind == KIND_UPML:
        return 1
    if desc.kind in (KIND_DRUDE, KIND_LORENTZ):
        return 2 * desc.ndrude
    if desc.kind == KIND_DCP:
        return 1 + 2 * desc.ndrude + 2 * desc.ncp
    return 0


class Scene:
    """Everything the engine needs to advance one grid.

    Attributes: ``n`` (whole_field_size), ``active`` (tuple of active
    component classes, E first), ``dr``, ``half``, ``dt``, ``cls`` (list of 6
    uint8 arrays or None), ``classes`` (list of 6 lists of ClassDesc; class
    0 is always Dummy), ``pmls`` (list of PML material objects), ``sources``
    (list of PointSourceSpec).
    """

    def __init__(self, n, active, dr, half, dt):
        self.n = tuple(int(v) for v in n)
        self.active = tuple(active)
        self.dr = tuple(float(v) for v in dr)
        self.half = tuple(float(v) for v in half)
        self.dt = float(dt)
        self.cls = [None] * 6
        self.classes = [[] for _ in range(6)]
        self.pmls = []
        self.sources = []

    @property
    def active_mask(self):
        m = 0
        for c in self.active:
            m |= 1 << c.index
        return m

    def shape(self, c):
        """Array shape of component index ``c``."""
        if not (self.active_mask >> c) & 1:
            return (1, 1, 1)
        own = c % 3
        return tuple(self.n[a] if a == own else self.n[a] + 1 for a in range(3))

    def naux(self, c):
        return max([naux_of(d) for d in self.classes[c]] + [0])

    @property
    def dispersive(self):
        return any(d.kind in (KIND_DRUDE, KIND_LORENTZ, KIND_DCP)
                   for c in range(3) for d in self.classes[c])

    @property
    def cells(self):
        return int(np.prod(self.n))

    def pml_index(self, pml):
        for i, p in enumerate(self.pmls):
            if p is pml:
                return i
        self.pmls.append(pml)
        return len(self.pmls) - 1

    def counts(self, c):
        """Points per class of component ``c`` (the reference's idx_size())."""
        if self.cls[c] is None:
            return {}
        cnt = np.bincount(self.cls[c].ravel(), minlength=len(self.classes[c]))
        return {i: int(v) for i, v in enumerate(cnt) if v}


def _edge_dummy(cls, c):
    """Mark the ghost planes of component ``c`` as Dummy (class 0)."""
    own = c % 3
    for ax in ((own + 1) % 3, (own + 2) % 3):
        sl = [slice(None)] * 3
        sl[ax] = -1 if c < 3 else 0
        cls[tuple(sl)] = 0


def compile_scene(space, geom_list, e_comps, h_comps, src_list, geom_tree, dt):
    active = tuple(e_comps) + tuple(h_comps)
    scene = Scene(space.whole_field_size, active, space.dr, space.half_size, dt)
    G = len(geom_list)
    for comp in active:
        c = comp.index
        shape = scene.shape(c)
        coords = [space.axis_coords(comp, a, shape[a]) for a in range(3)]
        owner, under = rasterize(geom_list, coords)
        code = owner.astype(np.int32) * (G + 1) + (under.astype(np.int32) + 1)
        present = np.zeros(G * (G + 1) + G + 1, bool)
        present[code.ravel()] = True
        lut = np.zeros(len(present), np.uint8)
        descs = [ClassDesc(KIND_DUMMY, 1.0)]
        keys = {}
        for cc in np.nonzero(present)[0]:
            m, u = divmod(int(cc), G + 1)
            u -= 1
            mat = geom_list[m].material
            underneath = geom_list[u].material if u >= 0 else None
            desc = mat.engine_class(comp, underneath)
            if desc.pml is not None:
                scene.pml_index(desc.pml)
            k = desc.key()
            if k not in keys:
                if len(descs) >= MAX_CLASSES:
                    raise ValueError(f"more than {MAX_CLASSES - 1} material classes "
                                     f"on component {comp.__name__}")
                keys[k] = len(descs)
                descs.append(desc)
            lut[cc] = keys[k]
        cls = lut[code]
        _edge_dummy(cls, c)
        scene.cls[c] = np.ascontiguousarray(cls)
        scene.classes[c] = descs
    # point sources: a later source at the same point replaces an earlier
    # one, as PwSource.attach/merge do (gmes/pw_source.py:25-36)
    specs = {}
    for src in src_list:
        if not hasattr(src, "resolve"):
            raise NotImplementedError(f"{type(src).__name__} is not supported by the GPU engine")
        for comp in active:
            spec = src.resolve(comp, scene.shape(comp.index), space, geom_tree)
            if spec is not None:
                specs[(comp.index, spec.idx)] = spec
    scene.sources = list(specs.values())
    return scene


def class_arrays(scene):
    """Flatten the class table into (gmes_class_desc rows, parameter pool, pml rows).

    Returns python lists of dicts/floats; ``engine`` converts them to the C
    structures and ``oracle`` reads them directly.
    """
    rows, pool = [], []
    for c in range(6):
        for d in scene.classes[c]:
            pml = scene.pml_index(d.pml) if d.pml is not None else -1
            rows.append(dict(kind=d.kind, pml=pml, npole=d.ndrude, ncp=d.ncp,
                             param_off=len(pool), nparam=len(d.params), eps=d.eps))
            pool.extend(d.params)
    pmls = []
    for p in scene.pmls:
        pmls.append(dict(
            kind=KIND_CPML if isinstance(p, Cpml) else KIND_UPML,
            sigma_max=[float(v) for v in p.sigma_max], m=p.m, kappa_max=p.kappa_max,
            m_a=getattr(p, "m_a", 0.0), a_max=getattr(p, "a_max", 0.0), d=float(p.d),
            center=[float(v) for v in p.center], half_size=[float(v) for v in p.half_size]))
    return rows, pool, pmls


def source_values(scene, dt, n0, nsteps):
    """Source values for steps whose first E half-step is at time step n0 + 0.5.

    Returns float64 array (nsteps, 2, nsrc): [s, 0] at n = n0 + s + 0.5 (E
    half), [s, 1] at n = n0 + s + 1 (H half), matching TimeStep.half_step_up
    (gmes/fdtd.py:47-50) and the time tag dt * n of gmes/pw_source.py:80.
    """
    ns = len(scene.sources)
    out = np.zeros((nsteps, 2, ns), np.float64)
    n = float(n0)
    for s in range(nsteps):
        n += 0.5
        for q, spec in enumerate(scene.sources):
            if spec.comp.index < 3:
                out[s, 0, q] = spec.value(dt, n)
        n += 0.5
        for q, spec in enumerate(scene.sources):
            if spec.comp.index >= 3:
                out[s, 1, q] = spec.value(dt, n)
    return out


def source_offsets(scene):
    """(comp, mode, linear offset) of every source."""
    out = []
    for spec in scene.sources:
        c = spec.comp.index
        sh = scene.shape(c)
        off = (spec.idx[0] * sh[1] + spec.idx[1]) * sh[2] + spec.idx[2]
        out.append((c, spec.mode, int(off)))
    return out
