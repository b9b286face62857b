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
from .material import (KIND_CPML, KIND_DCP, KIND_DCP_PLRC, KIND_DRUDE, KIND_DUMMY,
                       KIND_LORENTZ, KIND_UPML, ClassDesc, Cpml)

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
    if desc.kind == KIND_DCP_PLRC:
        return desc.ndrude + 2 * desc.ncp
    return 0


class Scene:
    """Everything the engine needs to advance one grid.

    Attributes: ``n`` (whole_field_size), ``active`` (tuple of active
    component classes, E first), ``dr``, ``half``, ``dt``, ``classes`` (list
    of 6 lists of ClassDesc; class 0 is always Dummy), ``pmls`` (list of PML
    material objects), ``sources`` (list of PointSourceSpec).

    Class maps: ``lut[c]`` maps (owner shape, underneath shape + 1) to a
    class id, and ``shapes`` holds the rasteriser records of the geometry
    list, so the engine can build the u8 class maps on the GPU
    (``gmes_rasterize``).  ``host_cls(c)`` builds the same map on the host
    (numpy); ``cls[c]`` caches it.
    """

    def __init__(self, n, active, dr, half, dt):
        self.n = tuple(int(v) for v in n)
        self.active = tuple(active)
        self.dr = tuple(float(v) for v in dr)
        self.half = tuple(float(v) for v in half)
        self.dt = float(dt)
        self.cls = [None] * 6
        self.lut = [None] * 6
        self.classes = [[] for _ in range(6)]
        self.pmls = []
        self.sources = []
        self.tfsf = None      # (incident Scene, [(comp, offset, faces)]) of a TFSF source
        self.cmplx = False    # complex fields with Bloch phases
        self.bloch_phase = np.zeros((6, 2, 2))
        self.shapes = None
        self._geom = None
        self._space = None

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
        return any(d.kind in (KIND_DRUDE, KIND_LORENTZ, KIND_DCP, KIND_DCP_PLRC)
                   for c in range(3) for d in self.classes[c])

    @property
    def cells(self):
        return int(np.prod(self.n))

    @property
    def device_raster(self):
        """True when the class maps can be built on the GPU."""
        return self.shapes is not None

    def pml_index(self, pml):
        for i, p in enumerate(self.pmls):
            if p is pml:
                return i
        self.pmls.append(pml)
        return len(self.pmls) - 1

    def host_cls(self, c):
        """u8 class map of component ``c`` rasterised on the host."""
        if self.cls[c] is None and (self.active_mask >> c) & 1:
            comp = next(a for a in self.active if a.index == c)
            shape = self.shape(c)
            coords = [self._space.axis_coords(comp, a, shape[a]) for a in range(3)]
            owner, under = rasterize(self._geom, coords)
            m = self.lut[c][owner.astype(np.intp), under.astype(np.intp) + 1]
            _edge_dummy(m, c)
            self.cls[c] = np.ascontiguousarray(m, np.uint8)
        return self.cls[c]

    def counts(self, c):
        """Points per class of component ``c`` (the reference's idx_size())."""
        m = self.host_cls(c)
        if m is None:
            return {}
        cnt = np.bincount(m.ravel(), minlength=len(self.classes[c]))
        return {i: int(v) for i, v in enumerate(cnt) if v}


def _edge_dummy(cls, c):
    """Mark the ghost planes of component ``c`` as Dummy (class 0)."""
    own = c % 3
    for ax in ((own + 1) % 3, (own + 2) % 3):
        sl = [slice(None)] * 3
        sl[ax] = -1 if c < 3 else 0
        cls[tuple(sl)] = 0


def _class_table(geom_list, comp, scene):
    """Class descriptors and the (owner, under + 1) -> class id table of one component.

    Every possible pair is numbered: a non-compound owner with under = -1,
    a compound owner (a PML) with each earlier shape as underneath
    (src/pygeom.pyx:425-441).  Distinct descriptors share an id.
    """
    G = len(geom_list)
    descs = [ClassDesc(KIND_DUMMY, 1.0)]
    keys = {}
    lut = np.zeros((G, G + 1), np.uint8)
    for m in range(G):
        mat = geom_list[m].material
        compound = getattr(mat, "compound", False) and m > 0
        for u in (range(m) if compound else (-1,)):
            desc = mat.engine_class(comp, geom_list[u].material if u >= 0 else None)
            k = desc.key()
            if k not in keys:
                if len(descs) >= MAX_CLASSES:
                    raise ValueError(f"more than {MAX_CLASSES - 1} material classes "
                                     f"on component {comp.__name__}")
                keys[k] = len(descs)
                descs.append(desc)
                if desc.pml is not None:
                    scene.pml_index(desc.pml)
            lut[m, u + 1] = keys[k]
    return descs, lut


def bloch_phases(space, scene, bloch):
    """Phase factor of each ghost copy (gmes/fdtd.py:811-1097): the E ghost
    plane (last) along axis a receives exp(1j k_a (x_last - x_0)) times plane
    0, the H ghost plane (0) exp(1j k_a (x_0 - x_last)) times the last plane;
    rows (component, h) with h = 0 for axis own+1 and 1 for own+2."""
    from cmath import exp as cexp
    ph = np.zeros((6, 2, 2))
    for comp in scene.active:
        c = comp.index
        own = c % 3
        sh = scene.shape(c)
        for h, a in enumerate(((own + 1) % 3, (own + 2) % 3)):
            last = [0, 0, 0]
            last[a] = sh[a] - 1
            x0 = space.index_to_space(comp, 0, 0, 0)[a]
            xl = space.index_to_space(comp, *last)[a]
            dest, src = (xl, x0) if c < 3 else (x0, xl)
            p = cexp(1j * bloch[a] * (dest - src))
            ph[c, h] = (p.real, p.imag)
    return ph


def compile_scene(space, geom_list, e_comps, h_comps, src_list, geom_tree, dt, bloch=None):
    """Class tables, rasteriser records and point sources of a scene.

    No per-point work happens here: the class maps are built on the GPU by
    the engine, or on the host on demand (``Scene.host_cls``).
    """
    active = tuple(e_comps) + tuple(h_comps)
    scene = Scene(space.whole_field_size, active, space.dr, space.half_size, dt)
    scene._geom = list(geom_list)
    scene._space = space
    if bloch is not None:
        scene.cmplx = True
        scene.bloch_phase = bloch_phases(space, scene, bloch)
    for comp in active:
        descs, lut = _class_table(geom_list, comp, scene)
        scene.classes[comp.index] = descs
        scene.lut[comp.index] = lut
    try:
        recs = [g.shape_record() for g in geom_list]
        scene.shapes = recs if 1 <= len(recs) <= 255 else None
    except NotImplementedError:
        scene.shapes = None
    # point sources: a later source at the same point replaces an earlier
    # one, as PwSource.attach/merge do (gmes/pw_source.py:25-36)
    specs = {}
    from .source import TotalFieldScatteredField
    for src in src_list:
        if isinstance(src, TotalFieldScatteredField):
            if scene.tfsf is not None:
                raise NotImplementedError("one TotalFieldScatteredField source per simulation")
            scene.tfsf = _compile_tfsf(src, scene, space, geom_tree, active)
            continue
        if not hasattr(src, "resolve"):
            raise NotImplementedError(f"{type(src).__name__} is not supported by the GPU engine")
        for comp in active:
            spec = src.resolve(comp, scene.shape(comp.index), space, geom_tree)
            if spec is not None:
                specs[(comp.index, spec.idx)] = spec
    scene.sources = list(specs.values())
    return scene


def _compile_tfsf(src, scene, space, geom_tree, active):
    """Incident-field scene and transparent points of a TFSF source."""
    from .tfsf import transparent_points
    aux = src.aux_fdtd.compile()
    aux_shapes = [aux.shape(c) for c in range(6)]
    points = []
    for comp in active:
        c = comp.index
        sh = scene.shape(c)
        for off, faces in transparent_points(src, comp, sh, space, scene._geom,
                                             src.aux_fdtd.space, aux_shapes).items():
            points.append((c, int(off), faces))
    return aux, points


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

    Returns (nsteps, 2, nsrc) float64 (complex128 for a complex scene):
    [s, 0] at n = n0 + s + 0.5 (E
    half), [s, 1] at n = n0 + s + 1 (H half), matching TimeStep.half_step_up
    (gmes/fdtd.py:47-50) and the time tag dt * n of gmes/pw_source.py:80.
    """
    ns = len(scene.sources)
    out = np.zeros((nsteps, 2, ns), np.complex128 if scene.cmplx else np.float64)
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
