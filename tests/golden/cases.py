"""Scene builders shared by the golden-vector generator and the tests.

Each builder takes a module exposing GMES's public API -- the reference
``gmes`` package (fixture generation in the build container) or
``gmes_gb300`` (tests) -- and returns ``(sim, nsteps)``.  Geometry and
parameters are seeded so both sides build exactly the same scene.
"""

import numpy as np


def tmz_regression(g):
    """tests/test_fdtd.py:55-79 of the reference: TMz + CPML + Continuous Ez, 5 steps."""
    space = g.Cartesian(size=(2, 2, 0), resolution=5)
    geometry = [g.DefaultMedium(material=g.Dielectric()), g.Shell(material=g.Cpml())]
    sources = [g.PointSource(src_time=g.Continuous(freq=0.8, width=0.5), center=(0, 0, 0),
                             component=g.Ez)]
    return g.TMzFDTD(space, geometry, sources, verbose=False), 5


def air2d(g):
    """examples/air2d.py: 200x200 TMz, vacuum + 20-cell CPML, Continuous(0.8) Ez, to t = 10."""
    space = g.Cartesian(size=(10, 10, 0), resolution=20)
    geometry = [g.DefaultMedium(material=g.Dielectric()), g.Shell(material=g.Cpml())]
    sources = [g.PointSource(src_time=g.Continuous(freq=0.8), center=(0, 0, 0), component=g.Ez)]
    return g.TMzFDTD(space, geometry, sources, verbose=False), 286


def random_objects(g, rng, n, half, rmin, rmax, dx, eps_lo=1.0, eps_hi=12.0):
    """Seeded spheres and blocks (50/50), radius / half-edge in [rmin, rmax] cells."""
    objs = []
    for _ in range(n):
        r = rng.uniform(rmin, rmax) * dx
        center = tuple(float(v) for v in rng.uniform(-half, half, 3))
        eps = float(rng.uniform(eps_lo, eps_hi))
        if rng.uniform() < 0.5:
            objs.append(g.Sphere(material=g.Dielectric(eps_inf=eps), center=center, radius=r))
        else:
            objs.append(g.Block(material=g.Dielectric(eps_inf=eps), center=center,
                                size=(2 * r, 2 * r, 2 * r)))
    return objs


def dielectric3d(g, size=2.0, res=10, pml_cells=4, nobj=5, seed=0, steps=150, kappa_max=None):
    """Small instance of the 256^3 benchmark scene: seeded dielectric spheres and
    blocks, CPML on all faces, Bandpass Ex point source.  ``kappa_max``: the
    CPML's kappa grading maximum (None: the default, 1)."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / res
    inner = size / 2 - pml_cells * dx
    space = g.Cartesian(size=(size, size, size), resolution=res)
    geometry = [g.DefaultMedium(material=g.Dielectric())]
    geometry += random_objects(g, rng, nobj, inner * 0.7, 2, 5, dx)
    cpml = g.Cpml() if kappa_max is None else g.Cpml(kappa_max=kappa_max)
    geometry.append(g.Shell(material=cpml, thickness=pml_cells * dx))
    sources = [g.PointSource(src_time=g.Bandpass(freq=0.5, fwidth=1.0), center=(0, 0, 0),
                             component=g.Ex)]
    return g.FDTD(space, geometry, sources, verbose=False), steps


def dispersive3d(g, size=2.0, res=10, pml_cells=4, seed=1, steps=150, courant_ratio=0.6):
    """Small instance of the 192^3 dispersive scene: eps = 2.25 background, a
    Drude sphere, a Lorentz slab, a DCP-ADE sphere, UPML on all faces.

    The reference derives dt from the background medium (gmes/fdtd.py:132-147):
    with eps = 2.25 the default Courant ratio 0.99 exceeds the stability limit
    of every eps < 2.25 region (eps_inf = 1 metal), so the scene runs at
    courant_ratio 0.6 (< 0.99 / 1.5)."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / res
    space = g.Cartesian(size=(size, size, size), resolution=res)
    cps = tuple(g.CriticalPoint(amp=float(rng.uniform(0.5, 2.0)),
                                phi=float(rng.uniform(-1.5, 1.5)),
                                omega=float(rng.uniform(2.0, 5.0)),
                                gamma=float(rng.uniform(0.2, 1.0))) for _ in range(2))
    geometry = [
        g.DefaultMedium(material=g.Dielectric(eps_inf=2.25)),
        g.Sphere(material=g.Drude(eps_inf=1, dps=(g.DrudePole(omega=9.0, gamma=0.07),)),
                 center=(-0.35, -0.3, 0.2), radius=0.3),
        g.Block(material=g.Lorentz(lps=(g.LorentzPole(amp=2.0, omega=3.0, gamma=0.1),)),
                center=(0.3, 0.0, 0.0), size=(0.2, 1.2, 1.2)),
        g.Sphere(material=g.DcpAde(eps_inf=1.1, dps=(g.DrudePole(omega=7.0, gamma=0.2),),
                                   cps=cps), center=(-0.2, 0.35, -0.3), radius=0.25),
        g.Shell(material=g.Upml(), thickness=pml_cells * dx),
    ]
    sources = [g.PointSource(src_time=g.Bandpass(freq=0.5, fwidth=1.0), center=(0, 0, 0),
                             component=g.Ez)]
    return g.FDTD(space, geometry, sources, verbose=False,
                  courant_ratio=courant_ratio), steps


def drude2d(g, steps=120):
    """TMz Drude medium (omega 1, gamma 0.1) with a dielectric slab running into the
    CPML (the PML's underneath eps differs from the background)."""
    space = g.Cartesian(size=(3, 3, 0), resolution=12)
    geometry = [
        g.DefaultMedium(material=g.Drude(dps=(g.DrudePole(omega=1.0, gamma=0.1),))),
        g.Block(material=g.Dielectric(eps_inf=4.0), center=(0, 0.6, 0), size=(10, 0.5, 1)),
        g.Shell(material=g.Cpml(), thickness=0.5),
    ]
    sources = [g.PointSource(src_time=g.Bandpass(freq=0.8, fwidth=1.0), center=(0.1, -0.2, 0),
                             component=g.Ez)]
    return g.TMzFDTD(space, geometry, sources, verbose=False), steps


def tez_upml_currents(g, steps=100):
    """TEz (Ex, Ey, Hz) with UPML, an electric-current (Jx) and a magnetic-current
    (Mz) source, DifferentiatedGaussian and Continuous time functions."""
    space = g.Cartesian(size=(2.5, 2, 0), resolution=12)
    geometry = [
        g.DefaultMedium(material=g.Dielectric(eps_inf=1.5, mu_inf=1.2)),
        g.Cylinder(material=g.Dielectric(eps_inf=6.0), center=(0.3, 0.1, 0), radius=0.3,
                   height=2),
        g.Shell(material=g.Upml(), thickness=0.4),
    ]
    sources = [
        g.PointSource(src_time=g.DifferentiatedGaussian(tw=0.3, t0=1.0), center=(-0.2, 0, 0),
                      component=g.Jx, amp=2.0),
        g.PointSource(src_time=g.Continuous(freq=1.2, width=0.8), center=(0.2, -0.3, 0),
                      component=g.Mz),
    ]
    return g.TEzFDTD(space, geometry, sources, verbose=False), steps


def tmx_cpml_hard(g, steps=80):
    """TMx (Ex; Hy, Hz), x collapsed, CPML, an Ellipsoid, a hard Hy source."""
    space = g.Cartesian(size=(0, 2.4, 2), resolution=10)
    geometry = [
        g.DefaultMedium(material=g.Dielectric()),
        g.Ellipsoid(material=g.Dielectric(eps_inf=3.0), center=(0, 0.2, -0.1),
                    size=(1, 0.8, 0.5)),
        g.Shell(material=g.Cpml(), thickness=0.5),
    ]
    sources = [
        g.PointSource(src_time=g.Bandpass(freq=1.0, fwidth=1.5), center=(0, -0.3, 0.2),
                      component=g.Ex),
        g.PointSource(src_time=g.Continuous(freq=0.7, width=0.5), center=(0, 0.4, 0.1),
                      component=g.Hy, amp=0.5),
    ]
    return g.TMxFDTD(space, geometry, sources, verbose=False), steps


def tfsf2d(g, steps=120):
    """TMz plane wave (+x, Ez-polarised) through a TFSF box around a dielectric
    sphere, CPML; the incident-field grid is the reference's matched-dispersion
    TEMz aux FDTD (gmes/source.py:579-651)."""
    space = g.Cartesian(size=(4, 4, 0), resolution=10)
    geometry = [g.DefaultMedium(material=g.Dielectric()),
                g.Sphere(material=g.Dielectric(eps_inf=4.0), center=(0.3, 0, 0), radius=0.5),
                g.Shell(material=g.Cpml(), thickness=0.6)]
    sources = [g.TotalFieldScatteredField(src_time=g.Bandpass(freq=1.0, fwidth=1.0, s=3),
                                          center=(0, 0, 0), size=(2.0, 2.0, 0),
                                          direction=(1, 0, 0), polarization=(0, 0, 1))]
    return g.TMzFDTD(space, geometry, sources, verbose=False), steps


def tfsf3d(g, steps=60):
    """3-D oblique plane wave through a TFSF box in an eps = 1.5 background
    around a dielectric sphere, CPML on all faces."""
    import numpy as np
    space = g.Cartesian(size=(2.4, 2.4, 2.4), resolution=10)
    geometry = [g.DefaultMedium(material=g.Dielectric(eps_inf=1.5)),
                g.Sphere(material=g.Dielectric(eps_inf=4.0), center=(0.1, 0, 0), radius=0.3),
                g.Shell(material=g.Cpml(), thickness=0.4)]
    k = np.array((1.0, 0.5, 0.2))
    pol = tuple(float(v) for v in np.cross(k / np.linalg.norm(k), (0, 0, 1)))
    sources = [g.TotalFieldScatteredField(src_time=g.Bandpass(freq=1.0, fwidth=1.0, s=3),
                                          center=(0, 0, 0), size=(1.2, 1.2, 1.2),
                                          direction=tuple(k), polarization=pol)]
    return g.FDTD(space, geometry, sources, verbose=False), steps


def bloch2d(g, steps=120):
    """TMz with a Bloch boundary (complex fields, phase-shifted ghost copies),
    no PML: a dielectric cylinder and a complex Continuous Ez source."""
    space = g.Cartesian(size=(3, 3, 0), resolution=10)
    geometry = [g.DefaultMedium(material=g.Dielectric()),
                g.Sphere(material=g.Dielectric(eps_inf=3.0), center=(0.3, -0.2, 0), radius=0.6)]
    sources = [g.PointSource(src_time=g.Continuous(freq=0.9, width=1.0), center=(-0.4, 0.1, 0),
                             component=g.Ez)]
    return g.TMzFDTD(space, geometry, sources, bloch=(0.5, 0.3, 0.0), verbose=False), steps


def bloch3d(g, steps=60):
    """3-D complex fields with a Bloch vector, a Drude sphere, a dielectric
    block, CPML on all faces and a Bandpass Ex source."""
    space = g.Cartesian(size=(1.6, 1.6, 1.6), resolution=10)
    geometry = [g.DefaultMedium(material=g.Dielectric()),
                g.Sphere(material=g.Drude(eps_inf=1, dps=(g.DrudePole(omega=3.0, gamma=0.3),)),
                         center=(0.2, 0.1, 0), radius=0.3),
                g.Block(material=g.Dielectric(eps_inf=2.5), center=(-0.3, 0, 0.2),
                        size=(0.3, 0.8, 0.3)),
                g.Shell(material=g.Cpml(), thickness=0.3)]
    sources = [g.PointSource(src_time=g.Bandpass(freq=1.0, fwidth=1.0, s=3), center=(0, 0, 0),
                             component=g.Ex)]
    return g.FDTD(space, geometry, sources, bloch=(0.4, 0.2, 0.1), verbose=False), steps


def bloch_tfsf2d(g, steps=100):
    """Complex TMz with a TFSF plane wave (the incident-field grid is complex
    too) and a Bloch vector along y."""
    space = g.Cartesian(size=(4, 4, 0), resolution=10)
    geometry = [g.DefaultMedium(material=g.Dielectric()),
                g.Sphere(material=g.Dielectric(eps_inf=4.0), center=(0.3, 0, 0), radius=0.5),
                g.Shell(material=g.Cpml(), thickness=0.6)]
    sources = [g.TotalFieldScatteredField(src_time=g.Bandpass(freq=1.0, fwidth=1.0, s=3),
                                          center=(0, 0, 0), size=(2.0, 2.0, 0),
                                          direction=(1, 0, 0), polarization=(0, 0, 1))]
    return g.TMzFDTD(space, geometry, sources, bloch=(0.0, 0.4, 0.0), verbose=False), steps


def dcp_plrc3d(g, steps=80, courant_ratio=0.6):
    """DcpPlrc (PLRC form) and DcpRc (RC form) Drude-critical-points media
    (src/pw_dcp.hh:406-746) in an eps = 2.25 background, CPML, Bandpass Ez."""
    rng = np.random.default_rng(3)
    cps = tuple(g.CriticalPoint(amp=float(rng.uniform(0.5, 2.0)),
                                phi=float(rng.uniform(-1.5, 1.5)),
                                omega=float(rng.uniform(2.0, 5.0)),
                                gamma=float(rng.uniform(0.2, 1.0))) for _ in range(2))
    space = g.Cartesian(size=(2.0, 2.0, 2.0), resolution=10)
    geometry = [
        g.DefaultMedium(material=g.Dielectric(eps_inf=2.25)),
        g.Sphere(material=g.DcpPlrc(eps_inf=1.1, dps=(g.DrudePole(omega=7.0, gamma=0.2),),
                                    cps=cps), center=(-0.25, 0.2, 0.1), radius=0.35),
        g.Block(material=g.DcpRc(eps_inf=1.5, sigma=0.1,
                                 dps=(g.DrudePole(omega=4.0, gamma=0.5),), cps=cps[:1]),
                center=(0.3, -0.2, -0.1), size=(0.4, 0.5, 0.6)),
        g.Shell(material=g.Cpml(), thickness=0.4),
    ]
    sources = [g.PointSource(src_time=g.Bandpass(freq=0.8, fwidth=1.0, s=3), center=(0, 0, 0),
                             component=g.Ez)]
    return g.FDTD(space, geometry, sources, verbose=False, courant_ratio=courant_ratio), steps


def dcp_plrc_bloch2d(g, steps=100):
    """Complex TMz with a Bloch vector and a DcpPlrc cylinder (the PLRC
    accumulators of the real and imaginary parts are separate)."""
    space = g.Cartesian(size=(3, 3, 0), resolution=10)
    cps = (g.CriticalPoint(amp=1.2, phi=0.4, omega=3.0, gamma=0.5),)
    geometry = [g.DefaultMedium(material=g.Dielectric()),
                g.Sphere(material=g.DcpPlrc(eps_inf=1.5, dps=(g.DrudePole(omega=5.0, gamma=0.3),),
                                            cps=cps), center=(0.2, -0.1, 0), radius=0.6)]
    sources = [g.PointSource(src_time=g.Continuous(freq=0.7, width=1.0), center=(-0.5, 0.2, 0),
                             component=g.Ez)]
    return g.TMzFDTD(space, geometry, sources, bloch=(0.3, -0.2, 0.0), verbose=False), steps


CASES = {
    "tmz_regression": tmz_regression,
    "air2d": air2d,
    "dielectric3d": dielectric3d,
    "dispersive3d": dispersive3d,
    "drude2d": drude2d,
    "tez_upml_currents": tez_upml_currents,
    "tmx_cpml_hard": tmx_cpml_hard,
    "tfsf2d": tfsf2d,
    "tfsf3d": tfsf3d,
    "bloch2d": bloch2d,
    "bloch3d": bloch3d,
    "bloch_tfsf2d": bloch_tfsf2d,
    "dcp_plrc3d": dcp_plrc3d,
    "dcp_plrc_bloch2d": dcp_plrc_bloch2d,
}

# ---------------------------------------------------------------------------
# Point-wise updaters (the reference's gmes.pw_material objects)
# ---------------------------------------------------------------------------
PW_MODELS = ("Dummy", "Const", "Dielectric", "Upml", "Cpml", "Drude", "Lorentz", "DcpAde",
             "DcpPlrc", "DcpRc")
PW_COMPS = ("ex", "ey", "ez", "hx", "hy", "hz")
PW_POINTS = ((1, 1, 1), (2, 1, 2), (1, 2, 1))
PW_SHAPE = (4, 4, 4)
PW_STEPS = 3


def pw_material(g, model):
    """A material of each point-wise model, initialised as FDTD.init would."""
    space = g.Cartesian((0, 0, 0))
    space.dt = 0.35
    rng = np.random.default_rng(5)
    cps = tuple(g.CriticalPoint(amp=float(rng.uniform(0.5, 2.0)), phi=float(rng.uniform(-1, 1)),
                                omega=float(rng.uniform(2.0, 5.0)),
                                gamma=float(rng.uniform(0.2, 1.0))) for _ in range(2))
    if model == "Dummy":
        m = g.Dummy(eps_inf=2.0, mu_inf=1.5)
    elif model == "Const":
        m = g.Const(value=0.75, eps_inf=2.5, mu_inf=1.25)
    elif model == "Dielectric":
        m = g.Dielectric(eps_inf=2.5, mu_inf=1.25)
    elif model in ("Upml", "Cpml"):
        m = g.Upml() if model == "Upml" else g.Cpml()
        m.init(space, ((0, 0, 0), (1.0, 1.0, 1.0), 0.6))
        return m
    elif model == "Drude":
        m = g.Drude(eps_inf=1.5, sigma=0.05, dps=(g.DrudePole(omega=3.0, gamma=0.3),
                                                 g.DrudePole(omega=1.0, gamma=0.1)))
    elif model == "Lorentz":
        m = g.Lorentz(eps_inf=1.2, lps=(g.LorentzPole(amp=2.0, omega=3.0, gamma=0.1),))
    elif model == "DcpAde":
        m = g.DcpAde(eps_inf=1.1, dps=(g.DrudePole(omega=7.0, gamma=0.2),), cps=cps)
    elif model == "DcpPlrc":
        m = g.DcpPlrc(eps_inf=1.1, dps=(g.DrudePole(omega=7.0, gamma=0.2),), cps=cps)
    else:
        m = g.DcpRc(eps_inf=1.3, sigma=0.1, dps=(g.DrudePole(omega=4.0, gamma=0.5),),
                    cps=cps[:1])
    m.init(space)
    return m


def pw_updater(g, model, comp, cmplx):
    """An updater with PW_POINTS attached (merged one point at a time)."""
    m = pw_material(g, model)
    get = getattr(m, "get_pw_material_" + comp)
    upd = None
    for q, idx in enumerate(PW_POINTS):
        coords = (0.55 + 0.1 * q, -0.7 + 0.05 * q, 0.8 - 0.1 * q)
        u = get(idx, coords, cmplx=cmplx)
        upd = u if upd is None else upd.merge(u)
    return upd


def pw_inputs(model, comp, cmplx, step):
    """Seeded inplace, in1, in2 arrays of one update_all call."""
    seed = (PW_MODELS.index(model) * 6 + PW_COMPS.index(comp)) * 2 + int(cmplx)
    rng = np.random.default_rng(1000 + 10 * seed + step)

    def arr():
        a = rng.standard_normal(PW_SHAPE)
        if cmplx:
            a = a + 1j * rng.standard_normal(PW_SHAPE)
        return np.ascontiguousarray(a)
    return arr(), arr(), arr()


def pw_run(g, model, comp, cmplx):
    """The target array after each of PW_STEPS update_all calls (state carried)."""
    upd = pw_updater(g, model, comp, cmplx)
    target = pw_inputs(model, comp, cmplx, 0)[0]
    out = []
    for step in range(PW_STEPS):
        _, in1, in2 = pw_inputs(model, comp, cmplx, step)
        upd.update_all(target, in1, in2, 0.4, 0.3, 0.35, step)
        out.append(target.copy())
    return np.stack(out)


# Cases whose golden file stores only Ez in full (and checksums of the rest)
# to keep the fixture small.
# Scenes pinned for the CPU oracle only (their GPU counterparts compare the
# engine with the oracle at other sizes): a CPML with kappa_max = 5, so that
# the curl terms inside the slabs are scaled by 1 / kappa.
ORACLE_CASES = {
    "cpml_kappa3d": lambda g: dielectric3d(g, kappa_max=5.0, steps=120),
}

SUMMARY_ONLY = {"air2d": ("ez",)}

COMP_NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")
