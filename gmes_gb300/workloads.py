"""Synthetic benchmark scenes (seeded), built through the public API.

The reference publishes no benchmark suite for these workloads; each scene
below is generated from a seed with the shapes, sizes and parameter
distributions of the benchmark configurations:

* ``air2d``     2-D TMz 200x200, vacuum, 20-cell CPML, Continuous(0.8) Ez
                point source, 286 steps (= examples/air2d.py to t = 10).
* ``cube``      3-D N^3 (default 256^3), 24 seeded dielectric spheres and
                blocks, radius / half-edge 8-32 cells, eps in [1, 12],
                10-cell CPML, Bandpass(0.5, 0.2) Ex point source, 1000 steps.
* ``dispersive`` 3-D N^3 (default 192^3) in eps = 2.25: a 4x4 lattice of
                Drude spheres (omega_p 9, gamma 0.07, radius 10-20 cells), a
                Lorentz slab (2.0, 3.0, 0.1), a DCP-ADE sphere (1 Drude term +
                2 seeded critical points), 12-cell UPML, a TFSF plane wave
                (+z, x-polarised, Bandpass(0.5, 0.2)), 2000 steps.
* ``design2d``  2-D TMz N^2 (default 512^2) differentiation scene: vacuum,
                20-cell CPML, an Ez-polarised line source (a column of Jz
                point sources, Bandpass(0.5, 0.5)) left of a 64x64-point
                design region, an 8x8 monitor patch right of it, 2000 steps,
                a batch of seeded designs with eps uniform in [1, 12].
"""

import numpy as np

from . import (Bandpass, Block, Cartesian, Continuous, Cpml, CriticalPoint, DcpAde,
               DefaultMedium, Dielectric, Drude, DrudePole, Ex, Ez, FDTD, Jz, Lorentz,
               LorentzPole, PointSource, Shell, Sphere, TMzFDTD, TotalFieldScatteredField, Upml)


def air2d(precision="fp64", verbose=False):
    space = Cartesian(size=(10, 10, 0), resolution=20)
    geom = [DefaultMedium(material=Dielectric()), Shell(material=Cpml())]
    src = [PointSource(src_time=Continuous(freq=0.8), center=(0, 0, 0), component=Ez)]
    return TMzFDTD(space, geom, src, verbose=verbose, precision=precision), 286


def cube(n=256, nobj=24, seed=0, pml_cells=10, precision="fp64", verbose=False, res=10,
         src_time=None, kappa_max=1.0):
    """The 3-D dielectric + CPML benchmark scene on an n^3 grid (resolution 10).

    ``src_time`` replaces the Bandpass(0.5, 0.2) pulse (peak at t = 50);
    ``kappa_max`` is the CPML's kappa grading maximum (1: the default CPML).
    """
    rng = np.random.default_rng(seed)
    dx = 1.0 / res
    size = n * dx
    inner = size / 2 - pml_cells * dx
    geom = [DefaultMedium(material=Dielectric())]
    scale = n / 256.0
    for _ in range(nobj):
        r = rng.uniform(8, 32) * scale * dx
        center = tuple(float(v) for v in rng.uniform(-(inner - r), inner - r, 3))
        eps = float(rng.uniform(1.0, 12.0))
        if rng.uniform() < 0.5:
            geom.append(Sphere(material=Dielectric(eps_inf=eps), center=center, radius=r))
        else:
            geom.append(Block(material=Dielectric(eps_inf=eps), center=center,
                              size=(2 * r, 2 * r, 2 * r)))
    geom.append(Shell(material=Cpml(kappa_max=kappa_max), thickness=pml_cells * dx))
    src = [PointSource(src_time=src_time or Bandpass(freq=0.5, fwidth=0.2), center=(0, 0, 0),
                       component=Ex)]
    space = Cartesian(size=(size, size, size), resolution=res)
    return FDTD(space, geom, src, verbose=verbose, precision=precision), 1000


def dispersive(n=192, seed=0, pml_cells=12, precision="fp64", verbose=False, res=20,
               courant_ratio=0.6, src_time=None, tfsf=True):
    """The 3-D dispersive + UPML benchmark scene on an n^3 grid (resolution 20).

    dt follows the background medium (eps = 2.25) as in the reference, so
    the Courant ratio is lowered to 0.6 to keep the eps_inf = 1 metal stable.
    Excitation: a +z plane wave, x-polarised, Bandpass(0.5, 0.2), through a
    TFSF box spanning 90% of the PML-free interior (``tfsf=False``: an Ez
    point source at the centre instead).
    """
    rng = np.random.default_rng(seed)
    dx = 1.0 / res
    size = n * dx
    inner = size / 2 - pml_cells * dx
    scale = n / 192.0
    geom = [DefaultMedium(material=Dielectric(eps_inf=2.25))]
    drude = Drude(eps_inf=1, dps=(DrudePole(omega=9.0, gamma=0.07),))
    pitch = 2 * inner / 4
    for ix in range(4):
        for iy in range(4):
            c = (-inner + pitch * (ix + 0.5), -inner + pitch * (iy + 0.5), -0.3 * inner)
            r = rng.uniform(10, 20) * scale * dx
            geom.append(Sphere(material=drude, center=c, radius=r))
    geom.append(Block(material=Lorentz(lps=(LorentzPole(amp=2.0, omega=3.0, gamma=0.1),)),
                      center=(0, 0, 0.35 * inner), size=(2 * inner, 2 * inner, 0.15 * inner)))
    cps = tuple(CriticalPoint(amp=float(rng.uniform(0.5, 2.0)),
                              phi=float(rng.uniform(-1.5, 1.5)),
                              omega=float(rng.uniform(2.0, 5.0)),
                              gamma=float(rng.uniform(0.2, 1.0))) for _ in range(2))
    geom.append(Sphere(material=DcpAde(eps_inf=1.1, dps=(DrudePole(omega=7.0, gamma=0.2),),
                                       cps=cps),
                       center=(0.4 * inner, -0.4 * inner, 0.7 * inner), radius=0.2 * inner))
    geom.append(Shell(material=Upml(), thickness=pml_cells * dx))
    st = src_time or Bandpass(freq=0.5, fwidth=0.2)
    if tfsf:
        box = 2 * inner * 0.9
        src = [TotalFieldScatteredField(src_time=st, center=(0, 0, 0), size=(box, box, box),
                                        direction=(0, 0, 1), polarization=(1, 0, 0))]
    else:
        src = [PointSource(src_time=st, center=(0, 0, 0), component=Ez)]
    space = Cartesian(size=(size, size, size), resolution=res)
    return FDTD(space, geom, src, verbose=verbose, precision=precision,
                courant_ratio=courant_ratio), 2000


def bytes_per_cell_update(scene, precision):
    """Algorithmic DRAM bytes of one full E+H step of ``scene``.

    Fields: every active component is read by the curl of the other half
    and read+written by its own update (3-D: 18 values per cell; 2-D TMz: 9).
    Per point: +1 byte class id per active component and half; +4 values per
    CPML point (psi1, psi2 read+write), +2 per UPML point, +4 per pole of a
    Drude/Lorentz point, +2+4P+4Q per DCP point.
    """
    from .scene import naux_of
    es = 4 if precision == "fp32" else 8
    total = 0
    for comp in scene.active:
        c = comp.index
        npts = int(np.prod(scene.shape(c)))
        total += 3 * es * npts + npts  # read by the curl, read + write own, class id
        counts = scene.counts(c)
        for cid, cnt in counts.items():
            total += 2 * naux_of(scene.classes[c][cid]) * es * cnt
    return total


def serving_jobs(njobs=512, seed=0, rate=None, max_steps=5000, min_steps=500, size_scale=1.0,
                 precision="fp64"):
    """The batched-serving request stream: (arrival, build, nsteps) triples.

    Half the jobs are 2-D TMz grids with side uniform in [128, 1024], half
    3-D grids with side uniform in [64, 160] (times ``size_scale``); the
    medium of a central sphere is drawn from {dielectric eps in [1, 12],
    Drude (omega_p 9, gamma 0.07), Lorentz (2.0, 3.0, 0.1)}; CPML 8-16
    cells; step counts uniform in [min_steps, max_steps]; Poisson arrivals
    with ``rate`` jobs per second (default: all at once).  The Drude jobs
    step at Courant ratio 0.6, as the dispersive benchmark scene does: at
    the default 0.99 their eps_inf = 1 metal diverges (the CPU oracle, the
    reference's arithmetic, reaches 1e34 within 1200 steps).
    """
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for q in range(njobs):
        if rate:
            t += float(rng.exponential(1.0 / rate))
        three_d = q % 2 == 1
        side = int(round((rng.uniform(64, 160) if three_d else rng.uniform(128, 1024))
                         * size_scale))
        side = max(side, 24)
        pml = min(int(rng.integers(8, 17)), side // 4)
        kind = int(rng.integers(0, 3))
        eps = float(rng.uniform(1.0, 12.0))
        nsteps = int(rng.integers(min_steps, max_steps + 1))
        out.append((t, _serving_builder(side, three_d, pml, kind, eps, precision), nsteps))
    return out


def _serving_builder(side, three_d, pml, kind, eps, precision):
    def build():
        res = 10
        dx = 1.0 / res
        size = side * dx
        if kind == 0:
            mat = Dielectric(eps_inf=eps)
        elif kind == 1:
            mat = Drude(eps_inf=1, dps=(DrudePole(omega=9.0, gamma=0.07),))
        else:
            mat = Lorentz(lps=(LorentzPole(amp=2.0, omega=3.0, gamma=0.1),))
        r = 0.25 * (size / 2 - pml * dx)
        geom = [DefaultMedium(material=Dielectric()),
                Sphere(material=mat, center=(0.3 * r, 0, 0), radius=r),
                Shell(material=Cpml(), thickness=pml * dx)]
        src = [PointSource(src_time=Bandpass(freq=0.8, fwidth=0.5), center=(-r, 0, 0),
                           component=Ez)]
        cr = 0.6 if kind == 1 else 0.99
        if three_d:
            space = Cartesian(size=(size, size, size), resolution=res)
            return FDTD(space, geom, src, verbose=False, precision=precision, courant_ratio=cr)
        space = Cartesian(size=(size, size, 0), resolution=res)
        return TMzFDTD(space, geom, src, verbose=False, precision=precision, courant_ratio=cr)
    return build


def design2d(n=512, res=20, pml_cells=20, design_px=64, monitor_px=8, nsteps=2000, batch=64,
             seed=0, hard=False, src_time=None, background=None):
    """The differentiation scene: returns (space, geom_list, src_list, design, monitor, eps, nsteps).

    The source column sits a quarter of the interior left of the centre,
    the design region is centred, the monitor patch a quarter right.
    ``hard`` uses hard Ez point sources instead of Jz current sources;
    ``background`` adds dielectric blocks (list of (center, size, eps)).
    ``eps`` is (batch, design_px, design_px) float64, uniform in [1, 12].
    """
    from .adjoint import DesignRegion
    dx = 1.0 / res
    size = n * dx
    inner = size / 2 - pml_cells * dx
    geom = [DefaultMedium(material=Dielectric())]
    for center, bsize, eps in background or []:
        geom.append(Block(material=Dielectric(eps_inf=eps), center=center, size=bsize))
    geom.append(Shell(material=Cpml(), thickness=pml_cells * dx))
    st = src_time or Bandpass(freq=0.5, fwidth=0.5)
    x_src = -inner / 2
    ny_src = int(round(2 * inner / dx)) - 1
    src = [PointSource(src_time=st, center=(x_src, -inner + (q + 1) * dx, 0),
                       component=Ez if hard else Jz) for q in range(ny_src)]
    space = Cartesian(size=(size, size, 0), resolution=res)
    design = DesignRegion(center=(0.0, 0.0), size=(design_px * dx, design_px * dx))
    monitor = DesignRegion(center=(inner / 2, 0.0), size=(monitor_px * dx, monitor_px * dx))
    rng = np.random.default_rng(seed)
    eps = rng.uniform(1.0, 12.0, (batch, design_px, design_px))
    return space, geom, src, design, monitor, eps, nsteps
