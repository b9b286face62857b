"""Time the reference's own FDTD.step() against the oracle port, on this host.

TEST INFRASTRUCTURE ONLY: it runs the reference built by
``oracle/build_ref.py`` (which needs the reference checkout, Cython and
pybind11, present only in the build container) and the C oracle on the same
scenes, with the timing method of the reference's benchmark
(benchmarks/field_updates.py:122-156: warm-up steps, then the median of R
repeats of K steps), and prints one JSON line per scene.  The GPU host has
neither the reference sources nor Cython, so there the CPU baseline is the
oracle port alone; this script records how the two compare on one host.

Usage: ``GMES_REFERENCE=<checkout> python oracle/time_reference.py``
"""
import json
import os
import statistics
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
# import this directory as the package ``oracle``, not its oracle.py module
sys.path = [p for p in sys.path if Path(p or ".").resolve() != HERE]
sys.path.insert(0, str(ROOT))


def scenes(g):
    """(name, sim builder, K) in the reference's and this package's API alike."""
    def air2d():
        space = g.Cartesian(size=(10, 10, 0), resolution=20)
        geom = [g.DefaultMedium(material=g.Dielectric()), g.Shell(material=g.Cpml())]
        src = [g.PointSource(src_time=g.Continuous(freq=0.8), center=(0, 0, 0), component=g.Ez)]
        return g.TMzFDTD(space, geom, src, verbose=False)

    def cube3d():
        space = g.Cartesian(size=(5, 5, 5), resolution=10)
        geom = [g.DefaultMedium(material=g.Dielectric()), g.Shell(material=g.Cpml())]
        src = [g.PointSource(src_time=g.Continuous(freq=0.8), center=(0, 0, 0), component=g.Ex)]
        return g.FDTD(space, geom, src, verbose=False)
    return [("air2d_tmz_200x200_cpml", air2d, 40), ("cube3d_50x50x50_cpml", cube3d, 10)]


def median_step(step, warmup=5, repeats=5, k=20):
    for _ in range(warmup):
        step()
    times = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        for _ in range(k):
            step()
        times.append((time.perf_counter() - t0) / k)
    return statistics.median(times)


def main():
    from oracle.refpkg import load_reference
    from oracle.oracle import Oracle
    import gmes_gb300 as G
    ref = load_reference()
    threads = os.cpu_count()
    for (name, build_ref, k), (_, build_ours, _) in zip(scenes(ref), scenes(G)):
        sim = build_ref()
        sim.init()
        cells = sim.space.whole_field_size
        n = int(cells[0]) * int(cells[1]) * int(cells[2])
        t_ref = median_step(sim.step, k=k)
        orc = Oracle(build_ours().compile())
        t_orc = median_step(lambda: orc.step(1), k=k)
        print(json.dumps({"scene": name, "cells": n, "host_threads": threads,
                          "reference_s_per_step": round(t_ref, 6),
                          "reference_gcells": round(n / t_ref / 1e9, 5),
                          "oracle_s_per_step": round(t_orc, 6),
                          "oracle_gcells": round(n / t_orc / 1e9, 5)}), flush=True)


if __name__ == "__main__":
    main()
