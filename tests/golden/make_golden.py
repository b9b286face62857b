"""Generate the golden vectors in tests/golden/ by running the REFERENCE.

Runs the reference GMES package (built by ``oracle/build_ref.py`` from the
reference checkout, which exists only in the build container) on every case
of ``cases.py`` and stores the resulting fields with the reference's time
bookkeeping.  The tests compare the CPU oracle and the CUDA engine against
these files; they never need the reference itself.

Usage:  python tests/golden/make_golden.py [case ...]   (cases.CASES and cases.ORACLE_CASES)
        python tests/golden/make_golden.py --probes [case ...]
        python tests/golden/make_golden.py --pw
"""

import json
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

from cases import CASES, COMP_NAMES, ORACLE_CASES, SUMMARY_ONLY  # noqa: E402

ALL_CASES = {**CASES, **ORACLE_CASES}


def checksum(a):
    a = np.asarray(a)
    if np.iscomplexobj(a):
        return [complex(np.sum(a)).real, complex(np.sum(a)).imag,
                float(np.sum(np.abs(a) ** 2)), float(np.max(np.abs(a)))]
    a = np.asarray(a, np.float64)
    return [float(np.sum(a)), float(np.sum(a * a)), float(np.max(np.abs(a)))]


def main(names):
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle.refpkg import load_reference
    gmes = load_reference()
    for name in names:
        t0 = time.time()
        sim, nsteps = ALL_CASES[name](gmes)
        sim.init()
        t1 = time.time()
        for _ in range(nsteps):
            sim.step()
        t2 = time.time()
        keep = SUMMARY_ONLY.get(name, COMP_NAMES)
        arrays = {}
        meta = {"case": name, "steps": nsteps, "n": sim.time_step.n, "t": sim.time_step.t,
                "dt": sim.time_step.dt, "shapes": {}, "checksums": {},
                "updaters": {}, "init_s": t1 - t0, "step_s": t2 - t1}
        for comp in COMP_NAMES:
            f = np.asarray(getattr(sim, comp))
            meta["shapes"][comp] = list(f.shape)
            meta["checksums"][comp] = checksum(f)
            if comp in keep:
                arrays[comp] = f
        for comp, ups in sim.pw_material.items():
            meta["updaters"][comp.__name__] = {type(u).__name__: int(u.idx_size())
                                               for u in ups.values()}
        np.savez_compressed(HERE / f"{name}.npz", **arrays)
        (HERE / f"{name}.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
        print(f"{name}: init {t1 - t0:.1f}s, {nsteps} steps {t2 - t1:.1f}s", flush=True)


# Probe recordings (FDTD.set_probe, gmes/fdtd.py:607-671): the reference's
# text files for these (case, point) pairs, stored as probe_<case>_<comp>.dat.
PROBES = {"tfsf2d": (0.2, 0.1, 0.0), "tmz_regression": (0.2, 0.1, 0.0)}


def probes(names):
    import tempfile
    from oracle.refpkg import load_reference
    gmes = load_reference()
    for name in names:
        if name not in PROBES:
            continue
        sim, nsteps = CASES[name](gmes)
        sim.init()
        with tempfile.TemporaryDirectory() as tmp:
            prefix = os.path.join(tmp, "p")
            sim.set_probe(PROBES[name], prefix)
            for _ in range(nsteps):
                sim.step()
            for rec in sim.e_recorder + sim.h_recorder:
                rec.close()
            for f in sorted(os.listdir(tmp)):
                comp = f[2:4]
                (HERE / f"probe_{name}_{comp}.dat").write_text(Path(tmp, f).read_text())
                print("probe", name, comp, flush=True)


def pw_updaters():
    """Every point-wise updater of the reference on seeded arrays -> pw_updaters.npz."""
    from cases import PW_COMPS, PW_MODELS, pw_run
    from oracle.refpkg import load_reference
    gmes = load_reference()
    out = {}
    for model in PW_MODELS:
        for comp in PW_COMPS:
            for cmplx in (False, True):
                key = f"{model}_{comp}_{'C' if cmplx else 'R'}"
                out[key] = pw_run(gmes, model, comp, cmplx)
    np.savez_compressed(HERE / "pw_updaters.npz", **out)
    print("pw_updaters:", len(out), "updaters", flush=True)


if __name__ == "__main__":
    args = sys.argv[1:]
    if args[:1] == ["--pw"]:
        pw_updaters()
    elif args[:1] == ["--probes"]:
        probes(args[1:] or list(PROBES))
    else:
        main(args or list(ALL_CASES))
