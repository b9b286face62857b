"""Build the reference (GMES) CPU implementation into ``oracle/_ref/``.

TEST INFRASTRUCTURE ONLY: the product never imports, links or runs what this
builds.  The build reads the reference sources where they lie (the
reference checkout named by ``--ref`` or the ``GMES_REFERENCE`` environment
variable) and writes only into ``oracle/_ref/`` (git-ignored):

* ``src/pygeom.pyx`` and ``src/material.pyx`` are cythonized and compiled
  unmodified, as ``gmes.pygeom`` and ``gmes.material``;
* ``src/pw_material.i`` needs SWIG, which is absent, so the unmodified
  ``src/pw_*.hh`` templates plus ``src/pw_material.cc`` are bound by the
  hand-written pybind11 shim ``oracle/ref_shim/pw_material_shim.cpp``
  (g++ -O2 -std=c++23 -fopenmp, as the reference's setup.py builds it);
* ``gmes.constant`` (also SWIG) is replaced by this package's own
  restatement of that interface, ``gmes_gb300/constant.py``.

The reference's pure-Python modules (``gmes/*.py``) are not copied: the
loader in ``oracle/refpkg.py`` builds the ``gmes`` package with a search
path of ``oracle/_ref/gmes_ext`` followed by the reference's own ``gmes/``
directory.  Only possible where the reference tree, Cython and pybind11 are
present (the build container); the GPU host has neither.

Usage: ``GMES_REFERENCE=<reference checkout> python oracle/build_ref.py``
or ``python oracle/build_ref.py --ref <reference checkout>``.
"""

import argparse
import os
import subprocess
import sys
import sysconfig
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
EXT = OUT / "gmes_ext"
BUILD = OUT / "build"

CONSTANT_SHIM = '''"""gmes.constant for the reference build: loads gmes_gb300/constant.py."""
import importlib.util as _u
import os as _os
_p = _os.path.join(_os.path.dirname(__file__), "..", "..", "..", "gmes_gb300", "constant.py")
_s = _u.spec_from_file_location("_gmes_gb300_constant", _os.path.abspath(_p))
_m = _u.module_from_spec(_s)
_s.loader.exec_module(_m)
globals().update({k: getattr(_m, k) for k in dir(_m) if not k.startswith("__")})
'''


def reference_from_env():
    """The reference checkout named by GMES_REFERENCE, or None when it is unset."""
    v = os.environ.get("GMES_REFERENCE", "").strip()
    return Path(v) if v else None


def _run(cmd):
    print(" ".join(str(c) for c in cmd), flush=True)
    subprocess.run([str(c) for c in cmd], check=True)


def build(ref: Path, jobs: int = 4) -> Path:
    import numpy
    import pybind11

    src = ref / "src"
    if not (src / "pw_material.hh").exists():
        raise FileNotFoundError(f"reference sources not found under {src}")
    EXT.mkdir(parents=True, exist_ok=True)
    BUILD.mkdir(parents=True, exist_ok=True)
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    py_inc = sysconfig.get_paths()["include"]
    common = ["-O2", "-std=c++23", "-fopenmp", "-fPIC", "-shared", f"-I{py_inc}",
              f"-I{numpy.get_include()}", f"-I{src}"]

    procs = []
    for mod in ("pygeom", "material"):
        cpp = BUILD / f"{mod}.cpp"
        _run([sys.executable, "-m", "cython", "-3", "--cplus", "--module-name",
              f"gmes.{mod}", "-o", cpp, src / f"{mod}.pyx"])
        cmd = ["g++", *common, cpp, "-o", EXT / f"{mod}{suffix}"]
        print(" ".join(str(c) for c in cmd), flush=True)
        procs.append(subprocess.Popen([str(c) for c in cmd]))
    shim = HERE / "ref_shim" / "pw_material_shim.cpp"
    cmd = ["g++", *common, f"-I{pybind11.get_include()}", shim, src / "pw_material.cc",
           "-o", EXT / f"pw_material{suffix}"]
    print(" ".join(str(c) for c in cmd), flush=True)
    procs.append(subprocess.Popen([str(c) for c in cmd]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference build step failed")
    (EXT / "constant.py").write_text(CONSTANT_SHIM)
    (OUT / "REF_PATH").write_text(str(ref))
    return EXT


if __name__ == "__main__":
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--ref", default=None,
                    help="reference checkout (default: the GMES_REFERENCE environment variable)")
    args = ap.parse_args()
    ref = Path(args.ref) if args.ref else reference_from_env()
    if ref is None:
        sys.exit("no reference checkout: pass --ref or set GMES_REFERENCE")
    print(build(ref))
