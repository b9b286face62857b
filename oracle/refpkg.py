"""Import the reference (GMES) package built by ``oracle/build_ref.py``.

TEST INFRASTRUCTURE ONLY (fixture generation and oracle pinning in the
build container).  ``load_reference()`` returns the reference's ``gmes``
package: its pure-Python modules are read from the reference checkout,
its compiled modules from ``oracle/_ref/gmes_ext``.
"""

import importlib.util
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
EXT = HERE / "_ref" / "gmes_ext"


def reference_root():
    """The checkout the build read (recorded in oracle/_ref/REF_PATH), else
    GMES_REFERENCE; None when neither names one."""
    p = HERE / "_ref" / "REF_PATH"
    if p.exists():
        return Path(p.read_text().strip())
    v = os.environ.get("GMES_REFERENCE", "").strip()
    return Path(v) if v else None


def available():
    root = reference_root()
    return (EXT / "constant.py").exists() and root is not None and (root / "gmes" / "fdtd.py").exists()


def load_reference():
    """Return the reference ``gmes`` package (imported once per process)."""
    if "gmes" in sys.modules and getattr(sys.modules["gmes"], "_gmes_reference", False):
        return sys.modules["gmes"]
    if not available():
        raise RuntimeError("reference build missing: run python oracle/build_ref.py")
    sys.dont_write_bytecode = True
    ref_pkg = reference_root() / "gmes"
    spec = importlib.util.spec_from_file_location(
        "gmes", ref_pkg / "__init__.py",
        submodule_search_locations=[str(EXT), str(ref_pkg)])
    mod = importlib.util.module_from_spec(spec)
    mod._gmes_reference = True
    sys.modules["gmes"] = mod
    spec.loader.exec_module(mod)
    return mod
