"""Build ``libgmes_gb300.so`` in-tree with nvcc for sm_103a.

The engine is plain CUDA C++ behind a C ABI (include/gmes_gb300.h); it is
compiled directly with nvcc (no torch extension machinery) so the library
links nothing but the CUDA runtime.  Translation units are compiled in
parallel and re-used when their sources have not changed.
"""

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgmes_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          f"-I{ROOT / 'include'}"]
# Per-file flags: the coefficient builder and the rasteriser reproduce the
# reference's FP64 operation order, so multiply-add contraction is disabled;
# the differentiation kernels write every fused multiply-add explicitly so
# that their one-step and temporally blocked forms round alike.
EXTRA = {"gmes_coef.cu": ["--fmad=false"], "gmes_raster.cu": ["--fmad=false"],
         "gmes_adjoint.cu": ["--fmad=false"]}
SOURCES = ["gmes_capi.cu", "gmes_coef.cu", "gmes_step.cu", "gmes_raster.cu", "gmes_adjoint.cu",
           "gmes_points.cu"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gmes_gb300")
    return exe


def _digest(src, flags):
    h = hashlib.sha256()
    h.update(" ".join(flags).encode())
    for p in sorted(list(CSRC.glob("*.cuh")) + [ROOT / "include" / "gmes_gb300.h", src]):
        h.update(p.read_bytes())
    return h.hexdigest()[:16]


def build(verbose=False, jobs=None):
    """Compile (if needed) and link the engine; return the library path."""
    BUILD.mkdir(exist_ok=True)
    exe = nvcc()
    objs = []
    tasks = []
    for name in SOURCES:
        src = CSRC / name
        flags = ARCH + COMMON + EXTRA.get(name, [])
        obj = BUILD / f"{src.stem}-{_digest(src, flags)}.o"
        objs.append(obj)
        if not obj.exists():
            tasks.append([exe, *flags, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for _ in ex.map(run, tasks):
            pass
    tmp = LIB.with_suffix(".so.tmp")
    run([exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
    os.replace(tmp, LIB)
    # objects of earlier sources or flags are not needed again
    keep = set(objs)
    for name in SOURCES:
        for old in BUILD.glob(f"{Path(name).stem}-*.o"):
            if old not in keep:
                old.unlink()
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
