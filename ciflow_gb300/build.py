"""Build libcigpu.so in-tree with nvcc (sm_103a only).

    python -m ciflow_gb300.build

Compiles every translation unit under ciflow_gb300/csrc in parallel into
ciflow_gb300/_lib/obj and links ciflow_gb300/_lib/libcigpu.so (CUDA runtime
linked statically, so the library loads without extra search paths); the same
sources with -DCIGPU_CHECKED give ciflow_gb300/_lib/libcigpu_checked.so, the
bounds-checked build (csrc/checked.cuh).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libcigpu.so")
# the checked build: every kernel's bounds checks compiled in (checked.cuh)
OBJ_CHECKED = os.path.join(OUT, "obj_checked")
LIB_CHECKED = os.path.join(OUT, "libcigpu_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(SRC, "*.cu")) + glob.glob(os.path.join(SRC, "*.cpp")))


def _compile(src: str, checked: bool = False) -> str:
    obj = os.path.join(OBJ_CHECKED if checked else OBJ, os.path.basename(src) + ".o")
    deps = sources() + glob.glob(os.path.join(SRC, "*.h")) + glob.glob(os.path.join(SRC, "*.cuh")) + \
        glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    extra = ["-DCIGPU_CHECKED"] if checked else []
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), *FLAGS, *extra, "-x", "cu", *ARCH, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, checked: bool = True) -> str:
    """Builds libcigpu.so and (checked=True) libcigpu_checked.so, all translation
    units of both compiled in parallel."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(OBJ_CHECKED, exist_ok=True)
    srcs = sources()
    jobs = [(s, False) for s in srcs] + ([(s, True) for s in srcs] if checked else [])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda j: _compile(*j), jobs))
    for lib, lo in ((LIB, objs[:len(srcs)]), (LIB_CHECKED, objs[len(srcs):])):
        if not lo:
            continue
        if not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in lo):
            cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *lo]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(lib)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
