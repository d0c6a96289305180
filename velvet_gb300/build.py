"""Builds the solver library in-tree: velvet_gb300/libvelvet_gb300.so (sm_103a).

Every .cu file under velvet_gb300/csrc is compiled in parallel by nvcc for
sm_103a only, then linked into one shared library whose C ABI is
include/velvet_gb300.h.  Flags that matter for results:
  -fmad=false                 no multiply-add contraction in device code
  -Xcompiler -ffp-contract=off  the same for host code (gcc on aarch64 contracts by default)
so every FP32 result is the IEEE-rounded value of the operations as written.

build(checked=True) makes libvelvet_gb300_checked.so from the same sources with
-DVT_CHECKED=1: data-dependent device indices are range-checked and a failure is reported
by the sync calls (the library the tests can load instead with VT_CHECKED=1).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OUT = PKG / "libvelvet_gb300.so"
OBJ = PKG / "_build"
OUT_CHECKED = PKG / "libvelvet_gb300_checked.so"
OBJ_CHECKED = PKG / "_build_checked"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", str(INCLUDE),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build velvet_gb300")


def _compile(src: Path, verbose_ptxas: bool, checked: bool = False) -> Path:
    obj = (OBJ_CHECKED if checked else OBJ) / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *(["-DVT_CHECKED=1"] if checked else []), "-c", str(src), "-o", str(obj)]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def up_to_date(out: Path = OUT) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return all(p.stat().st_mtime <= t for p in deps)


def build(force: bool = False, verbose_ptxas: bool = False, checked: bool = False) -> Path:
    """Compiles and links the library (or its bounds-checked twin) if any source is newer."""
    out, obj_dir = (OUT_CHECKED, OBJ_CHECKED) if checked else (OUT, OBJ)
    if not force and up_to_date(out):
        return out
    obj_dir.mkdir(exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas, checked), srcs))
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, checked="--checked" in sys.argv))
