"""Builds the solver library in-tree for sm_103a, in three variants of the same sources.

  exact    velvet_gb300/libvelvet_gb300.so          (the default library)
  checked  velvet_gb300/libvelvet_gb300_checked.so  exact + -DVT_CHECKED=1
  fast     velvet_gb300/libvelvet_gb300_fast.so     contracted arithmetic (see FAST_FLAGS)

Every .cu file under velvet_gb300/csrc is compiled in parallel by nvcc for sm_103a only,
then linked into one shared library whose C ABI is include/velvet_gb300.h.

exact: flags that fix every FP32 result to the IEEE-rounded value of the operations as
written, on the device and in host code alike:
  -fmad=false                   no multiply-add contraction in device code
  -Xcompiler -ffp-contract=off  the same for host code (gcc on aarch64 contracts by default)
checked: -DVT_CHECKED=1 range-checks data-dependent device indices; a failure is reported
by the sync calls (the library the tests can load instead with VT_CHECKED=1).
fast: the solver kernels are compiled as nvcc compiles by default (-fmad=true, so a
multiply followed by an add may become one FMA, as in the reference's own build) plus
approximate division and square root, with reciprocals taken once per vector division
and one division per distance correction (-DVT_FAST=1).  Results differ from the exact
build in the last bits of each operation; the tests bound the difference by the
solver's stated tolerance.  The spatial hash (vt_hash.cu), its allocation-free entry
point and the device grid builder (vt_build.cu) keep the exact flags, so cell keys, sort
order and neighbour lists of given positions, and a cloth built on the device, are
bit-identical in every variant; threshold decisions and the bending-angle chain inside
the fast kernels use exact operations too (vt_math.cuh).  Host code keeps
-ffp-contract=off.
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

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", str(INCLUDE),
]
EXACT_FLAGS = ["-fmad=false"]
FAST_FLAGS = ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-DVT_FAST=1"]
# sources compiled with the exact flags in every variant (bit-identical hashing)
EXACT_ONLY = {"vt_hash.cu", "vt_hash_noalloc.cu", "vt_build.cu"}

VARIANTS = {
    "exact": ("libvelvet_gb300.so", "_build", []),
    "checked": ("libvelvet_gb300_checked.so", "_build_checked", ["-DVT_CHECKED=1"]),
    "fast": ("libvelvet_gb300_fast.so", "_build_fast", None),
}
OUT = PKG / VARIANTS["exact"][0]


def library_path(variant: str = "exact") -> Path:
    return PKG / VARIANTS[variant][0]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build velvet_gb300")


def flags_for(src: Path, variant: str) -> list[str]:
    extra = VARIANTS[variant][2]
    if extra is None:  # fast
        return list(EXACT_FLAGS if src.name in EXACT_ONLY else FAST_FLAGS)
    return [*EXACT_FLAGS, *extra]


def _compile(src: Path, variant: str, verbose_ptxas: bool) -> Path:
    obj = PKG / VARIANTS[variant][1] / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, *COMMON_FLAGS, *flags_for(src, variant), "-c", str(src), "-o", str(obj)]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name} ({variant}):\n{r.stdout}\n{r.stderr}")
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


def build(force: bool = False, verbose_ptxas: bool = False, checked: bool = False,
          variant: str | None = None) -> Path:
    """Compiles and links one variant of the library if any source is newer."""
    variant = variant or ("checked" if checked else "exact")
    out, obj_dir = PKG / VARIANTS[variant][0], PKG / VARIANTS[variant][1]
    if not force and up_to_date(out):
        return out
    obj_dir.mkdir(exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, variant, verbose_ptxas), srcs))
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    v = next((a.split("=", 1)[1] for a in sys.argv if a.startswith("--variant=")),
             "checked" if "--checked" in sys.argv else "exact")
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, variant=v))
