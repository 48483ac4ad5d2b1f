"""Builds the native library ``greenpeas_gb300/_lib/libgpc.so`` in tree.

Compiles every translation unit under ``csrc/`` with nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and links them
into one shared library exporting the C ABI declared in ``include/gpc.h``.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "libgpc.so"
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build greenpeas_gb300")


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "gpc.h"]
    t = obj.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compiles (if stale) and links libgpc.so; returns its path."""
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    nv = nvcc()
    common = [nv, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
              f"-I{ROOT / 'include'}", f"-I{CSRC}"]
    jobs = []
    objs = []
    for src in sources():
        obj = OUT_DIR / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            lang = ["-x", "cu"] if src.suffix == ".cu" else ["-x", "c++"]
            jobs.append(common + lang + ["-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not LIB.exists():
        tmp = LIB.with_name(f"libgpc.so.tmp{os.getpid()}")
        run([nv, GENCODE, "-shared", "-o", str(tmp)] + [str(o) for o in objs])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
