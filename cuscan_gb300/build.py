"""Build the sm_103a shared library ``_build/libcuscan_gb300.so`` from ``csrc/``.

Each translation unit is compiled by nvcc in parallel for exactly one target
(``-gencode arch=compute_103a,code=sm_103a``) and linked with the static CUDA runtime, so the
library depends on nothing but the driver. The build is incremental on file times.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIBRARY = BUILD / "libcuscan_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers():
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")))


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return t < src.stat().st_mtime or t < newest_header


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    common = ["-O3", "-std=c++17", "-I", str(INCLUDE), "-I", str(CSRC), "-Xcompiler", "-fPIC"]
    jobs = []
    objects = []
    for src in _sources():
        obj = BUILD / (src.name + ".o")
        objects.append(obj)
        if not force and not _stale(obj, src, newest_header):
            continue
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, "-lineinfo", "--fmad=false", "-Xptxas", "-v" if verbose else "-O3",
                   *common, "-c", str(src), "-o", str(obj)]
        else:
            cmd = [nvcc, *common, "-x", "c++", "-c", str(src), "-o", str(obj)]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for log in ex.map(run, jobs):
                if verbose and log:
                    print(log, file=sys.stderr)
    newest_obj = max(o.stat().st_mtime for o in objects)
    if force or jobs or not LIBRARY.exists() or LIBRARY.stat().st_mtime < newest_obj:
        tmp = LIBRARY.with_suffix(f".{os.getpid()}.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp),
               *[str(o) for o in objects], "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
