"""Builds the CUDA library (libplgpu.so) in-tree with nvcc for sm_103a.

The library is plain C ABI (include/plgpu.h); this module only drives nvcc.
Sources compile in parallel, one translation unit per file, and the link
step produces ``plgpu/libplgpu.so`` next to this file.  A rebuild happens
only when a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
SRC_DIR = PKG_DIR.parent / "csrc"
REPO = PKG_DIR.parent.parent
INCLUDE = REPO / "include"
OBJ_DIR = PKG_DIR.parent / "_build"
LIB_PATH = PKG_DIR / "libplgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC,-O3",
    "-I",
    str(INCLUDE),
]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA library cannot be built")


def _sources() -> list[Path]:
    return sorted(SRC_DIR.glob("*.cu"))


def _headers() -> list[Path]:
    return sorted(SRC_DIR.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, ptxas_verbose: bool = False, force: bool = False) -> Path:
    """Compiles every csrc/*.cu and links libplgpu.so; returns its path."""
    nvcc = nvcc_path()
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    headers = _headers()
    srcs = _sources()
    objs = []
    jobs = []
    for src in srcs:
        obj = OBJ_DIR / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc] + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_verbose else []) + ["-c", str(src), "-o", str(obj)]
            jobs.append(cmd)
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            logs.append(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{r.stdout}\n{r.stderr}")
    if force or jobs or _stale(LIB_PATH, objs):
        tmp = LIB_PATH.with_suffix(".so.tmp")
        cmd = [nvcc] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed ({' '.join(cmd)}):\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    return LIB_PATH


if __name__ == "__main__":
    import sys

    print(build(verbose=True, ptxas_verbose="-v" in sys.argv, force="-f" in sys.argv))
