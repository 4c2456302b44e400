"""Build recipe of the native library ``libpathtracer_gb300.so``.

The CUDA translation units are compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), the host C++ layer with the
host compiler through nvcc, in parallel, and linked in-tree into
``pathtracer_gb300/_lib``.  No CMake and no torch extension machinery: the
library is a plain C-ABI shared object that ctypes (or any FFI) loads.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIBNAME = "libpathtracer_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pathtracer_gb300")
    return cand


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compiles every translation unit of csrc/ and links the shared library."""
    LIBDIR.mkdir(exist_ok=True)
    objdir = LIBDIR / "obj"
    objdir.mkdir(exist_ok=True)
    lib = LIBDIR / LIBNAME
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [REPO / "include" / "pathtracer_gb300.h"]
    srcs = _sources()
    nv = nvcc()
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC,-ffp-contract=off,-Wall,-Wno-unknown-pragmas",
              "-I", str(CSRC), "-I", str(REPO / "include")]
    jobs = []
    objs = []
    for s in srcs:
        o = objdir / (s.name + ".o")
        objs.append(o)
        if not force and not _stale(o, [s] + headers):
            continue
        if s.suffix == ".cu":
            cmd = [nv, *ARCH, "-lineinfo", "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills", *common,
                   "-c", str(s), "-o", str(o)]
        else:
            cmd = [nv, *common, "-c", str(s), "-o", str(o)]
        jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(lib, objs):
        _run([nv, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-cudart", "static", "-lpthread"])
    if verbose:
        print(f"built {lib}", file=sys.stderr)
    return lib


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
