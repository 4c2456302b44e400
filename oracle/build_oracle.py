"""Builds the CPU oracle (ORACLE: test infrastructure only) into
oracle/_lib/libpt_oracle.so with the host compiler.

-ffp-contract=off keeps every float operation separately rounded, so the
restatement computes the same bits on x86-64 and AArch64 hosts.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_lib" / "libpt_oracle.so"


def build(verbose: bool = False, force: bool = False) -> Path:
    srcs = [HERE / "pt_oracle.cpp"]
    deps = srcs + [HERE / "pt_oracle_math.hpp", HERE / "pt_oracle_bsdf.hpp",
                   HERE.parent / "include" / "pathtracer_gb300.h"]
    if not force and OUT.exists() and all(d.stat().st_mtime <= OUT.stat().st_mtime for d in deps):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cxx = shutil.which("g++") or "c++"
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", "-Wall",
           "-o", str(OUT), *map(str, srcs)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if verbose:
        print(f"built {OUT}", file=sys.stderr)
    return OUT


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
