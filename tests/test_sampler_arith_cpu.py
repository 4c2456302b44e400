"""The sampler arithmetic of pt_common.cuh, host side (tests/cpp/
sampler_arith_check.cpp): division by a Halton base through a precomputed
reciprocal equals hardware division (lowest and highest 2^20 operands and
2^22 hashed ones, all 25 bases); Kensler's permutation of {0, 1}
(gl::permutationElement, utils/utility.hpp:434-464) is one parity bit of the
hash; the Owen-scrambled radical inverse (sampler/digitPerm.hpp:99-133)
with its early termination and base-2 shortcut equals the every-digit loop
bit for bit (100 dimensions x 2^15 indices).  The device's sampler values
are held bit-exact against the oracle and the reference's fixtures in
tests/test_gpu_parity.py."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
SRC = REPO / "tests" / "cpp" / "sampler_arith_check.cpp"


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_sampler_arithmetic_matches_plain_forms(tmp_path):
    exe = tmp_path / "sampler_arith_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", str(SRC), "-o", str(exe)], check=True)
    proc = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    lines = proc.stdout.strip().split("\n")
    assert len(lines) == 3 and all(" 0 mismatches" in ln for ln in lines), proc.stdout
