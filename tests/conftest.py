"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and the built native library; the
others run on CPU only (oracle against the golden fixtures, host logic, the
C-ABI's exported symbols).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built native library")


@pytest.fixture(scope="session")
def renderer():
    from pathtracer_gb300 import native as N

    r = N.Renderer(0)
    yield r
    r.close()


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(GOLDEN / name)

    return load


def bsdf_cases():
    """Golden BSDF fixtures grouped by material name."""
    b = np.load(GOLDEN / "bsdf.npz")
    names = sorted(set(k.split("__")[0] for k in b.files))
    return {n: {k.split("__")[1]: b[k] for k in b.files if k.startswith(n + "__")} for n in names}


def rel_close(a, b, rtol=1e-4, atol=1e-6):
    """|a - b| <= atol + rtol * |b| elementwise (NaN equal to NaN)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    ok = np.abs(a - b) <= atol + rtol * np.abs(b)
    return np.all(ok | both_nan)


def material_mix_for_reference():
    """The 64-sphere material mix (Disney, hair, thin dielectric, Phong,
    Lambertian; 4 sphere and 2 area lights) as the reference renders it
    finitely through the harness: no medium (the harness builds none), hair
    with an explicit sigma_a instead of melanin, and each Phong replaced by a
    grey Lambertian -- the reference's Phong::scatter leaves pdf_val = 0 on
    its diffuse branch (material.hpp:355-365) and getRayColor divides by it,
    which writes inf/NaN into about a fifth of this image's pixels."""
    from pathtracer_gb300 import native as N
    from pathtracer_gb300 import scene as S

    sc, cam = S.material_divergence(2, seed=3, aspect=1.0)
    sc.medium = None
    mats = []
    for t, p, f in sc.materials:
        if t == N.PHONG:
            t, p, f = N.LAMBERTIAN, [0.5, 0.5, 0.5], 0
        elif t == N.HAIR:
            p, f = [0.3, 0.5, 0.9] + list(p[3:]), 0
        mats.append((t, p, f))
    sc.materials = mats
    return sc, cam
