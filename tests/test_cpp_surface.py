"""The reference-shaped C++ surface (include/pathtracer_gb300.hpp): Material::f
/ scatter_pdf / scatter (material.hpp:15-77), DiffuseEmitter::emit,
HaltonSampler (sampler.hpp:7-83), LightList / Light (lightList.hpp,
light.hpp:17-306) and getRayColor (maxdepth_nee.hpp:9) as a reference-style
program calls them (tests/cpp/api_surface_example.cpp).  CPU: it compiles and
links.  GPU: its values equal the C-ABI's on the same inputs (the C-ABI's own
parity with the reference is tests/test_gpu_parity.py, tests/test_lights.py,
tests/test_gpu_ray_color.py) and the oracle's Halton points bit for bit."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
SRC = REPO / "tests" / "cpp" / "api_surface_example.cpp"
LIBDIR = REPO / "pathtracer_gb300" / "_lib"


def _build(tmp_path):
    exe = tmp_path / "api_surface_example"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(REPO / "include"), str(SRC), "-o", str(exe),
                    "-L", str(LIBDIR), "-lpathtracer_gb300", f"-Wl,-rpath,{LIBDIR}"], check=True)
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_cpp_surface_compiles(tmp_path):
    assert _build(tmp_path).exists()


@pytest.mark.gpu
def test_cpp_surface_matches_c_abi(tmp_path, renderer):
    from oracle import pyoracle as O
    from pathtracer_gb300 import native as N
    from pathtracer_gb300 import scene as S

    proc = subprocess.run([str(_build(tmp_path))], capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr
    out = proc.stdout.split("\n")
    rows = [np.array([float(x) for x in ln.split()]) for ln in out if ln.strip()]
    gold = N.material(N.CONDUCTOR, [0.143, 0.374, 1.442, 3.983, 2.385, 1.603, 0.3, 0.3])
    wo = np.array([[0.3, -0.2, 0.932738]], np.float32)
    wi = np.array([[-0.4, 0.1, 0.910494]], np.float32)
    nrm = np.array([[0.0, 0.0, 1.0]], np.float32)
    f, pdf = renderer.bsdf_eval(gold, wo, wi, nrm, np.ones(1, np.uint8))
    assert np.array_equal(rows[0].astype(np.float32), f[0]) and np.float32(rows[1][0]) == pdf[0]
    ok, swi, att, spdf, ty = renderer.bsdf_sample(gold, wo, nrm, np.ones(1, np.uint8), np.array([0.37], np.float32),
                                                  np.array([[0.21, 0.83]], np.float32))
    assert rows[2][0] == ok[0] and rows[2][1] == ty[0] and np.float32(rows[2][2]) == spdf[0]
    assert np.array_equal(rows[3].astype(np.float32), swi[0]) and np.array_equal(rows[4].astype(np.float32), att[0])
    assert np.allclose(rows[5], [0.1, 0.2, 0.3])
    assert np.allclose(rows[6], [25.5, 18.0, 6.0]) and np.allclose(rows[7], 0.0)
    ref = O.sampler_eval(N.SAMPLER_HALTON_OWEN, 1, 3, 5)
    for i in range(3):
        assert rows[8 + i][0] == i + 1
        assert np.array_equal(rows[8 + i][1:].astype(np.float32), ref[i])
    k = 11
    n_lights = int(rows[k][0])
    k += 1
    sc = S.Scene(bg=(0.7, 0.8, 1.0))  # SceneInfo's default bg_color (renderManager.hpp:41)
    white = sc.add_material(N.LAMBERTIAN, [0.75, 0.75, 0.75])
    lm = sc.add_material(N.DIFFUSE_EMITTER, [17.0, 12.0, 4.0, 1.0])
    gm = sc.add_material(N.CONDUCTOR, [0.143, 0.374, 1.442, 3.983, 2.385, 1.603, 0.3, 0.3])
    sc.add_quad(1, 0.999, 0.375, 0.625, 0.375, 0.625, lm)
    sc.add_quad(0, 1.0, 0.0, 1.0, 0.0, 1.0, white)
    sc.add_quad(0, 0.0, 0.0, 1.0, 0.0, 1.0, white)
    sc.add_quad(1, 0.0, 0.0, 1.0, 0.0, 1.0, white)
    sc.add_quad(1, 1.0, 0.0, 1.0, 0.0, 1.0, white)
    sc.add_quad(2, 1.0, 0.0, 1.0, 0.0, 1.0, white)
    sc.add_sphere((0.5, 0.3, 0.55), 0.25, gm)
    sc.add_sphere((0.2, 0.8, 0.3), 0.05, lm)
    sid = renderer.upload(sc)
    assert n_lights == renderer.scene_info(sid)["lights"] == 2
    x = np.array([[0.5, 0.4, 0.5]], np.float32)
    for li in range(n_lights):
        r = renderer.light_sample(sid, li, np.array([[0.3, 0.7]], np.float32), x)
        for kk, name in enumerate(("point", "normal", "dir", "le")):
            assert np.array_equal(rows[k + kk].astype(np.float32), r[name][0]), (li, name)
        assert np.float32(rows[k + 4][0]) == r["pdf"][0] and np.float32(rows[k + 4][1]) == np.float32(r["area"])
        k += 5
    cam = S.camera((0.5, 0.5, -1.4), (0.0, 0.0, 1.0), 40.0, 1.0)
    d = np.array(rows[k:k + 64], np.float32)  # the directions the program built
    rays = np.concatenate([np.tile(np.float32([0.5, 0.5, -1.4]), (64, 1)), d], 1).astype(np.float32)
    want = renderer.ray_color(N.job_desc(sid, cam, 1, 1, 1, 1, 8), rays, first_index=101)
    got = np.array(rows[k + 64:k + 128], np.float32)
    assert np.array_equal(got, want)
    renderer.release(sid)
