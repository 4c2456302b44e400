"""The C++ scene API (include/pathtracer_gb300.hpp): a scene function written
like the reference's compiles against it (CPU) and renders the same image as
the same scene described through the Python binding (GPU)."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
SRC = REPO / "tests" / "cpp" / "cornell_example.cpp"
LIBDIR = REPO / "pathtracer_gb300" / "_lib"


def _build(tmp_path, src=SRC):
    exe = tmp_path / src.stem
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(REPO / "include"), str(src), "-o", str(exe),
                    "-L", str(LIBDIR), "-lpathtracer_gb300", f"-Wl,-rpath,{LIBDIR}"], check=True)
    return exe


TEXTURED = REPO / "tests" / "cpp" / "textured_example.cpp"


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_cpp_scene_compiles_and_links(tmp_path):
    assert _build(tmp_path).exists()
    assert _build(tmp_path, TEXTURED).exists()


@pytest.mark.gpu
def test_cpp_textured_scene_renders_like_python(tmp_path):
    from pathtracer_gb300 import native as N
    from pathtracer_gb300 import scene as S

    out = subprocess.run([str(_build(tmp_path, TEXTURED))], capture_output=True, text=True, check=True).stdout
    cpp_mean = np.array([float(x) for x in out.split()])
    sc = S.Scene()
    checker = sc.add_texture(N.TEX_CHECKER, (0.1, 0.1, 0.1), (0.8, 0.8, 0.8), scale=40.0)
    noise = sc.add_texture(N.TEX_NOISE, scale=8.0, fractal=4)
    lchk = sc.add_texture(N.TEX_CHECKER, (4.0, 2.0, 0.5), (20.0, 14.0, 5.0), scale=30.0)
    # materials in object order, as the C++ SceneInfo flattens them (one per object)
    m_light = sc.add_material(N.DIFFUSE_EMITTER, [0, 0, 0, 1.0], texture=lchk)
    m_w1 = sc.add_material(N.LAMBERTIAN, [0.75, 0.75, 0.75])
    m_green = sc.add_material(N.LAMBERTIAN, [0.14, 0.45, 0.09])
    m_floor = sc.add_material(N.LAMBERTIAN, [0, 0, 0], texture=checker)
    m_w2 = sc.add_material(N.LAMBERTIAN, [0.75, 0.75, 0.75])
    m_back = sc.add_material(N.LAMBERTIAN, [0, 0, 0], texture=noise)
    m_ball = sc.add_material(N.LAMBERTIAN, [0, 0, 0], texture=noise)
    sc.add_quad(1, 0.999, 0.3, 0.7, 0.3, 0.7, m_light)
    sc.add_quad(0, 1.0, 0.0, 1.0, 0.0, 1.0, m_w1)
    sc.add_quad(0, 0.0, 0.0, 1.0, 0.0, 1.0, m_green)
    sc.add_quad(1, 0.0, 0.0, 1.0, 0.0, 1.0, m_floor)
    sc.add_quad(1, 1.0, 0.0, 1.0, 0.0, 1.0, m_w2)
    sc.add_quad(2, 1.0, 0.0, 1.0, 0.0, 1.0, m_back)
    sc.add_sphere((0.5, 0.3, 0.55), 0.25, m_ball)
    cam = S.camera((0.5, 0.5, -1.4), (0.0, 0.0, 1.0), 40.0, 1.0)
    r = N.Renderer(0)
    sid = r.upload(sc)
    film = r.render(N.job_desc(sid, cam, 48, 48, 4, 4, 6, estimator=N.EST_NEE_MIS, env_sampling=N.ENV_ALIAS))
    r.close()
    np.testing.assert_allclose(cpp_mean, film.reshape(-1, 3).mean(0), rtol=1e-5)


@pytest.mark.gpu
def test_cpp_scene_renders_like_python(tmp_path):
    from pathtracer_gb300 import native as N
    from pathtracer_gb300 import scene as S

    out = subprocess.run([str(_build(tmp_path))], capture_output=True, text=True, check=True).stdout
    cpp_mean = np.array([float(x) for x in out.split()])
    sc = S.Scene()
    white = sc.add_material(N.LAMBERTIAN, [0.75, 0.75, 0.75])
    red = sc.add_material(N.LAMBERTIAN, [0.63, 0.065, 0.05])
    green = sc.add_material(N.LAMBERTIAN, [0.14, 0.45, 0.09])
    light = sc.add_material(N.DIFFUSE_EMITTER, [17.0, 12.0, 4.0, 1.0])
    gold = sc.add_material(N.CONDUCTOR, [*S.GOLD_ETA, *S.GOLD_K, 0.3, 0.3])
    sc.add_quad(1, 0.999, 0.375, 0.625, 0.375, 0.625, light)
    sc.add_quad(0, 1.0, 0.0, 1.0, 0.0, 1.0, red)
    sc.add_quad(0, 0.0, 0.0, 1.0, 0.0, 1.0, green)
    sc.add_quad(1, 0.0, 0.0, 1.0, 0.0, 1.0, white)
    sc.add_quad(1, 1.0, 0.0, 1.0, 0.0, 1.0, white)
    sc.add_quad(2, 1.0, 0.0, 1.0, 0.0, 1.0, white)
    sc.add_sphere((0.5, 0.3, 0.55), 0.25, gold)
    cam = S.camera((0.5, 0.5, -1.4), (0.0, 0.0, 1.0), 40.0, 1.0)
    r = N.Renderer(0)
    sid = r.upload(sc)
    film = r.render(N.job_desc(sid, cam, 48, 48, 4, 4, 8, estimator=N.EST_NEE_MIS, env_sampling=N.ENV_ALIAS))
    r.close()
    np.testing.assert_allclose(cpp_mean, film.reshape(-1, 3).mean(0), rtol=1e-5)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_cpp_image_files_load_like_python(tmp_path):
    """ImageTexture(filename, flip_y) and EnvironmentLight(hdri_filepath) in
    the C++ API load the same texels as pathtracer_gb300.native.load_image."""
    from pathtracer_gb300 import native as N
    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, (9, 14, 3), dtype=np.uint8)
    png = tmp_path / "tex.png"
    N.write_png(png, img)
    hdr = tmp_path / "env.hdr"
    rgbe = rng.integers(0, 256, (6, 10, 4), dtype=np.uint8)
    hdr.write_bytes(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 6 +X 10\n" + rgbe.tobytes())
    exe = _build(tmp_path, REPO / "tests" / "cpp" / "image_files_example.cpp")
    lines = subprocess.run([str(exe), str(png), str(hdr)], capture_output=True, text=True, check=True).stdout.split("\n")
    w, h = map(int, lines[0].split())
    got_png = np.array(lines[1:1 + w * h * 3], np.float32).reshape(h, w, 3)
    k = 1 + w * h * 3
    w2, h2 = map(int, lines[k].split())
    got_env = np.array(lines[k + 1:k + 1 + w2 * h2 * 3], np.float32).reshape(h2, w2, 3)
    assert (w, h, w2, h2) == (14, 9, 10, 6)
    assert np.array_equal(got_png, N.load_image(png, flip_y=True))
    assert np.array_equal(got_env, N.load_image(hdr, flip_y=False, hdr=True))
    assert lines[k + 1 + w2 * h2 * 3] == "missing-file error"
