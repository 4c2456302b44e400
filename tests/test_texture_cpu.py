"""Surface textures in the oracle and the host scene build (CPU only)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S


def test_textured_scene_builds_and_renders():
    sc, cam = S.textured_cornell(2)
    info = N.bvh_build(sc)
    assert info["items"] == 6 + 320
    job = N.job_desc(0, cam, 16, 16, 2, 2, 5, seed=3, estimator=N.EST_NEE_MIS)
    a, _ = O.render(sc, job)
    assert np.isfinite(a).all() and a.mean() > 0
    # the textures change the image
    plain, _ = S.textured_cornell(2)
    plain.materials = [(t, p, f & ((1 << N.MAT_TEXTURE_SHIFT) - 1)) for t, p, f in plain.materials]
    plain.materials = [(t, [0.5, 0.5, 0.5] + p[3:] if t == N.LAMBERTIAN else ([10, 10, 10] + p[3:] if t == N.DIFFUSE_EMITTER else p), f)
                       for t, p, f in plain.materials]
    b, _ = O.render(plain, job)
    assert not np.allclose(a, b)


def test_texture_index_is_validated():
    sc, _ = S.textured_cornell(1)
    t, p, f = sc.materials[1]
    sc.materials[1] = (t, p, (99 << N.MAT_TEXTURE_SHIFT))
    with pytest.raises(N.PtError):
        N.bvh_build(sc)
    sc, _ = S.textured_cornell(1)
    sc.textures[2]["texels"] = np.zeros((1, 5, 3), np.float32)  # image smaller than 2x2
    with pytest.raises(N.PtError):
        N.bvh_build(sc)


def _box_scene(as_box: bool):
    from pathtracer_gb300 import scene as S
    sc, cam = S.cornell_icosphere(1)
    grey = sc.add_material(N.LAMBERTIAN, [0.6, 0.6, 0.3])
    lo, hi = (0.15, 0.0, 0.5), (0.45, 0.35, 0.8)
    if as_box:
        sc.add_box(lo, hi, grey)
    else:  # the six faces as rectangles, in the Box's order
        sc.add_quad(0, hi[0], lo[1], hi[1], lo[2], hi[2], grey)
        sc.add_quad(0, lo[0], lo[1], hi[1], lo[2], hi[2], grey)
        sc.add_quad(1, hi[1], lo[0], hi[0], lo[2], hi[2], grey)
        sc.add_quad(1, lo[1], lo[0], hi[0], lo[2], hi[2], grey)
        sc.add_quad(2, hi[2], lo[0], hi[0], lo[1], hi[1], grey)
        sc.add_quad(2, lo[2], lo[0], hi[0], lo[1], hi[1], grey)
    return sc, cam


def test_box_is_its_six_faces():
    a_sc, cam = _box_scene(True)
    b_sc, _ = _box_scene(False)
    assert N.bvh_build(a_sc)["items"] == N.bvh_build(b_sc)["items"]
    job = N.job_desc(0, cam, 20, 20, 2, 2, 5, seed=6, estimator=N.EST_NEE_MIS)
    a, _ = O.render(a_sc, job)
    b, _ = O.render(b_sc, job)
    # same surfaces, different top-level tree: only exact edge ties may differ
    assert np.isclose(a, b, rtol=1e-5, atol=1e-6).all(-1).mean() > 0.99


def test_curves_build_and_render():
    sc, cam = S.hair_curves(40, seed=2)
    info = N.bvh_build(sc)
    assert info["items"] == 2 + 1 + 40
    job = N.job_desc(0, cam, 24, 24, 2, 2, 5, seed=1, estimator=N.EST_NEE_MIS)
    a, _ = O.render(sc, job)
    assert np.isfinite(a).all() and a.mean() > 0
    # rays straight down onto a strand's root hit it
    rays = []
    for cps, w0, w1, _ in sc.curves[:10]:
        x, _, z = cps[0]
        rays.append([x, 0.05, z - 1.0, 0.0, 0.0, 1.0])
    t, prim = O.OracleScene(sc).trace_closest(np.array(rays, np.float32))
    curve_prims = set(range(3, 3 + 40))  # after the two rectangles and the sphere
    assert sum(int(p) in curve_prims for p in prim) >= 8


def test_oracle_textures_match_reference_textures():
    """The oracle's CheckerTexture / NoiseTexture evaluation against the
    reference's own getTexelColor (texture.cpp:151-193, pattern.hpp:72-114)
    through the harness, where it is built: bit for bit at random (u, v),
    several scales and octave counts, including coordinates past the Perlin
    lattice's period."""
    from oracle.ref import refbind
    if not refbind.available():
        pytest.skip("reference harness not built")
    rng = np.random.default_rng(4)
    uv = rng.uniform(0.0, 1.0, (4000, 2)).astype(np.float32)
    c1, c2 = (0.1, 0.2, 0.6), (0.9, 0.8, 0.2)
    for scale in (1.0, 10.0, 37.5, 400.0):
        ours = O.tex_eval(N.TEX_CHECKER, uv, c1, c2, scale)
        ref = refbind.texture_eval(1, c1, c2, scale, 1, uv)
        assert np.array_equal(ours, ref), scale
        for fractal in (1, 3, 7):
            ours = O.tex_eval(N.TEX_NOISE, uv, scale=scale, fractal=fractal)
            ref = refbind.texture_eval(2, c1, c2, scale, fractal, uv)
            assert np.array_equal(ours, ref), (scale, fractal)


def test_oracle_box_and_curve_hits_match_reference():
    """Closest hits on Box objects (six rectangles, ObjectList rule) and on
    Curve objects (cylinder segments) in the oracle against the reference's
    own Box / Curve intersection (box.hpp, curve.hpp) under its BVHNode,
    through the harness, where it is built: same primitive, same t."""
    from oracle.ref import refbind
    if not refbind.available():
        pytest.skip("reference harness not built")
    sc, cam = S.hair_curves(60, seed=3)
    m = sc.add_material(N.LAMBERTIAN, [0.6, 0.5, 0.4])
    sc.add_box((-0.7, 0.0, 0.3), (-0.3, 0.5, 0.7), m)
    sc.add_box((0.2, 0.0, -0.6), (0.6, 0.3, -0.2), m)
    rng = np.random.default_rng(8)
    n = 8192
    o = np.tile(cam["position"], (n, 1)) + rng.normal(0, 0.02, (n, 3))
    d = np.stack([rng.uniform(-0.35, 0.35, n), rng.uniform(-0.45, 0.2, n), np.ones(n)], 1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d], 1).astype(np.float32)
    t_o, p_o = O.OracleScene(sc).trace_closest(rays)
    t_r, p_r, _, _, _ = refbind.RefScene(sc).trace_closest(rays)
    hit = p_r >= 0
    assert hit.sum() > 2000
    curve_base = len(sc.quads) + 6 * len(sc.boxes) + len(sc.spheres)
    assert ((p_r >= curve_base) & hit).sum() > 200 and ((p_r >= len(sc.quads)) & (p_r < curve_base) & hit).sum() > 200
    assert (p_o == p_r).mean() > 0.999
    same = (p_o == p_r) & hit
    assert np.array_equal(t_o[same], t_r[same])
