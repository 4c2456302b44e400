"""Surface textures (ColorVariant): checker, Perlin noise and image textures
on Lambertian albedos and on a light's colour, with texture coordinates from
rectangles, spheres, meshes with uvs and the planar fallback.  GPU images
against the oracle on the same sample streams."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _z(mean_a, var_a, mean_b, var_b, spp):
    se = np.sqrt((var_a + var_b).reshape(-1, 3).sum(0) / spp) / (mean_a.shape[0] * mean_a.shape[1])
    return (mean_a.reshape(-1, 3).mean(0) - mean_b.reshape(-1, 3).mean(0)) / se


def _compare(renderer, sc, job, spp, frac=0.9):
    sid = renderer.upload(sc)
    job.scene = sid
    film = renderer.render(job)
    renderer.release(sid)
    job.scene = 0
    m_o, v_o = O.render(sc, job)
    assert np.isfinite(film).all()
    z = _z(film, v_o, m_o, v_o, spp)
    assert np.all(np.abs(z) < 3.0), z
    close = np.isclose(film, m_o, rtol=1e-3, atol=1e-3).all(-1)
    assert close.mean() > frac, close.mean()
    return film


@pytest.mark.parametrize("estimator", [N.EST_REF_NEE, N.EST_NEE_MIS])
def test_textured_cornell_matches_oracle(renderer, estimator):
    sc, cam = S.textured_cornell(3)
    job = N.job_desc(0, cam, 48, 48, 4, 4, 6, seed=4, estimator=estimator)
    _compare(renderer, sc, job, 16)


def test_planar_fallback_and_spheres(renderer):
    sc, cam = S.textured_cornell(2)
    # the ball without uvs (planar fallback over its box) and a textured sphere light
    sc.meshes[0].uvs = None
    sc.add_sphere((0.25, 0.8, 0.4), 0.08, sc.add_material(N.DIFFUSE_EMITTER, [0, 0, 0, 3.0],
                                                          texture=sc.add_texture(N.TEX_CHECKER, (1, 1, 1),
                                                                                 (6, 5, 4), 12.0)))
    sc.add_sphere((0.75, 0.15, 0.3), 0.12, sc.add_material(N.LAMBERTIAN, [0, 0, 0], texture=0))
    job = N.job_desc(0, cam, 40, 40, 4, 4, 6, seed=9, estimator=N.EST_NEE_MIS)
    _compare(renderer, sc, job, 16)


def test_textures_move_with_objects(renderer):
    sc, cam = S.textured_cornell(2)
    S.with_motion(sc, seed=3, speed=0.5)
    job = N.job_desc(0, dict(cam, shutter=0.4), 40, 40, 4, 4, 6, seed=2, estimator=N.EST_NEE_MIS)
    _compare(renderer, sc, job, 16)


def test_box_matches_oracle(renderer):
    sc, cam = S.cornell_icosphere(2)
    tex = sc.add_texture(N.TEX_CHECKER, (0.1, 0.2, 0.6), (0.9, 0.8, 0.2), 25.0)
    sc.add_box((0.15, 0.0, 0.5), (0.45, 0.35, 0.8), sc.add_material(N.LAMBERTIAN, [0, 0, 0], texture=tex))
    sc.add_box((0.6, 0.0, 0.15), (0.85, 0.2, 0.4), sc.add_material(N.CONDUCTOR, [*S.GOLD_ETA, *S.GOLD_K, 0.2, 0.2]))
    job = N.job_desc(0, cam, 40, 40, 4, 4, 6, seed=3, estimator=N.EST_NEE_MIS)
    _compare(renderer, sc, job, 16)
    # closest-hit ids: the boxes' faces follow the scene's rectangles
    rng = np.random.default_rng(5)
    o = np.tile([0.5, 0.5, -1.0], (2048, 1)) + rng.normal(0, 0.02, (2048, 3))
    d = np.stack([rng.uniform(-0.35, 0.35, 2048), rng.uniform(-0.4, 0.2, 2048), np.ones(2048)], 1)
    rays = np.concatenate([o, d], 1).astype(np.float32)
    sid = renderer.upload(sc)
    t, prim, _ = renderer.trace_closest(sid, rays)
    renderer.release(sid)
    osc = O.OracleScene(sc)
    t_o, prim_o = osc.trace_closest(rays)
    assert (prim == prim_o).mean() > 0.999
    both = (prim == prim_o) & (prim >= 0)
    assert np.allclose(t[both], t_o[both], rtol=1e-5)


@pytest.mark.parametrize("estimator", [N.EST_REF_NEE, N.EST_NEE_MIS])
def test_hair_curves_match_oracle(renderer, estimator):
    sc, cam = S.hair_curves(120, seed=4)
    job = N.job_desc(0, cam, 40, 40, 4, 4, 6, seed=5, estimator=estimator)
    _compare(renderer, sc, job, 16, frac=0.85)
    # closest hits on curves: same primitive, t within 1e-5
    rng = np.random.default_rng(7)
    o = np.tile([0.0, 0.7, -3.0], (4096, 1))
    d = np.stack([rng.uniform(-0.3, 0.3, 4096), rng.uniform(-0.35, 0.15, 4096), np.ones(4096)], 1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d], 1).astype(np.float32)
    sid = renderer.upload(sc)
    t, prim, _ = renderer.trace_closest(sid, rays)
    renderer.release(sid)
    t_o, prim_o = O.OracleScene(sc).trace_closest(rays)
    assert (prim == prim_o).mean() > 0.995
    both = (prim == prim_o) & (prim >= 0)
    assert np.allclose(t[both], t_o[both], rtol=1e-5)
    assert (prim >= 3).sum() > 100  # the rays do hit curves


def test_hair_curves_match_reference_image(renderer, golden):
    """The GPU render of hair on curves (explicit sigma_a) against the
    reference's own render (fixture): image means within 3 sigma."""
    sc, cam = S.hair_curves(40, seed=2)
    sc.materials = [(t, ([0.25, 0.45, 0.9] + list(p[3:])) if t == N.HAIR else p, 0 if t == N.HAIR else f)
                    for t, p, f in sc.materials]
    g = golden("image_haircurves.npz")
    sid = renderer.upload(sc)
    film = renderer.render(N.job_desc(sid, cam, 24, 24, 16, 16, 6, seed=3))
    renderer.release(sid)
    se = np.sqrt(2.0 * g["var"].reshape(-1, 3).sum(0) / 256) / (24 * 24)
    z = (film.reshape(-1, 3).mean(0) - g["mean"].reshape(-1, 3).mean(0)) / se
    assert np.all(np.abs(z) < 3.0), z


def test_material_mix_matches_reference_image(renderer, golden):
    """Every surface family of the mix scene on the GPU (Disney, hair, thin
    dielectric, Lambertian; sphere and area lights) against the reference's
    own render (fixture): image means within 3 sigma per channel."""
    from conftest import material_mix_for_reference

    g = golden("image_materials.npz")
    sc, cam = material_mix_for_reference()
    sid = renderer.upload(sc)
    film = renderer.render(N.job_desc(sid, cam, 32, 32, 8, 8, 6, seed=3))
    renderer.release(sid)
    se = np.sqrt(2.0 * g["var"].reshape(-1, 3).sum(0) / 64) / (32 * 32)
    z = (film.reshape(-1, 3).mean(0) - g["mean"].reshape(-1, 3).mean(0)) / se
    assert np.all(np.abs(z) < 3.0), z
