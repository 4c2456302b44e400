"""Motion blur and depth of field (the batched form's camera features).

The reference camera already has a lens (a square aperture of radius
focalDist / aperture * 0.5, camera.cpp:42-56); motion blur is an extension:
each object moves linearly over the shutter and a path's rays all use the
path's own time.  The oracle restates both, so images are compared with it
statistically (per-channel image mean within 3 sigma) and path by path.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _img_z(mean_a, var_a, mean_b, var_b, spp):
    se = np.sqrt((var_a + var_b).reshape(-1, 3).sum(0) / spp) / (mean_a.shape[0] * mean_a.shape[1])
    return (mean_a.reshape(-1, 3).mean(0) - mean_b.reshape(-1, 3).mean(0)) / se


def _compare(renderer, sc, job, spp, close_frac=0.9):
    sid = renderer.upload(sc)
    job.scene = sid
    film = renderer.render(job)
    job.scene = 0
    m_o, v_o = O.render(sc, job)
    renderer.release(sid)
    assert np.isfinite(film).all()
    z = _img_z(film, v_o, m_o, v_o, spp)
    assert np.all(np.abs(z) < 3.0), z
    close = np.isclose(film, m_o, rtol=1e-3, atol=1e-3).all(-1)
    assert close.mean() > close_frac, close.mean()
    return film


@pytest.mark.parametrize("estimator", [N.EST_REF_NEE, N.EST_NEE_MIS])
def test_motion_blur_cornell_matches_oracle(renderer, estimator):
    sc, cam = S.cornell_icosphere(3)
    S.with_motion(sc, seed=5, speed=0.6)
    cam = dict(cam, shutter=0.5)
    job = N.job_desc(0, cam, 40, 40, 4, 4, 8, seed=6, estimator=estimator)
    _compare(renderer, sc, job, 16)


def test_motion_blur_moving_sphere_lights_in_medium(renderer):
    sc, cam = S.material_divergence(subdiv=2, seed=3, aspect=1.0)
    S.with_motion(sc, seed=9, speed=1.0)
    assert any(o[0] == N.OBJ_SPHERE and any(o[2]) for o in sc.objects)
    cam = dict(cam, shutter=0.4)
    job = N.job_desc(0, cam, 40, 40, 4, 4, 6, seed=5, estimator=N.EST_NEE_MIS, sampler=N.SAMPLER_STRATIFIED)
    _compare(renderer, sc, job, 16, close_frac=0.8)


def test_depth_of_field_matches_oracle(renderer):
    sc, cam = S.cornell_icosphere(3)
    cam = S.with_lens(cam, 0.05, focal_dist=1.9)
    job = N.job_desc(0, cam, 40, 40, 4, 4, 8, seed=7, estimator=N.EST_NEE_MIS)
    _compare(renderer, sc, job, 16)


def test_zero_shutter_equals_static(renderer):
    static, cam = S.cornell_icosphere(3)
    moving, _ = S.cornell_icosphere(3)
    S.with_motion(moving, seed=5, speed=0.6)
    a_id, b_id = renderer.upload(static), renderer.upload(moving)
    ja = N.job_desc(a_id, cam, 32, 32, 2, 2, 8, seed=2, estimator=N.EST_NEE_MIS)
    jb = N.job_desc(b_id, cam, 32, 32, 2, 2, 8, seed=2, estimator=N.EST_NEE_MIS)
    a, b = renderer.render(ja), renderer.render(jb)
    renderer.release(a_id)
    renderer.release(b_id)
    # the moving scene's boxes are swept, its hits at time 0 are the static ones
    assert np.array_equal(a, b)


def test_motion_blur_changes_only_with_shutter(renderer):
    sc, cam = S.cornell_icosphere(3)
    S.with_motion(sc, seed=5, speed=0.6)
    sid = renderer.upload(sc)
    sharp = renderer.render(N.job_desc(sid, cam, 48, 48, 4, 4, 8, seed=2))
    sharp2 = renderer.render(N.job_desc(sid, dict(cam, shutter=0.0), 48, 48, 4, 4, 8, seed=2))
    blurred = renderer.render(N.job_desc(sid, dict(cam, shutter=0.5), 48, 48, 4, 4, 8, seed=2))
    renderer.release(sid)
    assert np.array_equal(sharp, sharp2)
    assert np.isfinite(blurred).all()
    assert not np.array_equal(sharp, blurred)


def test_shutter_limits(renderer):
    sc, cam = S.cornell_icosphere(2)
    S.with_motion(sc, seed=5, shutter_max=0.25)
    sid = renderer.upload(sc)
    with pytest.raises(N.PtError):
        renderer.render(N.job_desc(sid, dict(cam, shutter=0.5), 16, 16, 1, 1, 4))
    renderer.render(N.job_desc(sid, dict(cam, shutter=0.25), 16, 16, 1, 1, 4))
    renderer.release(sid)
    sc.shutter_max = 0.0
    with pytest.raises(N.PtError):
        renderer.upload(sc)
