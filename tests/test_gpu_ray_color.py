"""GPU: pt_ray_color, getRayColor (include/integrator/maxdepth_nee.hpp:9-256)
for given primary rays, against the oracle's restatement of the reference
integrator on the same rays and sample streams (path i draws Halton index
first_index + i): per path within 1e-3 for >= 95 % of the paths (a path
whose roulette or lobe choice sits on an FP32 rounding edge may take the
other branch), and the mean radiance within 3 sigma."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _rays(n, rng, eye):
    o1 = np.tile(np.array(eye, np.float32), (n // 2, 1))
    tgt = np.stack([rng.uniform(0, 1, n // 2), rng.uniform(0, 1, n // 2), np.ones(n // 2)], 1)
    o2 = rng.uniform(0.05, 0.95, size=(n - n // 2, 3))
    d2 = rng.normal(size=(n - n // 2, 3))
    return np.concatenate([np.concatenate([o1, tgt - o1], 1), np.concatenate([o2, d2], 1)], 0).astype(np.float32)


def _compare(got, want):
    assert np.isfinite(got).all()
    close = np.isclose(got, want, rtol=1e-3, atol=1e-4).all(1)
    assert close.mean() >= 0.95, close.mean()
    se = want.std(0) / np.sqrt(len(want)) * np.sqrt(2.0) + 1e-6
    assert np.all(np.abs(got.mean(0) - want.mean(0)) < 3 * se), (got.mean(0), want.mean(0))


@pytest.mark.parametrize("estimator", [N.EST_REF_NEE, N.EST_NEE_MIS])
def test_ray_color_matches_oracle_cornell(renderer, estimator):
    sc, cam = S.cornell_icosphere(3)
    sid = renderer.upload(sc)
    rays = _rays(4096, np.random.default_rng(3), cam["position"])
    job = N.job_desc(sid, cam, 1, 1, 1, 1, 8, seed=11, estimator=estimator)
    got = renderer.ray_color(job, rays, first_index=1001)
    job.scene = 0
    want = O.OracleScene(sc).ray_color(job, rays, first_index=1001)
    _compare(got, want)
    # the index base moves the sample streams: another base, other paths
    job.scene = sid
    other = renderer.ray_color(job, rays, first_index=77)
    assert not np.array_equal(other, got)
    renderer.release(sid)


def test_ray_color_rough_glass_hdri_roulette(renderer):
    sc, cam = S.rough_glass(3)
    sid = renderer.upload(sc)
    rng = np.random.default_rng(8)
    eye = np.array(cam["position"], np.float32)
    d = np.array(cam["front"], np.float32) + rng.normal(scale=0.15, size=(3000, 3))
    rays = np.concatenate([np.tile(eye, (3000, 1)), d], 1).astype(np.float32)
    job = N.job_desc(sid, cam, 1, 1, 1, 1, 16, seed=2, rr_start=4, estimator=N.EST_NEE_MIS,
                     env_sampling=N.ENV_ALIAS)
    got = renderer.ray_color(job, rays, first_index=1)
    job.scene = 0
    want = O.OracleScene(sc).ray_color(job, rays, first_index=1)
    _compare(got, want)
    renderer.release(sid)


def test_ray_color_rejects_bad_index(renderer):
    sc, cam = S.cornell_icosphere(1)
    sid = renderer.upload(sc)
    job = N.job_desc(sid, cam, 1, 1, 1, 1, 4)
    with pytest.raises(N.PtError):
        renderer.ray_color(job, np.zeros((2, 6), np.float32) + 0.5, first_index=0)
    renderer.release(sid)
