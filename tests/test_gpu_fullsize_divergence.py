"""The material-divergence workload at its full size (64 icospheres of
20,480 triangles with Disney, hair, thin-dielectric, Phong and Lambertian
materials in a homogeneous medium, 4 sphere and 2 area lights, 1920x1080,
128 spp as 16 x 8, depth 12, stratified sampler, REF_NEE), checked through
properties that do not depend on size:

* determinism: the same job renders the same bits;
* windows: a window job equals those pixels of the full frame;
* parity: on windows of the full frame at every sample the oracle (same
  scene, same sample streams) agrees pixel by pixel, and the window means
  agree within 3 sigma.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S

pytestmark = pytest.mark.gpu

W, H = 1920, 1080


@pytest.fixture(scope="module")
def divergence(renderer):
    sc, cam = S.material_divergence(5)
    sid = renderer.upload(sc)
    yield sc, cam, sid
    renderer.release(sid)


def _job(sid, cam, b, e, estimator=N.EST_REF_NEE):
    return N.job_desc(sid, cam, W, H, 16, 8, 12, estimator=estimator, sampler=N.SAMPLER_STRATIFIED, seed=1,
                      spp_begin=b, spp_end=e)


def _window(job, x, y, w, h):
    job.width, job.height = w, h
    job.crop_x, job.crop_y, job.full_width, job.full_height = x, y, W, H
    return job


def test_divergence_full_frame_deterministic_and_windowed(renderer, divergence):
    _, cam, sid = divergence
    a = renderer.render(_job(sid, cam, 0, 2))
    b = renderer.render(_job(sid, cam, 0, 2))
    assert np.array_equal(a.view(np.int32), b.view(np.int32))
    win = renderer.render(_window(_job(sid, cam, 0, 2), 900, 500, 64, 40))
    assert np.array_equal(win, a[500:540, 900:964])
    assert np.isfinite(a).mean() > 0.999


@pytest.mark.parametrize("estimator", [N.EST_REF_NEE, N.EST_NEE_MIS])
@pytest.mark.parametrize("x,y", [(944, 524), (600, 300)])
def test_divergence_full_size_window_matches_oracle(renderer, divergence, estimator, x, y):
    sc, cam, sid = divergence
    win = _window(_job(sid, cam, 0, 128, estimator), x, y, 16, 16)
    film = renderer.render(win)
    win.scene = 0
    m_o, v_o = O.render(sc, win)
    fin = np.isfinite(m_o).all(-1) & np.isfinite(film).all(-1)
    close = np.isclose(film, m_o, rtol=1e-3, atol=1e-3).all(-1)
    assert close[fin].mean() > 0.9, close[fin].mean()
    se = np.sqrt(2 * v_o[fin].reshape(-1, 3).sum(0) / 128) / fin.sum()
    z = (film[fin].reshape(-1, 3).mean(0) - m_o[fin].reshape(-1, 3).mean(0)) / np.maximum(se, 1e-12)
    assert np.all(np.abs(z) < 3.0), z
