"""Frame windows and converged references.

A window job (crop_x/crop_y/full_width/full_height) renders pixels of a larger
frame with that frame's sample streams, so it equals those pixels of the full
render.  The benchmark's converged reference (65536 spp on a window, rendered
on the GPU) is spot-checked here against the oracle on a small window at high
spp: same sample streams, so the two agree pixel by pixel, and their image
means agree within 3 sigma.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _window(job, x0, y0, w, h, fw, fh):
    j = type(job).from_buffer_copy(job)
    j.width, j.height = w, h
    j.crop_x, j.crop_y, j.full_width, j.full_height = x0, y0, fw, fh
    return j


def test_window_equals_frame_pixels(renderer):
    sc, cam = S.material_divergence(subdiv=2, seed=3, aspect=1.0)
    sid = renderer.upload(sc)
    full = N.job_desc(sid, cam, 48, 40, 2, 2, 6, seed=4, estimator=N.EST_NEE_MIS, sampler=N.SAMPLER_STRATIFIED)
    a = renderer.render(full)
    b = renderer.render(_window(full, 13, 9, 17, 11, 48, 40))
    renderer.release(sid)
    assert np.array_equal(a[9:20, 13:30], b)


def test_window_outside_frame_rejected(renderer):
    sc, cam = S.cornell_icosphere(1)
    sid = renderer.upload(sc)
    full = N.job_desc(sid, cam, 16, 16, 1, 1, 2)
    with pytest.raises(N.PtError):
        renderer.render(_window(full, 10, 0, 8, 8, 16, 16))
    bad = N.job_desc(sid, cam, 16, 16, 1, 1, 2)
    bad.crop_x = 3  # an origin without a frame
    with pytest.raises(N.PtError):
        renderer.render(bad)
    renderer.release(sid)


@pytest.mark.parametrize("workload", ["cornell", "rough_glass"])
def test_converged_window_spot_check(renderer, workload):
    if workload == "cornell":
        sc, cam = S.cornell_icosphere(3)
        full = N.job_desc(0, cam, 256, 256, 64, 64, 8, seed=9, estimator=N.EST_NEE_MIS)
        win = _window(full, 120, 100, 8, 8, 256, 256)
    else:
        sc, cam = S.rough_glass(subdiv=4, env_w=256, env_h=128, seed=2)
        full = N.job_desc(0, cam, 1024, 1024, 64, 64, 16, seed=9, estimator=N.EST_NEE_MIS,
                          env_sampling=N.ENV_ALIAS, rr_start=4)
        win = _window(full, 508, 508, 8, 8, 1024, 1024)
    sid = renderer.upload(sc)
    win.scene = sid
    g = renderer.render(win)
    renderer.release(sid)
    win.scene = 0
    m_o, v_o = O.render(sc, win)
    spp = 64 * 64
    se = np.sqrt(2 * v_o.reshape(-1, 3).sum(0) / spp) / 64
    z = (g.reshape(-1, 3).mean(0) - m_o.reshape(-1, 3).mean(0)) / np.maximum(se, 1e-12)
    assert np.all(np.abs(z) < 3.0), z
    close = np.isclose(g, m_o, rtol=1e-2, atol=1e-3).all(-1)
    assert close.mean() > 0.9, close.mean()


@pytest.mark.parametrize("k,sigma", [(3, 0.8), (7, 2.0), (15, 5.0)])
def test_gaussian_blur_matches_oracle(renderer, k, sigma):
    rng = np.random.default_rng(k)
    film = (rng.random((23, 37, 3)) ** 3 * 20).astype(np.float32)
    got = renderer.gaussian_blur(film, k, sigma)
    want = O.gaussian_blur(film, k, sigma)
    assert np.array_equal(got, want)  # same weights, same tap order, no fused operations


def test_gaussian_blur_refused_arguments(renderer):
    film = np.random.default_rng(3).random((8, 8, 3)).astype(np.float32)
    for k, s in ((4, 1.0), (1, 1.0), (5, -1.0), (5, 0.0)):
        assert np.array_equal(renderer.gaussian_blur(film, k, s), film)
