"""Motion blur and depth of field in the oracle and the host-side helpers
(CPU only)."""
from __future__ import annotations

import numpy as np

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S


def test_oracle_zero_shutter_equals_static():
    static, cam = S.cornell_icosphere(2)
    moving, _ = S.cornell_icosphere(2)
    S.with_motion(moving, seed=5, speed=0.6)
    job = N.job_desc(0, cam, 12, 12, 2, 2, 6, seed=2, estimator=N.EST_NEE_MIS)
    a, _ = O.render(static, job)
    b, _ = O.render(moving, job)
    assert np.array_equal(a, b)


def test_oracle_motion_changes_image():
    sc, cam = S.cornell_icosphere(2)
    S.with_motion(sc, seed=5, speed=0.6)
    job0 = N.job_desc(0, cam, 12, 12, 2, 2, 6, seed=2)
    job1 = N.job_desc(0, dict(cam, shutter=0.5), 12, 12, 2, 2, 6, seed=2)
    a, _ = O.render(sc, job0)
    b, _ = O.render(sc, job1)
    assert not np.array_equal(a, b)
    assert np.isfinite(b).all()


def test_lens_mapping():
    cam = S.camera((0, 0, 0), (0, 0, 1), 40.0, 1.0, focal_dist=2.0)
    c = S.with_lens(cam, 0.05)
    # PerspectiveCamera: lens radius = focalDist / aperture * 0.5
    assert abs(c["focal_dist"] / c["aperture"] * 0.5 - 0.025) < 1e-9
    assert S.with_lens(cam, 0.0)["focal_dist"] / S.with_lens(cam, 0.0)["aperture"] < 1e-8


def test_job_mix_is_seeded_and_in_range():
    sc, cam = S.cornell_icosphere(1)
    a = S.job_mix({"cornell": (1, cam, 1.9)}, 40, seed=3)
    b = S.job_mix({"cornell": (1, cam, 1.9)}, 40, seed=3)
    assert [bytes(x) for x in a] == [bytes(x) for x in b]
    for j in a:
        assert 64 <= j.width <= 1024 and j.width == j.height
        assert 4 <= j.spp_x * j.spp_y <= 256
        assert 0.0 <= j.camera.shutter <= 0.5
        assert j.camera.focal_dist / j.camera.aperture <= 0.05 + 1e-6


def test_oracle_window_equals_frame_pixels():
    sc, cam = S.material_divergence(subdiv=1, seed=3, aspect=1.0)
    full = N.job_desc(0, cam, 20, 16, 2, 2, 4, seed=4, estimator=N.EST_NEE_MIS, sampler=N.SAMPLER_STRATIFIED)
    a, _ = O.render(sc, full)
    win = N.job_desc(0, cam, 7, 5, 2, 2, 4, seed=4, estimator=N.EST_NEE_MIS, sampler=N.SAMPLER_STRATIFIED)
    win.crop_x, win.crop_y, win.full_width, win.full_height = 9, 6, 20, 16
    b, _ = O.render(sc, win)
    assert np.array_equal(a[6:11, 9:16], b)
