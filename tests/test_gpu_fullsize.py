"""The headline workload at its full size (1,310,720-triangle rough-glass
scene, 1024x512 HDRI, 1024x1024, depth 16, roulette from 4, NEE+MIS, Owen
Halton, alias env sampling), checked through properties that do not depend
on size:

* determinism: the same job renders the same bits;
* non-finite samples: the rare sample whose arithmetic gives NaN (one pixel
  in 10^6 at 16 spp here) is the oracle's NaN too, at the same pixel and
  sample -- the reference's algorithm produces it; the film keeps it as the
  reference's pixel sum does and the tone map writes it as 0 as
  FrameBuffer::writeToFile does;
* sample-range additivity: samples [0, 8) then [8, 16) accumulated onto a
  device film give the bits of [0, 16) in one call (the film adds a pixel's
  samples one by one in sample order);
* windows: a window job equals those pixels of the full frame;
* parity: on a window of the full frame the oracle (same scene, same sample
  streams) agrees pixel by pixel, and the window means agree within 3 sigma.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S

pytestmark = pytest.mark.gpu

W = H = 1024


@pytest.fixture(scope="module")
def headline(renderer):
    sc, cam = S.rough_glass(8)
    sid = renderer.upload(sc)
    yield sc, cam, sid
    renderer.release(sid)


def _job(sid, cam, b, e, **kw):
    return N.job_desc(sid, cam, W, H, 16, 16, 16, rr_start=4, estimator=N.EST_NEE_MIS,
                      sampler=N.SAMPLER_HALTON_OWEN, env_sampling=N.ENV_ALIAS, seed=1, spp_begin=b, spp_end=e,
                      **kw)


def _device_film(renderer, jobs):
    film = torch.zeros(H * W * 3, dtype=torch.float32, device="cuda:0")
    for j in jobs:
        renderer.render_device(j, film.data_ptr(), sync=True)
    return film


def _bits(film):
    return film.view(torch.int32)


def test_full_size_deterministic_and_additive(renderer, headline):
    _, cam, sid = headline
    one = _device_film(renderer, [_job(sid, cam, 0, 16)])
    again = _device_film(renderer, [_job(sid, cam, 0, 16)])
    split = _device_film(renderer, [_job(sid, cam, 0, 8), _job(sid, cam, 8, 16)])
    assert torch.equal(_bits(one), _bits(again))
    assert torch.equal(_bits(one), _bits(split))
    fin = torch.isfinite(one)
    assert float(one[fin].min()) >= 0.0
    assert int((~fin).sum()) <= 3 * 8  # at most 8 pixels of 10^6


def test_full_size_non_finite_samples_are_the_oracles(renderer, headline):
    sc, cam, sid = headline
    film = renderer.render(_job(sid, cam, 0, 16))
    ys, xs = np.nonzero(~np.isfinite(film).all(-1))
    osc = O.OracleScene(sc) if len(ys) else None
    for y, x in list(zip(ys, xs))[:2]:
        found = False
        for k in range(16):
            w = _job(sid, cam, k, k + 1)
            w.width, w.height = 1, 1
            w.crop_x, w.crop_y, w.full_width, w.full_height = int(x), int(y), W, H
            g = renderer.render(w)
            if np.isfinite(g).all():
                continue
            w.scene = 0
            m, _ = osc.render(w)
            assert not np.isfinite(m).all(), (x, y, k, g, m)
            found = True
            break
        assert found
    # the tone map writes NaN as 0 (framebuffer.cpp:27-58), rows flipped
    if len(ys):
        rgb8 = renderer.tonemap(film)
        nan_c = np.isnan(film[ys[0], xs[0]])
        assert (rgb8[H - 1 - ys[0], xs[0]][nan_c] == 0).all()


def test_full_size_window_equals_frame(renderer, headline):
    _, cam, sid = headline
    full = renderer.render(_job(sid, cam, 0, 2))
    win = _job(sid, cam, 0, 2)
    win.width, win.height = 64, 48
    win.crop_x, win.crop_y, win.full_width, win.full_height = 480, 500, W, H
    assert np.array_equal(renderer.render(win), full[500:548, 480:544])


def test_full_size_window_matches_oracle(renderer, headline):
    sc, cam, sid = headline
    win = _job(sid, cam, 0, 16)
    win.width, win.height = 12, 12
    win.crop_x, win.crop_y, win.full_width, win.full_height = 506, 470, W, H  # the glass's silhouette
    film = renderer.render(win)
    win.scene = 0
    m_o, v_o = O.render(sc, win)
    close = np.isclose(film, m_o, rtol=1e-3, atol=1e-3).all(-1)
    assert close.mean() > 0.9, close.mean()
    se = np.sqrt(2 * v_o.reshape(-1, 3).sum(0) / 16) / (12 * 12)
    z = (film.reshape(-1, 3).mean(0) - m_o.reshape(-1, 3).mean(0)) / np.maximum(se, 1e-12)
    assert np.all(np.abs(z) < 3.0), z


def test_full_size_paired_tail_equals_separate(renderer, headline, monkeypatch):
    """A large wave with roulette traces each bounce's shadow rays with the
    next bounce's closest rays once the queues thin out (from the roulette
    start); the film has the bits of separate launches."""
    sc, cam, sid = headline
    monkeypatch.setenv("PT_PAIR_FROM_BOUNCE", "1000000")
    sep = N.Renderer(0)
    monkeypatch.delenv("PT_PAIR_FROM_BOUNCE")
    try:
        sid2 = sep.upload(sc)
        a = renderer.render(_job(sid, cam, 0, 2))
        b = sep.render(_job(sid2, cam, 0, 2))
        assert np.array_equal(a.view(np.int32), b.view(np.int32))
        sep.release(sid2)
    finally:
        sep.close()
