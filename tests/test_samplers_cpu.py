"""CPU: the oracle's stratified sample values (or_path_samples) keep the
strata of the reference's getOffsets (utils/random.hpp:47-63): the pixel grid
of FrameBuffer::setOffsets (framebuffer.cpp:131-145), one grid per frame with
sample k in cell (k / spp_y, k % spp_y); the per-vertex light-point grid of
maxdepth_nee.hpp:91; and the stratified per-bounce dimensions cover each
pixel's spp strata once.  (The reference draws the jitter with a
random-seeded mt19937; the build's counter generator replaces it, so the
strata are what pins these values, and the GPU matches the oracle bit for
bit.)"""
from __future__ import annotations

import numpy as np

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S


def test_oracle_pixel_grid_light_grid_and_strata():
    _, cam = S.cornell_icosphere(0)
    job = N.job_desc(0, cam, 6, 5, 4, 3, 4, seed=3, sampler=N.SAMPLER_STRATIFIED, light_samples=(2, 3))
    npix, spp = 30, 12
    pix, dv, lo = O.path_samples(job, 0, npix * spp, 6, 2)
    k = np.arange(npix * spp) // npix
    assert np.all((pix[:, 0] >= (k // 3) / 4) & (pix[:, 0] < (k // 3 + 1) / 4))
    assert np.all((pix[:, 1] >= (k % 3) / 3) & (pix[:, 1] < (k % 3 + 1) / 3))
    ls = np.arange(6)
    assert np.all((lo[..., 0] >= (ls // 3) / 2) & (lo[..., 0] < (ls // 3 + 1) / 2))
    assert np.all((lo[..., 1] >= (ls % 3) / 3) & (lo[..., 1] < (ls % 3 + 1) / 3))
    srt = np.sort(dv.reshape(spp, npix, 6).astype(np.float64), axis=0)
    kk = np.arange(spp)[:, None, None]
    assert np.all((srt >= kk / spp) & (srt <= (kk + 1) / spp))


def test_oracle_halton_dims_equal_sampler_eval():
    # with a Halton sampler the per-path dimensions are the sampler at the
    # path's index 1 + ((i * H + j) * spp + k) (renderManager.hpp:99-115 order)
    _, cam = S.cornell_icosphere(0)
    W, H, spp = 4, 3, 4
    job = N.job_desc(0, cam, W, H, 2, 2, 4, sampler=N.SAMPLER_HALTON_OWEN)
    _, dv, _ = O.path_samples(job, 0, W * H * spp, 9, 0)
    g = np.arange(W * H * spp)
    q, k = g % (W * H), g // (W * H)
    i, j = q % W, q // W
    idx = 1 + (i * H + j) * spp + k
    ref = O.sampler_eval(N.SAMPLER_HALTON_OWEN, 1, W * H * spp, 9)
    assert np.array_equal(dv.view(np.uint32), ref[idx - 1].view(np.uint32))
