"""GPU: the stratified sample values a job's paths draw (pt_sample_eval, the
device code of the camera and shade stages) against the oracle, bit for bit,
and their strata:

* the pixel grid of FrameBuffer::setOffsets / getOffsets
  (framebuffer.cpp:131-145, utils/random.hpp:47-63): one jittered
  spp_x x spp_y grid per frame, sample k in cell (k / spp_y, k % spp_y);
* the per-vertex light-point grid of maxdepth_nee.hpp:91 (getOffsets(2, 2)
  by default), light sample ls in cell (ls / ny, ls % ny);
* PT_SAMPLER_STRATIFIED per-bounce dimensions: over a pixel's spp samples
  every dimension takes each of the spp strata exactly once.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _job(sid, cam, sampler, sx=16, sy=8, w=12, h=10, **kw):
    return N.job_desc(sid, cam, w, h, sx, sy, 6, seed=kw.pop("seed", 9), sampler=sampler, **kw)


@pytest.fixture(scope="module")
def scene_id(renderer):
    sc, cam = S.cornell_icosphere(1)
    sid = renderer.upload(sc)
    yield sid, cam
    renderer.release(sid)


@pytest.mark.parametrize("sampler", [N.SAMPLER_STRATIFIED, N.SAMPLER_HALTON_OWEN, N.SAMPLER_HALTON_PERMUTE])
def test_path_samples_bit_exact_oracle(renderer, scene_id, sampler):
    sid, cam = scene_id
    job = _job(sid, cam, sampler, sampler_seed=4)
    npix = job.width * job.height
    for first, n in ((0, 3 * npix + 7), (57 * npix + 3, 2 * npix)):
        got = renderer.sample_eval(job, first, n, 24, 4)
        want = O.path_samples(job, first, n, 24, 4)
        for g, w in zip(got, want):
            assert g.shape == w.shape
            assert np.array_equal(g.view(np.uint32), w.view(np.uint32))


def test_path_samples_window_and_light_grid_bit_exact(renderer, scene_id):
    sid, cam = scene_id
    job = _job(sid, cam, N.SAMPLER_STRATIFIED, sx=3, sy=5, light_samples=(3, 2))
    job.crop_x, job.crop_y, job.full_width, job.full_height = 5, 2, 40, 30
    n = job.width * job.height * 15
    got = renderer.sample_eval(job, 0, n, 8, 3)
    want = O.path_samples(job, 0, n, 8, 3)
    for g, w in zip(got, want):
        assert np.array_equal(g.view(np.uint32), w.view(np.uint32))


def test_pixel_and_light_grids_are_stratified(renderer, scene_id):
    sid, cam = scene_id
    job = _job(sid, cam, N.SAMPLER_STRATIFIED, sx=16, sy=8)
    npix, spp = job.width * job.height, 128
    pix, dv, lo = renderer.sample_eval(job, 0, npix * spp, 12, 3)
    k = np.arange(npix * spp) // npix
    i, j = k // 8, k % 8
    assert np.all((pix[:, 0] >= i / 16) & (pix[:, 0] < (i + 1) / 16))
    assert np.all((pix[:, 1] >= j / 8) & (pix[:, 1] < (j + 1) / 8))
    # one grid per frame: every pixel draws the same offset for sample k
    assert np.array_equal(pix.reshape(spp, npix, 2), np.broadcast_to(pix.reshape(spp, npix, 2)[:, :1], (spp, npix, 2)))
    ls = np.arange(4)
    assert np.all((lo[..., 0] >= (ls // 2) / 2) & (lo[..., 0] < (ls // 2 + 1) / 2))
    assert np.all((lo[..., 1] >= (ls % 2) / 2) & (lo[..., 1] < (ls % 2 + 1) / 2))
    # per-bounce dimensions: each pixel's spp samples cover the spp strata
    # once -- the k-th smallest value lies in [k / spp, (k + 1) / spp] (closed:
    # stratum + jitter may round up to the next stratum's edge in FP32)
    assert np.all((dv >= 0) & (dv < 1))
    srt = np.sort(dv.reshape(spp, npix, 12).astype(np.float64), axis=0)
    k = np.arange(spp)[:, None, None]
    assert np.all((srt >= k / spp) & (srt <= (k + 1) / spp))


def test_path_samples_rejects_out_of_range(renderer, scene_id):
    sid, cam = scene_id
    job = _job(sid, cam, N.SAMPLER_STRATIFIED)
    with pytest.raises(N.PtError):
        renderer.sample_eval(job, job.width * job.height * 128 - 2, 4, 2, 0)
