"""GPU: pt_render_device_noalloc, the render entry point that allocates no
device memory.

It is meant for callers that cannot allocate device memory while they render
(a host whose own device memory pool forbids other allocators, a real-time
loop that must not block in the allocator).  Its work buffers live in one
fixed device array inside the library, so its result must equal
pt_render_device's on the same job, and after a warm-up call a render must
leave the device's free memory unchanged.  The file runs last so that a
failure here leaves every other test already run.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S

pytestmark = pytest.mark.gpu


def _film(renderer, fn, job):
    film = torch.zeros(job.height * job.width * 3, dtype=torch.float32, device="cuda:0")
    st = N.Stats()
    if fn == "noalloc":
        rc = renderer.lib.pt_render_device_noalloc(renderer.ctx, C.byref(job), C.c_void_p(film.data_ptr()),
                                                   C.byref(st))
    else:
        rc = renderer.lib.pt_render_device(renderer.ctx, C.byref(job), C.c_void_p(film.data_ptr()), 1,
                                           C.byref(st))
    assert rc == 0, rc
    torch.cuda.synchronize()
    return film.cpu().numpy().reshape(job.height, job.width, 3), st


def test_noalloc_matches_render_device_twice():
    r = N.Renderer(0)
    sc, cam = S.cornell_icosphere(3)
    sid = r.upload(sc)
    # 128 x 128 x 16 spp = 262,144 paths: more than one wave of the fixed array
    job = N.job_desc(sid, cam, 128, 128, 4, 4, 8, seed=21, estimator=N.EST_NEE_MIS)
    want, st_want = _film(r, "device", job)
    for _ in range(2):  # the shared array keeps the previous call's contents
        got, st = _film(r, "noalloc", job)
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
        assert st.paths == st_want.paths and st.segments == st_want.segments
    r.release(sid)
    r.close()


def test_noalloc_rejects_sizes_beyond_its_limit():
    r = N.Renderer(0)
    sc, cam = S.cornell_icosphere(1)
    sid = r.upload(sc)
    job = N.job_desc(sid, cam, 8, 8, 256, 128, 4)  # 32768 samples per pixel > 16384
    film = torch.zeros(8 * 8 * 3, dtype=torch.float32, device="cuda:0")
    rc = r.lib.pt_render_device_noalloc(r.ctx, C.byref(job), C.c_void_p(film.data_ptr()), None)
    assert rc == -8  # PT_ERR_TOO_LARGE
    buf = C.create_string_buffer(256)
    r.lib.pt_last_error(r.ctx, buf, 256)
    assert b"16384" in buf.value
    r.release(sid)
    r.close()


def test_noalloc_allocates_no_device_memory():
    # a fresh context that never ran pt_render_device, so no queue buffers of
    # the context exist; the warm-up call loads the array (lazy module loading)
    r = N.Renderer(0)
    sc, cam = S.cornell_icosphere(3)
    sid = r.upload(sc)
    job = N.job_desc(sid, cam, 128, 128, 4, 4, 8, seed=5, estimator=N.EST_NEE_MIS)  # several waves
    film = torch.zeros(job.height * job.width * 3, dtype=torch.float32, device="cuda:0")
    lib = r.lib
    assert lib.pt_render_device_noalloc(r.ctx, C.byref(job), C.c_void_p(film.data_ptr()), None) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(2):
        assert lib.pt_render_device_noalloc(r.ctx, C.byref(job), C.c_void_p(film.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0
    r.release(sid)
    r.close()
