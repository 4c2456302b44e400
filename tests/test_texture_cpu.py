"""Surface textures in the oracle and the host scene build (CPU only)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import pyoracle as O
from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S


def test_textured_scene_builds_and_renders():
    sc, cam = S.textured_cornell(2)
    info = N.bvh_build(sc)
    assert info["items"] == 6 + 320
    job = N.job_desc(0, cam, 16, 16, 2, 2, 5, seed=3, estimator=N.EST_NEE_MIS)
    a, _ = O.render(sc, job)
    assert np.isfinite(a).all() and a.mean() > 0
    # the textures change the image
    plain, _ = S.textured_cornell(2)
    plain.materials = [(t, p, f & ((1 << N.MAT_TEXTURE_SHIFT) - 1)) for t, p, f in plain.materials]
    plain.materials = [(t, [0.5, 0.5, 0.5] + p[3:] if t == N.LAMBERTIAN else ([10, 10, 10] + p[3:] if t == N.DIFFUSE_EMITTER else p), f)
                       for t, p, f in plain.materials]
    b, _ = O.render(plain, job)
    assert not np.allclose(a, b)


def test_texture_index_is_validated():
    sc, _ = S.textured_cornell(1)
    t, p, f = sc.materials[1]
    sc.materials[1] = (t, p, (99 << N.MAT_TEXTURE_SHIFT))
    with pytest.raises(N.PtError):
        N.bvh_build(sc)
    sc, _ = S.textured_cornell(1)
    sc.textures[2]["texels"] = np.zeros((1, 5, 3), np.float32)  # image smaller than 2x2
    with pytest.raises(N.PtError):
        N.bvh_build(sc)
