"""The Light interface (include/light/light.hpp:17-306, envLight.hpp:4-92) of
the lights a scene's render samples -- get_sample, get_normal_at, the
direction from a shading point, L_emit towards it and pdf_value, get_area --
against the reference's own QuadLight / SphereLight / EnvironmentLight on the
same scene (fixture tests/golden/lights.npz, written through oracle/ref from
the LightList that discover_emissive_objects_as_lights and the environment
give, in that order).

CPU: the oracle's restatement.  GPU: pt_light_sample through the C-ABI (the
device code next-event estimation runs).  Bars: points, normals, directions
and radiance within 1e-5 relative (the GPU evaluates sin/cos(2 pi u) as
sincospi, without the reference's rounding of 2 pi u; vector components
relative to the vector's length), pdf_value within
1e-4 relative, areas equal to 1e-6."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_close

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
GOLD = Path(__file__).resolve().parent / "golden" / "lights.npz"


def _light_scene():
    from make_golden import light_scene
    return light_scene()


def _check(g, li, got):
    pre = f"light{li}__"
    for k in ("point", "normal", "dir"):
        # vectors: component errors relative to the vector's length (an
        # environment point is a direction times 1e5)
        err = np.abs(got[k] - g[pre + k]).max(1) / np.linalg.norm(g[pre + k], axis=1)
        assert (err <= 1e-5).all(), (li, k, err.max())
    assert rel_close(got["le"], g[pre + "le"], rtol=1e-5, atol=1e-6), (li, np.abs(got["le"] - g[pre + "le"]).max())
    assert rel_close(got["pdf"], g[pre + "pdf"], rtol=1e-4, atol=1e-7), (li, np.abs(got["pdf"] - g[pre + "pdf"]).max())
    # pdf_value at other directions: equal where both agree that the ray
    # meets the light (a direction grazing a quad's edge may fall either side)
    a, b = got["pdf_at_dir"], g[pre + "pdf_at_dir"]
    assert ((a > 0) == (b > 0)).mean() >= 0.995, li
    both = (a > 0) & (b > 0)
    assert rel_close(a[both], b[both], rtol=1e-4, atol=1e-7), (li, np.abs(a - b)[both].max())
    a, b = got["area"], float(g[pre + "area"])
    assert (np.isinf(a) and np.isinf(b)) or abs(a - b) <= 1e-6 * abs(b), (li, a, b)


def test_oracle_lights_match_reference():
    from oracle import pyoracle as O
    g = np.load(GOLD)
    osc = O.OracleScene(_light_scene())
    assert osc.lib.or_scene_num_lights(osc.h) == int(g["n_lights"])
    for li in range(int(g["n_lights"])):
        got = osc.light_eval(li, g[f"light{li}__uv"], g[f"light{li}__x"])
        got["pdf_at_dir"] = osc.light_eval(li, g[f"light{li}__uv"], g[f"light{li}__x"], g[f"light{li}__pdf_dir"])["pdf"]
        _check(g, li, got)


@pytest.mark.gpu
def test_gpu_lights_match_reference(renderer):
    from pathtracer_gb300 import native as N
    g = np.load(GOLD)
    sid = renderer.upload(_light_scene())
    assert renderer.scene_info(sid)["lights"] == int(g["n_lights"])
    for li in range(int(g["n_lights"])):
        got = renderer.light_sample(sid, li, g[f"light{li}__uv"], g[f"light{li}__x"])
        got["pdf_at_dir"] = renderer.light_sample(sid, li, g[f"light{li}__uv"], g[f"light{li}__x"],
                                                  g[f"light{li}__pdf_dir"])["pdf"]
        _check(g, li, got)
    with pytest.raises(N.PtError):
        renderer.light_sample(sid, int(g["n_lights"]), g["light0__uv"][:1], g["light0__x"][:1])
    renderer.release(sid)
