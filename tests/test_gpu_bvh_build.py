"""BVH builders (pt_set_bvh_builder).  The device builder
(pt_bvh_build_device) builds the reference's median-split tree level by
level on the GPU: where no two centroids of a node tie along its split axis
it is the host recursion's tree node for node (equal content hash); with
ties it is another valid tree of the same split rule.  The SAH builder (the
default) builds other trees.  Every builder finds the same closest hits and
renders the same images as the reference's tree."""
from __future__ import annotations

import numpy as np
import pytest

from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_tree():
    """A context that uploads with the reference's trees."""
    r = N.Renderer(0)
    r.set_bvh_builder(N.BVH_BUILD_HOST)
    yield r
    r.close()


def _soup(n, seed):
    """n random small triangles in a box: distinct centroids on every axis."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, (n, 1, 3))
    pos = (c + rng.normal(0, 0.01, (n, 3, 3))).reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    return pos, idx


def _soup_scene(n, seed):
    sc = S.Scene()
    m = sc.add_material(N.LAMBERTIAN, [0.6, 0.6, 0.6])
    e = sc.add_material(N.DIFFUSE_EMITTER, [4.0, 4.0, 4.0, 1.0])
    pos, idx = _soup(n, seed)
    sc.add_mesh(S.Mesh(pos, idx, None, m))
    sc.add_quad(1, 3.0, -1.0, 1.0, -1.0, 1.0, e, flip=1)
    return sc


@pytest.mark.parametrize("n", [20000, 150001])
def test_device_tree_equals_host_tree_without_ties(renderer, n):
    sc = _soup_scene(n, seed=n)
    host = N.bvh_build(sc)
    dev = renderer.bvh_build_device(sc)
    assert dev["items"] == host["items"] and dev["nodes"] == host["nodes"] and dev["depth"] == host["depth"]
    assert dev["hash"] == host["hash"]


def test_device_tree_on_a_displaced_sphere(renderer):
    sc, _ = S.rough_glass(6)  # 81,920 triangles sharing vertices
    host, dev = N.bvh_build(sc), renderer.bvh_build_device(sc)
    assert dev["items"] == host["items"]
    assert abs(dev["depth"] - host["depth"]) <= 1


def test_device_tree_with_ties_traces_like_host_tree(ref_tree):
    renderer = ref_tree
    # an undisplaced icosphere: symmetric triangles share centroid coordinates
    sc, cam = S.cornell_icosphere(7)
    r_dev = N.Renderer(0)
    r_dev.set_bvh_builder(N.BVH_BUILD_DEVICE)
    try:
        s_host = renderer.upload(sc)
        s_dev = r_dev.upload(sc)
        rng = np.random.default_rng(3)
        o = np.tile([0.5, 0.5, -1.0], (1 << 15, 1)) + rng.normal(0, 0.01, (1 << 15, 3))
        d = np.stack([rng.uniform(-0.4, 0.4, 1 << 15), rng.uniform(-0.4, 0.4, 1 << 15), np.ones(1 << 15)], 1)
        rays = np.concatenate([o, d / np.linalg.norm(d, axis=1, keepdims=True)], 1).astype(np.float32)
        t_h, p_h, _ = renderer.trace_closest(s_host, rays)
        t_d, p_d, _ = r_dev.trace_closest(s_dev, rays)
        assert (p_h == p_d).mean() > 0.9999
        same = p_h == p_d
        assert np.array_equal(t_h[same], t_d[same])
        job_h = N.job_desc(s_host, cam, 48, 48, 4, 4, 6, seed=9, estimator=N.EST_NEE_MIS)
        job_d = N.job_desc(s_dev, cam, 48, 48, 4, 4, 6, seed=9, estimator=N.EST_NEE_MIS)
        f_h, f_d = renderer.render(job_h), r_dev.render(job_d)
        assert np.abs(f_h - f_d).max() < 1e-3 * max(1.0, float(np.abs(f_h).max())) or (f_h == f_d).mean() > 0.999
        renderer.release(s_host)
    finally:
        r_dev.close()


def test_device_built_scene_renders_identically(ref_tree):
    renderer = ref_tree
    sc = _soup_scene(60000, seed=4)
    cam = S.camera((0.0, 0.0, -3.5), (0.0, 0.0, 1.0), 45.0, 1.0)
    r_dev = N.Renderer(0)
    r_dev.set_bvh_builder(N.BVH_BUILD_DEVICE)
    try:
        s_h, s_d = renderer.upload(sc), r_dev.upload(sc)
        f_h = renderer.render(N.job_desc(s_h, cam, 40, 40, 4, 4, 5, seed=2, estimator=N.EST_NEE_MIS))
        f_d = r_dev.render(N.job_desc(s_d, cam, 40, 40, 4, 4, 5, seed=2, estimator=N.EST_NEE_MIS))
        assert np.array_equal(f_h, f_d)
        renderer.release(s_h)
    finally:
        r_dev.close()


def test_builder_selection_is_validated(renderer):
    with pytest.raises(N.PtError):
        renderer.set_bvh_builder(7)


def test_sah_trees_find_the_same_hits(ref_tree):
    renderer = ref_tree
    """PT_BVH_BUILD_SAH: another tree over the same primitives (meshes and
    the object level): the same closest hits and the same image."""
    sc, cam = S.material_divergence(3)
    r_sah = N.Renderer(0)
    r_sah.set_bvh_builder(N.BVH_BUILD_SAH)
    try:
        s_ref, s_sah = renderer.upload(sc), r_sah.upload(sc)
        rng = np.random.default_rng(5)
        n = 1 << 15
        o = np.tile(cam["position"], (n, 1)) + rng.normal(0, 0.05, (n, 3))
        d = rng.normal(0, 1, (n, 3)) * [0.4, 0.3, 0.0] + np.asarray(cam["front"])
        rays = np.concatenate([o, d / np.linalg.norm(d, axis=1, keepdims=True)], 1).astype(np.float32)
        t_r, p_r, _ = renderer.trace_closest(s_ref, rays)
        t_s, p_s, _ = r_sah.trace_closest(s_sah, rays)
        assert (p_r == p_s).mean() > 0.9999
        same = p_r == p_s
        assert np.array_equal(t_r[same], t_s[same])
        job_r = N.job_desc(s_ref, cam, 64, 36, 4, 2, 8, seed=4, estimator=N.EST_NEE_MIS,
                           sampler=N.SAMPLER_STRATIFIED)
        job_s = N.job_desc(s_sah, cam, 64, 36, 4, 2, 8, seed=4, estimator=N.EST_NEE_MIS,
                           sampler=N.SAMPLER_STRATIFIED)
        f_r, f_s = renderer.render(job_r), r_sah.render(job_s)
        assert (f_r == f_s).mean() > 0.999
        renderer.release(s_ref)
    finally:
        r_sah.close()
