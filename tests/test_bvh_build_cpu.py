"""Host BVH build (pt_bvh_build, no GPU): the parallel mesh build gives the
tree the sequential recursion gives, and invalid scenes fail loudly."""
from __future__ import annotations

import numpy as np
import pytest

from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S


def test_parallel_build_equals_sequential():
    sc, _ = S.rough_glass(subdiv=7, env_w=16, env_h=8, seed=3)
    one = N.bvh_build(sc, threads=1)
    many = N.bvh_build(sc, threads=8)
    assert one["hash"] == many["hash"]
    assert (one["nodes"], one["items"], one["depth"]) == (many["nodes"], many["items"], many["depth"])
    assert one["items"] == 327680 + 1  # every triangle and the ground quad, once


def test_build_is_deterministic_and_sees_motion():
    static, _ = S.material_divergence(subdiv=1, seed=2)
    a = N.bvh_build(static)
    b = N.bvh_build(static)
    assert a["hash"] == b["hash"]
    moving, _ = S.material_divergence(subdiv=1, seed=2)
    S.with_motion(moving, seed=4)
    c = N.bvh_build(moving)
    assert c["hash"] != a["hash"]  # swept root boxes, per-object subtrees


def test_invalid_scene_fails():
    sc, _ = S.cornell_icosphere(1)
    sc.meshes[0].indices[0, 0] = 10 ** 6  # vertex index out of range
    with pytest.raises(N.PtError):
        N.bvh_build(sc)
    empty = S.Scene()
    with pytest.raises(N.PtError):
        N.bvh_build(empty)


def test_non_finite_geometry_is_rejected():
    """NaN / inf positions, centres, radii or rectangle bounds are refused at
    build time (every builder bins or sorts by them)."""
    import pytest
    sc, _ = S.cornell_icosphere(1)
    pos = sc.meshes[0].positions.copy()
    pos[3, 1] = np.nan
    bad = S.Scene(materials=sc.materials, meshes=[S.Mesh(pos, sc.meshes[0].indices, None, sc.meshes[0].material)],
                  quads=sc.quads, spheres=sc.spheres, objects=sc.objects)
    for sah in (False, True):
        with pytest.raises(N.PtError):
            N.bvh_build(bad, sah=sah)
    sc2, _ = S.cornell_icosphere(1)
    sc2.add_sphere((0.5, np.inf, 0.5), 0.1, 0)
    with pytest.raises(N.PtError):
        N.bvh_build(sc2)


def test_sah_tree_holds_every_item_once():
    """The SAH builder places every primitive in exactly one leaf."""
    sc, _ = S.material_divergence(2)
    ref, sah = N.bvh_build(sc), N.bvh_build(sc, sah=True)
    assert sah["items"] == ref["items"]
    assert sah["depth"] <= 15


def test_parallel_collapse_equals_sequential_with_motion():
    """Large trees are collapsed into BVH4 nodes on host threads and spliced
    in child order: the same nodes, leaf items and motion records (content
    hash) as the one-thread collapse, moving objects included."""
    sc, _ = S.rough_glass(7)  # 327,680 triangles: above the parallel threshold
    moving = S.with_motion(sc, seed=3)
    for scene in (sc, moving):
        one = N.bvh_build(scene, threads=1)
        many = N.bvh_build(scene, threads=8)
        assert one["hash"] == many["hash"] and one["nodes"] == many["nodes"] and one["depth"] == many["depth"]
