"""OBJ ingest (pt_obj_load), CPU only.  The fixtures are written by the tests
themselves; the behaviour restated is loadOBJMesh (meshLoader.cpp:7-58) over
tinyobjloader."""
from __future__ import annotations

import numpy as np
import pytest

from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return p


def test_triangles_normals_uvs_and_index_forms(tmp_path):
    p = _write(tmp_path, "t.obj", """# comment
o thing
v 0 0 0
v 1 0 0
v 0 1 0
v 1 1 0
vn 0 0 1
vt 0 0
vt 1 0
vt 0 1
usemtl whatever
f 1/1/1 2/2/1 3/3/1
f 2//1 4//1 3//1
f -3/-2 -1/-1 -2/-3
f 1 2 3
""")
    m = N.obj_load(p)
    assert m["positions"].shape == (4, 3) and m["normals"].shape == (1, 3) and m["uvs"].shape == (3, 2)
    assert m["indices"].tolist() == [[0, 1, 2], [1, 3, 2], [1, 3, 2], [0, 1, 2]]
    assert m["normal_indices"].tolist() == [[0, 0, 0], [0, 0, 0], [-1, -1, -1], [-1, -1, -1]]
    assert m["uv_indices"].tolist() == [[0, 1, 2], [-1, -1, -1], [1, 2, 0], [-1, -1, -1]]


def test_quads_split_along_the_shorter_diagonal(tmp_path):
    # |v2 - v0| < |v3 - v1|: [0 1 2] [0 2 3]; otherwise [0 1 3] [1 2 3]
    p = _write(tmp_path, "q.obj", """v 0 0 0
v 2 0 0
v 1 0.5 0
v 0 3 0
f 1 2 3 4
v 10 0 0
v 11 0 0
v 13 4 0
v 10 1 0
f 5 6 7 8
""")
    m = N.obj_load(p)
    assert m["indices"].tolist() == [[0, 1, 2], [0, 2, 3], [4, 5, 7], [5, 6, 7]]


def test_polygon_fan_and_errors(tmp_path):
    p = _write(tmp_path, "p.obj", "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv -1 0.5 0\nf 1 2 3 4 5\n")
    assert N.obj_load(p)["indices"].tolist() == [[0, 1, 2], [0, 2, 3], [0, 3, 4]]
    with pytest.raises(N.PtError) as e:
        N.obj_load(tmp_path / "missing.obj")
    assert e.value.code == -4
    bad = _write(tmp_path, "bad.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 9\n")
    with pytest.raises(N.PtError) as e:
        N.obj_load(bad)
    assert e.value.code == -1 and "bad.obj:4" in str(e.value)


def test_obj_mesh_builds_the_same_bvh(tmp_path):
    # an icosphere written as OBJ text (exact float32 round trip) and read back
    # gives the same BVH as the in-memory mesh
    mesh = S.sphere_mesh(3, (0.1, 0.2, 0.3), 0.7, 0, displace=0.05, seed=4)
    lines = ["v %.9g %.9g %.9g" % tuple(float(x) for x in v) for v in mesh.positions]
    lines += ["vn %.9g %.9g %.9g" % tuple(float(x) for x in v) for v in mesh.normals]
    lines += ["f %d//%d %d//%d %d//%d" % (a + 1, a + 1, b + 1, b + 1, c + 1, c + 1) for a, b, c in mesh.indices]
    p = _write(tmp_path, "ico.obj", "\n".join(lines) + "\n")
    m = N.obj_load(p)
    assert np.array_equal(m["positions"], mesh.positions)
    assert np.array_equal(m["indices"], mesh.indices)
    sc1 = S.Scene()
    mat = sc1.add_material(N.LAMBERTIAN, [0.5, 0.5, 0.5])
    sc1.add_mesh(S.Mesh(mesh.positions, mesh.indices, mesh.normals, mat))
    sc2 = S.Scene()
    sc2.add_material(N.LAMBERTIAN, [0.5, 0.5, 0.5])
    sc2.add_mesh(S.Mesh(m["positions"], m["indices"], m["normals"], mat))
    assert N.bvh_build(sc1)["hash"] == N.bvh_build(sc2)["hash"]


def test_obj_load_matches_reference_loader(tmp_path):
    """pt_obj_load against the reference's own loadOBJMesh (tinyobjloader)
    through the harness, where it is built: triangles and quads with every
    index form, negative indices, comments and ignored records, and a
    seeded random quad mesh."""
    from oracle.ref import refbind
    if not refbind.available():
        pytest.skip("reference harness not built")
    files = [_write(tmp_path, "forms.obj", """# comment
o thing
v 0 0 0
v 1 0 0
v 0 1 0
v 1 1 0.5
vn 0 0 1
vn 0 0.6 0.8
vt 0 0
vt 1 0
vt 0 1
vt 1 1
usemtl whatever
s 1
f 1/1/1 2/2/1 3/3/2
f 2//1 4//2 3//1
f -3/-2 -1/-1 -2/-3
f 1 2 4 3
f 1/1/1 2/2/2 4/4/2 3/3/1
""")]
    rng = np.random.default_rng(6)
    n = 12
    lines = []
    grid = rng.uniform(-1, 1, (n, n)).astype(np.float32)
    for j in range(n):
        for i in range(n):
            lines.append(f"v {i / n:.6f} {grid[j, i]:.6f} {j / n:.6f}")
            lines.append(f"vt {i / n:.6f} {j / n:.6f}")
    for j in range(n - 1):
        for i in range(n - 1):
            a, b, c, d = j * n + i + 1, j * n + i + 2, (j + 1) * n + i + 2, (j + 1) * n + i + 1
            lines.append(f"f {a}/{a} {b}/{b} {c}/{c} {d}/{d}")
    files.append(_write(tmp_path, "grid.obj", "\n".join(lines) + "\n"))
    for p in files:
        ours, ref = N.obj_load(p), refbind.obj_load(p)
        for key in ("positions", "normals", "uvs", "indices", "normal_indices", "uv_indices"):
            assert np.array_equal(ours[key], ref[key]), (p.name, key)
