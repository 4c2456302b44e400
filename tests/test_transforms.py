"""The reference's decorators -- Translate, Rotate<X/Y/Z>, Scale, FlipFace
(utils/objectTransform.hpp:5-181, src/utils/objectTransform.cpp:95-213) --
as the C++ scene API bakes them into the uploaded geometry, against the
reference's own decorated objects (fixture tests/golden/transforms.npz, written
by the reference through oracle/ref): hit or miss, hit position and normal,
and HitRecord::is_inside, over meshes, rectangles and spheres, for rays from
outside and from inside the objects (unit directions, as the renderer traces).

Reference behaviour kept: Translate, Rotate and Scale call set_normal with the
child's already ray-facing normal, so every hit on a decorated object reports
is_inside = true (a FlipFace over one: false); hits from inside a translated
mesh are "front" hits.

CPU: the flattened geometry (tests/cpp/transforms_example.cpp, "flatten")
intersected by the oracle.  GPU: the same program uploads it and intersects
through pt_intersect ("trace")."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
SRC = REPO / "tests" / "cpp" / "transforms_example.cpp"
LIBDIR = REPO / "pathtracer_gb300" / "_lib"
GOLD = REPO / "tests" / "golden" / "transforms.npz"


def _cases():
    g = np.load(GOLD)
    names = sorted(set(k.split("__")[0] for k in g.files))
    return {n: {k.split("__")[1]: g[k] for k in g.files if k.startswith(n + "__")} for n in names}


def _input_file(tmp_path, cases):
    """The program's input: base objects as tests/golden/make_golden.py builds them."""
    from pathtracer_gb300 import scene as S
    lines = [str(len(cases))]
    for _, c in cases:
        kind = int(c["kind"])
        lines.append(str(kind))
        if kind == 0:
            v, f = S.icosphere(1)
            v = (0.5 * v).astype(np.float32)
            lines.append(f"{len(v)} {len(f)}")
            lines += [" ".join(f"{x:.9g}" for x in row) for row in v]
            lines += [" ".join(str(int(x)) for x in row) for row in f]
        elif kind == 1:
            lines.append("1 0.2 -0.5 0.5 -0.4 0.6")
        else:
            lines.append("0.1 -0.05 0.2 0.45")
        ops = c["ops"]
        lines.append(str(len(ops)))
        lines += [f"{int(o[0])} {o[1]:.9g} {o[2]:.9g} {o[3]:.9g}" for o in ops]
        lines.append(str(len(c["rays"])))
        lines += [" ".join(f"{x:.9g}" for x in r) for r in c["rays"]]
    p = tmp_path / "cases.txt"
    p.write_text("\n".join(lines) + "\n")
    return p


def _build(tmp_path):
    exe = tmp_path / "transforms_example"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(REPO / "include"), str(SRC), "-o", str(exe),
                    "-L", str(LIBDIR), "-lpathtracer_gb300", f"-Wl,-rpath,{LIBDIR}"], check=True)
    return exe


def _check(name, c, hit, pos, nrm, inside):
    want = c["hit"].astype(bool)
    # a ray grazing an edge may flip between neighbours: allow 1 in 200
    agree = hit == want
    assert agree.mean() >= 0.995, (name, np.nonzero(~agree))
    m = hit & want
    assert m.sum() > 20, name
    dp = np.abs(pos[m] - c["pos"][m]).max(1)
    dn = np.abs(nrm[m] - c["nrm"][m]).max(1)
    # positions within 1e-4 (scene scale ~1: baked vertices vs the
    # reference's transformed rays round differently), normals within 1e-4
    assert (dp < 1e-4).mean() >= 0.995, (name, dp.max())
    assert (dn < 1e-4).mean() >= 0.995, (name, dn.max())
    assert np.array_equal(inside[m].astype(bool), c["inside"][m].astype(bool)), name


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_baked_transforms_match_reference_on_cpu(tmp_path):
    from oracle import pyoracle as O
    from pathtracer_gb300 import native as N
    from pathtracer_gb300 import scene as S

    cases = sorted(_cases().items())
    exe = _build(tmp_path)
    out = subprocess.run([str(exe), "flatten", str(_input_file(tmp_path, cases))], capture_output=True, text=True,
                         check=True).stdout.split()
    k = 0
    for name, c in cases:
        face = int(out[k]); kind = int(out[k + 1]); k += 2
        sc = S.Scene()
        m = sc.add_material(N.LAMBERTIAN, [0.5, 0.5, 0.5])
        if kind == 0:
            nv, nt = int(out[k]), int(out[k + 1]); k += 2
            v = np.array(out[k:k + 3 * nv], np.float32).reshape(nv, 3); k += 3 * nv
            f = np.array(out[k:k + 3 * nt], np.int32).reshape(nt, 3); k += 3 * nt
            sc.add_mesh(S.Mesh(v, f, None, m))
        elif kind == 1:
            axis = int(out[k]); q = [float(x) for x in out[k + 1:k + 6]]; flip = int(out[k + 6]); k += 7
            sc.add_quad(axis, *q, m, flip=flip)
        else:
            ctr = [float(x) for x in out[k:k + 3]]; r = float(out[k + 3]); flip = int(out[k + 4]); k += 5
            sc.add_sphere(ctr, r, m, flip=flip)
        sc.objects[0] = (*sc.objects[0][:3], face)
        t, prim, pos, nrm, inside = O.OracleScene(sc).intersect(c["rays"])
        _check(name, c, prim >= 0, pos, nrm, inside)
    assert k == len(out)


@pytest.mark.gpu
def test_baked_transforms_match_reference_on_gpu(tmp_path):
    cases = sorted(_cases().items())
    exe = _build(tmp_path)
    out = subprocess.run([str(exe), "trace", str(_input_file(tmp_path, cases))], capture_output=True, text=True,
                         check=True).stdout.split("\n")
    k = 0
    for name, c in cases:
        n = len(c["rays"])
        rows = np.array([[float(x) for x in ln.split()] for ln in out[k:k + n]])
        k += n
        _check(name, c, rows[:, 0] > 0, rows[:, 2:5].astype(np.float32), rows[:, 5:8].astype(np.float32),
               rows[:, 8] > 0)
