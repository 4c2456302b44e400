"""Writes the golden fixtures of tests/golden/ by running the REFERENCE itself.

Run in a container that has the reference sources, after
``oracle/ref/build_ref.sh`` built ``oracle/_ref/libref_harness.so``:

    python tests/golden/make_golden.py

Every array written here comes out of the reference's own code (the
HaltonSampler class, BVHNode/MeshBVHNode/AARectangle/Sphere intersection,
Material::f / scatter_pdf / scatter, and getRayColor of
include/integrator/maxdepth_nee.hpp), driven through the harness in
oracle/ref/ref_harness.cpp.  Inputs are seeded, so the script is
reproducible.
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))

from oracle.ref import refbind as R  # noqa: E402
from pathtracer_gb300 import native as N  # noqa: E402
from pathtracer_gb300 import scene as S  # noqa: E402

OUT = Path(__file__).resolve().parent

# Material parameter sets exercised by the BSDF fixtures: (name, type, params, flags)
MATERIALS = [
    ("lambertian", N.LAMBERTIAN, [0.63, 0.065, 0.05], 0),
    ("conductor_gold_a03", N.CONDUCTOR, [*S.GOLD_ETA, *S.GOLD_K, 0.3, 0.3], 0),
    ("conductor_silver_aniso", N.CONDUCTOR, [*S.SILVER_ETA, *S.SILVER_K, 0.05, 0.4], 0),
    ("conductor_smooth", N.CONDUCTOR, [*S.GOLD_ETA, *S.GOLD_K, 1e-4, 1e-4], 0),
    ("mfdielectric_a005", N.MF_DIELECTRIC, [1.5, 0.05, 0.05], 0),
    ("mfdielectric_a04", N.MF_DIELECTRIC, [1.33, 0.4, 0.2], 0),
    ("mfdielectric_smooth", N.MF_DIELECTRIC, [1.5, 0.0, 0.0], 0),
    ("thindielectric", N.THIN_DIELECTRIC, [1.5], 0),
    ("phong", N.PHONG, [0.5, 0.3, 0.2, 0.4, 0.4, 0.4, 0.0, 0.0, 0.0, 30.0], 0),
    ("disney_a", N.DISNEY, [0.8, 0.3, 0.2, 0.3, 0.2, 0.5, 0.5, 0.4, 0.5, 0.3, 0.6, 0.5, 0.7, 0.4, 1.45], 0),
    ("disney_b", N.DISNEY, [0.2, 0.6, 0.9, 0.0, 0.9, 0.0, 0.5, 0.15, 0.0, 0.8, 0.0, 0.0, 1.0, 0.9, 1.3], 0),
    ("disney_c", N.DISNEY, [0.5, 0.5, 0.5, 0.9, 0.1, 0.2, 0.3, 0.6, 0.2, 0.0, 0.9, 0.9, 0.1, 0.5, 1.6], 0),
    ("hair_a", N.HAIR, [0.419, 0.697, 1.37, 0.1, 1.55, 0.3, 0.3, math.radians(2.0)], 0),
    ("hair_b", N.HAIR, [0.06, 0.1, 0.2, -0.4, 1.55, 0.15, 0.45, math.radians(3.0)], 0),
    ("emitter", N.DIFFUSE_EMITTER, [17.0, 12.0, 4.0, 1.0], 0),
]


def unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def bsdf_inputs(n, rng):
    nrm = unit(rng.normal(size=(n, 3)))
    # wo in the upper hemisphere of n (the integrator turns n towards the ray)
    wo = unit(rng.normal(size=(n, 3)))
    wo = np.where((np.sum(wo * nrm, 1) < 0)[:, None], -wo, wo)
    wi = unit(rng.normal(size=(n, 3)))
    # half of the wi in the upper hemisphere, half anywhere (transmission)
    up = rng.uniform(size=n) < 0.5
    wi = np.where((up & (np.sum(wi * nrm, 1) < 0))[:, None], -wi, wi)
    front = (rng.uniform(size=n) < 0.5).astype(np.uint8)
    uc = rng.uniform(size=n).astype(np.float32)
    u = rng.uniform(size=(n, 2)).astype(np.float32)
    return [a.astype(np.float32) for a in (wo, wi, nrm)] + [front, uc, u]


def make_samplers():
    out = {}
    for name, strat, seed in [("none", N.SAMPLER_HALTON_NONE, 0), ("permute", N.SAMPLER_HALTON_PERMUTE, 0),
                              ("permute7", N.SAMPLER_HALTON_PERMUTE, 7), ("owen", N.SAMPLER_HALTON_OWEN, 0)]:
        blocks = []
        for first, n in [(1, 512), (123457, 128), (100_000_000, 128), (4_000_000_000, 64)]:
            blocks.append(R.sampler_eval(strat, first, n, 25, seed))
            out[f"{name}_first_{first}"] = blocks[-1]
    np.savez_compressed(OUT / "samplers.npz", **out)


def cornell_rays(n, rng, cam):
    # camera-like rays from the eye plus rays from random points in the box
    o1 = np.tile(np.array(cam["position"], np.float32), (n // 2, 1))
    tgt = np.stack([rng.uniform(0, 1, n // 2), rng.uniform(0, 1, n // 2), np.ones(n // 2)], 1)
    d1 = unit(tgt - o1)
    o2 = rng.uniform(0.02, 0.98, size=(n - n // 2, 3))
    d2 = unit(rng.normal(size=(n - n // 2, 3)))
    rays = np.concatenate([np.concatenate([o1, d1], 1), np.concatenate([o2, d2], 1)], 0)
    return rays.astype(np.float32)


def make_trace():
    rng = np.random.default_rng(11)
    sc, cam = S.cornell_icosphere(4)
    rs = R.RefScene(sc)
    rays = cornell_rays(4096, rng, cam)
    t, prim, pos, nrm, front = rs.trace_closest(rays)
    # shadow-ray intervals (maxdepth_nee.hpp:165-166): [0.001, len - 0.001]
    tmax = rng.uniform(0.05, 1.5, size=rays.shape[0]).astype(np.float32)
    occ = np.zeros(rays.shape[0], np.uint8)
    for j in range(rays.shape[0]):
        _, pp, _, _, _ = rs.trace_closest(rays[j:j + 1], tmin=0.001, tmax=float(tmax[j]))
        occ[j] = 1 if pp[0] >= 0 else 0
    np.savez_compressed(OUT / "trace_cornell.npz", rays=rays, t=t, prim=prim, pos=pos, nrm=nrm, front=front,
                        shadow_tmax=tmax, occluded=occ)


# Decorator chains of the transform fixture (objectTransform.hpp), innermost
# first: (code, p0, p1, p2) with 0 Translate, 1 Rotate<X>, 2 Rotate<Y>,
# 3 Rotate<Z>, 4 Scale, 5 FlipFace; over a mesh (flat icosphere, radius 0.5),
# a rectangle (XZ at y = 0.2) or a sphere (radius 0.45 at (0.1, -0.05, 0.2)).
TRANSFORM_CASES = [
    ("mesh_translate", 0, [(0, 0.3, -0.2, 0.5)]),
    ("mesh_rotx", 0, [(1, 0.7, 0, 0)]),
    ("mesh_roty_translate", 0, [(2, -1.1, 0, 0), (0, 0.2, 0.1, 0.0)]),
    ("mesh_rotz", 0, [(3, 0.4, 0, 0)]),
    ("mesh_scale", 0, [(4, 1.7, 0, 0)]),
    ("mesh_flip", 0, [(5, 0, 0, 0)]),
    ("mesh_chain", 0, [(4, 0.5, 0, 0), (1, 0.3, 0, 0), (5, 0, 0, 0), (0, -0.1, 0.2, 0.3), (3, -0.8, 0, 0)]),
    ("quad_translate", 1, [(0, 0.1, 0.3, -0.2)]),
    ("quad_rotz", 1, [(3, 0.3, 0, 0)]),
    ("quad_rotx", 1, [(1, -0.5, 0, 0)]),
    ("quad_flip", 1, [(5, 0, 0, 0)]),
    ("quad_scale", 1, [(4, 1.4, 0, 0)]),
    ("sphere_scale", 2, [(4, 0.6, 0, 0)]),
    ("sphere_roty_translate", 2, [(2, 0.9, 0, 0), (0, -0.3, 0.2, 0.1)]),
    ("sphere_flip", 2, [(5, 0, 0, 0)]),
]


def transform_base(kind):
    """The untransformed object of a transform case (scene with one object)."""
    sc = S.Scene()
    m = sc.add_material(N.LAMBERTIAN, [0.5, 0.5, 0.5])
    if kind == 0:
        v, f = S.icosphere(1)
        sc.add_mesh(S.Mesh((0.5 * v).astype(np.float32), f.astype(np.int32), None, m))
    elif kind == 1:
        sc.add_quad(1, 0.2, -0.5, 0.5, -0.4, 0.6, m)
    else:
        sc.add_sphere((0.1, -0.05, 0.2), 0.45, m)
    return sc


def transform_rays(n, rng):
    # unit-length rays (as the renderer traces them) from a shell of radius 3
    # towards points near the object
    o = unit(rng.normal(size=(n, 3))) * 3.0
    tgt = rng.uniform(-0.8, 0.8, size=(n, 3))
    return np.concatenate([o, unit(tgt - o)], 1).astype(np.float32)


def transform_point(p, ops):
    """A point of the untransformed object seen in the world through the
    decorators (the inverse of the ray mappings of objectTransform)."""
    p = np.array(p, np.float64)
    for code, a, b, c in ops:
        if code == 0:
            p = p + np.array([a, b, c])
        elif code in (1, 2, 3):
            i, j = {1: (1, 2), 2: (0, 2), 3: (0, 1)}[code]
            cs, sn = math.cos(a), math.sin(a)
            p[i], p[j] = cs * p[i] + sn * p[j], -sn * p[i] + cs * p[j]
        elif code == 4:
            p = p * a
    return p


def make_transforms():
    rng = np.random.default_rng(23)
    out = {}
    for name, kind, ops in TRANSFORM_CASES:
        rs = R.RefScene(transform_base(kind))
        rs.transform(0, ops)
        rays = transform_rays(256, rng)
        if kind != 1:
            # rays from inside the object: back-face hits
            c = transform_point((0.0, 0.0, 0.0) if kind == 0 else (0.1, -0.05, 0.2), ops)
            o = c + rng.uniform(-0.05, 0.05, size=(64, 3))
            rays = np.concatenate([rays, np.concatenate([o, unit(rng.normal(size=(64, 3)))], 1)], 0)
            rays = rays.astype(np.float32)
        t, prim, pos, nrm, inside = rs.trace_closest(rays)
        out.update({f"{name}__kind": np.int32(kind), f"{name}__ops": np.array(ops, np.float32),
                    f"{name}__rays": rays, f"{name}__hit": (prim >= 0).astype(np.uint8), f"{name}__t": t,
                    f"{name}__pos": pos, f"{name}__nrm": nrm, f"{name}__inside": inside})
    np.savez_compressed(OUT / "transforms.npz", **out)


def light_scene():
    """Emitters discovered as lights (DiffuseEmitter rectangles of the three
    axes and spheres, a non-emitting rectangle and sphere between them) and a
    seeded environment map: the LightList the light fixture evaluates."""
    sc = S.Scene()
    grey = sc.add_material(N.LAMBERTIAN, [0.5, 0.5, 0.5])
    l1 = sc.add_material(N.DIFFUSE_EMITTER, [17.0, 12.0, 4.0, 1.0])
    l2 = sc.add_material(N.DIFFUSE_EMITTER, [2.0, 3.0, 4.0, 2.5])
    l3 = sc.add_material(N.DIFFUSE_EMITTER, [1.0, 0.5, 0.25, 3.0])
    l4 = sc.add_material(N.DIFFUSE_EMITTER, [5.0, 4.0, 3.0, 1.5])
    sc.add_quad(1, 0.999, 0.375, 0.625, 0.375, 0.625, l1)
    sc.add_quad(1, 0.0, 0.0, 1.0, 0.0, 1.0, grey)
    sc.add_quad(0, 0.05, 0.2, 0.5, 0.1, 0.7, l2)
    sc.add_sphere((0.5, 0.5, 0.5), 0.2, grey)
    sc.add_quad(2, 0.9, 0.1, 0.4, 0.6, 0.95, l3)
    sc.add_sphere((0.3, 0.6, 0.4), 0.1, l4)
    sc.add_sphere((0.7, 0.2, 0.6), 0.05, l2)
    rng = np.random.default_rng(41)
    h, w = 32, 64
    y = (np.arange(h) + 0.5) / h
    env = np.stack([0.2 + 0.8 * y, 0.3 + 0.6 * y, 0.9 - 0.3 * y], 1)[:, None, :] * np.ones((1, w, 1))
    env = env + rng.uniform(0.0, 0.5, (h, w, 3))
    sc.env = env.astype(np.float32)
    sc.env_intensity = 1.7
    return sc


def make_lights():
    rng = np.random.default_rng(43)
    rs = R.RefScene(light_scene())
    n_lights = rs.lib.ref_scene_num_lights(rs.h)
    out = {"n_lights": np.int32(n_lights)}
    for li in range(n_lights):
        uv = rng.uniform(0.0, 1.0, (512, 2)).astype(np.float32)
        x = rng.uniform(0.0, 1.0, (512, 3)).astype(np.float32)
        r = rs.light_eval(li, uv, x)
        out.update({f"light{li}__uv": uv, f"light{li}__x": x, f"light{li}__area": np.float32(r["area"])})
        out.update({f"light{li}__{k}": r[k] for k in ("point", "normal", "dir", "le", "pdf")})
        # pdf_value at directions that are not the sample's: towards points
        # near the light (often missing a quad) and random directions
        pd = unit(r["point"] + rng.normal(scale=0.1, size=(512, 3)) - x) if li < n_lights - 1 else \
            unit(rng.normal(size=(512, 3)))
        pd = pd.astype(np.float32)
        out[f"light{li}__pdf_dir"] = pd
        out[f"light{li}__pdf_at_dir"] = rs.light_eval(li, uv, x, pdf_dir=pd)["pdf"]
    np.savez_compressed(OUT / "lights.npz", **out)


def make_bsdf():
    rng = np.random.default_rng(5)
    out = {}
    for name, mtype, params, flags in MATERIALS:
        mat = N.material(mtype, params, flags)
        wo, wi, nrm, front, uc, u = bsdf_inputs(384, rng)
        f, pdf = R.bsdf_eval(mat, wo, wi, nrm, front)
        ok, swi, att, spdf, ty = R.bsdf_sample(mat, wo, nrm, front, uc, u)
        out[name] = dict(type=mtype, flags=flags, params=np.array(params, np.float32), wo=wo, wi=wi, nrm=nrm,
                         front=front, uc=uc, u=u, f=f, pdf=pdf, ok=ok, s_wi=swi, s_att=att, s_pdf=spdf, s_type=ty)
    flat = {f"{k}__{kk}": vv for k, v in out.items() for kk, vv in v.items()}
    np.savez_compressed(OUT / "bsdf.npz", **flat)


def make_images():
    # Cornell box + GGX gold icosphere, the reference integrator, 64 spp.
    sc, cam = S.cornell_icosphere(4)
    rs = R.RefScene(sc)
    job = N.job_desc(0, cam, 64, 64, 8, 8, 8, seed=3)
    mean, var = rs.render(job)
    np.savez_compressed(OUT / "image_cornell.npz", mean=mean, var=var, width=64, height=64, spp=64, depth=8)
    # Rough glass over a conductor ground, HDRI environment (small sizes).
    sc, cam = S.rough_glass(subdiv=3, env_w=128, env_h=64, seed=2)
    rs = R.RefScene(sc)
    job = N.job_desc(0, cam, 48, 48, 4, 4, 6, seed=4)
    mean, var = rs.render(job)
    np.savez_compressed(OUT / "image_roughglass.npz", mean=mean, var=var, width=48, height=48, spp=16, depth=6)
    # hair on curves (HairMarschner framed by the curve tangent for sampling,
    # by the normal for f / scatter_pdf), explicit sigma_a
    sc, cam = S.hair_curves(40, seed=2)
    sc.materials = [(t, ([0.25, 0.45, 0.9] + list(p[3:])) if t == N.HAIR else p, 0 if t == N.HAIR else f)
                    for t, p, f in sc.materials]
    job = N.job_desc(0, cam, 24, 24, 16, 16, 6, seed=3)
    mean, var = R.RefScene(sc).render(job)
    np.savez_compressed(OUT / "image_haircurves.npz", mean=mean, var=var, width=24, height=24, spp=256, depth=6)
    # every material family of the mix scene at once (tests/conftest.py's
    # material_mix_for_reference says what was changed for the reference)
    sys.path.insert(0, str(REPO / "tests"))
    from conftest import material_mix_for_reference
    sc, cam = material_mix_for_reference()
    job = N.job_desc(0, cam, 32, 32, 8, 8, 6, seed=3)
    mean, var = R.RefScene(sc).render(job)
    assert np.isfinite(mean).all()
    np.savez_compressed(OUT / "image_materials.npz", mean=mean, var=var, width=32, height=32, spp=64, depth=6)


def make_tonemap():
    """A film with values past 1, NaN and +inf written by the reference's
    FrameBuffer::writeToFile (gamma 2.2 and 1.0); the PNG's bytes (top row
    first) are decoded back with the repository's PNG reader."""
    import tempfile
    rng = np.random.default_rng(31)
    h, w = 48, 64
    film = rng.uniform(0.0, 1.5, (h, w, 3)).astype(np.float32)
    film[rng.integers(0, h, 20), rng.integers(0, w, 20), rng.integers(0, 3, 20)] = np.nan
    film[rng.integers(0, h, 10), rng.integers(0, w, 10), rng.integers(0, 3, 10)] = np.inf
    out = {"film": film}
    with tempfile.TemporaryDirectory() as td:
        for gamma in (2.2, 1.0):
            p = Path(td) / "tm.png"
            R.write_png(film, gamma, p)
            out[f"rgb8_gamma_{gamma}"] = np.rint(N.load_image(p, flip_y=True) * 255.0).astype(np.uint8)
    np.savez_compressed(OUT / "tonemap.npz", **out)


if __name__ == "__main__":
    if not R.available():
        raise SystemExit("build oracle/_ref first: oracle/ref/build_ref.sh")
    make_samplers()
    make_trace()
    make_transforms()
    make_lights()
    make_bsdf()
    make_images()
    make_tonemap()
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size)
