"""Scene description on the Python side and the seeded synthetic workloads.

A :class:`Scene` holds the same objects a reference scene builder puts into
its ``ObjectList`` (include/base/objectList.hpp), in insertion order:
triangle meshes (``TriangleMesh``), axis-aligned rectangles
(``AARectangle<axis>``) and spheres, each with a material
(``Lambertian``, ``Conductor`` ... ``DiffuseEmitter``), plus an optional
HDRI environment (``EnvironmentLight``) and an optional homogeneous medium.

The generators below build the benchmark scenes from seeds only: there are
no asset files.  ``cornell_icosphere`` is the plain small case,
``rough_glass`` the 1.3 M-triangle HDRI scene, ``material_divergence`` the
64-sphere mixed-material scene in a medium.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import native as N

GOLD_ETA = (0.14, 0.43, 1.38)      # commonMaterials.hpp:43-47
GOLD_K = (4.54, 2.455, 1.914)
SILVER_ETA = (0.04, 0.06, 0.04)    # commonMaterials.hpp:37-41
SILVER_K = (4.8, 3.586, 2.657)


@dataclass
class Mesh:
    positions: np.ndarray            # (V, 3) float32
    indices: np.ndarray              # (T, 3) int32
    normals: np.ndarray | None       # (V, 3) float32, indexed like positions
    material: int
    uvs: np.ndarray | None = None    # (V, 2) float32 texture coordinates, indexed like positions


@dataclass
class Scene:
    materials: list = field(default_factory=list)   # (type, params, flags)
    meshes: list = field(default_factory=list)
    quads: list = field(default_factory=list)       # (axis, k, d0min, d0max, d1min, d1max, material, flip)
    spheres: list = field(default_factory=list)     # ((cx, cy, cz), r, material, flip)
    objects: list = field(default_factory=list)     # (kind, index, velocity)
    env: np.ndarray | None = None                   # (H, W, 3), row 0 = bottom
    env_intensity: float = 1.0
    medium: tuple | None = None                     # (sigma_a[3], sigma_s[3], g)
    bg: tuple = (0.0, 0.0, 0.0)
    shutter_max: float = 0.0                        # motion blur: longest shutter of any job
    textures: list = field(default_factory=list)    # dicts: kind, color1, color2, scale, fractal, texels
    boxes: list = field(default_factory=list)       # (min_xyz, max_xyz, material)
    curves: list = field(default_factory=list)      # (4 control points, width0, width1, material)

    def add_material(self, mtype: int, params, flags: int = 0, texture: int | None = None) -> int:
        """A material; `texture` (an index from add_texture) replaces the
        Lambertian albedo / DiffuseEmitter colour p[0..2] (ColorVariant)."""
        if texture is not None:
            flags |= (texture + 1) << N.MAT_TEXTURE_SHIFT
        self.materials.append((mtype, list(params), flags))
        return len(self.materials) - 1

    def add_texture(self, kind: int, color1=(0.0, 0.0, 0.0), color2=(1.0, 1.0, 1.0), scale: float = 10.0,
                    fractal: int = 1, texels=None) -> int:
        """CheckerTexture(color1, color2, scale), NoiseTexture(scale, fractal),
        ConstantTexture(color1) or an image (texels (H, W, 3), row y as
        ImageTexture's texels[x][y])."""
        self.textures.append({"kind": kind, "color1": tuple(color1), "color2": tuple(color2), "scale": scale,
                              "fractal": fractal, "texels": texels})
        return len(self.textures) - 1

    def add_image_texture(self, path, flip_y: bool = False, hdr: bool = False) -> int:
        """ImageTexture(filename, flip_y, isHDR): a PNG or Radiance HDR file."""
        return self.add_texture(N.TEX_IMAGE, texels=N.load_image(path, flip_y, hdr))

    def set_environment(self, path, intensity: float = 1.0) -> None:
        """EnvironmentLight(hdri_filepath, intensity_scale): HDRITexture with
        flip_y = false, isHDR = true."""
        self.env = N.load_image(path, flip_y=False, hdr=True)
        self.env_intensity = float(intensity)

    def add_mesh(self, mesh: Mesh, velocity=(0.0, 0.0, 0.0)):
        self.meshes.append(mesh)
        self.objects.append((N.OBJ_MESH, len(self.meshes) - 1, tuple(velocity)))

    def add_quad(self, axis, k, d0min, d0max, d1min, d1max, material, flip=0, velocity=(0.0, 0.0, 0.0)):
        self.quads.append((axis, k, d0min, d0max, d1min, d1max, material, flip))
        self.objects.append((N.OBJ_QUAD, len(self.quads) - 1, tuple(velocity)))

    def add_sphere(self, center, radius, material, flip=0, velocity=(0.0, 0.0, 0.0)):
        self.spheres.append((tuple(center), radius, material, flip))
        self.objects.append((N.OBJ_SPHERE, len(self.spheres) - 1, tuple(velocity)))

    def add_box(self, min_xyz, max_xyz, material, velocity=(0.0, 0.0, 0.0)):
        """Box(min_xyz, max_xyz, material): one object of six rectangles."""
        self.boxes.append((tuple(min_xyz), tuple(max_xyz), material))
        self.objects.append((N.OBJ_BOX, len(self.boxes) - 1, tuple(velocity)))

    def add_curve(self, cps, width0, width1, material, velocity=(0.0, 0.0, 0.0)):
        """Curve(cps, width0, width1, CurveType::Cylinder, material)."""
        self.curves.append(([tuple(float(x) for x in p) for p in cps], width0, width1, material))
        self.objects.append((N.OBJ_CURVE, len(self.curves) - 1, tuple(velocity)))

    @property
    def has_motion(self) -> bool:
        return any(len(o) > 2 and any(v != 0.0 for v in o[2]) for o in self.objects)

    @property
    def n_triangles(self) -> int:
        return sum(int(m.indices.shape[0]) for m in self.meshes)


# ---------------------------------------------------------------- meshes
def icosphere(subdiv: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: 10*4^s + 2 vertices, 20*4^s triangles, outward CCW."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                  [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = v.shape[0]
        v = np.concatenate([v, mid], axis=0)
        nf = f.shape[0]
        ab, bc, ca = base + inv[:nf], base + inv[nf:2 * nf], base + inv[2 * nf:]
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                            np.stack([ab, bc, ca], 1)], axis=0)
    return v, f


def vertex_normals(v: np.ndarray, f: np.ndarray) -> np.ndarray:
    fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    n = np.zeros_like(v)
    for k in range(3):
        np.add.at(n, f[:, k], fn)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    return n


def sphere_mesh(subdiv: int, center, radius: float, material: int, displace: float = 0.0,
                seed: int = 0) -> Mesh:
    v, f = icosphere(subdiv)
    if displace:
        rng = np.random.default_rng(seed)
        k = 12
        dirs = rng.normal(size=(k, 3))
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        freq = rng.uniform(2.0, 9.0, size=k)
        phase = rng.uniform(0, 2 * math.pi, size=k)
        amp = rng.uniform(0.5, 1.0, size=k)
        noise = (amp[None, :] * np.sin(v @ dirs.T * freq[None, :] + phase[None, :])).sum(1) / amp.sum()
        v = v * (1.0 + displace * noise)[:, None]
        nrm = vertex_normals(v, f)
    else:
        nrm = v.copy()
    pos = v * radius + np.asarray(center, np.float64)[None, :]
    return Mesh(pos.astype(np.float32), f.astype(np.int32), nrm.astype(np.float32), material)


# ------------------------------------------------------------------ HDRI
def synthetic_hdri(width: int = 1024, height: int = 512, seed: int = 0, peak: float = 5e3,
                   lobes: int = 3) -> np.ndarray:
    """Sky gradient plus seeded Gaussian sun lobes, (H, W, 3), row 0 = bottom.

    Texel (x, y) maps to theta = pi*(y+0.5)/H from -Y and phi = 2*pi*(x+0.5)/W,
    the inverse of HDRITexture::getTexelColor (texture.hpp:105-115).
    """
    rng = np.random.default_rng(seed)
    th = math.pi * (np.arange(height) + 0.5) / height
    ph = 2 * math.pi * (np.arange(width) + 0.5) / width
    TH, PH = np.meshgrid(th, ph, indexing="ij")
    d = np.stack([-np.sin(TH) * np.cos(PH), -np.cos(TH), np.sin(TH) * np.sin(PH)], axis=-1)
    up = np.clip(d[..., 1], -1, 1)
    horizon = np.array([0.9, 0.85, 0.8])
    zenith = np.array([0.25, 0.45, 0.9])
    ground = np.array([0.25, 0.22, 0.2])
    s = np.clip(up, 0, 1)[..., None]
    img = np.where(up[..., None] >= 0, horizon * (1 - s) + zenith * s, ground * np.ones_like(s))
    for _ in range(lobes):
        el = rng.uniform(0.15, 1.2)
        az = rng.uniform(0, 2 * math.pi)
        sd = np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)])
        width_rad = rng.uniform(0.01, 0.04)
        color = rng.uniform(0.7, 1.0, size=3)
        cosang = np.clip(d @ sd, -1, 1)
        ang = np.arccos(cosang)
        img = img + peak * color[None, None, :] * np.exp(-0.5 * (ang / width_rad) ** 2)[..., None]
    return img.astype(np.float32)


# -------------------------------------------------------------- cameras
def camera(position, front, fov_deg: float, aspect: float, aperture: float = 1000.0,
           focal_dist: float = 10.0, up=(0.0, 1.0, 0.0), shutter: float = 0.0) -> dict:
    """PerspectiveCamera arguments (camera.cpp:7-35); lens radius is
    focal_dist / aperture * 0.5."""
    return {"fov": math.radians(fov_deg), "aspect": aspect, "focal_dist": focal_dist, "aperture": aperture,
            "up": tuple(up), "front": tuple(front), "position": tuple(position), "shutter": shutter}


# -------------------------------------------------------------- workloads
def cornell_icosphere(subdiv: int = 4) -> tuple[Scene, dict]:
    """Unit Cornell box, 5 Lambertian walls, a 0.25 x 0.25 light of radiance
    (17, 12, 4) below the ceiling, and an icosphere in GGX gold (alpha 0.3)."""
    sc = Scene()
    white = sc.add_material(N.LAMBERTIAN, [0.75, 0.75, 0.75])
    red = sc.add_material(N.LAMBERTIAN, [0.63, 0.065, 0.05])
    green = sc.add_material(N.LAMBERTIAN, [0.14, 0.45, 0.09])
    light = sc.add_material(N.DIFFUSE_EMITTER, [17.0, 12.0, 4.0, 1.0])
    gold = sc.add_material(N.CONDUCTOR, [*GOLD_ETA, *GOLD_K, 0.3, 0.3])
    sc.add_quad(1, 0.999, 0.375, 0.625, 0.375, 0.625, light)    # light, y = 0.999
    sc.add_quad(0, 1.0, 0.0, 1.0, 0.0, 1.0, red)                 # x = 1 (image left)
    sc.add_quad(0, 0.0, 0.0, 1.0, 0.0, 1.0, green)               # x = 0 (image right)
    sc.add_quad(1, 0.0, 0.0, 1.0, 0.0, 1.0, white)               # floor
    sc.add_quad(1, 1.0, 0.0, 1.0, 0.0, 1.0, white)               # ceiling
    sc.add_quad(2, 1.0, 0.0, 1.0, 0.0, 1.0, white)               # back wall
    sc.add_mesh(sphere_mesh(subdiv, (0.5, 0.3, 0.55), 0.25, gold))
    cam = camera((0.5, 0.5, -1.4), (0.0, 0.0, 1.0), 40.0, 1.0)
    return sc, cam


def rough_glass(subdiv: int = 8, env_w: int = 1024, env_h: int = 512, seed: int = 0) -> tuple[Scene, dict]:
    """Displaced icosphere (20*4^subdiv tris, radial noise 0.05) in rough
    glass (ior 1.5, alpha 0.05) over a GGX conductor ground (alpha 0.2), lit
    by a synthetic HDRI with three sun lobes of peak 5e3."""
    sc = Scene()
    glass = sc.add_material(N.MF_DIELECTRIC, [1.5, 0.05, 0.05])
    ground = sc.add_material(N.CONDUCTOR, [*SILVER_ETA, *SILVER_K, 0.2, 0.2])
    sc.add_mesh(sphere_mesh(subdiv, (0.0, 0.0, 0.0), 1.0, glass, displace=0.05, seed=seed))
    sc.add_quad(1, -1.1, -12.0, 12.0, -12.0, 12.0, ground)
    sc.env = synthetic_hdri(env_w, env_h, seed=seed + 1)
    sc.env_intensity = 1.0
    cam = camera((0.0, 0.6, -4.2), (0.0, -0.12, 1.0), 40.0, 1.0)
    return sc, cam


def material_divergence(subdiv: int = 5, seed: int = 0, aspect: float = 16 / 9) -> tuple[Scene, dict]:
    """64 icospheres with seeded materials from {Disney, hair, thin
    dielectric, Phong, Lambertian} in a homogeneous medium (sigma_t 0.05,
    albedo 0.9), lit by 4 sphere lights and 2 area lights."""
    rng = np.random.default_rng(seed)
    sc = Scene()
    fams = rng.integers(0, 5, size=64)
    mats = []
    for fam in fams:
        if fam == 0:
            p = rng.uniform(0, 1, size=15)
            p[14] = rng.uniform(1.0, 2.0)   # eta drawn in [1, 2]
            mats.append(sc.add_material(N.DISNEY, p))
        elif fam == 1:
            bm, bn = rng.uniform(0.1, 0.5, size=2)
            eu = rng.uniform(0.0, 3.0)
            mats.append(sc.add_material(N.HAIR, [0, 0, 0, 0.0, 1.55, bm, bn, math.radians(2.0), eu, 0.0],
                                        N.FLAG_MELANIN))
        elif fam == 2:
            mats.append(sc.add_material(N.THIN_DIELECTRIC, [rng.uniform(1.2, 1.8)]))
        elif fam == 3:
            d = rng.uniform(0.1, 0.8, size=3)
            s = rng.uniform(0.1, 0.6, size=3)
            mats.append(sc.add_material(N.PHONG, [*d, *s, 0, 0, 0, rng.uniform(5, 100)]))
        else:
            mats.append(sc.add_material(N.LAMBERTIAN, rng.uniform(0.1, 0.9, size=3)))
    base_v, base_f = icosphere(subdiv)
    for k in range(64):
        gx, gz = k % 8, k // 8
        c = np.array([(gx - 3.5) * 1.1, 0.0, (gz - 3.5) * 1.1])
        r = 0.45
        sc.add_mesh(Mesh((base_v * r + c).astype(np.float32), base_f.astype(np.int32),
                         base_v.astype(np.float32), mats[k]))
    for k in range(4):
        lm = sc.add_material(N.DIFFUSE_EMITTER, [*rng.uniform(0.6, 1.0, size=3), 40.0])
        ang = 2 * math.pi * k / 4
        sc.add_sphere((6.0 * math.cos(ang), 2.5, 6.0 * math.sin(ang)), 0.5, lm)
    for k in range(2):
        lm = sc.add_material(N.DIFFUSE_EMITTER, [*rng.uniform(0.6, 1.0, size=3), 6.0])
        x0 = -3.0 + 4.0 * k
        sc.add_quad(1, 4.0, x0, x0 + 2.0, -1.0, 1.0, lm)
    sc.medium = ((0.005, 0.005, 0.005), (0.045, 0.045, 0.045), 0.0)
    cam = camera((0.0, 5.5, -10.5), (0.0, -0.45, 1.0), 45.0, aspect)
    return sc, cam


# --------------------------------------------------- batched / served mixes
def with_motion(sc: Scene, seed: int, speed: float = 0.4, shutter_max: float = 0.5,
                kinds=(N.OBJ_MESH, N.OBJ_SPHERE)) -> Scene:
    """Gives the scene's meshes and spheres seeded linear velocities
    (|v| uniform in [0, speed] scene units per unit time, random direction);
    walls, ground and area lights stay put.  Jobs may then use a shutter up
    to ``shutter_max``."""
    rng = np.random.default_rng(seed)
    objs = []
    for o in sc.objects:
        if o[0] in kinds:
            v = rng.normal(size=3)
            v = v / np.linalg.norm(v) * rng.uniform(0.0, speed)
            objs.append((o[0], o[1], tuple(float(x) for x in v)))
        else:
            objs.append(o)
    sc.objects = objs
    sc.shutter_max = shutter_max
    return sc


def with_lens(cam: dict, lens_diameter: float, focal_dist: float | None = None) -> dict:
    """Depth of field in the reference's camera terms: PerspectiveCamera's
    lens radius is focalDist / aperture * 0.5 (camera.cpp:44), so a lens of
    diameter D takes aperture = focalDist / D (D = 0: a pinhole)."""
    c = dict(cam)
    if focal_dist is not None:
        c["focal_dist"] = float(focal_dist)
    c["aperture"] = c["focal_dist"] / lens_diameter if lens_diameter > 0 else 1e9
    return c


# per workload: depth, RR start, sampler, env sampling of its plain config
MIX_SETTINGS = {
    "cornell": dict(max_depth=8, rr_start=-1, sampler=N.SAMPLER_HALTON_OWEN, env_sampling=N.ENV_UNIFORM),
    "rough_glass": dict(max_depth=16, rr_start=4, sampler=N.SAMPLER_HALTON_OWEN, env_sampling=N.ENV_ALIAS),
    "divergence": dict(max_depth=12, rr_start=-1, sampler=N.SAMPLER_STRATIFIED, env_sampling=N.ENV_UNIFORM),
}


def _spp_grid(spp: int) -> tuple[int, int]:
    x = int(math.isqrt(spp))
    while spp % x:
        x -= 1
    return spp // x, x


def job_mix(scenes: dict, n_jobs: int, seed: int, res=(64, 1024), spp=(4, 256), lens_max: float = 0.05,
            shutter_max: float = 0.5) -> list:
    """Seeded render jobs over resident scenes: square resolution
    log-uniform in ``res``, spp uniform in ``spp``, a seeded camera (position
    and direction jitter around the scene's own), a lens of diameter
    U[0, lens_max] focused on the scene centre, and a shutter U[0,
    shutter_max].  ``scenes`` maps a workload name (cornell, rough_glass,
    divergence) to (scene id, base camera, focus distance)."""
    rng = np.random.default_rng(seed)
    names = sorted(scenes)
    jobs = []
    for k in range(n_jobs):
        name = names[int(rng.integers(len(names)))]
        sid, cam, focus = scenes[name]
        side = int(round(math.exp(rng.uniform(math.log(res[0]), math.log(res[1])))))
        s = int(rng.integers(spp[0], spp[1] + 1))
        sx, sy = _spp_grid(s)
        c = dict(cam)
        c["aspect"] = 1.0
        scale = 0.02 * focus
        c["position"] = tuple(float(p + rng.uniform(-scale, scale)) for p in cam["position"])
        fr = np.asarray(cam["front"], np.float64)
        fr = fr / np.linalg.norm(fr) + rng.uniform(-0.02, 0.02, size=3)
        c["front"] = tuple(float(x) for x in fr)
        c = with_lens(c, float(rng.uniform(0.0, lens_max)), focal_dist=focus)
        c["shutter"] = float(rng.uniform(0.0, shutter_max))
        st = MIX_SETTINGS[name]
        jobs.append(N.job_desc(sid, c, side, side, sx, sy, st["max_depth"], estimator=N.EST_NEE_MIS,
                               sampler=st["sampler"], rr_start=st["rr_start"], env_sampling=st["env_sampling"],
                               seed=seed * 1000 + k))
    return jobs


def textured_cornell(subdiv: int = 3, seed: int = 0) -> tuple[Scene, dict]:
    """The Cornell box with ColorVariant textures: a checker floor, a noise
    back wall, an image on the left wall, a checker-textured light, and the
    sphere a Lambertian mesh with per-vertex uvs (spherical mapping) under a
    noise texture."""
    rng = np.random.default_rng(seed)
    sc = Scene()
    checker = sc.add_texture(N.TEX_CHECKER, (0.1, 0.1, 0.1), (0.8, 0.8, 0.8), scale=40.0)
    noise = sc.add_texture(N.TEX_NOISE, scale=8.0, fractal=4)
    img = (rng.random((16, 24, 3)) * 0.8 + 0.1).astype(np.float32)
    image = sc.add_texture(N.TEX_IMAGE, texels=img)
    lchk = sc.add_texture(N.TEX_CHECKER, (4.0, 2.0, 0.5), (20.0, 14.0, 5.0), scale=30.0)
    snoise = sc.add_texture(N.TEX_NOISE, scale=20.0, fractal=2)
    white = sc.add_material(N.LAMBERTIAN, [0.75, 0.75, 0.75])
    floor = sc.add_material(N.LAMBERTIAN, [0, 0, 0], texture=checker)
    back = sc.add_material(N.LAMBERTIAN, [0, 0, 0], texture=noise)
    left = sc.add_material(N.LAMBERTIAN, [0, 0, 0], texture=image)
    green = sc.add_material(N.LAMBERTIAN, [0.14, 0.45, 0.09])
    light = sc.add_material(N.DIFFUSE_EMITTER, [0, 0, 0, 1.0], texture=lchk)
    ball = sc.add_material(N.LAMBERTIAN, [0, 0, 0], texture=snoise)
    sc.add_quad(1, 0.999, 0.3, 0.7, 0.3, 0.7, light)
    sc.add_quad(0, 1.0, 0.0, 1.0, 0.0, 1.0, left)
    sc.add_quad(0, 0.0, 0.0, 1.0, 0.0, 1.0, green)
    sc.add_quad(1, 0.0, 0.0, 1.0, 0.0, 1.0, floor)
    sc.add_quad(1, 1.0, 0.0, 1.0, 0.0, 1.0, white)
    sc.add_quad(2, 1.0, 0.0, 1.0, 0.0, 1.0, back)
    m = sphere_mesh(subdiv, (0.5, 0.3, 0.55), 0.25, ball)
    d = m.normals.astype(np.float64)
    uvs = np.stack([0.5 + np.arctan2(d[:, 2], d[:, 0]) / (2 * math.pi), 0.5 + np.arcsin(np.clip(d[:, 1], -1, 1)) / math.pi],
                   axis=1).astype(np.float32)
    m.uvs = uvs
    sc.add_mesh(m)
    cam = camera((0.5, 0.5, -1.4), (0.0, 0.0, 1.0), 40.0, 1.0)
    return sc, cam


def hair_curves(n: int = 200, seed: int = 0) -> tuple[Scene, dict]:
    """Strands of cubic Bezier curves (Curve, cylinder segments) in
    Marschner hair of seeded melanin over a Lambertian ground, lit by a quad
    light and a sphere light: the hair BSDF's frame is the curve tangent."""
    rng = np.random.default_rng(seed)
    sc = Scene()
    ground = sc.add_material(N.LAMBERTIAN, [0.5, 0.45, 0.4])
    light = sc.add_material(N.DIFFUSE_EMITTER, [1.0, 0.95, 0.9, 12.0])
    mats = [sc.add_material(N.HAIR, [0, 0, 0, 0.0, 1.55, float(rng.uniform(0.2, 0.4)), float(rng.uniform(0.2, 0.4)),
                                     math.radians(2.0), float(rng.uniform(0.3, 2.5)), 0.0], N.FLAG_MELANIN)
            for _ in range(4)]
    sc.add_quad(1, 0.0, -2.0, 2.0, -2.0, 2.0, ground)
    sc.add_quad(1, 2.5, -0.5, 0.5, -0.5, 0.5, light)
    sc.add_sphere((1.5, 1.5, -1.0), 0.2, light)
    for _ in range(n):
        base = np.array([rng.uniform(-0.8, 0.8), 0.0, rng.uniform(-0.8, 0.8)])
        lean = rng.normal(0, 0.25, size=3)
        lean[1] = 0.0
        h = rng.uniform(0.6, 1.2)
        cps = [base, base + np.array([0, h / 3, 0]) + lean * 0.2, base + np.array([0, 2 * h / 3, 0]) + lean * 0.6,
               base + np.array([0, h, 0]) + lean]
        sc.add_curve(cps, 0.012, 0.004, mats[int(rng.integers(len(mats)))])
    cam = camera((0.0, 0.7, -3.0), (0.0, -0.1, 1.0), 40.0, 1.0)
    return sc, cam
