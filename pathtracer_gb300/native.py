"""ctypes binding of the C-ABI in include/pathtracer_gb300.h.

This is the Python face of the drop-in boundary: the structures mirror the C
header field by field, and :class:`Renderer` wraps a ``pt_context``.  The
library is loaded from the package's ``_lib`` directory; if it is missing
the import fails loudly (there is no CPU fallback on the product path).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libpathtracer_gb300.so"

PT_OK = 0
ERRORS = {
    -1: "PT_ERR_INVALID", -2: "PT_ERR_CUDA", -3: "PT_ERR_NOMEM", -4: "PT_ERR_NOT_FOUND",
    -5: "PT_ERR_DEVICE", -6: "PT_ERR_BUSY", -7: "PT_ERR_CANCELLED", -8: "PT_ERR_TOO_LARGE",
}

# material types (pathtracer_gb300.h)
LAMBERTIAN, CONDUCTOR, MF_DIELECTRIC, THIN_DIELECTRIC, PHONG, DISNEY, HAIR, DIFFUSE_EMITTER = range(8)
FLAG_SPLIT_RAY, FLAG_MELANIN = 1, 2
OBJ_MESH, OBJ_QUAD, OBJ_SPHERE, OBJ_BOX, OBJ_CURVE = 0, 1, 2, 3, 4
EST_REF_NEE, EST_NEE_MIS = 0, 1
SAMPLER_HALTON_NONE, SAMPLER_HALTON_PERMUTE, SAMPLER_HALTON_OWEN, SAMPLER_STRATIFIED = range(4)
ENV_UNIFORM, ENV_ALIAS = 0, 1
BVH_BUILD_HOST, BVH_BUILD_DEVICE, BVH_BUILD_SAH = 0, 1, 2
SERVE_FAIR, SERVE_SRPT = 0, 1
BATCH_GRAPH, BATCH_PERSISTENT = 0, 1

# exported symbols of the C-ABI, in header order
EXPORTS = [
    "pt_create", "pt_destroy", "pt_last_error", "pt_version", "pt_scene_upload", "pt_scene_release",
    "pt_bvh_build", "pt_set_bvh_builder", "pt_bvh_build_device", "pt_bvh_build_sah", "pt_obj_load", "pt_obj_free", "pt_load_image", "pt_free_image", "pt_scene_info", "pt_render", "pt_render_device", "pt_render_device_noalloc", "pt_ray_color",
    "pt_profile_begin",
    "pt_profile_end", "pt_tonemap", "pt_gaussian_blur", "pt_write_png", "pt_sampler_eval", "pt_sample_eval", "pt_trace_closest",
    "pt_trace_any", "pt_intersect", "pt_light_sample", "pt_bsdf_eval", "pt_bsdf_sample", "pt_render_batch", "pt_set_batch_mode", "pt_autotune", "pt_server_create",
    "pt_server_destroy", "pt_submit", "pt_server_step", "pt_poll", "pt_cancel", "pt_server_set_policy",
    "pt_request_times",
]

f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)
u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)


class TextureDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("color1", C.c_float * 3), ("color2", C.c_float * 3), ("scale", C.c_float),
                ("fractal", C.c_int32), ("texels", C.POINTER(C.c_float)), ("width", C.c_int32),
                ("height", C.c_int32)]


TEX_CONSTANT, TEX_CHECKER, TEX_NOISE, TEX_IMAGE = range(4)
MAT_TEXTURE_SHIFT = 8


class MaterialDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("flags", C.c_int32), ("p", C.c_float * 30)]


class MeshDesc(C.Structure):
    _fields_ = [
        ("positions", f32p), ("n_positions", C.c_int32),
        ("normals", f32p), ("n_normals", C.c_int32),
        ("uvs", f32p), ("n_uvs", C.c_int32),
        ("indices", i32p), ("normal_indices", i32p), ("uv_indices", i32p),
        ("n_triangles", C.c_int32), ("material", C.c_int32),
    ]


class QuadDesc(C.Structure):
    _fields_ = [("axis", C.c_int32), ("k", C.c_float), ("d0_min", C.c_float), ("d0_max", C.c_float),
                ("d1_min", C.c_float), ("d1_max", C.c_float), ("material", C.c_int32), ("flip_face", C.c_int32)]


class SphereDesc(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("radius", C.c_float), ("material", C.c_int32),
                ("flip_face", C.c_int32)]


class ObjectDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("index", C.c_int32), ("velocity", C.c_float * 3), ("face", C.c_int32)]


class BoxDesc(C.Structure):
    _fields_ = [("min_xyz", C.c_float * 3), ("max_xyz", C.c_float * 3), ("material", C.c_int32)]


class CurveDesc(C.Structure):
    _fields_ = [("cps", (C.c_float * 3) * 4), ("width0", C.c_float), ("width1", C.c_float), ("material", C.c_int32)]


class EnvDesc(C.Structure):
    _fields_ = [("texels", f32p), ("width", C.c_int32), ("height", C.c_int32), ("intensity", C.c_float)]


class MediumDesc(C.Structure):
    _fields_ = [("sigma_a", C.c_float * 3), ("sigma_s", C.c_float * 3), ("g", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [
        ("materials", C.POINTER(MaterialDesc)), ("n_materials", C.c_int32),
        ("meshes", C.POINTER(MeshDesc)), ("n_meshes", C.c_int32),
        ("quads", C.POINTER(QuadDesc)), ("n_quads", C.c_int32),
        ("spheres", C.POINTER(SphereDesc)), ("n_spheres", C.c_int32),
        ("objects", C.POINTER(ObjectDesc)), ("n_objects", C.c_int32),
        ("env", C.POINTER(EnvDesc)), ("medium", C.POINTER(MediumDesc)),
        ("bg_color", C.c_float * 3), ("bvh_mode", C.c_int32), ("shutter_max", C.c_float),
        ("textures", C.POINTER(TextureDesc)), ("n_textures", C.c_int32),
        ("boxes", C.POINTER(BoxDesc)), ("n_boxes", C.c_int32),
        ("curves", C.POINTER(CurveDesc)), ("n_curves", C.c_int32),
    ]


class CameraDesc(C.Structure):
    _fields_ = [("fov", C.c_float), ("aspect", C.c_float), ("focal_dist", C.c_float), ("aperture", C.c_float),
                ("up", C.c_float * 3), ("front", C.c_float * 3), ("position", C.c_float * 3),
                ("shutter", C.c_float)]


class JobDesc(C.Structure):
    _fields_ = [
        ("scene", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
        ("spp_x", C.c_int32), ("spp_y", C.c_int32), ("spp_begin", C.c_int32), ("spp_end", C.c_int32),
        ("max_depth", C.c_int32), ("rr_start", C.c_int32), ("estimator", C.c_int32), ("sampler", C.c_int32),
        ("env_sampling", C.c_int32), ("light_samples_x", C.c_int32), ("light_samples_y", C.c_int32),
        ("seed", C.c_uint32), ("sampler_seed", C.c_uint32), ("camera", CameraDesc), ("gamma", C.c_float),
        ("crop_x", C.c_int32), ("crop_y", C.c_int32), ("full_width", C.c_int32), ("full_height", C.c_int32),
    ]


class Stats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("segments", C.c_uint64), ("rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("ms", C.c_double), ("algorithmic_bytes", C.c_uint64)]


class Tuning(C.Structure):
    _fields_ = [("wave_paths", C.c_int32), ("sort_by_material", C.c_int32), ("trace_blocks", C.c_int32),
                ("shade_blocks", C.c_int32), ("best_ms", C.c_double), ("default_ms", C.c_double),
                ("candidates", C.c_int32)]


class RequestDesc(C.Structure):
    _fields_ = [("job", JobDesc), ("target_rmse", C.c_float), ("spp_cap", C.c_int32),
                ("spp_per_pass", C.c_int32), ("paths_per_pass", C.c_int32)]


_lib = None


def load() -> C.CDLL:
    """Loads the native library (building nothing): raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"native library missing: {LIB_PATH} (run __graft_entry__.build())")
    lib = C.CDLL(str(LIB_PATH))
    vp = C.c_void_p
    sig = {
        "pt_create": [C.POINTER(vp), C.c_int],
        "pt_destroy": [vp],
        "pt_last_error": [vp, C.c_char_p, C.c_size_t],
        "pt_version": [],
        "pt_scene_upload": [vp, C.POINTER(SceneDesc), i32p],
        "pt_scene_release": [vp, C.c_int32],
        "pt_bvh_build": [C.POINTER(SceneDesc), C.c_int32, C.POINTER(C.c_int64)],
        "pt_set_bvh_builder": [C.c_void_p, C.c_int32],
        "pt_bvh_build_sah": [C.POINTER(SceneDesc), C.c_int32, C.POINTER(C.c_int64)],
        "pt_bvh_build_device": [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(C.c_int64)],
        "pt_obj_load": [C.c_char_p, C.POINTER(MeshDesc)],
        "pt_obj_free": [C.POINTER(MeshDesc)],
        "pt_load_image": [C.c_char_p, C.c_int32, C.c_int32, C.POINTER(f32p), C.POINTER(C.c_int32),
                          C.POINTER(C.c_int32)],
        "pt_free_image": [f32p],
        "pt_scene_info": [vp, C.c_int32, C.POINTER(C.c_int64)],
        "pt_render": [vp, C.POINTER(JobDesc), f32p, C.POINTER(Stats)],
        "pt_render_device": [vp, C.POINTER(JobDesc), vp, C.c_int, C.POINTER(Stats)],
        "pt_render_device_noalloc": [vp, C.POINTER(JobDesc), vp, C.POINTER(Stats)],
        "pt_ray_color": [vp, C.POINTER(JobDesc), f32p, C.c_int32, C.c_uint32, f32p],
        "pt_profile_begin": [vp],
        "pt_profile_end": [vp, C.POINTER(C.c_double), C.POINTER(C.c_int64)],
        "pt_tonemap": [vp, f32p, C.c_int32, C.c_int32, C.c_float, u8p],
        "pt_gaussian_blur": [vp, f32p, f32p, C.c_int32, C.c_int32, C.c_int32, C.c_float],
        "pt_write_png": [C.c_char_p, u8p, C.c_int32, C.c_int32],
        "pt_sampler_eval": [vp, C.c_int32, C.c_uint32, C.c_uint32, C.c_int32, C.c_int32, f32p],
        "pt_sample_eval": [vp, C.POINTER(JobDesc), C.c_int64, C.c_int32, C.c_int32, C.c_int32, f32p, f32p, f32p],
        "pt_trace_closest": [vp, C.c_int32, f32p, C.c_int32, C.c_float, C.c_float, f32p, i32p, f32p],
        "pt_trace_any": [vp, C.c_int32, f32p, f32p, C.c_int32, C.c_float, u8p],
        "pt_intersect": [vp, C.c_int32, f32p, C.c_int32, C.c_float, C.c_float, f32p, i32p, f32p, f32p, u8p],
        "pt_light_sample": [vp, C.c_int32, C.c_int32, C.c_int32, f32p, f32p, f32p, f32p, f32p, f32p, f32p, f32p,
                            f32p],
        "pt_bsdf_eval": [vp, C.POINTER(MaterialDesc), C.c_int32, f32p, f32p, f32p, u8p, f32p, f32p],
        "pt_bsdf_sample": [vp, C.POINTER(MaterialDesc), C.c_int32, f32p, f32p, u8p, f32p, f32p, u8p, f32p,
                           f32p, f32p, u32p],
        "pt_render_batch": [vp, C.POINTER(JobDesc), C.c_int32, C.POINTER(f32p), C.POINTER(Stats)],
        "pt_set_batch_mode": [vp, C.c_int32],
        "pt_autotune": [vp, C.POINTER(JobDesc), C.c_int32, C.POINTER(Tuning)],
        "pt_server_create": [vp, C.c_int64, C.c_int32, C.POINTER(vp)],
        "pt_server_destroy": [vp],
        "pt_submit": [vp, C.POINTER(RequestDesc), C.POINTER(C.c_int64)],
        "pt_server_step": [vp, i32p],
        "pt_poll": [vp, C.c_int64, i32p, f32p, i32p, C.POINTER(C.c_double)],
        "pt_cancel": [vp, C.c_int64],
        "pt_server_set_policy": [vp, C.c_int32, C.c_int64, C.c_int32],
        "pt_request_times": [vp, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double)],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    _lib = lib
    return lib


class PtError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def material(mtype: int, params, flags: int = 0) -> MaterialDesc:
    m = MaterialDesc()
    m.type = mtype
    m.flags = flags
    for i, v in enumerate(params):
        m.p[i] = float(v)
    return m


class SceneBuffers:
    """Keeps the numpy arrays alive that a SceneDesc points into."""

    def __init__(self):
        self.keep = []
        self.desc = SceneDesc()

    def hold(self, a):
        self.keep.append(a)
        return a


def make_scene_desc(scene) -> SceneBuffers:
    """Builds the C description of a :class:`pathtracer_gb300.scene.Scene`."""
    sb = SceneBuffers()
    d = sb.desc
    mats = (MaterialDesc * max(1, len(scene.materials)))(*[material(*m) for m in scene.materials])
    sb.hold(mats)
    d.materials = mats
    d.n_materials = len(scene.materials)
    meshes = (MeshDesc * max(1, len(scene.meshes)))()
    for i, m in enumerate(scene.meshes):
        md = meshes[i]
        pos = sb.hold(np.ascontiguousarray(m.positions, dtype=np.float32))
        idx = sb.hold(np.ascontiguousarray(m.indices, dtype=np.int32))
        md.positions = _ptr(pos, C.c_float)
        md.n_positions = pos.shape[0]
        md.indices = _ptr(idx, C.c_int32)
        md.n_triangles = idx.shape[0]
        if m.normals is not None:
            nrm = sb.hold(np.ascontiguousarray(m.normals, dtype=np.float32))
            md.normals = _ptr(nrm, C.c_float)
            md.n_normals = nrm.shape[0]
        if getattr(m, "uvs", None) is not None:
            uv = sb.hold(np.ascontiguousarray(m.uvs, dtype=np.float32))
            md.uvs = _ptr(uv, C.c_float)
            md.n_uvs = uv.shape[0]
        md.material = m.material
    sb.hold(meshes)
    d.meshes = meshes
    d.n_meshes = len(scene.meshes)
    quads = (QuadDesc * max(1, len(scene.quads)))()
    for i, q in enumerate(scene.quads):
        quads[i] = QuadDesc(q[0], *[float(x) for x in q[1:6]], q[6], q[7] if len(q) > 7 else 0)
    sb.hold(quads)
    d.quads = quads
    d.n_quads = len(scene.quads)
    spheres = (SphereDesc * max(1, len(scene.spheres)))()
    for i, s in enumerate(scene.spheres):
        sd = spheres[i]
        sd.center[:] = [float(x) for x in s[0]]
        sd.radius = float(s[1])
        sd.material = s[2]
        sd.flip_face = s[3] if len(s) > 3 else 0
    sb.hold(spheres)
    d.spheres = spheres
    d.n_spheres = len(scene.spheres)
    objs = (ObjectDesc * max(1, len(scene.objects)))(
        *[ObjectDesc(o[0], o[1], (C.c_float * 3)(*[float(x) for x in (o[2] if len(o) > 2 else (0, 0, 0))]),
                     int(o[3]) if len(o) > 3 else 0)
          for o in scene.objects])
    sb.hold(objs)
    d.objects = objs
    d.n_objects = len(scene.objects)
    if scene.env is not None:
        tex = sb.hold(np.ascontiguousarray(scene.env, dtype=np.float32))
        ed = EnvDesc(_ptr(tex, C.c_float), tex.shape[1], tex.shape[0], float(scene.env_intensity))
        sb.hold(ed)
        d.env = C.pointer(ed)
    if scene.medium is not None:
        sa, ss, g = scene.medium
        md = MediumDesc((C.c_float * 3)(*sa), (C.c_float * 3)(*ss), float(g))
        sb.hold(md)
        d.medium = C.pointer(md)
    d.bg_color[:] = [float(x) for x in scene.bg]
    d.shutter_max = float(getattr(scene, "shutter_max", 0.0))
    boxes = getattr(scene, "boxes", [])
    if boxes:
        barr = (BoxDesc * len(boxes))(*[BoxDesc((C.c_float * 3)(*[float(x) for x in b[0]]),
                                                (C.c_float * 3)(*[float(x) for x in b[1]]), b[2]) for b in boxes])
        sb.hold(barr)
        d.boxes = barr
        d.n_boxes = len(boxes)
    curves = getattr(scene, "curves", [])
    if curves:
        carr = (CurveDesc * len(curves))()
        for i, (cps, w0, w1, mat) in enumerate(curves):
            for k in range(4):
                carr[i].cps[k][:] = [float(x) for x in cps[k]]
            carr[i].width0, carr[i].width1, carr[i].material = float(w0), float(w1), mat
        sb.hold(carr)
        d.curves = carr
        d.n_curves = len(curves)
    texs = getattr(scene, "textures", [])
    if texs:
        arr = (TextureDesc * len(texs))()
        for i, t in enumerate(texs):
            td = arr[i]
            td.kind = t["kind"]
            td.color1[:] = [float(x) for x in t.get("color1", (0, 0, 0))]
            td.color2[:] = [float(x) for x in t.get("color2", (1, 1, 1))]
            td.scale = float(t.get("scale", 10.0))
            td.fractal = int(t.get("fractal", 1))
            if t["kind"] == TEX_IMAGE:
                img = sb.hold(np.ascontiguousarray(t["texels"], dtype=np.float32))
                td.texels = _ptr(img, C.c_float)
                td.height, td.width = img.shape[0], img.shape[1]
        sb.hold(arr)
        d.textures = arr
        d.n_textures = len(texs)
    return sb


def job_desc(scene_id: int, cam, width: int, height: int, spp_x: int, spp_y: int, max_depth: int,
             estimator: int = EST_REF_NEE, sampler: int = SAMPLER_HALTON_OWEN, rr_start: int = -1,
             env_sampling: int = ENV_UNIFORM, seed: int = 0, spp_begin: int = 0, spp_end: int = 0,
             light_samples=(2, 2), sampler_seed: int = 0, gamma: float = 2.0) -> JobDesc:
    j = JobDesc()
    j.scene = scene_id
    j.width, j.height = width, height
    j.spp_x, j.spp_y = spp_x, spp_y
    j.spp_begin, j.spp_end = spp_begin, spp_end
    j.max_depth = max_depth
    j.rr_start = rr_start
    j.estimator = estimator
    j.sampler = sampler
    j.env_sampling = env_sampling
    j.light_samples_x, j.light_samples_y = light_samples
    j.seed = seed
    j.sampler_seed = sampler_seed
    j.camera = camera_desc(cam)
    j.gamma = gamma
    return j


def camera_desc(cam) -> CameraDesc:
    c = CameraDesc()
    c.fov = float(cam["fov"])
    c.aspect = float(cam["aspect"])
    c.focal_dist = float(cam["focal_dist"])
    c.aperture = float(cam["aperture"])
    c.up[:] = [float(x) for x in cam["up"]]
    c.front[:] = [float(x) for x in cam["front"]]
    c.position[:] = [float(x) for x in cam["position"]]
    c.shutter = float(cam.get("shutter", 0.0))
    return c


class Renderer:
    """A pt_context on one CUDA device."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.ctx = C.c_void_p()
        self._check(self.lib.pt_create(C.byref(self.ctx), device), None)

    def close(self):
        if self.ctx:
            self.lib.pt_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, ctx=-1):
        if rc != PT_OK:
            buf = C.create_string_buffer(512)
            self.lib.pt_last_error(self.ctx if ctx == -1 else ctx, buf, 512)
            raise PtError(rc, buf.value.decode())

    # -- scenes
    def upload(self, scene) -> int:
        sb = make_scene_desc(scene)
        sid = C.c_int32()
        self._check(self.lib.pt_scene_upload(self.ctx, C.byref(sb.desc), C.byref(sid)))
        return sid.value

    def release(self, sid: int):
        self._check(self.lib.pt_scene_release(self.ctx, sid))

    def set_bvh_builder(self, builder: int):
        """BVH_BUILD_HOST (the reference's trees, default), BVH_BUILD_DEVICE
        (the reference's split rule, large meshes built on the GPU) or
        BVH_BUILD_SAH (binned-SAH trees) for later uploads; all give the same
        hits up to exact ties in t."""
        self._check(self.lib.pt_set_bvh_builder(self.ctx, int(builder)))

    def bvh_build_device(self, scene) -> dict:
        """pt_bvh_build_device: the scene's BVH4 with large meshes built on the
        GPU, not kept (same keys as bvh_build)."""
        sb = make_scene_desc(scene)
        out = (C.c_int64 * 5)()
        self._check(self.lib.pt_bvh_build_device(self.ctx, C.byref(sb.desc), out))
        return {"nodes": out[0], "items": out[1], "depth": out[2], "hash": out[3] & 0xffffffffffffffff,
                "build_us": out[4]}

    def scene_info(self, sid: int):
        out = (C.c_int64 * 6)()
        self._check(self.lib.pt_scene_info(self.ctx, sid, out))
        return dict(zip(["triangles", "quads", "spheres", "bvh4_nodes", "lights", "device_bytes"], list(out)))

    # -- rendering
    def render(self, job: JobDesc, stats: bool = False):
        film = np.zeros((job.height, job.width, 3), np.float32)
        st = Stats()
        self._check(self.lib.pt_render(self.ctx, C.byref(job), _ptr(film, C.c_float), C.byref(st)))
        return (film, st) if stats else film

    def render_device(self, job: JobDesc, d_film_ptr: int, sync: bool = False, stats: bool = False):
        st = Stats()
        self._check(self.lib.pt_render_device(self.ctx, C.byref(job), C.c_void_p(d_film_ptr), int(sync),
                                              C.byref(st) if stats else None))
        return st

    def ray_color(self, job: JobDesc, rays: np.ndarray, first_index: int = 1) -> np.ndarray:
        """pt_ray_color: one path's radiance per given primary ray (n, 3)."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        out = np.zeros((rays.shape[0], 3), np.float32)
        self._check(self.lib.pt_ray_color(self.ctx, C.byref(job), _ptr(rays, C.c_float), rays.shape[0], first_index,
                                          _ptr(out, C.c_float)))
        return out

    STAGES = ["camera", "trace", "sort", "shade", "shadow", "film"]

    def profile_begin(self):
        self._check(self.lib.pt_profile_begin(self.ctx))

    def profile_end(self) -> dict:
        ms = (C.c_double * 6)()
        nl = (C.c_int64 * 6)()
        self._check(self.lib.pt_profile_end(self.ctx, ms, nl))
        return {k: (ms[i], nl[i]) for i, k in enumerate(self.STAGES)}

    def gaussian_blur(self, film: np.ndarray, kernel: int, sigma: float) -> np.ndarray:
        """pt_gaussian_blur of an (H, W, 3) float32 film."""
        f = np.ascontiguousarray(film, dtype=np.float32)
        out = np.empty_like(f)
        self._check(self.lib.pt_gaussian_blur(self.ctx, _ptr(f, C.c_float), _ptr(out, C.c_float), f.shape[1],
                                              f.shape[0], kernel, sigma))
        return out

    def tonemap(self, film: np.ndarray, gamma: float = 2.0) -> np.ndarray:
        film = np.ascontiguousarray(film, dtype=np.float32)
        h, w = film.shape[:2]
        out = np.zeros((h, w, 3), np.uint8)
        self._check(self.lib.pt_tonemap(self.ctx, _ptr(film, C.c_float), w, h, gamma, _ptr(out, C.c_uint8)))
        return out

    # -- batch test entry points
    def render_batch(self, jobs, stats: bool = False):
        """pt_render_batch: one graph launch for all jobs; returns the mean films."""
        n = len(jobs)
        arr = (JobDesc * n)(*jobs)
        films = [np.zeros((j.height, j.width, 3), np.float32) for j in jobs]
        ptrs = (f32p * n)(*[_ptr(f, C.c_float) for f in films])
        st = Stats()
        self._check(self.lib.pt_render_batch(self.ctx, arr, n, ptrs, C.byref(st)))
        return (films, st) if stats else films

    def set_batch_mode(self, mode: int):
        """pt_set_batch_mode: BATCH_GRAPH (per-stage kernels in one graph) or
        BATCH_PERSISTENT (one cooperative launch per scene group)."""
        self._check(self.lib.pt_set_batch_mode(self.ctx, mode))

    def autotune(self, jobs) -> dict:
        n = len(jobs)
        arr = (JobDesc * n)(*jobs)
        t = Tuning()
        self._check(self.lib.pt_autotune(self.ctx, arr, n, C.byref(t)))
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def sampler_eval(self, strategy: int, first_index: int, n: int, dims: int, seed: int = 0) -> np.ndarray:
        out = np.zeros((n, dims), np.float32)
        self._check(self.lib.pt_sampler_eval(self.ctx, strategy, seed, first_index, n, dims,
                                             _ptr(out, C.c_float)))
        return out

    def sample_eval(self, job: JobDesc, first_path: int, n: int, dims: int, bounces: int = 0):
        """pt_sample_eval: (pixel offsets (n, 2), dimension values (n, dims),
        light offsets (n, bounces, LN, 2)) of the job's paths first_path..+n."""
        ln = job.light_samples_x * job.light_samples_y
        pix = np.zeros((n, 2), np.float32)
        dv = np.zeros((n, dims), np.float32)
        lo = np.zeros((n, bounces, ln, 2), np.float32)
        self._check(self.lib.pt_sample_eval(self.ctx, C.byref(job), first_path, n, dims, bounces,
                                            _ptr(pix, C.c_float), _ptr(dv, C.c_float), _ptr(lo, C.c_float)))
        return pix, dv, lo

    def trace_closest(self, sid: int, rays: np.ndarray, tmin: float = 1e-4, tmax: float = 1e5):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[0]
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        uv = np.zeros((n, 2), np.float32)
        self._check(self.lib.pt_trace_closest(self.ctx, sid, _ptr(rays, C.c_float), n, tmin, tmax,
                                              _ptr(t, C.c_float), _ptr(prim, C.c_int32), _ptr(uv, C.c_float)))
        return t, prim, uv

    def trace_any(self, sid: int, rays: np.ndarray, tmax: np.ndarray, tmin: float = 1e-3):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        tmax = np.ascontiguousarray(tmax, dtype=np.float32)
        occ = np.zeros(rays.shape[0], np.uint8)
        self._check(self.lib.pt_trace_any(self.ctx, sid, _ptr(rays, C.c_float), _ptr(tmax, C.c_float),
                                          rays.shape[0], tmin, _ptr(occ, C.c_uint8)))
        return occ

    def intersect(self, sid: int, rays: np.ndarray, tmin: float = 1e-4, tmax: float = 1e5):
        """pt_intersect: (t, prim, position, normal, is_inside) of each ray's closest hit."""
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[0]
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        pos = np.zeros((n, 3), np.float32)
        nrm = np.zeros((n, 3), np.float32)
        ins = np.zeros(n, np.uint8)
        self._check(self.lib.pt_intersect(self.ctx, sid, _ptr(rays, C.c_float), n, tmin, tmax, _ptr(t, C.c_float),
                                          _ptr(prim, C.c_int32), _ptr(pos, C.c_float), _ptr(nrm, C.c_float),
                                          _ptr(ins, C.c_uint8)))
        return t, prim, pos, nrm, ins

    def light_sample(self, sid: int, light: int, uv: np.ndarray, x: np.ndarray, pdf_dir=None):
        """pt_light_sample: dict of point, normal, dir, le, pdf (per item) and
        area; pdf at pdf_dir (n, 3) when given, else at the sample's direction."""
        uv = np.ascontiguousarray(uv, dtype=np.float32).reshape(-1, 2)
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 3)
        pd = None if pdf_dir is None else np.ascontiguousarray(pdf_dir, dtype=np.float32).reshape(-1, 3)
        n = uv.shape[0]
        out = {k: np.zeros((n, 3), np.float32) for k in ("point", "normal", "dir", "le")}
        out["pdf"] = np.zeros(n, np.float32)
        area = C.c_float()
        self._check(self.lib.pt_light_sample(self.ctx, sid, light, n, _ptr(uv, C.c_float), _ptr(x, C.c_float),
                                             None if pd is None else _ptr(pd, C.c_float),
                                             *(_ptr(out[k], C.c_float) for k in ("point", "normal", "dir", "le",
                                                                                 "pdf")), C.byref(area)))
        out["area"] = area.value
        return out

    def bsdf_eval(self, mat: MaterialDesc, wo, wi, normal, front):
        wo, wi, normal = (np.ascontiguousarray(a, dtype=np.float32) for a in (wo, wi, normal))
        front = np.ascontiguousarray(front, dtype=np.uint8)
        n = wo.shape[0]
        f = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        self._check(self.lib.pt_bsdf_eval(self.ctx, C.byref(mat), n, _ptr(wo, C.c_float), _ptr(wi, C.c_float),
                                          _ptr(normal, C.c_float), _ptr(front, C.c_uint8), _ptr(f, C.c_float),
                                          _ptr(pdf, C.c_float)))
        return f, pdf

    def bsdf_sample(self, mat: MaterialDesc, wo, normal, front, uc, u):
        wo, normal, uc, u = (np.ascontiguousarray(a, dtype=np.float32) for a in (wo, normal, uc, u))
        front = np.ascontiguousarray(front, dtype=np.uint8)
        n = wo.shape[0]
        ok = np.zeros(n, np.uint8)
        wi = np.zeros((n, 3), np.float32)
        att = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        ty = np.zeros(n, np.uint32)
        self._check(self.lib.pt_bsdf_sample(self.ctx, C.byref(mat), n, _ptr(wo, C.c_float), _ptr(normal, C.c_float),
                                            _ptr(front, C.c_uint8), _ptr(uc, C.c_float), _ptr(u, C.c_float),
                                            _ptr(ok, C.c_uint8), _ptr(wi, C.c_float), _ptr(att, C.c_float),
                                            _ptr(pdf, C.c_float), _ptr(ty, C.c_uint32)))
        return ok.astype(bool), wi, att, pdf, ty


def load_image(path, flip_y: bool = False, hdr: bool = False) -> np.ndarray:
    """pt_load_image, ImageTexture(path, flip_y, isHDR)'s texels: (H, W, 3)
    float32 whose row y is the reference's texels[x][y] (y = 0 the bottom row
    of the image, its top row with flip_y)."""
    lib = load()
    p = f32p()
    w, h = C.c_int32(), C.c_int32()
    rc = lib.pt_load_image(str(path).encode(), int(flip_y), int(hdr), C.byref(p), C.byref(w), C.byref(h))
    if rc != PT_OK:
        buf = C.create_string_buffer(512)
        lib.pt_last_error(None, buf, 512)
        raise PtError(rc, buf.value.decode())
    try:
        return np.ctypeslib.as_array(p, shape=(h.value * w.value * 3,)).reshape(h.value, w.value, 3).copy()
    finally:
        lib.pt_free_image(p)


def write_png(path, rgb8: np.ndarray) -> None:
    """pt_write_png of an (H, W, 3) uint8 image (row 0 = top)."""
    lib = load()
    a = np.ascontiguousarray(rgb8, dtype=np.uint8)
    rc = lib.pt_write_png(str(path).encode(), _ptr(a, C.c_uint8), a.shape[1], a.shape[0])
    if rc != PT_OK:
        buf = C.create_string_buffer(512)
        lib.pt_last_error(None, buf, 512)
        raise PtError(rc, buf.value.decode())


def bvh_build(scene, threads: int = 0, sah: bool = False) -> dict:
    """pt_bvh_build (the reference's trees) or pt_bvh_build_sah: the scene's
    BVH4 built on the host only (no GPU)."""
    lib = load()
    sb = make_scene_desc(scene)
    out = (C.c_int64 * 5)()
    rc = (lib.pt_bvh_build_sah if sah else lib.pt_bvh_build)(C.byref(sb.desc), threads, out)
    if rc != PT_OK:
        buf = C.create_string_buffer(512)
        lib.pt_last_error(None, buf, 512)
        raise PtError(rc, buf.value.decode())
    return {"nodes": out[0], "items": out[1], "depth": out[2], "hash": out[3] & 0xffffffffffffffff,
            "build_us": out[4]}


def obj_load(path) -> dict:
    """pt_obj_load: an OBJ file as numpy arrays (positions, normals, uvs,
    indices, normal_indices, uv_indices; -1 where a face has no normal/uv)."""
    lib = load()
    md = MeshDesc()
    rc = lib.pt_obj_load(str(path).encode(), C.byref(md))
    if rc != PT_OK:
        buf = C.create_string_buffer(512)
        lib.pt_last_error(None, buf, 512)
        raise PtError(rc, buf.value.decode())
    try:
        def arr(ptr, n, w, dt):
            if not ptr or n == 0:
                return np.zeros((0, w), dt)
            return np.ctypeslib.as_array(ptr, shape=(n * w,)).reshape(n, w).astype(dt, copy=True)
        return {"positions": arr(md.positions, md.n_positions, 3, np.float32),
                "normals": arr(md.normals, md.n_normals, 3, np.float32),
                "uvs": arr(md.uvs, md.n_uvs, 2, np.float32),
                "indices": arr(md.indices, md.n_triangles, 3, np.int32),
                "normal_indices": arr(md.normal_indices, md.n_triangles, 3, np.int32),
                "uv_indices": arr(md.uv_indices, md.n_triangles, 3, np.int32)}
    finally:
        lib.pt_obj_free(C.byref(md))


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_CANCELLED, REQ_FAILED = range(5)


class Server:
    """Request loop over a :class:`Renderer` (pt_server_* / pt_submit / pt_poll).

    Each ``step()`` admits queued requests while slots and the HBM budget
    allow, then adds ``spp_per_pass`` samples to every active request in one
    batched launch.
    """

    def __init__(self, renderer: Renderer, hbm_budget: int = 8 << 30, max_slots: int = 64):
        self.r = renderer
        self.lib = renderer.lib
        self.handle = C.c_void_p()
        renderer._check(self.lib.pt_server_create(renderer.ctx, hbm_budget, max_slots, C.byref(self.handle)))
        self.shapes = {}

    def close(self):
        if self.handle:
            self.lib.pt_server_destroy(self.handle)
            self.handle = C.c_void_p()

    def submit(self, job: JobDesc, target_rmse: float = 0.0, spp_cap: int = 0, spp_per_pass: int = 1,
               paths_per_pass: int = 0) -> int:
        req = RequestDesc()
        req.job = job
        req.target_rmse = target_rmse
        req.spp_cap = spp_cap if spp_cap > 0 else job.spp_x * job.spp_y
        req.spp_per_pass = spp_per_pass
        req.paths_per_pass = paths_per_pass
        rid = C.c_int64()
        self.r._check(self.lib.pt_submit(self.handle, C.byref(req), C.byref(rid)))
        self.shapes[rid.value] = (job.height, job.width, 3)
        return rid.value

    def set_policy(self, policy: int, pass_paths: int = 0, max_queue: int = 0):
        """pt_server_set_policy: SERVE_FAIR or SERVE_SRPT (shortest remaining
        work first, pass_paths per pass); max_queue > 0 refuses submissions
        (PtError PT_ERR_BUSY) while that many requests are queued."""
        self.r._check(self.lib.pt_server_set_policy(self.handle, policy, pass_paths, max_queue))

    def times(self, rid: int):
        """(queue_ms, latency_ms) of a request, -1 where not reached."""
        q, lat = C.c_double(), C.c_double()
        self.r._check(self.lib.pt_request_times(self.handle, rid, C.byref(q), C.byref(lat)))
        return q.value, lat.value

    def step(self) -> int:
        active = C.c_int32()
        self.r._check(self.lib.pt_server_step(self.handle, C.byref(active)))
        return active.value

    def poll(self, rid: int):
        """(state, film or None, spp_done, latency_ms)."""
        st = C.c_int32()
        done = C.c_int32()
        lat = C.c_double()
        film = np.zeros(self.shapes[rid], np.float32)
        self.r._check(self.lib.pt_poll(self.handle, rid, C.byref(st), _ptr(film, C.c_float), C.byref(done),
                                       C.byref(lat)))
        return st.value, (film if st.value == REQ_DONE else None), done.value, lat.value

    def state(self, rid: int):
        """(state, spp_done) without copying the film."""
        st = C.c_int32()
        done = C.c_int32()
        self.r._check(self.lib.pt_poll(self.handle, rid, C.byref(st), None, C.byref(done), None))
        return st.value, done.value

    def cancel(self, rid: int):
        self.r._check(self.lib.pt_cancel(self.handle, rid))
