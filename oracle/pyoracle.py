"""Python binding of the CPU oracle (oracle/pt_oracle.cpp).

ORACLE: test infrastructure.  Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use it, as the checker of the CUDA path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from pathtracer_gb300 import native as N

from .build_oracle import OUT, build

f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)
u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)

_lib = None


def load():
    global _lib
    if _lib is None:
        if not OUT.exists():
            build()
        lib = C.CDLL(str(OUT))
        lib.or_scene_create.argtypes = [C.POINTER(N.SceneDesc)]
        lib.or_scene_create.restype = C.c_void_p
        lib.or_scene_destroy.argtypes = [C.c_void_p]
        lib.or_scene_num_lights.argtypes = [C.c_void_p]
        lib.or_sampler_eval.argtypes = [C.c_int, C.c_uint32, C.c_uint32, C.c_int, C.c_int, f32p]
        lib.or_ray_color.argtypes = [C.c_void_p, C.POINTER(N.JobDesc), f32p, C.c_int, C.c_uint32, f32p, C.c_int]
        lib.or_light_eval.argtypes = [C.c_void_p, C.c_int, C.c_int, f32p, f32p, f32p, f32p, f32p, f32p, f32p, f32p,
                                      f32p]
        lib.or_intersect.argtypes = [C.c_void_p, f32p, C.c_int, C.c_float, C.c_float, f32p, i32p, f32p, f32p, u8p]
        lib.or_path_samples.argtypes = [C.POINTER(N.JobDesc), C.c_int64, C.c_int, C.c_int, C.c_int, f32p, f32p,
                                        f32p]
        lib.or_trace_closest.argtypes = [C.c_void_p, f32p, C.c_int, C.c_float, C.c_float, f32p, i32p]
        lib.or_bsdf_eval.argtypes = [C.POINTER(N.MaterialDesc), C.c_int, f32p, f32p, f32p, u8p, f32p, f32p]
        lib.or_bsdf_sample.argtypes = [C.POINTER(N.MaterialDesc), C.c_int, f32p, f32p, u8p, f32p, f32p, u8p, f32p,
                                       f32p, f32p, u32p]
        lib.or_render.argtypes = [C.c_void_p, C.POINTER(N.JobDesc), f32p, f32p, C.c_int, C.c_int]
        lib.or_gaussian_blur.argtypes = [f32p, f32p, C.c_int, C.c_int, C.c_int, C.c_float]
        lib.or_tex_eval.argtypes = [C.POINTER(N.TextureDesc), C.c_int, f32p, f32p]
        _lib = lib
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class OracleScene:
    def __init__(self, scene):
        self.lib = load()
        self.sb = N.make_scene_desc(scene)
        self.h = self.lib.or_scene_create(C.byref(self.sb.desc))

    def __del__(self):
        try:
            self.lib.or_scene_destroy(self.h)
        except Exception:
            pass

    def trace_closest(self, rays, tmin=1e-4, tmax=1e5):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        self.lib.or_trace_closest(self.h, _p(rays, C.c_float), n, tmin, tmax, _p(t, C.c_float), _p(prim, C.c_int32))
        return t, prim

    def ray_color(self, job, rays, first_index=1, recursive=True):
        """or_ray_color: one path's radiance per given primary ray (n, 3)."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        out = np.zeros((rays.shape[0], 3), np.float32)
        self.lib.or_ray_color(self.h, C.byref(job), _p(rays, C.c_float), rays.shape[0], first_index,
                              _p(out, C.c_float), 1 if recursive else 0)
        return out

    def light_eval(self, light: int, uv, x, pdf_dir=None):
        """or_light_eval: dict of point, normal, dir, le, pdf per item and area
        (pdf at pdf_dir when given)."""
        uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
        pd = None if pdf_dir is None else np.ascontiguousarray(pdf_dir, np.float32).reshape(-1, 3)
        n = uv.shape[0]
        out = {k: np.zeros((n, 3), np.float32) for k in ("point", "normal", "dir", "le")}
        out["pdf"] = np.zeros(n, np.float32)
        area = C.c_float()
        if self.lib.or_light_eval(self.h, light, n, _p(uv, C.c_float), _p(x, C.c_float),
                                  None if pd is None else _p(pd, C.c_float),
                                  *(_p(out[k], C.c_float) for k in ("point", "normal", "dir", "le", "pdf")),
                                  C.byref(area)) != 0:
            raise ValueError("bad light index")
        out["area"] = area.value
        return out

    def intersect(self, rays, tmin=1e-4, tmax=1e5):
        """(t, prim, position, normal, is_inside) of each ray's closest hit."""
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        pos = np.zeros((n, 3), np.float32)
        nrm = np.zeros((n, 3), np.float32)
        ins = np.zeros(n, np.uint8)
        self.lib.or_intersect(self.h, _p(rays, C.c_float), n, tmin, tmax, _p(t, C.c_float), _p(prim, C.c_int32),
                              _p(pos, C.c_float), _p(nrm, C.c_float), _p(ins, C.c_uint8))
        return t, prim, pos, nrm, ins

    def render(self, job, threads=0, recursive=True):
        mean = np.zeros((job.height, job.width, 3), np.float32)
        var = np.zeros_like(mean)
        self.lib.or_render(self.h, C.byref(job), _p(mean, C.c_float), _p(var, C.c_float), threads,
                           1 if recursive else 0)
        return mean, var


def render(scene, job, threads=0, recursive=True):
    return OracleScene(scene).render(job, threads, recursive)


def sampler_eval(strategy, first_index, n, dims, seed=0):
    out = np.zeros((n, dims), np.float32)
    load().or_sampler_eval(strategy, seed, first_index, n, dims, _p(out, C.c_float))
    return out


def path_samples(job, first_path, n, dims, bounces=0):
    """or_path_samples: (pixel offsets (n, 2), dimension values (n, dims),
    light offsets (n, bounces, LN, 2)) of the job's paths first_path..+n."""
    ln = job.light_samples_x * job.light_samples_y
    pix = np.zeros((n, 2), np.float32)
    dv = np.zeros((n, max(dims, 1)), np.float32)
    lo = np.zeros((n, max(bounces, 1), ln, 2), np.float32)
    load().or_path_samples(C.byref(job), first_path, n, dims, bounces, _p(pix, C.c_float), _p(dv, C.c_float),
                           _p(lo, C.c_float))
    return pix, dv[:, :dims], lo[:, :bounces]


def bsdf_eval(mat, wo, wi, nrm, front):
    wo, wi, nrm = (np.ascontiguousarray(a, np.float32) for a in (wo, wi, nrm))
    front = np.ascontiguousarray(front, np.uint8)
    n = wo.shape[0]
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    load().or_bsdf_eval(C.byref(mat), n, _p(wo, C.c_float), _p(wi, C.c_float), _p(nrm, C.c_float),
                        _p(front, C.c_uint8), _p(f, C.c_float), _p(pdf, C.c_float))
    return f, pdf


def bsdf_sample(mat, wo, nrm, front, uc, u):
    wo, nrm, uc, u = (np.ascontiguousarray(a, np.float32) for a in (wo, nrm, uc, u))
    front = np.ascontiguousarray(front, np.uint8)
    n = wo.shape[0]
    ok = np.zeros(n, np.uint8)
    wi = np.zeros((n, 3), np.float32)
    att = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    ty = np.zeros(n, np.uint32)
    load().or_bsdf_sample(C.byref(mat), n, _p(wo, C.c_float), _p(nrm, C.c_float), _p(front, C.c_uint8),
                          _p(uc, C.c_float), _p(u, C.c_float), _p(ok, C.c_uint8), _p(wi, C.c_float),
                          _p(att, C.c_float), _p(pdf, C.c_float), _p(ty, C.c_uint32))
    return ok, wi, att, pdf, ty


def tex_eval(kind: int, uv: np.ndarray, color1=(0, 0, 0), color2=(1, 1, 1), scale: float = 10.0,
             fractal: int = 1, texels: np.ndarray | None = None) -> np.ndarray:
    """A surface texture evaluated at each (u, v) (or_tex_eval)."""
    d = N.TextureDesc()
    d.kind, d.scale, d.fractal = kind, scale, fractal
    d.color1[:] = list(color1)
    d.color2[:] = list(color2)
    keep = None
    if texels is not None:
        keep = np.ascontiguousarray(texels, np.float32)
        d.texels = _p(keep, C.c_float)
        d.height, d.width = keep.shape[0], keep.shape[1]
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    out = np.zeros((uv.shape[0], 3), np.float32)
    if load().or_tex_eval(C.byref(d), uv.shape[0], _p(uv, C.c_float), _p(out, C.c_float)) != 0:
        raise ValueError("bad texture description")
    return out


def gaussian_blur(film, kernel, sigma):
    """FrameBuffer::gaussianBlur restated on the CPU (or_gaussian_blur)."""
    lib = load()
    f = np.ascontiguousarray(film, dtype=np.float32)
    out = np.empty_like(f)
    lib.or_gaussian_blur(_p(f, C.c_float), _p(out, C.c_float), f.shape[1], f.shape[0], kernel, sigma)
    return out
