"""ctypes binding of oracle/_ref/libref_harness.so (the harness around the
unmodified reference sources, built by oracle/ref/build_ref.sh).

ORACLE INFRASTRUCTURE ONLY: used by tests/golden/make_golden.py to write the
golden fixtures, and by CPU tests in this container when the reference
sources are present.  It exists only where the reference builds (never on
the GPU machine).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from pathtracer_gb300 import native as N

LIB = Path(__file__).resolve().parents[1] / "_ref" / "libref_harness.so"


def _ref_root():
    """The reference sources the harness was built from: $REF_ROOT, else the
    root build_ref.sh recorded beside the library; None when neither exists."""
    if os.environ.get("REF_ROOT"):
        return Path(os.environ["REF_ROOT"])
    rec = LIB.parent / "REF_ROOT"
    return Path(rec.read_text().strip()) if rec.exists() else None


REF_ROOT = _ref_root()

f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)
u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)


def available() -> bool:
    return LIB.exists()


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(LIB))
        lib.ref_scene_create.argtypes = [C.POINTER(N.SceneDesc)]
        lib.ref_scene_create.restype = C.c_void_p
        lib.ref_scene_destroy.argtypes = [C.c_void_p]
        lib.ref_scene_num_lights.argtypes = [C.c_void_p]
        lib.ref_trace_closest.argtypes = [C.c_void_p, f32p, C.c_int, C.c_float, C.c_float, f32p, i32p, f32p, f32p,
                                          u8p]
        lib.ref_light_eval.argtypes = [C.c_void_p, C.c_int, C.c_int, f32p, f32p, f32p, f32p, f32p, f32p, f32p, f32p,
                                       f32p]
        lib.ref_scene_transform.argtypes = [C.c_void_p, C.c_int, C.c_int, i32p, f32p]
        lib.ref_bsdf_eval.argtypes = [C.POINTER(N.MaterialDesc), C.c_int, f32p, f32p, f32p, u8p, f32p, f32p]
        lib.ref_bsdf_sample.argtypes = [C.POINTER(N.MaterialDesc), C.c_int, f32p, f32p, u8p, f32p, f32p, u8p, f32p,
                                        f32p, f32p, u32p]
        lib.ref_sampler_eval.argtypes = [C.c_int, C.c_uint32, C.c_uint32, C.c_int, C.c_int, f32p]
        lib.ref_offsets.argtypes = [C.c_int, C.c_int, C.c_uint64, f32p]
        lib.ref_render.argtypes = [C.c_void_p, C.POINTER(N.JobDesc), f32p, f32p, C.c_int]
        lib.ref_render_time.argtypes = [C.c_void_p, C.POINTER(N.JobDesc), C.c_int]
        lib.ref_render_time.restype = C.c_double
        lib.ref_image_texels.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, f32p, f32p]
        lib.ref_texture_eval.argtypes = [C.c_int, f32p, f32p, C.c_float, C.c_int, C.c_int, f32p, f32p]
        lib.ref_gaussian_blur.argtypes = [f32p, C.c_int, C.c_int, C.c_int, C.c_float, f32p]
        lib.ref_write_png.argtypes = [f32p, C.c_int, C.c_int, C.c_float, C.c_char_p]
        lib.ref_obj_load.argtypes = [C.c_char_p, C.POINTER(C.c_int64), f32p, f32p, f32p, i32p, i32p, i32p]
        _lib = lib
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class RefScene:
    def __init__(self, scene):
        self.lib = load()
        self.sb = N.make_scene_desc(scene)
        self.h = self.lib.ref_scene_create(C.byref(self.sb.desc))

    def __del__(self):
        try:
            self.lib.ref_scene_destroy(self.h)
        except Exception:
            pass

    def trace_closest(self, rays, tmin=1e-4, tmax=1e5):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        pos = np.zeros((n, 3), np.float32)
        nrm = np.zeros((n, 3), np.float32)
        front = np.zeros(n, np.uint8)
        self.lib.ref_trace_closest(self.h, _p(rays, C.c_float), n, tmin, tmax, _p(t, C.c_float),
                                   _p(prim, C.c_int32), _p(pos, C.c_float), _p(nrm, C.c_float),
                                   _p(front, C.c_uint8))
        return t, prim, pos, nrm, front

    def light_eval(self, light: int, uv, x, pdf_dir=None):
        """Light methods of light `light` (ref_light_eval): dict of point,
        normal, dir, le, pdf per item and area (pdf at pdf_dir when given)."""
        uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
        pd = None if pdf_dir is None else np.ascontiguousarray(pdf_dir, np.float32).reshape(-1, 3)
        n = uv.shape[0]
        out = {k: np.zeros((n, 3), np.float32) for k in ("point", "normal", "dir", "le")}
        out["pdf"] = np.zeros(n, np.float32)
        area = C.c_float()
        if self.lib.ref_light_eval(self.h, light, n, _p(uv, C.c_float), _p(x, C.c_float),
                                   None if pd is None else _p(pd, C.c_float),
                                   *(_p(out[k], C.c_float) for k in ("point", "normal", "dir", "le", "pdf")),
                                   C.byref(area)) != 0:
            raise ValueError("bad light index")
        out["area"] = area.value
        return out

    def transform(self, obj: int, ops):
        """Wraps object `obj` in the reference's decorators, innermost first:
        ops = [(code, p0, p1, p2)] with code 0 Translate, 1 Rotate<X>,
        2 Rotate<Y>, 3 Rotate<Z>, 4 Scale, 5 FlipFace; rebuilds the BVH."""
        codes = np.array([o[0] for o in ops], np.int32)
        params = np.array([list(o[1:]) + [0.0] * (3 - len(o[1:])) for o in ops], np.float32).reshape(-1)
        if self.lib.ref_scene_transform(self.h, obj, len(ops), _p(codes, C.c_int32), _p(params, C.c_float)) != 0:
            raise ValueError("bad transform")

    def render(self, job, threads=0):
        mean = np.zeros((job.height, job.width, 3), np.float32)
        var = np.zeros_like(mean)
        self.lib.ref_render(self.h, C.byref(job), _p(mean, C.c_float), _p(var, C.c_float), threads)
        return mean, var

    def render_time(self, job, threads=0) -> float:
        return self.lib.ref_render_time(self.h, C.byref(job), threads)


def bsdf_eval(mat, wo, wi, nrm, front):
    lib = load()
    wo, wi, nrm = (np.ascontiguousarray(a, np.float32) for a in (wo, wi, nrm))
    front = np.ascontiguousarray(front, np.uint8)
    n = wo.shape[0]
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    lib.ref_bsdf_eval(C.byref(mat), n, _p(wo, C.c_float), _p(wi, C.c_float), _p(nrm, C.c_float),
                      _p(front, C.c_uint8), _p(f, C.c_float), _p(pdf, C.c_float))
    return f, pdf


def bsdf_sample(mat, wo, nrm, front, uc, u):
    lib = load()
    wo, nrm, uc, u = (np.ascontiguousarray(a, np.float32) for a in (wo, nrm, uc, u))
    front = np.ascontiguousarray(front, np.uint8)
    n = wo.shape[0]
    ok = np.zeros(n, np.uint8)
    wi = np.zeros((n, 3), np.float32)
    att = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    ty = np.zeros(n, np.uint32)
    lib.ref_bsdf_sample(C.byref(mat), n, _p(wo, C.c_float), _p(nrm, C.c_float), _p(front, C.c_uint8),
                        _p(uc, C.c_float), _p(u, C.c_float), _p(ok, C.c_uint8), _p(wi, C.c_float),
                        _p(att, C.c_float), _p(pdf, C.c_float), _p(ty, C.c_uint32))
    return ok, wi, att, pdf, ty


def sampler_eval(strategy, first_index, n, dims, seed=0):
    lib = load()
    out = np.zeros((n, dims), np.float32)
    lib.ref_sampler_eval(strategy, seed, first_index, n, dims, _p(out, C.c_float))
    return out


def image_texels(path, flip_y: bool, is_hdr: bool, uv: np.ndarray) -> np.ndarray:
    """ImageTexture(path, flip_y, is_hdr).getTexelColor at each (u, v)."""
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    out = np.zeros((uv.shape[0], 3), np.float32)
    rc = load().ref_image_texels(str(path).encode(), int(flip_y), int(is_hdr), uv.shape[0], _p(uv, C.c_float),
                                 _p(out, C.c_float))
    if rc != 0:
        raise RuntimeError(f"reference ImageTexture failed to load {path}")
    return out


def obj_load(path) -> dict:
    """loadOBJMesh(path) through the harness: the MeshData arrays."""
    lib = load()
    counts = (C.c_int64 * 4)()
    if lib.ref_obj_load(str(path).encode(), counts, None, None, None, None, None, None) != 0:
        raise RuntimeError(f"reference loadOBJMesh failed on {path}")
    nv, nn, nt, nf = list(counts)
    out = {"positions": np.zeros((nv, 3), np.float32), "normals": np.zeros((nn, 3), np.float32),
           "uvs": np.zeros((nt, 2), np.float32), "indices": np.zeros((nf, 3), np.int32),
           "normal_indices": np.zeros((nf, 3), np.int32), "uv_indices": np.zeros((nf, 3), np.int32)}
    lib.ref_obj_load(str(path).encode(), counts, _p(out["positions"], C.c_float), _p(out["normals"], C.c_float),
                     _p(out["uvs"], C.c_float), _p(out["indices"], C.c_int32), _p(out["normal_indices"], C.c_int32),
                     _p(out["uv_indices"], C.c_int32))
    return out


def texture_eval(kind: int, c1, c2, scale: float, fractal: int, uv: np.ndarray) -> np.ndarray:
    """CheckerTexture (kind 1) / NoiseTexture (kind 2).getTexelColor at each (u, v)."""
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    a, b = np.asarray(c1, np.float32), np.asarray(c2, np.float32)
    out = np.zeros((uv.shape[0], 3), np.float32)
    if load().ref_texture_eval(kind, _p(a, C.c_float), _p(b, C.c_float), scale, fractal, uv.shape[0],
                               _p(uv, C.c_float), _p(out, C.c_float)) != 0:
        raise RuntimeError("unknown texture kind")
    return out


def gaussian_blur(img: np.ndarray, kernel: int, sigma: float) -> np.ndarray:
    """FrameBuffer::gaussianBlur of an (H, W, 3) image through the harness."""
    a = np.ascontiguousarray(img, np.float32)
    out = np.zeros_like(a)
    load().ref_gaussian_blur(_p(a, C.c_float), a.shape[1], a.shape[0], kernel, sigma, _p(out, C.c_float))
    return out


def write_png(film: np.ndarray, gamma: float, path) -> None:
    """FrameBuffer::writeToFile of an (H, W, 3) film through the harness."""
    a = np.ascontiguousarray(film, np.float32)
    load().ref_write_png(_p(a, C.c_float), a.shape[1], a.shape[0], gamma, str(path).encode())
