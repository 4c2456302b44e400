/*
 * pathtracer_gb300.h -- C-ABI of the GB300 wavefront NEE(+MIS) path integrator.
 *
 * This is the drop-in boundary for the render loop of 747745124/PathTracer.
 * The reference exposes C++ virtual interfaces and one free function per
 * integrator; every entry point below names the reference interface it
 * replaces (file:line within the reference project).  All functions are
 * `extern "C"`, take plain pointers and sizes, never throw, and return an
 * int status: PT_OK (0) or a negative PT_ERR_* code.  The message of the last
 * failure on a context is read with pt_last_error().
 *
 * Threading: one pt_context per host thread, or external locking.  Device
 * work of a context runs on that context's own CUDA stream.
 */
#ifndef PATHTRACER_GB300_H
#define PATHTRACER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  PT_OK = 0,
  PT_ERR_INVALID = -1,     /* bad argument / malformed scene or job        */
  PT_ERR_CUDA = -2,        /* a CUDA call failed                           */
  PT_ERR_NOMEM = -3,       /* device or host allocation failed             */
  PT_ERR_NOT_FOUND = -4,   /* unknown scene / request id                   */
  PT_ERR_DEVICE = -5,      /* device-side error flag (iteration cap hit)   */
  PT_ERR_BUSY = -6,        /* admission refused: the server's queue is full */
  PT_ERR_CANCELLED = -7,   /* request was cancelled                        */
  PT_ERR_TOO_LARGE = -8    /* size beyond a fixed, documented maximum      */
};

/* ------------------------------------------------------------- materials
 * Mirrors the reference's Material family (include/material/material.hpp:15-77)
 * and its subclasses.  p[] holds the constructor arguments in order:
 *   LAMBERTIAN        Lambertian(albedo)                      material.hpp:79
 *                       p[0..2] albedo
 *   CONDUCTOR         Conductor(eta, k, alpha_x, alpha_y)     conductor.hpp:4
 *                       p[0..2] eta, p[3..5] k, p[6] alpha_x, p[7] alpha_y
 *   MF_DIELECTRIC     MFDielectric(eta, alpha_x, alpha_y)     dielectric.hpp:15
 *                       p[0] eta, p[1] alpha_x, p[2] alpha_y
 *   THIN_DIELECTRIC   ThinDielectric(eta, use_split_ray)      thinDielectric.hpp:10
 *                       p[0] eta, flags bit0 = use_split_ray
 *   PHONG             Phong(diffuse, specular, ambient, n)    material.hpp:303
 *                       p[0..2] diffuse, p[3..5] specular, p[6..8] ambient,
 *                       p[9] shininess
 *   DISNEY            DisneyPrincipledBSDF(13 params)         disneyPrincipledBSDF.hpp:34
 *                       p[0..2] baseColor, p[3] specular_transmission,
 *                       p[4] metallic, p[5] subsurface, p[6] specular,
 *                       p[7] roughness, p[8] specular_tint, p[9] anisotropic,
 *                       p[10] sheen, p[11] sheen_tint, p[12] clearcoat,
 *                       p[13] clearcoat_gloss, p[14] eta
 *   HAIR              HairMarschner(sigma_a, h, eta, beta_m, beta_n, alpha)
 *                                                             hairMarsch.hpp:7
 *                       p[0..2] sigma_a, p[3] h, p[4] eta, p[5] beta_m,
 *                       p[6] beta_n, p[7] alpha (radians).
 *                       flags bit1: sigma_a is derived from p[8] eumelanin and
 *                       p[9] pheomelanin concentrations (extension).
 *   DIFFUSE_EMITTER   DiffuseEmitter(color, intensity)        material.hpp:467
 *                       p[0..2] color, p[3] intensity
 */
enum {
  PT_MAT_LAMBERTIAN = 0,
  PT_MAT_CONDUCTOR = 1,
  PT_MAT_MF_DIELECTRIC = 2,
  PT_MAT_THIN_DIELECTRIC = 3,
  PT_MAT_PHONG = 4,
  PT_MAT_DISNEY = 5,
  PT_MAT_HAIR = 6,
  PT_MAT_DIFFUSE_EMITTER = 7,
  PT_MAT_COUNT = 8
};
#define PT_MAT_FLAG_SPLIT_RAY 1
#define PT_MAT_FLAG_MELANIN 2
/* ColorVariant (include/texture/texture.hpp:134-163): a Lambertian albedo or
 * a DiffuseEmitter colour given by a texture instead of p[0..2]: flags bits
 * 8..31 hold the texture's index in pt_scene_desc.textures + 1 (0: the
 * constant colour p[0..2]). */
#define PT_MAT_TEXTURE_SHIFT 8

/* Texture2D kinds (include/texture/texture.hpp:20-95, texture.cpp:95-193):
 * CONSTANT color1; CHECKER color1 where sin(u*scale)*sin(v*scale) < 0 else
 * color2; NOISE the fractal 2-D Perlin noise of pattern.hpp:72-114 at
 * (u*scale, v*scale) with `fractal` octaves, grey; IMAGE bilinear lookup of
 * width*height RGB texels stored as ImageTexture's texels[x][y]:
 * texels[(y*width + x)*3 + c]. */
enum { PT_TEX_CONSTANT = 0, PT_TEX_CHECKER = 1, PT_TEX_NOISE = 2, PT_TEX_IMAGE = 3 };
typedef struct pt_texture_desc {
  int32_t kind;
  float color1[3];
  float color2[3];
  float scale;
  int32_t fractal;
  const float *texels; /* IMAGE only */
  int32_t width, height;
} pt_texture_desc;

typedef struct pt_material_desc {
  int32_t type;
  int32_t flags;
  float p[30];
} pt_material_desc; /* 128 bytes */

/* ------------------------------------------------------------- geometry
 * A triangle mesh in world space: TriangleMesh(MeshData, material)
 * (include/primitives/triangleMesh.hpp:8, include/mesh_io/meshData.hpp:6).
 * normals / uvs and their index arrays are optional (NULL).  Decorators of
 * the reference (Translate/Rotate/Scale/FlipFace, utils/objectTransform.hpp)
 * are applied by the host C++ layer before upload. */
typedef struct pt_mesh_desc {
  const float *positions;       /* 3 * n_positions */
  int32_t n_positions;
  const float *normals;         /* 3 * n_normals, optional */
  int32_t n_normals;
  const float *uvs;             /* 2 * n_uvs, optional */
  int32_t n_uvs;
  const int32_t *indices;       /* 3 * n_triangles */
  const int32_t *normal_indices;/* 3 * n_triangles, optional */
  const int32_t *uv_indices;    /* 3 * n_triangles, optional */
  int32_t n_triangles;
  int32_t material;
} pt_mesh_desc;

/* AARectangle<axis>(k, d0_min, d0_max, d1_min, d1_max, material)
 * (include/base/primitive.hpp:205-269).  axis 0 = X (YZRectangle),
 * 1 = Y (XZRectangle), 2 = Z (XYRectangle). flip_face mirrors FlipFace. */
typedef struct pt_quad_desc {
  int32_t axis;
  float k, d0_min, d0_max, d1_min, d1_max;
  int32_t material;
  int32_t flip_face;
} pt_quad_desc;

/* Sphere(center, radius, material) (include/base/primitive.hpp:81-203). */
typedef struct pt_sphere_desc {
  float center[3];
  float radius;
  int32_t material;
  int32_t flip_face;
} pt_sphere_desc;

/* Entry of the scene's ObjectList in insertion order (objectList.hpp:176).
 * The order fixes the top-level BVH build (bvh.hpp:46-102) and light
 * discovery order (lightDiscovery.hpp:5-81). */
enum { PT_OBJ_MESH = 0, PT_OBJ_QUAD = 1, PT_OBJ_SPHERE = 2, PT_OBJ_BOX = 3, PT_OBJ_CURVE = 4 };

/* Curve(cps, width0, width1, material) (include/primitives/curve.hpp:13-157):
 * a cubic Bezier intersected as 8 cylinder segments, radius the mean of the
 * linearly interpolated width at the segment's ends; its hit carries the
 * curve tangent (HitRecord::hair_tangent), which HairMarschner uses as its
 * frame.  Not discovered as a light. */
typedef struct pt_curve_desc {
  float cps[4][3];
  float width0, width1;
  int32_t material;
} pt_curve_desc;

/* Box(min_xyz, max_xyz, material) (include/primitives/box.hpp:5-53): one
 * object of six rectangles, x1, x0, y1, y0, z1, z0 faces in that order,
 * intersected as its ObjectList (closest of the six); its faces are not
 * discovered as lights. */
typedef struct pt_box_desc {
  float min_xyz[3];
  float max_xyz[3];
  int32_t material;
} pt_box_desc;
typedef struct pt_object_desc {
  int32_t kind;
  int32_t index;
  /* Extension (motion blur): linear velocity in scene units per unit of
   * shutter time; the object sits at its described position + velocity * t
   * for a ray of time t in [0, camera.shutter].  Zero: static. */
  float velocity[3];
  /* HitRecord::is_inside of every hit on the object: PT_FACE_AS_HIT (the
   * front-face test of set_normal, then flip_face / a reversed winding),
   * PT_FACE_FRONT (always true) or PT_FACE_BACK (always false).  A reference
   * object under Translate, Rotate or Scale reports is_inside = true for
   * every hit: their intersect calls set_normal with the child's normal,
   * which already faces the ray (objectTransform.hpp:56-57, 168,
   * objectTransform.cpp:131, 172, 210); a FlipFace over such an object
   * reports false.  The C++ API's decorators set this field. */
  int32_t face;
} pt_object_desc;
enum { PT_FACE_AS_HIT = 0, PT_FACE_FRONT = 1, PT_FACE_BACK = 2 };

/* EnvironmentLight + HDRITexture (include/light/envLight.hpp:4,
 * include/texture/texture.hpp:97).  texels are RGB float, width*height*3,
 * stored as the reference's texels[x][y] with y = 0 the BOTTOM row:
 * texels[(y * width + x) * 3 + c]. */
typedef struct pt_env_desc {
  const float *texels;
  int32_t width;
  int32_t height;
  float intensity;
} pt_env_desc;

/* HomogeneousMedium(sigma_a, sigma_s, scale, Le, Le_scale, g)
 * (include/medium/homogeneous.hpp:31-68), filling the whole scene. */
typedef struct pt_medium_desc {
  float sigma_a[3];
  float sigma_s[3];
  float g;
} pt_medium_desc;

typedef struct pt_scene_desc {
  const pt_material_desc *materials;
  int32_t n_materials;
  const pt_mesh_desc *meshes;
  int32_t n_meshes;
  const pt_quad_desc *quads;
  int32_t n_quads;
  const pt_sphere_desc *spheres;
  int32_t n_spheres;
  const pt_object_desc *objects;
  int32_t n_objects;
  const pt_env_desc *env;       /* NULL: no environment light */
  const pt_medium_desc *medium; /* NULL: vacuum */
  float bg_color[3];            /* SceneInfo::bg_color, renderManager.hpp:41 */
  int32_t bvh_mode;             /* PT_BVH_REFERENCE (default) */
  /* Extension (motion blur): the longest shutter a job may use on this
   * scene; the BVH boxes of moving objects cover their motion over
   * [0, shutter_max].  Jobs with camera.shutter > shutter_max are rejected
   * when the scene has moving objects. */
  float shutter_max;
  /* Textures referenced by materials (PT_MAT_TEXTURE_SHIFT). */
  const pt_texture_desc *textures;
  int32_t n_textures;
  const pt_box_desc *boxes;     /* objects of kind PT_OBJ_BOX index these */
  int32_t n_boxes;
  const pt_curve_desc *curves;  /* objects of kind PT_OBJ_CURVE index these */
  int32_t n_curves;
} pt_scene_desc;

enum { PT_BVH_REFERENCE = 0 };

/* ------------------------------------------------------------------ jobs
 * PerspectiveCamera(fov, aspect, focalDist, aperture, up, front, position)
 * (src/base/camera.cpp:7-35).  Lens radius = focalDist / aperture * 0.5. */
typedef struct pt_camera_desc {
  float fov;        /* radians */
  float aspect;
  float focal_dist;
  float aperture;
  float up[3];
  float front[3];
  float position[3];
  float shutter;    /* motion-blur shutter length (extension); 0 = off.  A
                     * path's time is shutter * u, u from its own counter
                     * stream, and every ray of the path uses it. */
} pt_camera_desc;

/* Estimator.  REF_NEE restates include/integrator/maxdepth_nee.hpp:9-256
 * (light-sampled direct light only, BSDF-sampled emitter hits dropped, the
 * environment counted by both strategies).  NEE_MIS combines light and
 * BSDF sampling with the power heuristic of maxdepth_mis.hpp:10-15. */
enum { PT_EST_REF_NEE = 0, PT_EST_NEE_MIS = 1 };

/* Sampler for the per-bounce dimensions (sampler.hpp:5 RandomStrategy),
 * plus a jittered stratified sampler. */
enum {
  PT_SAMPLER_HALTON_NONE = 0,
  PT_SAMPLER_HALTON_PERMUTE = 1,
  PT_SAMPLER_HALTON_OWEN = 2,
  PT_SAMPLER_STRATIFIED = 3
};

/* Environment light sampling: the reference's uniform sphere
 * (texture.hpp:120-131) or a luminance alias table (extension). */
enum { PT_ENV_UNIFORM = 0, PT_ENV_ALIAS = 1 };

typedef struct pt_job_desc {
  int32_t scene;
  int32_t width, height;
  int32_t spp_x, spp_y;      /* stratified pixel grid, framebuffer.cpp:131 */
  int32_t spp_begin;         /* render samples [spp_begin, spp_end) of the grid */
  int32_t spp_end;           /* 0 = spp_x * spp_y */
  int32_t max_depth;         /* MAX_RAY_DEPTH, config.hpp:7 */
  int32_t rr_start;          /* Russian roulette from this depth; -1 = off */
  int32_t estimator;         /* PT_EST_* */
  int32_t sampler;           /* PT_SAMPLER_* */
  int32_t env_sampling;      /* PT_ENV_* */
  int32_t light_samples_x;   /* LIGHT_SAMPLE_X, config.hpp:5 (default 2) */
  int32_t light_samples_y;   /* LIGHT_SAMPLE_Y, config.hpp:6 (default 2) */
  uint32_t seed;             /* seeds every non-Halton draw */
  uint32_t sampler_seed;     /* HaltonSampler seed (PermuteDigits only) */
  pt_camera_desc camera;
  float gamma;               /* GAMMA, config.hpp:10 */
  /* Window of a larger frame (extension; converged references, tiles): the
   * job renders pixels [crop_x, crop_x + width) x [crop_y, crop_y + height)
   * of a full_width x full_height frame with the sample streams of the full
   * frame's pixels, so a window equals the same pixels of the full render.
   * full_width = full_height = 0: the job is the whole frame. */
  int32_t crop_x, crop_y;
  int32_t full_width, full_height;
} pt_job_desc;

typedef struct pt_stats {
  uint64_t paths;
  uint64_t segments;     /* path vertices shaded */
  uint64_t rays;         /* closest-hit rays traced */
  uint64_t shadow_rays;  /* any-hit rays traced */
  double ms;             /* device time of the render */
  uint64_t algorithmic_bytes; /* 192*segments + 88*shadow_rays + 24*paths */
} pt_stats;

/* -------------------------------------------------------------- context */
int pt_create(void **ctx, int device);
int pt_destroy(void *ctx);
/* Copies the last error message of ctx (or of the library if ctx is NULL)
 * into buf (NUL-terminated, at most n bytes). */
int pt_last_error(void *ctx, char *buf, size_t n);
int pt_version(void);

/* Flattens and uploads a scene (replaces the scene set-up part of
 * SceneInfo::render, include/render/renderManager.hpp:80-95: BVH build,
 * light discovery).  Host arrays are copied; the caller keeps ownership.
 * The traversal stack of the scene's kernels is sized by its BVH4 depth (3
 * entries per level + 4, in shared memory); a tree deeper than 15 levels is
 * refused with PT_ERR_TOO_LARGE. */
int pt_scene_upload(void *ctx, const pt_scene_desc *desc, int32_t *scene_id);
int pt_scene_release(void *ctx, int32_t scene_id);

/* Host-only build of a scene's BVH (no device, no context; no reference
 * counterpart): validates the description and builds the BVH4 exactly as
 * pt_scene_upload does, with `threads` workers for the mesh BVHs (0: all
 * hardware threads).  out5: BVH4 nodes, leaf items, depth, a 64-bit content
 * hash of nodes and items (same hash, same tree, whatever the thread count),
 * build time in microseconds.  Errors: pt_last_error(NULL, ...). */
int pt_bvh_build(const pt_scene_desc *desc, int32_t threads, int64_t *out5);

/* BVH builder of a context's later pt_scene_upload calls (the reference
 * builds one way only, on the host).  A BVH decides which boxes a ray visits,
 * not what it hits: every builder gives the same closest hits up to exact
 * ties in t.  PT_BVH_BUILD_HOST (default): the reference's own trees
 * (MeshBVHNode, meshBVH.cpp:6-55; BVHNode, bvh.hpp:46-102) on host threads.
 * PT_BVH_BUILD_DEVICE: meshes of >= 16384 triangles built on the GPU with the
 * reference's split rule, level by level -- the reference's tree whenever no
 * two centroids of a node tie along its split axis (ties: by triangle
 * index); the fastest upload of large meshes.  PT_BVH_BUILD_SAH: binned-SAH
 * trees instead of the reference's, fewer node visits per ray. */
#define PT_BVH_BUILD_HOST 0
#define PT_BVH_BUILD_DEVICE 1
/* Binned-SAH trees (meshes and the object level) on host threads: not the
 * reference's tree -- the same hits (up to exact ties in t), fewer node
 * visits where the reference's median / insertion-order splits are poor. */
#define PT_BVH_BUILD_SAH 2
/* pt_bvh_build with PT_BVH_BUILD_SAH trees (host only, no context). */
int pt_bvh_build_sah(const pt_scene_desc *desc, int32_t threads, int64_t *out5);
int pt_set_bvh_builder(void *ctx, int32_t builder);
/* pt_bvh_build with the context's device builder for large meshes: the
 * scene is validated and built (BVH4, items) but not kept.  Same out5. */
int pt_bvh_build_device(void *ctx, const pt_scene_desc *desc, int64_t *out5);

/* OBJ ingest: loadOBJMesh (src/mesh_io/meshLoader.cpp:7-58), which reads the
 * file with tinyobjloader.  "v", "vn", "vt" and "f" records; face vertices
 * "v", "v/vt", "v//vn", "v/vt/vn" with 1-based or negative indices; an
 * absent normal / uv index is -1 (a face without normals is shaded flat);
 * quads split along the shorter diagonal as tinyobjloader does, longer
 * polygons fanned from their first vertex; other records ignored.  Fills
 * *mesh (material = -1, to be set by the caller) with arrays owned by the
 * library until pt_obj_free.  No context; errors (missing file:
 * PT_ERR_NOT_FOUND, malformed record or out-of-range index:
 * PT_ERR_INVALID) through pt_last_error(NULL, ...). */
int pt_obj_load(const char *path, pt_mesh_desc *mesh);
int pt_obj_free(pt_mesh_desc *mesh);

/* Image file -> texels, the ImageTexture(filename, flip_y, isHDR)
 * constructor (src/texture/texture.cpp:3-93, decoding through stb_image):
 * *texels = width*height*3 floats laid out as the reference's texels[x][y],
 * y = 0 the image's bottom row (its top row with flip_y) -- the layout of
 * pt_env_desc and pt_texture_desc image texels.  Radiance RGBE (.hdr, flat or
 * RLE scanlines) and PNG (every colour type / bit depth, Adam7); LDR texels
 * are byte / 255, is_hdr linearises LDR files as stbi_loadf does.  Free with
 * pt_free_image.  No context; errors through pt_last_error(NULL, ...). */
int pt_load_image(const char *path, int32_t flip_y, int32_t is_hdr, float **texels, int32_t *width,
                  int32_t *height);
int pt_free_image(float *texels);
/* Counts of the flattened scene: [0] triangles, [1] quads, [2] spheres,
 * [3] BVH4 nodes, [4] lights, [5] device bytes. */
int pt_scene_info(void *ctx, int32_t scene_id, int64_t *out6);

/* Renders one job synchronously (replaces the pixel loop of
 * SceneInfo::render, renderManager.hpp:97-155, calling getRayColor,
 * maxdepth_nee.hpp:9).  film_rgb is a HOST buffer of width*height*3 floats
 * indexed [j][i][c] with j = 0 the bottom row (FrameBuffer::_pixel_color,
 * framebuffer.cpp:23); it receives the mean over samples
 * [spp_begin, spp_end).  stats may be NULL. */
int pt_render(void *ctx, const pt_job_desc *job, float *film_rgb,
              pt_stats *stats);
/* Same, into a DEVICE buffer of width*height*3 floats that receives the
 * SUM (not the mean) of the samples rendered, accumulated onto its contents.
 * Runs on the context's stream, returns after the work is enqueued unless
 * sync != 0. */
int pt_render_device(void *ctx, const pt_job_desc *job, float *d_film_sum,
                     int sync, pt_stats *stats);

/* pt_render_device for callers that cannot allocate device memory while
 * they render (a host whose own device memory pool forbids other allocators
 * on its GPUs, a real-time loop that must never block in the allocator).  No
 * counterpart in the reference, which has no device code.  It calls no
 * cudaMalloc/cudaFree: every work buffer of the render (path state,
 * ray/hit/shadow queues, offset and permutation tables, counters) lives in
 * one fixed 32 MiB device array inside this library; jobs are rendered in as
 * many waves as that array's path capacity needs.  Same arguments and result
 * as pt_render_device (sum of the samples added onto d_film_sum), always
 * synchronous; stats->ms is -1 (not timed).  Limit: spp_x * spp_y <= 16384
 * (PT_ERR_TOO_LARGE beyond).  The first call on a device does the set-up:
 * with CUDA's lazy module loading it loads the module that holds the array,
 * which allocates the 32 MiB on that device (kept until the process exits),
 * and it looks up the array's device address -- make one warm-up call on
 * each device before entering a region that must not allocate.  Every call
 * synchronises the context's stream and reads its error word and counts back
 * before it returns.  All calls share the one array, which keeps the last
 * call's contents: calls that overlap on the GPU (other host threads, other
 * contexts of the same device) race and must be serialised by the caller. */
int pt_render_device_noalloc(void *ctx, const pt_job_desc *job, float *d_film_sum, pt_stats *stats);

/* getRayColor (include/integrator/maxdepth_nee.hpp:9-256, the integrator
 * SceneInfo::render calls per sample) for n given primary rays of scene
 * job->scene: radiance (host, 3n floats) receives one path's estimate per
 * ray, with the job's integrator settings (estimator, max_depth, rr_start,
 * sampler, env_sampling, light samples, seed, camera shutter); its camera,
 * size, spp and window are not used.  rays: n * 6 floats (origin,
 * direction; the direction is normalised, as the render's camera rays are).
 * Path i draws Halton index first_index + i (HaltonSampler::startSample,
 * sampler.hpp:34-39; first_index >= 1) and that index's counter streams --
 * the same draws as sample k of frame pixel (i, j) of a render when
 * first_index + i = 1 + (i * height + j) * spp + k. */
int pt_ray_color(void *ctx, const pt_job_desc *job, const float *rays, int32_t n, uint32_t first_index,
                 float *radiance);

/* Per-stage device timing of the wave kernels (no counterpart in the
 * reference, which times only the whole render, renderManager.hpp:164-173).
 * pt_profile_begin clears and enables CUDA-event timing on the context's
 * stream; pt_profile_end synchronises and returns, per stage (0 camera,
 * 1 closest-hit trace, 2 material sort, 3 shade, 4 shadow trace, 5 film),
 * the summed milliseconds and the number of kernel launches. */
int pt_profile_begin(void *ctx);
int pt_profile_end(void *ctx, double *stage_ms /*[6]*/, int64_t *stage_launches /*[6]*/);

/* FrameBuffer::writeToFile pixel path (framebuffer.cpp:27-58): NaN -> 0,
 * pow(c, 1/gamma), clamp [0,1], *255 truncated to u8, rows flipped so that
 * row 0 of rgb8 is the top of the image.  Host buffers. */
int pt_tonemap(void *ctx, const float *film_rgb, int32_t width, int32_t height,
               float gamma, uint8_t *rgb8);

/* FrameBuffer::gaussianBlur (framebuffer.cpp:60-129): a k x k Gaussian of
 * standard deviation sigma (normalised weights, clamp to edge) over the film,
 * on the GPU; film_out may equal film_in.  Host buffers.  As the reference,
 * k even or < 3 or sigma < 0 leave the film unchanged (PT_OK); sigma = 0 is
 * also left unchanged (the reference divides by zero). */
int pt_gaussian_blur(void *ctx, const float *film_in, float *film_out, int32_t width,
                     int32_t height, int32_t kernel, float sigma);

/* FrameBuffer::writeToFile's file step (framebuffer.cpp:47-49, stb's PNG
 * writer): rgb8 as pt_tonemap gives it (row 0 = top) to an 8-bit RGB PNG
 * (uncompressed deflate blocks).  No context; errors through
 * pt_last_error(NULL, ...). */
int pt_write_png(const char *path, const uint8_t *rgb8, int32_t width, int32_t height);

/* ------------------------------------------------- batch test entry points
 * Sampler sequences (HaltonSampler::SampleDimension, sampler.hpp:54-73):
 * out[i * dims + d] = sample of dimension d at sample index first_index + i. */
int pt_sampler_eval(void *ctx, int32_t strategy, uint32_t seed,
                    uint32_t first_index, int32_t n, int32_t dims, float *out);

/* The sample values a job's paths draw, computed by the device code of the
 * render, for paths [first_path, first_path + n) in render order (pixel
 * q = g % (width * height), grid sample k = spp_begin + g / (width * height)):
 *   pixel_offsets (2n, may be NULL): the pixel-grid offset of the path's
 *     sample k -- FrameBuffer::setOffsets (framebuffer.cpp:131-145) with
 *     getOffsets(spp_x, spp_y) (utils/random.hpp:47-63): one jittered grid per
 *     frame, stratum (i, j) = (k / spp_y, k % spp_y);
 *   dim_values (n * dims): sampler dimensions 0..dims-1 of the job's sampler
 *     (HaltonSampler::SampleDimension, sampler.hpp:54-73, at the path's
 *     index; PT_SAMPLER_STRATIFIED: the jittered stratum of sample k among the
 *     pixel's spp_x * spp_y, permuted per pixel and dimension);
 *   light_offsets (n * bounces * LN * 2, LN = light_samples_x *
 *     light_samples_y): the light-point offsets of the vertex at each bounce,
 *     the per-vertex getOffsets(light_samples_x, light_samples_y) grid of
 *     maxdepth_nee.hpp:91, stratum (ls / light_samples_y, ls % light_samples_y). */
int pt_sample_eval(void *ctx, const pt_job_desc *job, int64_t first_path, int32_t n, int32_t dims,
                   int32_t bounces, float *pixel_offsets, float *dim_values, float *light_offsets);

/* Closest hit (BVHNode::intersect, bvh.hpp:27-41 and the primitives below
 * it).  rays: n * 6 floats (origin, direction), tmin/tmax per call.
 * Outputs: t (FLT_MAX on miss), prim (-1 on miss; triangles are numbered
 * mesh by mesh in upload order, then quads, then spheres), uv barycentrics. */
int pt_trace_closest(void *ctx, int32_t scene_id, const float *rays, int32_t n,
                     float tmin, float tmax, float *t, int32_t *prim,
                     float *uv);
/* Occlusion test with the shadow-ray intervals of maxdepth_nee.hpp:117-166:
 * occluded[i] = 1 if anything is hit in [tmin, tmax_i]. */
int pt_trace_any(void *ctx, int32_t scene_id, const float *rays,
                 const float *tmax, int32_t n, float tmin, uint8_t *occluded);

/* Hittable::intersect (base/primitive.hpp:30-79) through the scene's BVH:
 * the HitRecord of the closest hit in [tmin, tmax] of each ray (rays: n * 6
 * floats, origin and direction).  Outputs t (FLT_MAX on miss), prim (-1 on
 * miss), position (3n), normal (3n: HitRecord::normal, turned towards the
 * ray by set_normal, materialBase.hpp:47-52) and is_inside (n: the
 * front-face flag, toggled by FlipFace, objectTransform.hpp:5-38).  Objects
 * under Translate / Rotate / Scale are resident with the transform applied
 * to their geometry. */
int pt_intersect(void *ctx, int32_t scene_id, const float *rays, int32_t n, float tmin, float tmax,
                 float *t, int32_t *prim, float *position, float *normal, uint8_t *is_inside);

/* The Light interface (include/light/light.hpp:17-53) of light `light` of a
 * resident scene -- the records the render's NEE samples.  Lights are
 * numbered in discovery order (DiffuseEmitter rectangles and spheres in
 * object order, lightDiscovery.hpp:5-81), the environment last; their count
 * is pt_scene_info's [4].  For item i, with offsets (u, v) = uv[2i], uv[2i+1]
 * and shading point x[3i..3i+2]:
 *   point[3i]  get_sample(u, v)   QuadLight light.hpp:131-137 (v0 + u e1 + v e2),
 *              SphereLight :254-264 (the whole sphere), EnvironmentLight
 *              envLight.hpp:20-36 (uniform sphere direction * 1e5)
 *   normal[3i] get_normal_at(point)          light.hpp:139-145, 266-271; envLight.hpp:48-51
 *   dir[3i]    normalize(point - x)           (maxdepth_nee.hpp:114, 141-144)
 *   le[3i]     L_emit at the sample towards x, texCoords (u, v)  light.hpp:157-165,
 *              296-303; envLight.hpp:73-90 (the HDRI along dir)
 *   pdf[i]     pdf_value(x, dir)              light.hpp:164-205, 279-294; envLight.hpp:58-70
 *              -- or pdf_value(x, pdf_dir[3i..]) when pdf_dir (3n) is not NULL
 * and *area (may be NULL) = get_area() (INFINITY for the environment). */
int pt_light_sample(void *ctx, int32_t scene_id, int32_t light, int32_t n, const float *uv, const float *x,
                    const float *pdf_dir, float *point, float *normal, float *dir, float *le, float *pdf,
                    float *area);

/* BSDF evaluation (Material::f and Material::scatter_pdf(wo, wi, rec),
 * material.hpp:32-61).  Arrays of n items, 3 floats per vector. `front` is
 * HitRecord::is_inside (materialBase.hpp:47-52: true when the ray hit the
 * front face).  Outputs f (3n) and pdf (n). */
int pt_bsdf_eval(void *ctx, const pt_material_desc *mat, int32_t n,
                 const float *wo, const float *wi, const float *normal,
                 const uint8_t *front, float *f, float *pdf);
/* BSDF sampling (Material::scatter, material.hpp:18-27) with the sampler
 * values uc, u (2n).  Outputs: ok (scatter's return), wi (3n),
 * attenuation (3n), pdf_val (n), sampled_type (BxDFFlags bits). */
int pt_bsdf_sample(void *ctx, const pt_material_desc *mat, int32_t n,
                   const float *wo, const float *normal, const uint8_t *front,
                   const float *uc, const float *u, uint8_t *ok, float *wi,
                   float *attenuation, float *pdf_val, uint32_t *sampled_type);

/* ----------------------------------------------------- batched rendering
 * Many jobs (different scenes, sizes, spp) in one persistent launch per
 * bounce, replayed from a captured CUDA graph.  films[k] are host buffers
 * receiving each job's mean image.  Extension: no counterpart in the
 * reference, which renders one scene per process. */
int pt_render_batch(void *ctx, const pt_job_desc *jobs, int32_t n_jobs,
                    float **films, pt_stats *stats);

/* How pt_render_batch (and the server's passes) run the groups of jobs of one
 * scene: PT_BATCH_GRAPH (default) -- per-stage kernels of merged waves, each
 * group a branch of one CUDA graph; PT_BATCH_PERSISTENT -- ONE cooperative
 * launch per group that runs all its waves and bounces (camera, closest hit,
 * generic shading, shadow rays, films) with grid barriers between stages;
 * groups one after another.  Both give each job the same samples. */
enum { PT_BATCH_GRAPH = 0, PT_BATCH_PERSISTENT = 1 };
int pt_set_batch_mode(void *ctx, int32_t mode);

/* Launch autotuner (extension): renders the batch under candidate launch
 * configurations -- paths per wave of each job, material sorting on/off,
 * blocks per SM of the traversal and shade kernels -- keeps the fastest for
 * later renders on this context and reports it.  films of the tuning renders
 * are discarded. */
typedef struct pt_tuning {
  int32_t wave_paths;
  int32_t sort_by_material;
  int32_t trace_blocks;
  int32_t shade_blocks;
  double best_ms;
  double default_ms;
  int32_t candidates;
} pt_tuning;
int pt_autotune(void *ctx, const pt_job_desc *jobs, int32_t n_jobs, pt_tuning *out);

/* ------------------------------------------------------------- serving
 * A request loop over resident scenes with continuous batching.  Requests
 * are admitted while free HBM allows; each owns a device film that is
 * refined until its target RMSE estimate or spp cap.  Extension. */
typedef struct pt_request_desc {
  pt_job_desc job;
  float target_rmse;   /* stop when the estimated RMSE falls below this */
  int32_t spp_cap;     /* ... or when this many samples were taken */
  int32_t spp_per_pass;/* samples added per scheduling pass (at least) */
  int32_t paths_per_pass;/* > 0: per pass, enough samples for about this many
                          * paths (width * height * spp), never fewer than
                          * spp_per_pass -- small requests finish in fewer
                          * passes.  Passes alternate between the two half
                          * films whatever their size. */
} pt_request_desc;

int pt_server_create(void *ctx, int64_t hbm_budget_bytes, int32_t max_slots,
                     void **server);
int pt_server_destroy(void *server);
int pt_submit(void *server, const pt_request_desc *req, int64_t *request_id);
/* Runs one scheduling pass (admission + one batched step over all active
 * requests).  Returns the number of requests still active in *active. */
int pt_server_step(void *server, int32_t *active);
/* state: 0 queued, 1 running, 2 done, 3 cancelled, 4 failed.  When done,
 * film (host, may be NULL) receives the mean image; spp_done and the
 * latency (submit to completion, ms) are reported. */
int pt_poll(void *server, int64_t request_id, int32_t *state, float *film,
            int32_t *spp_done, double *latency_ms);
int pt_cancel(void *server, int64_t request_id);

/* Scheduling policy of a server.  PT_SERVE_FAIR (default): admission in
 * arrival order, and every pass renders the next chunk of every active
 * request.  PT_SERVE_SRPT (shortest remaining work first): the queued request
 * of least total work (width * height * spp cap) is admitted first, and a pass
 * takes the active requests in order of remaining paths until it holds
 * pass_paths (0: all; at least one request per pass) -- small requests finish
 * in few passes while large ones wait.  max_queue > 0: pt_submit refuses with
 * PT_ERR_BUSY while that many requests wait for admission (0: unbounded). */
enum { PT_SERVE_FAIR = 0, PT_SERVE_SRPT = 1 };
int pt_server_set_policy(void *server, int32_t policy, int64_t pass_paths, int32_t max_queue);
/* Queueing delay of a request (submit to admission; -1 while queued) and its
 * latency (submit to completion; -1 until done), milliseconds. */
int pt_request_times(void *server, int64_t request_id, double *queue_ms, double *latency_ms);

#ifdef __cplusplus
}
#endif
#endif /* PATHTRACER_GB300_H */
