// ref_harness.cpp -- test harness around the UNMODIFIED reference sources.
//
// ORACLE INFRASTRUCTURE ONLY.  Built by oracle/ref/build_ref.sh from the
// reference's own headers and src/*.cpp where they lie, into oracle/_ref/.
// It exists to pin the CPU restatement (oracle/pt_oracle.cpp) and to generate
// the golden fixtures under tests/golden/.  Nothing in the product links it.
//
// What the harness adds around the reference (nothing of the reference's
// arithmetic is changed):
//  * scenes are built from the C-ABI description (include/pathtracer_gb300.h)
//    with the reference's own classes (Lambertian, Conductor, AARectangle,
//    TriangleMesh, BVHNode, discover_emissive_objects_as_lights, ...);
//  * the pixel loop of SceneInfo::render (include/render/renderManager.hpp:
//    97-155) is re-stated with explicit sizes, one std::thread per row band,
//    the Halton sample index set to the single-thread value
//    1 + ((i*H + j)*S + k), and the primary direction normalised;
//  * gl::rand_num draws come from one seeded thread-local mt19937 per thread
//    (shim in oracle/ref/shim/ref_rng.hpp) so that runs are reproducible.
// Standard headers first, so that the access override below reaches only the
// reference's own classes.
#include <array>
#include <cfloat>
#include <chrono>
#include <complex>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <variant>
#include <vector>
#include <omp.h>
#include <unistd.h>

// The harness reads private state of the reference classes (sampler index,
// HDRI texels, MeshBVHNode::hitTriangle); access specifiers do not change
// the layout of these classes under GCC.
#define private public
#define protected public
#include "header.hpp"  // must come first: config.hpp <-> renderManager.hpp cycle
#include "base/lightDiscovery.hpp"
#include "material/conductor.hpp"
#include "material/dielectric.hpp"
#include "material/disneyPrincipledBSDF.hpp"
#include "material/hairMarsch.hpp"
#include "material/thinDielectric.hpp"
#include "primitives/meshBVH.hpp"
#include "primitives/triangleMesh.hpp"
#include "mesh_io/meshLoader.hpp"
#include "primitives/box.hpp"
#include "primitives/curve.hpp"
#include "utils/objectTransform.hpp"
#undef private
#undef protected

#include "../../include/pathtracer_gb300.h"

namespace {

using gl::vec2;
using gl::vec3;

vec3 V3(const float *p) { return vec3(p[0], p[1], p[2]); }

std::shared_ptr<Material> make_material(const pt_material_desc &m) {
  const float *p = m.p;
  switch (m.type) {
  case PT_MAT_LAMBERTIAN:
    return std::make_shared<Lambertian>(V3(p));
  case PT_MAT_CONDUCTOR:
    return std::make_shared<Conductor>(V3(p), V3(p + 3), p[6], p[7]);
  case PT_MAT_MF_DIELECTRIC:
    return std::make_shared<MFDielectric>(p[0], p[1], p[2]);
  case PT_MAT_THIN_DIELECTRIC:
    return std::make_shared<ThinDielectric>(p[0], (m.flags & PT_MAT_FLAG_SPLIT_RAY) != 0);
  case PT_MAT_PHONG:
    return std::make_shared<Phong>(V3(p), V3(p + 3), V3(p + 6), p[9]);
  case PT_MAT_DISNEY:
    return std::make_shared<DisneyPrincipledBSDF>(V3(p), p[3], p[4], p[5], p[6], p[7], p[8],
                                                  p[9], p[10], p[11], p[12], p[13], p[14]);
  case PT_MAT_HAIR:
    return std::make_shared<HairMarschner>(V3(p), p[3], p[4], p[5], p[6], p[7]);
  case PT_MAT_DIFFUSE_EMITTER:
    return std::make_shared<DiffuseEmitter>(V3(p), p[3]);
  default:
    return nullptr;
  }
}

// A tiny valid Radiance .hdr so that EnvironmentLight's constructor (which
// only takes a file path) succeeds; its texels are then replaced.
std::string tiny_hdr_path() {
  static std::string path;
  if (!path.empty()) return path;
  char buf[64];
  std::snprintf(buf, sizeof buf, "/tmp/ref_harness_%d.hdr", (int)getpid());
  FILE *f = std::fopen(buf, "wb");
  if (!f) return "";
  std::fputs("#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 2 +X 2\n", f);
  unsigned char px[4] = {128, 128, 128, 129};
  for (int i = 0; i < 4; ++i) std::fwrite(px, 1, 4, f);
  std::fclose(f);
  path = buf;
  return path;
}

struct RefScene {
  ObjectList objects;
  std::shared_ptr<BVHNode> bvh;
  LightList lights;
  std::shared_ptr<EnvironmentLight> env;
  vec3 bg;
  // identification of hits: material instance -> (object index)
  std::vector<const Material *> obj_material;
  std::vector<int> obj_kind, obj_index, obj_prim_base;
  // per object: a Box's six faces in its own order (to name the face hit)
  std::vector<std::vector<std::shared_ptr<Hittable>>> box_faces;
  std::vector<std::shared_ptr<TriangleMesh>> meshes;  // by object, may be null
};

int total_triangles_before(const pt_scene_desc *d, int mesh) {
  int s = 0;
  for (int m = 0; m < mesh; ++m) s += d->meshes[m].n_triangles;
  return s;
}

}  // namespace

extern "C" {

void *ref_scene_create(const pt_scene_desc *d) {
  auto *S = new RefScene();
  S->bg = V3(d->bg_color);
  int n_tris = total_triangles_before(d, d->n_meshes);
  const int n_boxes = d->boxes ? d->n_boxes : 0;
  const int n_quads_all = d->n_quads + 6 * n_boxes;  // a box's faces follow the rectangles
  for (int o = 0; o < d->n_objects; ++o) {
    S->box_faces.emplace_back();
    const pt_object_desc &od = d->objects[o];
    std::shared_ptr<Hittable> h;
    int mat_index = -1, prim_base = 0;
    std::shared_ptr<TriangleMesh> tm;
    if (od.kind == PT_OBJ_MESH) {
      const pt_mesh_desc &md = d->meshes[od.index];
      mat_index = md.material;
      MeshData data;
      for (int i = 0; i < md.n_positions; ++i)
        data.positions.emplace_back(md.positions[3 * i], md.positions[3 * i + 1], md.positions[3 * i + 2]);
      if (md.normals)
        for (int i = 0; i < md.n_normals; ++i)
          data.normals.emplace_back(md.normals[3 * i], md.normals[3 * i + 1], md.normals[3 * i + 2]);
      if (md.uvs)
        for (int i = 0; i < md.n_uvs; ++i) data.uvs.emplace_back(md.uvs[2 * i], md.uvs[2 * i + 1]);
      for (int t = 0; t < md.n_triangles; ++t) {
        data.indices.push_back({md.indices[3 * t], md.indices[3 * t + 1], md.indices[3 * t + 2]});
        if (md.normals) {
          const int32_t *ni = md.normal_indices ? md.normal_indices : md.indices;
          data.normalIndices.push_back({ni[3 * t], ni[3 * t + 1], ni[3 * t + 2]});
        }
        if (md.uvs) {
          const int32_t *ui = md.uv_indices ? md.uv_indices : md.indices;
          data.uvIndices.push_back({ui[3 * t], ui[3 * t + 1], ui[3 * t + 2]});
        }
      }
      auto mat = make_material(d->materials[mat_index]);
      tm = std::make_shared<TriangleMesh>(std::move(data), mat);
      h = tm;
      prim_base = total_triangles_before(d, od.index);
      S->obj_material.push_back(mat.get());
    } else if (od.kind == PT_OBJ_QUAD) {
      const pt_quad_desc &q = d->quads[od.index];
      auto mat = make_material(d->materials[q.material]);
      if (q.axis == 0)
        h = std::make_shared<AARectangle<Axis::X>>(q.k, q.d0_min, q.d0_max, q.d1_min, q.d1_max, mat);
      else if (q.axis == 1)
        h = std::make_shared<AARectangle<Axis::Y>>(q.k, q.d0_min, q.d0_max, q.d1_min, q.d1_max, mat);
      else
        h = std::make_shared<AARectangle<Axis::Z>>(q.k, q.d0_min, q.d0_max, q.d1_min, q.d1_max, mat);
      if (q.flip_face) h = std::make_shared<FlipFace>(h);
      prim_base = n_tris + od.index;
      S->obj_material.push_back(mat.get());
    } else if (od.kind == PT_OBJ_BOX) {
      const pt_box_desc &b = d->boxes[od.index];
      auto mat = make_material(d->materials[b.material]);
      auto box = std::make_shared<Box>(V3(b.min_xyz), V3(b.max_xyz), mat);
      S->box_faces.back() = box->_faces.getLists();
      h = box;
      prim_base = n_tris + d->n_quads + 6 * od.index;
      S->obj_material.push_back(mat.get());
    } else if (od.kind == PT_OBJ_CURVE) {
      const pt_curve_desc &c = d->curves[od.index];
      auto mat = make_material(d->materials[c.material]);
      std::array<gl::vec3, 4> cps = {V3(c.cps[0]), V3(c.cps[1]), V3(c.cps[2]), V3(c.cps[3])};
      h = std::make_shared<Curve>(cps, c.width0, c.width1, CurveType::Cylinder, mat);
      prim_base = n_tris + n_quads_all + d->n_spheres + od.index;
      S->obj_material.push_back(mat.get());
    } else {
      const pt_sphere_desc &s = d->spheres[od.index];
      auto mat = make_material(d->materials[s.material]);
      h = std::make_shared<Sphere>(V3(s.center), s.radius, mat);
      if (s.flip_face) h = std::make_shared<FlipFace>(h);
      prim_base = n_tris + n_quads_all + od.index;
      S->obj_material.push_back(mat.get());
    }
    S->objects.addObject(h);
    S->obj_kind.push_back(od.kind);
    S->obj_index.push_back(od.index);
    S->obj_prim_base.push_back(prim_base);
    S->meshes.push_back(tm);
  }
  std::srand(1);  // BVHNode draws its split axis from rand() (bvh.hpp:50)
  S->bvh = std::make_shared<BVHNode>(S->objects);
  S->lights = discover_emissive_objects_as_lights(S->objects);
  if (d->env) {
    S->env = std::make_shared<EnvironmentLight>(tiny_hdr_path(), d->env->intensity);
    auto tex = std::dynamic_pointer_cast<HDRITexture>(S->env->texture);
    int W = d->env->width, H = d->env->height;
    tex->_width = W;
    tex->_height = H;
    tex->texels.assign(W, std::vector<vec3>(H));
    for (int x = 0; x < W; ++x)
      for (int y = 0; y < H; ++y) tex->texels[x][y] = V3(d->env->texels + 3 * (y * W + x));
    S->lights.addLight(S->env);
  }
  return S;
}

void ref_scene_destroy(void *s) { delete static_cast<RefScene *>(s); }

int ref_scene_num_lights(void *s) { return (int)static_cast<RefScene *>(s)->lights.size(); }

// Closest hit through the reference BVH.  prim is recovered from the hit's
// material instance (one instance per object) and, for meshes, from the one
// triangle whose Moller-Trumbore t equals the returned t bit for bit.
void ref_trace_closest(void *s, const float *rays, int n, float tmin, float tmax, float *t_out,
                       int *prim_out, float *pos_out, float *nrm_out, uint8_t *front_out) {
  auto *S = static_cast<RefScene *>(s);
  for (int i = 0; i < n; ++i) {
    Ray ray(V3(rays + 6 * i), V3(rays + 6 * i + 3));
    HitRecord rec;
    bool hit = S->bvh->intersect(ray, rec, tmin, tmax);
    t_out[i] = hit ? rec.t : FLT_MAX;
    prim_out[i] = -1;
    for (int c = 0; c < 3; ++c) {
      pos_out[3 * i + c] = hit ? rec.position[c] : 0.f;
      nrm_out[3 * i + c] = hit ? rec.normal[c] : 0.f;
    }
    front_out[i] = hit ? (rec.is_inside ? 1 : 0) : 0;
    if (!hit) continue;
    for (size_t o = 0; o < S->obj_material.size(); ++o) {
      if (S->obj_material[o] != rec.material.get()) continue;
      if (S->obj_kind[o] == PT_OBJ_BOX) {
        // the face the Box's ObjectList kept: the last one accepted (box.hpp:40-43)
        float closest = tmax;
        for (size_t f = 0; f < S->box_faces[o].size(); ++f) {
          HitRecord tmp;
          if (S->box_faces[o][f]->intersect(ray, tmp, tmin, closest)) {
            closest = tmp.t;
            prim_out[i] = S->obj_prim_base[o] + (int)f;
          }
        }
      } else if (S->obj_kind[o] != PT_OBJ_MESH || !S->meshes[o]) {
        prim_out[i] = S->obj_prim_base[o];
      } else {
        const MeshBVHNode *root = S->meshes[o]->bvh.get();
        int ntri = (int)S->meshes[o]->mesh.indices.size();
        for (int tri = 0; tri < ntri; ++tri) {
          HitRecord tmp;
          if (root->hitTriangle(tri, ray, rec.t, rec.t, tmp) && tmp.t == rec.t) {
            prim_out[i] = S->obj_prim_base[o] + tri;  // the last match wins, as in the leaf loop
          }
        }
      }
      break;
    }
  }
}

// Wraps object `object` of a scene in the reference's decorators
// (utils/objectTransform.hpp:5-181, objectTransform.cpp:95-213), innermost
// first -- op 0 Translate(p0, p1, p2), 1 Rotate<X>(p0), 2 Rotate<Y>(p0),
// 3 Rotate<Z>(p0), 4 Scale(p0), 5 FlipFace; three params per op -- and
// rebuilds the scene's BVHNode.  Hits of a transformed mesh report the
// object's first primitive id (ref_trace_closest recovers triangle ids from
// untransformed rays only).
int ref_scene_transform(void *s, int object, int n_ops, const int *ops, const float *params) {
  auto *S = static_cast<RefScene *>(s);
  if (object < 0 || object >= (int)S->objects.objects.size()) return -1;
  std::shared_ptr<Hittable> h = S->objects.objects[object];
  for (int k = 0; k < n_ops; ++k) {
    const float *p = params + 3 * k;
    switch (ops[k]) {
    case 0: h = std::make_shared<Translate>(h, vec3(p[0], p[1], p[2])); break;
    case 1: h = std::make_shared<Rotate<Axis::X>>(h, p[0]); break;
    case 2: h = std::make_shared<Rotate<Axis::Y>>(h, p[0]); break;
    case 3: h = std::make_shared<Rotate<Axis::Z>>(h, p[0]); break;
    case 4: h = std::make_shared<Scale>(h, p[0]); break;
    case 5: h = std::make_shared<FlipFace>(h); break;
    default: return -1;
    }
  }
  S->objects.objects[object] = h;
  S->meshes[object] = nullptr;
  std::srand(1);
  S->bvh = std::make_shared<BVHNode>(S->objects);
  return 0;
}

// The Light methods of light `light` of a scene (LightList order: the
// discovered emitters, then the environment) at n items (u, v, x), as
// maxdepth_nee.hpp:104-189 calls them: point = get_sample(u, v), normal =
// get_normal_at(point), dir = normalize(point - x), L_emit (an area light
// with rec.normal = normal and texCoords (u, v) towards -dir; the
// environment with rec.normal = -dir along dir), pdf = pdf_value(x, dir);
// *area = get_area().  pdf_dir (may be NULL): pdf = pdf_value(x, pdf_dir[i]).
int ref_light_eval(void *s, int light, int n, const float *uv, const float *x, const float *pdf_dir, float *point,
                   float *normal, float *dir, float *le, float *pdf, float *area) {
  auto *S = static_cast<RefScene *>(s);
  if (light < 0 || light >= (int)S->lights.size()) return -1;
  std::shared_ptr<Light> L = S->lights.get(light);
  *area = L->get_area();
  for (int i = 0; i < n; ++i) {
    const vec3 p = L->get_sample(uv[2 * i], uv[2 * i + 1]);
    const vec3 nl = L->get_normal_at(p);
    const vec3 w = (p - V3(x + 3 * i)).normalize();
    HitRecord rec;
    rec.position = p;
    vec3 e;
    if (L->type == LightType::ENVIRONMENT_LIGHT) {
      rec.normal = -w;
      e = L->L_emit(rec, w);
    } else {
      rec.normal = nl;
      rec.texCoords = vec2(uv[2 * i], uv[2 * i + 1]);
      e = L->L_emit(rec, -w);
    }
    for (int c = 0; c < 3; ++c) {
      point[3 * i + c] = p[c];
      normal[3 * i + c] = nl[c];
      dir[3 * i + c] = w[c];
      le[3 * i + c] = e[c];
    }
    pdf[i] = L->pdf_value(V3(x + 3 * i), pdf_dir ? V3(pdf_dir + 3 * i) : w);
  }
  return 0;
}

// HitRecord for BSDF calls: the reference materials read normal, position,
// is_inside and texCoords.
static HitRecord make_rec(const float *n, uint8_t front) {
  HitRecord rec;
  rec.normal = V3(n);
  rec.position = vec3(0.f);
  rec.is_inside = front != 0;
  rec.texCoords = vec2(0.5f, 0.5f);
  return rec;
}

void ref_bsdf_eval(const pt_material_desc *md, int n, const float *wo, const float *wi,
                   const float *nrm, const uint8_t *front, float *f, float *pdf) {
  auto mat = make_material(*md);
  for (int i = 0; i < n; ++i) {
    HitRecord rec = make_rec(nrm + 3 * i, front[i]);
    vec3 fv = mat->f(V3(wo + 3 * i), V3(wi + 3 * i), rec, MODE);
    for (int c = 0; c < 3; ++c) f[3 * i + c] = fv[c];
    pdf[i] = mat->scatter_pdf(V3(wo + 3 * i), V3(wi + 3 * i), rec, MODE);
  }
}

void ref_bsdf_sample(const pt_material_desc *md, int n, const float *wo, const float *nrm,
                     const uint8_t *front, const float *uc, const float *u, uint8_t *ok,
                     float *wi, float *att, float *pdf_val, uint32_t *type) {
  auto mat = make_material(*md);
  for (int i = 0; i < n; ++i) {
    HitRecord rec = make_rec(nrm + 3 * i, front[i]);
    ScatterRecord srec;
    Ray in(vec3(0.f), -V3(wo + 3 * i));
    bool r = mat->scatter(in, rec, srec, uc[i], vec2(u[2 * i], u[2 * i + 1]), MODE);
    ok[i] = r ? 1 : 0;
    vec3 d = srec.sampled_ray.getDirection();
    for (int c = 0; c < 3; ++c) {
      wi[3 * i + c] = r ? d[c] : 0.f;
      att[3 * i + c] = r ? srec.attenuation[c] : 0.f;
    }
    pdf_val[i] = r ? srec.pdf_val : 0.f;
    type[i] = r ? srec.sampled_type : 0u;
  }
}

// HaltonSampler sequences (sampler.hpp:54-73) evaluated through the class.
void ref_sampler_eval(int strategy, uint32_t seed, uint32_t first_index, int n, int dims,
                      float *out) {
  RandomStrategy st = strategy == PT_SAMPLER_HALTON_NONE      ? RandomStrategy::None
                      : strategy == PT_SAMPLER_HALTON_PERMUTE ? RandomStrategy::PermuteDigits
                                                              : RandomStrategy::Owen;
  HaltonSampler hs(seed, st);
  for (int i = 0; i < n; ++i) {
    hs.sampleIndex_ = first_index + (uint32_t)i - 1u;
    hs.startSample();
    for (int d = 0; d < dims; ++d) out[(size_t)i * dims + d] = hs.get1D();
  }
}

void ref_rng_seed(uint64_t seed);  // oracle/ref/shim/ref_rng.cpp

// Stratified pixel-offset grid of FrameBuffer::setOffsets (framebuffer.cpp:
// 131-145) drawn after seeding the thread's generator.
void ref_offsets(int spp_x, int spp_y, uint64_t seed, float *out) {
  ref_rng_seed(seed);
  FrameBuffer fb(1, 1, spp_x, spp_y);
  auto off = fb.getOffsets();
  for (size_t k = 0; k < off.size(); ++k) {
    out[2 * k] = off[k][0];
    out[2 * k + 1] = off[k][1];
  }
}

// Render with the reference integrator getRayColor (maxdepth_nee.hpp:9).
// mean/var: width*height*3, [j][i][c]; var is the per-sample variance.
int ref_render(void *s, const pt_job_desc *job, float *mean, float *var, int threads) {
  auto *S = static_cast<RefScene *>(s);
  const pt_camera_desc &c = job->camera;
  PerspectiveCamera cam(c.fov, c.aspect, c.focal_dist, c.aperture, V3(c.up), V3(c.front),
                        V3(c.position));
  const int W = job->width, H = job->height;
  const int S_ = job->spp_x * job->spp_y;
  std::vector<vec2> offsets;
  {
    ref_rng_seed(job->seed);
    FrameBuffer fb(1, 1, job->spp_x, job->spp_y);
    offsets = fb.getOffsets();
  }
  if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
  std::vector<std::thread> pool;
  for (int th = 0; th < threads; ++th) {
    pool.emplace_back([&, th]() {
      for (int i = th; i < W; i += threads) {
        ref_rng_seed(((uint64_t)job->seed << 32) ^ (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull);
        for (int j = 0; j < H; ++j) {
          double sum[3] = {0, 0, 0}, sq[3] = {0, 0, 0};
          for (int k = 0; k < S_; ++k) {
            halton_sampler.sampleIndex_ = (uint32_t)((i * H + j) * S_ + k);
            halton_sampler.startSample();
            vec2 uv = (vec2((float)i, (float)j) + offsets[k]) / vec2((float)W, (float)H);
            Ray ray = cam.generateRay(uv.u(), uv.v());
            ray.direction = ray.direction.normalize();
            vec3 col = getRayColor(ray, S->objects, S->bg, S->lights, (uint)job->max_depth, S->bvh);
            for (int ch = 0; ch < 3; ++ch) {
              sum[ch] += col[ch];
              sq[ch] += (double)col[ch] * col[ch];
            }
          }
          for (int ch = 0; ch < 3; ++ch) {
            double m = sum[ch] / S_;
            mean[(j * W + i) * 3 + ch] = (float)m;
            var[(j * W + i) * 3 + ch] = (float)(S_ > 1 ? (sq[ch] - S_ * m * m) / (S_ - 1) : 0.0);
          }
        }
      }
    });
  }
  for (auto &t : pool) t.join();
  return 0;
}

// Single-thread timing loop in the reference's own order (i, j, k) with the
// reference's global sampler counter; returns seconds.
double ref_render_time(void *s, const pt_job_desc *job, int threads) {
  std::vector<float> m((size_t)job->width * job->height * 3), v(m.size());
  auto t0 = std::chrono::steady_clock::now();
  ref_render(s, job, m.data(), v.data(), threads);
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// ImageTexture(filename, flip_y, isHDR) (texture.cpp:3-93) sampled by its
// own getTexelColor at n points (u, v); returns -1 when the constructor
// throws (file missing or undecodable).
int ref_image_texels(const char *path, int flip_y, int is_hdr, int n, const float *uv, float *rgb) {
  try {
    ImageTexture tex(path, flip_y != 0, is_hdr != 0);
    for (int k = 0; k < n; ++k) {
      gl::vec3 c = tex.getTexelColor(uv[2 * k], uv[2 * k + 1]);
      rgb[3 * k] = c[0];
      rgb[3 * k + 1] = c[1];
      rgb[3 * k + 2] = c[2];
    }
    return 0;
  } catch (...) {
    return -1;
  }
}

// CheckerTexture(c1, c2, scale) (kind 1) or NoiseTexture(scale, fractal)
// (kind 2) sampled by its own getTexelColor (texture.cpp:151-193) at n
// points (u, v).
int ref_texture_eval(int kind, const float *c1, const float *c2, float scale, int fractal, int n, const float *uv,
                     float *rgb) {
  std::shared_ptr<Texture2D> tex;
  if (kind == 1)
    tex = std::make_shared<CheckerTexture>(gl::vec3(c1[0], c1[1], c1[2]), gl::vec3(c2[0], c2[1], c2[2]), scale);
  else if (kind == 2)
    tex = std::make_shared<NoiseTexture>(scale, fractal);
  else
    return -1;
  for (int k = 0; k < n; ++k) {
    gl::vec3 c = tex->getTexelColor(uv[2 * k], uv[2 * k + 1]);
    rgb[3 * k] = c[0];
    rgb[3 * k + 1] = c[1];
    rgb[3 * k + 2] = c[2];
  }
  return 0;
}

// FrameBuffer::gaussianBlur (framebuffer.cpp:60-129) of an H x W RGB image
// given row by row ([row][column][channel], the framebuffer's [u][v]).
void ref_gaussian_blur(const float *in, int W, int H, int kernel, float sigma, float *out) {
  FrameBuffer fb((uint)W, (uint)H, 1, 1);
  for (int i = 0; i < H; ++i)
    for (int j = 0; j < W; ++j) {
      const float *p = in + 3 * ((size_t)i * W + j);
      fb.setPixelColor((uint)i, (uint)j, gl::vec3(p[0], p[1], p[2]));
    }
  fb.gaussianBlur(kernel, sigma);
  for (int i = 0; i < H; ++i)
    for (int j = 0; j < W; ++j) {
      gl::vec3 c = fb.getPixelColor((uint)i, (uint)j);
      float *q = out + 3 * ((size_t)i * W + j);
      q[0] = c[0];
      q[1] = c[1];
      q[2] = c[2];
    }
}

// FrameBuffer::writeToFile (framebuffer.cpp:27-58) of an H x W RGB film
// given row by row: NaN -> 0, pow(1 / gamma), clamp, 8-bit truncation, PNG
// flipped vertically on write.  Returns 0 on success.
int ref_write_png(const float *in, int W, int H, float gamma, const char *path) {
  FrameBuffer fb((uint)W, (uint)H, 1, 1);
  for (int i = 0; i < H; ++i)
    for (int j = 0; j < W; ++j) {
      const float *p = in + 3 * ((size_t)i * W + j);
      fb.setPixelColor((uint)i, (uint)j, gl::vec3(p[0], p[1], p[2]));
    }
  fb.writeToFile(path, gamma);
  return 0;
}

// loadOBJMesh (meshLoader.cpp:7-58): counts[0..3] = positions, normals,
// uvs, faces; with non-null arrays also the data (faces: 3 indices each,
// normal / uv indices -1 where absent).  Returns -1 when the load throws.
int ref_obj_load(const char *path, int64_t *counts, float *pos, float *nrm, float *uv, int32_t *idx,
                 int32_t *nidx, int32_t *uvidx) {
  try {
    auto mesh = loadOBJMesh(path, nullptr);
    const MeshData &m = mesh->getMeshData();
    counts[0] = (int64_t)m.positions.size();
    counts[1] = (int64_t)m.normals.size();
    counts[2] = (int64_t)m.uvs.size();
    counts[3] = (int64_t)m.indices.size();
    if (!pos) return 0;
    for (size_t i = 0; i < m.positions.size(); ++i)
      for (int a = 0; a < 3; ++a) pos[3 * i + a] = m.positions[i][a];
    for (size_t i = 0; i < m.normals.size(); ++i)
      for (int a = 0; a < 3; ++a) nrm[3 * i + a] = m.normals[i][a];
    for (size_t i = 0; i < m.uvs.size(); ++i)
      for (int a = 0; a < 2; ++a) uv[2 * i + a] = m.uvs[i][a];
    for (size_t f = 0; f < m.indices.size(); ++f)
      for (int k = 0; k < 3; ++k) {
        idx[3 * f + k] = m.indices[f][k];
        nidx[3 * f + k] = f < m.normalIndices.size() ? m.normalIndices[f][k] : -1;
        uvidx[3 * f + k] = f < m.uvIndices.size() ? m.uvIndices[f][k] : -1;
      }
    return 0;
  } catch (...) {
    return -1;
  }
}

}  // extern "C"
