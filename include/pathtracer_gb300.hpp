// pathtracer_gb300.hpp -- C++ scene API over the C-ABI (header only).
//
// Mirrors the scene-building surface of 747745124/PathTracer so that a scene
// function written against the reference compiles against this header with
// `using namespace ptgb;`: materials (material.hpp:79-506, conductor.hpp,
// dielectric.hpp, thinDielectric.hpp, disneyPrincipledBSDF.hpp,
// hairMarsch.hpp), primitives (primitive.hpp:81-273, triangleMesh.hpp,
// mesh_io/meshData.hpp), decorators (utils/objectTransform.hpp), lights
// (envLight.hpp), the camera (base/camera.hpp) and SceneInfo
// (render/renderManager.hpp:35-176).  SceneInfo::render flattens the object
// list and renders it on the GPU through include/pathtracer_gb300.h instead
// of looping over pixels with getRayColor.
//
// Transforms are baked into the uploaded geometry: Translate/Scale keep
// rectangles axis aligned; a rotated rectangle becomes a two-triangle mesh.
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "pathtracer_gb300.h"

namespace ptgb {

struct vec3 {
  float v[3] = {0, 0, 0};
  vec3() = default;
  explicit vec3(float s) : v{s, s, s} {}
  vec3(float a, float b, float c) : v{a, b, c} {}
  float x() const { return v[0]; }
  float y() const { return v[1]; }
  float z() const { return v[2]; }
  float operator[](int i) const { return v[i]; }
  float &operator[](int i) { return v[i]; }
};
inline vec3 operator+(vec3 a, vec3 b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
inline vec3 operator*(vec3 a, float s) { return {a[0] * s, a[1] * s, a[2] * s}; }
struct vec2 {
  float v[2] = {0, 0};
  vec2() = default;
  vec2(float a, float b) : v{a, b} {}
};
inline float to_radian(float deg) { return deg * 3.14159265358979323846f / 180.f; }

enum class TransportMode { Radiance, Importance };
enum class Axis { X = 0, Y = 1, Z = 2 };

namespace detail {
inline void check(int rc, void *ctx) {
  if (rc != PT_OK) {
    char buf[512] = {0};
    pt_last_error(ctx, buf, sizeof buf);
    throw std::runtime_error(std::string("pathtracer_gb300: ") + buf);
  }
}
// The device context of the API's calls made outside SceneInfo::render
// (Material::f / scatter / scatter_pdf, HaltonSampler): one per host thread,
// on device 0, created at first use and destroyed with the thread.
inline void *thread_context() {
  struct Holder {
    void *ctx = nullptr;
    ~Holder() {
      if (ctx) pt_destroy(ctx);
    }
  };
  thread_local Holder h;
  if (!h.ctx) check(pt_create(&h.ctx, 0), nullptr);
  return h.ctx;
}
}  // namespace detail

// ------------------------------------------------------------- records
// Ray (base/ray.hpp), HitRecord / ScatterRecord (material/materialBase.hpp:
// 11-53) with the fields the materials and lights read, BxDFFlags
// (material/materialFlags.hpp:3-17).
struct Ray {
  Ray() = default;
  Ray(vec3 origin, vec3 direction) : o(origin), d(direction) {}
  vec3 getOrigin() const { return o; }
  vec3 getDirection() const { return d; }
  vec3 o, d;
};
enum BxDFFlags : uint32_t {
  Reflection = 1u << 0,
  Transmission = 1u << 1,
  Diffuse = 1u << 2,
  Glossy = 1u << 3,
  Specular = 1u << 4,
  DiffuseReflection = Diffuse | Reflection,
  DiffuseTransmission = Diffuse | Transmission,
  GlossyReflection = Glossy | Reflection,
  GlossyTransmission = Glossy | Transmission,
  SpecularReflection = Specular | Reflection,
  SpecularTransmission = Specular | Transmission,
  All = ~0u
};
struct HitRecord {
  float t = 3.402823466e+38f;
  vec3 normal;       // turned towards the incoming ray (set_normal)
  vec3 position;
  vec2 texCoords;
  bool is_inside = false;  // the front-face flag (materialBase.hpp:47-52)
};
struct ScatterRecord {
  Ray sampled_ray;
  uint32_t sampled_type = All;
  float pdf_val = 0.f;
  vec3 attenuation;
  bool is_specular() const { return (sampled_type & Specular) != 0; }
  bool is_specular_reflection() const { return (sampled_type & SpecularReflection) == SpecularReflection; }
  bool is_specular_transmission() const { return (sampled_type & SpecularTransmission) == SpecularTransmission; }
};

// ------------------------------------------------------------- materials
// ------------------------------------------------------------ textures
// Texture2D and its kinds (texture/texture.hpp:20-95); an ImageTexture takes
// its texels in memory ([y][x] RGB, as ImageTexture's texels[x][y]).
class Texture2D {
 public:
  virtual ~Texture2D() = default;
  virtual pt_texture_desc desc() const = 0;
};
class ConstantTexture : public Texture2D {
 public:
  explicit ConstantTexture(vec3 c) : c(c) {}
  pt_texture_desc desc() const override {
    pt_texture_desc d{};
    d.kind = PT_TEX_CONSTANT;
    for (int k = 0; k < 3; ++k) d.color1[k] = c[k];
    return d;
  }
  vec3 c;
};
class CheckerTexture : public Texture2D {
 public:
  explicit CheckerTexture(float scale = 10.f) : c1(0.f), c2(1.f), scale(scale) {}
  CheckerTexture(vec3 color1, vec3 color2, float scale = 10.f) : c1(color1), c2(color2), scale(scale) {}
  pt_texture_desc desc() const override {
    pt_texture_desc d{};
    d.kind = PT_TEX_CHECKER;
    for (int k = 0; k < 3; ++k) {
      d.color1[k] = c1[k];
      d.color2[k] = c2[k];
    }
    d.scale = scale;
    return d;
  }
  vec3 c1, c2;
  float scale;
};
class NoiseTexture : public Texture2D {
 public:
  NoiseTexture(float scale, int fractal = 1) : scale(scale), fractal(fractal) {}
  pt_texture_desc desc() const override {
    pt_texture_desc d{};
    d.kind = PT_TEX_NOISE;
    d.scale = scale;
    d.fractal = fractal;
    return d;
  }
  float scale;
  int fractal;
};
namespace detail {
// ImageTexture(filename, flip_y, isHDR)'s texels (texture.cpp:3-93) through
// pt_load_image; throws std::runtime_error like the reference.
inline std::vector<float> load_texels(const std::string &path, bool flip_y, bool is_hdr, int &w, int &h) {
  float *p = nullptr;
  int32_t W = 0, H = 0;
  if (pt_load_image(path.c_str(), flip_y, is_hdr, &p, &W, &H) != PT_OK) {
    char buf[512] = {0};
    pt_last_error(nullptr, buf, sizeof buf);
    throw std::runtime_error(buf);
  }
  std::vector<float> v(p, p + (size_t)W * H * 3);
  pt_free_image(p);
  w = W;
  h = H;
  return v;
}
}  // namespace detail

class ImageTexture : public Texture2D {
 public:
  ImageTexture(std::vector<float> texels, int width, int height)
      : texels(std::move(texels)), width(width), height(height) {}
  // texture.hpp:55: a PNG or Radiance HDR file
  explicit ImageTexture(const std::string &filename, bool flip_y = false, bool isHDR = false)
      : texels(detail::load_texels(filename, flip_y, isHDR, width, height)) {}
  pt_texture_desc desc() const override {
    pt_texture_desc d{};
    d.kind = PT_TEX_IMAGE;
    d.texels = texels.data();
    d.width = width;
    d.height = height;
    return d;
  }
  std::vector<float> texels;
  int width, height;
};

class Material {
 public:
  virtual ~Material() = default;
  virtual pt_material_desc desc() const = 0;
  virtual bool is_emitter() const { return false; }
  // ColorVariant: the texture of the albedo / emission colour, if any
  virtual std::shared_ptr<Texture2D> texture() const { return nullptr; }

  // Material::f (material.hpp:32-38): the BSDF for outgoing wo and incident
  // wi at rec (its normal and is_inside), evaluated by the device code the
  // render runs (pt_bsdf_eval).  The device implements the reference's
  // configured transport mode, TransportMode::Importance (config.hpp:23);
  // Radiance and textured colours are rejected (std::invalid_argument).
  vec3 f(const vec3 &wo, const vec3 &wi, const HitRecord &rec,
         TransportMode mode = TransportMode::Importance) const {
    float fv[3], pdf;
    eval(wo, wi, rec, mode, fv, pdf);
    return vec3(fv[0], fv[1], fv[2]);
  }
  // Material::scatter_pdf(wo, wi, rec) (material.hpp:50-61).
  float scatter_pdf(const vec3 &wo, const vec3 &wi, const HitRecord &rec,
                    TransportMode mode = TransportMode::Importance) const {
    float fv[3], pdf;
    eval(wo, wi, rec, mode, fv, pdf);
    return pdf;
  }
  // Material::scatter (material.hpp:18-27): samples the incident direction
  // for ray_in at rec with the sampler values uc, u (pt_bsdf_sample); srec
  // gets the sampled ray (from rec.position), attenuation, pdf_val and
  // sampled_type.  False: no scattering (an emitter, or an invalid sample).
  bool scatter(const Ray &ray_in, HitRecord &rec, ScatterRecord &srec, float uc, const vec2 &u,
               TransportMode mode = TransportMode::Importance) const {
    const pt_material_desc d = checked_desc(mode);
    const vec3 dd = ray_in.getDirection();
    const float wo[3] = {-dd[0], -dd[1], -dd[2]};
    const float nrm[3] = {rec.normal[0], rec.normal[1], rec.normal[2]};
    const uint8_t front = rec.is_inside ? 1 : 0;
    const float uu[2] = {u.v[0], u.v[1]};
    uint8_t ok = 0;
    float wi[3], att[3], pdf = 0.f;
    uint32_t type = 0;
    void *ctx = detail::thread_context();
    detail::check(pt_bsdf_sample(ctx, &d, 1, wo, nrm, &front, &uc, uu, &ok, wi, att, &pdf, &type), ctx);
    if (!ok) return false;
    srec.sampled_ray = Ray(rec.position, vec3(wi[0], wi[1], wi[2]));
    srec.attenuation = vec3(att[0], att[1], att[2]);
    srec.pdf_val = pdf;
    srec.sampled_type = type;
    return true;
  }
  // Material::emit (material.hpp:483-488 for DiffuseEmitter): its colour times
  // intensity where the ray meets the normal's side, else black; zero for
  // every other material.
  vec3 emit(const Ray &ray_in, const HitRecord &rec) const {
    if (!is_emitter()) return vec3(0.f);
    if (texture()) throw std::invalid_argument("emit(): textured emitters are evaluated by the render only");
    const pt_material_desc d = desc();
    const vec3 dd = ray_in.getDirection();
    const float c = -(rec.normal[0] * dd[0] + rec.normal[1] * dd[1] + rec.normal[2] * dd[2]);
    return c > 0.f ? vec3(d.p[0] * d.p[3], d.p[1] * d.p[3], d.p[2] * d.p[3]) : vec3(0.f);
  }

 private:
  pt_material_desc checked_desc(TransportMode mode) const {
    if (mode != TransportMode::Importance)
      throw std::invalid_argument("the device BSDFs implement TransportMode::Importance (config.hpp:23)");
    if (texture()) throw std::invalid_argument("textured colours are evaluated by the render only");
    return desc();
  }
  void eval(const vec3 &wo, const vec3 &wi, const HitRecord &rec, TransportMode mode, float *fv, float &pdf) const {
    const pt_material_desc d = checked_desc(mode);
    const float o[3] = {wo[0], wo[1], wo[2]}, w[3] = {wi[0], wi[1], wi[2]};
    const float nrm[3] = {rec.normal[0], rec.normal[1], rec.normal[2]};
    const uint8_t front = rec.is_inside ? 1 : 0;
    void *ctx = detail::thread_context();
    detail::check(pt_bsdf_eval(ctx, &d, 1, o, w, nrm, &front, fv, &pdf), ctx);
  }
};
namespace detail {
inline pt_material_desc make(int32_t type, std::initializer_list<float> p, int32_t flags = 0) {
  pt_material_desc d{};
  d.type = type;
  d.flags = flags;
  int i = 0;
  for (float x : p) d.p[i++] = x;
  return d;
}
}  // namespace detail

class Lambertian : public Material {
 public:
  explicit Lambertian(vec3 albedo) : a(albedo) {}
  explicit Lambertian(std::shared_ptr<Texture2D> t) : a(0.f), tex(std::move(t)) {}
  pt_material_desc desc() const override { return detail::make(PT_MAT_LAMBERTIAN, {a[0], a[1], a[2]}); }
  std::shared_ptr<Texture2D> texture() const override { return tex; }
  vec3 a;
  std::shared_ptr<Texture2D> tex;
};
class Conductor : public Material {
 public:
  Conductor(vec3 eta, vec3 k, float ax, float ay) : eta(eta), k(k), ax(ax), ay(ay) {}
  pt_material_desc desc() const override {
    return detail::make(PT_MAT_CONDUCTOR, {eta[0], eta[1], eta[2], k[0], k[1], k[2], ax, ay});
  }
  vec3 eta, k;
  float ax, ay;
};
class MFDielectric : public Material {
 public:
  MFDielectric(float eta, float ax, float ay) : eta(eta), ax(ax), ay(ay) {}
  pt_material_desc desc() const override { return detail::make(PT_MAT_MF_DIELECTRIC, {eta, ax, ay}); }
  float eta, ax, ay;
};
class ThinDielectric : public Material {
 public:
  explicit ThinDielectric(float eta, bool split = false) : eta(eta), split(split) {}
  pt_material_desc desc() const override {
    return detail::make(PT_MAT_THIN_DIELECTRIC, {eta}, split ? PT_MAT_FLAG_SPLIT_RAY : 0);
  }
  float eta;
  bool split;
};
class Phong : public Material {
 public:
  Phong(vec3 diffuse, vec3 specular, vec3 ambient, float shininess)
      : d(diffuse), s(specular), a(ambient), n(shininess) {}
  pt_material_desc desc() const override {
    return detail::make(PT_MAT_PHONG, {d[0], d[1], d[2], s[0], s[1], s[2], a[0], a[1], a[2], n});
  }
  vec3 d, s, a;
  float n;
};
class DisneyPrincipledBSDF : public Material {
 public:
  DisneyPrincipledBSDF(vec3 base, float specular_transmission, float metallic, float subsurface, float specular,
                       float roughness, float specular_tint, float anisotropic, float sheen, float sheen_tint,
                       float clearcoat, float clearcoat_gloss, float eta)
      : p{base[0], base[1], base[2], specular_transmission, metallic, subsurface, specular, roughness,
          specular_tint, anisotropic, sheen, sheen_tint, clearcoat, clearcoat_gloss, eta} {}
  pt_material_desc desc() const override {
    pt_material_desc d{};
    d.type = PT_MAT_DISNEY;
    for (int i = 0; i < 15; ++i) d.p[i] = p[i];
    return d;
  }
  float p[15];
};
class HairMarschner : public Material {
 public:
  HairMarschner(vec3 sigma_a, float h, float eta, float beta_m, float beta_n, float alpha)
      : p{sigma_a[0], sigma_a[1], sigma_a[2], h, eta, beta_m, beta_n, alpha} {}
  pt_material_desc desc() const override {
    pt_material_desc d{};
    d.type = PT_MAT_HAIR;
    for (int i = 0; i < 8; ++i) d.p[i] = p[i];
    return d;
  }
  float p[8];
};
class DiffuseEmitter : public Material {
 public:
  explicit DiffuseEmitter(vec3 color, float intensity = 1.0f) : c(color), i(intensity) {}
  DiffuseEmitter(std::shared_ptr<Texture2D> t, float intensity = 1.0f) : c(0.f), i(intensity), tex(std::move(t)) {}
  pt_material_desc desc() const override { return detail::make(PT_MAT_DIFFUSE_EMITTER, {c[0], c[1], c[2], i}); }
  bool is_emitter() const override { return true; }
  std::shared_ptr<Texture2D> texture() const override { return tex; }
  vec3 c;
  float i;
  std::shared_ptr<Texture2D> tex;
};

// ------------------------------------------------------------ geometry
struct MeshData {  // mesh_io/meshData.hpp:6-13
  std::vector<vec3> positions, normals;
  std::vector<vec2> uvs;
  std::vector<std::array<int, 3>> indices, normalIndices, uvIndices;
};

// Flattened geometry of one object, in world space.
struct Flat {
  enum Kind { MESH, QUAD, SPHERE, BOX, CURVE } kind = MESH;
  std::vector<float> pos, nrm;   // positions; normals (a list, see nidx)
  std::vector<int32_t> idx;      // 3 position indices per triangle
  std::vector<int32_t> nidx;     // 3 normal indices per triangle (-1: none)
  std::vector<float> uv;         // texture coordinates (a list, see uvidx)
  std::vector<int32_t> uvidx;    // 3 uv indices per triangle (-1: none)
  pt_quad_desc quad{};
  pt_sphere_desc sphere{};
  pt_box_desc box{};
  pt_curve_desc curve{};
  // pt_object_desc.face: HitRecord::is_inside as hit, or fixed by the
  // decorators (Translate / Rotate / Scale give true, a FlipFace over them false)
  int32_t face = PT_FACE_AS_HIT;
  std::shared_ptr<Material> mat;
};

class Hittable {
 public:
  virtual ~Hittable() = default;
  virtual Flat flatten() const = 0;
};

class Sphere : public Hittable {
 public:
  Sphere(vec3 c, float r, std::shared_ptr<Material> m) : c(c), r(r), m(std::move(m)) {}
  Flat flatten() const override {
    Flat f;
    f.kind = Flat::SPHERE;
    f.sphere.center[0] = c[0];
    f.sphere.center[1] = c[1];
    f.sphere.center[2] = c[2];
    f.sphere.radius = r;
    f.mat = m;
    return f;
  }
  vec3 c;
  float r;
  std::shared_ptr<Material> m;
};

template <Axis A>
class AARectangle : public Hittable {
 public:
  AARectangle(float k, float d0_min, float d0_max, float d1_min, float d1_max, std::shared_ptr<Material> m)
      : k(k), a0(d0_min), a1(d0_max), b0(d1_min), b1(d1_max), m(std::move(m)) {}
  Flat flatten() const override {
    Flat f;
    f.kind = Flat::QUAD;
    f.quad = pt_quad_desc{(int32_t)A, k, a0, a1, b0, b1, 0, 0};
    f.mat = m;
    return f;
  }
  float k, a0, a1, b0, b1;
  std::shared_ptr<Material> m;
};
using XYRectangle = AARectangle<Axis::Z>;
using XZRectangle = AARectangle<Axis::Y>;
using YZRectangle = AARectangle<Axis::X>;

class TriangleMesh : public Hittable {
 public:
  TriangleMesh(MeshData &&d, std::shared_ptr<Material> m) : d(std::move(d)), m(std::move(m)) {}
  Flat flatten() const override {
    Flat f;
    f.kind = Flat::MESH;
    for (auto &p : d.positions) f.pos.insert(f.pos.end(), {p[0], p[1], p[2]});
    // normals stay a list indexed per corner (normalIndices; -1: the face
    // has none and is shaded with its geometric normal)
    const bool has_n = !d.normals.empty() && d.normalIndices.size() == d.indices.size();
    if (has_n)
      for (auto &n : d.normals) f.nrm.insert(f.nrm.end(), {n[0], n[1], n[2]});
    const bool has_uv = !d.uvs.empty() && d.uvIndices.size() == d.indices.size();
    if (has_uv)
      for (auto &u : d.uvs) f.uv.insert(f.uv.end(), {u.v[0], u.v[1]});
    for (size_t t = 0; t < d.indices.size(); ++t)
      for (int k = 0; k < 3; ++k) {
        f.idx.push_back(d.indices[t][k]);
        if (has_n) f.nidx.push_back(d.normalIndices[t][k]);
        if (has_uv) f.uvidx.push_back(d.uvIndices[t][k]);
      }
    f.mat = m;
    return f;
  }
  MeshData d;
  std::shared_ptr<Material> m;
};

namespace detail {
inline Flat quad_to_mesh(const Flat &q) {
  Flat f;
  f.kind = Flat::MESH;
  f.mat = q.mat;
  const pt_quad_desc &d = q.quad;
  auto put = [&](float a, float b) {
    float v[3];
    v[d.axis] = d.k;
    v[d.axis == 0 ? 1 : 0] = a;
    v[d.axis == 2 ? 1 : 2] = b;
    f.pos.insert(f.pos.end(), {v[0], v[1], v[2]});
  };
  put(d.d0_min, d.d1_min);
  put(d.d0_max, d.d1_min);
  put(d.d0_max, d.d1_max);
  put(d.d0_min, d.d1_max);
  f.idx = {0, 1, 2, 0, 2, 3};
  return f;
}
// A Box as a mesh of its six faces (x1, x0, y1, y0, z1, z0), for rotations.
inline Flat box_to_mesh(const Flat &b) {
  Flat f;
  f.kind = Flat::MESH;
  f.mat = b.mat;
  const float *lo = b.box.min_xyz, *hi = b.box.max_xyz;
  const pt_quad_desc faces[6] = {{0, hi[0], lo[1], hi[1], lo[2], hi[2], 0, 0}, {0, lo[0], lo[1], hi[1], lo[2], hi[2], 0, 0},
                                 {1, hi[1], lo[0], hi[0], lo[2], hi[2], 0, 0}, {1, lo[1], lo[0], hi[0], lo[2], hi[2], 0, 0},
                                 {2, hi[2], lo[0], hi[0], lo[1], hi[1], 0, 0}, {2, lo[2], lo[0], hi[0], lo[1], hi[1], 0, 0}};
  for (const pt_quad_desc &q : faces) {
    Flat qf;
    qf.kind = Flat::QUAD;
    qf.quad = q;
    Flat m = quad_to_mesh(qf);
    const int32_t base = (int32_t)(f.pos.size() / 3);
    f.pos.insert(f.pos.end(), m.pos.begin(), m.pos.end());
    for (int32_t i : m.idx) f.idx.push_back(base + i);
  }
  return f;
}
}  // namespace detail

// Curve(cps, width0, width1, CurveType::Cylinder, material)
// (primitives/curve.hpp:13-157).
class Curve : public Hittable {
 public:
  Curve(const std::array<vec3, 4> &cps, float width0, float width1, std::shared_ptr<Material> m)
      : cps(cps), w0(width0), w1(width1), m(std::move(m)) {}
  Flat flatten() const override {
    Flat f;
    f.kind = Flat::CURVE;
    for (int k = 0; k < 4; ++k)
      for (int c = 0; c < 3; ++c) f.curve.cps[k][c] = cps[k][c];
    f.curve.width0 = w0;
    f.curve.width1 = w1;
    f.mat = m;
    return f;
  }
  std::array<vec3, 4> cps;
  float w0, w1;
  std::shared_ptr<Material> m;
};

// Box(min_xyz, max_xyz, material) (primitives/box.hpp:5-53).
class Box : public Hittable {
 public:
  Box(vec3 min_xyz, vec3 max_xyz, std::shared_ptr<Material> m) : lo(min_xyz), hi(max_xyz), m(std::move(m)) {}
  Flat flatten() const override {
    Flat f;
    f.kind = Flat::BOX;
    for (int c = 0; c < 3; ++c) {
      f.box.min_xyz[c] = lo[c];
      f.box.max_xyz[c] = hi[c];
    }
    f.mat = m;
    return f;
  }
  vec3 lo, hi;
  std::shared_ptr<Material> m;
};

// objectTransform.hpp decorators, baked into the flattened geometry
class FlipFace : public Hittable {
 public:
  explicit FlipFace(std::shared_ptr<Hittable> o) : o(std::move(o)) {}
  Flat flatten() const override {
    Flat f = o->flatten();
    if (f.face != PT_FACE_AS_HIT) {  // a fixed is_inside toggles
      f.face = f.face == PT_FACE_FRONT ? PT_FACE_BACK : PT_FACE_FRONT;
      return f;
    }
    if (f.kind == Flat::BOX) f = detail::box_to_mesh(f);
    if (f.kind == Flat::QUAD) f.quad.flip_face ^= 1;
    if (f.kind == Flat::SPHERE) f.sphere.flip_face ^= 1;
    if (f.kind == Flat::MESH)  // reversed winding toggles the front-face flag
      for (size_t t = 0; t + 2 < f.idx.size(); t += 3) std::swap(f.idx[t + 1], f.idx[t + 2]);
    return f;
  }
  std::shared_ptr<Hittable> o;
};
class Translate : public Hittable {
 public:
  Translate(std::shared_ptr<Hittable> o, vec3 off) : o(std::move(o)), off(off) {}
  Flat flatten() const override {
    Flat f = o->flatten();
    if (f.kind == Flat::MESH)
      for (size_t i = 0; i < f.pos.size(); ++i) f.pos[i] += off[(int)(i % 3)];
    if (f.kind == Flat::SPHERE)
      for (int c = 0; c < 3; ++c) f.sphere.center[c] += off[c];
    if (f.kind == Flat::BOX)
      for (int c = 0; c < 3; ++c) {
        f.box.min_xyz[c] += off[c];
        f.box.max_xyz[c] += off[c];
      }
    if (f.kind == Flat::CURVE)
      for (int k = 0; k < 4; ++k)
        for (int c = 0; c < 3; ++c) f.curve.cps[k][c] += off[c];
    if (f.kind == Flat::QUAD) {
      const int a = f.quad.axis, a0 = a == 0 ? 1 : 0, a1 = a == 2 ? 1 : 2;
      f.quad.k += off[a];
      f.quad.d0_min += off[a0];
      f.quad.d0_max += off[a0];
      f.quad.d1_min += off[a1];
      f.quad.d1_max += off[a1];
    }
    // Translate::intersect calls set_normal with the child's ray-facing
    // normal (objectTransform.hpp:56-57): is_inside is always true
    f.face = PT_FACE_FRONT;
    return f;
  }
  std::shared_ptr<Hittable> o;
  vec3 off;
};
class Scale : public Hittable {
 public:
  Scale(std::shared_ptr<Hittable> o, float s) : o(std::move(o)), s(s) {}
  Flat flatten() const override {
    Flat f = o->flatten();
    for (float &x : f.pos) x *= s;
    if (f.kind == Flat::SPHERE) {
      for (int c = 0; c < 3; ++c) f.sphere.center[c] *= s;
      f.sphere.radius *= s;
    }
    if (f.kind == Flat::BOX)
      for (int c = 0; c < 3; ++c) {
        f.box.min_xyz[c] *= s;
        f.box.max_xyz[c] *= s;
      }
    if (f.kind == Flat::CURVE) {
      for (int k = 0; k < 4; ++k)
        for (int c = 0; c < 3; ++c) f.curve.cps[k][c] *= s;
      f.curve.width0 *= s;
      f.curve.width1 *= s;
    }
    if (f.kind == Flat::QUAD) {
      f.quad.k *= s;
      f.quad.d0_min *= s;
      f.quad.d0_max *= s;
      f.quad.d1_min *= s;
      f.quad.d1_max *= s;
    }
    f.face = PT_FACE_FRONT;  // Scale::intersect's set_normal (objectTransform.hpp:168)
    return f;
  }
  std::shared_ptr<Hittable> o;
  float s;
};
template <Axis A>
class Rotate : public Hittable {
 public:
  Rotate(std::shared_ptr<Hittable> o, float radians) : o(std::move(o)), r(radians) {}
  Flat flatten() const override {
    Flat f = o->flatten();
    if (f.kind == Flat::QUAD) f = detail::quad_to_mesh(f);
    if (f.kind == Flat::BOX) f = detail::box_to_mesh(f);
    // Rotate<axis>::intersect (objectTransform.cpp:95-213) turns the ray
    // into the child's frame with (c a - s b, s a + c b) over the axis pair
    // (a, b) = (y, z), (x, z), (x, y) and maps the hit back with the inverse,
    // (c a + s b, -s a + c b): the child's geometry seen in the world
    const float c = std::cos(r), s = std::sin(r);
    const int i = A == Axis::X ? 1 : 0, j = A == Axis::Z ? 1 : 2;
    auto rot = [&](float *p) {
      float a = p[i], b = p[j];
      p[i] = c * a + s * b;
      p[j] = -s * a + c * b;
    };
    for (size_t k = 0; k + 2 < f.pos.size(); k += 3) rot(&f.pos[k]);
    for (size_t k = 0; k + 2 < f.nrm.size(); k += 3) rot(&f.nrm[k]);
    if (f.kind == Flat::SPHERE) rot(f.sphere.center);
    if (f.kind == Flat::CURVE)
      for (int k = 0; k < 4; ++k) rot(f.curve.cps[k]);
    f.face = PT_FACE_FRONT;  // Rotate<axis>::intersect's set_normal (objectTransform.cpp:131, 172, 210)
    return f;
  }
  std::shared_ptr<Hittable> o;
  float r;
};

// loadOBJMesh (src/mesh_io/meshLoader.cpp:7-58) through pt_obj_load.
inline std::shared_ptr<TriangleMesh> loadOBJMesh(const std::string &path, std::shared_ptr<Material> mat) {
  pt_mesh_desc m{};
  if (pt_obj_load(path.c_str(), &m) != PT_OK) {
    char buf[512] = {0};
    pt_last_error(nullptr, buf, sizeof buf);
    throw std::runtime_error(buf);
  }
  MeshData d;
  for (int i = 0; i < m.n_positions; ++i)
    d.positions.push_back(vec3{m.positions[3 * i], m.positions[3 * i + 1], m.positions[3 * i + 2]});
  for (int i = 0; i < m.n_normals; ++i)
    d.normals.push_back(vec3{m.normals[3 * i], m.normals[3 * i + 1], m.normals[3 * i + 2]});
  for (int i = 0; i < m.n_uvs; ++i) d.uvs.push_back(vec2{m.uvs[2 * i], m.uvs[2 * i + 1]});
  for (int t = 0; t < m.n_triangles; ++t) {
    d.indices.push_back({m.indices[3 * t], m.indices[3 * t + 1], m.indices[3 * t + 2]});
    d.normalIndices.push_back({m.normal_indices[3 * t], m.normal_indices[3 * t + 1], m.normal_indices[3 * t + 2]});
    d.uvIndices.push_back({m.uv_indices[3 * t], m.uv_indices[3 * t + 1], m.uv_indices[3 * t + 2]});
  }
  pt_obj_free(&m);
  return std::make_shared<TriangleMesh>(std::move(d), std::move(mat));
}

class ObjectList {  // base/objectList.hpp
 public:
  void addObject(std::shared_ptr<Hittable> h) { objects.push_back(std::move(h)); }
  const std::vector<std::shared_ptr<Hittable>> &getLists() const { return objects; }
  std::vector<std::shared_ptr<Hittable>> objects;
};

// EnvironmentLight over texels given in memory (row 0 = bottom, RGB) or
// loaded from an HDR image file.
class EnvironmentLight {
 public:
  EnvironmentLight(std::vector<float> texels, int width, int height, float intensity = 1.0f)
      : texels(std::move(texels)), width(width), height(height), intensity(intensity) {}
  // envLight.hpp:7: HDRITexture(hdri_filepath, flip_y = false, isHDR = true)
  explicit EnvironmentLight(const std::string &hdri_filepath, float intensity_scale = 1.0f)
      : texels(detail::load_texels(hdri_filepath, false, true, width, height)), intensity(intensity_scale) {}
  std::vector<float> texels;
  int width, height;
  float intensity;
};

class PerspectiveCamera {  // base/camera.hpp
 public:
  PerspectiveCamera(float fov, float aspect, float focalDist, float aperture, vec3 up, vec3 front, vec3 position)
      : fov(fov), aspect(aspect), focalDist(focalDist), aperture(aperture), up(up), front(front), position(position) {}
  float fov, aspect, focalDist, aperture;
  vec3 up, front, position;
};

// ------------------------------------------------------------ samplers
// Sampler / HaltonSampler (sampler/sampler.hpp:7-83): the sample index
// advances with startSample() and the dimension counter restarts; get1D /
// get2D take the next dimensions of the index's point, computed by the device
// code the render runs (pt_sampler_eval, fetched 32 dimensions at a time).
enum class RandomStrategy { None, PermuteDigits, Owen };
class Sampler {
 public:
  virtual ~Sampler() = default;
  virtual float get1D() = 0;
  virtual vec2 get2D() = 0;
};
class HaltonSampler : public Sampler {
 public:
  explicit HaltonSampler(uint32_t seed = 0, RandomStrategy strat = RandomStrategy::Owen)
      : strategy(strat), seed_(seed) {}
  void startSample() {
    ++sampleIndex_;
    dimension_ = 0;
    block_.clear();
  }
  float get1D() override { return dim(dimension_++); }
  vec2 get2D() override {
    const float x = dim(dimension_++);
    const float y = dim(dimension_++);
    return vec2(x, y);
  }
  // The current sample index (the reference's sampleIndex_; the render's
  // path (i, j, k) of a W x H x spp frame uses 1 + ((i H + j) spp + k)).
  uint32_t sampleIndex() const { return sampleIndex_; }
  void setSampleIndex(uint32_t index) {
    sampleIndex_ = index;
    dimension_ = 0;
    block_.clear();
  }

 private:
  float dim(int d) {
    if (d >= (int)block_.size()) {
      const int dims = (d / 32 + 1) * 32;
      block_.assign((size_t)dims, 0.f);
      void *ctx = detail::thread_context();
      detail::check(pt_sampler_eval(ctx, (int32_t)strategy, seed_, sampleIndex_, 1, dims, block_.data()), ctx);
    }
    return block_[(size_t)d];
  }
  RandomStrategy strategy;
  uint32_t seed_;
  uint32_t sampleIndex_ = 0;
  int dimension_ = 0;
  std::vector<float> block_;  // dimensions of the current index fetched so far
};

// ------------------------------------------------------------- lights
// Light (light/light.hpp:17-53): light `index` of a scene uploaded to ctx,
// in the LightList order the render samples (lightDiscovery.hpp:5-81: the
// DiffuseEmitter rectangles and spheres in object order, then the
// environment), evaluated by the device code of next-event estimation
// (pt_light_sample).  get_normal_at and L_emit are taken at the point
// get_sample(u, v) gives, the only points the reference's NEE asks about
// (maxdepth_nee.hpp:171-176).
enum class LightType { QUAD_LIGHT, SPHERE_LIGHT, ENVIRONMENT_LIGHT };
struct LightSample {
  vec3 point, normal, dir, Le;
  float pdf = 0.f;
};
class Light {
 public:
  Light(void *ctx, int32_t scene, int32_t index) : ctx(ctx), scene(scene), index(index) {}
  // get_sample(u, v) with get_normal_at there, the direction from x to it,
  // L_emit towards x (texCoords (u, v)) and pdf_value(x, that direction)
  LightSample sample(float u, float v, const vec3 &x) const { return eval(u, v, x, nullptr); }
  vec3 get_sample(float u, float v) const { return eval(u, v, vec3(0.f), nullptr).point; }
  vec3 get_normal_at_sample(float u, float v) const { return eval(u, v, vec3(0.f), nullptr).normal; }
  vec3 L_emit_towards(float u, float v, const vec3 &x) const { return eval(u, v, x, nullptr).Le; }
  float pdf_value(const vec3 &origin, const vec3 &dir) const { return eval(0.5f, 0.5f, origin, &dir).pdf; }
  float get_area() const {
    float a = 0.f;
    detail::check(pt_light_sample(ctx, scene, index, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                  nullptr, nullptr, &a),
                  ctx);
    return a;
  }

 private:
  LightSample eval(float u, float v, const vec3 &x, const vec3 *pdf_dir) const {
    const float uv[2] = {u, v}, xx[3] = {x[0], x[1], x[2]};
    float pd[3] = {0.f, 0.f, 0.f};
    if (pdf_dir)
      for (int c = 0; c < 3; ++c) pd[c] = (*pdf_dir)[c];
    float p[3], n[3], w[3], le[3], pdf;
    detail::check(pt_light_sample(ctx, scene, index, 1, uv, xx, pdf_dir ? pd : nullptr, p, n, w, le, &pdf, nullptr),
                  ctx);
    LightSample r;
    r.point = vec3(p[0], p[1], p[2]);
    r.normal = vec3(n[0], n[1], n[2]);
    r.dir = vec3(w[0], w[1], w[2]);
    r.Le = vec3(le[0], le[1], le[2]);
    r.pdf = pdf;
    return r;
  }
  void *ctx;
  int32_t scene, index;
};
// LightList (base/lightList.hpp:5-40) of a scene uploaded to ctx.
class LightList {
 public:
  LightList(void *ctx, int32_t scene) : ctx(ctx), scene(scene) {
    int64_t info[6] = {0};
    detail::check(pt_scene_info(ctx, scene, info), ctx);
    n = (int)info[4];
  }
  size_t size() const { return (size_t)n; }
  Light get(int i) const {
    if (i < 0 || i >= n) throw std::out_of_range("light index");
    return Light(ctx, scene, i);
  }

 private:
  void *ctx;
  int32_t scene;
  int n = 0;
};

// getRayColor (integrator/maxdepth_nee.hpp:9-256) for rays through a scene
// uploaded to ctx, on the device (pt_ray_color): one path per ray, ray i with
// Halton index first_index + i.  estimator PT_EST_REF_NEE is the reference's
// NEE integrator; light samples 2 x 2 (LIGHT_SAMPLE_X/Y, config.hpp:5-6).
inline std::vector<vec3> getRayColor(void *ctx, int32_t scene, const std::vector<Ray> &rays, uint32_t max_depth,
                                     uint32_t first_index = 1, int32_t estimator = PT_EST_REF_NEE,
                                     uint32_t seed = 0) {
  std::vector<float> r;
  for (const Ray &ray : rays)
    for (int c = 0; c < 6; ++c) r.push_back(c < 3 ? ray.getOrigin()[c] : ray.getDirection()[c - 3]);
  pt_job_desc j{};
  j.scene = scene;
  j.width = j.height = j.spp_x = j.spp_y = 1;
  j.max_depth = (int32_t)max_depth;
  j.rr_start = -1;
  j.estimator = estimator;
  j.sampler = PT_SAMPLER_HALTON_OWEN;
  j.env_sampling = PT_ENV_UNIFORM;
  j.light_samples_x = j.light_samples_y = 2;
  j.seed = seed;
  j.gamma = 1.f;
  std::vector<float> out(rays.size() * 3);
  detail::check(pt_ray_color(ctx, &j, r.data(), (int32_t)rays.size(), first_index, out.data()), ctx);
  std::vector<vec3> c;
  for (size_t i = 0; i < rays.size(); ++i) c.push_back(vec3(out[3 * i], out[3 * i + 1], out[3 * i + 2]));
  return c;
}

// SceneInfo (render/renderManager.hpp:35-176): render() uploads the scene and
// renders it through the C-ABI; the film and the tone-mapped bytes are kept.
struct SceneInfo {
  std::shared_ptr<PerspectiveCamera> camera;
  ObjectList objects;
  std::shared_ptr<EnvironmentLight> environment_light;
  vec3 bg_color = vec3(0.7f, 0.8f, 1.0f);
  uint32_t _width = 800, _height = 800, spp_x = 2, spp_y = 2;
  float _gamma = 1.0f;
  uint32_t max_depth = 10;                   // MAX_RAY_DEPTH (config.hpp:7)
  int32_t estimator = PT_EST_NEE_MIS;
  int32_t device = 0;
  std::vector<float> film;                   // mean radiance [j][i][c], j = 0 bottom
  std::vector<uint8_t> rgb8;                 // tone-mapped, row 0 top

  // Flattens the object list (decorators baked into the geometry, light
  // discovery and BVH build in the library) and uploads it to ctx; returns
  // the scene id (the scene set-up of SceneInfo::render,
  // renderManager.hpp:80-95).
  int32_t upload(void *ctx) const {
    if (objects.getLists().empty()) throw std::runtime_error("No objects in the scene!");
    std::vector<pt_material_desc> mats;
    std::vector<Flat> flats;
    std::vector<pt_mesh_desc> meshes;
    std::vector<pt_quad_desc> quads;
    std::vector<pt_sphere_desc> spheres;
    std::vector<pt_object_desc> objs;
    std::vector<pt_box_desc> boxes;
    std::vector<pt_curve_desc> curves;
    std::vector<pt_texture_desc> texs;
    std::vector<std::shared_ptr<Texture2D>> tex_objs;
    for (auto &h : objects.getLists()) flats.push_back(h->flatten());
    meshes.reserve(flats.size());
    for (auto &f : flats) {
      mats.push_back(f.mat->desc());
      const int32_t mi = (int32_t)mats.size() - 1;
      if (auto t = f.mat->texture()) {
        int ti = -1;
        for (size_t k = 0; k < tex_objs.size(); ++k)
          if (tex_objs[k] == t) ti = (int)k;
        if (ti < 0) {
          ti = (int)tex_objs.size();
          tex_objs.push_back(t);
          texs.push_back(t->desc());
        }
        mats[mi].flags |= (ti + 1) << PT_MAT_TEXTURE_SHIFT;
      }
      if (f.kind == Flat::MESH) {
        pt_mesh_desc m{};
        m.positions = f.pos.data();
        m.n_positions = (int32_t)(f.pos.size() / 3);
        if (!f.nrm.empty()) {
          m.normals = f.nrm.data();
          m.n_normals = (int32_t)(f.nrm.size() / 3);
          m.normal_indices = f.nidx.data();
        }
        if (!f.uv.empty()) {
          m.uvs = f.uv.data();
          m.n_uvs = (int32_t)(f.uv.size() / 2);
          m.uv_indices = f.uvidx.data();
        }
        m.indices = f.idx.data();
        m.n_triangles = (int32_t)(f.idx.size() / 3);
        m.material = mi;
        meshes.push_back(m);
        objs.push_back({PT_OBJ_MESH, (int32_t)meshes.size() - 1, {0.f, 0.f, 0.f}, f.face});
      } else if (f.kind == Flat::CURVE) {
        f.curve.material = mi;
        curves.push_back(f.curve);
        objs.push_back({PT_OBJ_CURVE, (int32_t)curves.size() - 1, {0.f, 0.f, 0.f}, f.face});
      } else if (f.kind == Flat::BOX) {
        f.box.material = mi;
        boxes.push_back(f.box);
        objs.push_back({PT_OBJ_BOX, (int32_t)boxes.size() - 1, {0.f, 0.f, 0.f}, f.face});
      } else if (f.kind == Flat::QUAD) {
        f.quad.material = mi;
        quads.push_back(f.quad);
        objs.push_back({PT_OBJ_QUAD, (int32_t)quads.size() - 1, {0.f, 0.f, 0.f}, f.face});
      } else {
        f.sphere.material = mi;
        spheres.push_back(f.sphere);
        objs.push_back({PT_OBJ_SPHERE, (int32_t)spheres.size() - 1, {0.f, 0.f, 0.f}, f.face});
      }
    }
    pt_scene_desc d{};
    d.materials = mats.data();
    d.n_materials = (int32_t)mats.size();
    d.meshes = meshes.data();
    d.n_meshes = (int32_t)meshes.size();
    d.quads = quads.data();
    d.n_quads = (int32_t)quads.size();
    d.spheres = spheres.data();
    d.n_spheres = (int32_t)spheres.size();
    d.objects = objs.data();
    d.n_objects = (int32_t)objs.size();
    d.textures = texs.data();
    d.n_textures = (int32_t)texs.size();
    d.boxes = boxes.data();
    d.n_boxes = (int32_t)boxes.size();
    d.curves = curves.data();
    d.n_curves = (int32_t)curves.size();
    pt_env_desc env{};
    if (environment_light) {
      env = pt_env_desc{environment_light->texels.data(), environment_light->width, environment_light->height,
                        environment_light->intensity};
      d.env = &env;
    }
    for (int c = 0; c < 3; ++c) d.bg_color[c] = bg_color[c];
    int32_t sid = 0;
    check(pt_scene_upload(ctx, &d, &sid), ctx);
    return sid;
  }

  void render(const std::string &out_path = "") {
    if (!camera) throw std::runtime_error("Camera is not initialized!");
    void *ctx = nullptr;
    check(pt_create(&ctx, device), nullptr);
    int32_t sid = 0;
    try {
      sid = upload(ctx);
      pt_job_desc j{};
      j.scene = sid;
      j.width = (int32_t)_width;
      j.height = (int32_t)_height;
      j.spp_x = (int32_t)spp_x;
      j.spp_y = (int32_t)spp_y;
      j.max_depth = (int32_t)max_depth;
      j.rr_start = -1;
      j.estimator = estimator;
      j.sampler = PT_SAMPLER_HALTON_OWEN;
      j.env_sampling = estimator == PT_EST_NEE_MIS ? PT_ENV_ALIAS : PT_ENV_UNIFORM;
      j.light_samples_x = 2;
      j.light_samples_y = 2;
      const PerspectiveCamera &c = *camera;
      j.camera = pt_camera_desc{c.fov, c.aspect, c.focalDist, c.aperture, {c.up[0], c.up[1], c.up[2]},
                                {c.front[0], c.front[1], c.front[2]},
                                {c.position[0], c.position[1], c.position[2]}, 0.f};
      j.gamma = _gamma;
      film.assign((size_t)_width * _height * 3, 0.f);
      check(pt_render(ctx, &j, film.data(), nullptr), ctx);
      rgb8.assign(film.size(), 0);
      check(pt_tonemap(ctx, film.data(), (int32_t)_width, (int32_t)_height, _gamma, rgb8.data()), ctx);
      pt_scene_release(ctx, sid);
    } catch (...) {
      pt_destroy(ctx);
      throw;
    }
    pt_destroy(ctx);
    if (!out_path.empty()) write_ppm(out_path);
  }

  // Binary PPM of the tone-mapped image (PNG output is host I/O left to the caller).
  void write_ppm(const std::string &path) const {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot open " + path);
    std::fprintf(f, "P6\n%u %u\n255\n", _width, _height);
    std::fwrite(rgb8.data(), 1, rgb8.size(), f);
    std::fclose(f);
  }

 private:
  static void check(int rc, void *ctx) {
    if (rc != PT_OK) {
      char buf[512] = {0};
      pt_last_error(ctx, buf, sizeof buf);
      throw std::runtime_error(std::string("pathtracer_gb300: ") + buf);
    }
  }
};

}  // namespace ptgb
