// The reference-shaped C++ surface over the C-ABI: Material::f / scatter_pdf
// / scatter, HaltonSampler, LightList / Light and getRayColor, as code
// written against the reference calls them.  Prints one value per line.
#include <cstdio>
#include <memory>
#include <vector>

#include "pathtracer_gb300.hpp"

using namespace ptgb;

static void put(const vec3 &v) { std::printf("%.9g %.9g %.9g\n", v[0], v[1], v[2]); }

int main() {
  // Material::f / scatter_pdf / scatter: GGX gold, alpha 0.3
  auto gold = std::make_shared<Conductor>(vec3(0.143f, 0.374f, 1.442f), vec3(3.983f, 2.385f, 1.603f), 0.3f, 0.3f);
  HitRecord rec;
  rec.normal = vec3(0.f, 0.f, 1.f);
  rec.position = vec3(0.1f, 0.2f, 0.3f);
  rec.is_inside = true;
  const vec3 wo(0.3f, -0.2f, 0.932738f), wi(-0.4f, 0.1f, 0.910494f);
  put(gold->f(wo, wi, rec));
  std::printf("%.9g\n", gold->scatter_pdf(wo, wi, rec));
  ScatterRecord srec;
  const bool ok = gold->scatter(Ray(vec3(0.f), vec3(-0.3f, 0.2f, -0.932738f)), rec, srec, 0.37f, vec2(0.21f, 0.83f));
  std::printf("%d %u %.9g\n", ok ? 1 : 0, srec.sampled_type, srec.pdf_val);
  put(srec.sampled_ray.getDirection());
  put(srec.attenuation);
  put(srec.sampled_ray.getOrigin());
  // DiffuseEmitter::emit, two sides
  auto light = std::make_shared<DiffuseEmitter>(vec3(17.f, 12.f, 4.f), 1.5f);
  put(light->emit(Ray(vec3(0.f), vec3(0.f, 0.f, -1.f)), rec));
  put(light->emit(Ray(vec3(0.f), vec3(0.f, 0.f, 1.f)), rec));
  // HaltonSampler (Owen): indices 1..3, five dimensions each
  HaltonSampler hs;
  for (int i = 0; i < 3; ++i) {
    hs.startSample();
    const float a = hs.get1D();
    const vec2 b = hs.get2D();
    const vec2 c = hs.get2D();
    std::printf("%u %.9g %.9g %.9g %.9g %.9g\n", hs.sampleIndex(), a, b.v[0], b.v[1], c.v[0], c.v[1]);
  }
  // a Cornell box: its lights and getRayColor
  void *ctx = nullptr;
  if (pt_create(&ctx, 0) != PT_OK) return 3;
  SceneInfo scene;
  auto white = std::make_shared<Lambertian>(vec3(0.75f));
  auto lm = std::make_shared<DiffuseEmitter>(vec3(17.f, 12.f, 4.f));
  scene.objects.addObject(std::make_shared<XZRectangle>(0.999f, 0.375f, 0.625f, 0.375f, 0.625f, lm));
  scene.objects.addObject(std::make_shared<YZRectangle>(1.f, 0.f, 1.f, 0.f, 1.f, white));
  scene.objects.addObject(std::make_shared<YZRectangle>(0.f, 0.f, 1.f, 0.f, 1.f, white));
  scene.objects.addObject(std::make_shared<XZRectangle>(0.f, 0.f, 1.f, 0.f, 1.f, white));
  scene.objects.addObject(std::make_shared<XZRectangle>(1.f, 0.f, 1.f, 0.f, 1.f, white));
  scene.objects.addObject(std::make_shared<XYRectangle>(1.f, 0.f, 1.f, 0.f, 1.f, white));
  scene.objects.addObject(std::make_shared<Sphere>(vec3(0.5f, 0.3f, 0.55f), 0.25f, gold));
  scene.objects.addObject(std::make_shared<Sphere>(vec3(0.2f, 0.8f, 0.3f), 0.05f, lm));
  const int32_t sid = scene.upload(ctx);
  LightList lights(ctx, sid);
  std::printf("%zu\n", lights.size());
  for (size_t li = 0; li < lights.size(); ++li) {
    const Light L = lights.get((int)li);
    const LightSample s = L.sample(0.3f, 0.7f, vec3(0.5f, 0.4f, 0.5f));
    put(s.point);
    put(s.normal);
    put(s.dir);
    put(s.Le);
    std::printf("%.9g %.9g %.9g\n", s.pdf, L.get_area(), L.pdf_value(vec3(0.5f, 0.4f, 0.5f), s.dir));
  }
  std::vector<Ray> rays;
  for (int i = 0; i < 64; ++i)
    rays.push_back(Ray(vec3(0.5f, 0.5f, -1.4f), vec3(-0.2f + 0.4f * (i % 8) / 7.f, -0.2f + 0.4f * (i / 8) / 7.f, 1.f)));
  for (const Ray &r : rays) put(r.getDirection());  // the rays as this program rounded them
  for (const vec3 &c : getRayColor(ctx, sid, rays, 8, 101)) put(c);
  pt_scene_release(ctx, sid);
  pt_destroy(ctx);
  return 0;
}
