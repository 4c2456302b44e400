// The Cornell box with ColorVariant textures, written the way the
// reference's scene functions are (Lambertian(std::shared_ptr<Texture2D>),
// DiffuseEmitter(texture, intensity)), rendered through the C++ API.  Prints
// the per-channel image mean.
#include <cstdio>
#include <memory>

#include "pathtracer_gb300.hpp"

using namespace ptgb;

SceneInfo textured_cornell() {
  using std::make_shared;
  SceneInfo scene;
  ObjectList objects;
  auto checker = make_shared<CheckerTexture>(vec3(0.1f), vec3(0.8f), 40.f);
  auto noise = make_shared<NoiseTexture>(8.f, 4);
  auto lchk = make_shared<CheckerTexture>(vec3(4.f, 2.f, 0.5f), vec3(20.f, 14.f, 5.f), 30.f);
  auto white = make_shared<Lambertian>(vec3(0.75f));
  auto floor = make_shared<Lambertian>(checker);
  auto back = make_shared<Lambertian>(noise);
  auto green = make_shared<Lambertian>(vec3(0.14f, 0.45f, 0.09f));
  auto light = make_shared<DiffuseEmitter>(lchk, 1.f);
  auto ball = make_shared<Lambertian>(noise);
  objects.addObject(make_shared<AARectangle<Axis::Y>>(0.999f, 0.3f, 0.7f, 0.3f, 0.7f, light));
  objects.addObject(make_shared<AARectangle<Axis::X>>(1.f, 0.f, 1.f, 0.f, 1.f, white));
  objects.addObject(make_shared<AARectangle<Axis::X>>(0.f, 0.f, 1.f, 0.f, 1.f, green));
  objects.addObject(make_shared<AARectangle<Axis::Y>>(0.f, 0.f, 1.f, 0.f, 1.f, floor));
  objects.addObject(make_shared<AARectangle<Axis::Y>>(1.f, 0.f, 1.f, 0.f, 1.f, white));
  objects.addObject(make_shared<AARectangle<Axis::Z>>(1.f, 0.f, 1.f, 0.f, 1.f, back));
  objects.addObject(make_shared<Sphere>(vec3(0.5f, 0.3f, 0.55f), 0.25f, ball));
  scene.objects = objects;
  scene._width = 48;
  scene._height = 48;
  scene.spp_x = 4;
  scene.spp_y = 4;
  scene._gamma = 2.0f;
  scene.max_depth = 6;
  scene.bg_color = vec3(0.f);
  scene.camera = make_shared<PerspectiveCamera>(to_radian(40.f), 1.f, 10.f, 1000.f, vec3(0, 1, 0), vec3(0, 0, 1),
                                                vec3(0.5f, 0.5f, -1.4f));
  return scene;
}

int main() {
  SceneInfo scene = textured_cornell();
  scene.render("");
  double m[3] = {0, 0, 0};
  for (size_t i = 0; i < scene.film.size(); ++i) m[i % 3] += scene.film[i];
  const double n = (double)scene.film.size() / 3;
  std::printf("%.7f %.7f %.7f\n", m[0] / n, m[1] / n, m[2] / n);
  return 0;
}
