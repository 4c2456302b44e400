// A scene written the way the reference's scene functions are written
// (include/scenes/scenes_01.hpp:cornell_box), rendered through the C++ API
// of include/pathtracer_gb300.hpp.  Prints the per-channel image mean.
#include <cstdio>
#include <memory>

#include "pathtracer_gb300.hpp"

using namespace ptgb;

SceneInfo cornell_sphere() {
  using std::make_shared;
  SceneInfo scene;
  ObjectList objects;
  auto white = make_shared<Lambertian>(vec3(0.75f));
  auto red = make_shared<Lambertian>(vec3(0.63f, 0.065f, 0.05f));
  auto green = make_shared<Lambertian>(vec3(0.14f, 0.45f, 0.09f));
  auto light = make_shared<DiffuseEmitter>(vec3(17.f, 12.f, 4.f), 1.f);
  auto gold = make_shared<Conductor>(vec3(0.14f, 0.43f, 1.38f), vec3(4.54f, 2.455f, 1.914f), 0.3f, 0.3f);
  objects.addObject(make_shared<AARectangle<Axis::Y>>(0.999f, 0.375f, 0.625f, 0.375f, 0.625f, light));
  objects.addObject(make_shared<AARectangle<Axis::X>>(1.f, 0.f, 1.f, 0.f, 1.f, red));
  objects.addObject(make_shared<AARectangle<Axis::X>>(0.f, 0.f, 1.f, 0.f, 1.f, green));
  objects.addObject(make_shared<AARectangle<Axis::Y>>(0.f, 0.f, 1.f, 0.f, 1.f, white));
  objects.addObject(make_shared<AARectangle<Axis::Y>>(1.f, 0.f, 1.f, 0.f, 1.f, white));
  objects.addObject(make_shared<AARectangle<Axis::Z>>(1.f, 0.f, 1.f, 0.f, 1.f, white));
  objects.addObject(make_shared<Sphere>(vec3(0.5f, 0.3f, 0.55f), 0.25f, gold));
  scene.objects = objects;
  scene._width = 48;
  scene._height = 48;
  scene.spp_x = 4;
  scene.spp_y = 4;
  scene._gamma = 2.0f;
  scene.max_depth = 8;
  scene.bg_color = vec3(0.f);
  scene.camera = make_shared<PerspectiveCamera>(to_radian(40.f), 1.f, 10.f, 1000.f, vec3(0, 1, 0), vec3(0, 0, 1),
                                                vec3(0.5f, 0.5f, -1.4f));
  return scene;
}

int main(int argc, char **argv) {
  SceneInfo scene = cornell_sphere();
  scene.render(argc > 1 ? argv[1] : "");
  double m[3] = {0, 0, 0};
  for (size_t i = 0; i < scene.film.size(); ++i) m[i % 3] += scene.film[i];
  const double n = (double)scene.film.size() / 3;
  std::printf("%.7f %.7f %.7f\n", m[0] / n, m[1] / n, m[2] / n);
  return 0;
}
