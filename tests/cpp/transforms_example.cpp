// Decorated objects built with the C++ scene API (Translate, Rotate<axis>,
// Scale, FlipFace over meshes, rectangles and spheres, as a scene written
// against the reference builds them), then either flattened (the geometry
// with the transforms baked in, "flatten") or uploaded and intersected on the
// GPU through pt_intersect ("trace").  Input (text, argv[2]): the number of
// cases, then per case
//   kind (0 mesh, 1 rectangle, 2 sphere) and its data:
//     mesh: n_positions n_triangles, positions (3 each), indices (3 each)
//     rectangle: axis k d0_min d0_max d1_min d1_max
//     sphere: cx cy cz r
//   n_ops, then per op: code p0 p1 p2 (0 Translate(p0,p1,p2), 1 Rotate<X>(p0),
//     2 Rotate<Y>(p0), 3 Rotate<Z>(p0), 4 Scale(p0), 5 FlipFace), innermost first
//   n_rays, then per ray origin and direction (6 floats).
#include <cstdio>
#include <fstream>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "pathtracer_gb300.hpp"

using namespace ptgb;

static std::shared_ptr<Hittable> read_case(std::istream &in, std::vector<float> &rays) {
  auto mat = std::make_shared<Lambertian>(vec3(0.5f));
  int kind = 0;
  in >> kind;
  std::shared_ptr<Hittable> h;
  if (kind == 0) {
    int np = 0, nt = 0;
    in >> np >> nt;
    MeshData d;
    for (int i = 0; i < np; ++i) {
      float x, y, z;
      in >> x >> y >> z;
      d.positions.push_back(vec3(x, y, z));
    }
    for (int t = 0; t < nt; ++t) {
      int a, b, c;
      in >> a >> b >> c;
      d.indices.push_back({a, b, c});
    }
    h = std::make_shared<TriangleMesh>(std::move(d), mat);
  } else if (kind == 1) {
    int axis;
    float k, a0, a1, b0, b1;
    in >> axis >> k >> a0 >> a1 >> b0 >> b1;
    if (axis == 0) h = std::make_shared<YZRectangle>(k, a0, a1, b0, b1, mat);
    else if (axis == 1) h = std::make_shared<XZRectangle>(k, a0, a1, b0, b1, mat);
    else h = std::make_shared<XYRectangle>(k, a0, a1, b0, b1, mat);
  } else {
    float x, y, z, r;
    in >> x >> y >> z >> r;
    h = std::make_shared<Sphere>(vec3(x, y, z), r, mat);
  }
  int nops = 0;
  in >> nops;
  for (int k = 0; k < nops; ++k) {
    int code;
    float p0, p1, p2;
    in >> code >> p0 >> p1 >> p2;
    switch (code) {
    case 0: h = std::make_shared<Translate>(h, vec3(p0, p1, p2)); break;
    case 1: h = std::make_shared<Rotate<Axis::X>>(h, p0); break;
    case 2: h = std::make_shared<Rotate<Axis::Y>>(h, p0); break;
    case 3: h = std::make_shared<Rotate<Axis::Z>>(h, p0); break;
    case 4: h = std::make_shared<Scale>(h, p0); break;
    default: h = std::make_shared<FlipFace>(h); break;
    }
  }
  int nr = 0;
  in >> nr;
  rays.resize((size_t)nr * 6);
  for (auto &v : rays) in >> v;
  return h;
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  const std::string mode = argv[1];
  std::ifstream in(argv[2]);
  int ncases = 0;
  in >> ncases;
  void *ctx = nullptr;
  if (mode == "trace" && pt_create(&ctx, 0) != PT_OK) return 3;
  for (int c = 0; c < ncases; ++c) {
    std::vector<float> rays;
    std::shared_ptr<Hittable> h = read_case(in, rays);
    if (mode == "flatten") {
      const Flat f = h->flatten();
      std::printf("%d\n", f.face);
      if (f.kind == Flat::MESH) {
        std::printf("0 %zu %zu\n", f.pos.size() / 3, f.idx.size() / 3);
        for (float x : f.pos) std::printf("%.9g\n", x);
        for (int i : f.idx) std::printf("%d\n", i);
      } else if (f.kind == Flat::QUAD) {
        std::printf("1 %d %.9g %.9g %.9g %.9g %.9g %d\n", f.quad.axis, f.quad.k, f.quad.d0_min, f.quad.d0_max,
                    f.quad.d1_min, f.quad.d1_max, f.quad.flip_face);
      } else {
        std::printf("2 %.9g %.9g %.9g %.9g %d\n", f.sphere.center[0], f.sphere.center[1], f.sphere.center[2],
                    f.sphere.radius, f.sphere.flip_face);
      }
      continue;
    }
    SceneInfo scene;
    scene.objects.addObject(h);
    const int32_t sid = scene.upload(ctx);
    const int n = (int)(rays.size() / 6);
    std::vector<float> t(n), pos(3 * n), nrm(3 * n);
    std::vector<int32_t> prim(n);
    std::vector<uint8_t> inside(n);
    if (pt_intersect(ctx, sid, rays.data(), n, 1e-4f, 1e5f, t.data(), prim.data(), pos.data(), nrm.data(),
                     inside.data()) != PT_OK)
      return 4;
    for (int i = 0; i < n; ++i)
      std::printf("%d %.9g %.9g %.9g %.9g %.9g %.9g %.9g %d\n", prim[i] >= 0 ? 1 : 0, t[i], pos[3 * i],
                  pos[3 * i + 1], pos[3 * i + 2], nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2], inside[i]);
    pt_scene_release(ctx, sid);
  }
  if (ctx) pt_destroy(ctx);
  return 0;
}
