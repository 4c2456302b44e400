// pt_obj.cpp -- OBJ ingest of the C-ABI (pt_obj_load / pt_obj_free).
//
// Restates loadOBJMesh (src/mesh_io/meshLoader.cpp:7-58), which reads the
// file through tinyobjloader (vendored as include/external/tiny_obj_loader.h)
// and copies positions, optional normals and uvs, and per-face vertex /
// normal / uv indices into MeshData: "v", "vn", "vt" and "f" records; face
// vertices "v", "v/vt", "v//vn", "v/vt/vn"; 1-based or negative (relative to
// the records read so far) indices; an absent normal or uv index is -1.
// tinyobjloader triangulates quads along the shorter diagonal (v0-v2 if
// |v2 - v0|^2 < |v3 - v1|^2, else v1-v3) and that rule is kept; longer
// polygons are fanned from their first vertex (tinyobjloader ear-clips them).
// Every other record (groups, objects, materials, smoothing) is ignored, as
// loadOBJMesh ignores it.  Unlike tinyobjloader, which skips faces with
// out-of-range indices with a warning, such a face is an error here.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "pt_host.h"

namespace pt {
namespace {

struct ObjData {
  std::vector<float> pos, nrm, uv;
  std::vector<int32_t> vi, ni, ti;
};

// Resolves a 1-based or negative OBJ index against `count` records read so
// far; 0 is invalid.
bool resolve(long v, size_t count, int32_t &out) {
  if (v > 0) {
    out = (int32_t)(v - 1);
    return true;
  }
  if (v < 0 && (size_t)(-v) <= count) {
    out = (int32_t)((long)count + v);
    return true;
  }
  return false;
}

struct FaceVertex {
  int32_t v, t, n;
};

void parse(const char *path, ObjData &D) {
  FILE *f = std::fopen(path, "rb");
  if (!f) fail(PT_ERR_NOT_FOUND, std::string("cannot open OBJ file: ") + path);
  std::string line;
  std::vector<char> buf(1 << 16);
  std::vector<FaceVertex> face;
  long lineno = 0;
  auto error = [&](const std::string &msg) {
    std::fclose(f);
    fail(PT_ERR_INVALID, std::string(path) + ":" + std::to_string(lineno) + ": " + msg);
  };
  for (;;) {
    line.clear();
    bool got = false;
    while (std::fgets(buf.data(), (int)buf.size(), f)) {
      got = true;
      line += buf.data();
      if (!line.empty() && line.back() == '\n') break;
    }
    if (!got) break;
    ++lineno;
    const char *p = line.c_str();
    while (*p == ' ' || *p == '\t') ++p;
    if (p[0] == 'v' && (p[1] == ' ' || p[1] == '\t')) {
      char *e;
      float x = std::strtof(p + 2, &e), y = std::strtof(e, &e), z = std::strtof(e, &e);
      D.pos.insert(D.pos.end(), {x, y, z});
    } else if (p[0] == 'v' && p[1] == 'n' && (p[2] == ' ' || p[2] == '\t')) {
      char *e;
      float x = std::strtof(p + 3, &e), y = std::strtof(e, &e), z = std::strtof(e, &e);
      D.nrm.insert(D.nrm.end(), {x, y, z});
    } else if (p[0] == 'v' && p[1] == 't' && (p[2] == ' ' || p[2] == '\t')) {
      char *e;
      float u = std::strtof(p + 3, &e), v = std::strtof(e, &e);
      D.uv.insert(D.uv.end(), {u, v});
    } else if (p[0] == 'f' && (p[1] == ' ' || p[1] == '\t')) {
      face.clear();
      const char *q = p + 2;
      const size_t nv = D.pos.size() / 3, nn = D.nrm.size() / 3, nt = D.uv.size() / 2;
      for (;;) {
        while (*q == ' ' || *q == '\t') ++q;
        if (*q == '\0' || *q == '\n' || *q == '\r' || *q == '#') break;
        char *e;
        FaceVertex fv{-1, -1, -1};
        long v = std::strtol(q, &e, 10);
        if (e == q || !resolve(v, nv, fv.v)) error("bad vertex index");
        q = e;
        if (*q == '/') {
          ++q;
          if (*q != '/') {
            long t = std::strtol(q, &e, 10);
            if (e == q || !resolve(t, nt, fv.t)) error("bad uv index");
            q = e;
          }
          if (*q == '/') {
            ++q;
            long n = std::strtol(q, &e, 10);
            if (e == q || !resolve(n, nn, fv.n)) error("bad normal index");
            q = e;
          }
        }
        if ((size_t)fv.v >= nv || (fv.t >= 0 && (size_t)fv.t >= nt) || (fv.n >= 0 && (size_t)fv.n >= nn))
          error("index out of range");
        face.push_back(fv);
      }
      if (face.size() < 3) continue;  // degenerate face: skipped, as tinyobjloader does
      auto emit = [&](const FaceVertex &a, const FaceVertex &b, const FaceVertex &c) {
        D.vi.insert(D.vi.end(), {a.v, b.v, c.v});
        D.ni.insert(D.ni.end(), {a.n, b.n, c.n});
        D.ti.insert(D.ti.end(), {a.t, b.t, c.t});
      };
      if (face.size() == 4) {
        auto P = [&](int k, int a) { return D.pos[3 * (size_t)face[k].v + a]; };
        float e02[3], e13[3];
        for (int a = 0; a < 3; ++a) {
          e02[a] = P(2, a) - P(0, a);
          e13[a] = P(3, a) - P(1, a);
        }
        float s02 = e02[0] * e02[0] + e02[1] * e02[1] + e02[2] * e02[2];
        float s13 = e13[0] * e13[0] + e13[1] * e13[1] + e13[2] * e13[2];
        if (s02 < s13) {
          emit(face[0], face[1], face[2]);
          emit(face[0], face[2], face[3]);
        } else {
          emit(face[0], face[1], face[3]);
          emit(face[1], face[2], face[3]);
        }
      } else {
        for (size_t k = 1; k + 1 < face.size(); ++k) emit(face[0], face[k], face[k + 1]);
      }
    }
  }
  std::fclose(f);
}

template <class T>
T *copy_out(const std::vector<T> &v) {
  if (v.empty()) return nullptr;
  T *p = static_cast<T *>(std::malloc(v.size() * sizeof(T)));
  if (!p) throw std::bad_alloc();
  std::memcpy(p, v.data(), v.size() * sizeof(T));
  return p;
}

}  // namespace
}  // namespace pt

using namespace pt;

extern "C" {

int pt_obj_load(const char *path, pt_mesh_desc *mesh) {
  if (!path || !mesh) return PT_ERR_INVALID;
  std::memset(mesh, 0, sizeof *mesh);
  try {
    ObjData D;
    parse(path, D);
    mesh->positions = copy_out(D.pos);
    mesh->n_positions = (int32_t)(D.pos.size() / 3);
    mesh->normals = copy_out(D.nrm);
    mesh->n_normals = (int32_t)(D.nrm.size() / 3);
    mesh->uvs = copy_out(D.uv);
    mesh->n_uvs = (int32_t)(D.uv.size() / 2);
    mesh->indices = copy_out(D.vi);
    mesh->normal_indices = copy_out(D.ni);
    mesh->uv_indices = copy_out(D.ti);
    mesh->n_triangles = (int32_t)(D.vi.size() / 3);
    mesh->material = -1;
    return PT_OK;
  } catch (const PtError &e) {
    pt_obj_free(mesh);
    return record_error(e.code, e.what());
  } catch (const std::bad_alloc &) {
    pt_obj_free(mesh);
    return record_error(PT_ERR_NOMEM, "host out of memory");
  }
}

int pt_obj_free(pt_mesh_desc *mesh) {
  if (!mesh) return PT_ERR_INVALID;
  std::free(const_cast<float *>(mesh->positions));
  std::free(const_cast<float *>(mesh->normals));
  std::free(const_cast<float *>(mesh->uvs));
  std::free(const_cast<int32_t *>(mesh->indices));
  std::free(const_cast<int32_t *>(mesh->normal_indices));
  std::free(const_cast<int32_t *>(mesh->uv_indices));
  std::memset(mesh, 0, sizeof *mesh);
  return PT_OK;
}

}  // extern "C"
