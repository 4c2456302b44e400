// pt_scene.cuh -- device layout of a flattened scene and of a render job.
//
// A scene is uploaded once (pt_scene_upload) and stays resident in HBM:
//   * BVH4 nodes, 128 B each (one L2 line): child boxes as SoA float4 rows,
//     child references and leaf item counts;
//   * leaf items, 48 B each (3 x float4), in leaf order: a triangle keeps
//     v0, e1 = v1 - v0, e2 = v2 - v0 exactly as the reference's hitTriangle
//     computes them (meshBVH.cpp:91-93), an AARectangle its plane and
//     extent, a sphere its centre and radius;
//   * per-primitive shading records (material, vertex normals);
//   * the material table, the light table (discovered like
//     lightDiscovery.hpp:5-81) and the environment map with its alias table.
#pragma once
#include "pt_common.cuh"

// Entries of the per-thread traversal stack (shared memory).  A BVH4 of
// depth D needs at most 3 * D + 1 entries; scene upload rejects deeper trees.
// Largest traversal stack, in entries per thread.  A scene's kernels get
// SceneView::stack_entries (3 * its BVH4 depth + 4) entries each, in dynamic
// shared memory: a shallow tree leaves more of the SM's on-chip memory to the
// L1 cache that serves the node loads.
#ifndef PT_STACK
#define PT_STACK 48
#endif

namespace pt {

enum ItemType : int32_t { ITEM_TRI = 0, ITEM_QUAD = 1, ITEM_SPHERE = 2, ITEM_CURVE = 3 };

struct alignas(128) Bvh4Node {
  float lo_x[4], hi_x[4];
  float lo_y[4], hi_y[4];
  float lo_z[4], hi_z[4];
  int32_t child[4];  // internal: node index; leaf: first item index
  int32_t count[4];  // internal: 0; leaf: number of items; empty slot: -1 --
                     // in the uploaded copy: each child's traversal reference
                     // (trav_ref), which the node visit reads as is
};
static_assert(sizeof(Bvh4Node) == 128, "BVH4 node must be one 128-byte line");

// Traversal references (a node's children on the device, the stack): a node
// index (>= 0; PT_INST_BIT: entering a moving object), a leaf
// ~(first_item << 3 | count - 1) (count <= 8), PT_FRAME_END (stack only) or
// PT_REF_EMPTY (an empty child slot; as the next reference: nothing pending).
#define PT_REF_EMPTY ((int32_t)0x80000001)
PT_HD int32_t leaf_ref(int32_t first, int32_t count) { return ~((first << 3) | (count - 1)); }
// A child's reference from its (child, count) pair.
PT_HD int32_t trav_ref(int32_t child, int32_t count) {
  return count < 0 ? PT_REF_EMPTY : count == 0 ? child : leaf_ref(child, count);
}

// Leaf item (48 B).  a.w / b.w carry the primitive id and the item type as
// integer bits.
struct alignas(16) Item {
  float a[4];
  float b[4];
  float c[4];
};

// Shading record of a primitive (64 B): everything the shade stage needs,
// so a hit costs one dependent 64-byte load.
//   triangle: n0..n2 vertex normals (if smooth), ng = cross(e1, e2)
//   rectangle: axis in flags bits 4-5
//   sphere: centre in n0
struct alignas(16) PrimShade {
  int32_t material;
  int32_t flags;     // bit0 smooth normals, bit1 FlipFace, bits 2-3 kind, bits 4-5 axis
  int32_t item;      // index of the primitive's leaf item
  int32_t light;     // index in the light table (-1: not a light)
  float n0[3], n1[3], n2[3];
  float ng[3];
};
static_assert(sizeof(PrimShade) == 64, "PrimShade must be 64 bytes");
#define PT_PRIM_SMOOTH 1
#define PT_PRIM_FLIP 2
// pt_object_desc.face != PT_FACE_AS_HIT: is_inside is fixed, to FACE_FRONT's value
#define PT_PRIM_FACE_FIXED 64
#define PT_PRIM_FACE_FRONT 128
#define PT_PRIM_KIND(f) (((f) >> 2) & 3)
#define PT_PRIM_AXIS(f) (((f) >> 4) & 3)
#define PT_PRIM_MOTION(f) ((f) >> 8)  // motion index + 1 (0: static)

// Material record: the C-ABI description plus constants derived once on the
// host (Disney lobe weights, hair v[p], s, sin/cos 2^k alpha ...).
struct alignas(16) MatRec {
  int32_t type;
  int32_t flags;
  float p[30];
  float d[32];  // derived
};

enum LightType : int32_t { LIGHT_QUAD = 0, LIGHT_SPHERE = 1, LIGHT_ENV = 2 };
struct alignas(16) LightRec {
  int32_t type;
  int32_t prim;     // primitive id of the emitter (quads/spheres)
  float intensity;
  float area;
  float v0[3];      // quad: vertices[0]; sphere: centre
  float radius;
  float e1[3];      // quad: vertices[1] - vertices[0]
  int32_t motion;   // motion index + 1 (0: static)
  float e2[3];      // quad: vertices[3] - vertices[0]
  float pad1;
  float normal[3];  // quad: normalize(cross(e1, e2))
  float pad2;
  float color[3];   // ConstantTexture colour
  int32_t texture;  // texture index + 1 of the emitter's colour (0: color)
  float v2[3];      // quad: vertices[2] (QuadLight::pdf_value's second triangle)
  float pad3;
};

struct EnvMap {
  const float4 *texels;   // width*height, [y][x], y = 0 bottom row
  const float *alias_prob;// width*height
  const int32_t *alias_idx;
  const float *pdf;       // per texel, discrete probability
  int32_t width, height;
  float intensity;
  int32_t present;
};

// A surface texture (pt_texture_desc), image texels as float4.
struct alignas(16) TexRec {
  int32_t kind, fractal, width, height;
  float c1[3], scale;
  float c2[3], pad;
  const float4 *texels;
  const float4 *pad_ptr;
};

// Texture-coordinate records (2 x float4 per primitive, only for scenes with
// textured materials): kind in the second record's z.
enum UvKind : int32_t { PT_UV_TRI = 1, PT_UV_PLANAR = 2, PT_UV_QUAD = 3, PT_UV_SPHERE = 4 };

struct SceneView {
  const Bvh4Node *nodes;
  const Item *items;
  const PrimShade *shade;
  const MatRec *materials;
  const LightRec *lights;
  int32_t n_lights;
  int32_t n_nodes;
  int32_t n_prims;
  EnvMap env;
  float bg[3];
  int32_t has_medium;
  float sigma_a[3], sigma_s[3], sigma_t_max, medium_g;
  // motion blur (extension): velocity per moving object; items, shading
  // records and lights of a moving object carry its index + 1
  const float4 *motion;
  const int32_t *node_motion;  // per BVH4 node: motion index + 1 of the moving object it roots
  int32_t has_motion;
  int32_t trav_cap;  // steps one ray's traversal may take before the device error flag is set
  int32_t stack_entries;  // traversal stack entries per thread: 3 * BVH4 depth + 4 (<= PT_STACK)
  const TexRec *textures;  // surface textures (materials' flags >> PT_MAT_TEXTURE_SHIFT)
  const float4 *prim_uv;   // per primitive texture-coordinate records (null: no textures)
  int32_t n_textures;
  const float4 *curves;    // per curve: (cp0, width0), (cp1, width1), (cp2, 0), (cp3, 0)
};

// Dynamic shared memory of a traversal kernel's stack: the scene's entries
// per thread, for `threads` threads (one column per thread).
inline size_t stack_bytes(const SceneView &S, int threads) {
  return (size_t)S.stack_entries * (size_t)threads * sizeof(int32_t);
}

// Child references of a BVH4 node entering a moving object's subtree carry
// PT_INST_BIT; the traversal then pushes PT_FRAME_END (never a leaf
// reference: items < 2^28 - 8) and continues in the object's frame until it
// pops it.
#define PT_INST_BIT (1 << 30)
// Default bound on the steps of one ray's traversal (SceneView::trav_cap).
#define PT_TRAVERSAL_CAP (1 << 22)
#define PT_FRAME_END ((int32_t)0x80000000)

// Camera constants of PerspectiveCamera (camera.cpp:7-35).
struct CameraView {
  float position[3];
  float bottom_left[3];
  float horizontal[3];
  float vertical[3];
  float h_vec[3];
  float v_vec[3];
  float lens_radius;
};

struct JobView {
  int32_t width, height;  // the rendered window (the film)
  int32_t crop_x, crop_y; // window origin in the frame
  int32_t full_w, full_h; // the frame: camera and sample streams
  int32_t spp;            // spp_x * spp_y
  int32_t spp_begin;      // first grid sample of this render
  int32_t spp_x, spp_y;
  int32_t max_depth;
  int32_t rr_start;
  int32_t estimator;
  int32_t sampler;
  int32_t env_sampling;
  int32_t light_nx, light_ny;
  uint32_t seed;
  float shutter;          // motion blur: a path's time is shutter * u
  CameraView cam;
  const float2 *offsets;  // per grid sample k: jittered pixel offset
  const float *rays;      // given primary rays (origin, direction per film pixel), or null: the camera's
};

}  // namespace pt
