// pt_texture.cuh -- surface textures (ColorVariant, include/texture/texture.hpp:
// 134-163) and the texture coordinates of a hit (HitRecord::texCoords).
//
//   CheckerTexture::getTexelColor    texture.cpp:164-181
//   NoiseTexture::getTexelColor      texture.cpp:183-193 over
//     gl::fractal_perlin_2D / perlin_noise_2D   utils/pattern.hpp:72-114
//   ImageTexture::getTexelColor      texture.cpp:95-149 (bilinear)
//   texCoords: triangles  meshBVH.cpp:134-138 (barycentric uv), planar
//     fallback triangleMesh.cpp:39-51; rectangles primitive.cpp:55-57;
//     spheres primitive.hpp:158-164
#pragma once
#include "../../include/pathtracer_gb300.h"
#include "pt_scene.cuh"

namespace pt {

// Ken Perlin's permutation of 0..255 ("Improving Noise", SIGGRAPH 2002,
// reference implementation), the table pattern.hpp:8 holds twice.
static __device__ const unsigned char c_perlin_perm[256] = {
    151, 160, 137, 91,  90,  15,  131, 13,  201, 95,  96,  53,  194, 233, 7,   225, 140, 36,  103, 30,  69,  142,
    8,   99,  37,  240, 21,  10,  23,  190, 6,   148, 247, 120, 234, 75,  0,   26,  197, 62,  94,  252, 219, 203,
    117, 35,  11,  32,  57,  177, 33,  88,  237, 149, 56,  87,  174, 20,  125, 136, 171, 168, 68,  175, 74,  165,
    71,  134, 139, 48,  27,  166, 77,  146, 158, 231, 83,  111, 229, 122, 60,  211, 133, 230, 220, 105, 92,  41,
    55,  46,  245, 40,  244, 102, 143, 54,  65,  25,  63,  161, 1,   216, 80,  73,  209, 76,  132, 187, 208, 89,
    18,  169, 200, 196, 135, 130, 116, 188, 159, 86,  164, 100, 109, 198, 173, 186, 3,   64,  52,  217, 226, 250,
    124, 123, 5,   202, 38,  147, 118, 126, 255, 82,  85,  212, 207, 206, 59,  227, 47,  16,  58,  17,  182, 189,
    28,  42,  223, 183, 170, 213, 119, 248, 152, 2,   44,  154, 163, 70,  221, 153, 101, 155, 167, 43,  172, 9,
    129, 22,  39,  253, 19,  98,  108, 110, 79,  113, 224, 232, 178, 185, 112, 104, 218, 246, 97,  228, 251, 34,
    242, 193, 238, 210, 144, 12,  191, 179, 162, 241, 81,  51,  145, 235, 249, 14,  239, 107, 49,  192, 214, 31,
    181, 199, 106, 157, 184, 84,  204, 176, 115, 121, 50,  45,  127, 4,   150, 254, 138, 236, 205, 93,  222, 114,
    67,  29,  24,  72,  243, 141, 128, 195, 78,  66,  215, 61,  156, 180};

__device__ __forceinline__ int perlin_p(int i) { return c_perlin_perm[i & 255]; }

// gradient of a lattice corner: the eight directions of pattern.hpp:43-66
__device__ __forceinline__ float perlin_grad(int hash, float x, float y) {
  switch (hash & 7) {
  case 0: return x + y;
  case 1: return -x + y;
  case 2: return x - y;
  case 3: return -x - y;
  case 4: return x;
  case 5: return -x;
  case 6: return y;
  default: return -y;
  }
}

// perlin_noise_2D (pattern.hpp:72-98) with its lattice of period 256:
// smoothstep 6t^5 - 15t^4 + 10t^3, bilinear blend of corner gradients,
// mapped to [0, 1].
__device__ __forceinline__ float perlin_2d(float ux, float uy) {
  float x = fmodf(ux, 256.f), y = fmodf(uy, 256.f);
  const int X = (int)floorf(x) & 255, Y = (int)floorf(y) & 255;
  x = x - floorf(x);
  y = y - floorf(y);
  auto smooth = [](float t) {
    t = fminf(fmaxf(t, 0.f), 1.f);
    return t * t * t * (t * (t * 6.f - 15.f) + 10.f);
  };
  const float u = smooth(x), v = smooth(y);
  const int X1 = (X + 1) % 256, Y1 = (Y + 1) % 256;
  const int aa = perlin_p(perlin_p(X) + Y), ab = perlin_p(perlin_p(X) + Y1);
  const int ba = perlin_p(perlin_p(X1) + Y), bb = perlin_p(perlin_p(X1) + Y1);
  auto lerp = [](float a, float b, float t) { return a + t * (b - a); };
  const float x1 = lerp(perlin_grad(aa, x, y), perlin_grad(ba, x - 1.f, y), u);
  const float x2 = lerp(perlin_grad(ab, x, y - 1.f), perlin_grad(bb, x - 1.f, y - 1.f), u);
  return (lerp(x1, x2, v) + 1.f) * 0.5f;
}

// fractal_perlin_2D (pattern.hpp:100-114): octaves of halving amplitude and
// doubling frequency, |sum| clamped to [0, 1].
__device__ __forceinline__ float fractal_perlin_2d(float x, float y, int octaves) {
  float total = 0.f, amp = 1.f, freq = 1.f;
  for (int i = 0; i < octaves && i < 32; ++i) {
    total += amp * perlin_2d(x * freq, y * freq);
    amp *= 0.5f;
    freq *= 2.f;
  }
  return fminf(fmaxf(fabsf(total), 0.f), 1.f);
}

// ImageTexture::getTexelColor, bilinear (texture.cpp:112-143): the cell
// index is clamped to width-2 / height-2 after the fraction is taken.
__device__ __forceinline__ V3 image_bilinear(const float4 *texels, int W, int H, float u, float v) {
  float fu = u * W, fv = v * H;
  unsigned x = (unsigned)fu, y = (unsigned)fv;
  float x1 = fu - (float)x, y1 = fv - (float)y;
  x = min(x, (unsigned)(W - 2));
  y = min(y, (unsigned)(H - 2));
  float x2 = 1.0f - x1, y2 = 1.0f - y1;
  float4 c1 = __ldg(texels + y * W + x), c2 = __ldg(texels + y * W + x + 1);
  float4 c3 = __ldg(texels + (y + 1) * W + x), c4 = __ldg(texels + (y + 1) * W + x + 1);
  V3 c12 = v3(c1.x, c1.y, c1.z) * x2 + v3(c2.x, c2.y, c2.z) * x1;
  V3 c34 = v3(c3.x, c3.y, c3.z) * x2 + v3(c4.x, c4.y, c4.z) * x1;
  return c12 * y2 + c34 * y1;
}

__device__ inline V3 tex_eval(const TexRec &T, float u, float v) {
  switch (T.kind) {
  case PT_TEX_CHECKER: {
    const float s = sinf(u * T.scale) * sinf(v * T.scale);
    return s < 0.f ? v3(T.c1[0], T.c1[1], T.c1[2]) : v3(T.c2[0], T.c2[1], T.c2[2]);
  }
  case PT_TEX_NOISE: return v3(fractal_perlin_2d(u * T.scale, v * T.scale, T.fractal));
  case PT_TEX_IMAGE: return image_bilinear(T.texels, T.width, T.height, u, v);
  default: return v3(T.c1[0], T.c1[1], T.c1[2]);
  }
}

// Texture coordinates of a surface hit.  p: the hit point, n: its shading
// normal, (bu, bv): the triangle barycentrics of the hit.
__device__ inline float2 surface_uv(const SceneView &S, int prim, V3 p, V3 n, float bu, float bv) {
  const float4 *r = S.prim_uv + 2 * (size_t)prim;
  const float4 a = __ldg(r), b = __ldg(r + 1);
  switch ((int)b.z) {
  case PT_UV_TRI: {  // (1 - u - v) uv0 + u uv1 + v uv2
    const float w = 1.f - bu - bv;
    return make_float2(w * a.x + bu * a.z + bv * b.x, w * a.y + bu * a.w + bv * b.y);
  }
  case PT_UV_PLANAR: {  // axes from |n|, position in the mesh's box, clamped
    const float mn[3] = {a.x, a.y, a.z}, mx[3] = {a.w, b.x, b.y};
    const V3 an = v3(fabsf(n.x), fabsf(n.y), fabsf(n.z));
    const int au = (an.x > an.y && an.x > an.z) ? 1 : 0;
    const int av = (au == 1) ? 2 : (an.y > an.z ? 2 : 1);
    const float pc[3] = {p.x, p.y, p.z};
    const float u = (pc[au] - mn[au]) / (mx[au] - mn[au]), v = (pc[av] - mn[av]) / (mx[av] - mn[av]);
    return make_float2(fminf(fmaxf(u, 0.f), 1.f), fminf(fmaxf(v, 0.f), 1.f));
  }
  case PT_UV_QUAD: {  // (d0 - d0_min) / (d0_max - d0_min), (d1 - d1_min) / (d1_max - d1_min)
    const int axis = (int)b.w;
    const float pc[3] = {p.x, p.y, p.z};
    const float d0 = pc[axis == 0 ? 1 : 0], d1 = pc[axis == 2 ? 1 : 2];
    return make_float2((d0 - a.x) / (a.y - a.x), (d1 - a.z) / (a.w - a.z));
  }
  default: {  // sphere: longitude / latitude, u shifted by 0.75
    const V3 q = normalize(p - v3(a.x, a.y, a.z));
    const float phi = atan2f(q.z, q.x), theta = asinf(fminf(fmaxf(q.y, -1.f), 1.f));
    float u = 1.f - (phi + (float)PT_PI) / (2.f * (float)PT_PI);
    const float v = (theta + (float)(PT_PI / 2)) / (float)PT_PI;
    u = fmodf(u + 0.75f, 1.0f);
    return make_float2(u, v);
  }
  }
}

}  // namespace pt
