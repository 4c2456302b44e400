// pt_wave.cuh -- device code of the wavefront stages whose work depends on
// the job of each path: camera, closest-hit traversal (medium free flight),
// the paired closest + shadow traversal of small waves, and shading.  Included by pt_kernels.cu (single-job waves, MJ = false: the
// job is a kernel argument) and by pt_kernels_multi.cu (merged waves of many
// jobs, MJ = true: a job table in HBM and a job index per path); the two
// translation units compile in parallel.  The estimator restates getRayColor
// (maxdepth_nee.hpp:9-256) iteratively; see k_shade for the correspondence.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include "pt_bsdf.cuh"
#include "pt_trace.cuh"
#include "pt_kernels.h"
#include "pt_texture.cuh"

namespace pt {

// Halton tables in constant memory, one copy per translation unit (each
// unit's upload function fills its own).
static __constant__ HaltonTables c_halton;

// ---------------------------------------------------------------- helpers
// Queue records are read through the read-only data cache (ld.global.nc):
// a per-stage kernel never reads records it wrote itself.  The persistent
// form runs all stages in one kernel, so its later stages read what earlier
// ones wrote; it defines PT_QUEUE_LOADS_COHERENT and reads them from L2
// (ld.global.cg).
#ifdef PT_QUEUE_LOADS_COHERENT
__device__ __forceinline__ float4 ld4(const float4 *p) { return __ldcg(p); }
#else
__device__ __forceinline__ float4 ld4(const float4 *p) { return __ldg(p); }
#endif

// Warp-aggregated slot allocation in a queue counter.
__device__ __forceinline__ int warp_alloc(int *counter, bool want) {
  unsigned mask = __ballot_sync(0xffffffffu, want);
  if (!mask) return -1;
  int lane = threadIdx.x & 31;
  int leader = __ffs(mask) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader);
  return want ? base + __popc(mask & ((1u << lane) - 1u)) : -1;
}
__device__ __forceinline__ void warp_count(unsigned long long *counter, int n) {
  // sums n over the warp, one atomic per warp
  for (int off = 16; off > 0; off >>= 1) n += __shfl_down_sync(0xffffffffu, n, off);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(counter, (unsigned long long)n);
}

__device__ __forceinline__ float sampler_dim(const DeviceJob &J, int dim, uint32_t index,
                                             uint64_t key, int pixel, int k) {
  switch (J.job.sampler) {
  case PT_SAMPLER_HALTON_NONE: return radical_inverse(c_halton, dim, index);
  case PT_SAMPLER_HALTON_PERMUTE: return permuted_radical_inverse(c_halton, J.perm, dim, index);
  case PT_SAMPLER_STRATIFIED: {
    // Jittered strata over the pixel's spp samples, permuted per (pixel,
    // dimension) with the reference's permutationElement.
    const uint32_t S = (uint32_t)J.job.spp;
    uint32_t h = (uint32_t)mix_bits(((uint64_t)pixel << 20) ^ ((uint64_t)dim << 8) ^ J.job.seed);
    uint32_t stratum = permutation_element((uint32_t)k, S, h);
    float jit = rand01(key, 4096u + (uint32_t)dim);
    return fminf(((float)stratum + jit) / (float)S, 0x1.fffffep-1f);
  }
  default: return owen_radical_inverse(c_halton, dim, index);
  }
}

// HDRITexture::getTexelColor(dir) (texture.hpp:105-115) with
// ImageTexture's bilinear lookup (texture.cpp:112-143, including its clamp
// of the cell index to width-2 / height-2 after the fraction is taken).
__device__ inline V3 env_lookup(const EnvMap &E, V3 dir) {
  V3 dn = normalize(dir);
  float theta = acosf(-dn.y);
  float phi = atan2f(-dn.z, dn.x) + (float)PT_PI;
  float u = phi / (2.0f * (float)PT_PI), v = theta / (float)PT_PI;
  const int W = E.width, H = E.height;
  float fu = u * W, fv = v * H;
  unsigned x = (unsigned)fu, y = (unsigned)fv;
  float x1 = fu - (float)x, y1 = fv - (float)y;
  x = min(x, (unsigned)(W - 2));
  y = min(y, (unsigned)(H - 2));
  float x2 = 1.0f - x1, y2 = 1.0f - y1;
  float4 c1 = __ldg(E.texels + y * W + x), c2 = __ldg(E.texels + y * W + x + 1);
  float4 c3 = __ldg(E.texels + (y + 1) * W + x), c4 = __ldg(E.texels + (y + 1) * W + x + 1);
  V3 c12 = v3(c1.x, c1.y, c1.z) * x2 + v3(c2.x, c2.y, c2.z) * x1;
  V3 c34 = v3(c3.x, c3.y, c3.z) * x2 + v3(c4.x, c4.y, c4.z) * x1;
  return (c12 * y2 + c34 * y1) * E.intensity;
}

// Luminance alias-table sampling of the environment (extension).
__device__ inline V3 env_alias_sample(const EnvMap &E, float u0, float u1, float u2, float &pdf) {
  const int N = E.width * E.height;
  float f = u0 * N;
  int i = min((int)f, N - 1);
  float r = f - (float)i;
  int cell = (r < __ldg(E.alias_prob + i)) ? i : __ldg(E.alias_idx + i);
  int cx = cell % E.width, cy = cell / E.width;
  float u = (cx + u1) / E.width, v = (cy + u2) / E.height;
  float st, ct, sp, cp;  // theta = pi v, phi = 2 pi u
  sincospi_(v, &st, &ct);
  sincospi_(2.f * u, &sp, &cp);
  V3 d = v3(-st * cp, -ct, st * sp);
  pdf = (st > 0.f) ? __ldg(E.pdf + cell) * (float)N / (2.f * (float)(PT_PI * PT_PI) * st) : 0.f;
  return d;
}
__device__ inline float env_alias_pdf(const EnvMap &E, V3 dir) {
  V3 dn = normalize(dir);
  float theta = acosf(fminf(fmaxf(-dn.y, -1.f), 1.f));
  float phi = atan2f(-dn.z, dn.x) + (float)PT_PI;
  float u = phi / (2.f * (float)PT_PI), v = theta / (float)PT_PI;
  int cx = min((int)(u * E.width), E.width - 1), cy = min((int)(v * E.height), E.height - 1);
  float st = sinf(theta);
  if (st <= 0.f) return 0.f;
  const int N = E.width * E.height;
  return __ldg(E.pdf + cy * E.width + cx) * (float)N / (2.f * (float)(PT_PI * PT_PI) * st);
}

// Surface record at a hit (HitRecord after intersect + set_normal).
struct Surf {
  V3 p;       // position
  V3 n;       // shading normal, turned towards the ray
  V3 ng;      // un-flipped geometric/analytic normal (for emitter-side tests)
  bool front; // HitRecord::is_inside (front-face flag; FlipFace toggles it)
  int mat;
  int light;
  int motion;  // motion index + 1 of the primitive (0: static)
  bool has_tan;  // a curve hit: HitRecord::hair_tangent is set
  V3 tan;        // the curve tangent (HairMarschner's frame)
};

// Position of a moving object's point at `time` (rounded, never fused).
__device__ __forceinline__ V3 moved_point(const SceneView &S, int motion, V3 p, float time) {
  const float4 v = __ldg(S.motion + (motion - 1));
  return v3(xadd(p.x, xmul(v.x, time)), xadd(p.y, xmul(v.y, time)), xadd(p.z, xmul(v.z, time)));
}

__device__ inline Surf surface_at(const SceneView &S, V3 o, V3 d, const HitRec &h, float time) {
  Surf s;
  const float4 *pp = reinterpret_cast<const float4 *>(S.shade + h.prim);
  const float4 q0 = __ldg(pp), q1 = __ldg(pp + 1), q2 = __ldg(pp + 2), q3 = __ldg(pp + 3);
  PrimShade ps;
  ps.material = __float_as_int(q0.x);
  ps.flags = __float_as_int(q0.y);
  ps.light = __float_as_int(q0.w);
  ps.n0[0] = q1.x; ps.n0[1] = q1.y; ps.n0[2] = q1.z;
  ps.n1[0] = q1.w; ps.n1[1] = q2.x; ps.n1[2] = q2.y;
  ps.n2[0] = q2.z; ps.n2[1] = q2.w; ps.n2[2] = q3.x;
  ps.ng[0] = q3.y; ps.ng[1] = q3.z; ps.ng[2] = q3.w;
  s.mat = ps.material;
  s.light = ps.light;
  s.motion = PT_PRIM_MOTION(ps.flags);
  s.has_tan = false;
  s.tan = v3(0.f);
  const int type = PT_PRIM_KIND(ps.flags);
  V3 n;
  if (type == ITEM_TRI) {
    // MeshBVHNode::hitTriangle (meshBVH.cpp:112-131) then TriangleMesh::intersect
    V3 Ng = v3(ps.ng[0], ps.ng[1], ps.ng[2]);
    if (ps.flags & PT_PRIM_SMOOTH) {
      float w = 1.f - h.u - h.v;
      n = normalize(w * v3(ps.n0[0], ps.n0[1], ps.n0[2]) + h.u * v3(ps.n1[0], ps.n1[1], ps.n1[2]) +
                    h.v * v3(ps.n2[0], ps.n2[1], ps.n2[2]));
    } else {
      n = normalize(Ng);
    }
    if (dot(n, Ng) < 0.f) n = -n;
    s.p = xat(o, d, h.t);
  } else if (type == ITEM_QUAD) {
    const int axis = PT_PRIM_AXIS(ps.flags);
    n = v3(axis == 0 ? 1.f : 0.f, axis == 1 ? 1.f : 0.f, axis == 2 ? 1.f : 0.f);
    s.p = xat(o, xnormalize(d), h.t);
  } else if (type == ITEM_CURVE) {
    // Curve::intersect's hit record (curve.hpp:104-121): tangent from the two
    // Bezier derivatives at the segment's ends, normal from the segment's
    // axis to the hit point, in the curve's frame (h.u segment, h.v
    // fraction of its length)
    s.p = xat(o, d, h.t);
    const float4 *cp = S.curves + 4 * (size_t)f2u(ps.n0[0]);
    const V3 hp = s.motion ? moved_point(S, s.motion, s.p, -time) : s.p;
    const int i = (int)h.u;
    const float u0 = float(i) / 8, u1 = float(i + 1) / 8;
    const V3 pa = bezier_point(cp, u0), pb = bezier_point(cp, u1);
    const V3 ab = pb - pa;
    const V3 axis = ab / length(ab);
    const float proj = dot(hp - pa, axis);
    const V3 d0 = bezier_tangent(cp, u0), d1 = bezier_tangent(cp, u1);
    s.tan = normalize(d0 + (d1 - d0) * h.v);
    s.has_tan = true;
    const V3 rv = hp - (pa + axis * proj);
    n = normalize(rv - dot(rv, s.tan) * s.tan);
  } else {
    V3 dn = xnormalize(d);
    s.p = xat(o, dn, h.t);
    V3 c = v3(ps.n0[0], ps.n0[1], ps.n0[2]);
    if (PT_PRIM_MOTION(ps.flags)) c = moved_point(S, PT_PRIM_MOTION(ps.flags), c, time);
    n = normalize(s.p - c);
  }
  s.ng = n;
  s.front = dot(d, n) < 0.f;  // set_normal (materialBase.hpp:48-52)
  s.n = s.front ? n : -n;
  if (ps.flags & PT_PRIM_FLIP) s.front = !s.front;
  if (ps.flags & PT_PRIM_FACE_FIXED) s.front = (ps.flags & PT_PRIM_FACE_FRONT) != 0;
  return s;
}

// ---------------------------------------------------------- wavefront
// Path identity inside a wave: slot -> global path g = g0 + slot,
// pixel q = g % npix, grid sample k = spp_begin + g / npix.
struct PathId {
  int q, i, j, k;  // film pixel, frame column / row, grid sample
  int pix;         // frame pixel index j * full_w + i
  uint32_t halton_index;
  uint64_t key;
};
__device__ __forceinline__ PathId path_id(const DeviceJob &J, long long g) {
  PathId P;
  const long long npix = (long long)J.job.width * J.job.height;
  P.q = (int)(g % npix);
  P.k = J.job.spp_begin + (int)(g / npix);
  P.i = J.job.crop_x + P.q % J.job.width;
  P.j = J.job.crop_y + P.q / J.job.width;
  P.pix = P.j * J.job.full_w + P.i;
  // single-thread order of renderManager.hpp:99-115: i outer, j, k inner
  uint64_t lin = ((uint64_t)P.i * J.job.full_h + P.j) * (uint64_t)J.job.spp + P.k;
  P.halton_index = (uint32_t)(lin + 1u);
  P.key = path_key(J.job.seed, lin);
  return P;
}

// The job of a path.  Single-job waves (MJ = false): the kernel's DeviceJob
// and the path's index g0 + slot.  Merged waves of many jobs (MJ = true):
// the job index k_camera stored for the path's slot and the path's index
// within its job.
template <bool MJ>
__device__ __forceinline__ const DeviceJob &path_job(const DeviceJob &J, const JobTable &T, const Queues &Q,
                                                     int slot, long long g0, long long &g) {
  if (!MJ) {
    g = g0 + slot;
    return J;
  }
  const int k = Q.job[slot];
  g = g0 + slot - __ldg(T.start + k);
  return T.jobs[k];
}

// k_camera: PerspectiveCamera::generateRay (camera.cpp:42-56) for every path
// of the wave; the direction is normalised (the one documented deviation:
// it makes hit distances of every primitive kind comparable).
// Merged waves: the path's job by binary search of the jobs' first merged
// indices (start[0] = 0 <= g < start[n]), stored for the later stages.
template <bool MJ>
__device__ __forceinline__ void camera_body(const DeviceJob &J0, const JobTable &T, const Queues &Q, long long g0,
                                            int n) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    long long g = g0 + s;
    int jk = 0;
    if (MJ) {
      int lo = 0, hi = T.n;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(T.start + mid) <= g) lo = mid;
        else hi = mid;
      }
      jk = lo;
      Q.job[s] = jk;
      g -= __ldg(T.start + jk);
    }
    const DeviceJob &J = MJ ? T.jobs[jk] : J0;
    PathId P = path_id(J, g);
    V3 ps, dir;
    if (!MJ && J.job.rays) {
      // pt_ray_color: the given primary ray of the path's film pixel
      const float *rr = J.job.rays + 6 * (size_t)P.q;
      ps = v3(rr[0], rr[1], rr[2]);
      dir = normalize(v3(rr[3], rr[4], rr[5]));
    } else {
      const CameraView &C = J.job.cam;
      float2 off = __ldg(J.job.offsets + P.k);
      float u = ((float)P.i + off.x) / (float)J.job.full_w;
      float v = ((float)P.j + off.y) / (float)J.job.full_h;
      const float r = C.lens_radius;
      float lx = -r + (r - -r) * rand01(P.key, 1u);
      float ly = -r + (r - -r) * rand01(P.key, 2u);
      V3 hv = v3(C.h_vec[0], C.h_vec[1], C.h_vec[2]), vv = v3(C.v_vec[0], C.v_vec[1], C.v_vec[2]);
      ps = v3(C.position[0], C.position[1], C.position[2]) + (hv * lx + vv * ly);
      dir = v3(C.bottom_left[0], C.bottom_left[1], C.bottom_left[2]) +
            u * v3(C.horizontal[0], C.horizontal[1], C.horizontal[2]) +
            v * v3(C.vertical[0], C.vertical[1], C.vertical[2]) - ps;
      dir = normalize(dir);
    }
    // motion blur: the path's time, used by every ray of the path
    const float time = J.job.shutter > 0.f ? J.job.shutter * rand01(P.key, 3u) : 0.f;
    Q.ray_o[0][s] = make_float4(ps.x, ps.y, ps.z, __int_as_float(s));
    Q.ray_d[0][s] = make_float4(dir.x, dir.y, dir.z, time);
    Q.beta[s] = make_float4(1.f, 1.f, 1.f, -1.f);  // w < 0: previous vertex delta / camera
    Q.L[s] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    Q.counts[0] = n;
    atomicAdd(&Q.stats[0], (unsigned long long)n);
  }
}
template <bool MJ>
__global__ void k_camera(DeviceJob J0, JobTable T, Queues Q, long long g0, int n) {
  camera_body<MJ>(J0, T, Q, g0, n);
}

// Persistent traversal warps with dynamic ray fetch (Aila and Laine,
// "Understanding the efficiency of ray traversal on GPUs", HPG 2009, and the
// 2012 addendum): each lane walks its ray one step at a time, and as soon as
// PT_FETCH_IDLE lanes of a warp have finished, the warp claims that many new
// rays from the queue with one atomic.  Incoherent rays of very different
// lengths then no longer hold a warp until its longest ray ends.
#define PT_FETCH_IDLE 16
// Shadow rays refill sooner (8 idle lanes): an any-hit ray's length varies
// more (an early blocker ends it), and on the rough-glass workload the
// shadow launches ran 274 -> 253 ms over 8 steps with 8 instead of 16,
// while closest-hit launches on the Cornell box were slower with 8.
#define PT_FETCH_IDLE_SHADOW 8

__device__ __forceinline__ unsigned lanemask_lt() {
  return (1u << (threadIdx.x & 31)) - 1u;
}

// k_trace_closest: the RayQueue through the BVH.  In a participating medium
// the free-flight distance of the segment is drawn when the ray is fetched
// (dimension dpb*bounce) and used as tmax: a segment that reaches it without
// a surface hit is a medium event (prim = PT_HIT_MEDIUM, t = free-flight
// distance).  That is the same decision as comparing the distance with the
// closest hit.
template <bool MJ, bool CURVES>
__device__ __forceinline__ void trace_closest_body(const SceneView &S, const DeviceJob &J, const JobTable &T,
                                                   const Queues &Q, int qsel, int bounce, long long g0,
                                                   int32_t *stack) {
  const int n = Q.counts[qsel];
  int *fetch = Q.counts + 4;
  const int lane = threadIdx.x & 31;
  int32_t *my_stack = stack + threadIdx.x;
  TravRay R;
  bool active = false, exhausted = false;
  int ray = 0, rays = 0;
  float t_s = INFINITY;
  for (;;) {
    unsigned idle = __ballot_sync(0xffffffffu, !active);
    if (!exhausted && __popc(idle) >= PT_FETCH_IDLE) {
      const int k = __popc(idle);
      int base = 0;
      if (lane == 0) base = atomicAdd(fetch, k);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + k >= n) exhausted = true;
      if (!active) {
        const int r = base + __popc(idle & lanemask_lt());
        if (r < n) {
          float4 ro = ld4(Q.ray_o[qsel] + r), rd = ld4(Q.ray_d[qsel] + r);
          float tmax = 1e5f;
          t_s = INFINITY;
          if (S.has_medium) {
            long long g;
            const DeviceJob &Jp = path_job<MJ>(J, T, Q, __float_as_int(ro.w), g0, g);
            if (bounce < Jp.job.max_depth) {
              PathId P = path_id(Jp, g);
              float uf = sampler_dim(Jp, 4 * bounce, P.halton_index, P.key, P.pix, P.k);
              t_s = -logf(1.f - uf) / S.sigma_t_max;
              tmax = fminf(tmax, t_s);
            }
          }
          trav_init(R, v3(ro.x, ro.y, ro.z), v3(rd.x, rd.y, rd.z), 1e-4f, tmax, rd.w);
          ray = r;
          active = true;
          ++rays;
        }
      }
      idle = __ballot_sync(0xffffffffu, !active);
    }
    if (idle == 0xffffffffu) {
      if (exhausted) break;
      continue;
    }
    const bool lt = warp_leaf_turn(active, R.ref);
    if (lane_turn(active, R.ref, lt) && trav_step<false, CURVES>(S, R, my_stack, blockDim.x, Q.err)) {
      const bool hit = R.found;
      int prim = hit ? R.hit.prim : (t_s < 1e5f ? PT_HIT_MEDIUM : -1);
      float t = hit ? R.hit.t : (prim == PT_HIT_MEDIUM ? t_s : FLT_MAX);
      Q.hit[ray] = make_float4(t, __int_as_float(prim), R.hit.u, R.hit.v);
      active = false;
    }
  }
  warp_count(&Q.stats[2], rays);
}
template <bool MJ, bool CURVES>
__global__ void __launch_bounds__(128) k_trace_closest(SceneView S, DeviceJob J, JobTable T, Queues Q, int qsel,
                                                       int bounce, long long g0) {
  extern __shared__ int32_t stack[];  // S.stack_entries x 128
  trace_closest_body<MJ, CURVES>(S, J, T, Q, qsel, bounce, g0, stack);
}

// k_trace_pair: the closest-hit rays of bounce `bounce` (RayQueue qsel)
// and the shadow rays of the bounce before it (ShadowQueue, LN light
// samples per vertex) in ONE persistent launch.  Both queues come from the
// same shade pass and neither reads the other's output, so one index space
// [0, n_closest + n_shadow) is fetched with one counter (Q.counts[4]):
// closest rays first (the sort and shade passes wait on them), then shadow
// rays.  A bounce then has one sparse tail instead of two.  Per ray the work
// is exactly k_trace_closest's or k_trace_shadow's, so results are the same;
// the shadow terms are still added (k_shadow_resolve) before the next shade
// pass, in the same order.
template <bool MJ, bool CURVES>
__device__ __forceinline__ void trace_pair_body(const SceneView &S, const DeviceJob &J, const JobTable &T,
                                                const Queues &Q, int qsel, int bounce, long long g0, int LN,
                                                int32_t *stack) {
  const int nc = Q.counts[qsel];
  const int n = nc + Q.counts[2] * LN;
  int *fetch = Q.counts + 4;
  const int lane = threadIdx.x & 31;
  int32_t *my_stack = stack + threadIdx.x;
  TravRay R;
  bool active = false, exhausted = false, shadow = false;
  size_t slot = 0;  // closest: ray index; shadow: ShadowQueue slot
  int crays = 0, srays = 0;
  float t_s = INFINITY;
  for (;;) {
    unsigned idle = __ballot_sync(0xffffffffu, !active);
    if (!exhausted && __popc(idle) >= PT_FETCH_IDLE) {
      const int k = __popc(idle);
      int base = 0;
      if (lane == 0) base = atomicAdd(fetch, k);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + k >= n) exhausted = true;
      if (!active) {
        const int r = base + __popc(idle & lanemask_lt());
        if (r < nc) {
          float4 ro = ld4(Q.ray_o[qsel] + r), rd = ld4(Q.ray_d[qsel] + r);
          float tmax = 1e5f;
          t_s = INFINITY;
          if (S.has_medium) {
            long long g;
            const DeviceJob &Jp = path_job<MJ>(J, T, Q, __float_as_int(ro.w), g0, g);
            if (bounce < Jp.job.max_depth) {
              PathId P = path_id(Jp, g);
              float uf = sampler_dim(Jp, 4 * bounce, P.halton_index, P.key, P.pix, P.k);
              t_s = -logf(1.f - uf) / S.sigma_t_max;
              tmax = fminf(tmax, t_s);
            }
          }
          trav_init(R, v3(ro.x, ro.y, ro.z), v3(rd.x, rd.y, rd.z), 1e-4f, tmax, rd.w);
          slot = (size_t)r;
          shadow = false;
          active = true;
          ++crays;
        } else if (r < n) {
          const int v = (r - nc) / LN, ls = (r - nc) - v * LN;
          slot = (size_t)ls * Q.cap + v;
          float4 dd = ld4(Q.sh_d + slot);
          if (dd.w >= 0.f) {
            float4 so = ld4(Q.sh_o + v);
            const float time = S.has_motion ? ld4(Q.sh_c + slot).w : 0.f;
            trav_init(R, v3(so.x, so.y, so.z), v3(dd.x, dd.y, dd.z), 0.001f, dd.w, time);
            shadow = true;
            active = true;
            ++srays;
          }
        }
      }
      idle = __ballot_sync(0xffffffffu, !active);
    }
    if (idle == 0xffffffffu) {
      if (exhausted) break;
      continue;
    }
    const bool lt = warp_leaf_turn(active, R.ref);
    const bool turn = lane_turn(active, R.ref, lt);
    if (turn && !shadow && trav_step<false, CURVES>(S, R, my_stack, blockDim.x, Q.err)) {
      const bool hit = R.found;
      int prim = hit ? R.hit.prim : (t_s < 1e5f ? PT_HIT_MEDIUM : -1);
      float t = hit ? R.hit.t : (prim == PT_HIT_MEDIUM ? t_s : FLT_MAX);
      Q.hit[slot] = make_float4(t, __int_as_float(prim), R.hit.u, R.hit.v);
      active = false;
    }
    if (turn && shadow && trav_step<true, CURVES>(S, R, my_stack, blockDim.x, Q.err)) {
      Q.sh_vis[slot] = R.found ? 0 : 1;
      active = false;
    }
  }
  warp_count(&Q.stats[2], crays);
  warp_count(&Q.stats[3], srays);
}
template <bool MJ, bool CURVES>
__global__ void __launch_bounds__(128, 7) k_trace_pair(SceneView S, DeviceJob J, JobTable T, Queues Q, int qsel,
                                                    int bounce, long long g0, int LN) {
  extern __shared__ int32_t stack[];  // S.stack_entries x 128
  trace_pair_body<MJ, CURVES>(S, J, T, Q, qsel, bounce, g0, LN, stack);
}

// The hit point in its object's rest frame (texture coordinates of moving
// objects follow the object).
__device__ __forceinline__ V3 uv_point(const SceneView &S, const Surf &sf, float time) {
  return sf.motion ? moved_point(S, sf.motion, sf.p, -time) : sf.p;
}

// Texture index + 1 of a material's colour (0: the constant p[0..2]).
__device__ __forceinline__ int mat_texture(const MatRec &M) { return (int)((uint32_t)M.flags >> PT_MAT_TEXTURE_SHIFT); }

// DiffuseEmitter::emit (material.hpp:483-488) with its colour texture looked
// up at the hit's texture coordinates.
__device__ __forceinline__ V3 emit_at(const SceneView &S, const MatRec &M, const Surf &sf, V3 d, const HitRec &h,
                                      float time) {
  const int ti = mat_texture(M);
  if (!ti) return mat_emit(M, sf.n, d);
  if (!(dot(sf.n, -d) > 0.f)) return v3(0.f);
  const float2 uv = surface_uv(S, h.prim, uv_point(S, sf, time), sf.n, h.u, h.v);
  return tex_eval(S.textures[ti - 1], uv.x, uv.y) * M.p[3];
}

__device__ __forceinline__ float power_heuristic(float nf, float fpdf, float ng, float gpdf) {
  float f = nf * fpdf, g = ng * gpdf;  // maxdepth_mis.hpp:10-15 with sample counts
  if (isinf(f)) return 1.f;
  float f2 = f * f, g2 = g * g;
  return (f2 + g2) > 0.f ? f2 / (f2 + g2) : 0.f;
}

// Light-point offset of light sample ls at a vertex: the jittered
// light_nx x light_ny grid of getOffsets (random.hpp:47-63) that
// maxdepth_nee.hpp:91 draws per shading vertex, stratum (i, j) = (ls / ny,
// ls % ny), i outer; the jitter from the path's counter stream at the
// vertex's slot base rbase.
__device__ __forceinline__ float2 light_offset(const DeviceJob &J, uint64_t key, uint32_t rbase, int ls) {
  const int si = ls / J.job.light_ny, sj = ls % J.job.light_ny;
  return make_float2(((float)si + rand01(key, rbase + 2u * ls)) / (float)J.job.light_nx,
                     ((float)sj + rand01(key, rbase + 2u * ls + 1u)) / (float)J.job.light_ny);
}

// A light sample seen from x (maxdepth_nee.hpp:104-189): the point of
// Light::get_sample(u, v) (QuadLight light.hpp:131-137: v0 + u e1 + v e2;
// SphereLight :254-264: the whole sphere; EnvironmentLight envLight.hpp:20-36:
// HDRITexture's uniform sphere direction, texture.hpp:120-124, times 1e5),
// the normal get_normal_at gives there (light.hpp:139-145, 266-271,
// envLight.hpp:48-51), the normalised direction w from x and the distance,
// and L_emit towards x (light.hpp:157-165, 296-303: one-sided, the colour
// texture at texCoords (u, v), maxdepth_nee.hpp:175-176; envLight.hpp:73-90:
// the HDRI along w).  A moving light is taken at `time`.
struct LightPoint {
  V3 p, n, w, Le;
  float len;
};
__device__ __forceinline__ LightPoint light_point(const SceneView &S, const LightRec &Lr, float ox, float oy, V3 x,
                                                  float time) {
  LightPoint L;
  if (Lr.type == LIGHT_ENV) {
    // uniformSampleSphere * 1e5 (texture.hpp:120-124, envLight.hpp:26-43)
    float z = 1.f - 2.f * ox;
    float rr = sqrtf(fmaxf(0.f, 1.f - z * z));
    float sp, cp;
    sincospi_(2.f * oy, &sp, &cp);
    L.p = v3(rr * cp, rr * sp, z) * 1e5f;
    L.w = normalize(L.p - x);
    L.len = length(L.p - x);
    L.n = -normalize(L.p);
    L.Le = env_lookup(S.env, L.w);
    return L;
  }
  if (Lr.type == LIGHT_QUAD) {
    // QuadLight::get_sample / get_normal_at (light.hpp:131-147)
    L.p = v3(Lr.v0[0], Lr.v0[1], Lr.v0[2]) + ox * v3(Lr.e1[0], Lr.e1[1], Lr.e1[2]) +
          oy * v3(Lr.e2[0], Lr.e2[1], Lr.e2[2]);
    if (Lr.motion) L.p = moved_point(S, Lr.motion, L.p, time);
    L.n = v3(Lr.normal[0], Lr.normal[1], Lr.normal[2]);
  } else {
    // SphereLight::get_sample (light.hpp:254-264): the whole sphere
    float sth, cth, sph, cph;
    sincospi_(2.f * ox, &sth, &cth);
    float phi = acosf(2.f * oy - 1.f);
    sincos_(phi, &sph, &cph);
    V3 c = v3(Lr.v0[0], Lr.v0[1], Lr.v0[2]);
    if (Lr.motion) c = moved_point(S, Lr.motion, c, time);
    L.p = c + Lr.radius * v3(sph * cth, sph * sth, cph);
    L.n = normalize(L.p - c);
  }
  V3 ld = L.p - x;
  L.len = length(ld);
  L.w = normalize(ld);
  // L_emit of the light (light.hpp:157-165, 296-303); a textured light
  // is looked up at the sample's offsets (maxdepth_nee.hpp:175-176)
  const V3 lcol = Lr.texture ? tex_eval(S.textures[Lr.texture - 1], ox, oy)
                             : v3(Lr.color[0], Lr.color[1], Lr.color[2]);
  L.Le = (dot(L.n, -L.w) > 0.f) ? lcol * Lr.intensity : v3(0.f);
  return L;
}

// Light::pdf_value(origin, dir): the solid-angle density of sampling dir
// from origin.  QuadLight (light.hpp:164-205): the quad's plane hit, inside
// one of its two triangles by the reference's edge tests (the first test is
// the triangle's own orientation, so a triangle checks two of its edges),
// dist^2 / (area |cos|); SphereLight (:279-294): 1 / the solid angle of the
// visible cap, 1 / (4 pi) from inside; EnvironmentLight (envLight.hpp:58-70):
// HDRITexture::pdf_direction, uniform 1 / (4 pi) (texture.hpp:126-131).
__device__ inline float light_pdf_value(const LightRec &Lr, V3 origin, V3 dir) {
  if (Lr.type == LIGHT_ENV) return (float)(1.0 / (4.0 * PT_PI));
  if (Lr.type == LIGHT_SPHERE) {
    const V3 wc = v3(Lr.v0[0], Lr.v0[1], Lr.v0[2]) - origin;
    const float dc2 = dot(wc, wc), r2 = Lr.radius * Lr.radius;
    if (dc2 <= r2) return (float)(1.0 / (4.0 * PT_PI));
    const float cos_max = sqrtf(1.f - r2 / dc2);
    const float omega = (float)(2.0 * PT_PI * (double)(1.f - cos_max));
    return 1.f / omega;
  }
  const V3 v0 = v3(Lr.v0[0], Lr.v0[1], Lr.v0[2]);
  const V3 v1 = v0 + v3(Lr.e1[0], Lr.e1[1], Lr.e1[2]), v3_ = v0 + v3(Lr.e2[0], Lr.e2[1], Lr.e2[2]);
  const V3 v2 = v3(Lr.v2[0], Lr.v2[1], Lr.v2[2]);
  const V3 N = v3(Lr.normal[0], Lr.normal[1], Lr.normal[2]);
  const float denom = dot(N, dir);
  if (fabsf(denom) < 1e-6f) return 0.f;
  const float t = dot(v0 - origin, N) / denom;
  if (t <= 0.f) return 0.f;
  const V3 P = origin + dir * t;
  auto in_tri = [&](V3 A, V3 B, V3 C) {
    if (dot(cross(B - A, C - A), N) < 0.f) return false;
    if (dot(cross(C - B, P - B), N) < 0.f) return false;
    if (dot(cross(A - C, P - C), N) < 0.f) return false;
    return true;
  };
  if (!in_tri(v0, v1, v2) && !in_tri(v0, v2, v3_)) return 0.f;
  const float dist2 = dot(P - origin, P - origin);
  const float cos_t = fabsf(dot(N, -dir));
  return dist2 / (Lr.area * cos_t);
}

// Next-event estimation at one vertex (maxdepth_nee.hpp:89-232): LN light
// samples on a stratified x-by-y grid, each a ShadowQueue entry with its
// unoccluded contribution.  MED: the vertex is a medium scattering event
// (isotropic phase function instead of a BSDF, no surface cosine).
template <int FAM, bool MED>
__device__ __forceinline__ void next_event(const SceneView &S, const DeviceJob &J, const Queues &Q, int sslot,
                                           int path, uint64_t key, uint32_t rbase, const Surf &sf, int mat,
                                           V3 wo, V3 beta, int LN, bool mis, float time, bool tex_alb,
                                           V3 alb) {
  const float phase = (float)(1.0 / (4.0 * PT_PI));
  Q.sh_o[sslot] = make_float4(sf.p.x, sf.p.y, sf.p.z, __int_as_float(path));
  const float inv_ln = 1.f / (float)LN;
  const bool med = S.has_medium != 0;
  for (int ls = 0; ls < LN; ++ls) {
    float4 shd = make_float4(0.f, 0.f, 0.f, -1.f), shc = make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 lo = light_offset(J, key, rbase, ls);
    const float ox = lo.x, oy = lo.y;
    int li = (int)(rand01(key, rbase + 20u + ls) * S.n_lights) % S.n_lights;
    const LightRec &Lr = S.lights[li];
    V3 wl, Le;
    float tmax, pdf_l, G, NoI, tr = 1.f;
    bool valid = true;
    if (Lr.type == LIGHT_ENV) {
      float pdir;
      if (J.job.env_sampling == PT_ENV_ALIAS) {
        wl = env_alias_sample(S.env, ox, oy, rand01(key, rbase + 28u + ls), pdir);
        Le = env_lookup(S.env, wl);
      } else {
        const LightPoint P = light_point(S, Lr, ox, oy, sf.p, time);
        wl = P.w;
        Le = P.Le;
        pdir = (float)(1.0 / (4.0 * PT_PI));
      }
      tmax = FLT_MAX;
      pdf_l = pdir / (float)S.n_lights;
      NoI = MED ? 1.f : fmaxf(0.f, dot(sf.n, wl));
      G = NoI;
      valid = pdf_l > 1e-7f && !med;  // no light reaches through an infinite medium
    } else {
      const LightPoint P = light_point(S, Lr, ox, oy, sf.p, time);
      const V3 ln = P.n;
      const float len = P.len;
      wl = P.w;
      Le = P.Le;
      if (len < 0.001f) valid = false;
      tmax = len - 0.001f;
      pdf_l = (Lr.area <= 1e-7f) ? 0.f : 1.f / (Lr.area * (float)S.n_lights);
      NoI = MED ? 1.f : fmaxf(0.f, dot(sf.n, wl));
      float NoL = fmaxf(0.f, dot(ln, -wl));
      float d2 = len * len;
      G = (d2 < 1e-7f) ? 0.f : NoL * NoI / d2;
      if (!(pdf_l > 1e-7f)) valid = false;
      if (mis && valid && NoL > 0.f) {
        pdf_l = pdf_l * d2 / NoL;  // solid-angle pdf
        G = NoI;
      }
      if (med) tr = expf(-S.sigma_t_max * len);
    }
    if (valid && G > 0.f) {
      V3 f;
      float pb;
      if (MED) {
        f = v3(phase);
        pb = phase;
      } else {
        // f and scatter_pdf: every BSDF in the shading normal's frame --
        // HairMarschner's too (hairMarsch.hpp:49, hairMarsch.cpp:115), even on
        // a curve, whose tangent only frames its sampling
        bsdf_eval_t<FAM>(S.materials[mat], wo, wl, sf.n, sf.front, f, pb);
        if ((FAM == 0 || FAM < 0) && tex_alb) f = alb * PT_INV_PI_F;  // textured Lambertian albedo
      }
      float w = mis ? power_heuristic((float)LN, pdf_l, 1.f, pb) : 1.f;
      V3 c = beta * (f * Le * (G / pdf_l * w * inv_ln)) * tr;
      if (c.x != 0.f || c.y != 0.f || c.z != 0.f) {
        shd = make_float4(wl.x, wl.y, wl.z, tmax);
        shc = make_float4(c.x, c.y, c.z, time);
      }
    }
    Q.sh_d[(size_t)ls * Q.cap + sslot] = shd;
    Q.sh_c[(size_t)ls * Q.cap + sslot] = shc;
  }
}

// k_shade<FAM>: one path vertex per thread.  FAM 0..6 processes the
// material-sorted segment of that BSDF family with its code compiled alone;
// FAM PT_FAM_MISC the misses, emitter hits and medium events; FAM -1 the
// whole unsorted queue with run-time dispatch.  Correspondence with
// getRayColor (maxdepth_nee.hpp):
//   :16-17   depth limit -> continuations are queued while bounce + 1 < max_depth
//   :26-37   miss -> env / bg
//   :44-45   scatter() false -> emit()
//   :47-78   specular (delta) branches: no NEE, beta *= attenuation
//   :91-232  NEE (next_event, resolved by k_trace_shadow)
//   :238-247 continuation hitting an emitter is dropped (REF_NEE)
//   :251-255 beta *= f * |cos| / pdf
// NEE_MIS weights light and BSDF sampling with the power heuristic and
// always performs NEE at non-delta vertices.  The loop runs in phases so
// that the queue slot allocations (warp ballots) see every lane.
// Resident blocks per SM a shade kernel is compiled for: families whose BSDF
// code fits 102 registers without spilling run 5 blocks of 128 threads per
// SM (the compiler's default allocation gave them 96-128 registers, 4-5
// blocks); the Disney and hair kernels and the generic one, which spill
// below 128 registers, run 4.  Single-job and merged-wave variants get the
// same bound: a tighter one (6 blocks, 80 registers) changes how the
// compiler contracts multiply-adds, and the two variants must compute the
// same bits (a batched job equals its plain render).
constexpr int shade_min_blocks(int fam, bool) { return (fam == 5 || fam == 6 || fam < 0) ? 4 : 5; }

template <int FAM, bool MJ>
__device__ __forceinline__ void shade_body(const SceneView &S, const DeviceJob &J, const JobTable &T, const Queues &Q,
                                           int qsel, int bounce, long long g0) {
  int lo = 0, hi = Q.counts[qsel];
  if (FAM >= 0) {
    lo = Q.seg[FAM];
    hi = (FAM == PT_FAM_MISC) ? Q.seg[PT_KEY_MEDIUM + 1] : Q.seg[FAM + 1];
  }
  const int n = hi - lo;
  const int nq = qsel ^ 1;
  const uint32_t rbase = 64u + 32u * (uint32_t)bounce;
  const bool med = S.has_medium != 0;
  const int dpb = med ? 4 : 3;  // sampler dimensions per bounce
  const float phase = (float)(1.0 / (4.0 * PT_PI));  // isotropic Henyey-Greenstein, g = 0
  constexpr bool DO_MISC = (FAM < 0 || FAM == PT_FAM_MISC);
  constexpr bool DO_SURF = (FAM != PT_FAM_MISC);
  int segs = 0;
  const int stride = gridDim.x * blockDim.x;
  const int nround = (n + stride - 1) / stride * stride;
  for (int ii = blockIdx.x * blockDim.x + threadIdx.x; ii < nround; ii += stride) {
    // ---------------- phase A: hit logic and BSDF sampling
    bool do_nee = false, push = false, nee_medium = false;
    int path = 0, mat = 0;
    Surf sf;
    sf.p = v3(0.f);
    sf.n = v3(0.f, 0.f, 1.f);
    sf.front = false;
    V3 wo = v3(0.f), beta = v3(0.f), wi = v3(0.f), nb = v3(0.f);
    float npdf = -1.f;
    uint64_t key = 0;
    float time = 0.f;
    int LN = 1;
    bool mis = false;
    bool tex_alb = false;  // textured Lambertian albedo of this vertex
    V3 alb = v3(0.f);
    if (ii < n) {
      const int i = (FAM >= 0) ? Q.order[lo + ii] : ii;
      float4 ro = ld4(Q.ray_o[qsel] + i), rd = ld4(Q.ray_d[qsel] + i);
      float4 hh = ld4(Q.hit + i);
      path = __float_as_int(ro.w);
      time = rd.w;
      V3 o = v3(ro.x, ro.y, ro.z), d = v3(rd.x, rd.y, rd.z);
      float4 b4 = Q.beta[path];
      beta = v3(b4.x, b4.y, b4.z);
      const float prev_pdf = b4.w;  // < 0: camera ray or previous vertex delta
      long long g;
      const DeviceJob &Jp = path_job<MJ>(J, T, Q, path, g0, g);
      LN = Jp.job.light_nx * Jp.job.light_ny;
      mis = Jp.job.estimator == PT_EST_NEE_MIS;
      const int max_depth = Jp.job.max_depth;
      const int limit = mis ? max_depth + 1 : max_depth;
      PathId P = path_id(Jp, g);
      key = P.key;
      const int prim = __float_as_int(hh.y);
      V3 Ladd = v3(0.f);
      if (med && bounce >= max_depth) beta = beta * expf(-S.sigma_t_max * (prim >= 0 ? hh.x : INFINITY));
      if (DO_MISC && prim == PT_HIT_MEDIUM) {
        // ---- medium scattering event (extension): weight sigma_s / sigma_t
        ++segs;
        sf.p = o + hh.x * normalize(d);
        beta = beta * v3(S.sigma_s[0] / (S.sigma_a[0] + S.sigma_s[0]), S.sigma_s[1] / (S.sigma_a[1] + S.sigma_s[1]),
                         S.sigma_s[2] / (S.sigma_a[2] + S.sigma_s[2]));
        do_nee = S.n_lights > 0;
        nee_medium = true;
        if (bounce + 1 < limit) {
          float u0 = sampler_dim(Jp, dpb * bounce + 2, P.halton_index, P.key, P.pix, P.k);
          float u1 = sampler_dim(Jp, dpb * bounce + 3, P.halton_index, P.key, P.pix, P.k);
          float z = 1.f - 2.f * u0, rr = sqrtf(fmaxf(0.f, 1.f - z * z));
          float sp, cp;
          sincospi_(2.f * u1, &sp, &cp);
          wi = v3(rr * cp, rr * sp, z);
          nb = beta;
          npdf = phase;
          push = true;
        }
      } else if (DO_MISC && prim < 0) {
        // ---- miss (maxdepth_nee.hpp:26-37)
        if (S.env.present) {
          V3 Le = env_lookup(S.env, d);
          float w = 1.f;
          if (mis && prev_pdf >= 0.f && S.n_lights > 0) {
            float pl = (Jp.job.env_sampling == PT_ENV_ALIAS) ? env_alias_pdf(S.env, d) : (float)(1.0 / (4.0 * PT_PI));
            w = power_heuristic(1.f, prev_pdf, (float)LN, pl / (float)S.n_lights);
          }
          Ladd = beta * Le * w;
        } else {
          Ladd = beta * v3(S.bg[0], S.bg[1], S.bg[2]);
        }
      } else if (prim >= 0) {
        HitRec h;
        h.t = hh.x;
        h.prim = prim;
        h.u = hh.z;
        h.v = hh.w;
        sf = surface_at(S, o, d, h, time);
        mat = sf.mat;
        const MatRec &M = S.materials[mat];
        if (DO_MISC && mat_is_emitter(M)) {
          // DiffuseEmitter: scatter() is false (material.hpp:475-481)
          if (prev_pdf < 0.f) {
            Ladd = beta * emit_at(S, M, sf, d, h, time);
          } else if (mis) {
            if (sf.light >= 0) {
              const LightRec &Lr = S.lights[sf.light];
              // one-sided emission of the light, as NEE evaluates it
              V3 lc = v3(Lr.v0[0], Lr.v0[1], Lr.v0[2]);
              if (Lr.motion) lc = moved_point(S, Lr.motion, lc, time);
              V3 ln = (Lr.type == LIGHT_QUAD) ? v3(Lr.normal[0], Lr.normal[1], Lr.normal[2]) : normalize(sf.p - lc);
              float cl = dot(ln, -normalize(d));
              if (cl > 0.f) {
                V3 lcol = v3(Lr.color[0], Lr.color[1], Lr.color[2]);
                if (Lr.texture) {
                  const float2 uv = surface_uv(S, h.prim, uv_point(S, sf, time), sf.n, h.u, h.v);
                  lcol = tex_eval(S.textures[Lr.texture - 1], uv.x, uv.y);
                }
                V3 Le = lcol * Lr.intensity;
                float pl = h.t * h.t / (cl * Lr.area * (float)S.n_lights);
                Ladd = beta * Le * power_heuristic(1.f, prev_pdf, (float)LN, pl);
              }
            } else {
              Ladd = beta * emit_at(S, M, sf, d, h, time);
            }
          }
          // REF_NEE after a non-delta vertex: dropped (maxdepth_nee.hpp:246-247)
        } else if (DO_SURF && !mat_is_emitter(M) && bounce < max_depth) {
          ++segs;
          const int dim0 = dpb * bounce + (med ? 1 : 0);
          float uc = sampler_dim(Jp, dim0, P.halton_index, P.key, P.pix, P.k);
          float u0 = sampler_dim(Jp, dim0 + 1, P.halton_index, P.key, P.pix, P.k);
          float u1 = sampler_dim(Jp, dim0 + 2, P.halton_index, P.key, P.pix, P.k);
          wo = -normalize(d);
          // HairMarschner::scatter on a curve samples the direction and its
          // pdf in the curve tangent's frame (hairMarsch.cpp:12-24) while its
          // attenuation is f(), framed by the normal (hairMarsch.hpp:49)
          const bool hair_tan = (FAM == 6 || FAM < 0) && sf.has_tan && M.type == PT_MAT_HAIR;
          BsdfSample bs = bsdf_sample_t<FAM>(M, wo, hair_tan ? sf.tan : sf.n, sf.front, uc, u0, u1);
          if (hair_tan && bs.ok) bs.att = hair_f(M, wo, bs.wi, sf.n);
          if ((FAM == 0 || FAM < 0) && M.type == PT_MAT_LAMBERTIAN && mat_texture(M)) {
            // Lambertian with a ColorVariant texture: albedo at the hit's
            // texCoords (material.hpp:100, 133)
            const float2 uv = surface_uv(S, prim, uv_point(S, sf, time), sf.n, h.u, h.v);
            tex_alb = true;
            alb = tex_eval(S.textures[mat_texture(M) - 1], uv.x, uv.y);
            bs.att = alb * PT_INV_PI_F;
          }
          const bool spec_r = (bs.type & BX_SPECULAR_R) == BX_SPECULAR_R;
          const bool spec_t = (bs.type & BX_SPECULAR_T) == BX_SPECULAR_T;
          if (bs.ok && (spec_r || spec_t)) {
            // specular: emit + attenuation * L(next) (maxdepth_nee.hpp:47-78);
            // the split-ray case follows one child chosen with probability R
            // (thin_sample), the expectation of the two-child sum.
            if (bounce + 1 < limit) {
              push = true;
              wi = bs.wi;
              nb = beta * ((spec_r && spec_t) ? v3(1.f) : bs.att);
              npdf = -1.f;
            }
          } else if (bs.ok || mis) {
            do_nee = S.n_lights > 0;
            if (bs.ok && bounce + 1 < limit) {
              // ---- continuation (maxdepth_nee.hpp:234-255)
              wi = normalize(bs.wi);
              float c = fabsf(dot(sf.n, wi));
              nb = beta * bs.att * (c / bs.pdf);
              npdf = bs.pdf;
              push = true;
              if (Jp.job.rr_start >= 0 && bounce >= Jp.job.rr_start) {
                // roulette_naive.hpp:35-38 applied to the continuation
                float q = clampf(max_comp(bs.att), 0.5f, 1.0f);
                if (rand01(P.key, rbase + 31u) > q) push = false;
                nb = nb * (1.f / q);
              }
            }
          }
        }
      }
      if (Ladd.x != 0.f || Ladd.y != 0.f || Ladd.z != 0.f) {
        float4 L4 = Q.L[path];
        Q.L[path] = make_float4(L4.x + Ladd.x, L4.y + Ladd.y, L4.z + Ladd.z, 0.f);
      }
      if (push) Q.beta[path] = make_float4(nb.x, nb.y, nb.z, npdf);
    }
    // ---------------- phase B: queue slots (all lanes)
    const int sslot = warp_alloc(&Q.counts[2], do_nee);
    const int slot = warp_alloc(&Q.counts[nq], push);
    if (push) {
      Q.ray_o[nq][slot] = make_float4(sf.p.x, sf.p.y, sf.p.z, __int_as_float(path));
      Q.ray_d[nq][slot] = make_float4(wi.x, wi.y, wi.z, time);
    }
    // ---------------- phase C: next-event estimation
    if (do_nee) {
      long long g;
      const DeviceJob &Jp = path_job<MJ>(J, T, Q, path, g0, g);
      if (DO_MISC && nee_medium)
        next_event<FAM, true>(S, Jp, Q, sslot, path, key, rbase, sf, mat, wo, beta, LN, mis, time, false, alb);
      else if (DO_SURF)
        next_event<FAM, false>(S, Jp, Q, sslot, path, key, rbase, sf, mat, wo, beta, LN, mis, time, tex_alb, alb);
    }
  }
  warp_count(&Q.stats[1], segs);
}
template <int FAM, bool MJ>
__global__ void __launch_bounds__(128, shade_min_blocks(FAM, MJ)) k_shade(SceneView S, DeviceJob J, JobTable T, Queues Q, int qsel, int bounce,
                                               long long g0) {
  shade_body<FAM, MJ>(S, J, T, Q, qsel, bounce, g0);
}

// k_trace_shadow: the ShadowQueue's rays (vertex v, light sample ls; ray
// r = v * LN + ls) through the BVH, any-hit, with the persistent warps of
// k_trace_closest.  Each ray's visibility goes to Q.sh_vis; k_shadow_resolve
// then adds the visible terms of every vertex to its path in a fixed order,
// so the result does not depend on which warp traced which ray.
template <bool CURVES>
__device__ __forceinline__ void trace_shadow_body(const SceneView &S, const Queues &Q, int LN, int32_t *stack) {
  const int n = Q.counts[2] * LN;
  int *fetch = Q.counts + 3;
  const int lane = threadIdx.x & 31;
  int32_t *my_stack = stack + threadIdx.x;
  TravRay R;
  bool active = false, exhausted = false;
  size_t slot = 0;
  int rays = 0;
  for (;;) {
    unsigned idle = __ballot_sync(0xffffffffu, !active);
    if (!exhausted && __popc(idle) >= PT_FETCH_IDLE_SHADOW) {
      const int k = __popc(idle);
      int base = 0;
      if (lane == 0) base = atomicAdd(fetch, k);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + k >= n) exhausted = true;
      if (!active) {
        const int r = base + __popc(idle & lanemask_lt());
        if (r < n) {
          const int v = r / LN, ls = r - v * LN;
          slot = (size_t)ls * Q.cap + v;
          float4 dd = ld4(Q.sh_d + slot);
          if (dd.w >= 0.f) {
            float4 so = ld4(Q.sh_o + v);
            const float time = S.has_motion ? ld4(Q.sh_c + slot).w : 0.f;
            trav_init(R, v3(so.x, so.y, so.z), v3(dd.x, dd.y, dd.z), 0.001f, dd.w, time);
            active = true;
            ++rays;
          }
        }
      }
      idle = __ballot_sync(0xffffffffu, !active);
    }
    if (idle == 0xffffffffu) {
      if (exhausted) break;
      continue;
    }
    const bool lt = warp_leaf_turn(active, R.ref);
    if (lane_turn(active, R.ref, lt) && trav_step<true, CURVES>(S, R, my_stack, blockDim.x, Q.err)) {
      Q.sh_vis[slot] = R.found ? 0 : 1;
      active = false;
    }
  }
  warp_count(&Q.stats[3], rays);
}

// k_shadow_resolve: per vertex, the visible NEE terms in light-sample order
// added to the path's L.  Rays that were never traced (no contribution) have
// a zero term, whatever their stale visibility byte says.
__device__ __forceinline__ void shadow_resolve_body(const Queues &Q, int LN) {
  const int n = Q.counts[2];
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    V3 acc = v3(0.f);
    for (int ls = 0; ls < LN; ++ls) {
      const size_t slot = (size_t)ls * Q.cap + v;
      if (Q.sh_vis[slot]) {
        float4 cc = ld4(Q.sh_c + slot);
        acc += v3(cc.x, cc.y, cc.z);
      }
    }
    if (acc.x != 0.f || acc.y != 0.f || acc.z != 0.f) {
      const int path = __float_as_int(ld4(Q.sh_o + v).w);
      float4 L = Q.L[path];
      Q.L[path] = make_float4(L.x + acc.x, L.y + acc.y, L.z + acc.z, 0.f);
    }
  }
}

// k_film: per pixel, adds the wave's paths to the film one by one in sample
// order.  Adding sample by sample (not a per-wave partial sum) makes the film
// independent of how the samples are split into waves, so a job gives the
// same bits alone, in a batch, or in a served mix.
__device__ __forceinline__ void film_body(const DeviceJob &J, const Queues &Q, long long g0, int n, long long slot0,
                                          float *film) {
  const long long npix = (long long)J.job.width * J.job.height;
  const long long g1 = g0 + n;
  const long long plane0 = g0 / npix, plane1 = (g1 - 1) / npix;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < npix;
       t += (long long)gridDim.x * blockDim.x) {
    bool any = false;
    float ax = 0.f, ay = 0.f, az = 0.f;
    for (long long pl = plane0; pl <= plane1; ++pl) {
      long long g = pl * npix + t;
      if (g < g0 || g >= g1) continue;
      if (!any) {
        ax = film[3 * t];
        ay = film[3 * t + 1];
        az = film[3 * t + 2];
        any = true;
      }
      float4 L = Q.L[g - g0 + slot0];
      ax += L.x;
      ay += L.y;
      az += L.z;
    }
    if (any) {
      film[3 * t] = ax;
      film[3 * t + 1] = ay;
      film[3 * t + 2] = az;
    }
  }
}

static inline int grid_for(long long n, int block, int max_blocks) {
  long long b = (n + block - 1) / block;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (int)b;
}

// Camera and the bounces of one wave (single job or merged jobs):
// trace -> [sort] -> shade -> shadow per bounce.
template <bool MJ>
void launch_wave_stages(const SceneView &S, const DeviceJob &J, const JobTable &T, const Queues &Q, long long g0,
                        int n, int LN, int bounces, const LaunchCfg &cfg, cudaStream_t st, Profiler &P,
                        const ShadeStreams *ss) {
  P.begin(STAGE_CAMERA, st);
  k_camera<MJ><<<grid_for(n, 256, cfg.max_blocks_simple), 256, 0, st>>>(J, T, Q, g0, n);
  P.end(st);
  P.count(STAGE_CAMERA, 1);
  int qsel = 0;
  // bounce b's closest rays are traced together with bounce b - 1's shadow
  // rays (paired) in small waves, and in large ones once the queues thin
  // out: from the job's roulette start (single-job waves), or from
  // cfg.pair_from_bounce when set
  int from = cfg.pair_from_bounce;
  if (from <= 0) from = (!MJ && J.job.rr_start >= 0) ? std::max(1, (int)J.job.rr_start) : (1 << 20);
  auto paired = [&](int b) { return b > 0 && b < bounces && (n <= cfg.pair_trace || b >= from); };
  for (int b = 0; b < bounces; ++b) {
    const bool pair = paired(b);
    // reset next-queue and fetch counters (device side, graph friendly)
    // ([2] shadow queue, [3] shadow fetch, [4] closest-hit fetch); a
    // pending shadow queue of the previous bounce keeps [2]
    cudaMemsetAsync(Q.counts + (qsel ^ 1), 0, sizeof(int), st);
    if (!pair)
      cudaMemsetAsync(Q.counts + 2, 0, 3 * sizeof(int), st);
    else
      cudaMemsetAsync(Q.counts + 4, 0, sizeof(int), st);
    P.begin(STAGE_TRACE, st);
    if (pair) {
      // this bounce's closest rays with the previous bounce's shadow rays
      if (S.curves)
        k_trace_pair<MJ, true><<<cfg.trace_blocks, 128, stack_bytes(S, 128), st>>>(S, J, T, Q, qsel, b, g0, LN);
      else
        k_trace_pair<MJ, false><<<cfg.trace_blocks, 128, stack_bytes(S, 128), st>>>(S, J, T, Q, qsel, b, g0, LN);
    } else if (S.curves) {
      k_trace_closest<MJ, true><<<cfg.trace_blocks, 128, stack_bytes(S, 128), st>>>(S, J, T, Q, qsel, b, g0);
    } else {
      k_trace_closest<MJ, false><<<cfg.trace_blocks, 128, stack_bytes(S, 128), st>>>(S, J, T, Q, qsel, b, g0);
    }
    P.end(st);
    P.count(STAGE_TRACE, 1);
    if (pair) {
      // the previous bounce's shadow terms, before this bounce's shading
      P.begin(STAGE_SHADOW, st);
      launch_shadow_resolve(Q, LN, cfg, st);
      cudaMemsetAsync(Q.counts + 2, 0, 2 * sizeof(int), st);
      P.end(st);
      P.count(STAGE_SHADOW, 1);
    }
    if (cfg.sort_by_material) {
      // sort-by-material queues: one specialised shade kernel per family
      P.begin(STAGE_SORT, st);
      launch_sort(S, Q, qsel, cfg, st);
      P.end(st);
      P.count(STAGE_SORT, 2);
      P.begin(STAGE_SHADE, st);
      // the families present, then misses / emitters / medium events, each
      // on the next of the stream and its side streams (round robin)
      int used = 0;  // side streams forked
      int k = 0;     // kernels launched
      auto next_stream = [&]() -> cudaStream_t {
        const int slot = ss ? k % (ShadeStreams::N + 1) : 0;
        ++k;
        if (slot == 0) return st;
        if (slot > used) {
          if (used == 0) cudaEventRecord(ss->fork, st);
          cudaStreamWaitEvent(ss->aux[slot - 1], ss->fork, 0);
          used = slot;
        }
        return ss->aux[slot - 1];
      };
      if (cfg.family_mask & (1u << 0)) k_shade<0, MJ><<<cfg.shade_fam_blocks[0], 128, 0, next_stream()>>>(S, J, T, Q, qsel, b, g0);
      if (cfg.family_mask & (1u << 1)) k_shade<1, MJ><<<cfg.shade_fam_blocks[1], 128, 0, next_stream()>>>(S, J, T, Q, qsel, b, g0);
      if (cfg.family_mask & (1u << 2)) k_shade<2, MJ><<<cfg.shade_fam_blocks[2], 128, 0, next_stream()>>>(S, J, T, Q, qsel, b, g0);
      if (cfg.family_mask & (1u << 3)) k_shade<3, MJ><<<cfg.shade_fam_blocks[3], 128, 0, next_stream()>>>(S, J, T, Q, qsel, b, g0);
      if (cfg.family_mask & (1u << 4)) k_shade<4, MJ><<<cfg.shade_fam_blocks[4], 128, 0, next_stream()>>>(S, J, T, Q, qsel, b, g0);
      if (cfg.family_mask & (1u << 5)) k_shade<5, MJ><<<cfg.shade_fam_blocks[5], 128, 0, next_stream()>>>(S, J, T, Q, qsel, b, g0);
      if (cfg.family_mask & (1u << 6)) k_shade<6, MJ><<<cfg.shade_fam_blocks[6], 128, 0, next_stream()>>>(S, J, T, Q, qsel, b, g0);
      k_shade<PT_FAM_MISC, MJ><<<cfg.shade_fam_blocks[PT_FAM_MISC], 128, 0, next_stream()>>>(S, J, T, Q, qsel, b, g0);
      for (int u = 0; u < used; ++u) {
        cudaEventRecord(ss->join[u], ss->aux[u]);
        cudaStreamWaitEvent(st, ss->join[u], 0);
      }
      P.end(st);
      P.count(STAGE_SHADE, 1 + __builtin_popcount(cfg.family_mask & 0x7fu));
    } else {
      P.begin(STAGE_SHADE, st);
      k_shade<-1, MJ><<<cfg.shade_fam_blocks[PT_FAM_MISC + 1], 128, 0, st>>>(S, J, T, Q, qsel, b, g0);
      P.end(st);
      P.count(STAGE_SHADE, 1);
    }
    if (!paired(b + 1)) {
      P.begin(STAGE_SHADOW, st);
      launch_shadow(S, Q, LN, cfg, st);
      P.end(st);
      P.count(STAGE_SHADOW, 2);
    }
    qsel ^= 1;
  }
}

}  // namespace pt
