// pt_kernels.cu -- the wavefront stages of the NEE(+MIS) path integrator for
// single-job waves, the job-independent stages shared with merged waves, and
// the batch test kernels behind the C-ABI.
//
// One wave = a contiguous range of (sample, pixel) paths.  Per bounce:
//   k_trace_closest  RayQueue -> HitQueue            (BVH4, shared-mem stack)
//   k_sort_*         HitQueue -> order by material family (counting sort)
//   k_shade<FAM>     logic + BSDF sample + NEE: writes next RayQueue
//                    (warp-aggregated compaction) and ShadowQueue
//   k_trace_shadow   ShadowQueue any-hit visibility
//   k_shadow_resolve visible NEE terms added to L in a fixed order
// and once per wave k_camera (RayQueue 0) and k_film (ordered per-pixel
// accumulation).  Small waves trace a bounce's shadow rays together with the
// next bounce's closest-hit rays (k_trace_pair, pt_wave.cuh).
#include "pt_wave.cuh"

namespace pt {

// ------------------------------------------------------------ test kernels
__global__ void k_sampler_eval(int strategy, const uint16_t *perm, uint32_t first, int n, int dims,
                               float *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)n * dims;
       i += (long long)gridDim.x * blockDim.x) {
    int s = (int)(i / dims), d = (int)(i % dims);
    uint32_t idx = first + (uint32_t)s;
    float v;
    if (strategy == PT_SAMPLER_HALTON_NONE)
      v = radical_inverse(c_halton, d, idx);
    else if (strategy == PT_SAMPLER_HALTON_PERMUTE)
      v = permuted_radical_inverse(c_halton, perm, d, idx);
    else
      v = owen_radical_inverse(c_halton, d, idx);
    out[i] = v;
  }
}

// Sample values of the paths [first, first + n) of a single-job wave, from
// the device functions the camera and shade stages call: the pixel-grid
// offset of the path's sample (k_camera), the sampler dimensions
// 0..dims-1 (sampler_dim) and, per bounce b < bounces, the LN light-point
// offsets (light_offset at the vertex's slot base 64 + 32 b).
__global__ void k_path_samples(DeviceJob J, long long first, int n, int dims, int bounces, int LN, float *pix,
                               float *dv, float *lo) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const PathId P = path_id(J, first + s);
    if (pix) {
      const float2 o = J.job.offsets[P.k];
      pix[2 * (size_t)s] = o.x;
      pix[2 * (size_t)s + 1] = o.y;
    }
    if (dv)
      for (int d = 0; d < dims; ++d)
        dv[(size_t)s * dims + d] = sampler_dim(J, d, P.halton_index, P.key, P.pix, P.k);
    if (lo)
      for (int b = 0; b < bounces; ++b)
        for (int ls = 0; ls < LN; ++ls) {
          const float2 o = light_offset(J, P.key, 64u + 32u * (uint32_t)b, ls);
          const size_t i = (((size_t)s * bounces + b) * LN + ls) * 2;
          lo[i] = o.x;
          lo[i + 1] = o.y;
        }
  }
}

void launch_path_samples(const DeviceJob &J, long long first, int n, int dims, int bounces, float *pix, float *dv,
                         float *lo, cudaStream_t st) {
  const int LN = J.job.light_nx * J.job.light_ny;
  k_path_samples<<<grid_for(n, 128, 152 * 8), 128, 0, st>>>(J, first, n, dims, bounces, LN, pix, dv, lo);
}

template <bool ANY>
__global__ void __launch_bounds__(128) k_trace_test(SceneView S, const float *rays, const float *tmaxs,
                                                    int n, float tmin, float tmax, float *t_out,
                                                    int *prim_out, float *uv_out, uint8_t *occ,
                                                    int *err) {
  extern __shared__ int32_t stack[];  // S.stack_entries x 128
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    V3 o = v3(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]);
    V3 d = v3(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]);
    HitRec h;
    float tm = ANY ? tmaxs[i] : tmax;
    bool r = traverse<ANY>(S, o, d, tmin, tm, h, stack + threadIdx.x, blockDim.x, err);
    if (ANY) {
      occ[i] = r ? 1 : 0;
    } else {
      t_out[i] = r ? h.t : FLT_MAX;
      prim_out[i] = r ? h.prim : -1;
      uv_out[2 * i] = h.u;
      uv_out[2 * i + 1] = h.v;
    }
  }
}

// Hittable::intersect's HitRecord (base/primitive.hpp:30-79) at the closest
// hit: t, primitive, position, the normal turned towards the ray
// (HitRecord::set_normal) and is_inside (the front-face flag, FlipFace
// toggled) -- what surface_at gives the shade stage.
__global__ void __launch_bounds__(128) k_intersect(SceneView S, const float *rays, int n, float tmin, float tmax,
                                                   float *t_out, int *prim_out, float *pos, float *nrm,
                                                   uint8_t *front, int *err) {
  extern __shared__ int32_t stack[];  // S.stack_entries x 128
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const V3 o = v3(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]);
    const V3 d = v3(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]);
    HitRec h;
    const bool r = traverse<false>(S, o, d, tmin, tmax, h, stack + threadIdx.x, blockDim.x, err);
    Surf sf;
    sf.p = sf.n = v3(0.f);
    sf.front = false;
    if (r) sf = surface_at(S, o, d, h, 0.f);
    t_out[i] = r ? h.t : FLT_MAX;
    prim_out[i] = r ? h.prim : -1;
    pos[3 * i] = sf.p.x;
    pos[3 * i + 1] = sf.p.y;
    pos[3 * i + 2] = sf.p.z;
    nrm[3 * i] = sf.n.x;
    nrm[3 * i + 1] = sf.n.y;
    nrm[3 * i + 2] = sf.n.z;
    front[i] = (r && sf.front) ? 1 : 0;
  }
}

void launch_intersect(const SceneView &S, const float *rays, int n, float tmin, float tmax, float *t, int *prim,
                      float *pos, float *nrm, uint8_t *front, int *err, cudaStream_t st) {
  k_intersect<<<grid_for(n, 128, 152 * 8), 128, stack_bytes(S, 128), st>>>(S, rays, n, tmin, tmax, t, prim, pos, nrm,
                                                                         front, err);
}

// The Light methods of one light of a resident scene at n (u, v, x) items:
// get_sample, get_normal_at, the direction from x, L_emit towards x and
// pdf_value(x, dir) -- light_point / light_pdf_value, the code NEE runs.
__global__ void k_light_eval(SceneView S, int light, int n, const float *uv, const float *x, const float *pdf_dir,
                             float *point, float *normal, float *dir, float *le, float *pdf) {
  const LightRec &Lr = S.lights[light];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const V3 xi = v3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
    const LightPoint P = light_point(S, Lr, uv[2 * i], uv[2 * i + 1], xi, 0.f);
    const V3 pd = pdf_dir ? v3(pdf_dir[3 * i], pdf_dir[3 * i + 1], pdf_dir[3 * i + 2]) : P.w;
    const float pv = light_pdf_value(Lr, xi, pd);
    const V3 out[4] = {P.p, P.n, P.w, P.Le};
    float *dst[4] = {point, normal, dir, le};
    for (int k = 0; k < 4; ++k) {
      dst[k][3 * i] = out[k].x;
      dst[k][3 * i + 1] = out[k].y;
      dst[k][3 * i + 2] = out[k].z;
    }
    pdf[i] = pv;
  }
}

void launch_light_eval(const SceneView &S, int light, int n, const float *uv, const float *x, const float *pdf_dir,
                       float *point, float *normal, float *dir, float *le, float *pdf, cudaStream_t st) {
  k_light_eval<<<grid_for(n, 128, 152 * 8), 128, 0, st>>>(S, light, n, uv, x, pdf_dir, point, normal, dir, le, pdf);
}

__global__ void k_bsdf_eval(const MatRec *m, int n, const float *wo, const float *wi,
                            const float *nrm, const uint8_t *front, float *f, float *pdf) {
  MatRec mat = *m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    V3 o = v3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
    V3 w = v3(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
    V3 nn = v3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
    V3 fv = bsdf_f(mat, o, w, nn, front[i] != 0);
    f[3 * i] = fv.x;
    f[3 * i + 1] = fv.y;
    f[3 * i + 2] = fv.z;
    pdf[i] = bsdf_pdf(mat, o, w, nn, front[i] != 0);
  }
}

__global__ void k_bsdf_sample(const MatRec *m, int n, const float *wo, const float *nrm,
                              const uint8_t *front, const float *uc, const float *u, uint8_t *ok,
                              float *wi, float *att, float *pdf, uint32_t *type) {
  MatRec mat = *m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    V3 o = v3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
    V3 nn = v3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
    BsdfSample s = bsdf_sample(mat, o, nn, front[i] != 0, uc[i], u[2 * i], u[2 * i + 1]);
    ok[i] = s.ok ? 1 : 0;
    wi[3 * i] = s.ok ? s.wi.x : 0.f;
    wi[3 * i + 1] = s.ok ? s.wi.y : 0.f;
    wi[3 * i + 2] = s.ok ? s.wi.z : 0.f;
    att[3 * i] = s.ok ? s.att.x : 0.f;
    att[3 * i + 1] = s.ok ? s.att.y : 0.f;
    att[3 * i + 2] = s.ok ? s.att.z : 0.f;
    pdf[i] = s.ok ? s.pdf : 0.f;
    type[i] = s.ok ? s.type : 0u;
  }
}

// Sort keys: material type 0..7 of the surface hit, PT_KEY_MISS,
// PT_KEY_MEDIUM.  Counting sort in two passes (histogram, scatter); the
// second pass also publishes the segment bounds Q.seg[0..PT_SORT_BINS].
__device__ __forceinline__ int sort_key(const SceneView &S, float4 hit) {
  int prim = __float_as_int(hit.y);
  if (prim == PT_HIT_MEDIUM) return PT_KEY_MEDIUM;
  if (prim < 0) return PT_KEY_MISS;
  return S.materials[__ldg(&S.shade[prim].material)].type;
}
__global__ void k_sort_hist(SceneView S, Queues Q, int qsel) {
  __shared__ int h[PT_SORT_BINS];
  for (int b = threadIdx.x; b < PT_SORT_BINS; b += blockDim.x) h[b] = 0;
  __syncthreads();
  const int n = Q.counts[qsel];
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * blockDim.x;
  const int nround = (n + stride - 1) / stride * stride;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nround; i += stride) {
    const bool act = i < n;
    int key = -1;
    if (act) {
      key = sort_key(S, ld4(Q.hit + i));
      Q.sort_key[i] = key;
    }
    // one shared atomic per (warp, key)
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (act && lane == __ffs(peers) - 1) atomicAdd(&h[key], __popc(peers));
  }
  __syncthreads();
  for (int b = threadIdx.x; b < PT_SORT_BINS; b += blockDim.x)
    if (h[b]) atomicAdd(&Q.bins[b], h[b]);
}
__global__ void k_sort_scatter(Queues Q, int qsel) {
  __shared__ int base[PT_SORT_BINS + 1];
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int b = 0; b < PT_SORT_BINS; ++b) {
      base[b] = acc;
      acc += Q.bins[b];
    }
    base[PT_SORT_BINS] = acc;
    if (blockIdx.x == 0)
      for (int b = 0; b <= PT_SORT_BINS; ++b) Q.seg[b] = base[b];
  }
  __syncthreads();
  // per tile of blockDim entries: warp-aggregated ranks in shared memory, one
  // global atomic per (tile, key) to reserve the tile's range of each key
  __shared__ int cnt[PT_SORT_BINS], gbase[PT_SORT_BINS];
  const int n = Q.counts[qsel];
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * blockDim.x;
  const int nround = (n + stride - 1) / stride * stride;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nround; i += stride) {
    if (threadIdx.x < PT_SORT_BINS) cnt[threadIdx.x] = 0;
    __syncthreads();
    const bool act = i < n;
    const int key = act ? Q.sort_key[i] : PT_SORT_BINS - 1;
    const unsigned peers = __match_any_sync(0xffffffffu, act ? key : -1);
    const int leader = __ffs(peers) - 1;
    const int rank = __popc(peers & ((1u << lane) - 1u));
    int wbase = 0;
    if (act && lane == leader) wbase = atomicAdd(&cnt[key], __popc(peers));
    wbase = __shfl_sync(0xffffffffu, wbase, leader);
    __syncthreads();
    if (threadIdx.x < PT_SORT_BINS) {
      const int c = cnt[threadIdx.x];
      gbase[threadIdx.x] = c ? atomicAdd(&Q.bins[PT_SORT_BINS + threadIdx.x], c) : 0;
    }
    __syncthreads();
    if (act) Q.order[base[key] + gbase[key] + wbase + rank] = i;
    __syncthreads();
  }
}

// k_trace_shadow, k_shadow_resolve, k_film: their bodies are in pt_wave.cuh
// (trace_shadow_body, shadow_resolve_body, film_body).
template <bool CURVES>
__global__ void __launch_bounds__(128) k_trace_shadow(SceneView S, Queues Q, int LN) {
  extern __shared__ int32_t stack[];  // S.stack_entries x 128
  trace_shadow_body<CURVES>(S, Q, LN, stack);
}
__global__ void k_shadow_resolve(Queues Q, int LN) { shadow_resolve_body(Q, LN); }
__global__ void k_film(DeviceJob J, Queues Q, long long g0, int n, long long slot0, float *film) {
  film_body(J, Q, g0, n, slot0, film);
}

// Serving: RMSE of a request's mean image estimated from its two
// independent half films A (even passes) and B (odd passes),
// 0.5 * sqrt(mean((A/na - B/nb)^2)), for many requests in one launch.  Fixed
// grid and fixed-order reductions: the estimate, and hence when a request
// stops, does not depend on what else is being served.
__global__ void __launch_bounds__(256) k_film_rmse(const FilmPair *pairs, double *partials) {
  const FilmPair P = pairs[blockIdx.y];
  double acc = 0.0;
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < P.n; i += (long long)gridDim.x * 256) {
    double d = (double)P.a[i] * P.ia - (double)P.b[i] * P.ib;
    if (isfinite(d)) acc += d * d;
  }
  __shared__ double sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = sh[0];
}
__global__ void k_film_rmse_finish(const FilmPair *pairs, int npairs, int per, const double *partials,
                                   double *out) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int k = 0; k < per; ++k) acc += partials[(size_t)p * per + k];
    out[p] = 0.5 * sqrt(acc / (double)pairs[p].n);
  }
}
// a = (a + b) * inv: the mean image of a request from its two half films.
__global__ void k_film_combine(float *a, const float *b, float inv, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = (a[i] + b[i]) * inv;
}

// FrameBuffer::gaussianBlur (framebuffer.cpp:60-129): the full k x k kernel
// (weights computed on the host exactly as the reference does) over the film
// with clamp-to-edge, taps summed row-major in the reference's order with
// rounded, never-fused operations, one thread per pixel.
__global__ void k_gaussian_blur(const float *in, float *out, int W, int H, int K, const float *w) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < W * H; p += gridDim.x * blockDim.x) {
    const int i = p / W, j = p % W;  // row, column (row 0 = bottom, as the film)
    float cx = 0.f, cy = 0.f, cz = 0.f;
    for (int s = 0; s < K; ++s) {
      const int ix = min(max(i - K / 2 + s, 0), H - 1);
      for (int t = 0; t < K; ++t) {
        const int iy = min(max(j - K / 2 + t, 0), W - 1);
        const float wt = __ldg(w + s * K + t);
        const float *q = in + 3 * ((size_t)ix * W + iy);
        cx = __fadd_rn(cx, __fmul_rn(__ldg(q), wt));
        cy = __fadd_rn(cy, __fmul_rn(__ldg(q + 1), wt));
        cz = __fadd_rn(cz, __fmul_rn(__ldg(q + 2), wt));
      }
    }
    out[3 * (size_t)p] = cx;
    out[3 * (size_t)p + 1] = cy;
    out[3 * (size_t)p + 2] = cz;
  }
}

// FrameBuffer::writeToFile pixel path (framebuffer.cpp:27-58).
__global__ void k_tonemap(const float *film, int W, int H, float inv_gamma, uint8_t *out) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < W * H * 3; t += gridDim.x * blockDim.x) {
    int c = t % 3, p = t / 3, i = p % W, j = p / W;
    float v = film[t];
    if (v != v)
      v = 0.f;
    else
      v = powf(v, inv_gamma);
    v = fminf(fmaxf(v, 0.f), 1.f);
    out[((H - 1 - j) * W + i) * 3 + c] = (uint8_t)(v * 255.f);
  }
}

// ---------------------------------------------------------------- launchers
void upload_halton_tables(const HaltonTables &T, cudaStream_t st) {
  cudaMemcpyToSymbolAsync(c_halton, &T, sizeof(T), 0, cudaMemcpyHostToDevice, st);
}


void launch_sampler_eval(int strategy, const uint16_t *perm, uint32_t first, int n, int dims,
                         float *out, cudaStream_t st) {
  long long tot = (long long)n * dims;
  k_sampler_eval<<<grid_for((int)std::min<long long>(tot, 1 << 30), 256, 152 * 16), 256, 0, st>>>(
      strategy, perm, first, n, dims, out);
}

void launch_trace_test(const SceneView &S, bool any, const float *rays, const float *tmaxs, int n,
                       float tmin, float tmax, float *t, int *prim, float *uv, uint8_t *occ, int *err,
                       cudaStream_t st) {
  int g = grid_for(n, 128, 152 * 8);
  if (any)
    k_trace_test<true><<<g, 128, stack_bytes(S, 128), st>>>(S, rays, tmaxs, n, tmin, tmax, t, prim, uv, occ, err);
  else
    k_trace_test<false><<<g, 128, stack_bytes(S, 128), st>>>(S, rays, tmaxs, n, tmin, tmax, t, prim, uv, occ, err);
}

void launch_bsdf_eval(const MatRec *m, int n, const float *wo, const float *wi, const float *nrm,
                      const uint8_t *front, float *f, float *pdf, cudaStream_t st) {
  k_bsdf_eval<<<grid_for(n, 128, 152 * 8), 128, 0, st>>>(m, n, wo, wi, nrm, front, f, pdf);
}
void launch_bsdf_sample(const MatRec *m, int n, const float *wo, const float *nrm,
                        const uint8_t *front, const float *uc, const float *u, uint8_t *ok,
                        float *wi, float *att, float *pdf, uint32_t *type, cudaStream_t st) {
  k_bsdf_sample<<<grid_for(n, 128, 152 * 8), 128, 0, st>>>(m, n, wo, nrm, front, uc, u, ok, wi, att,
                                                          pdf, type);
}

// One wave of a single job: camera, max_depth (+1 for MIS) bounces, film.
void launch_wave(const SceneView &S, const DeviceJob &J, const Queues &Q, long long g0, int n,
                 float *film, const LaunchCfg &cfg, cudaStream_t st, Profiler *prof, cudaEvent_t film_after,
                 cudaEvent_t film_done, const ShadeStreams *ss) {
  const int LN = J.job.light_nx * J.job.light_ny;
  const int bounces = J.job.max_depth + (J.job.estimator == PT_EST_NEE_MIS ? 1 : 0);
  Profiler dummy;
  Profiler &P = prof ? *prof : dummy;
  const JobTable none{nullptr, nullptr, 0};
  launch_wave_stages<false>(S, J, none, Q, g0, n, LN, bounces, cfg, st, P, ss);
  if (film_after) cudaStreamWaitEvent(st, film_after, 0);
  P.begin(STAGE_FILM, st);
  launch_film(J, Q, g0, n, 0, film, cfg, st);
  P.end(st);
  P.count(STAGE_FILM, 1);
  if (film_done) cudaEventRecord(film_done, st);
}

void launch_sort(const SceneView &S, const Queues &Q, int qsel, const LaunchCfg &cfg, cudaStream_t st) {
  cudaMemsetAsync(Q.bins, 0, sizeof(int) * 2 * PT_SORT_BINS, st);
  k_sort_hist<<<cfg.max_blocks_simple, 256, 0, st>>>(S, Q, qsel);
  k_sort_scatter<<<cfg.max_blocks_simple, 256, 0, st>>>(Q, qsel);
}

void launch_shadow(const SceneView &S, const Queues &Q, int LN, const LaunchCfg &cfg, cudaStream_t st) {
  if (S.curves)
    k_trace_shadow<true><<<cfg.trace_blocks, 128, stack_bytes(S, 128), st>>>(S, Q, LN);
  else
    k_trace_shadow<false><<<cfg.trace_blocks, 128, stack_bytes(S, 128), st>>>(S, Q, LN);
  k_shadow_resolve<<<cfg.max_blocks_simple, 256, 0, st>>>(Q, LN);
}
void launch_shadow_resolve(const Queues &Q, int LN, const LaunchCfg &cfg, cudaStream_t st) {
  k_shadow_resolve<<<cfg.max_blocks_simple, 256, 0, st>>>(Q, LN);
}

void launch_film(const DeviceJob &J, const Queues &Q, long long lo, int cnt, long long slot0, float *film,
                 const LaunchCfg &cfg, cudaStream_t st) {
  k_film<<<grid_for(std::min<long long>((long long)J.job.width * J.job.height, 1 << 30), 256,
                    cfg.max_blocks_simple),
           256, 0, st>>>(J, Q, lo, cnt, slot0, film);
}

void launch_film_rmse(const FilmPair *pairs, int npairs, double *partials, double *out, cudaStream_t st) {
  if (npairs <= 0) return;
  k_film_rmse<<<dim3(PT_RMSE_BLOCKS, npairs), 256, 0, st>>>(pairs, partials);
  k_film_rmse_finish<<<grid_for(npairs, 128, 152), 128, 0, st>>>(pairs, npairs, PT_RMSE_BLOCKS, partials, out);
}
void launch_film_combine(float *a, const float *b, float inv, long long n, cudaStream_t st) {
  k_film_combine<<<grid_for((int)std::min<long long>(n, 1 << 30), 256, 152 * 8), 256, 0, st>>>(a, b, inv, n);
}

void launch_gaussian_blur(const float *in, float *out, int W, int H, int K, const float *w, cudaStream_t st) {
  k_gaussian_blur<<<grid_for((long long)W * H, 128, 152 * 16), 128, 0, st>>>(in, out, W, H, K, w);
}

void launch_tonemap(const float *film, int W, int H, float gamma, uint8_t *out, cudaStream_t st) {
  k_tonemap<<<grid_for(W * H * 3, 256, 152 * 8), 256, 0, st>>>(film, W, H, 1.f / gamma, out);
}

void kernel_attributes(KernelInfo *info) {
  cudaFuncAttributes a;
  cudaFuncGetAttributes(&a, k_trace_closest<false, false>);
  info->trace_regs = a.numRegs;
  cudaFuncGetAttributes(&a, k_shade<-1, false>);
  info->shade_regs = a.numRegs;
  int nb = 0;
  // occupancy at the largest stack (the grids must fit every scene)
  const size_t smax = (size_t)PT_STACK * 128 * sizeof(int32_t);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_trace_closest<false, false>, 128, smax);
  info->trace_blocks_per_sm = nb;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_shade<-1, false>, 128, 0);
  info->shade_blocks_per_sm = nb;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_trace_shadow<false>, 128, smax);
  info->shadow_blocks_per_sm = nb;
  int *fb = info->shade_fam_blocks_per_sm;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fb[0], k_shade<0, false>, 128, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fb[1], k_shade<1, false>, 128, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fb[2], k_shade<2, false>, 128, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fb[3], k_shade<3, false>, 128, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fb[4], k_shade<4, false>, 128, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fb[5], k_shade<5, false>, 128, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fb[6], k_shade<6, false>, 128, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fb[PT_FAM_MISC], k_shade<PT_FAM_MISC, false>, 128, 0);
  fb[PT_FAM_MISC + 1] = info->shade_blocks_per_sm;
}

}  // namespace pt
