// pt_kernels.h -- host-visible interface of the wavefront kernels
// (pt_kernels.cu) used by the C-ABI layer (pt_host.cpp).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>
#include "../../include/pathtracer_gb300.h"
#include "pt_scene.cuh"

#define PT_MAX_LIGHT_SAMPLES 16
#define PT_SORT_BINS 16
// Sort keys: material type 0..7 of a surface hit, then misses and medium
// events.  The shade kernel of family PT_FAM_MISC covers keys 7..9
// (emitters, misses, medium events).
#define PT_KEY_MISS 8
#define PT_KEY_MEDIUM 9
#define PT_FAM_MISC 7
#define PT_HIT_MEDIUM (-2)

namespace pt {

struct DeviceJob {
  JobView job;
  const uint16_t *perm;  // PermuteDigits tables for job.sampler_seed
};

// Jobs of a merged wave (batched and served forms): the merged path index
// g in [start[k], start[k+1]) is path g - start[k] of job k.
struct JobTable {
  const DeviceJob *jobs;   // [n]
  const long long *start;  // [n + 1], start[0] = 0
  int n;
};

// Work queues of one context, sized for `cap` paths per wave (SoA in HBM).
struct Queues {
  int cap;
  float4 *beta;       // throughput.xyz, pdf of the sampled continuation (<0: delta)
  float4 *L;          // radiance accumulated by the path
  float4 *ray_o[2];   // RayQueue ping-pong: origin.xyz, path slot (int bits)
  float4 *ray_d[2];   //                     direction.xyz
  float4 *hit;        // HitQueue: t, prim (int bits), u, v
  float4 *sh_o;       // ShadowQueue: origin.xyz, path slot
  float4 *sh_d;       // [light sample][cap]: direction.xyz, tmax (<0: none)
  float4 *sh_c;       // [light sample][cap]: unoccluded contribution
  uint8_t *sh_vis;    // [light sample][cap]: 1 = the shadow ray reached the light
  int *counts;        // [0],[1] ray queues, [2] shadow queue, [3] [4] fetch counters
  unsigned long long *stats;  // [0] paths [1] segments [2] rays [3] shadow rays
  int *err;           // device error flag (stack overflow / iteration cap)
  int *job;           // [cap] merged waves: job index of the path in each slot
  int *sort_key, *order, *bins;
  int *seg;           // [PT_SORT_BINS + 1] segment bounds of the sorted order
};

struct LaunchCfg {
  int trace_blocks;
  int shade_blocks;                       // grid of the generic shade kernel
  int shade_fam_blocks[PT_FAM_MISC + 2];  // grid per family (0..PT_FAM_MISC), generic last
  int max_blocks_simple;
  int sort_by_material;
  unsigned family_mask;  // material types present in the scene (bit per type)
  int pair_trace;        // waves of at most this many paths trace the shadow rays of
                         // bounce b with the closest rays of b + 1 (0: never)
  int pair_from_bounce;  // larger waves do so from this bounce on (0: from the
                         // roulette start of a single-job wave)
};

// Side streams of one wave's stream: a bounce's per-family shade kernels
// are independent (each owns its segment of the sorted queue and its paths;
// queue slots come from atomics), so they run concurrently on the wave's
// stream and these, forked and joined by events -- in a captured graph,
// parallel branches.  One set per stream that runs waves.
struct ShadeStreams {
  static constexpr int N = 3;
  cudaStream_t aux[N] = {};
  cudaEvent_t fork = nullptr, join[N] = {};
  bool ready() const { return fork != nullptr; }
  void create() {
    if (fork) return;
    for (int i = 0; i < N; ++i) {
      cudaStreamCreateWithFlags(&aux[i], cudaStreamNonBlocking);
      cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming);
    }
    cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
  }
  void destroy() {
    if (!fork) return;
    for (int i = 0; i < N; ++i) {
      cudaStreamDestroy(aux[i]);
      cudaEventDestroy(join[i]);
      aux[i] = nullptr;
      join[i] = nullptr;
    }
    cudaEventDestroy(fork);
    fork = nullptr;
  }
};

// Per-stage CUDA-event timing of the wave kernels (pt_profile_begin/end).
enum StageKind { STAGE_CAMERA = 0, STAGE_TRACE, STAGE_SORT, STAGE_SHADE, STAGE_SHADOW, STAGE_FILM, STAGE_COUNT };
struct Profiler {
  bool on = false;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  std::vector<int> kinds;  // per begin/end event pair
  long long kernels[STAGE_COUNT] = {};  // kernel launches per stage while on
  void count(int kind, int n) {
    if (on) kernels[kind] += n;
  }
  cudaEvent_t take() {
    if (used == pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pool.push_back(e);
    }
    return pool[used++];
  }
  void begin(int kind, cudaStream_t st) {
    if (!on) return;
    cudaEventRecord(take(), st);
    kinds.push_back(kind);
  }
  void end(cudaStream_t st) {
    if (!on) return;
    cudaEventRecord(take(), st);
  }
};

struct KernelInfo {
  int trace_regs, shade_regs;
  int trace_blocks_per_sm, shade_blocks_per_sm, shadow_blocks_per_sm;
  int shade_fam_blocks_per_sm[PT_FAM_MISC + 2];  // per family, generic last
};

void upload_halton_tables(const HaltonTables &T, cudaStream_t st);
void launch_light_eval(const SceneView &S, int light, int n, const float *uv, const float *x, const float *pdf_dir,
                       float *point, float *normal, float *dir, float *le, float *pdf, cudaStream_t st);
void launch_intersect(const SceneView &S, const float *rays, int n, float tmin, float tmax, float *t, int *prim,
                      float *pos, float *nrm, uint8_t *front, int *err, cudaStream_t st);
void launch_path_samples(const DeviceJob &J, long long first, int n, int dims, int bounces, float *pix, float *dv,
                         float *lo, cudaStream_t st);
void launch_sampler_eval(int strategy, const uint16_t *perm, uint32_t first, int n, int dims,
                         float *out, cudaStream_t st);
void launch_trace_test(const SceneView &S, bool any, const float *rays, const float *tmaxs, int n,
                       float tmin, float tmax, float *t, int *prim, float *uv, uint8_t *occ,
                       int *err, cudaStream_t st);
void launch_bsdf_eval(const MatRec *m, int n, const float *wo, const float *wi, const float *nrm,
                      const uint8_t *front, float *f, float *pdf, cudaStream_t st);
void launch_bsdf_sample(const MatRec *m, int n, const float *wo, const float *nrm,
                        const uint8_t *front, const float *uc, const float *u, uint8_t *ok,
                        float *wi, float *att, float *pdf, uint32_t *type, cudaStream_t st);
// film_after (may be null): the film stage waits for it; film_done (may be
// null) is recorded after this wave's film stage (wave order across streams).
// ss (may be null): the stream's side streams for concurrent shade kernels.
void launch_wave(const SceneView &S, const DeviceJob &J, const Queues &Q, long long g0, int n,
                 float *film, const LaunchCfg &cfg, cudaStream_t st, Profiler *prof,
                 cudaEvent_t film_after = nullptr, cudaEvent_t film_done = nullptr,
                 const ShadeStreams *ss = nullptr);
// Job-independent stages (pt_kernels.cu), also used by merged waves.
void launch_sort(const SceneView &S, const Queues &Q, int qsel, const LaunchCfg &cfg, cudaStream_t st);
void launch_shadow(const SceneView &S, const Queues &Q, int LN, const LaunchCfg &cfg, cudaStream_t st);
void launch_shadow_resolve(const Queues &Q, int LN, const LaunchCfg &cfg, cudaStream_t st);
// Adds paths [lo, lo + cnt) of job J (held in wave slots slot0..) to its
// film, per pixel in sample order.
void launch_film(const DeviceJob &J, const Queues &Q, long long lo, int cnt, long long slot0, float *film,
                 const LaunchCfg &cfg, cudaStream_t st);

// A merged wave over the jobs of one scene (pt_kernels_multi.cu): device job
// table + host copies for the per-job film stage.
struct MergedJobs {
  JobTable T;                    // device pointers
  std::vector<DeviceJob> jobs;   // host copies
  std::vector<long long> start;  // host copy, n + 1 entries
  std::vector<float *> films;    // device film of each job (samples are added)
  int bounces = 0;               // max over the jobs of max_depth (+1 with MIS)
  int LN = 1;                    // light samples per vertex (equal for all jobs)
};
// film_after (may be null): the film stage waits for it (the previous
// wave's films, on another stream); film_done (may be null) is recorded after
// this wave's films.
void launch_wave_multi(const SceneView &S, const MergedJobs &M, const Queues &Q, long long g0, int n,
                       const LaunchCfg &cfg, cudaStream_t st, Profiler *prof, cudaEvent_t film_after = nullptr,
                       cudaEvent_t film_done = nullptr, const ShadeStreams *ss = nullptr);
void upload_halton_tables_multi(const HaltonTables &T, cudaStream_t st);
// Persistent form of a merged group (pt_kernels_persist.cu): every wave and
// bounce of the group in one cooperative launch of `grid` blocks;
// d_barrier: 16 zeroed bytes (the grid barrier; its third int is set when a
// barrier wait ran out).  persistent_grid: the resident-block grid.
void upload_halton_tables_persist(const HaltonTables &T, cudaStream_t st);
int persistent_grid(const SceneView &S, int num_sms);
cudaError_t launch_group_persistent(const SceneView &S, const JobTable &T, const Queues &Q, float *const *d_films,
                                    long long total, int wave, int LN, int bounces, void *d_barrier, int grid,
                                    cudaStream_t st);
void launch_tonemap(const float *film, int W, int H, float gamma, uint8_t *out, cudaStream_t st);
void launch_gaussian_blur(const float *in, float *out, int W, int H, int K, const float *w, cudaStream_t st);

// Serving: RMSE estimates from half films (see k_film_rmse) and the final
// mean image.  partials holds PT_RMSE_BLOCKS doubles per pair.
#define PT_RMSE_BLOCKS 64
struct FilmPair {
  const float *a, *b;
  double ia, ib;  // 1 / samples in a, b
  long long n;    // floats per film
};
void launch_film_rmse(const FilmPair *pairs, int npairs, double *partials, double *out, cudaStream_t st);
void launch_film_combine(float *a, const float *b, float inv, long long n, cudaStream_t st);
void kernel_attributes(KernelInfo *info);

}  // namespace pt
