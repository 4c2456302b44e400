// pt_batch.cpp -- batched rendering: many jobs (different scenes, sizes, spp)
// in ONE CUDA-graph launch.
//
// Every job of a batch gets its own work queues, offset table and device
// film (reused across calls) and its own branch of the graph: the branch runs
// the job's waves (camera, bounces of trace / sort / shade / shadow, film) on
// a stream forked from the context's stream, so the jobs' kernels run
// concurrently on the device and share the resident scenes' BVHs.  The graph
// is captured once per batch composition and replayed while the composition
// is unchanged.  Results per job are independent of the batch: a path's
// sample streams depend only on its own job.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "pt_batch.h"

namespace pt {

Batch::~Batch() {
  if (exec) cudaGraphExecDestroy(exec);
  for (auto &s : slots) s.release();
  if (fork) cudaEventDestroy(fork);
}

void BatchSlot::release() {
  for (void *p : mem) cudaFree(p);
  mem.clear();
  cap = ln = 0;
  if (offsets) cudaFree(offsets);
  offsets = nullptr;
  offsets_cap = 0;
  if (film) cudaFree(film);
  film = nullptr;
  film_cap = 0;
  if (stream) cudaStreamDestroy(stream);
  stream = nullptr;
  if (done) cudaEventDestroy(done);
  done = nullptr;
}

void BatchSlot::ensure(int want_cap, int want_ln, size_t film_floats, int spp) {
  if (!stream) cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
  if (!done) cuda_check(cudaEventCreateWithFlags(&done, cudaEventDisableTiming), "cudaEventCreate");
  if (want_cap > cap || want_ln > ln) {
    for (void *p : mem) cudaFree(p);
    mem.clear();
    auto alloc = [&](size_t bytes) {
      void *p = nullptr;
      cuda_check(cudaMalloc(&p, bytes), "cudaMalloc(batch queues)");
      mem.push_back(p);
      return p;
    };
    const size_t c = (size_t)want_cap;
    Q.cap = want_cap;
    Q.beta = (float4 *)alloc(c * 16);
    Q.L = (float4 *)alloc(c * 16);
    Q.ray_o[0] = (float4 *)alloc(c * 16);
    Q.ray_o[1] = (float4 *)alloc(c * 16);
    Q.ray_d[0] = (float4 *)alloc(c * 16);
    Q.ray_d[1] = (float4 *)alloc(c * 16);
    Q.hit = (float4 *)alloc(c * 16);
    Q.sh_o = (float4 *)alloc(c * 16);
    Q.sh_d = (float4 *)alloc(c * 16 * want_ln);
    Q.sh_c = (float4 *)alloc(c * 16 * want_ln);
    Q.sh_vis = (uint8_t *)alloc(c * want_ln);
    Q.counts = (int *)alloc(64);
    Q.stats = (unsigned long long *)alloc(64);
    Q.err = (int *)alloc(16);
    Q.sort_key = (int *)alloc(c * 4);
    Q.order = (int *)alloc(c * 4);
    Q.bins = (int *)alloc(sizeof(int) * 2 * PT_SORT_BINS);
    Q.seg = (int *)alloc(sizeof(int) * (PT_SORT_BINS + 1));
    cuda_check(cudaMemset(Q.err, 0, 16), "memset err");
    cap = want_cap;
    ln = want_ln;
  }
  if (spp > offsets_cap) {
    if (offsets) cudaFree(offsets);
    offsets = nullptr;
    cuda_check(cudaMalloc(&offsets, sizeof(float2) * spp), "cudaMalloc(batch offsets)");
    offsets_cap = spp;
  }
  if (film_floats > film_cap) {
    if (film) cudaFree(film);
    film = nullptr;
    cuda_check(cudaMalloc(&film, film_floats * sizeof(float)), "cudaMalloc(batch film)");
    film_cap = film_floats;
  }
}

static std::string signature(const pt_job_desc *jobs, int n, const LaunchCfg &cfg, int per_job_cap,
                             float **targets) {
  std::string s((const char *)jobs, (const char *)(jobs + n));
  s.append((const char *)&cfg, sizeof cfg);
  s.append((const char *)&per_job_cap, sizeof per_job_cap);
  if (targets) s.append((const char *)targets, sizeof(float *) * n);
  return s;
}

// Renders the batch; films[k] (host, may be null) receive job k's mean image.
void render_batch(Context *c, const pt_job_desc *jobs, int n, float **films, pt_stats *stats,
                  float **targets) {
  Batch &B = c->batch;
  if (!B.fork) cuda_check(cudaEventCreateWithFlags(&B.fork, cudaEventDisableTiming), "cudaEventCreate");
  if ((int)B.slots.size() < n) B.slots.resize(n);
  std::vector<DeviceJob> dj(n);
  std::vector<Scene *> scenes(n);
  std::vector<long long> total(n);
  std::vector<int> wave(n);
  for (int k = 0; k < n; ++k) {
    const pt_job_desc &j = jobs[k];
    validate_job(j);
    scenes[k] = c->scene(j.scene);
    dj[k] = c->device_job(j, scenes[k]);
    const long long npix = (long long)j.width * j.height;
    const int e = j.spp_end ? j.spp_end : j.spp_x * j.spp_y;
    total[k] = npix * (e - j.spp_begin);
    int w = c->batch_wave_cap;
    if (npix <= w) w = (int)((w / npix) * npix);
    if ((long long)w > total[k]) w = (int)total[k];
    wave[k] = w;
    BatchSlot &s = B.slots[k];
    s.ensure(w, j.light_samples_x * j.light_samples_y, (size_t)npix * 3, j.spp_x * j.spp_y);
    std::vector<float2> off = make_offsets(j);
    cuda_check(cudaMemcpyAsync(s.offsets, off.data(), off.size() * sizeof(float2), cudaMemcpyHostToDevice,
                               c->stream),
               "upload offsets");
    dj[k].job.offsets = s.offsets;
  }
  cuda_check(cudaStreamSynchronize(c->stream), "batch set-up");
  const std::string sig = signature(jobs, n, c->cfg, c->batch_wave_cap, targets);
  if (!B.exec || sig != B.sig) {
    cudaGraph_t graph = nullptr;
    cuda_check(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaEventRecord(B.fork, c->stream);
    for (int k = 0; k < n; ++k) {
      BatchSlot &s = B.slots[k];
      const pt_job_desc &j = jobs[k];
      cudaStreamWaitEvent(s.stream, B.fork, 0);
      cudaMemsetAsync(s.Q.stats, 0, 64, s.stream);
      // targets: device films the samples are added onto; else the slot film
      float *dst = targets ? targets[k] : s.film;
      if (!targets) cudaMemsetAsync(s.film, 0, sizeof(float) * (size_t)j.width * j.height * 3, s.stream);
      LaunchCfg lc = c->cfg;
      lc.family_mask = scenes[k]->family_mask;
      for (long long g0 = 0; g0 < total[k]; g0 += wave[k]) {
        int cnt = (int)std::min<long long>(wave[k], total[k] - g0);
        launch_wave(scenes[k]->view, dj[k], s.Q, g0, cnt, dst, lc, s.stream, nullptr);
      }
      cudaEventRecord(s.done, s.stream);
      cudaStreamWaitEvent(c->stream, s.done, 0);
    }
    cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
    cuda_check(ce, "end capture");
    // Same topology (e.g. the next pass of the same requests, only sample
    // ranges and films changed): update the executable graph's parameters in
    // place; otherwise instantiate anew.
    bool updated = false;
    if (B.exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(B.exec, graph, &info) == cudaSuccess) {
        updated = true;
        ++B.updates;
      } else {
        (void)cudaGetLastError();
        cudaGraphExecDestroy(B.exec);
        B.exec = nullptr;
      }
    }
    if (!updated) {
      cudaError_t ie = cudaGraphInstantiate(&B.exec, graph, 0);
      if (ie != cudaSuccess) {
        cudaGraphDestroy(graph);
        B.exec = nullptr;
        cuda_check(ie, "graph instantiate");
      }
      ++B.captures;
    }
    cudaGraphDestroy(graph);
    B.sig = sig;
  }
  ++B.launches;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c->stream);
  cuda_check(cudaGraphLaunch(B.exec, c->stream), "graph launch");
  cudaEventRecord(e1, c->stream);
  cuda_check(cudaStreamSynchronize(c->stream), "batch render");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  pt_stats tot;
  std::memset(&tot, 0, sizeof tot);
  for (int k = 0; k < n; ++k) {
    BatchSlot &s = B.slots[k];
    int herr = 0;
    cuda_check(cudaMemcpy(&herr, s.Q.err, sizeof(int), cudaMemcpyDeviceToHost), "read err");
    if (herr) {
      cudaMemset(s.Q.err, 0, sizeof(int));
      fail(PT_ERR_DEVICE, "device traversal error flag in batch job " + std::to_string(k));
    }
    unsigned long long h[4];
    cuda_check(cudaMemcpy(h, s.Q.stats, sizeof h, cudaMemcpyDeviceToHost), "read stats");
    tot.paths += h[0];
    tot.segments += h[1];
    tot.rays += h[2];
    tot.shadow_rays += h[3];
    const pt_job_desc &j = jobs[k];
    if (!targets && films && films[k]) {
      const size_t nf = (size_t)j.width * j.height * 3;
      cuda_check(cudaMemcpy(films[k], s.film, nf * sizeof(float), cudaMemcpyDeviceToHost), "film d2h");
      const int e = j.spp_end ? j.spp_end : j.spp_x * j.spp_y;
      const float inv = 1.f / (float)(e - j.spp_begin);
      for (size_t i = 0; i < nf; ++i) films[k][i] *= inv;
    }
  }
  tot.ms = ms;
  tot.algorithmic_bytes = 192ull * tot.segments + 88ull * tot.shadow_rays + 24ull * tot.paths;
  if (stats) *stats = tot;
}

// Autotuner: renders the batch under candidate launch configurations
// (wave capacity per job, material sorting, blocks per SM of the traversal
// and shade kernels), keeps the fastest in the context and reports it.
void autotune(Context *c, const pt_job_desc *jobs, int n, pt_tuning *out) {
  const LaunchCfg base = c->cfg;
  const int base_wave = c->batch_wave_cap;
  struct Cand {
    int wave, sort, tmul, smul;
  };
  std::vector<Cand> cands;
  for (int wave : {1 << 20, 1 << 22, 1 << 24})
    for (int sort : {0, 1})
      for (int tmul : {1, 2})
        for (int smul : {1, 2}) cands.push_back({wave, sort, tmul, smul});
  double best = 1e30, dflt = -1.0;
  Cand bc = {base_wave, base.sort_by_material, 1, 1};
  for (const Cand &cd : cands) {
    c->cfg = base;
    c->cfg.sort_by_material = cd.sort;
    c->cfg.trace_blocks = base.trace_blocks * cd.tmul;
    c->cfg.shade_blocks = base.shade_blocks * cd.smul;
    c->batch_wave_cap = cd.wave;
    pt_stats st;
    render_batch(c, jobs, n, nullptr, &st);  // capture + warm
    double t = 1e30;
    for (int r = 0; r < 2; ++r) {
      render_batch(c, jobs, n, nullptr, &st);
      t = std::min(t, st.ms);
    }
    if (cd.wave == base_wave && cd.sort == base.sort_by_material && cd.tmul == 1 && cd.smul == 1) dflt = t;
    if (t < best) {
      best = t;
      bc = cd;
    }
  }
  c->cfg = base;
  c->cfg.sort_by_material = bc.sort;
  c->cfg.trace_blocks = base.trace_blocks * bc.tmul;
  c->cfg.shade_blocks = base.shade_blocks * bc.smul;
  c->batch_wave_cap = bc.wave;
  if (out) {
    out->wave_paths = bc.wave;
    out->sort_by_material = bc.sort;
    out->trace_blocks = c->cfg.trace_blocks;
    out->shade_blocks = c->cfg.shade_blocks;
    out->best_ms = best;
    out->default_ms = dflt;
    out->candidates = (int32_t)cands.size();
  }
}

}  // namespace pt
