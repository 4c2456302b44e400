// pt_batch.cpp -- batched rendering: many jobs (different scenes, sizes, spp,
// cameras) in ONE CUDA-graph launch of merged waves.
//
// The jobs are grouped by scene and light-sample count.  A group's jobs are
// concatenated into one sequence of paths (job k owns merged indices
// [start[k], start[k+1])) and rendered in waves over that sequence: every
// kernel of a bounce processes the paths of all the group's jobs at once,
// looking up each path's job in a table in HBM, so a small job costs its
// paths and not a chain of kernel launches of its own.  Each group runs on
// its own branch of the graph (a stream forked from the context's stream);
// the groups share nothing but the resident scenes.  The graph is captured
// per batch composition and updated in place when only parameters change.
//
// A job's result does not depend on the batch: a path's sample streams depend
// only on its own job, and films add samples one by one in sample order
// whatever the wave boundaries.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "pt_batch.h"

namespace pt {

Batch::~Batch() {
  if (exec) cudaGraphExecDestroy(exec);
  for (auto &s : slots) s.release();
  if (fork) cudaEventDestroy(fork);
  for (cudaEvent_t e : film_events) cudaEventDestroy(e);
}

void BatchSlot::release() {
  for (void *p : mem) cudaFree(p);
  mem.clear();
  cap = ln = 0;
  auto fr = [](auto *&p) {
    if (p) cudaFree(p);
    p = nullptr;
  };
  fr(d_jobs);
  fr(d_start);
  fr(offsets);
  fr(films);
  fr(d_films);
  fr(d_barrier);
  d_films_cap = 0;
  jobs_cap = 0;
  offsets_cap = films_cap = 0;
  for (int h = 0; h < 2; ++h) {
    if (stream[h]) cudaStreamDestroy(stream[h]);
    stream[h] = nullptr;
    if (done[h]) cudaEventDestroy(done[h]);
    done[h] = nullptr;
    side[h].destroy();
  }
}

void BatchSlot::ensure(int want_cap, int want_ln, int n_jobs, size_t n_offsets, size_t film_floats) {
  for (int h = 0; h < 2; ++h) {
    if (!stream[h]) cuda_check(cudaStreamCreateWithFlags(&stream[h], cudaStreamNonBlocking), "cudaStreamCreate");
    if (!done[h]) cuda_check(cudaEventCreateWithFlags(&done[h], cudaEventDisableTiming), "cudaEventCreate");
    side[h].create();
  }
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
    for (int h = 0; h < 2; ++h) {
      Queues &Q = this->Q[h];
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
      Q.job = (int *)alloc(c * 4);
      Q.bins = (int *)alloc(sizeof(int) * 2 * PT_SORT_BINS);
      Q.seg = (int *)alloc(sizeof(int) * (PT_SORT_BINS + 1));
      cuda_check(cudaMemset(Q.err, 0, 16), "memset err");
    }
    cap = want_cap;
    ln = want_ln;
  }
  if (n_jobs > jobs_cap) {
    if (d_jobs) cudaFree(d_jobs);
    if (d_start) cudaFree(d_start);
    d_jobs = nullptr;
    d_start = nullptr;
    cuda_check(cudaMalloc(&d_jobs, sizeof(DeviceJob) * n_jobs), "cudaMalloc(batch jobs)");
    cuda_check(cudaMalloc(&d_start, sizeof(long long) * (n_jobs + 1)), "cudaMalloc(batch starts)");
    jobs_cap = n_jobs;
  }
  if (n_offsets > offsets_cap) {
    if (offsets) cudaFree(offsets);
    offsets = nullptr;
    cuda_check(cudaMalloc(&offsets, sizeof(float2) * n_offsets), "cudaMalloc(batch offsets)");
    offsets_cap = n_offsets;
  }
  if (film_floats > films_cap) {
    if (films) cudaFree(films);
    films = nullptr;
    cuda_check(cudaMalloc(&films, film_floats * sizeof(float)), "cudaMalloc(batch films)");
    films_cap = film_floats;
  }
}

// One merged group: the jobs (indices into the batch) of one scene and one
// light-sample count, in batch order.
struct Group {
  int scene;
  int ln;
  std::vector<int> members;
  MergedJobs M;
  long long total = 0;
  int wave = 0;
  std::vector<size_t> film_off;  // offset of each member's film in the slot's film array
  size_t film_floats = 0;
};

static std::string signature(const pt_job_desc *jobs, int n, const LaunchCfg &cfg, int per_group_cap,
                             float **targets) {
  std::string s((const char *)jobs, (const char *)(jobs + n));
  s.append((const char *)&cfg, sizeof cfg);
  s.append((const char *)&per_group_cap, sizeof per_group_cap);
  if (targets) s.append((const char *)targets, sizeof(float *) * n);
  return s;
}

// The groups as branches of ONE CUDA graph (captured per batch composition,
// updated in place when only parameters change): per-stage kernels of merged
// waves; returns the graph's device milliseconds.
static float render_groups_graph(Context *c, const pt_job_desc *jobs, int n, std::vector<Group> &groups,
                                 float **targets) {
  Batch &B = c->batch;
  const std::string sig = signature(jobs, n, c->cfg, c->batch_wave_cap, targets);
  if (!B.exec || sig != B.sig) {
    cudaGraph_t graph = nullptr;
    cuda_check(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaEventRecord(B.fork, c->stream);
    size_t n_events = 0;
    for (const Group &G : groups) n_events += (size_t)((G.total + G.wave - 1) / G.wave);
    while (B.film_events.size() < n_events) {
      cudaEvent_t e;
      cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
      B.film_events.push_back(e);
    }
    size_t ev = 0;
    for (size_t gi = 0; gi < groups.size(); ++gi) {
      Group &G = groups[gi];
      BatchSlot &slot = B.slots[gi];
      Scene *S = c->scene(G.scene);
      for (int h = 0; h < 2; ++h) {
        cudaStreamWaitEvent(slot.stream[h], B.fork, 0);
        cudaMemsetAsync(slot.Q[h].stats, 0, 64, slot.stream[h]);
      }
      if (!targets) cudaMemsetAsync(slot.films, 0, sizeof(float) * G.film_floats, slot.stream[0]);
      LaunchCfg lc = c->cfg;
      lc.family_mask = S->family_mask;
      if (lc.pair_from_bounce <= 0) {
        // paired tracing once the queues thin out: from the group's earliest
        // roulette start when every member uses roulette
        int from = 1 << 20;
        bool all_rr = true;
        for (int m : G.members) {
          if (jobs[m].rr_start < 0)
            all_rr = false;
          else
            from = std::min(from, (int)jobs[m].rr_start);
        }
        lc.pair_from_bounce = all_rr ? std::max(1, from) : (1 << 20);
      }
      // consecutive waves alternate between two queue sets on two streams,
      // so one wave's sparse last bounces overlap the next wave's first
      // ones; the film stages stay in wave order (event chain), which keeps
      // every pixel's samples added in sample order
      cudaEvent_t prev = nullptr;
      int w = 0;
      for (long long g0 = 0; g0 < G.total; g0 += G.wave, ++w) {
        const int cnt = (int)std::min<long long>(G.wave, G.total - g0);
        const int h = w & 1;
        if (w == 1 && !targets) {
          // the film clear on stream 0 precedes every film stage
          cudaEventRecord(slot.done[0], slot.stream[0]);
          cudaStreamWaitEvent(slot.stream[1], slot.done[0], 0);
        }
        cudaEvent_t mine = B.film_events[ev++];
        launch_wave_multi(S->view, G.M, slot.Q[h], g0, cnt, lc, slot.stream[h], nullptr, prev, mine, &slot.side[h]);
        prev = mine;
      }
      for (int h = 0; h < 2; ++h) {
        cudaEventRecord(slot.done[h], slot.stream[h]);
        cudaStreamWaitEvent(c->stream, slot.done[h], 0);
      }
    }
    cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
    cuda_check(ce, "end capture");
    // Same topology (e.g. the server's next pass of the same requests: only
    // sample ranges and target films changed): update the executable graph's
    // parameters in place; otherwise instantiate anew.
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
  return ms;
}

// The groups in the persistent form: one cooperative launch per group that
// runs all its waves and bounces (pt_kernels_persist.cu), the groups one
// after another on the context's stream; returns device milliseconds.
static float render_groups_persistent(Context *c, std::vector<Group> &groups, bool targets) {
  Batch &B = c->batch;
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
  cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
  cudaEventRecord(e0, c->stream);
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    Group &G = groups[gi];
    BatchSlot &slot = B.slots[gi];
    Scene *S = c->scene(G.scene);
    const int nm = (int)G.members.size();
    if (nm > slot.d_films_cap) {
      if (slot.d_films) cudaFree(slot.d_films);
      slot.d_films = nullptr;
      cuda_check(cudaMalloc(&slot.d_films, sizeof(float *) * nm), "cudaMalloc(film table)");
      slot.d_films_cap = nm;
    }
    if (!slot.d_barrier) cuda_check(cudaMalloc(&slot.d_barrier, 16), "cudaMalloc(grid barrier)");
    cuda_check(cudaMemcpyAsync(slot.d_films, G.M.films.data(), sizeof(float *) * nm, cudaMemcpyHostToDevice,
                               c->stream),
               "upload film table");
    cuda_check(cudaMemsetAsync(slot.d_barrier, 0, 16, c->stream), "memset barrier");
    cuda_check(cudaMemsetAsync(slot.Q[0].stats, 0, 64, c->stream), "memset stats");
    cuda_check(cudaMemsetAsync(slot.Q[1].stats, 0, 64, c->stream), "memset stats");
    if (!targets) cuda_check(cudaMemsetAsync(slot.films, 0, sizeof(float) * G.film_floats, c->stream), "memset films");
    const int grid = persistent_grid(S->view, c->num_sms);
    cuda_check(launch_group_persistent(S->view, G.M.T, slot.Q[0], slot.d_films, G.total, G.wave, G.M.LN,
                                       G.M.bounces, slot.d_barrier, grid, c->stream),
               "persistent group launch");
  }
  cudaEventRecord(e1, c->stream);
  cuda_check(cudaStreamSynchronize(c->stream), "batch render");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    int bar[4] = {0, 0, 0, 0};
    cuda_check(cudaMemcpy(bar, B.slots[gi].d_barrier, 16, cudaMemcpyDeviceToHost), "read barrier");
    if (bar[2]) fail(PT_ERR_DEVICE, "persistent batch: a grid barrier wait ran out in group " + std::to_string(gi));
  }
  return ms;
}

// Renders the batch; films[k] (host, may be null) receive job k's mean image;
// with targets, job k's samples are added onto the device film targets[k].
void render_batch(Context *c, const pt_job_desc *jobs, int n, float **films, pt_stats *stats,
                  float **targets) {
  Batch &B = c->batch;
  if (!B.fork) cuda_check(cudaEventCreateWithFlags(&B.fork, cudaEventDisableTiming), "cudaEventCreate");
  // ---- groups
  std::vector<Group> groups;
  std::map<std::pair<int, int>, int> gidx;
  for (int k = 0; k < n; ++k) {
    const pt_job_desc &j = jobs[k];
    validate_job(j);
    c->scene(j.scene);
    const int ln = j.light_samples_x * j.light_samples_y;
    auto key = std::make_pair(j.scene, ln);
    auto it = gidx.find(key);
    if (it == gidx.end()) {
      it = gidx.emplace(key, (int)groups.size()).first;
      groups.push_back(Group{j.scene, ln, {}, {}, 0, 0, {}, 0});
    }
    groups[it->second].members.push_back(k);
  }
  if ((int)B.slots.size() < (int)groups.size()) B.slots.resize(groups.size());
  // ---- tables
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    Group &G = groups[gi];
    Scene *S = c->scene(G.scene);
    MergedJobs &M = G.M;
    M.LN = G.ln;
    M.start.push_back(0);
    size_t n_off = 0, film_floats = 0;
    for (int k : G.members) {
      const pt_job_desc &j = jobs[k];
      const long long npix = (long long)j.width * j.height;
      const int e = j.spp_end ? j.spp_end : j.spp_x * j.spp_y;
      M.start.push_back(M.start.back() + npix * (e - j.spp_begin));
      M.bounces = std::max(M.bounces, j.max_depth + (j.estimator == PT_EST_NEE_MIS ? 1 : 0));
      n_off += (size_t)j.spp_x * j.spp_y;
      G.film_off.push_back(film_floats);
      film_floats += (size_t)npix * 3;
    }
    G.total = M.start.back();
    G.film_floats = film_floats;
    G.wave = (int)std::min<long long>(c->batch_wave_cap, G.total);
    BatchSlot &slot = B.slots[gi];
    slot.ensure(G.wave, G.ln, (int)G.members.size(), n_off, targets ? 1 : film_floats);
    std::vector<float2> offs;
    offs.reserve(n_off);
    for (size_t m = 0; m < G.members.size(); ++m) {
      const pt_job_desc &j = jobs[G.members[m]];
      DeviceJob dj = c->device_job(j, S);
      dj.job.offsets = slot.offsets + offs.size();
      std::vector<float2> o = make_offsets(j);
      offs.insert(offs.end(), o.begin(), o.end());
      M.jobs.push_back(dj);
      M.films.push_back(targets ? targets[G.members[m]] : slot.films + G.film_off[m]);
    }
    cuda_check(cudaMemcpyAsync(slot.offsets, offs.data(), offs.size() * sizeof(float2), cudaMemcpyHostToDevice,
                               c->stream),
               "upload offsets");
    cuda_check(cudaMemcpyAsync(slot.d_jobs, M.jobs.data(), sizeof(DeviceJob) * M.jobs.size(),
                               cudaMemcpyHostToDevice, c->stream),
               "upload job table");
    cuda_check(cudaMemcpyAsync(slot.d_start, M.start.data(), sizeof(long long) * M.start.size(),
                               cudaMemcpyHostToDevice, c->stream),
               "upload job starts");
    M.T = JobTable{slot.d_jobs, slot.d_start, (int)G.members.size()};
  }
  cuda_check(cudaStreamSynchronize(c->stream), "batch set-up");
  float ms = 0.f;
  if (c->batch_mode == PT_BATCH_PERSISTENT)
    ms = render_groups_persistent(c, groups, targets != nullptr);
  else
    ms = render_groups_graph(c, jobs, n, groups, targets);
  // ---- results
  pt_stats tot;
  std::memset(&tot, 0, sizeof tot);
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    Group &G = groups[gi];
    BatchSlot &slot = B.slots[gi];
    for (int q = 0; q < 2; ++q) {
      int herr = 0;
      cuda_check(cudaMemcpy(&herr, slot.Q[q].err, sizeof(int), cudaMemcpyDeviceToHost), "read err");
      if (herr) {
        cudaMemset(slot.Q[q].err, 0, sizeof(int));
        fail(PT_ERR_DEVICE, "device traversal error flag in batch group " + std::to_string(gi));
      }
      unsigned long long h[4];
      cuda_check(cudaMemcpy(h, slot.Q[q].stats, sizeof h, cudaMemcpyDeviceToHost), "read stats");
      tot.paths += h[0];
      tot.segments += h[1];
      tot.rays += h[2];
      tot.shadow_rays += h[3];
    }
    if (targets || !films) continue;
    for (size_t m = 0; m < G.members.size(); ++m) {
      const int k = G.members[m];
      if (!films[k]) continue;
      const pt_job_desc &j = jobs[k];
      const size_t nf = (size_t)j.width * j.height * 3;
      cuda_check(cudaMemcpy(films[k], slot.films + G.film_off[m], nf * sizeof(float), cudaMemcpyDeviceToHost),
                 "film d2h");
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
// (merged wave capacity per group, material sorting, blocks per SM of the
// traversal and shade kernels), keeps the fastest in the context and
// reports it.
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
    for (int f = 0; f < PT_FAM_MISC + 2; ++f) c->cfg.shade_fam_blocks[f] = base.shade_fam_blocks[f] * cd.smul;
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
  for (int f = 0; f < PT_FAM_MISC + 2; ++f) c->cfg.shade_fam_blocks[f] = base.shade_fam_blocks[f] * bc.smul;
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
