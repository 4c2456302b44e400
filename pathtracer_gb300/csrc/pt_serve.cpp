// pt_serve.cpp -- batched rendering and the request server of the C-ABI.
//
// pt_render_batch renders many jobs against resident scenes from one call.
// The server admits requests while free HBM and slots allow, keeps each
// request's film on the device, and in every scheduling pass adds
// spp_per_pass samples to every active request (continuous batching: a
// request submitted while others run joins at the next pass).  Each
// request's result depends only on its own job (seed, sample range), never on
// what else is in flight, so it is identical alone and in a mix.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "pt_batch.h"

namespace pt {

struct Request {
  int64_t id;
  pt_request_desc desc;
  int state = 0;  // 0 queued, 1 running, 2 done, 3 cancelled, 4 failed
  int spp_done = 0;
  float *film_a = nullptr;  // sum of even passes
  float *film_b = nullptr;  // sum of odd passes
  int spp_a = 0, spp_b = 0;
  int passes = 0;  // scheduling passes rendered (even ones go to film_a)
  size_t bytes = 0;
  std::chrono::steady_clock::time_point t_submit, t_admit, t_done;
  bool admitted = false;
  std::vector<float> result;
  std::string error;
  double last_rmse = INFINITY;  // latest estimate of the mean image's RMSE
};

struct Server {
  Context *ctx;
  int64_t budget;
  int max_slots;
  int64_t next_id = 1;
  std::map<int64_t, Request> reqs;
  std::deque<int64_t> queue;
  std::vector<int64_t> active;
  int64_t used = 0;
  // scheduling (pt_server_set_policy)
  int policy = PT_SERVE_FAIR;
  int64_t pass_paths = 0;  // SRPT: paths per pass (0: no limit)
  int max_queue = 0;       // > 0: pt_submit refuses beyond this many queued requests
  // device scratch of the RMSE estimates: pairs, partial sums, results
  FilmPair *d_pairs = nullptr;
  double *d_partials = nullptr, *d_out = nullptr;
  int pairs_cap = 0;
  void ensure_pairs(int n) {
    if (n <= pairs_cap) return;
    free_pairs();
    cuda_check(cudaMalloc(&d_pairs, sizeof(FilmPair) * n), "cudaMalloc(rmse pairs)");
    cuda_check(cudaMalloc(&d_partials, sizeof(double) * PT_RMSE_BLOCKS * n), "cudaMalloc(rmse partials)");
    cuda_check(cudaMalloc(&d_out, sizeof(double) * n), "cudaMalloc(rmse out)");
    pairs_cap = n;
  }
  void free_pairs() {
    if (d_pairs) cudaFree(d_pairs);
    if (d_partials) cudaFree(d_partials);
    if (d_out) cudaFree(d_out);
    d_pairs = nullptr;
    d_partials = d_out = nullptr;
    pairs_cap = 0;
  }
};

// The request's samples cap and the paths still to render (SRPT's key).
static int request_cap(const Request &r) {
  return std::min(r.desc.spp_cap, r.desc.job.spp_x * r.desc.job.spp_y);
}
static long long remaining_paths(const Request &r) {
  return (long long)r.desc.job.width * r.desc.job.height * (request_cap(r) - r.spp_done);
}

static void release_films(Request &r, Server &s) {
  if (r.film_a) cudaFree(r.film_a);
  if (r.film_b) cudaFree(r.film_b);
  r.film_a = r.film_b = nullptr;
  s.used -= (int64_t)r.bytes;
  r.bytes = 0;
}

}  // namespace pt

using namespace pt;

static int serr(void *ctx, int code, const std::string &m) {
  if (ctx) static_cast<Context *>(ctx)->last_error = m;
  return code;
}

extern "C" {

int pt_render_batch(void *ctx, const pt_job_desc *jobs, int32_t n_jobs, float **films, pt_stats *stats) {
  if (!ctx || !jobs || n_jobs < 0) return serr(ctx, PT_ERR_INVALID, "bad batch args");
  if (n_jobs == 0) return PT_OK;
  Context *c = static_cast<Context *>(ctx);
  try {
    cuda_check(cudaSetDevice(c->device), "cudaSetDevice");
    render_batch(c, jobs, n_jobs, films, stats);
    return PT_OK;
  } catch (const PtError &e) {
    return serr(ctx, e.code, e.what());
  } catch (const std::exception &e) {
    return serr(ctx, PT_ERR_INVALID, e.what());
  }
}

int pt_set_batch_mode(void *ctx, int32_t mode) {
  if (!ctx) return PT_ERR_INVALID;
  if (mode != PT_BATCH_GRAPH && mode != PT_BATCH_PERSISTENT) return serr(ctx, PT_ERR_INVALID, "bad batch mode");
  static_cast<Context *>(ctx)->batch_mode = mode;
  return PT_OK;
}

int pt_autotune(void *ctx, const pt_job_desc *jobs, int32_t n_jobs, pt_tuning *out) {
  if (!ctx || !jobs || n_jobs <= 0) return serr(ctx, PT_ERR_INVALID, "bad autotune args");
  Context *c = static_cast<Context *>(ctx);
  try {
    cuda_check(cudaSetDevice(c->device), "cudaSetDevice");
    autotune(c, jobs, n_jobs, out);
    return PT_OK;
  } catch (const PtError &e) {
    return serr(ctx, e.code, e.what());
  } catch (const std::exception &e) {
    return serr(ctx, PT_ERR_INVALID, e.what());
  }
}

int pt_server_create(void *ctx, int64_t hbm_budget_bytes, int32_t max_slots, void **server) {
  if (!ctx || !server || max_slots <= 0) return serr(ctx, PT_ERR_INVALID, "bad server args");
  Server *s = new Server();
  s->ctx = static_cast<Context *>(ctx);
  s->budget = hbm_budget_bytes;
  s->max_slots = max_slots;
  *server = s;
  return PT_OK;
}

int pt_server_destroy(void *server) {
  if (!server) return PT_ERR_INVALID;
  Server *s = static_cast<Server *>(server);
  cudaStreamSynchronize(s->ctx->stream);
  for (auto &kv : s->reqs) release_films(kv.second, *s);
  s->free_pairs();
  delete s;
  return PT_OK;
}

int pt_submit(void *server, const pt_request_desc *req, int64_t *request_id) {
  if (!server || !req || !request_id) return PT_ERR_INVALID;
  Server *s = static_cast<Server *>(server);
  try {
    validate_job(req->job);
    s->ctx->scene(req->job.scene);
  } catch (const std::exception &e) {
    return serr(s->ctx, PT_ERR_INVALID, e.what());
  }
  if (req->spp_cap <= 0 || req->spp_per_pass <= 0 || req->paths_per_pass < 0)
    return serr(s->ctx, PT_ERR_INVALID, "bad spp cap / pass");
  if (s->max_queue > 0 && (int)s->queue.size() >= s->max_queue)
    return serr(s->ctx, PT_ERR_BUSY, "admission refused: " + std::to_string(s->queue.size()) + " requests queued");
  Request r;
  r.id = s->next_id++;
  r.desc = *req;
  r.t_submit = std::chrono::steady_clock::now();
  s->reqs[r.id] = r;
  s->queue.push_back(r.id);
  *request_id = r.id;
  return PT_OK;
}

int pt_server_step(void *server, int32_t *active_out) {
  if (!server) return PT_ERR_INVALID;
  Server *s = static_cast<Server *>(server);
  Context *c = s->ctx;
  // admission while slots and HBM allow: FIFO, or (SRPT) the queued request
  // of least total work first
  while (!s->queue.empty() && (int)s->active.size() < s->max_slots) {
    if (s->policy == PT_SERVE_SRPT) {
      auto best = s->queue.begin();
      for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
        if (remaining_paths(s->reqs[*it]) < remaining_paths(s->reqs[*best])) best = it;
      std::iter_swap(s->queue.begin(), best);
    }
    Request &r = s->reqs[s->queue.front()];
    if (r.state == 3) {
      s->queue.pop_front();
      continue;
    }
    const size_t nf = (size_t)r.desc.job.width * r.desc.job.height * 3;
    const size_t need = 2 * nf * sizeof(float);
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    if ((int64_t)(s->used + need) > s->budget || need + (size_t)(256ull << 20) > free_b) break;
    if (cudaMalloc(&r.film_a, nf * 4) != cudaSuccess || cudaMalloc(&r.film_b, nf * 4) != cudaSuccess) {
      release_films(r, *s);
      break;
    }
    cudaMemsetAsync(r.film_a, 0, nf * 4, c->stream);
    cudaMemsetAsync(r.film_b, 0, nf * 4, c->stream);
    r.bytes = need;
    s->used += (int64_t)need;
    r.state = 1;
    r.admitted = true;
    r.t_admit = std::chrono::steady_clock::now();
    s->active.push_back(r.id);
    s->queue.pop_front();
  }
  // one pass over the active requests: a batch with one job per request (its
  // next spp_per_pass samples), rendered as one graph launch.  FAIR: every
  // active request; SRPT: in order of remaining paths until the pass holds
  // pass_paths (at least one request), the others wait for a later pass
  std::vector<int64_t> still, live, order;
  std::vector<pt_job_desc> jobs;
  std::vector<float *> targets;
  std::vector<int> ends;
  std::vector<bool> to_a_v;
  for (int64_t id : s->active) {
    Request &r = s->reqs[id];
    if (r.state != 1) {
      release_films(r, *s);
      continue;
    }
    order.push_back(id);
  }
  if (s->policy == PT_SERVE_SRPT)
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
      return remaining_paths(s->reqs[a]) < remaining_paths(s->reqs[b]);
    });
  long long pass_sum = 0;
  for (int64_t id : order) {
    Request &r = s->reqs[id];
    if (s->policy == PT_SERVE_SRPT && s->pass_paths > 0 && !jobs.empty() && pass_sum >= s->pass_paths) {
      still.push_back(id);  // not in this pass
      continue;
    }
    pt_job_desc j = r.desc.job;
    const int spp_total = j.spp_x * j.spp_y;
    const int cap = std::min(r.desc.spp_cap, spp_total);
    long long step = r.desc.spp_per_pass;
    if (r.desc.paths_per_pass > 0) {
      const long long px = std::max<long long>(1, (long long)j.width * j.height);
      step = std::max(step, (r.desc.paths_per_pass + px - 1) / px);
    }
    const int b = r.spp_done, e = (int)std::min<long long>(cap, b + step);
    j.spp_begin = b;
    j.spp_end = e;
    const bool to_a = (r.passes % 2) == 0;
    jobs.push_back(j);
    targets.push_back(to_a ? r.film_a : r.film_b);
    ends.push_back(e);
    to_a_v.push_back(to_a);
    live.push_back(id);
    pass_sum += (long long)j.width * j.height * (e - b);
  }
  if (!jobs.empty()) {
    try {
      render_batch(c, jobs.data(), (int)jobs.size(), nullptr, nullptr, targets.data());
    } catch (const std::exception &ex) {
      for (int64_t id : live) {
        Request &r = s->reqs[id];
        r.state = 4;
        r.error = ex.what();
        release_films(r, *s);
      }
      live.clear();
    }
  }
  // bookkeeping; RMSE estimates of the requests that have a target, on the
  // device in one launch (the mean image's RMSE from the two half films:
  // E|A - B|^2 / 4 = var(mean of all samples) for equal halves)
  std::vector<FilmPair> pairs;
  std::vector<int> pair_of(live.size(), -1);
  for (size_t q = 0; q < live.size(); ++q) {
    Request &r = s->reqs[live[q]];
    const pt_job_desc &j = jobs[q];
    (to_a_v[q] ? r.spp_a : r.spp_b) += ends[q] - j.spp_begin;
    r.spp_done = ends[q];
    ++r.passes;
    const int cap = std::min(r.desc.spp_cap, j.spp_x * j.spp_y);
    if (r.spp_done < cap && r.desc.target_rmse > 0.f && r.spp_a > 0 && r.spp_b > 0) {
      pair_of[q] = (int)pairs.size();
      pairs.push_back(FilmPair{r.film_a, r.film_b, 1.0 / r.spp_a, 1.0 / r.spp_b, (long long)j.width * j.height * 3});
    }
  }
  std::vector<double> est(pairs.size());
  try {
    if (!pairs.empty()) {
      s->ensure_pairs((int)pairs.size());
      cuda_check(cudaMemcpyAsync(s->d_pairs, pairs.data(), sizeof(FilmPair) * pairs.size(), cudaMemcpyHostToDevice,
                                 c->stream),
                 "upload rmse pairs");
      launch_film_rmse(s->d_pairs, (int)pairs.size(), s->d_partials, s->d_out, c->stream);
      cuda_check(cudaMemcpyAsync(est.data(), s->d_out, sizeof(double) * pairs.size(), cudaMemcpyDeviceToHost,
                                 c->stream),
                 "read rmse");
      cuda_check(cudaStreamSynchronize(c->stream), "rmse estimate");
    }
  } catch (const std::exception &ex) {
    for (int64_t id : live) {
      Request &r = s->reqs[id];
      r.state = 4;
      r.error = ex.what();
      release_films(r, *s);
    }
    live.clear();
  }
  for (size_t q = 0; q < live.size(); ++q) {
    const int64_t id = live[q];
    Request &r = s->reqs[id];
    const pt_job_desc &j = jobs[q];
    const int cap = std::min(r.desc.spp_cap, j.spp_x * j.spp_y);
    r.last_rmse = pair_of[q] >= 0 ? est[pair_of[q]] : r.last_rmse;
    bool done = r.spp_done >= cap || (pair_of[q] >= 0 && est[pair_of[q]] <= r.desc.target_rmse);
    if (done) {
      const long long nf = (long long)j.width * j.height * 3;
      r.result.resize((size_t)nf);
      launch_film_combine(r.film_a, r.film_b, 1.f / (float)r.spp_done, nf, c->stream);
      cudaMemcpyAsync(r.result.data(), r.film_a, (size_t)nf * 4, cudaMemcpyDeviceToHost, c->stream);
      cudaError_t e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) {
        r.state = 4;
        r.error = cudaGetErrorString(e);
      } else {
        r.state = 2;
      }
      r.t_done = std::chrono::steady_clock::now();
      release_films(r, *s);
    } else {
      still.push_back(id);
    }
  }
  s->active = still;
  cudaStreamSynchronize(c->stream);
  if (active_out) *active_out = (int32_t)(s->active.size() + s->queue.size());
  return PT_OK;
}

int pt_server_set_policy(void *server, int32_t policy, int64_t pass_paths, int32_t max_queue) {
  if (!server) return PT_ERR_INVALID;
  Server *s = static_cast<Server *>(server);
  if ((policy != PT_SERVE_FAIR && policy != PT_SERVE_SRPT) || pass_paths < 0 || max_queue < 0)
    return serr(s->ctx, PT_ERR_INVALID, "bad server policy");
  s->policy = policy;
  s->pass_paths = pass_paths;
  s->max_queue = max_queue;
  return PT_OK;
}

int pt_request_times(void *server, int64_t request_id, double *queue_ms, double *latency_ms) {
  if (!server) return PT_ERR_INVALID;
  Server *s = static_cast<Server *>(server);
  auto it = s->reqs.find(request_id);
  if (it == s->reqs.end()) return serr(s->ctx, PT_ERR_NOT_FOUND, "unknown request");
  const Request &r = it->second;
  using ms = std::chrono::duration<double, std::milli>;
  if (queue_ms) *queue_ms = r.admitted ? ms(r.t_admit - r.t_submit).count() : -1.0;
  if (latency_ms) *latency_ms = r.state == 2 ? ms(r.t_done - r.t_submit).count() : -1.0;
  return PT_OK;
}

int pt_poll(void *server, int64_t request_id, int32_t *state, float *film, int32_t *spp_done, double *latency_ms) {
  if (!server) return PT_ERR_INVALID;
  Server *s = static_cast<Server *>(server);
  auto it = s->reqs.find(request_id);
  if (it == s->reqs.end()) return serr(s->ctx, PT_ERR_NOT_FOUND, "unknown request");
  Request &r = it->second;
  if (state) *state = r.state;
  if (spp_done) *spp_done = r.spp_done;
  if (latency_ms)
    *latency_ms = r.state == 2 ? std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count() : -1.0;
  if (film && r.state == 2) std::memcpy(film, r.result.data(), r.result.size() * sizeof(float));
  if (r.state == 4) return serr(s->ctx, PT_ERR_DEVICE, r.error);
  return PT_OK;
}

int pt_cancel(void *server, int64_t request_id) {
  if (!server) return PT_ERR_INVALID;
  Server *s = static_cast<Server *>(server);
  auto it = s->reqs.find(request_id);
  if (it == s->reqs.end()) return serr(s->ctx, PT_ERR_NOT_FOUND, "unknown request");
  if (it->second.state <= 1) it->second.state = 3;
  return PT_OK;
}

}  // extern "C"
