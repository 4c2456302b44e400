// pt_kernels_multi.cu -- merged waves: the paths of many jobs of one scene
// in one wave (batched and served forms).  A wave is a contiguous range of
// the jobs' concatenated path indices; the job-dependent stages (camera,
// closest hit, shade) look up each path's job in a table in HBM, the
// job-independent ones (sort, shadow rays) are the single-job kernels, and
// the film stage adds each job's share of the wave to its own film.
#include "pt_wave.cuh"

namespace pt {

void upload_halton_tables_multi(const HaltonTables &T, cudaStream_t st) {
  cudaMemcpyToSymbolAsync(c_halton, &T, sizeof(T), 0, cudaMemcpyHostToDevice, st);
}

void launch_wave_multi(const SceneView &S, const MergedJobs &M, const Queues &Q, long long g0, int n,
                       const LaunchCfg &cfg, cudaStream_t st, Profiler *prof, cudaEvent_t film_after,
                       cudaEvent_t film_done, const ShadeStreams *ss) {
  Profiler dummy;
  Profiler &P = prof ? *prof : dummy;
  DeviceJob none;
  std::memset(&none, 0, sizeof none);
  launch_wave_stages<true>(S, none, M.T, Q, g0, n, M.LN, M.bounces, cfg, st, P, ss);
  if (film_after) cudaStreamWaitEvent(st, film_after, 0);
  P.begin(STAGE_FILM, st);
  const long long g1 = g0 + n;
  for (size_t k = 0; k + 1 < M.start.size(); ++k) {
    const long long a = std::max(g0, M.start[k]), b = std::min(g1, M.start[k + 1]);
    if (a >= b) continue;
    launch_film(M.jobs[k], Q, a - M.start[k], (int)(b - a), a - g0, M.films[k], cfg, st);
    P.count(STAGE_FILM, 1);
  }
  P.end(st);
  if (film_done) cudaEventRecord(film_done, st);
}

}  // namespace pt
