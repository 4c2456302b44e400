// pt_noalloc.cu -- pt_render_device_noalloc: the wavefront render without
// any device allocation.
//
// Some callers cannot allocate device memory while they render: a host that
// runs its own device memory pool or arena and forbids other allocators on
// its devices, or a real-time loop that must never block on the allocator.
// For them this entry point keeps every buffer the render needs -- the
// path-state and ray/hit/shadow queues, the pixel-offset table, the
// digit-permutation tables and the counters -- in ONE file-scope device
// array of fixed size, PT_NOALLOC_SCRATCH_BYTES.  With CUDA's lazy module
// loading (the default) the array is allocated on a device when this file's
// module is first loaded there, i.e. in the first call's
// cudaGetSymbolAddress, and it stays allocated until the process exits; a
// caller makes one warm-up call per device before its no-allocation region.
// The caller still passes its inputs (a scene already resident through
// pt_scene_upload, the job) and its output (a device film).  Large jobs are
// rendered in as many waves as the array's path capacity requires.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pt_host.h"

namespace pt {

// 32 MiB of scratch per device.
#define PT_NOALLOC_SCRATCH_BYTES (32u << 20)
#define PT_NOALLOC_MAX_SPP 16384
#define PT_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[PT_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per device, looked up once per device
// with that device current.  In host code the symbol itself is only a
// host-side stand-in, so it is never passed to a kernel.
static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_ptr[PT_NOALLOC_MAX_DEVICES] = {nullptr};

static unsigned char *noalloc_scratch(int device) {
  if (device < 0 || device >= PT_NOALLOC_MAX_DEVICES) fail(PT_ERR_INVALID, "device id out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void *p = nullptr;
    cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
    g_noalloc_ptr[device] = static_cast<unsigned char *>(p);
  }
  return g_noalloc_ptr[device];
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

void render_device_noalloc(Context *c, const pt_job_desc &j, float *d_film, pt_stats *stats) {
  validate_job(j);
  const int spp = j.spp_x * j.spp_y;
  if (spp > PT_NOALLOC_MAX_SPP)
    fail(PT_ERR_TOO_LARGE, "pt_render_device_noalloc: spp_x * spp_y = " + std::to_string(spp) +
                               " exceeds the fixed maximum of " + std::to_string(PT_NOALLOC_MAX_SPP));
  Scene *S = c->scene(j.scene);
  cuda_check(cudaSetDevice(c->device), "cudaSetDevice");
  unsigned char *base = noalloc_scratch(c->device);

  // ---- carve the scratch array
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    off = align_up(off, 256);
    unsigned char *p = base + off;
    off += bytes;
    return p;
  };
  Queues Q{};
  Q.counts = (int *)carve(64);
  Q.stats = (unsigned long long *)carve(64);
  Q.err = (int *)carve(16);
  Q.bins = (int *)carve(sizeof(int) * 2 * PT_SORT_BINS);
  Q.seg = (int *)carve(sizeof(int) * (PT_SORT_BINS + 1));
  float2 *d_off = (float2 *)carve(sizeof(float2) * PT_NOALLOC_MAX_SPP);
  std::vector<uint16_t> perm;
  if (j.sampler == PT_SAMPLER_HALTON_PERMUTE) perm = make_digit_permutations(c->halton, j.sampler_seed);
  uint16_t *d_perm = (uint16_t *)carve(perm.size() * sizeof(uint16_t) + 16);
  const int LN = j.light_samples_x * j.light_samples_y;
  off = align_up(off, 256);
  const size_t per_path = 16 * 8 + 2 * 16 * (size_t)LN + (size_t)LN + 3 * 4;
  const size_t avail = PT_NOALLOC_SCRATCH_BYTES - off - 18 * 256;  // alignment slack of 18 arrays
  const int cap = (int)std::min<size_t>(avail / per_path, (size_t)1 << 30);
  if (cap < 1024) fail(PT_ERR_TOO_LARGE, "pt_render_device_noalloc: scratch too small for the light samples");
  const size_t c4 = (size_t)cap * 16;
  Q.cap = cap;
  Q.beta = (float4 *)carve(c4);
  Q.L = (float4 *)carve(c4);
  Q.ray_o[0] = (float4 *)carve(c4);
  Q.ray_o[1] = (float4 *)carve(c4);
  Q.ray_d[0] = (float4 *)carve(c4);
  Q.ray_d[1] = (float4 *)carve(c4);
  Q.hit = (float4 *)carve(c4);
  Q.sh_o = (float4 *)carve(c4);
  Q.sh_d = (float4 *)carve(c4 * LN);
  Q.sh_c = (float4 *)carve(c4 * LN);
  Q.sh_vis = (uint8_t *)carve((size_t)cap * LN);
  Q.sort_key = (int *)carve((size_t)cap * 4);
  Q.order = (int *)carve((size_t)cap * 4);
  Q.job = (int *)carve((size_t)cap * 4);
  if (off > PT_NOALLOC_SCRATCH_BYTES) fail(PT_ERR_TOO_LARGE, "pt_render_device_noalloc: scratch layout overflow");

  // ---- job constants (as Context::device_job, with the tables in scratch)
  DeviceJob J;
  std::memset(&J, 0, sizeof J);
  set_window(J.job, j);
  J.job.spp_x = j.spp_x;
  J.job.spp_y = j.spp_y;
  J.job.spp = spp;
  J.job.spp_begin = j.spp_begin;
  J.job.max_depth = j.max_depth;
  J.job.rr_start = j.rr_start;
  J.job.estimator = j.estimator;
  J.job.sampler = j.sampler;
  J.job.env_sampling = S->view.env.present ? j.env_sampling : PT_ENV_UNIFORM;
  J.job.light_nx = j.light_samples_x;
  J.job.light_ny = j.light_samples_y;
  J.job.seed = j.seed;
  J.job.shutter = j.camera.shutter;
  if (S->view.has_motion && j.camera.shutter > S->shutter_max)
    fail(PT_ERR_INVALID, "camera shutter longer than the scene's shutter_max");
  J.job.cam = make_camera(j.camera);
  std::vector<float2> offs = make_offsets(j);
  cuda_check(cudaMemcpyAsync(d_off, offs.data(), offs.size() * sizeof(float2), cudaMemcpyHostToDevice, c->stream),
             "upload offsets");
  J.job.offsets = d_off;
  if (!perm.empty()) {
    cuda_check(cudaMemcpyAsync(d_perm, perm.data(), perm.size() * sizeof(uint16_t), cudaMemcpyHostToDevice,
                               c->stream),
               "upload permutations");
    J.perm = d_perm;
  }
  // the array keeps the previous call's contents: clear what starts at zero
  cuda_check(cudaMemsetAsync(Q.counts, 0, 64, c->stream), "memset counts");
  cuda_check(cudaMemsetAsync(Q.stats, 0, 64, c->stream), "memset stats");
  cuda_check(cudaMemsetAsync(Q.err, 0, 16, c->stream), "memset err");

  // ---- waves
  const long long npix = (long long)j.width * j.height;
  const int e = j.spp_end ? j.spp_end : spp;
  const long long total = npix * (e - j.spp_begin);
  int n = cap;
  if (npix <= cap) n = (int)((cap / npix) * npix);
  if ((long long)n > total) n = (int)total;
  LaunchCfg lc = c->cfg;
  lc.family_mask = S->family_mask;
  for (long long g0 = 0; g0 < total; g0 += n) {
    int cnt = (int)std::min<long long>(n, total - g0);
    launch_wave(S->view, J, Q, g0, cnt, d_film, lc, c->stream, nullptr);
  }
  cuda_check(cudaGetLastError(), "launch");
  cuda_check(cudaStreamSynchronize(c->stream), "render");
  int herr = 0;
  cuda_check(cudaMemcpy(&herr, Q.err, sizeof(int), cudaMemcpyDeviceToHost), "read err");
  if (herr) fail(PT_ERR_DEVICE, "device traversal error flag " + std::to_string(herr));
  if (stats) {
    unsigned long long h[4];
    cuda_check(cudaMemcpy(h, Q.stats, sizeof h, cudaMemcpyDeviceToHost), "read stats");
    stats->paths = h[0];
    stats->segments = h[1];
    stats->rays = h[2];
    stats->shadow_rays = h[3];
    stats->ms = -1.0;  // not timed: timing would need CUDA events
    stats->algorithmic_bytes = 192ull * h[1] + 88ull * h[3] + 24ull * h[0];
  }
}

}  // namespace pt

extern "C" int pt_render_device_noalloc(void *ctx, const pt_job_desc *job, float *d_film_sum, pt_stats *stats) {
  pt::Context *c = static_cast<pt::Context *>(ctx);
  if (!c || !job || !d_film_sum) return PT_ERR_INVALID;
  try {
    pt::render_device_noalloc(c, *job, d_film_sum, stats);
    return PT_OK;
  } catch (const pt::PtError &e) {
    c->last_error = e.what();
    return e.code;
  } catch (const std::exception &e) {
    c->last_error = e.what();
    return PT_ERR_INVALID;
  }
}
