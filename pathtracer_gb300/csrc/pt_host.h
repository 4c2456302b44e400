// pt_host.h -- host-side objects behind the C-ABI: resident scenes and the
// per-thread rendering context (stream, work queues, device buffers).
#pragma once
#include <cstddef>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "pt_bsdf.cuh"
#include "pt_kernels.h"

namespace pt {

// Error raised inside the library; the C-ABI turns it into its status code.
struct PtError : std::runtime_error {
  int code;
  PtError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const std::string &msg);
void cuda_check(cudaError_t e, const char *what);

HaltonTables make_halton_tables();
std::vector<uint16_t> make_digit_permutations(const HaltonTables &T, uint32_t seed);
MatRec derive_material(const pt_material_desc &m);
CameraView make_camera(const pt_camera_desc &c);
std::vector<float2> make_offsets(const pt_job_desc &j);
void set_window(JobView &v, const pt_job_desc &j);
// Records an error for pt_last_error(NULL, ...) (entry points without a
// context); returns code.
int record_error(int code, const std::string &msg);
std::vector<float> gaussian_weights(int k, float sigma);
void write_png(const char *path, const uint8_t *rgb, int W, int H);
void validate_job(const pt_job_desc &j);

// A flattened scene resident in HBM.
struct Scene {
  SceneView view;
  Bvh4Node *nodes = nullptr;
  Item *items = nullptr;
  PrimShade *shade = nullptr;
  MatRec *materials = nullptr;
  LightRec *lights = nullptr;
  std::vector<LightRec> host_lights;  // the lights' records (pt_light_sample's get_area)
  std::vector<void *> owned;
  int n_tris = 0, n_quads = 0, n_spheres = 0, bvh_depth = 0;
  int env_w = 0, env_h = 0;
  unsigned family_mask = 0;  // BSDF families (material types 0..6) present
  float shutter_max = 0.f;   // moving objects' boxes cover [0, shutter_max]
  size_t device_bytes = 0;
  uint64_t bvh_hash = 0;     // content hash of the BVH4 nodes and leaf items
  int64_t n_nodes = 0, n_items = 0;
  ~Scene();
};

// builder: PT_BVH_BUILD_HOST (the reference's trees), PT_BVH_BUILD_DEVICE
// (meshes of at least PT_GPU_BVH_MIN triangles built on st's device with the
// same rule), PT_BVH_BUILD_SAH (binned-SAH trees on the host).
std::unique_ptr<Scene> build_scene(const pt_scene_desc *d, cudaStream_t st, bool device, int threads,
                                   int trav_cap, int builder = PT_BVH_BUILD_HOST, bool want_hash = false);
constexpr int PT_GPU_BVH_MIN = 1 << 14;

// Device buffers of one merged group of a batch (the jobs of one scene with
// the same light-sample count), reused across batched renders.
struct BatchSlot {
  Queues Q[2]{};                // two queue sets: consecutive waves overlap
  std::vector<void *> mem;
  int cap = 0, ln = 0;
  DeviceJob *d_jobs = nullptr;  // job table
  long long *d_start = nullptr;
  int jobs_cap = 0;
  float2 *offsets = nullptr;    // the jobs' offset tables, concatenated
  size_t offsets_cap = 0;
  float *films = nullptr;       // the jobs' films (when no targets are given), concatenated
  size_t films_cap = 0;
  // persistent form (PT_BATCH_PERSISTENT): the members' film pointers on the
  // device and the group's grid barrier
  float **d_films = nullptr;
  int d_films_cap = 0;
  void *d_barrier = nullptr;
  cudaStream_t stream[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  ShadeStreams side[2];  // side streams of stream[0], stream[1]
  void ensure(int want_cap, int want_ln, int n_jobs, size_t n_offsets, size_t film_floats);
  void release();
};

// A batch: one graph branch per merged group, captured per composition and
// updated in place when only parameters change.
struct Batch {
  std::vector<BatchSlot> slots;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> film_events;  // per wave: its films are done
  std::string sig;
  int captures = 0;  // graph instantiations
  int updates = 0;   // in-place parameter updates of the executable graph
  int launches = 0;  // graph launches
  ~Batch();
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  HaltonTables halton;
  KernelInfo kinfo;
  LaunchCfg cfg;
  int wave_cap = 1 << 22;
  int trav_cap = 0;  // 0: PT_TRAVERSAL_CAP
  int bvh_builder = PT_BVH_BUILD_HOST;
  std::string last_error;
  std::map<int, std::unique_ptr<Scene>> scenes;
  int next_scene = 1;
  std::map<uint32_t, uint16_t *> perms;

  Queues Q{};
  std::vector<void *> qmem;
  int q_cap = 0, q_ln = 0;
  // second queue set and stream: consecutive waves of one render overlap
  Queues Q2{};
  std::vector<void *> qmem2;
  int q2_cap = 0, q2_ln = 0;
  cudaStream_t stream2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  ShadeStreams side1, side2;  // side streams of stream, stream2
  std::vector<cudaEvent_t> film_ev;
  void ensure_queues2(int cap, int ln);
  float *d_film = nullptr;
  size_t film_cap = 0;
  float2 *d_offsets = nullptr;
  int offsets_cap = 0;
  void *d_scratch = nullptr;
  size_t scratch_cap = 0;
  int *d_err = nullptr;
  Profiler prof;
  Batch batch;
  int batch_wave_cap = 1 << 22;  // paths per wave of each batched job
  int batch_mode = PT_BATCH_GRAPH;  // pt_set_batch_mode

  explicit Context(int dev);
  ~Context();
  void free_queues();
  void ensure_queues(int cap, int ln);
  const uint16_t *perm_for(uint32_t seed);
  Scene *scene(int id);
  DeviceJob device_job(const pt_job_desc &j, Scene *S);
  // d_rays (device, 6 floats per film pixel): given primary rays instead of
  // the camera's (pt_ray_color)
  void render_device(const pt_job_desc &j, float *d_film, pt_stats *stats, bool sync,
                     const float *d_rays = nullptr);
  float *film_buffer(size_t floats);
  void *scratch(size_t bytes);
};

}  // namespace pt
