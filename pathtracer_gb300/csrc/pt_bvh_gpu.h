// pt_bvh_gpu.h -- mesh BVH construction on the device (pt_bvh_gpu.cu).
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace pt {

struct GpuBvhError : std::runtime_error {
  explicit GpuBvhError(const std::string &m) : std::runtime_error(m) {}
};

// A node of the device-built binary tree: padded box, its segment of the
// leaf order, and its first child (the second is left + 1; -1: a leaf).
struct GpuBvhNode {
  float lo[3], hi[3];
  int start, count;
  int left;
  int axis;   // split axis (internal nodes)
  int paxis;  // the parent's split axis (-1: the root)
  int pad;
};

// Builds the median-split BVH of one triangle mesh on the current device.
// nodes[0] is the root; leaf_perm[k] is the triangle at leaf slot k (a leaf
// holds slots [start, start + count)).  Synchronous on st.
void gpu_mesh_bvh(const float *positions, int n_positions, const int32_t *indices, int n_triangles,
                  cudaStream_t st, std::vector<GpuBvhNode> &nodes, std::vector<int32_t> &leaf_perm);

}  // namespace pt
