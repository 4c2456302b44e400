// pt_bvh_gpu.cu -- mesh BVH construction on the device.
//
// The reference builds a mesh's BVH on the host (MeshBVHNode,
// src/primitives/meshBVH.cpp:6-55): a node's box is the box of its
// triangles' vertices +- 1e-3; a node of <= 4 triangles is a leaf; otherwise
// its triangles are sorted by centroid ((v0 + v1 + v2) / 3) along the longest
// axis of the unpadded box and split at count / 2.  This file builds the same
// tree on the GPU, level by level, without sorting per node:
//
//   1. per triangle: box and centroid; three stable LSD radix sorts (8-bit
//      digits) order the triangles by centroid x, y and z (ties by triangle
//      index).  Each node owns the same segment [start, start + count) of
//      all three lists, sorted by its axis in each list.
//   2. per level: node boxes by a segmented min/max (order-preserving
//      integer keys, warp-aggregated atomics); each internal node picks its
//      axis and marks the first count / 2 triangles of its segment in that
//      axis's list as "left"; all three lists are stably partitioned by that
//      mark (exclusive scans), so every list stays sorted within each child.
//   3. a child of <= 4 triangles is a leaf whose triangles keep the order of
//      its parent's axis list -- the order the reference's leaf has after its
//      parent's sort.
//
// When no two centroids of a node tie along its split axis the tree is the
// reference's (same node boxes, split sets and leaf order); ties are broken
// by triangle index here and by std::sort's order in the reference.  Every
// loop is bounded by its input sizes and nothing waits on another block.
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "pt_bvh_gpu.h"

namespace pt {
namespace {

constexpr int SCAN_THREADS = 256, SCAN_ITEMS = 16, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr int RADIX_THREADS = 256, RADIX_ITEMS = 16, RADIX_TILE = RADIX_THREADS * RADIX_ITEMS;

__device__ __forceinline__ uint32_t f2key(float f) {  // order-preserving float -> uint32
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key2f(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// per triangle: vertex box (6 floats, SoA) and the centroid keys of the 3 axes
__global__ void k_tri_prep(const float *pos, const int32_t *idx, int n, float *tbox, uint32_t *ckey) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const float *p0 = pos + 3 * (size_t)idx[3 * (size_t)t];
    const float *p1 = pos + 3 * (size_t)idx[3 * (size_t)t + 1];
    const float *p2 = pos + 3 * (size_t)idx[3 * (size_t)t + 2];
    for (int a = 0; a < 3; ++a) {
      tbox[(size_t)a * n + t] = fminf(fminf(p0[a], p1[a]), p2[a]);
      tbox[(size_t)(3 + a) * n + t] = fmaxf(fmaxf(p0[a], p1[a]), p2[a]);
      // ((v0 + v1) + v2) / 3.0f, each operation rounded on its own
      ckey[(size_t)a * n + t] = f2key(__fdiv_rn(__fadd_rn(__fadd_rn(p0[a], p1[a]), p2[a]), 3.0f));
    }
  }
}

__global__ void k_iota(int32_t *v, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

// ------------------------------------------------------------ exclusive scan
// Batched over blockIdx.y: array y is in + y * stride (n elements).
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const int32_t *in, long long stride, int n,
                                                              int32_t *sums, int nb) {
  in += blockIdx.y * stride;
  const long long base = (long long)blockIdx.x * SCAN_TILE;
  int s = 0;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const long long i = base + (long long)k * SCAN_THREADS + threadIdx.x;
    if (i < n) s += in[i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  __shared__ int ws[SCAN_THREADS / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < SCAN_THREADS / 32; ++w) t += ws[w];
    sums[blockIdx.y * nb + blockIdx.x] = t;
  }
}

// One block per batch entry: exclusive scan of nb block sums in place.
__global__ void __launch_bounds__(1024) k_scan_sums(int32_t *sums, int nb) {
  sums += blockIdx.x * nb;
  __shared__ int buf[1024];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int c0 = 0; c0 < nb; c0 += 1024) {
    const int i = c0 + threadIdx.x;
    const int v = i < nb ? sums[i] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele
      const int add = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
      __syncthreads();
      buf[threadIdx.x] += add;
      __syncthreads();
    }
    if (i < nb) sums[i] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
}

// Exclusive prefix of each element: thread t owns SCAN_ITEMS consecutive
// elements of its block's tile.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(const int32_t *in, long long stride, int n,
                                                            const int32_t *sums, int nb, int32_t *out) {
  in += blockIdx.y * stride;
  out += blockIdx.y * stride;
  const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS], s = 0;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  // exclusive scan of the thread sums across the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = s;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  __shared__ int wsum[SCAN_THREADS / 32];
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  int wpre = 0;
  for (int w = 0; w < warp; ++w) wpre += wsum[w];
  int run = sums[blockIdx.y * nb + blockIdx.x] + wpre + inc - s;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

// ------------------------------------------------------------ radix sort
// hist[digit * nb + block]: count of each 8-bit digit per tile.
__global__ void __launch_bounds__(RADIX_THREADS) k_radix_hist(const uint32_t *keys, int n, int shift, int32_t *hist,
                                                              int nb) {
  __shared__ int cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * RADIX_TILE;
  for (int k = 0; k < RADIX_ITEMS; ++k) {
    const long long i = base + (long long)k * RADIX_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  hist[threadIdx.x * nb + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter: the tile is walked in order, 256 elements at a time; an
// element's rank among equal digits comes from its warp (match + popc) and
// the counts of the warps before it.
__global__ void __launch_bounds__(RADIX_THREADS) k_radix_scatter(const uint32_t *kin, const int32_t *vin,
                                                                 uint32_t *kout, int32_t *vout, int n, int shift,
                                                                 const int32_t *hist, int nb) {
  constexpr int NW = RADIX_THREADS / 32;
  __shared__ int run[256];
  __shared__ int wcnt[NW][257];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  run[threadIdx.x] = hist[threadIdx.x * nb + blockIdx.x];
  const long long base = (long long)blockIdx.x * RADIX_TILE;
  for (int k = 0; k < RADIX_ITEMS; ++k) {
    for (int w = 0; w < NW; ++w) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const long long i = base + (long long)k * RADIX_THREADS + threadIdx.x;
    const bool ok = i < n;
    const uint32_t key = ok ? kin[i] : 0u;
    const int d = ok ? (int)((key >> shift) & 255u) : 256;  // 256: no element
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (ok && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (ok) {
      int before = 0;
      for (int w = 0; w < warp; ++w) before += wcnt[w][d];
      const int dst = run[d] + before + rank;
      kout[dst] = key;
      vout[dst] = vin[i];
    }
    __syncthreads();
    int tot = 0;
    for (int w = 0; w < NW; ++w) tot += wcnt[w][threadIdx.x];
    run[threadIdx.x] += tot;
    __syncthreads();
  }
}

// ------------------------------------------------------------ levels
using DNode = GpuBvhNode;

__global__ void k_level_init(DNode *nodes, int b, int e, uint32_t *bkey) {
  for (int x = b + blockIdx.x * blockDim.x + threadIdx.x; x < e; x += gridDim.x * blockDim.x) {
    uint32_t *k = bkey + 6 * (size_t)(x - b);
    for (int a = 0; a < 3; ++a) {
      k[a] = 0xffffffffu;  // min
      k[3 + a] = 0u;       // max
    }
  }
}

// Segmented min / max of the triangle boxes of each level node.
__global__ void k_level_box(const int32_t *list0, const int32_t *node_of, int n, int b, int e, const float *tbox,
                            uint32_t *bkey) {
  const int lane = threadIdx.x & 31;
  for (long long p0 = (long long)blockIdx.x * blockDim.x; p0 < n; p0 += (long long)gridDim.x * blockDim.x) {
    const long long p = p0 + threadIdx.x;
    int x = -1;
    uint32_t k[6];
    if (p < n) {
      x = node_of[p];
      if (x >= b && x < e) {
        const int t = list0[p];
        for (int c = 0; c < 6; ++c) k[c] = f2key(tbox[(size_t)c * n + t]);
      } else {
        x = -1;
      }
    }
    const int x0 = __shfl_sync(0xffffffffu, x, 0);
    if (__all_sync(0xffffffffu, x == x0)) {
      if (x0 < 0) continue;
      for (int c = 0; c < 6; ++c)
        for (int o = 16; o > 0; o >>= 1) {
          const uint32_t y = __shfl_down_sync(0xffffffffu, k[c], o);
          k[c] = c < 3 ? min(k[c], y) : max(k[c], y);
        }
      if (lane == 0) {
        uint32_t *dst = bkey + 6 * (size_t)(x0 - b);
        for (int c = 0; c < 3; ++c) atomicMin(dst + c, k[c]);
        for (int c = 3; c < 6; ++c) atomicMax(dst + c, k[c]);
      }
    } else if (x >= 0) {
      uint32_t *dst = bkey + 6 * (size_t)(x - b);
      for (int c = 0; c < 3; ++c) atomicMin(dst + c, k[c]);
      for (int c = 3; c < 6; ++c) atomicMax(dst + c, k[c]);
    }
  }
}

// Boxes, leaves, split axes and the children of the next level.
__global__ void k_level_nodes(DNode *nodes, int b, int e, const uint32_t *bkey, int *n_nodes, int cap) {
  for (int x = b + blockIdx.x * blockDim.x + threadIdx.x; x < e; x += gridDim.x * blockDim.x) {
    DNode &N = nodes[x];
    const uint32_t *k = bkey + 6 * (size_t)(x - b);
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = key2f(k[a]);
      hi[a] = key2f(k[3 + a]);
      N.lo[a] = __fsub_rn(lo[a], 1e-3f);
      N.hi[a] = __fadd_rn(hi[a], 1e-3f);
    }
    N.left = -1;
    N.axis = -1;
    if (N.count <= 4) continue;
    const float ex = __fsub_rn(hi[0], lo[0]), ey = __fsub_rn(hi[1], lo[1]), ez = __fsub_rn(hi[2], lo[2]);
    const int axis = ex > ey && ex > ez ? 0 : ey > ez ? 1 : 2;
    const int c = atomicAdd(n_nodes, 2);
    if (c + 2 > cap) continue;  // cannot happen: a tree of leaves >= 2 has < n nodes
    N.axis = axis;
    N.left = c;
    const int mid = N.count / 2;
    DNode L{}, R{};
    L.start = N.start;
    L.count = mid;
    R.start = N.start + mid;
    R.count = N.count - mid;
    L.paxis = R.paxis = axis;
    L.left = R.left = -1;
    nodes[c] = L;
    nodes[c + 1] = R;
  }
}

// Marks, per triangle, whether it goes to its node's left child.
__global__ void k_level_flags(const int32_t *lists, int n, const int32_t *node_of, const DNode *nodes, int b, int e,
                              uint8_t *flag) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const int x = node_of[p];
    if (x < b || x >= e) continue;
    const DNode &N = nodes[x];
    if (N.left < 0) continue;
    const int t = lists[(size_t)N.axis * n + p];
    flag[t] = (p - N.start) < N.count / 2 ? 1 : 0;
  }
}

// vals[l][p] = 1 when the triangle at p of list l goes left (internal nodes
// of this level only).
__global__ void k_level_vals(const int32_t *lists, int n, const int32_t *node_of, const DNode *nodes, int b, int e,
                             const uint8_t *flag, int32_t *vals) {
  const int l = blockIdx.y;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const int x = node_of[p];
    int v = 0;
    if (x >= b && x < e && nodes[x].left >= 0) v = flag[lists[(size_t)l * n + p]];
    vals[(size_t)l * n + p] = v;
  }
}

// Stable partition of the three lists; leaf slots get their final order.
// vals: the left marks in list order, pre: their exclusive prefix.
__global__ void k_level_scatter(const int32_t *lists, int32_t *lists_out, int n, const int32_t *node_of,
                                int32_t *node_of_out, const DNode *nodes, int b, int e, const int32_t *vals,
                                const int32_t *pre, int32_t *leaf_perm) {
  const int l = blockIdx.y;
  const int32_t *L = lists + (size_t)l * n;
  int32_t *O = lists_out + (size_t)l * n;
  const int32_t *V = vals + (size_t)l * n;
  const int32_t *P = pre + (size_t)l * n;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const int x = node_of[p];
    const int t = L[p];
    if (x < b || x >= e) {  // in a leaf finished at an earlier level
      O[p] = t;
      if (l == 0) node_of_out[p] = -1;
      continue;
    }
    const DNode &N = nodes[x];
    if (N.left < 0) {  // a leaf of this level: its triangles in its parent's axis order
      O[p] = t;
      if (l == 0) node_of_out[p] = -1;
      if (l == (N.paxis < 0 ? 0 : N.paxis)) leaf_perm[p] = t;
      continue;
    }
    const int mid = N.count / 2;
    const int lrank = P[p] - P[N.start];  // left-going triangles before p in the segment
    const int q = V[p] ? N.start + lrank : N.start + mid + (int)(p - N.start) - lrank;
    O[q] = t;
    if (l == 0) node_of_out[q] = V[p] ? N.left : N.left + 1;
  }
}

int grid(long long n, int threads, int cap) {
  long long g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  return (int)(g < cap ? g : cap);
}

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw GpuBvhError(std::string(what) + ": " + cudaGetErrorString(e));
}

// Exclusive scan of `batch` arrays of n ints (stride n) into out.
void scan(const int32_t *in, int32_t *out, int n, int batch, int32_t *sums, cudaStream_t st) {
  const int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_reduce<<<dim3(nb, batch), SCAN_THREADS, 0, st>>>(in, n, n, sums, nb);
  k_scan_sums<<<batch, 1024, 0, st>>>(sums, nb);
  k_scan_down<<<dim3(nb, batch), SCAN_THREADS, 0, st>>>(in, n, n, sums, nb, out);
}

template <class T>
struct DBuf {
  T *p = nullptr;
  explicit DBuf(size_t n) { check(cudaMalloc(&p, sizeof(T) * (n ? n : 1)), "cudaMalloc(bvh build)"); }
  ~DBuf() { cudaFree(p); }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
};

}  // namespace

void gpu_mesh_bvh(const float *positions, int n_positions, const int32_t *indices, int n, cudaStream_t st,
                  std::vector<GpuBvhNode> &out_nodes, std::vector<int32_t> &leaf_perm) {
  if (n < 5) throw GpuBvhError("device BVH build needs at least 5 triangles");
  const int cap_grid = 152 * 16;
  DBuf<float> pos((size_t)n_positions * 3);
  DBuf<int32_t> idx((size_t)n * 3);
  check(cudaMemcpyAsync(pos.p, positions, sizeof(float) * 3 * (size_t)n_positions, cudaMemcpyHostToDevice, st),
        "upload positions");
  check(cudaMemcpyAsync(idx.p, indices, sizeof(int32_t) * 3 * (size_t)n, cudaMemcpyHostToDevice, st),
        "upload indices");
  DBuf<float> tbox((size_t)n * 6);
  DBuf<uint32_t> ckey((size_t)n * 3), kalt(n);
  DBuf<int32_t> lists((size_t)n * 3), lists2((size_t)n * 3), valt(n);
  k_tri_prep<<<grid(n, 256, cap_grid), 256, 0, st>>>(pos.p, idx.p, n, tbox.p, ckey.p);
  check(cudaGetLastError(), "k_tri_prep");

  // three stable radix sorts by centroid key (ties: triangle index)
  const int rnb = (n + RADIX_TILE - 1) / RADIX_TILE;
  DBuf<int32_t> hist((size_t)256 * rnb), hist_pre((size_t)256 * rnb);
  const int snb_max = ((n > 256 * rnb ? n : 256 * rnb) + SCAN_TILE - 1) / SCAN_TILE;
  DBuf<int32_t> sums((size_t)3 * snb_max);
  for (int a = 0; a < 3; ++a) {
    uint32_t *k0 = ckey.p + (size_t)a * n, *k1 = kalt.p;
    int32_t *v0 = lists.p + (size_t)a * n, *v1 = valt.p;
    k_iota<<<grid(n, 256, cap_grid), 256, 0, st>>>(v0, n);
    for (int shift = 0; shift < 32; shift += 8) {  // 4 passes: the result lands back in k0 / v0
      k_radix_hist<<<rnb, RADIX_THREADS, 0, st>>>(k0, n, shift, hist.p, rnb);
      scan(hist.p, hist_pre.p, 256 * rnb, 1, sums.p, st);
      k_radix_scatter<<<rnb, RADIX_THREADS, 0, st>>>(k0, v0, k1, v1, n, shift, hist_pre.p, rnb);
      std::swap(k0, k1);
      std::swap(v0, v1);
    }
    check(cudaGetLastError(), "radix sort");
  }

  // levels
  const int cap = n + 1;  // leaves hold >= 2 triangles (count >= 5 splits into >= 2 + 3)
  DBuf<DNode> nodes(cap);
  DBuf<int32_t> node_of(n), node_of2(n), vals((size_t)n * 3), pre((size_t)n * 3), perm(n), counter(1);
  DBuf<uint8_t> flag(n);
  DBuf<uint32_t> bkey((size_t)6 * cap);
  {
    DNode root{};
    root.start = 0;
    root.count = n;
    root.left = -1;
    root.paxis = -1;
    check(cudaMemcpyAsync(nodes.p, &root, sizeof root, cudaMemcpyHostToDevice, st), "root");
    const int one = 1;
    check(cudaMemcpyAsync(counter.p, &one, sizeof one, cudaMemcpyHostToDevice, st), "counter");
    check(cudaMemsetAsync(node_of.p, 0, sizeof(int32_t) * n, st), "node_of");
  }
  int32_t *L = lists.p, *L2 = lists2.p, *NO = node_of.p, *NO2 = node_of2.p;
  int b = 0, e = 1, total = 1;
  for (int level = 0; b < e; ++level) {
    if (level > 64) throw GpuBvhError("device BVH build did not converge");
    const int m = e - b;
    k_level_init<<<grid(m, 256, cap_grid), 256, 0, st>>>(nodes.p, b, e, bkey.p);
    k_level_box<<<grid(n, 256, cap_grid), 256, 0, st>>>(L, NO, n, b, e, tbox.p, bkey.p);
    k_level_nodes<<<grid(m, 256, cap_grid), 256, 0, st>>>(nodes.p, b, e, bkey.p, counter.p, cap);
    k_level_flags<<<grid(n, 256, cap_grid), 256, 0, st>>>(L, n, NO, nodes.p, b, e, flag.p);
    k_level_vals<<<dim3(grid(n, 256, cap_grid), 3), 256, 0, st>>>(L, n, NO, nodes.p, b, e, flag.p, vals.p);
    scan(vals.p, pre.p, n, 3, sums.p, st);
    k_level_scatter<<<dim3(grid(n, 256, cap_grid), 3), 256, 0, st>>>(L, L2, n, NO, NO2, nodes.p, b, e, vals.p,
                                                                     pre.p, perm.p);
    check(cudaGetLastError(), "BVH level");
    std::swap(L, L2);
    std::swap(NO, NO2);
    check(cudaMemcpyAsync(&total, counter.p, sizeof total, cudaMemcpyDeviceToHost, st), "node count");
    check(cudaStreamSynchronize(st), "BVH level");
    if (total > cap) throw GpuBvhError("device BVH node capacity exceeded");
    b = e;
    e = total;
  }
  out_nodes.resize(total);
  check(cudaMemcpyAsync(out_nodes.data(), nodes.p, sizeof(DNode) * (size_t)total, cudaMemcpyDeviceToHost, st),
        "nodes");
  leaf_perm.resize(n);
  check(cudaMemcpyAsync(leaf_perm.data(), perm.p, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, st), "perm");
  check(cudaStreamSynchronize(st), "BVH download");
}

}  // namespace pt
