// pt_host.cpp -- C-ABI of the GB300 path integrator (include/pathtracer_gb300.h):
// scene flattening and BVH construction with the reference's split rules,
// light discovery, device residency, the wave loop of pt_render, and the
// batch test entry points.  No exception crosses the ABI.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "pt_host.h"
#include "pt_bvh_gpu.h"

namespace pt {

// ------------------------------------------------------------- errors
static std::mutex g_err_mu;
static std::string g_last_error;

void fail(int code, const std::string &msg) { throw PtError(code, msg); }
void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) fail(PT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// ------------------------------------------------------- Halton tables
// gl::Primes (utility.hpp:400-402), digit counts and inverse radix powers
// exactly as the double loop of owenScrambledRadicalInverse computes them
// (digitPerm.hpp:105-128).
HaltonTables make_halton_tables() {
  static const int primes[PT_PRIME_COUNT] = {2,  3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37, 41,
                                             43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97};
  HaltonTables T;
  int off = 0;
  for (int b = 0; b < PT_PRIME_COUNT; ++b) {
    const int base = primes[b];
    T.prime[b] = base;
    const double inv_base = 1.0 / (double)base;
    double inv_base_m = 1.0;
    int nd = 0;
    while (1.0 - (base - 1) * inv_base_m < 1.0) {
      ++nd;
      inv_base_m *= inv_base;
    }
    T.ndigits[b] = nd;
    T.inv_base_m[b] = inv_base_m;
    T.perm_offset[b] = off;
    off += nd * base;
    div_invariant((uint32_t)base, T.div_magic[b], T.div_shift[b]);
    int check = 0;
    for (uint64_t p = 1; p < (1ull << 38) && check < nd; p *= (uint64_t)base) ++check;
    uint64_t tail = 1;
    for (int r = check; r < nd; ++r) tail *= (uint64_t)base;
    T.owen_check[b] = check;
    T.owen_tail[b] = tail;
  }
  return T;
}

// MurmurHash64A (Austin Appleby, public domain), the byte hash that
// pbrt::hash applies to its packed arguments (hash.hpp:10-58, 84-91).
static uint64_t murmur64a(const unsigned char *key, size_t len, uint64_t seed) {
  const uint64_t m = 0xc6a4a7935bd1e995ull;
  const int r = 47;
  uint64_t h = seed ^ (len * m);
  const unsigned char *end = key + 8 * (len / 8);
  for (; key != end; key += 8) {
    uint64_t k;
    std::memcpy(&k, key, 8);
    k *= m;
    k ^= k >> r;
    k *= m;
    h ^= k;
    h *= m;
  }
  const size_t rem = len & 7;
  for (size_t b = rem; b > 0; --b) h ^= uint64_t(key[b - 1]) << (8 * (b - 1));
  if (rem) h *= m;
  h ^= h >> r;
  h *= m;
  h ^= h >> r;
  return h;
}

// DigitPermutation tables (digitPerm.hpp:14-39) for every base.
std::vector<uint16_t> make_digit_permutations(const HaltonTables &T, uint32_t seed) {
  size_t total = 0;
  for (int b = 0; b < PT_PRIME_COUNT; ++b) total += (size_t)T.ndigits[b] * T.prime[b];
  std::vector<uint16_t> perm(total);
  for (int b = 0; b < PT_PRIME_COUNT; ++b) {
    const int base = T.prime[b];
    for (int di = 0; di < T.ndigits[b]; ++di) {
      unsigned char buf[12];
      int32_t bb = base, dd = di;
      std::memcpy(buf, &bb, 4);
      std::memcpy(buf + 4, &dd, 4);
      std::memcpy(buf + 8, &seed, 4);
      uint64_t dseed = murmur64a(buf, 12, 0);
      for (int v = 0; v < base; ++v)
        perm[T.perm_offset[b] + (size_t)di * base + v] =
            (uint16_t)permutation_element((uint32_t)v, (uint32_t)base, (uint32_t)dseed);
    }
  }
  return perm;
}

// ------------------------------------------------------------ materials
MatRec derive_material(const pt_material_desc &m) {
  MatRec r;
  std::memset(&r, 0, sizeof r);
  r.type = m.type;
  r.flags = m.flags;
  std::memcpy(r.p, m.p, sizeof r.p);
  if (m.type < 0 || m.type >= PT_MAT_COUNT) fail(PT_ERR_INVALID, "unknown material type");
  if (m.type == PT_MAT_DISNEY) {
    // DisneyPrincipledBSDF ctor (disneyPrincipledBSDF.hpp:34-66)
    const float st = m.p[3], metallic = m.p[4], sheen = m.p[10], cc = m.p[12];
    r.d[0] = (1 - metallic) * (1 - st);
    r.d[1] = (1 - st * (1 - metallic));
    r.d[2] = (1 - metallic) * st;
    r.d[3] = (float)(0.25 * cc);
    r.d[4] = (1 - metallic) * sheen;
    TR t = tr_from_roughness(m.p[7], m.p[9]);
    r.d[5] = t.ax;
    r.d[6] = t.ay;
    const float g = m.p[13];
    r.d[7] = (1.f - g) * 0.1f + g * 0.001f;  // ClearcoatTRD::fromClearcoatGloss
  } else if (m.type == PT_MAT_HAIR) {
    // HairMarschner ctor (hairMarsch.hpp:9-34)
    const float bm = m.p[5], bn = m.p[6], alpha = m.p[7];
    float v0 = sqr(0.726f * bm + 0.812f * sqr(bm) + 3.7f * std::pow(bm, 20.f));
    r.d[0] = v0;
    r.d[1] = (float)(.25 * v0);
    r.d[2] = 4 * v0;
    r.d[3] = r.d[2];
    const float sqrt_pi_over8 = 0.626657069f;
    r.d[4] = sqrt_pi_over8 * (0.265f * bn + 1.194f * sqr(bn) + 5.372f * std::pow(bn, 22.f));
    float s2k[3], c2k[3];
    s2k[0] = std::sin(alpha);
    c2k[0] = safe_sqrt(1 - sqr(s2k[0]));
    for (int i = 1; i < 3; ++i) {
      s2k[i] = 2 * c2k[i - 1] * s2k[i - 1];
      c2k[i] = sqr(c2k[i - 1]) - sqr(s2k[i - 1]);
    }
    for (int i = 0; i < 3; ++i) {
      r.d[5 + i] = s2k[i];
      r.d[8 + i] = c2k[i];
    }
    if (m.flags & PT_MAT_FLAG_MELANIN) {
      // Absorption from melanin concentrations (d'Eon et al. 2011, as
      // tabulated in pbrt-v3 HairBSDF::SigmaAFromConcentration): extension.
      const float eu[3] = {0.419f, 0.697f, 1.37f}, ph[3] = {0.187f, 0.4f, 1.05f};
      for (int c = 0; c < 3; ++c) r.d[11 + c] = m.p[8] * eu[c] + m.p[9] * ph[c];
    } else {
      for (int c = 0; c < 3; ++c) r.d[11 + c] = m.p[c];
    }
  }
  return r;
}

// Runs f(i) for i in [0, n) on up to `threads` host threads (0: all
// hardware threads), in contiguous chunks; f must touch disjoint state per i.
template <class F>
static void parallel_for(size_t n, int threads, F f) {
  unsigned hw = threads > 0 ? (unsigned)threads : std::max(1u, std::thread::hardware_concurrency());
  const size_t grain = 1 << 15;
  const unsigned nt = (unsigned)std::min<size_t>(hw, (n + grain - 1) / grain);
  if (nt <= 1) {
    for (size_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> pool;
  for (unsigned w = 0; w < nt; ++w)
    pool.emplace_back([&, w] {
      const size_t b = n * w / nt, e = n * (w + 1) / nt;
      for (size_t i = b; i < e; ++i) f(i);
    });
  for (auto &t : pool) t.join();
}

// ---------------------------------------------------------------- scene
struct Box {
  float lo[3], hi[3];
};
static Box box_empty() {
  Box b;
  for (int a = 0; a < 3; ++a) {
    b.lo[a] = INFINITY;
    b.hi[a] = -INFINITY;
  }
  return b;
}
static Box box_merge(const Box &x, const Box &y) {
  Box b;
  for (int a = 0; a < 3; ++a) {
    b.lo[a] = std::min(x.lo[a], y.lo[a]);
    b.hi[a] = std::max(x.hi[a], y.hi[a]);
  }
  return b;
}
static float box_area(const Box &b) {
  float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  if (!(dx >= 0.f)) return 0.f;
  return 2.f * (dx * dy + dy * dz + dz * dx);
}

// Binary tree in the shape the reference builds.
struct BNode {
  Box box;
  int left = -1, right = -1;  // internal
  int first = -1, count = 0;  // leaf: range of leaf_prims
};

struct Builder {
  const pt_scene_desc *d;
  int box_quad_base = 0;          // first rectangle of the boxes' faces
  int curve_base = 0;             // first curve primitive
  int threads = 0;               // mesh BVH build workers (0: hardware threads)
  bool gpu_bvh = false;          // large meshes built by the device builder
  bool sah = false;              // SAH trees instead of the reference's
  cudaStream_t gpu_stream = nullptr;
  std::vector<int> obj_motion;   // per object: motion index + 1 (0: static)
  std::vector<BNode> nodes;
  std::vector<int> inst_motion;  // per node: motion index + 1 if it roots a moving object's subtree
  std::vector<int> leaf_prims;    // global prim ids in leaf order
  std::vector<int> tri_base;      // first global prim id of each mesh
  int n_tris = 0;

  const float *pos(int mesh, int v) const { return d->meshes[mesh].positions + 3 * v; }

  // MeshBVHNode (meshBVH.cpp:6-55): box of the triangles +- 1e-3; leaf at
  // <= 4 triangles; otherwise split at the median of the centroids along
  // the longest axis, sorted with std::sort and the reference's comparator.
  // The centroids are computed once per mesh with the comparator's own
  // arithmetic ((v0 + v1 + v2) / 3.0f per component), so the sort sees the
  // same comparisons and gives the same order.  Large subtrees are built on
  // worker threads into their own arrays and spliced back in preorder: the
  // tree (node numbering, leaf order) is the one the sequential recursion
  // builds.
  struct Part {
    std::vector<BNode> nodes;
    std::vector<int> prims;
  };

  void mesh_centroids(int mesh, std::vector<float> cen[3]) const {
    const pt_mesh_desc &m = d->meshes[mesh];
    for (int a = 0; a < 3; ++a) cen[a].resize(m.n_triangles);
    for (int t = 0; t < m.n_triangles; ++t) {
      const float *p0 = pos(mesh, m.indices[3 * t]), *p1 = pos(mesh, m.indices[3 * t + 1]),
                  *p2 = pos(mesh, m.indices[3 * t + 2]);
      for (int a = 0; a < 3; ++a) cen[a][t] = ((p0[a] + p1[a]) + p2[a]) / 3.0f;
    }
  }

  void build_mesh_part(int mesh, std::vector<int> ids, const std::vector<float> *cen, Part &out,
                       int par_depth) const {
    const pt_mesh_desc &m = d->meshes[mesh];
    Box b = box_empty();
    for (int id : ids)
      for (int k = 0; k < 3; ++k) {
        const float *p = pos(mesh, m.indices[3 * id + k]);
        for (int a = 0; a < 3; ++a) {
          b.lo[a] = std::min(b.lo[a], p[a]);
          b.hi[a] = std::max(b.hi[a], p[a]);
        }
      }
    const float eps = 1e-3f;
    Box pb;
    for (int a = 0; a < 3; ++a) {
      pb.lo[a] = b.lo[a] - eps;
      pb.hi[a] = b.hi[a] + eps;
    }
    const int me = (int)out.nodes.size();
    out.nodes.push_back(BNode());
    out.nodes[me].box = pb;
    const int count = (int)ids.size();
    if (count <= 4) {
      out.nodes[me].first = (int)out.prims.size();
      out.nodes[me].count = count;
      for (int id : ids) out.prims.push_back(tri_base[mesh] + id);
      return;
    }
    float ext[3] = {b.hi[0] - b.lo[0], b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]};
    const int axis = ext[0] > ext[1] && ext[0] > ext[2] ? 0 : ext[1] > ext[2] ? 1 : 2;
    const std::vector<float> &c = cen[axis];
    std::sort(ids.begin(), ids.end(), [&](int x, int y) { return c[x] < c[y]; });
    const int mid = count / 2;
    std::vector<int> lids(ids.begin(), ids.begin() + mid), rids(ids.begin() + mid, ids.end());
    ids.clear();
    ids.shrink_to_fit();
    if (par_depth > 0 && count > (1 << 15)) {
      Part lp, rp;
      std::thread th([&] { build_mesh_part(mesh, std::move(lids), cen, lp, par_depth - 1); });
      build_mesh_part(mesh, std::move(rids), cen, rp, par_depth - 1);
      th.join();
      splice(out, me, lp, rp);
    } else {
      const int l = (int)out.nodes.size();
      build_mesh_part(mesh, std::move(lids), cen, out, 0);
      const int r = (int)out.nodes.size();
      build_mesh_part(mesh, std::move(rids), cen, out, 0);
      out.nodes[me].left = l;
      out.nodes[me].right = r;
    }
  }

  // Appends the left then the right subtree (each rooted at its index 0)
  // behind node `me`, renumbering nodes and leaf ranges.
  static void splice(Part &out, int me, const Part &lp, const Part &rp) {
    auto append = [&](const Part &p) {
      const int nb = (int)out.nodes.size(), pb = (int)out.prims.size();
      for (BNode n : p.nodes) {
        if (n.left >= 0) {
          n.left += nb;
          n.right += nb;
        } else {
          n.first += pb;
        }
        out.nodes.push_back(n);
      }
      out.prims.insert(out.prims.end(), p.prims.begin(), p.prims.end());
      return nb;
    };
    const int l = append(lp);
    const int r = append(rp);
    out.nodes[me].left = l;
    out.nodes[me].right = r;
  }

  int build_mesh(int mesh, std::vector<int> ids) {
    std::vector<float> cen[3];
    mesh_centroids(mesh, cen);
    unsigned hw = threads > 0 ? (unsigned)threads : std::max(1u, std::thread::hardware_concurrency());
    int par_depth = 0;
    while ((1u << par_depth) < hw && par_depth < 6) ++par_depth;
    if (ids.size() <= (1u << 16)) par_depth = 0;
    Part p;
    build_mesh_part(mesh, std::move(ids), cen, p, par_depth);
    return append_part(p);
  }

  // The same tree from the device builder (pt_bvh_gpu.cu), renumbered in
  // the host recursion's preorder.
  int build_mesh_gpu(int mesh) {
    const pt_mesh_desc &m = d->meshes[mesh];
    std::vector<GpuBvhNode> g;
    std::vector<int32_t> perm;
    try {
      gpu_mesh_bvh(m.positions, m.n_positions, m.indices, m.n_triangles, gpu_stream, g, perm);
    } catch (const GpuBvhError &e) {
      fail(PT_ERR_CUDA, e.what());
    }
    // appended to the scene's nodes in preorder (node, left subtree, right
    // subtree; an explicit stack of (device node, parent slot to patch))
    const int root = (int)nodes.size(), pb = (int)leaf_prims.size();
    nodes.reserve(nodes.size() + g.size());
    leaf_prims.resize(pb + perm.size());
    for (size_t k = 0; k < perm.size(); ++k) leaf_prims[pb + k] = tri_base[mesh] + perm[k];
    std::vector<std::pair<int, int>> stack = {{0, -1}};
    while (!stack.empty()) {
      auto [x, parent] = stack.back();
      stack.pop_back();
      if (x < 0 || x >= (int)g.size()) fail(PT_ERR_CUDA, "device BVH: bad child index");
      const GpuBvhNode &G = g[x];
      const int me = (int)nodes.size();
      nodes.push_back(BNode());
      BNode &N = nodes[me];
      for (int a = 0; a < 3; ++a) {
        N.box.lo[a] = G.lo[a];
        N.box.hi[a] = G.hi[a];
      }
      if (parent >= 0) {  // parent slot: 2 * node + side
        BNode &P = nodes[parent >> 1];
        (parent & 1 ? P.right : P.left) = me;
      }
      if (G.left < 0) {
        if (G.count < 1 || G.count > 4) fail(PT_ERR_CUDA, "device BVH: bad leaf");
        N.first = pb + G.start;
        N.count = G.count;
      } else {
        stack.push_back({G.left + 1, 2 * me + 1});  // right after the whole left subtree
        stack.push_back({G.left, 2 * me});
      }
    }
    return root;
  }

  // ------------------------------------------------------------ SAH trees
  // Binned surface-area-heuristic build (16 bins per axis over the centroid
  // box; cost 1 per node visit + 1 per item, leaves of up to 8 items).  Not
  // the reference's tree: the hits are the same (a BVH only decides which
  // boxes are visited), found with fewer visits where the median split of
  // the reference is far from the cost optimum.
  struct SahInput {
    const float *lo[3], *hi[3], *c[3];  // per item: box and centroid
  };
  static constexpr int SAH_BINS = 16, SAH_LEAF_MAX = 8;

  void sah_part(const SahInput &in, int *ids, int n, Part &out, int par_depth) const {
    Box b = box_empty(), cb = box_empty();
    for (int k = 0; k < n; ++k) {
      const int i = ids[k];
      for (int a = 0; a < 3; ++a) {
        b.lo[a] = std::min(b.lo[a], in.lo[a][i]);
        b.hi[a] = std::max(b.hi[a], in.hi[a][i]);
        cb.lo[a] = std::min(cb.lo[a], in.c[a][i]);
        cb.hi[a] = std::max(cb.hi[a], in.c[a][i]);
      }
    }
    const int me = (int)out.nodes.size();
    out.nodes.push_back(BNode());
    for (int a = 0; a < 3; ++a) {
      out.nodes[me].box.lo[a] = b.lo[a] - 1e-3f;
      out.nodes[me].box.hi[a] = b.hi[a] + 1e-3f;
    }
    auto make_leaf = [&] {
      out.nodes[me].first = (int)out.prims.size();
      out.nodes[me].count = n;
      for (int k = 0; k < n; ++k) out.prims.push_back(ids[k]);
    };
    if (n <= 2) return make_leaf();
    // best split over the three axes' bin boundaries
    float best = INFINITY;
    int best_axis = -1, best_bin = -1;
    for (int a = 0; a < 3; ++a) {
      const float ext = cb.hi[a] - cb.lo[a];
      if (!(ext > 0.f)) continue;
      Box bb[SAH_BINS];
      int cnt[SAH_BINS] = {0};
      for (int k = 0; k < SAH_BINS; ++k) bb[k] = box_empty();
      const float scale = SAH_BINS / ext;
      for (int k = 0; k < n; ++k) {
        const int i = ids[k];
        const int bin = std::min(SAH_BINS - 1, (int)((in.c[a][i] - cb.lo[a]) * scale));
        ++cnt[bin];
        for (int q = 0; q < 3; ++q) {
          bb[bin].lo[q] = std::min(bb[bin].lo[q], in.lo[q][i]);
          bb[bin].hi[q] = std::max(bb[bin].hi[q], in.hi[q][i]);
        }
      }
      float right_area[SAH_BINS];
      int right_cnt[SAH_BINS];
      Box acc = box_empty();
      int ac = 0;
      for (int k = SAH_BINS - 1; k > 0; --k) {
        acc = box_merge(acc, bb[k]);
        ac += cnt[k];
        right_area[k] = box_area(acc);
        right_cnt[k] = ac;
      }
      acc = box_empty();
      ac = 0;
      for (int k = 0; k < SAH_BINS - 1; ++k) {
        acc = box_merge(acc, bb[k]);
        ac += cnt[k];
        if (ac == 0 || right_cnt[k + 1] == 0) continue;
        const float cost = box_area(acc) * ac + right_area[k + 1] * right_cnt[k + 1];
        if (cost < best) {
          best = cost;
          best_axis = a;
          best_bin = k;
        }
      }
    }
    const float parent_area = std::max(box_area(b), 1e-30f);
    const float split_cost = 1.f + best / parent_area;
    if (best_axis < 0 || (n <= SAH_LEAF_MAX && split_cost >= (float)n)) {
      if (n <= SAH_LEAF_MAX) return make_leaf();
    }
    int mid;
    if (best_axis < 0) {  // all centroids equal: halves
      mid = n / 2;
    } else {
      const float ext = cb.hi[best_axis] - cb.lo[best_axis], scale = SAH_BINS / ext;
      int *p = std::partition(ids, ids + n, [&](int i) {
        return std::min(SAH_BINS - 1, (int)((in.c[best_axis][i] - cb.lo[best_axis]) * scale)) <= best_bin;
      });
      mid = (int)(p - ids);
      if (mid == 0 || mid == n) mid = n / 2;
    }
    if (par_depth > 0 && n > (1 << 15)) {
      Part lp, rp;
      std::thread th([&] { sah_part(in, ids, mid, lp, par_depth - 1); });
      sah_part(in, ids + mid, n - mid, rp, par_depth - 1);
      th.join();
      splice(out, me, lp, rp);
    } else {
      const int l = (int)out.nodes.size();
      sah_part(in, ids, mid, out, 0);
      const int r = (int)out.nodes.size();
      sah_part(in, ids + mid, n - mid, out, 0);
      out.nodes[me].left = l;
      out.nodes[me].right = r;
    }
  }

  int build_mesh_sah(int mesh) {
    const pt_mesh_desc &m = d->meshes[mesh];
    const int n = m.n_triangles;
    std::vector<float> arr(9 * (size_t)n);
    SahInput in;
    for (int a = 0; a < 3; ++a) {
      in.lo[a] = arr.data() + (size_t)a * n;
      in.hi[a] = arr.data() + (size_t)(3 + a) * n;
      in.c[a] = arr.data() + (size_t)(6 + a) * n;
    }
    parallel_for((size_t)n, threads, [&](size_t t) {
      const float *p0 = pos(mesh, m.indices[3 * t]), *p1 = pos(mesh, m.indices[3 * t + 1]),
                  *p2 = pos(mesh, m.indices[3 * t + 2]);
      for (int a = 0; a < 3; ++a) {
        arr[(size_t)a * n + t] = std::min(std::min(p0[a], p1[a]), p2[a]);
        arr[(size_t)(3 + a) * n + t] = std::max(std::max(p0[a], p1[a]), p2[a]);
        arr[(size_t)(6 + a) * n + t] = ((p0[a] + p1[a]) + p2[a]) / 3.0f;
      }
    });
    std::vector<int> ids(n);
    std::iota(ids.begin(), ids.end(), 0);
    unsigned hw = threads > 0 ? (unsigned)threads : std::max(1u, std::thread::hardware_concurrency());
    int par_depth = 0;
    while ((1u << par_depth) < hw && par_depth < 6) ++par_depth;
    Part p;
    sah_part(in, ids.data(), n, p, n > (1 << 16) ? par_depth : 0);
    for (int &x : p.prims) x += tri_base[mesh];
    return append_part(p);
  }

  // Top level over objects with the same heuristic (object boxes); its
  // leaves are the objects' subtrees.
  int sah_top(std::vector<int> objs) {
    if (objs.size() == 1) return object_subtree(objs[0]);
    Box cb = box_empty();
    std::vector<Box> ob(objs.size());
    for (size_t k = 0; k < objs.size(); ++k) {
      ob[k] = object_box(objs[k]);
      for (int a = 0; a < 3; ++a) {
        const float c = 0.5f * (ob[k].lo[a] + ob[k].hi[a]);
        cb.lo[a] = std::min(cb.lo[a], c);
        cb.hi[a] = std::max(cb.hi[a], c);
      }
    }
    // exact sweep over the sorted order of each axis (object counts are small)
    float best = INFINITY;
    int best_axis = -1, best_k = -1;
    std::vector<int> order(objs.size());
    const int n = (int)objs.size();
    for (int a = 0; a < 3; ++a) {
      std::iota(order.begin(), order.end(), 0);
      std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return ob[x].lo[a] + ob[x].hi[a] < ob[y].lo[a] + ob[y].hi[a];
      });
      std::vector<float> ra(n);
      Box acc = box_empty();
      for (int k = n - 1; k > 0; --k) {
        acc = box_merge(acc, ob[order[k]]);
        ra[k] = box_area(acc);
      }
      acc = box_empty();
      for (int k = 0; k < n - 1; ++k) {
        acc = box_merge(acc, ob[order[k]]);
        const float cost = box_area(acc) * (k + 1) + ra[k + 1] * (n - k - 1);
        if (cost < best) {
          best = cost;
          best_axis = a;
          best_k = k;
        }
      }
    }
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      return ob[x].lo[best_axis] + ob[x].hi[best_axis] < ob[y].lo[best_axis] + ob[y].hi[best_axis];
    });
    std::vector<int> lo_objs, hi_objs;
    for (int k = 0; k < n; ++k) (k <= best_k ? lo_objs : hi_objs).push_back(objs[order[k]]);
    const int l = sah_top(std::move(lo_objs));
    const int r = sah_top(std::move(hi_objs));
    const int me = (int)nodes.size();
    nodes.push_back(BNode());
    nodes[me].left = l;
    nodes[me].right = r;
    nodes[me].box = box_merge(nodes[l].box, nodes[r].box);
    return me;
  }

  // Appends a mesh tree (rooted at its index 0) to the scene's nodes.
  int append_part(Part &p) {
    Part top;
    top.nodes = std::move(nodes);
    top.prims = std::move(leaf_prims);
    const int root = (int)top.nodes.size(), pb = (int)top.prims.size();
    for (BNode n : p.nodes) {
      if (n.left >= 0) {
        n.left += root;
        n.right += root;
      } else {
        n.first += pb;
      }
      top.nodes.push_back(n);
    }
    top.prims.insert(top.prims.end(), p.prims.begin(), p.prims.end());
    nodes = std::move(top.nodes);
    leaf_prims = std::move(top.prims);
    return root;
  }

  Box object_box(int o) const {
    const pt_object_desc &od = d->objects[o];
    Box b;
    if (od.kind == PT_OBJ_MESH) {  // TriangleMesh::meshAABB (triangleMesh.cpp:10-18)
      const pt_mesh_desc &m = d->meshes[od.index];
      b = box_empty();
      for (int v = 0; v < m.n_positions; ++v)
        for (int a = 0; a < 3; ++a) {
          b.lo[a] = std::min(b.lo[a], m.positions[3 * v + a]);
          b.hi[a] = std::max(b.hi[a], m.positions[3 * v + a]);
        }
      for (int a = 0; a < 3; ++a) {
        b.lo[a] -= 1e-3f;
        b.hi[a] += 1e-3f;
      }
    } else if (od.kind == PT_OBJ_CURVE) {  // Curve::getAABB (curve.hpp:33-46)
      const pt_curve_desc &cv = d->curves[od.index];
      b = box_empty();
      for (int k = 0; k < 4; ++k)
        for (int a = 0; a < 3; ++a) {
          b.lo[a] = std::min(b.lo[a], cv.cps[k][a]);
          b.hi[a] = std::max(b.hi[a], cv.cps[k][a]);
        }
      const float r = std::max(cv.width0, cv.width1);
      for (int a = 0; a < 3; ++a) {
        b.lo[a] -= r;
        b.hi[a] += r;
      }
    } else if (od.kind == PT_OBJ_BOX) {  // Box::getAABB (box.hpp:36)
      const pt_box_desc &bx = d->boxes[od.index];
      for (int a = 0; a < 3; ++a) {
        b.lo[a] = bx.min_xyz[a];
        b.hi[a] = bx.max_xyz[a];
      }
    } else if (od.kind == PT_OBJ_QUAD) {  // AARectangle::getAABB (primitive.cpp:6-28)
      const pt_quad_desc &q = d->quads[od.index];
      int a0 = q.axis == 0 ? 1 : 0, a1 = q.axis == 2 ? 1 : 2;
      b.lo[q.axis] = q.k - 1e-3f;
      b.hi[q.axis] = q.k + 1e-3f;
      b.lo[a0] = q.d0_min;
      b.hi[a0] = q.d0_max;
      b.lo[a1] = q.d1_min;
      b.hi[a1] = q.d1_max;
    } else {  // Sphere::getAABB (primitive.hpp:117-122)
      const pt_sphere_desc &s = d->spheres[od.index];
      for (int a = 0; a < 3; ++a) {
        b.lo[a] = s.center[a] - s.radius;
        b.hi[a] = s.center[a] + s.radius;
      }
    }
    return b;
  }

  // Motion blur: a moving object's subtree keeps its boxes at rest (it is
  // traversed in the object's frame at the ray's time); only its root box,
  // seen from the world, covers the motion over [0, shutter_max].
  void sweep_root(int root, int o) {
    if (!obj_motion[o]) return;
    const float *v = d->objects[o].velocity;
    Box &b = nodes[root].box;
    for (int a = 0; a < 3; ++a) {
      const float s = v[a] * d->shutter_max;
      b.lo[a] = std::min(b.lo[a], b.lo[a] + s);
      b.hi[a] = std::max(b.hi[a], b.hi[a] + s);
    }
    if (nodes[root].left >= 0) inst_motion[root] = obj_motion[o];
  }

  int object_subtree(int o) {
    const pt_object_desc &od = d->objects[o];
    int me;
    if (od.kind == PT_OBJ_MESH) {
      const pt_mesh_desc &m = d->meshes[od.index];
      std::vector<int> ids(m.n_triangles);
      std::iota(ids.begin(), ids.end(), 0);
      if (sah && m.n_triangles > 4)
        me = build_mesh_sah(od.index);
      else if (gpu_bvh && m.n_triangles >= PT_GPU_BVH_MIN)
        me = build_mesh_gpu(od.index);
      else
        me = build_mesh(od.index, ids);
    } else {
      me = (int)nodes.size();
      nodes.push_back(BNode());
      nodes[me].box = object_box(o);
      nodes[me].first = (int)leaf_prims.size();
      if (od.kind == PT_OBJ_CURVE) {
        nodes[me].count = 1;
        leaf_prims.push_back(curve_base + od.index);
      } else if (od.kind == PT_OBJ_BOX) {  // one leaf: the six faces in the box's order
        nodes[me].count = 6;
        for (int k = 0; k < 6; ++k) leaf_prims.push_back(n_tris + box_quad_base + 6 * od.index + k);
      } else {
        nodes[me].count = 1;
        int prim = od.kind == PT_OBJ_QUAD ? n_tris + od.index : n_tris + d->n_quads + od.index;
        leaf_prims.push_back(prim);
      }
    }
    inst_motion.resize(nodes.size(), 0);
    sweep_root(me, o);
    return me;
  }

  // BVHNode (bvh.hpp:46-102).  The reference sorts a local copy of the
  // object list and then recurses on the UNSORTED list, so the subtrees
  // split the insertion order in halves; the split axis drawn from rand()
  // only orders the two children of a two-object node.  rand() is called
  // once per node, in construction order, as the reference does.
  int build_top(int i, int j) {
    int axis = std::rand() % 3;
    if (j - i == 1) return object_subtree(i);
    if (j - i == 2) {
      Box a = object_box(i), b = object_box(i + 1);
      bool first_left = (a.lo[axis] + a.hi[axis]) * 0.5f < (b.lo[axis] + b.hi[axis]) * 0.5f;
      int l = object_subtree(first_left ? i : i + 1);
      int r = object_subtree(first_left ? i + 1 : i);
      int me = (int)nodes.size();
      nodes.push_back(BNode());
      nodes[me].left = l;
      nodes[me].right = r;
      nodes[me].box = box_merge(nodes[l].box, nodes[r].box);
      return me;
    }
    int mid = i + (j - i) / 2;
    int l = build_top(i, mid);
    int r = build_top(mid, j);
    int me = (int)nodes.size();
    nodes.push_back(BNode());
    nodes[me].left = l;
    nodes[me].right = r;
    nodes[me].box = box_merge(nodes[l].box, nodes[r].box);
    return me;
  }
};

struct Bvh4Out {
  std::vector<Bvh4Node> nodes;
  std::vector<int> node_motion;   // per node: motion index + 1 of the moving object it roots
  std::vector<int> leaf_order;    // leaf prims in item order
  std::vector<char> leaf_world;   // per item: tested from the world frame (not inside a moving subtree)
  int max_depth = 0;
};

static int motion_of(const Builder &B, int bn) {
  return bn < (int)B.inst_motion.size() ? B.inst_motion[bn] : 0;
}

// Collapses the binary tree under `bn` into BVH4 node `me`.  A moving
// object's subtree root met from the world frame is never merged into a world
// node: it becomes a child of its own (reference flagged PT_INST_BIT) whose
// subtree is traversed in the object's frame.
// Appends a subtree collapsed on its own (its root at index 0) behind `out`
// and returns the root's index there: internal child references and leaf
// item ranges are offset, so the result is the sequential collapse's.
static int splice_collapsed(Bvh4Out &out, Bvh4Out &sub) {
  const int base = (int)out.nodes.size(), lbase = (int)out.leaf_order.size();
  for (Bvh4Node N : sub.nodes) {
    for (int k = 0; k < 4; ++k) {
      if (N.count[k] == 0)
        N.child[k] = (N.child[k] & PT_INST_BIT) | ((N.child[k] & ~PT_INST_BIT) + base);
      else if (N.count[k] > 0)
        N.child[k] += lbase;
    }
    out.nodes.push_back(N);
  }
  out.node_motion.insert(out.node_motion.end(), sub.node_motion.begin(), sub.node_motion.end());
  out.leaf_order.insert(out.leaf_order.end(), sub.leaf_order.begin(), sub.leaf_order.end());
  out.leaf_world.insert(out.leaf_world.end(), sub.leaf_world.begin(), sub.leaf_world.end());
  out.max_depth = std::max(out.max_depth, sub.max_depth);
  return base;
}

// par > 0: the internal children's subtrees are collapsed on their own
// threads (par - 1 levels further down) and spliced in child order, which
// numbers nodes and leaf items exactly as the sequential recursion does.
static void collapse(const Builder &B, int bn, Bvh4Out &out, int depth, int me, bool in_inst, int par = 0) {
  // gather up to 4 children by expanding the largest internal child
  int ch[4], nch = 2;
  ch[0] = B.nodes[bn].left;
  ch[1] = B.nodes[bn].right;
  if (B.nodes[bn].left < 0) {  // a leaf as the root
    ch[0] = bn;
    nch = 1;
  }
  while (nch < 4) {
    int best = -1;
    float ba = -1.f;
    for (int k = 0; k < nch; ++k) {
      const BNode &c = B.nodes[ch[k]];
      if (c.left >= 0 && (in_inst || !motion_of(B, ch[k])) && box_area(c.box) > ba) {
        ba = box_area(c.box);
        best = k;
      }
    }
    if (best < 0) break;
    const int x = ch[best];
    for (int k = nch; k > best + 1; --k) ch[k] = ch[k - 1];
    ch[best] = B.nodes[x].left;
    ch[best + 1] = B.nodes[x].right;
    ++nch;
  }
  out.max_depth = std::max(out.max_depth, depth + 1);
  Bvh4Node &N0 = out.nodes[me];
  for (int k = 0; k < 4; ++k) {
    N0.lo_x[k] = N0.lo_y[k] = N0.lo_z[k] = INFINITY;
    N0.hi_x[k] = N0.hi_y[k] = N0.hi_z[k] = -INFINITY;
    N0.child[k] = 0;
    N0.count[k] = -1;
  }
  if (par > 0) {
    Bvh4Out subs[4];
    bool enters[4] = {false, false, false, false};
    std::vector<std::thread> pool;
    for (int k = 0; k < nch; ++k) {
      const BNode &c = B.nodes[ch[k]];
      if (c.left < 0) continue;
      enters[k] = !in_inst && motion_of(B, ch[k]);
      subs[k].nodes.push_back(Bvh4Node());
      subs[k].node_motion.push_back(enters[k] ? motion_of(B, ch[k]) : 0);
      pool.emplace_back([&, k] { collapse(B, ch[k], subs[k], depth + 1, 0, in_inst || enters[k], par - 1); });
    }
    for (auto &t : pool) t.join();
    for (int k = 0; k < nch; ++k) {
      const BNode &c = B.nodes[ch[k]];
      Bvh4Node &N = out.nodes[me];
      N.lo_x[k] = c.box.lo[0];
      N.lo_y[k] = c.box.lo[1];
      N.lo_z[k] = c.box.lo[2];
      N.hi_x[k] = c.box.hi[0];
      N.hi_y[k] = c.box.hi[1];
      N.hi_z[k] = c.box.hi[2];
      if (c.left < 0) {
        N.child[k] = (int)out.leaf_order.size();
        N.count[k] = c.count;
        for (int t = 0; t < c.count; ++t) {
          out.leaf_order.push_back(B.leaf_prims[c.first + t]);
          out.leaf_world.push_back(in_inst ? 0 : 1);
        }
      } else {
        const int idx = splice_collapsed(out, subs[k]);
        out.nodes[me].child[k] = enters[k] ? (idx | PT_INST_BIT) : idx;
        out.nodes[me].count[k] = 0;
      }
    }
    return;
  }
  for (int k = 0; k < nch; ++k) {
    const BNode &c = B.nodes[ch[k]];
    Bvh4Node &N = out.nodes[me];
    N.lo_x[k] = c.box.lo[0];
    N.lo_y[k] = c.box.lo[1];
    N.lo_z[k] = c.box.lo[2];
    N.hi_x[k] = c.box.hi[0];
    N.hi_y[k] = c.box.hi[1];
    N.hi_z[k] = c.box.hi[2];
    if (c.left < 0) {
      N.child[k] = (int)out.leaf_order.size();
      N.count[k] = c.count;
      for (int t = 0; t < c.count; ++t) {
        out.leaf_order.push_back(B.leaf_prims[c.first + t]);
        out.leaf_world.push_back(in_inst ? 0 : 1);
      }
    } else {
      int idx = (int)out.nodes.size();
      out.nodes.push_back(Bvh4Node());
      out.node_motion.push_back(0);
      const bool enter = !in_inst && motion_of(B, ch[k]);
      out.nodes[me].child[k] = enter ? (idx | PT_INST_BIT) : idx;
      out.nodes[me].count[k] = 0;
      if (enter) out.node_motion[idx] = motion_of(B, ch[k]);
      collapse(B, ch[k], out, depth + 1, idx, in_inst || enter);
    }
  }
}

template <class T>
static T *dupload(const std::vector<T> &v, std::vector<void *> &owned, cudaStream_t st) {
  if (v.empty()) return nullptr;
  void *p = nullptr;
  cuda_check(cudaMalloc(&p, sizeof(T) * v.size()), "cudaMalloc(scene)");
  owned.push_back(p);
  cuda_check(cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st),
             "upload scene");
  return static_cast<T *>(p);
}

// FrameBuffer::gaussianBlur's kernel (framebuffer.cpp:60-87): k x k weights
// exp(-r^2 / (2 sigma^2)) / (2 pi sigma^2), r = sqrt(x^2 + y^2), divided by
// their float sum; row-major [s][t].  Empty when the reference refuses the
// arguments (k even or < 3, sigma < 0; sigma = 0 divides by zero there and
// is refused here too).
std::vector<float> gaussian_weights(int k, float sigma) {
  std::vector<float> w;
  if (k % 2 == 0 || k < 3 || !(sigma > 0.f)) return w;
  w.resize((size_t)k * k);
  float sum = 0.0f;
  for (int x = -k / 2; x <= k / 2; x++)
    for (int y = -k / 2; y <= k / 2; y++) {
      float r = (float)std::sqrt((double)(x * x + y * y));
      float e = std::exp(-(r * r) / (2 * sigma * sigma));
      float v = (float)((double)e / (2 * M_PI * sigma * sigma));
      w[(size_t)(x + k / 2) * k + (y + k / 2)] = v;
      sum += v;
    }
  for (float &v : w) v /= sum;
  return w;
}

// Minimal PNG encoder: 8-bit RGB, filter 0 rows, zlib stream of stored
// (uncompressed) deflate blocks, CRC-32 and Adler-32 from their published
// definitions (PNG spec, RFC 1950/1951).
static uint32_t crc32_update(uint32_t c, const unsigned char *p, size_t n) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t v = i;
      for (int k = 0; k < 8; ++k) v = (v & 1) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
      table[i] = v;
    }
    init = true;
  }
  for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xff] ^ (c >> 8);
  return c;
}

void write_png(const char *path, const uint8_t *rgb, int W, int H) {
  std::vector<unsigned char> raw;
  raw.reserve((size_t)H * (3 * W + 1));
  for (int y = 0; y < H; ++y) {
    raw.push_back(0);
    raw.insert(raw.end(), rgb + (size_t)y * W * 3, rgb + (size_t)(y + 1) * W * 3);
  }
  std::vector<unsigned char> z = {0x78, 0x01};
  uint32_t a = 1, b = 0;
  for (unsigned char ch : raw) {
    a = (a + ch) % 65521u;
    b = (b + a) % 65521u;
  }
  for (size_t off = 0; off < raw.size() || off == 0;) {
    const size_t len = std::min<size_t>(65535, raw.size() - off);
    const bool last = off + len >= raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((unsigned char)(len & 0xff));
    z.push_back((unsigned char)(len >> 8));
    z.push_back((unsigned char)(~len & 0xff));
    z.push_back((unsigned char)((~len >> 8) & 0xff));
    z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
    off += len;
    if (last) break;
  }
  const uint32_t adler = (b << 16) | a;
  for (int s = 24; s >= 0; s -= 8) z.push_back((unsigned char)(adler >> s));
  FILE *f = std::fopen(path, "wb");
  if (!f) fail(PT_ERR_INVALID, std::string("cannot write ") + path);
  auto be32 = [](unsigned char *o, uint32_t v) {
    o[0] = (unsigned char)(v >> 24); o[1] = (unsigned char)(v >> 16); o[2] = (unsigned char)(v >> 8); o[3] = (unsigned char)v;
  };
  auto chunk = [&](const char *type, const unsigned char *data, size_t n) {
    unsigned char hdr[8];
    be32(hdr, (uint32_t)n);
    std::memcpy(hdr + 4, type, 4);
    uint32_t c = crc32_update(0xffffffffu, hdr + 4, 4);
    c = crc32_update(c, data, n) ^ 0xffffffffu;
    unsigned char tail[4];
    be32(tail, c);
    std::fwrite(hdr, 1, 8, f);
    if (n) std::fwrite(data, 1, n, f);
    std::fwrite(tail, 1, 4, f);
  };
  static const unsigned char sig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
  std::fwrite(sig, 1, 8, f);
  unsigned char ihdr[13];
  be32(ihdr, (uint32_t)W);
  be32(ihdr + 4, (uint32_t)H);
  ihdr[8] = 8;   // bit depth
  ihdr[9] = 2;   // colour type RGB
  ihdr[10] = 0;  // deflate
  ihdr[11] = 0;  // filter method 0
  ihdr[12] = 0;  // no interlace
  chunk("IHDR", ihdr, 13);
  chunk("IDAT", z.data(), z.size());
  chunk("IEND", nullptr, 0);
  const bool ok = std::fclose(f) == 0;
  if (!ok) fail(PT_ERR_INVALID, std::string("cannot write ") + path);
}

static uint64_t fnv1a(const void *p, size_t n, uint64_t h) {
  const unsigned char *b = static_cast<const unsigned char *>(p);
  for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 0x100000001b3ull;
  return h;
}

// Builds a scene; with device = false only the host part (validation, BVH,
// tables) runs, without touching the GPU.  threads: worker threads of the
// mesh BVH build (0: all hardware threads).
// Box faces (box.hpp:16-33): YZ at x1, x0; XZ at y1, y0; XY at z1, z0.
static void box_faces(const pt_box_desc &b, std::vector<pt_quad_desc> &out) {
  const float *lo = b.min_xyz, *hi = b.max_xyz;
  out.push_back(pt_quad_desc{0, hi[0], lo[1], hi[1], lo[2], hi[2], b.material, 0});
  out.push_back(pt_quad_desc{0, lo[0], lo[1], hi[1], lo[2], hi[2], b.material, 0});
  out.push_back(pt_quad_desc{1, hi[1], lo[0], hi[0], lo[2], hi[2], b.material, 0});
  out.push_back(pt_quad_desc{1, lo[1], lo[0], hi[0], lo[2], hi[2], b.material, 0});
  out.push_back(pt_quad_desc{2, hi[2], lo[0], hi[0], lo[1], hi[1], b.material, 0});
  out.push_back(pt_quad_desc{2, lo[2], lo[0], hi[0], lo[1], hi[1], b.material, 0});
}

std::unique_ptr<Scene> build_scene(const pt_scene_desc *d_in, cudaStream_t st, bool device, int threads,
                                   int trav_cap, int builder, bool want_hash) {
  if (!d_in) fail(PT_ERR_INVALID, "null scene description");
  // boxes become six rectangles each, after the scene's own rectangles
  pt_scene_desc aug = *d_in;
  std::vector<pt_quad_desc> all_quads;
  const int n_boxes = d_in->boxes ? d_in->n_boxes : 0;
  if (n_boxes < 0) fail(PT_ERR_INVALID, "negative box count");
  if (n_boxes > 0) {
    all_quads.assign(d_in->quads, d_in->quads + std::max(0, d_in->n_quads));
    for (int b = 0; b < n_boxes; ++b) box_faces(d_in->boxes[b], all_quads);
    aug.quads = all_quads.data();
    aug.n_quads = (int32_t)all_quads.size();
  }
  const pt_scene_desc *d = &aug;
  const int n_user_quads = d_in->n_quads;
  if (d->n_objects <= 0) fail(PT_ERR_INVALID, "scene has no objects");  // renderManager.hpp:64
  auto S = std::make_unique<Scene>();
  Builder B;
  B.d = d;
  B.threads = threads;
  B.gpu_bvh = builder == PT_BVH_BUILD_DEVICE;
  B.sah = builder == PT_BVH_BUILD_SAH;
  B.gpu_stream = st;
  B.box_quad_base = n_user_quads;
  for (int m = 0; m < d->n_meshes; ++m) {
    const pt_mesh_desc &md = d->meshes[m];
    if (md.n_triangles < 0 || (md.n_triangles > 0 && (!md.positions || !md.indices)))
      fail(PT_ERR_INVALID, "mesh without positions or indices");
    if (md.material < 0 || md.material >= d->n_materials) fail(PT_ERR_INVALID, "mesh material out of range");
    for (int t = 0; t < 3 * md.n_triangles; ++t)
      if (md.indices[t] < 0 || md.indices[t] >= md.n_positions)
        fail(PT_ERR_INVALID, "mesh index out of range");
    for (int v = 0; v < 3 * md.n_positions; ++v)
      if (!std::isfinite(md.positions[v])) fail(PT_ERR_INVALID, "mesh position not finite");
    B.tri_base.push_back(B.n_tris);
    B.n_tris += md.n_triangles;
  }
  auto finite = [](std::initializer_list<float> xs) {
    for (float x : xs)
      if (!std::isfinite(x)) return false;
    return true;
  };
  for (int q = 0; q < d->n_quads; ++q) {
    const pt_quad_desc &Q = d->quads[q];
    if (Q.material < 0 || Q.material >= d->n_materials || Q.axis < 0 || Q.axis > 2 ||
        !finite({Q.k, Q.d0_min, Q.d0_max, Q.d1_min, Q.d1_max}))
      fail(PT_ERR_INVALID, "bad quad");
  }
  for (int s = 0; s < d->n_spheres; ++s) {
    const pt_sphere_desc &P = d->spheres[s];
    if (P.material < 0 || P.material >= d->n_materials || !finite({P.center[0], P.center[1], P.center[2], P.radius}))
      fail(PT_ERR_INVALID, "bad sphere");
  }
  const int n_curves = d->curves ? d->n_curves : 0;
  if (n_curves < 0) fail(PT_ERR_INVALID, "negative curve count");
  for (int o = 0; o < d->n_objects; ++o) {
    const pt_object_desc &od = d->objects[o];
    int lim = od.kind == PT_OBJ_MESH  ? d->n_meshes
              : od.kind == PT_OBJ_QUAD  ? n_user_quads
              : od.kind == PT_OBJ_BOX   ? n_boxes
              : od.kind == PT_OBJ_CURVE ? n_curves
                                        : d->n_spheres;
    if (od.kind < 0 || od.kind > 4 || od.index < 0 || od.index >= lim)
      fail(PT_ERR_INVALID, "bad object entry");
  }
  for (int c = 0; c < n_curves; ++c) {
    const pt_curve_desc &K = d->curves[c];
    bool ok = K.material >= 0 && K.material < d->n_materials && finite({K.width0, K.width1});
    for (int k = 0; k < 4; ++k) ok = ok && finite({K.cps[k][0], K.cps[k][1], K.cps[k][2]});
    if (!ok) fail(PT_ERR_INVALID, "bad curve");
  }
  const int curve_base = B.n_tris + d->n_quads + d->n_spheres;  // first curve primitive
  B.curve_base = curve_base;
  const int n_prims = curve_base + n_curves;
  // motion blur: one motion record per moving object, index + 1 on its
  // primitives (a mesh shared by several objects takes the last one's)
  std::vector<float4> motion;
  std::vector<int> prim_motion(n_prims, 0);
  // pt_object_desc.face per primitive: PT_PRIM_FACE_* flags (0: as hit)
  std::vector<int> prim_face(n_prims, 0);
  B.obj_motion.assign(d->n_objects, 0);
  for (int o = 0; o < d->n_objects; ++o) {
    const pt_object_desc &od = d->objects[o];
    if (od.face < PT_FACE_AS_HIT || od.face > PT_FACE_BACK) fail(PT_ERR_INVALID, "bad object face mode");
    if (od.face == PT_FACE_AS_HIT) continue;
    const int ff = PT_PRIM_FACE_FIXED | (od.face == PT_FACE_FRONT ? PT_PRIM_FACE_FRONT : 0);
    if (od.kind == PT_OBJ_MESH)
      for (int t = 0; t < d->meshes[od.index].n_triangles; ++t) prim_face[B.tri_base[od.index] + t] = ff;
    else if (od.kind == PT_OBJ_BOX)
      for (int k = 0; k < 6; ++k) prim_face[B.n_tris + n_user_quads + 6 * od.index + k] = ff;
    else if (od.kind == PT_OBJ_CURVE)
      prim_face[curve_base + od.index] = ff;
    else
      prim_face[od.kind == PT_OBJ_QUAD ? B.n_tris + od.index : B.n_tris + d->n_quads + od.index] = ff;
  }
  for (int o = 0; o < d->n_objects; ++o) {
    const pt_object_desc &od = d->objects[o];
    const float *v = od.velocity;
    if (!std::isfinite(v[0]) || !std::isfinite(v[1]) || !std::isfinite(v[2]))
      fail(PT_ERR_INVALID, "object velocity must be finite");
    if (v[0] == 0.f && v[1] == 0.f && v[2] == 0.f) continue;
    motion.push_back(make_float4(v[0], v[1], v[2], 0.f));
    const int m = (int)motion.size();
    B.obj_motion[o] = m;
    if (od.kind == PT_OBJ_MESH) {
      for (int t = 0; t < d->meshes[od.index].n_triangles; ++t) prim_motion[B.tri_base[od.index] + t] = m;
    } else {
      if (od.kind == PT_OBJ_BOX)
        for (int k = 0; k < 6; ++k) prim_motion[B.n_tris + n_user_quads + 6 * od.index + k] = m;
      else if (od.kind == PT_OBJ_CURVE)
        prim_motion[curve_base + od.index] = m;
      else
        prim_motion[od.kind == PT_OBJ_QUAD ? B.n_tris + od.index : B.n_tris + d->n_quads + od.index] = m;
    }
  }
  if (!motion.empty() && !(d->shutter_max > 0.f) )
    fail(PT_ERR_INVALID, "moving objects need shutter_max > 0");
  std::srand(1);  // the reference's BVH build draws from rand() with its default seed
  int root;
  if (B.sah) {
    std::vector<int> all(d->n_objects);
    std::iota(all.begin(), all.end(), 0);
    root = B.sah_top(std::move(all));
  } else {
    root = B.build_top(0, d->n_objects);
  }

  B.inst_motion.resize(B.nodes.size(), 0);
  // large trees are collapsed on host threads (two levels of fan-out)
  const int collapse_par = (threads != 1 && B.nodes.size() > (1u << 16)) ? 2 : 0;
  Bvh4Out out;
  out.nodes.push_back(Bvh4Node());
  out.node_motion.push_back(0);
  if (motion_of(B, root)) {
    // the whole scene is one moving object: a world node above its subtree
    Bvh4Node &R = out.nodes[0];
    for (int k = 0; k < 4; ++k) {
      R.lo_x[k] = R.lo_y[k] = R.lo_z[k] = INFINITY;
      R.hi_x[k] = R.hi_y[k] = R.hi_z[k] = -INFINITY;
      R.child[k] = 0;
      R.count[k] = -1;
    }
    const Box &b = B.nodes[root].box;
    R.lo_x[0] = b.lo[0]; R.lo_y[0] = b.lo[1]; R.lo_z[0] = b.lo[2];
    R.hi_x[0] = b.hi[0]; R.hi_y[0] = b.hi[1]; R.hi_z[0] = b.hi[2];
    R.child[0] = 1 | PT_INST_BIT;
    R.count[0] = 0;
    out.nodes.push_back(Bvh4Node());
    out.node_motion.push_back(motion_of(B, root));
    collapse(B, root, out, 1, 1, true, collapse_par);
  } else {
    collapse(B, root, out, 0, 0, false, collapse_par);
  }
  if (out.nodes.size() >= (size_t)PT_INST_BIT) fail(PT_ERR_TOO_LARGE, "too many BVH nodes");
  if (out.leaf_order.size() >= ((size_t)1 << 28) - 8) fail(PT_ERR_TOO_LARGE, "too many leaf items");
  if (3 * out.max_depth + 2 > PT_STACK)
    fail(PT_ERR_TOO_LARGE, "BVH deeper than the traversal stack (" + std::to_string(out.max_depth) + ")");

  // leaf items and shading records
  std::vector<Item> items(out.leaf_order.size());
  std::vector<PrimShade> shade(n_prims);
  std::vector<int> prim_item(n_prims, -1);
  std::vector<int> prim_mesh(B.n_tris), prim_tri(B.n_tris);
  for (int m = 0; m < d->n_meshes; ++m)
    for (int t = 0; t < d->meshes[m].n_triangles; ++t) {
      prim_mesh[B.tri_base[m] + t] = m;
      prim_tri[B.tri_base[m] + t] = t;
    }
  parallel_for(out.leaf_order.size(), threads, [&](size_t k) {
    const int prim = out.leaf_order[k];
    Item &it = items[k];
    std::memset(&it, 0, sizeof it);
    it.a[3] = u2f((uint32_t)prim);
    // a moving primitive tested from the world frame moves itself; inside a
    // moving object's subtree the ray is already in the object's frame
    it.c[3] = u2f((uint32_t)(out.leaf_world[k] ? prim_motion[prim] : 0));
    prim_item[prim] = (int)k;
    if (prim < B.n_tris) {
      const pt_mesh_desc &m = d->meshes[prim_mesh[prim]];
      const int t = prim_tri[prim];
      const float *p0 = m.positions + 3 * m.indices[3 * t];
      const float *p1 = m.positions + 3 * m.indices[3 * t + 1];
      const float *p2 = m.positions + 3 * m.indices[3 * t + 2];
      for (int a = 0; a < 3; ++a) {
        it.a[a] = p0[a];
        it.b[a] = p1[a] - p0[a];  // e1 = p1 - p0 (meshBVH.cpp:91)
        it.c[a] = p2[a] - p0[a];  // e2 = p2 - p0 (meshBVH.cpp:92)
      }
      it.b[3] = u2f(ITEM_TRI);
    } else if (prim < B.n_tris + d->n_quads) {
      const pt_quad_desc &q = d->quads[prim - B.n_tris];
      it.a[0] = q.k;
      it.a[1] = q.d0_min;
      it.a[2] = q.d0_max;
      it.b[0] = q.d1_min;
      it.b[1] = q.d1_max;
      it.b[2] = (float)q.axis;
      it.b[3] = u2f(ITEM_QUAD);
    } else if (prim >= curve_base) {
      it.a[0] = u2f((uint32_t)(prim - curve_base));
      it.b[3] = u2f(ITEM_CURVE);
    } else {
      const pt_sphere_desc &s = d->spheres[prim - B.n_tris - d->n_quads];
      it.a[0] = s.center[0];
      it.a[1] = s.center[1];
      it.a[2] = s.center[2];
      it.b[0] = s.radius;
      it.b[3] = u2f(ITEM_SPHERE);
    }
  });
  parallel_for((size_t)n_prims, threads, [&](size_t pi) {
    const int prim = (int)pi;
    PrimShade &ps = shade[prim];
    std::memset(&ps, 0, sizeof ps);
    ps.item = prim_item[prim];
    ps.light = -1;
    ps.flags = (prim_motion[prim] << 8) | prim_face[prim];
    if (prim < B.n_tris) {
      const pt_mesh_desc &m = d->meshes[prim_mesh[prim]];
      const int t = prim_tri[prim];
      ps.material = m.material;
      ps.flags |= ITEM_TRI << 2;
      {
        const Item &it = items[prim_item[prim]];
        V3 e1 = v3(it.b[0], it.b[1], it.b[2]), e2 = v3(it.c[0], it.c[1], it.c[2]);
        V3 ng = cross(e1, e2);
        ps.ng[0] = ng.x;
        ps.ng[1] = ng.y;
        ps.ng[2] = ng.z;
      }
      if (m.normals && m.n_normals > 0) {
        const int32_t *ni = m.normal_indices ? m.normal_indices : m.indices;
        bool okn = true;
        for (int k = 0; k < 3; ++k) okn = okn && ni[3 * t + k] >= 0 && ni[3 * t + k] < m.n_normals;
        if (okn) {
          ps.flags |= PT_PRIM_SMOOTH;
          for (int a = 0; a < 3; ++a) {
            ps.n0[a] = m.normals[3 * ni[3 * t] + a];
            ps.n1[a] = m.normals[3 * ni[3 * t + 1] + a];
            ps.n2[a] = m.normals[3 * ni[3 * t + 2] + a];
          }
        }
      }
    } else if (prim < B.n_tris + d->n_quads) {
      const pt_quad_desc &q = d->quads[prim - B.n_tris];
      ps.material = q.material;
      ps.flags |= (ITEM_QUAD << 2) | (q.axis << 4);
      if (q.flip_face) ps.flags |= PT_PRIM_FLIP;
    } else if (prim >= curve_base) {
      ps.material = d->curves[prim - curve_base].material;
      ps.flags |= ITEM_CURVE << 2;
      ps.n0[0] = u2f((uint32_t)(prim - curve_base));
    } else {
      const pt_sphere_desc &s = d->spheres[prim - B.n_tris - d->n_quads];
      ps.material = s.material;
      ps.flags |= ITEM_SPHERE << 2;
      for (int a = 0; a < 3; ++a) ps.n0[a] = s.center[a];
      if (s.flip_face) ps.flags |= PT_PRIM_FLIP;
    }
  });

  // materials
  std::vector<MatRec> mats;
  for (int i = 0; i < d->n_materials; ++i) mats.push_back(derive_material(d->materials[i]));
  for (int prim = 0; prim < n_prims; ++prim) {
    const int t = mats[shade[prim].material].type;
    if (t < PT_MAT_DIFFUSE_EMITTER) S->family_mask |= 1u << t;
  }

  // textures (ColorVariant): the table, an image texel pool, and per
  // primitive texture-coordinate records when a material uses one
  const int n_tex = d->textures ? d->n_textures : 0;
  if (n_tex < 0) fail(PT_ERR_INVALID, "negative texture count");
  std::vector<TexRec> texs(n_tex);
  std::vector<float4> texel_pool;
  std::vector<size_t> texel_off(n_tex, 0);
  for (int k = 0; k < n_tex; ++k) {
    const pt_texture_desc &t = d->textures[k];
    TexRec &T = texs[k];
    std::memset(&T, 0, sizeof T);
    if (t.kind < PT_TEX_CONSTANT || t.kind > PT_TEX_IMAGE) fail(PT_ERR_INVALID, "bad texture kind");
    T.kind = t.kind;
    T.fractal = t.fractal;
    T.scale = t.scale;
    for (int c = 0; c < 3; ++c) {
      T.c1[c] = t.color1[c];
      T.c2[c] = t.color2[c];
    }
    if (t.kind == PT_TEX_IMAGE) {
      if (!t.texels || t.width < 2 || t.height < 2) fail(PT_ERR_INVALID, "image texture smaller than 2x2");
      T.width = t.width;
      T.height = t.height;
      texel_off[k] = texel_pool.size();
      for (size_t i = 0; i < (size_t)t.width * t.height; ++i)
        texel_pool.push_back(make_float4(t.texels[3 * i], t.texels[3 * i + 1], t.texels[3 * i + 2], 0.f));
    }
  }
  bool any_textured = false;
  for (const MatRec &m : mats) {
    const int ti = (int)((uint32_t)m.flags >> PT_MAT_TEXTURE_SHIFT);
    if (ti > n_tex) fail(PT_ERR_INVALID, "material texture index out of range");
    if (ti && (m.type == PT_MAT_LAMBERTIAN || m.type == PT_MAT_DIFFUSE_EMITTER)) any_textured = true;
  }
  std::vector<float4> prim_uv;
  if (any_textured) {
    prim_uv.assign(2 * (size_t)n_prims, make_float4(0.f, 0.f, 0.f, 0.f));
    for (int prim = 0; prim < n_prims; ++prim) {
      float4 &a = prim_uv[2 * prim], &b = prim_uv[2 * prim + 1];
      if (prim < B.n_tris) {
        const int mi = prim_mesh[prim], t = prim_tri[prim];
        const pt_mesh_desc &m = d->meshes[mi];
        if (m.uvs && m.n_uvs > 0) {
          // MeshBVHNode::hitTriangle's uv interpolation (meshBVH.cpp:134-138);
          // a face without valid uv indices keeps (0, 0)
          const int32_t *ui = m.uv_indices ? m.uv_indices : m.indices;
          bool ok = true;
          for (int k = 0; k < 3; ++k) ok = ok && ui[3 * t + k] >= 0 && ui[3 * t + k] < m.n_uvs;
          if (ok) {
            const float *u0 = m.uvs + 2 * ui[3 * t], *u1 = m.uvs + 2 * ui[3 * t + 1], *u2 = m.uvs + 2 * ui[3 * t + 2];
            a = make_float4(u0[0], u0[1], u1[0], u1[1]);
            b = make_float4(u2[0], u2[1], (float)PT_UV_TRI, 0.f);
          } else {
            b = make_float4(0.f, 0.f, (float)PT_UV_TRI, 0.f);
          }
        } else {
          // TriangleMesh::intersect's planar fallback over the mesh's box
          // (triangleMesh.cpp:39-51, box as triangleMesh.cpp:10-18)
          float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
          for (int v = 0; v < m.n_positions; ++v)
            for (int c = 0; c < 3; ++c) {
              mn[c] = std::min(mn[c], m.positions[3 * v + c]);
              mx[c] = std::max(mx[c], m.positions[3 * v + c]);
            }
          for (int c = 0; c < 3; ++c) {
            mn[c] -= 1e-3f;
            mx[c] += 1e-3f;
          }
          a = make_float4(mn[0], mn[1], mn[2], mx[0]);
          b = make_float4(mx[1], mx[2], (float)PT_UV_PLANAR, 0.f);
        }
      } else if (prim < B.n_tris + d->n_quads) {
        const pt_quad_desc &q = d->quads[prim - B.n_tris];
        a = make_float4(q.d0_min, q.d0_max, q.d1_min, q.d1_max);
        b = make_float4(0.f, 0.f, (float)PT_UV_QUAD, (float)q.axis);
      } else if (prim >= curve_base) {
        b = make_float4(0.f, 0.f, (float)PT_UV_TRI, 0.f);  // Curve sets no texCoords: (0, 0)
      } else {
        const pt_sphere_desc &sp = d->spheres[prim - B.n_tris - d->n_quads];
        a = make_float4(sp.center[0], sp.center[1], sp.center[2], sp.radius);
        b = make_float4(0.f, 0.f, (float)PT_UV_SPHERE, 0.f);
      }
    }
  }

  // light discovery (lightDiscovery.hpp:5-81): emissive quads and spheres in
  // object order, then the environment light (renderManager.hpp:115-118).
  std::vector<LightRec> lights;
  for (int o = 0; o < d->n_objects; ++o) {
    const pt_object_desc &od = d->objects[o];
    if (od.kind == PT_OBJ_MESH || od.kind == PT_OBJ_BOX || od.kind == PT_OBJ_CURVE) continue;  // not lights
    int mi = od.kind == PT_OBJ_QUAD ? d->quads[od.index].material : d->spheres[od.index].material;
    const pt_material_desc &md = d->materials[mi];
    if (md.type != PT_MAT_DIFFUSE_EMITTER || md.p[3] <= 0.f) continue;
    LightRec L;
    std::memset(&L, 0, sizeof L);
    L.intensity = md.p[3];
    for (int c = 0; c < 3; ++c) L.color[c] = md.p[c];
    if (od.kind == PT_OBJ_QUAD) {
      // QuadLight(AARectangle<axis>) vertices (light.hpp:71-108)
      const pt_quad_desc &q = d->quads[od.index];
      float v0[3], v1[3], v3_[3];
      auto put = [&](float *v, float a, float b) {
        if (q.axis == 0) { v[0] = q.k; v[1] = a; v[2] = b; }
        else if (q.axis == 1) { v[0] = a; v[1] = q.k; v[2] = b; }
        else { v[0] = a; v[1] = b; v[2] = q.k; }
      };
      float v2[3];
      put(v0, q.d0_min, q.d1_min);
      put(v1, q.d0_max, q.d1_min);
      put(v2, q.d0_max, q.d1_max);
      put(v3_, q.d0_min, q.d1_max);
      for (int a = 0; a < 3; ++a) L.v2[a] = v2[a];
      L.type = LIGHT_QUAD;
      L.prim = B.n_tris + od.index;
      V3 e1 = v3(v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]);
      V3 e2 = v3(v3_[0] - v0[0], v3_[1] - v0[1], v3_[2] - v0[2]);
      V3 c = cross(e1, e2);
      V3 nn = normalize(c);
      for (int a = 0; a < 3; ++a) L.v0[a] = v0[a];
      L.e1[0] = e1.x; L.e1[1] = e1.y; L.e1[2] = e1.z;
      L.e2[0] = e2.x; L.e2[1] = e2.y; L.e2[2] = e2.z;
      L.normal[0] = nn.x; L.normal[1] = nn.y; L.normal[2] = nn.z;
      L.area = length(c);
    } else {
      const pt_sphere_desc &s = d->spheres[od.index];
      L.type = LIGHT_SPHERE;
      L.prim = B.n_tris + d->n_quads + od.index;
      for (int a = 0; a < 3; ++a) L.v0[a] = s.center[a];
      L.radius = s.radius;
      L.area = (float)(4 * PT_PI * s.radius * s.radius);
    }
    L.motion = prim_motion[L.prim];
    L.texture = (int32_t)((uint32_t)md.flags >> PT_MAT_TEXTURE_SHIFT);
    shade[L.prim].light = (int)lights.size();
    lights.push_back(L);
  }

  // environment map + luminance alias table
  std::vector<float4> tex;
  std::vector<float> aprob, apdf;
  std::vector<int32_t> aidx;
  if (d->env) {
    const pt_env_desc &e = *d->env;
    if (!e.texels || e.width < 2 || e.height < 2) fail(PT_ERR_INVALID, "environment map smaller than 2x2");
    const int W = e.width, H = e.height, N = W * H;
    tex.resize(N);
    for (int i = 0; i < N; ++i) tex[i] = make_float4(e.texels[3 * i], e.texels[3 * i + 1], e.texels[3 * i + 2], 0.f);
    // cell (x, y) covers u in [x/W, (x+1)/W): weight = mean luminance of the
    // texels the bilinear lookup blends there, times sin(theta), plus a floor
    std::vector<double> w(N);
    double sum = 0.0;
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        double l = 0.0;
        for (int dy = 0; dy < 2; ++dy)
          for (int dx = 0; dx < 2; ++dx) {
            int xx = std::min(x + dx, W - 1), yy = std::min(y + dy, H - 1);
            const float4 &t = tex[yy * W + xx];
            l += 0.2126 * t.x + 0.7152 * t.y + 0.0722 * t.z;
          }
        double st = std::sin(PT_PI * (y + 0.5) / H);
        w[y * W + x] = std::max(0.0, l * 0.25) * st;
        sum += w[y * W + x];
      }
    double floor_w = (sum > 0 ? sum / N : 1.0) * 1e-3;
    sum = 0.0;
    for (int y = 0; y < H; ++y) {
      double st = std::sin(PT_PI * (y + 0.5) / H);
      for (int x = 0; x < W; ++x) {
        w[y * W + x] += floor_w * st;
        sum += w[y * W + x];
      }
    }
    apdf.resize(N);
    for (int i = 0; i < N; ++i) apdf[i] = (float)(w[i] / sum);
    // Vose's alias method
    aprob.assign(N, 1.f);
    aidx.resize(N);
    std::vector<double> sc(N);
    std::vector<int> small, large;
    for (int i = 0; i < N; ++i) {
      sc[i] = w[i] / sum * N;
      aidx[i] = i;
      (sc[i] < 1.0 ? small : large).push_back(i);
    }
    while (!small.empty() && !large.empty()) {
      int s = small.back(); small.pop_back();
      int l = large.back(); large.pop_back();
      aprob[s] = (float)sc[s];
      aidx[s] = l;
      sc[l] = (sc[l] + sc[s]) - 1.0;
      (sc[l] < 1.0 ? small : large).push_back(l);
    }
    LightRec L;
    std::memset(&L, 0, sizeof L);
    L.type = LIGHT_ENV;
    L.prim = -1;
    L.intensity = e.intensity;
    L.area = INFINITY;
    lights.push_back(L);
    S->env_w = W;
    S->env_h = H;
  }

  // content hash of the BVH (nodes and leaf items): equal hashes, equal trees
  if (want_hash)
    S->bvh_hash = fnv1a(items.data(), items.size() * sizeof(Item),
                        fnv1a(out.nodes.data(), out.nodes.size() * sizeof(Bvh4Node), 0xcbf29ce484222325ull));
  S->n_nodes = (int64_t)out.nodes.size();
  S->n_items = (int64_t)items.size();

  // upload
  auto up = [&](const auto &v) { return device ? dupload(v, S->owned, st) : nullptr; };
  {
    // the device copy carries each child's traversal reference in place of
    // its count (the node visit then needs neither the child row nor any
    // decoding); the host tree and its hash keep (child, count)
    std::vector<Bvh4Node> dev = out.nodes;
    for (Bvh4Node &N : dev)
      for (int k = 0; k < 4; ++k) {
        if (N.count[k] > 8) fail(PT_ERR_INVALID, "leaf of more than 8 items");
        N.count[k] = trav_ref(N.child[k], N.count[k]);
      }
    S->nodes = up(dev);
  }
  S->items = up(items);
  S->shade = up(shade);
  S->materials = up(mats);
  S->lights = up(lights);
  SceneView &V = S->view;
  std::memset(&V, 0, sizeof V);
  V.nodes = S->nodes;
  V.items = S->items;
  V.shade = S->shade;
  V.materials = S->materials;
  V.lights = S->lights;
  V.n_lights = (int)lights.size();
  S->host_lights = lights;
  V.n_nodes = (int)out.nodes.size();
  V.n_prims = n_prims;
  V.trav_cap = trav_cap > 0 ? trav_cap : PT_TRAVERSAL_CAP;
  // a node visit pushes at most 3 entries per level, plus a moving object's
  // frame marker; 2 entries to spare
  V.stack_entries = std::min(PT_STACK, 3 * out.max_depth + 4);
  for (int c = 0; c < 3; ++c) V.bg[c] = d->bg_color[c];
  if (d->env) {
    V.env.texels = up(tex);
    V.env.alias_prob = up(aprob);
    V.env.alias_idx = up(aidx);
    V.env.pdf = up(apdf);
    V.env.width = d->env->width;
    V.env.height = d->env->height;
    V.env.intensity = d->env->intensity;
    V.env.present = 1;
  }
  if (!texs.empty()) {
    const float4 *pool = up(texel_pool);
    for (int k = 0; k < n_tex; ++k)
      if (texs[k].kind == PT_TEX_IMAGE) texs[k].texels = pool ? pool + texel_off[k] : nullptr;
    V.textures = up(texs);
    V.n_textures = n_tex;
  }
  if (!prim_uv.empty()) V.prim_uv = up(prim_uv);
  if (n_curves > 0) {
    std::vector<float4> cv(4 * (size_t)n_curves);
    for (int c = 0; c < n_curves; ++c) {
      const pt_curve_desc &k = d->curves[c];
      for (int j = 0; j < 4; ++j)
        cv[4 * c + j] = make_float4(k.cps[j][0], k.cps[j][1], k.cps[j][2],
                                    j == 0 ? k.width0 : j == 1 ? k.width1 : 0.f);
    }
    V.curves = up(cv);
  }
  if (!motion.empty()) {
    V.motion = up(motion);
    V.node_motion = up(out.node_motion);
    V.has_motion = 1;
    S->shutter_max = d->shutter_max;
  }
  if (d->medium) {
    V.has_medium = 1;
    float tmax = 0.f;
    for (int c = 0; c < 3; ++c) {
      V.sigma_a[c] = d->medium->sigma_a[c];
      V.sigma_s[c] = d->medium->sigma_s[c];
      tmax = std::max(tmax, V.sigma_a[c] + V.sigma_s[c]);
    }
    V.sigma_t_max = tmax;
    V.medium_g = d->medium->g;
  }
  S->n_tris = B.n_tris;
  S->n_quads = d->n_quads;
  S->n_spheres = d->n_spheres;
  S->bvh_depth = out.max_depth;
  size_t bytes = 0;
  bytes += out.nodes.size() * sizeof(Bvh4Node) + items.size() * sizeof(Item) + shade.size() * sizeof(PrimShade);
  bytes += mats.size() * sizeof(MatRec) + lights.size() * sizeof(LightRec);
  bytes += tex.size() * sizeof(float4) + aprob.size() * 12;
  S->device_bytes = bytes;
  if (device) cuda_check(cudaStreamSynchronize(st), "scene upload");
  return S;
}

Scene::~Scene() {
  for (void *p : owned) cudaFree(p);
}

// -------------------------------------------------------------- context
Context::Context(int dev) : device(dev) {
  cuda_check(cudaSetDevice(dev), "cudaSetDevice");
  cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
  side1.create();
  cudaDeviceProp prop;
  cuda_check(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
  num_sms = prop.multiProcessorCount;
  halton = make_halton_tables();
  upload_halton_tables(halton, stream);
  upload_halton_tables_multi(halton, stream);
  upload_halton_tables_persist(halton, stream);
  kernel_attributes(&kinfo);
  cfg.trace_blocks = num_sms * std::max(1, kinfo.trace_blocks_per_sm);
  cfg.shade_blocks = num_sms * std::max(1, kinfo.shade_blocks_per_sm);
  for (int f = 0; f < PT_FAM_MISC + 2; ++f)
    cfg.shade_fam_blocks[f] = num_sms * std::max(1, kinfo.shade_fam_blocks_per_sm[f]);
  cfg.max_blocks_simple = num_sms * 8;
  cfg.sort_by_material = 1;
  cfg.family_mask = 0x7f;
  const char *cap = std::getenv("PT_WAVE_PATHS");
  wave_cap = cap ? std::max(1024, std::atoi(cap)) : (1 << 24);
  if (cap) batch_wave_cap = wave_cap;  // batched waves of the same size (tests of many-wave renders)
  // bound on one ray's traversal steps (scenes uploaded by this context);
  // exceeding it sets the device error flag, reported as PT_ERR_DEVICE
  const char *tc = std::getenv("PT_TRAVERSAL_CAP");
  trav_cap = tc ? std::max(1, std::atoi(tc)) : 0;
  const char *srt = std::getenv("PT_SORT_BY_MATERIAL");
  if (srt) cfg.sort_by_material = std::atoi(srt);
  // paired tracing pays where a bounce's two sparse tails dominate (1 M-path
  // waves: +12 %) and costs 3 % on 16.8 M-path waves (a larger kernel)
  cfg.pair_trace = 1 << 21;
  const char *pair = std::getenv("PT_PAIR_TRACE");
  if (pair) cfg.pair_trace = std::max(0, std::atoi(pair));
  cfg.pair_from_bounce = 0;
  const char *pfb = std::getenv("PT_PAIR_FROM_BOUNCE");
  if (pfb) cfg.pair_from_bounce = std::max(0, std::atoi(pfb));
  cuda_check(cudaMalloc(&d_err, sizeof(int)), "cudaMalloc(err)");
  cuda_check(cudaMemsetAsync(d_err, 0, sizeof(int), stream), "memset err");
  cuda_check(cudaStreamSynchronize(stream), "context init");
}

Context::~Context() {
  cudaSetDevice(device);
  free_queues();
  for (void *p : qmem2) cudaFree(p);
  if (stream2) cudaStreamDestroy(stream2);
  side1.destroy();
  side2.destroy();
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  for (cudaEvent_t e : film_ev) cudaEventDestroy(e);
  for (auto &kv : perms) cudaFree(kv.second);
  if (d_film) cudaFree(d_film);
  if (d_offsets) cudaFree(d_offsets);
  if (d_scratch) cudaFree(d_scratch);
  if (d_err) cudaFree(d_err);
  for (cudaEvent_t e : prof.pool) cudaEventDestroy(e);
  if (stream) cudaStreamDestroy(stream);
}

void Context::free_queues() {
  for (void *p : qmem) cudaFree(p);
  qmem.clear();
  q_cap = 0;
  q_ln = 0;
}

// Work queues for `cap` paths per wave and `ln` light samples per vertex.
static void alloc_queues(Queues &Q, std::vector<void *> &mem, int cap, int ln, int *d_err) {
  for (void *p : mem) cudaFree(p);
  mem.clear();
  auto alloc = [&](size_t bytes) {
    void *p = nullptr;
    cuda_check(cudaMalloc(&p, bytes), "cudaMalloc(queues)");
    mem.push_back(p);
    return p;
  };
  const size_t c = (size_t)cap;
  Q.cap = cap;
  Q.beta = (float4 *)alloc(c * 16);
  Q.L = (float4 *)alloc(c * 16);
  Q.ray_o[0] = (float4 *)alloc(c * 16);
  Q.ray_o[1] = (float4 *)alloc(c * 16);
  Q.ray_d[0] = (float4 *)alloc(c * 16);
  Q.ray_d[1] = (float4 *)alloc(c * 16);
  Q.hit = (float4 *)alloc(c * 16);
  Q.sh_o = (float4 *)alloc(c * 16);
  Q.sh_d = (float4 *)alloc(c * 16 * ln);
  Q.sh_c = (float4 *)alloc(c * 16 * ln);
  Q.sh_vis = (uint8_t *)alloc(c * ln);
  Q.counts = (int *)alloc(64);
  Q.stats = (unsigned long long *)alloc(64);
  Q.sort_key = (int *)alloc(c * 4);
  Q.order = (int *)alloc(c * 4);
  Q.bins = (int *)alloc(sizeof(int) * 2 * PT_SORT_BINS);
  Q.seg = (int *)alloc(sizeof(int) * (PT_SORT_BINS + 1));
  Q.job = (int *)alloc(c * 4);
  Q.err = d_err;
}

void Context::ensure_queues(int cap, int ln) {
  if (cap <= q_cap && ln <= q_ln) return;
  free_queues();
  alloc_queues(Q, qmem, cap, ln, d_err);
  q_cap = cap;
  q_ln = ln;
}

void Context::ensure_queues2(int cap, int ln) {
  if (!stream2) cuda_check(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking), "cudaStreamCreate");
  side2.create();
  if (!ev_fork) cuda_check(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming), "cudaEventCreate");
  if (!ev_join) cuda_check(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming), "cudaEventCreate");
  if (cap <= q2_cap && ln <= q2_ln) return;
  alloc_queues(Q2, qmem2, cap, ln, d_err);
  q2_cap = cap;
  q2_ln = ln;
}

const uint16_t *Context::perm_for(uint32_t seed) {
  auto it = perms.find(seed);
  if (it != perms.end()) return it->second;
  std::vector<uint16_t> p = make_digit_permutations(halton, seed);
  uint16_t *dp = nullptr;
  cuda_check(cudaMalloc(&dp, p.size() * 2), "cudaMalloc(perm)");
  cuda_check(cudaMemcpyAsync(dp, p.data(), p.size() * 2, cudaMemcpyHostToDevice, stream), "upload perm");
  cuda_check(cudaStreamSynchronize(stream), "upload perm");
  perms[seed] = dp;
  return dp;
}

Scene *Context::scene(int id) {
  auto it = scenes.find(id);
  if (it == scenes.end()) fail(PT_ERR_NOT_FOUND, "unknown scene id " + std::to_string(id));
  return it->second.get();
}

// PerspectiveCamera constructor (camera.cpp:7-35).
CameraView make_camera(const pt_camera_desc &c) {
  CameraView C;
  const float m = 1.0f;
  float theta = c.fov / 2.f;
  float h = std::tan(theta);
  float ph = m * h * 2.0f;
  float pw = ph * c.aspect;
  V3 up = v3(c.up[0], c.up[1], c.up[2]), front = v3(c.front[0], c.front[1], c.front[2]);
  V3 pos = v3(c.position[0], c.position[1], c.position[2]);
  V3 lookat = -normalize(front);
  V3 hv = normalize(cross(up, lookat));
  V3 vv = normalize(cross(lookat, hv));
  V3 hor = hv * pw * c.focal_dist;
  V3 ver = vv * ph * c.focal_dist;
  V3 bl = pos - hor / 2.0f - ver / 2.0f;
  bl = bl - lookat * c.focal_dist;
  auto put = [](float *d, V3 v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; };
  put(C.position, pos);
  put(C.bottom_left, bl);
  put(C.horizontal, hor);
  put(C.vertical, ver);
  put(C.h_vec, hv);
  put(C.v_vec, vv);
  C.lens_radius = c.focal_dist / c.aperture * 0.5f;
  return C;
}

// FrameBuffer::setOffsets (framebuffer.cpp:131-145): one jittered spp_x by
// spp_y grid per frame, shared by every pixel, i outer.
std::vector<float2> make_offsets(const pt_job_desc &j) {
  std::vector<float2> off;
  const uint64_t key = path_key(j.seed ^ 0x5bd1e995u, 0xffffffffffull);
  for (int i = 0; i < j.spp_x; ++i)
    for (int k = 0; k < j.spp_y; ++k) {
      const uint32_t s = (uint32_t)(i * j.spp_y + k);
      float a = (float)i / (float)j.spp_x, b = (float)(i + 1) / (float)j.spp_x;
      float c = (float)k / (float)j.spp_y, d = (float)(k + 1) / (float)j.spp_y;
      off.push_back(make_float2(a + (b - a) * rand01(key, 2 * s), c + (d - c) * rand01(key, 2 * s + 1)));
    }
  return off;
}

void validate_job(const pt_job_desc &j) {
  if (j.width <= 0 || j.height <= 0 || j.spp_x <= 0 || j.spp_y <= 0)
    fail(PT_ERR_INVALID, "job size must be positive");
  if (j.max_depth < 0) fail(PT_ERR_INVALID, "max_depth must be >= 0");
  if (j.light_samples_x <= 0 || j.light_samples_y <= 0 ||
      j.light_samples_x * j.light_samples_y > PT_MAX_LIGHT_SAMPLES)
    fail(PT_ERR_INVALID, "light samples must be in [1, 16]");
  const int spp = j.spp_x * j.spp_y;
  const int e = j.spp_end ? j.spp_end : spp;
  if (j.spp_begin < 0 || e > spp || j.spp_begin >= e) fail(PT_ERR_INVALID, "bad sample range");
  if (j.estimator < 0 || j.estimator > 1 || j.sampler < 0 || j.sampler > 3 || j.env_sampling < 0 ||
      j.env_sampling > 1)
    fail(PT_ERR_INVALID, "bad enum in job");
  if (j.camera.aperture == 0.f) fail(PT_ERR_INVALID, "camera aperture must be non-zero");
  if (!(j.camera.shutter >= 0.f) || !std::isfinite(j.camera.shutter))
    fail(PT_ERR_INVALID, "camera shutter must be finite and >= 0");
  if (j.full_width > 0 || j.full_height > 0) {
    if (j.crop_x < 0 || j.crop_y < 0 || (int64_t)j.crop_x + j.width > j.full_width ||
        (int64_t)j.crop_y + j.height > j.full_height)
      fail(PT_ERR_INVALID, "window outside the frame");
  } else if (j.crop_x != 0 || j.crop_y != 0) {
    fail(PT_ERR_INVALID, "window origin without a frame size");
  }
}

void set_window(JobView &v, const pt_job_desc &j) {
  v.width = j.width;
  v.height = j.height;
  const bool win = j.full_width > 0 || j.full_height > 0;
  v.crop_x = win ? j.crop_x : 0;
  v.crop_y = win ? j.crop_y : 0;
  v.full_w = win ? j.full_width : j.width;
  v.full_h = win ? j.full_height : j.height;
}

DeviceJob Context::device_job(const pt_job_desc &j, Scene *S) {
  DeviceJob J;
  std::memset(&J, 0, sizeof J);
  set_window(J.job, j);
  J.job.spp_x = j.spp_x;
  J.job.spp_y = j.spp_y;
  J.job.spp = j.spp_x * j.spp_y;
  J.job.spp_begin = j.spp_begin;
  J.job.max_depth = j.max_depth;
  J.job.rr_start = j.rr_start;
  J.job.estimator = j.estimator;
  J.job.sampler = j.sampler;
  J.job.env_sampling = (S->view.env.present ? j.env_sampling : PT_ENV_UNIFORM);
  J.job.light_nx = j.light_samples_x;
  J.job.light_ny = j.light_samples_y;
  J.job.seed = j.seed;
  J.job.shutter = j.camera.shutter;
  J.job.cam = make_camera(j.camera);
  J.perm = j.sampler == PT_SAMPLER_HALTON_PERMUTE ? perm_for(j.sampler_seed) : nullptr;
  if (S->view.has_motion && j.camera.shutter > S->shutter_max)
    fail(PT_ERR_INVALID, "camera shutter longer than the scene's shutter_max");
  return J;
}

void Context::render_device(const pt_job_desc &j, float *d_film, pt_stats *stats, bool sync, const float *d_rays) {
  validate_job(j);
  Scene *S = scene(j.scene);
  DeviceJob J = device_job(j, S);
  J.job.rays = d_rays;
  // offsets table
  std::vector<float2> off = make_offsets(j);
  if ((int)off.size() > offsets_cap) {
    if (d_offsets) cudaFree(d_offsets);
    cuda_check(cudaMalloc(&d_offsets, off.size() * sizeof(float2)), "cudaMalloc(offsets)");
    offsets_cap = (int)off.size();
  }
  cuda_check(cudaMemcpyAsync(d_offsets, off.data(), off.size() * sizeof(float2), cudaMemcpyHostToDevice, stream),
             "upload offsets");
  J.job.offsets = d_offsets;
  const long long npix = (long long)j.width * j.height;
  const int e = j.spp_end ? j.spp_end : j.spp_x * j.spp_y;
  const long long total = npix * (e - j.spp_begin);
  int n = wave_cap;
  if (npix <= wave_cap) n = (int)((wave_cap / npix) * npix);
  if ((long long)n > total) n = (int)total;
  const int LN = j.light_samples_x * j.light_samples_y;
  ensure_queues(n, LN);
  cuda_check(cudaMemsetAsync(Q.stats, 0, 64, stream), "memset stats");
  auto t0 = std::chrono::steady_clock::now();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, stream);
  LaunchCfg lc = cfg;
  lc.family_mask = S->family_mask;
  const long long waves = (total + n - 1) / n;
  if (waves == 1) {
    launch_wave(S->view, J, Q, 0, (int)total, d_film, lc, stream, &prof, nullptr, nullptr, &side1);
  } else {
    // consecutive waves alternate between two queue sets on two streams so
    // that one wave's sparse last bounces overlap the next wave's first ones;
    // the film stages stay in wave order (event chain)
    ensure_queues2(n, LN);
    while ((long long)film_ev.size() < waves) {
      cudaEvent_t ev;
      cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
      film_ev.push_back(ev);
    }
    cuda_check(cudaMemsetAsync(Q2.stats, 0, 64, stream), "memset stats");
    cudaEventRecord(ev_fork, stream);
    cudaStreamWaitEvent(stream2, ev_fork, 0);
    int w = 0;
    for (long long g0 = 0; g0 < total; g0 += n, ++w) {
      const int cnt = (int)std::min<long long>(n, total - g0);
      const bool odd = (w & 1) != 0;
      launch_wave(S->view, J, odd ? Q2 : Q, g0, cnt, d_film, lc, odd ? stream2 : stream, &prof,
                  w > 0 ? film_ev[w - 1] : nullptr, film_ev[w], odd ? &side2 : &side1);
    }
    cudaEventRecord(ev_join, stream2);
    cudaStreamWaitEvent(stream, ev_join, 0);
  }
  cudaEventRecord(e1, stream);
  cuda_check(cudaGetLastError(), "launch");
  if (sync || stats) {
    cuda_check(cudaStreamSynchronize(stream), "render");
    int herr = 0;
    cuda_check(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost), "read err");
    if (herr) {
      cudaMemset(d_err, 0, sizeof(int));
      fail(PT_ERR_DEVICE, "device traversal error flag " + std::to_string(herr));
    }
  }
  if (stats) {
    unsigned long long h[4];
    cuda_check(cudaMemcpy(h, Q.stats, sizeof h, cudaMemcpyDeviceToHost), "read stats");
    if (waves > 1) {
      unsigned long long h2[4];
      cuda_check(cudaMemcpy(h2, Q2.stats, sizeof h2, cudaMemcpyDeviceToHost), "read stats");
      for (int k = 0; k < 4; ++k) h[k] += h2[k];
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    stats->paths = h[0];
    stats->segments = h[1];
    stats->rays = h[2];
    stats->shadow_rays = h[3];
    stats->ms = ms;
    stats->algorithmic_bytes = 192ull * h[1] + 88ull * h[3] + 24ull * h[0];
  }
  (void)t0;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
}

float *Context::film_buffer(size_t floats) {
  if (floats > film_cap) {
    if (d_film) cudaFree(d_film);
    d_film = nullptr;
    cuda_check(cudaMalloc(&d_film, floats * sizeof(float)), "cudaMalloc(film)");
    film_cap = floats;
  }
  return d_film;
}

void *Context::scratch(size_t bytes) {
  if (bytes > scratch_cap) {
    if (d_scratch) cudaFree(d_scratch);
    d_scratch = nullptr;
    cuda_check(cudaMalloc(&d_scratch, bytes), "cudaMalloc(scratch)");
    scratch_cap = bytes;
  }
  return d_scratch;
}

}  // namespace pt

// ================================================================ C-ABI
using namespace pt;

static int set_error(Context *c, int code, const std::string &msg) {
  if (c) c->last_error = msg;
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error = msg;
  return code;
}

namespace pt {
int record_error(int code, const std::string &msg) { return set_error(nullptr, code, msg); }
}  // namespace pt

#define PT_GUARD(ctxptr, body)                                   \
  try {                                                          \
    body;                                                        \
    return PT_OK;                                                \
  } catch (const PtError &e) {                                   \
    return set_error(ctxptr, e.code, e.what());                  \
  } catch (const std::bad_alloc &) {                             \
    return set_error(ctxptr, PT_ERR_NOMEM, "host out of memory"); \
  } catch (const std::exception &e) {                            \
    return set_error(ctxptr, PT_ERR_INVALID, e.what());          \
  } catch (...) {                                                \
    return set_error(ctxptr, PT_ERR_INVALID, "unknown error");   \
  }

static Context *as_ctx(void *p) {
  if (!p) fail(PT_ERR_INVALID, "null context");
  return static_cast<Context *>(p);
}

extern "C" {

int pt_version(void) { return 1; }

int pt_create(void **ctx, int device) {
  PT_GUARD(nullptr, {
    if (!ctx) fail(PT_ERR_INVALID, "null output pointer");
    *ctx = new Context(device);
  });
}

int pt_destroy(void *ctx) {
  PT_GUARD(nullptr, { delete static_cast<Context *>(ctx); });
}

int pt_last_error(void *ctx, char *buf, size_t n) {
  if (!buf || n == 0) return PT_ERR_INVALID;
  std::string m;
  if (ctx) {
    m = static_cast<Context *>(ctx)->last_error;
  } else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    m = g_last_error;
  }
  std::snprintf(buf, n, "%s", m.c_str());
  return PT_OK;
}

int pt_profile_begin(void *ctx) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    cuda_check(cudaStreamSynchronize(c->stream), "sync");
    c->prof.used = 0;
    c->prof.kinds.clear();
    c->prof.on = true;
  });
}

int pt_profile_end(void *ctx, double *stage_ms, int64_t *stage_launches) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    cuda_check(cudaStreamSynchronize(c->stream), "sync");
    for (int k = 0; k < STAGE_COUNT; ++k) {
      if (stage_ms) stage_ms[k] = 0.0;
      if (stage_launches) stage_launches[k] = 0;
    }
    for (size_t i = 0; i < c->prof.kinds.size(); ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c->prof.pool[2 * i], c->prof.pool[2 * i + 1]);
      const int k = c->prof.kinds[i];
      if (stage_ms) stage_ms[k] += ms;
    }
    for (int k = 0; k < STAGE_COUNT; ++k) {
      if (stage_launches) stage_launches[k] = c->prof.kernels[k];
      c->prof.kernels[k] = 0;
    }
    c->prof.on = false;
    c->prof.used = 0;
    c->prof.kinds.clear();
  });
}

int pt_scene_upload(void *ctx, const pt_scene_desc *desc, int32_t *scene_id) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (!scene_id) fail(PT_ERR_INVALID, "null scene_id");
    cuda_check(cudaSetDevice(c->device), "cudaSetDevice");
    auto S = build_scene(desc, c->stream, true, 0, c->trav_cap, c->bvh_builder);
    int id = c->next_scene++;
    c->scenes[id] = std::move(S);
    *scene_id = id;
  });
}

int pt_scene_release(void *ctx, int32_t scene_id) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    cuda_check(cudaStreamSynchronize(c->stream), "sync");
    if (!c->scenes.erase(scene_id)) fail(PT_ERR_NOT_FOUND, "unknown scene id");
  });
}

int pt_scene_info(void *ctx, int32_t scene_id, int64_t *out6) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    Scene *S = c->scene(scene_id);
    out6[0] = S->n_tris;
    out6[1] = S->n_quads;
    out6[2] = S->n_spheres;
    out6[3] = S->view.n_nodes;
    out6[4] = S->view.n_lights;
    out6[5] = (int64_t)S->device_bytes;
  });
}

int pt_bvh_build(const pt_scene_desc *desc, int32_t threads, int64_t *out5) {
  PT_GUARD(nullptr, {
    if (!out5) fail(PT_ERR_INVALID, "null output");
    auto t0 = std::chrono::steady_clock::now();
    auto S = build_scene(desc, nullptr, false, threads, 0, PT_BVH_BUILD_HOST, true);
    auto t1 = std::chrono::steady_clock::now();
    out5[0] = S->n_nodes;
    out5[1] = S->n_items;
    out5[2] = S->bvh_depth;
    uint64_t h = S->bvh_hash;
    std::memcpy(&out5[3], &h, sizeof h);
    out5[4] = (int64_t)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
  });
}

int pt_bvh_build_sah(const pt_scene_desc *desc, int32_t threads, int64_t *out5) {
  PT_GUARD(nullptr, {
    if (!out5) fail(PT_ERR_INVALID, "null output");
    auto t0 = std::chrono::steady_clock::now();
    auto S = build_scene(desc, nullptr, false, threads, 0, PT_BVH_BUILD_SAH, true);
    auto t1 = std::chrono::steady_clock::now();
    out5[0] = S->n_nodes;
    out5[1] = S->n_items;
    out5[2] = S->bvh_depth;
    uint64_t h = S->bvh_hash;
    std::memcpy(&out5[3], &h, sizeof h);
    out5[4] = (int64_t)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
  });
}

int pt_set_bvh_builder(void *ctx, int32_t builder) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (builder != PT_BVH_BUILD_HOST && builder != PT_BVH_BUILD_DEVICE && builder != PT_BVH_BUILD_SAH)
      fail(PT_ERR_INVALID, "unknown BVH builder");
    c->bvh_builder = builder;
  });
}

int pt_bvh_build_device(void *ctx, const pt_scene_desc *desc, int64_t *out5) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (!out5) fail(PT_ERR_INVALID, "null output");
    cuda_check(cudaSetDevice(c->device), "cudaSetDevice");
    auto t0 = std::chrono::steady_clock::now();
    auto S = build_scene(desc, c->stream, false, 0, 0, PT_BVH_BUILD_DEVICE, true);
    auto t1 = std::chrono::steady_clock::now();
    out5[0] = S->n_nodes;
    out5[1] = S->n_items;
    out5[2] = S->bvh_depth;
    uint64_t h = S->bvh_hash;
    std::memcpy(&out5[3], &h, sizeof h);
    out5[4] = (int64_t)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
  });
}

int pt_render_device(void *ctx, const pt_job_desc *job, float *d_film_sum, int sync, pt_stats *stats) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (!job || !d_film_sum) fail(PT_ERR_INVALID, "null job or film");
    cuda_check(cudaSetDevice(c->device), "cudaSetDevice");
    c->render_device(*job, d_film_sum, stats, sync != 0);
  });
}

int pt_render(void *ctx, const pt_job_desc *job, float *film_rgb, pt_stats *stats) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (!job || !film_rgb) fail(PT_ERR_INVALID, "null job or film");
    validate_job(*job);
    cuda_check(cudaSetDevice(c->device), "cudaSetDevice");
    const size_t nf = (size_t)job->width * job->height * 3;
    float *df = c->film_buffer(nf);
    cuda_check(cudaMemsetAsync(df, 0, nf * sizeof(float), c->stream), "memset film");
    c->render_device(*job, df, stats, false);
    cuda_check(cudaMemcpyAsync(film_rgb, df, nf * sizeof(float), cudaMemcpyDeviceToHost, c->stream), "film d2h");
    cuda_check(cudaStreamSynchronize(c->stream), "render");
    int herr = 0;
    cuda_check(cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost), "read err");
    if (herr) {
      cudaMemset(c->d_err, 0, sizeof(int));
      fail(PT_ERR_DEVICE, "device traversal error flag " + std::to_string(herr));
    }
    const int e = job->spp_end ? job->spp_end : job->spp_x * job->spp_y;
    const float inv = 1.f / (float)(e - job->spp_begin);
    for (size_t i = 0; i < nf; ++i) film_rgb[i] *= inv;
  });
}

// pt_ray_color's job: one film pixel per ray, one sample -- path i is frame
// pixel (first_index - 1 + i, 0) of a one-row frame at 1 spp, i.e. Halton
// index first_index + i, and its film pixel receives its radiance.  The
// camera is not used (the rays are given) beyond its shutter.
static pt_job_desc ray_color_job(const pt_job_desc &job, int32_t n, uint32_t first_index) {
  pt_job_desc j = job;
  const float shutter = job.camera.shutter;
  j.camera = pt_camera_desc{1.f, 1.f, 1.f, 1e3f, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}, {0.f, 0.f, 0.f}, shutter};
  j.width = n;
  j.height = 1;
  j.spp_x = j.spp_y = 1;
  j.spp_begin = 0;
  j.spp_end = 0;
  j.crop_x = (int32_t)(first_index - 1u);
  j.crop_y = 0;
  j.full_width = (int32_t)((int64_t)first_index - 1 + n);
  j.full_height = 1;
  return j;
}

int pt_ray_color(void *ctx, const pt_job_desc *job, const float *rays, int32_t n, uint32_t first_index,
                 float *radiance) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (!job || n < 0 || (n > 0 && (!rays || !radiance)) || first_index < 1)
      fail(PT_ERR_INVALID, "bad ray-color args");
    if (n == 0) return PT_OK;
    cuda_check(cudaSetDevice(c->device), "cudaSetDevice");
    if ((int64_t)first_index - 1 + n > INT32_MAX) fail(PT_ERR_INVALID, "first_index + n beyond 2^31");
    const pt_job_desc j = ray_color_job(*job, n, first_index);
    const size_t nn = (size_t)n;
    float *df = c->film_buffer(nn * 3);
    float *dr = (float *)c->scratch(nn * 24);
    cuda_check(cudaMemcpyAsync(dr, rays, nn * 24, cudaMemcpyHostToDevice, c->stream), "h2d rays");
    cuda_check(cudaMemsetAsync(df, 0, nn * 12, c->stream), "memset film");
    c->render_device(j, df, nullptr, false, dr);
    cuda_check(cudaMemcpyAsync(radiance, df, nn * 12, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaStreamSynchronize(c->stream), "ray color");
    int herr = 0;
    cuda_check(cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost), "read err");
    if (herr) {
      cudaMemset(c->d_err, 0, sizeof(int));
      fail(PT_ERR_DEVICE, "device traversal error flag " + std::to_string(herr));
    }
  });
}

int pt_tonemap(void *ctx, const float *film_rgb, int32_t width, int32_t height, float gamma, uint8_t *rgb8) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (!film_rgb || !rgb8 || width <= 0 || height <= 0 || gamma <= 0.f) fail(PT_ERR_INVALID, "bad tonemap args");
    const size_t nf = (size_t)width * height * 3;
    char *buf = (char *)c->scratch(nf * 5);
    float *df = (float *)buf;
    uint8_t *d8 = (uint8_t *)(buf + nf * 4);
    cuda_check(cudaMemcpyAsync(df, film_rgb, nf * 4, cudaMemcpyHostToDevice, c->stream), "h2d");
    launch_tonemap(df, width, height, gamma, d8, c->stream);
    cuda_check(cudaMemcpyAsync(rgb8, d8, nf, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaStreamSynchronize(c->stream), "tonemap");
  });
}

int pt_gaussian_blur(void *ctx, const float *film_in, float *film_out, int32_t width, int32_t height, int32_t kernel,
                     float sigma) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (!film_in || !film_out || width <= 0 || height <= 0) fail(PT_ERR_INVALID, "bad blur args");
    const size_t nf = (size_t)width * height * 3;
    std::vector<float> w = gaussian_weights(kernel, sigma);
    if (w.empty()) {
      // FrameBuffer::gaussianBlur returns without blurring (framebuffer.cpp:62-67)
      if (film_out != film_in) std::memcpy(film_out, film_in, nf * sizeof(float));
      return PT_OK;
    }
    char *buf = (char *)c->scratch(nf * 8 + w.size() * 4);
    float *din = (float *)buf;
    float *dout = din + nf;
    float *dw = dout + nf;
    cuda_check(cudaMemcpyAsync(din, film_in, nf * 4, cudaMemcpyHostToDevice, c->stream), "h2d");
    cuda_check(cudaMemcpyAsync(dw, w.data(), w.size() * 4, cudaMemcpyHostToDevice, c->stream), "h2d");
    launch_gaussian_blur(din, dout, width, height, kernel, dw, c->stream);
    cuda_check(cudaMemcpyAsync(film_out, dout, nf * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaStreamSynchronize(c->stream), "blur");
  });
}

int pt_write_png(const char *path, const uint8_t *rgb8, int32_t width, int32_t height) {
  PT_GUARD(nullptr, {
    if (!path || !rgb8 || width <= 0 || height <= 0) fail(PT_ERR_INVALID, "bad png args");
    write_png(path, rgb8, width, height);
  });
}

int pt_sampler_eval(void *ctx, int32_t strategy, uint32_t seed, uint32_t first_index, int32_t n, int32_t dims,
                    float *out) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (n < 0 || dims <= 0 || !out || strategy < 0 || strategy > 2) fail(PT_ERR_INVALID, "bad sampler args");
    if (n == 0) return PT_OK;
    const size_t bytes = (size_t)n * dims * sizeof(float);
    float *d = (float *)c->scratch(bytes);
    const uint16_t *perm = strategy == PT_SAMPLER_HALTON_PERMUTE ? c->perm_for(seed) : nullptr;
    launch_sampler_eval(strategy, perm, first_index, n, dims, d, c->stream);
    cuda_check(cudaGetLastError(), "sampler launch");
    cuda_check(cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaStreamSynchronize(c->stream), "sampler");
  });
}

int pt_sample_eval(void *ctx, const pt_job_desc *job, int64_t first_path, int32_t n, int32_t dims, int32_t bounces,
                   float *pixel_offsets, float *dim_values, float *light_offsets) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (!job || n < 0 || dims < 0 || bounces < 0 || (dims > 0 && !dim_values) ||
        (bounces > 0 && !light_offsets))
      fail(PT_ERR_INVALID, "bad sample-eval args");
    validate_job(*job);
    const long long npix = (long long)job->width * job->height;
    const int e = job->spp_end ? job->spp_end : job->spp_x * job->spp_y;
    if (first_path < 0 || first_path + n > npix * (e - job->spp_begin))
      fail(PT_ERR_INVALID, "paths outside the job's sample range");
    if (n == 0) return PT_OK;
    Scene *S = c->scene(job->scene);
    DeviceJob J = c->device_job(*job, S);
    const std::vector<float2> off = make_offsets(*job);
    const int LN = job->light_samples_x * job->light_samples_y;
    const size_t nn = (size_t)n;
    // byte sizes of the offsets table and the three outputs, 256-byte aligned
    const size_t b_off = (off.size() * sizeof(float2) + 255) / 256 * 256;
    const size_t b_pix = (nn * 8 + 255) / 256 * 256;
    const size_t b_dim = (nn * dims * 4 + 255) / 256 * 256;
    const size_t b_lo = (nn * bounces * LN * 8 + 255) / 256 * 256;
    char *buf = (char *)c->scratch(b_off + b_pix + b_dim + b_lo);
    float2 *d_off = (float2 *)buf;
    float *d_pix = (float *)(buf + b_off);
    float *d_dim = (float *)(buf + b_off + b_pix);
    float *d_lo = (float *)(buf + b_off + b_pix + b_dim);
    cuda_check(cudaMemcpyAsync(d_off, off.data(), off.size() * sizeof(float2), cudaMemcpyHostToDevice, c->stream),
               "h2d offsets");
    J.job.offsets = d_off;
    launch_path_samples(J, first_path, n, dims, bounces, pixel_offsets ? d_pix : nullptr, dims ? d_dim : nullptr,
                        bounces ? d_lo : nullptr, c->stream);
    cuda_check(cudaGetLastError(), "sample-eval launch");
    if (pixel_offsets)
      cuda_check(cudaMemcpyAsync(pixel_offsets, d_pix, nn * 8, cudaMemcpyDeviceToHost, c->stream), "d2h");
    if (dims)
      cuda_check(cudaMemcpyAsync(dim_values, d_dim, nn * dims * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    if (bounces)
      cuda_check(cudaMemcpyAsync(light_offsets, d_lo, nn * bounces * LN * 8, cudaMemcpyDeviceToHost, c->stream),
                 "d2h");
    cuda_check(cudaStreamSynchronize(c->stream), "sample eval");
  });
}

static int trace_common(void *ctx, int32_t scene_id, bool any, const float *rays, const float *tmaxs, int32_t n,
                        float tmin, float tmax, float *t, int32_t *prim, float *uv, uint8_t *occ) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (n < 0 || !rays) fail(PT_ERR_INVALID, "bad trace args");
    if (n == 0) return PT_OK;
    Scene *S = c->scene(scene_id);
    const size_t nn = (size_t)n;
    char *buf = (char *)c->scratch(nn * (24 + 4 + 4 + 4 + 8 + 1) + 256);
    float *dr = (float *)buf;
    float *dtm = (float *)(buf + nn * 24);
    float *dt = (float *)(buf + nn * 28);
    int *dp = (int *)(buf + nn * 32);
    float *duv = (float *)(buf + nn * 36);
    uint8_t *docc = (uint8_t *)(buf + nn * 44);
    cuda_check(cudaMemcpyAsync(dr, rays, nn * 24, cudaMemcpyHostToDevice, c->stream), "h2d rays");
    if (any) cuda_check(cudaMemcpyAsync(dtm, tmaxs, nn * 4, cudaMemcpyHostToDevice, c->stream), "h2d tmax");
    launch_trace_test(S->view, any, dr, dtm, n, tmin, tmax, dt, dp, duv, docc, c->d_err, c->stream);
    cuda_check(cudaGetLastError(), "trace launch");
    if (any) {
      cuda_check(cudaMemcpyAsync(occ, docc, nn, cudaMemcpyDeviceToHost, c->stream), "d2h");
    } else {
      cuda_check(cudaMemcpyAsync(t, dt, nn * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
      cuda_check(cudaMemcpyAsync(prim, dp, nn * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
      if (uv) cuda_check(cudaMemcpyAsync(uv, duv, nn * 8, cudaMemcpyDeviceToHost, c->stream), "d2h");
    }
    cuda_check(cudaStreamSynchronize(c->stream), "trace");
    int herr = 0;
    cuda_check(cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost), "read err");
    if (herr) {
      cudaMemset(c->d_err, 0, sizeof(int));
      fail(PT_ERR_DEVICE, "device traversal error flag " + std::to_string(herr));
    }
  });
}

int pt_trace_closest(void *ctx, int32_t scene_id, const float *rays, int32_t n, float tmin, float tmax, float *t,
                     int32_t *prim, float *uv) {
  if (!t || !prim) return PT_ERR_INVALID;
  return trace_common(ctx, scene_id, false, rays, nullptr, n, tmin, tmax, t, prim, uv, nullptr);
}

int pt_trace_any(void *ctx, int32_t scene_id, const float *rays, const float *tmax, int32_t n, float tmin,
                 uint8_t *occluded) {
  if (!tmax || !occluded) return PT_ERR_INVALID;
  return trace_common(ctx, scene_id, true, rays, tmax, n, tmin, 0.f, nullptr, nullptr, nullptr, occluded);
}

int pt_intersect(void *ctx, int32_t scene_id, const float *rays, int32_t n, float tmin, float tmax, float *t,
                 int32_t *prim, float *position, float *normal, uint8_t *is_inside) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (n < 0 || !rays || !t || !prim || !position || !normal || !is_inside) fail(PT_ERR_INVALID, "bad intersect args");
    if (n == 0) return PT_OK;
    Scene *S = c->scene(scene_id);
    const size_t nn = (size_t)n;
    char *buf = (char *)c->scratch(nn * (24 + 4 + 4 + 12 + 12 + 1) + 256);
    float *dr = (float *)buf;
    float *dt = (float *)(buf + nn * 24);
    int *dp = (int *)(buf + nn * 28);
    float *dpos = (float *)(buf + nn * 32);
    float *dn = (float *)(buf + nn * 44);
    uint8_t *df = (uint8_t *)(buf + nn * 56);
    cuda_check(cudaMemcpyAsync(dr, rays, nn * 24, cudaMemcpyHostToDevice, c->stream), "h2d rays");
    launch_intersect(S->view, dr, n, tmin, tmax, dt, dp, dpos, dn, df, c->d_err, c->stream);
    cuda_check(cudaGetLastError(), "intersect launch");
    cuda_check(cudaMemcpyAsync(t, dt, nn * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(prim, dp, nn * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(position, dpos, nn * 12, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(normal, dn, nn * 12, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(is_inside, df, nn, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaStreamSynchronize(c->stream), "intersect");
    int herr = 0;
    cuda_check(cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost), "read err");
    if (herr) {
      cudaMemset(c->d_err, 0, sizeof(int));
      fail(PT_ERR_DEVICE, "device traversal error flag " + std::to_string(herr));
    }
  });
}

int pt_light_sample(void *ctx, int32_t scene_id, int32_t light, int32_t n, const float *uv, const float *x,
                    const float *pdf_dir, float *point, float *normal, float *dir, float *le, float *pdf,
                    float *area) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (n < 0 || (n > 0 && (!uv || !x || !point || !normal || !dir || !le || !pdf)))
      fail(PT_ERR_INVALID, "bad light-sample args");
    Scene *S = c->scene(scene_id);
    if (light < 0 || light >= S->view.n_lights) fail(PT_ERR_INVALID, "light index out of range");
    const LightRec &L = S->host_lights[light];
    if (area) *area = L.type == LIGHT_ENV ? INFINITY : L.area;
    if (n == 0) return PT_OK;
    const size_t nn = (size_t)n;
    char *buf = (char *)c->scratch(nn * (8 + 12 + 12 + 12 * 4 + 4) + 256);
    float *duv = (float *)buf;
    float *dx = (float *)(buf + nn * 8);
    float *dpd = (float *)(buf + nn * 20);
    float *dout = (float *)(buf + nn * 32);  // point, normal, dir, le (3n each), pdf (n)
    cuda_check(cudaMemcpyAsync(duv, uv, nn * 8, cudaMemcpyHostToDevice, c->stream), "h2d uv");
    cuda_check(cudaMemcpyAsync(dx, x, nn * 12, cudaMemcpyHostToDevice, c->stream), "h2d x");
    if (pdf_dir) cuda_check(cudaMemcpyAsync(dpd, pdf_dir, nn * 12, cudaMemcpyHostToDevice, c->stream), "h2d dir");
    launch_light_eval(S->view, light, n, duv, dx, pdf_dir ? dpd : nullptr, dout, dout + 3 * nn, dout + 6 * nn,
                      dout + 9 * nn, dout + 12 * nn, c->stream);
    cuda_check(cudaGetLastError(), "light launch");
    cuda_check(cudaMemcpyAsync(point, dout, 12 * nn, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(normal, dout + 3 * nn, 12 * nn, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(dir, dout + 6 * nn, 12 * nn, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(le, dout + 9 * nn, 12 * nn, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(pdf, dout + 12 * nn, 4 * nn, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaStreamSynchronize(c->stream), "light sample");
  });
}

int pt_bsdf_eval(void *ctx, const pt_material_desc *mat, int32_t n, const float *wo, const float *wi,
                 const float *normal, const uint8_t *front, float *f, float *pdf) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (!mat || n < 0 || !wo || !wi || !normal || !front || !f || !pdf) fail(PT_ERR_INVALID, "bad bsdf args");
    if (n == 0) return PT_OK;
    MatRec m = derive_material(*mat);
    const size_t nn = (size_t)n;
    char *buf = (char *)c->scratch(sizeof(MatRec) + nn * (12 * 3 + 1 + 12 + 4) + 1024);
    MatRec *dm = (MatRec *)buf;
    float *dwo = (float *)(buf + 256);
    float *dwi = dwo + 3 * nn;
    float *dn = dwi + 3 * nn;
    float *df = dn + 3 * nn;
    float *dpdf = df + 3 * nn;
    uint8_t *dfr = (uint8_t *)(dpdf + nn);
    cuda_check(cudaMemcpyAsync(dm, &m, sizeof m, cudaMemcpyHostToDevice, c->stream), "h2d");
    cuda_check(cudaMemcpyAsync(dwo, wo, nn * 12, cudaMemcpyHostToDevice, c->stream), "h2d");
    cuda_check(cudaMemcpyAsync(dwi, wi, nn * 12, cudaMemcpyHostToDevice, c->stream), "h2d");
    cuda_check(cudaMemcpyAsync(dn, normal, nn * 12, cudaMemcpyHostToDevice, c->stream), "h2d");
    cuda_check(cudaMemcpyAsync(dfr, front, nn, cudaMemcpyHostToDevice, c->stream), "h2d");
    launch_bsdf_eval(dm, n, dwo, dwi, dn, dfr, df, dpdf, c->stream);
    cuda_check(cudaGetLastError(), "bsdf launch");
    cuda_check(cudaMemcpyAsync(f, df, nn * 12, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(pdf, dpdf, nn * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaStreamSynchronize(c->stream), "bsdf");
  });
}

int pt_bsdf_sample(void *ctx, const pt_material_desc *mat, int32_t n, const float *wo, const float *normal,
                   const uint8_t *front, const float *uc, const float *u, uint8_t *ok, float *wi,
                   float *attenuation, float *pdf_val, uint32_t *sampled_type) {
  Context *c = static_cast<Context *>(ctx);
  PT_GUARD(c, {
    c = as_ctx(ctx);
    if (!mat || n < 0 || !wo || !normal || !front || !uc || !u || !ok || !wi || !attenuation || !pdf_val ||
        !sampled_type)
      fail(PT_ERR_INVALID, "bad bsdf args");
    if (n == 0) return PT_OK;
    MatRec m = derive_material(*mat);
    const size_t nn = (size_t)n;
    char *buf = (char *)c->scratch(sizeof(MatRec) + nn * 80 + 1024);
    MatRec *dm = (MatRec *)buf;
    float *dwo = (float *)(buf + 256);
    float *dn = dwo + 3 * nn;
    float *duc = dn + 3 * nn;
    float *du = duc + nn;
    float *dwi = du + 2 * nn;
    float *datt = dwi + 3 * nn;
    float *dpdf = datt + 3 * nn;
    uint32_t *dty = (uint32_t *)(dpdf + nn);
    uint8_t *dfr = (uint8_t *)(dty + nn);
    uint8_t *dok = dfr + nn;
    cuda_check(cudaMemcpyAsync(dm, &m, sizeof m, cudaMemcpyHostToDevice, c->stream), "h2d");
    cuda_check(cudaMemcpyAsync(dwo, wo, nn * 12, cudaMemcpyHostToDevice, c->stream), "h2d");
    cuda_check(cudaMemcpyAsync(dn, normal, nn * 12, cudaMemcpyHostToDevice, c->stream), "h2d");
    cuda_check(cudaMemcpyAsync(duc, uc, nn * 4, cudaMemcpyHostToDevice, c->stream), "h2d");
    cuda_check(cudaMemcpyAsync(du, u, nn * 8, cudaMemcpyHostToDevice, c->stream), "h2d");
    cuda_check(cudaMemcpyAsync(dfr, front, nn, cudaMemcpyHostToDevice, c->stream), "h2d");
    launch_bsdf_sample(dm, n, dwo, dn, dfr, duc, du, dok, dwi, datt, dpdf, dty, c->stream);
    cuda_check(cudaGetLastError(), "bsdf launch");
    cuda_check(cudaMemcpyAsync(ok, dok, nn, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(wi, dwi, nn * 12, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(attenuation, datt, nn * 12, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(pdf_val, dpdf, nn * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaMemcpyAsync(sampled_type, dty, nn * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    cuda_check(cudaStreamSynchronize(c->stream), "bsdf");
  });
}

}  // extern "C"
