// pt_kernels_persist.cu -- the batched form as ONE persistent launch per
// merged group: camera, every bounce's closest-hit trace, shade, shadow rays
// and their resolve, and the films, for every wave of the group, run by one
// cooperative kernel whose blocks stay resident and move from stage to stage
// through grid barriers instead of kernel boundaries.  The stage bodies are
// the ones the per-stage kernels run (pt_wave.cuh); shading uses the generic
// body (run-time material dispatch, no material sort), and from bounce 1 on
// each bounce's closest-hit rays are traced together with the previous
// bounce's shadow rays, whose terms are added (resolve) before the next
// shade -- the order of additions into a path's radiance is the per-stage
// form's, so films agree.
//
// Grid barrier: one arrival counter and a generation word per group.  Thread
// 0 of every block arrives with an atomic; the last block to arrive runs the
// barrier's counter resets (the queue and fetch counters the next stage
// starts from), then bumps the generation; the others wait for the bump.
// Every wait is bounded (PT_BARRIER_SPINS polls with a nanosleep between
// them, seconds in all): a block that gives up sets the barrier's error word
// and every block returns at its next barrier, so a fault ends the kernel
// with an error the host reports, never a hang.  The cooperative launch
// guarantees that every block of the grid is resident, which the barrier
// needs.  Stages read queue records that earlier stages of the same kernel
// wrote, so they are read from L2 (PT_QUEUE_LOADS_COHERENT), not through the
// read-only cache the per-stage kernels use.
#define PT_QUEUE_LOADS_COHERENT
#include "pt_wave.cuh"

namespace pt {

void upload_halton_tables_persist(const HaltonTables &T, cudaStream_t st) {
  cudaMemcpyToSymbolAsync(c_halton, &T, sizeof(T), 0, cudaMemcpyHostToDevice, st);
}

#define PT_BARRIER_SPINS (1u << 24)
#define PT_PERSIST_THREADS 128
#define PT_PERSIST_MIN_BLOCKS 4

struct GridBarrier {
  unsigned count;
  unsigned gen;
  int err;
  int pad;
};

// Arrive and wait; `last` runs in the last arriving block's thread 0 before
// the others are released.  False: the barrier failed (a wait ran out, here
// or in another block) and the kernel must return.
template <class Last>
__device__ __forceinline__ bool grid_sync(GridBarrier *b, Last last) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile GridBarrier *vb = b;
    ok = vb->err == 0;
    if (ok) {
      const unsigned g = vb->gen;
      __threadfence();
      if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
        last();
        b->count = 0;
        __threadfence();
        atomicAdd(&b->gen, 1u);
      } else {
        unsigned spins = 0;
        while (vb->gen == g) {
          if (vb->err || ++spins > PT_BARRIER_SPINS) {
            atomicExch(&b->err, 1);
            ok = 0;
            break;
          }
          __nanosleep(128);
        }
      }
      __threadfence();
    }
  }
  __syncthreads();
  // every thread orders its later loads after the other blocks' stores
  __threadfence();
  return ok != 0;
}

struct NoReset {
  __device__ void operator()() const {}
};

// The stages as separately compiled functions: each gets its own register
// allocation (the traversal does not inherit the shading's register pressure
// and spills), and reads the kernel's parameters in place (__grid_constant__).
template <bool CURVES>
__device__ __noinline__ void st_trace(const SceneView &S, const DeviceJob &none, const JobTable &T, const Queues &Q,
                                      int qsel, int b, long long g0, int LN, int32_t *stack) {
  if (b > 0)
    trace_pair_body<true, CURVES>(S, none, T, Q, qsel, b, g0, LN, stack);
  else
    trace_closest_body<true, CURVES>(S, none, T, Q, qsel, b, g0, stack);
}
__device__ __noinline__ void st_shade(const SceneView &S, const DeviceJob &none, const JobTable &T, const Queues &Q,
                                      int qsel, int b, long long g0) {
  shade_body<-1, true>(S, none, T, Q, qsel, b, g0);
}
template <bool CURVES>
__device__ __noinline__ void st_shadow(const SceneView &S, const Queues &Q, int LN, int32_t *stack) {
  trace_shadow_body<CURVES>(S, Q, LN, stack);
}

// The whole group: for each wave of `wave` paths over [0, total), camera ->
// per bounce (trace [+ previous shadow rays] -> resolve -> shade) -> last
// shadow rays -> resolve -> films.
template <bool CURVES>
__global__ void __launch_bounds__(PT_PERSIST_THREADS, PT_PERSIST_MIN_BLOCKS)
    k_group_persistent(const __grid_constant__ SceneView S, const __grid_constant__ JobTable T,
                       const __grid_constant__ Queues Q, float *const *films, long long total, int wave, int LN,
                       int bounces, GridBarrier *bar) {
  extern __shared__ int32_t stack[];  // S.stack_entries x PT_PERSIST_THREADS
  __shared__ DeviceJob none;  // unused by merged waves (each path's job comes from T)
  if (threadIdx.x == 0) memset(&none, 0, sizeof none);
  __syncthreads();
  int *cnt = Q.counts;
  for (long long g0 = 0; g0 < total; g0 += wave) {
    const int n = (int)min((long long)wave, total - g0);
    camera_body<true>(none, T, Q, g0, n);
    if (!grid_sync(bar, [=] { cnt[1] = 0; cnt[2] = 0; cnt[3] = 0; cnt[4] = 0; })) return;
    int qsel = 0;
    for (int b = 0; b < bounces; ++b) {
      st_trace<CURVES>(S, none, T, Q, qsel, b, g0, LN, stack);
      const int nq = qsel ^ 1;
      if (!grid_sync(bar, [=] { cnt[nq] = 0; cnt[4] = 0; })) return;
      if (b > 0) {
        shadow_resolve_body(Q, LN);
        if (!grid_sync(bar, [=] { cnt[2] = 0; cnt[3] = 0; })) return;
      }
      st_shade(S, none, T, Q, qsel, b, g0);
      if (!grid_sync(bar, NoReset())) return;
      qsel = nq;
    }
    st_shadow<CURVES>(S, Q, LN, stack);
    if (!grid_sync(bar, NoReset())) return;
    shadow_resolve_body(Q, LN);
    if (!grid_sync(bar, NoReset())) return;
    // films: each job's share of the wave, pixels grid-strided per job
    const long long g1 = g0 + n;
    for (int k = 0; k < T.n; ++k) {
      const long long a = max(g0, T.start[k]), e = min(g1, T.start[k + 1]);
      if (a >= e) continue;
      film_body(T.jobs[k], Q, a - T.start[k], (int)(e - a), a - g0, films[k]);
    }
    if (!grid_sync(bar, NoReset())) return;
  }
}

int persistent_grid(const SceneView &S, int num_sms) {
  int per = 0;
  const size_t smem = stack_bytes(S, PT_PERSIST_THREADS);
  if (S.curves)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_group_persistent<true>, PT_PERSIST_THREADS, smem);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_group_persistent<false>, PT_PERSIST_THREADS, smem);
  return std::max(1, per) * num_sms;
}

cudaError_t launch_group_persistent(const SceneView &S, const JobTable &T, const Queues &Q, float *const *d_films,
                                    long long total, int wave, int LN, int bounces, void *d_barrier, int grid,
                                    cudaStream_t st) {
  SceneView s = S;
  JobTable t = T;
  Queues q = Q;
  float *const *f = d_films;
  GridBarrier *b = static_cast<GridBarrier *>(d_barrier);
  void *args[] = {&s, &t, &q, &f, &total, &wave, &LN, &bounces, &b};
  const void *fn = S.curves ? (const void *)k_group_persistent<true> : (const void *)k_group_persistent<false>;
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(PT_PERSIST_THREADS), args,
                                     stack_bytes(S, PT_PERSIST_THREADS), st);
}

}  // namespace pt
