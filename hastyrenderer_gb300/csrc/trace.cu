// Closest-hit ray queries (the role of Embree's rtcIntersect1 in
// core/src/Scene.cpp:281-303: tnear 1e-6, tfar +inf, u/v = weights of the
// triangle's 2nd/3rd vertex) over the compressed 8-wide BVH (default) or the
// binary BVH. One thread per queued ray.
//
// The traversal routines (traverse.cuh) are host+device: the host build runs
// the same code on the CPU for the loader/builder tests
// (hasty_debug_host_trace).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include "hasty_types.h"
#include "wavefront.h"
#include "traverse.cuh"

namespace hasty {
namespace {

// Minimum resident blocks per SM for the closest-hit kernels (0: none).
#ifndef HASTY_TRACE_MIN_BLOCKS
#define HASTY_TRACE_MIN_BLOCKS 0
#endif
#if HASTY_TRACE_MIN_BLOCKS > 0
#define TRACE_BOUNDS __launch_bounds__(128, HASTY_TRACE_MIN_BLOCKS)
#else
#define TRACE_BOUNDS __launch_bounds__(128)
#endif

// Persistent closest-hit kernels (Aila and Laine 2009, dynamic fetch): a
// grid of the SMs' resident blocks loops until the ray queue is drained.
// Whenever kRefill lanes of a warp are idle, the warp takes that many rays
// from the queue with one atomic on the fetch counter, so lanes whose rays
// finish early do not idle while their warp's longest ray is traversed. Each
// ray's traversal is the same sequence of steps as trace_binary/trace_wide.
// kRefill on the 1080p sphere field (M samples/s): 4: 917, 8: 945, 12: 931; again
// later (closest hits, ms per bounce launch): 4: 0.877, 8: 0.845, 12: 0.852, 16: 0.894.
#ifndef HASTY_TRACE_REFILL
#define HASTY_TRACE_REFILL 8
#endif
constexpr int kRefill = HASTY_TRACE_REFILL;
// Persistent traversal pays for the wide BVH (one node per step, long and
// uneven rays); the binary BVH's leaf-to-leaf steps are too short to carry
// the refill bookkeeping, so it runs one ray per thread.
template <int KIND> constexpr bool kPersistent = KIND == 1;

template <int KIND> struct TravOf { using T = TravBinary; };
template <> struct TravOf<1> { using T = TravWide; };

// First thread of a bounce's closest-hit launch: counts the rays and clears
// the queue counters the bounce's shading kernels fill (path and ray queue
// q^1, the sample queue), which nothing reads until then, so the host
// enqueues no memsets between the kernels. (The fetch counter this launch
// uses was cleared by the kernel before it: ray generation or resolve.)
__device__ __forceinline__ void start_bounce_counters(const PathsDev& P, int q, uint32_t n) {
  P.counts[q ^ 1] = 0;
  P.counts[2 + (q ^ 1)] = 0;
  P.counts[kSampleCount] = 0;
  if (n) atomicAdd(&P.stats[ST_RAYS], (unsigned long long)n);
}

// Adds this warp's count of rays whose traversal stack overflowed to `stat`
// (one atomic per warp, only when there are any).
__device__ __forceinline__ void add_overflows(unsigned long long* stat, uint32_t mine) {
  const unsigned b = __ballot_sync(kFullMask, mine != 0);
  if (!b) return;
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(kFullMask, mine, o);
  if ((threadIdx.x & 31u) == 0) atomicAdd(stat, (unsigned long long)mine);
}

// Returns the number of this thread's rays whose traversal stack overflowed.
template <int KIND, class Fetch, class Done>
__device__ __forceinline__ uint32_t persistent_trace(uint32_t n, uint32_t* next, Fetch fetch, Done done) {
  typename TravOf<KIND>::T tr;
  typename TravOf<KIND>::T::Entry stack[TravOf<KIND>::T::kDepth];
  const float4* nodes = nullptr;
  const float4* tris = nullptr;
  int rid = 0;
  uint32_t overflows = 0;
  bool active = false;
  bool drained = false;                 // warp-uniform: the queue has been handed out
  const uint32_t lane = threadIdx.x & 31u;
  for (;;) {
    if (!drained) {
      const unsigned idle = __ballot_sync(kFullMask, !active);
      const uint32_t n_idle = uint32_t(__popc(idle));
      if (n_idle >= uint32_t(kRefill)) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(next, n_idle);
        base = __shfl_sync(kFullMask, base, 0);
        if (base >= n || n - base <= n_idle) drained = true;
        if (!active) {
          const uint32_t k = base + uint32_t(__popc(idle & ((1u << lane) - 1u)));
          if (k < n) {
            fetch(k, tr, nodes, tris, rid);
            active = true;
          }
        }
      }
    }
    if (__ballot_sync(kFullMask, active) == 0) break;   // drained: an all-idle warp always refills otherwise
    if (active && tr.step(nodes, tris, stack)) {
      done(rid, tr.best);
      overflows += tr.overflow ? 1u : 0u;
      active = false;
    }
  }
  return overflows;
}

// One ray per thread over a grid-sized stride, for BVHs of a few nodes
// (short rays of similar length: the dynamic fetch's bookkeeping and its
// partly idle warps can cost more than it saves there). Same steps per ray
// as persistent_trace, so the same hits.
template <int KIND, class Fetch, class Done>
__device__ __forceinline__ uint32_t simple_trace(uint32_t n, Fetch fetch, Done done) {
  typename TravOf<KIND>::T tr;
  typename TravOf<KIND>::T::Entry stack[TravOf<KIND>::T::kDepth];
  const float4* nodes = nullptr;
  const float4* tris = nullptr;
  int rid = 0;
  uint32_t overflows = 0;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    fetch(k, tr, nodes, tris, rid);
    while (!tr.step(nodes, tris, stack)) {}
    done(rid, tr.best);
    overflows += tr.overflow ? 1u : 0u;
  }
  return overflows;
}

template <int KIND, bool SIMPLE = false>
__global__ void TRACE_BOUNDS k_trace(SceneDev sc, PathsDev P, int q) {
  const uint32_t n = P.counts[2 + q];
  if (blockIdx.x == 0 && threadIdx.x == 0) start_bounce_counters(P, q, n);
  // blocks past the queue exit at once (the persistent blocks before them take all the rays)
  if (blockIdx.x * blockDim.x >= n) return;
  const int32_t* rq = P.rq[q];
  if (!kPersistent<KIND>) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      int rid = rq[i];
      if (!HASTY_IN_BOUNDS(rid >= 0 && rid < 2 * P.capacity, BB_QUEUE)) rid = 0;
      float4 o = P.ray_o[rid], d = P.ray_d[rid];
      Hit h = trace_any<KIND>(sc.nodes, sc.isect_tris, o.x, o.y, o.z, d.x, d.y, d.z);
      P.hit[rid] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
    }
    return;
  }
  // Light-sample rays (odd ids) of a scene whose only light is the
  // environment are visible iff they hit nothing (Scene.cpp:575-585 with no
  // emissive triangle), so they stop at their first hit.
  const bool nee_any = sc.n_light_tris == 0;
  auto fetch = [&](uint32_t k, typename TravOf<KIND>::T& tr, const float4*& nodes, const float4*& tris, int& rid) {
    rid = rq[k];
    if (!HASTY_IN_BOUNDS(rid >= 0 && rid < 2 * P.capacity, BB_QUEUE)) rid = 0;
    float4 o = P.ray_o[rid], d = P.ray_d[rid];
    tr.init(o.x, o.y, o.z, d.x, d.y, d.z);
    tr.any = nee_any && (rid & 1);
    nodes = sc.nodes;
    tris = sc.isect_tris;
    HASTY_TRAV_LIMITS(tr, sc.n_nodes, sc.n_tris);
  };
  auto done = [&](int rid, const Hit& h) { P.hit[rid] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri)); };
  const uint32_t overflows = SIMPLE ? simple_trace<KIND>(n, fetch, done)
                                    : persistent_trace<KIND>(n, &P.counts[kFetchCounter], fetch, done);
  add_overflows(&P.stats[ST_STACK_OVERFLOW], overflows);
}

template <int KIND>
__global__ void k_trace_rays(SceneDev sc, const float* rays, int n, float4* hits) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = rays + 6 * int64_t(i);
  Hit h = trace_any<KIND>(sc.nodes, sc.isect_tris, r[0], r[1], r[2], r[3], r[4], r[5]);
  hits[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
}

// Packed multi-job batches: each ray names its chunk in ray_o.w (bits), and
// the chunk's BVH comes from the kernel-parameter table.
template <int KIND, bool SIMPLE = false>
__global__ void TRACE_BOUNDS k_trace_packed(const __grid_constant__ TraceTable T, PathsDev P, int q) {
  const uint32_t n = P.counts[2 + q];
  if (blockIdx.x == 0 && threadIdx.x == 0) start_bounce_counters(P, q, n);
  // blocks past the queue exit at once (the persistent blocks before them take all the rays)
  if (blockIdx.x * blockDim.x >= n) return;
  const int32_t* rq = P.rq[q];
  if (!kPersistent<KIND>) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      int rid = rq[i];
      if (!HASTY_IN_BOUNDS(rid >= 0 && rid < 2 * P.capacity, BB_QUEUE)) rid = 0;
      float4 o = P.ray_o[rid], d = P.ray_d[rid];
      const TraceChunk& c = T.c[__float_as_uint(o.w)];
      Hit h = trace_any<KIND>(c.nodes, c.tris, o.x, o.y, o.z, d.x, d.y, d.z);
      P.hit[rid] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
    }
    return;
  }
  auto fetch = [&](uint32_t k, typename TravOf<KIND>::T& tr, const float4*& nodes, const float4*& tris, int& rid) {
    rid = rq[k];
    if (!HASTY_IN_BOUNDS(rid >= 0 && rid < 2 * P.capacity, BB_QUEUE)) rid = 0;
    float4 o = P.ray_o[rid], d = P.ray_d[rid];
    const TraceChunk& c = T.c[__float_as_uint(o.w)];
    tr.init(o.x, o.y, o.z, d.x, d.y, d.z);
    tr.any = c.nee_first_hit != 0 && (rid & 1);   // as k_trace
    nodes = c.nodes;
    tris = c.tris;
    HASTY_TRAV_LIMITS(tr, c.n_nodes, c.n_tris);
  };
  auto done = [&](int rid, const Hit& h) { P.hit[rid] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri)); };
  const uint32_t overflows = SIMPLE ? simple_trace<KIND>(n, fetch, done)
                                    : persistent_trace<KIND>(n, &P.counts[kFetchCounter], fetch, done);
  add_overflows(&P.stats[ST_STACK_OVERFLOW], overflows);
}

// Multi-job engine: each ray belongs to the job of its path slot (ray id / 2).
// All jobs of one engine share the BVH layout of their context (KIND).
template <int KIND>
__global__ void TRACE_BOUNDS k_trace_multi(PathsDev P, MultiDev m) {
  const uint32_t q = m.ctl[0];
  const uint32_t n = P.counts[2 + q];
  if (blockIdx.x == 0 && threadIdx.x == 0 && n) atomicAdd(&P.stats[ST_RAYS], (unsigned long long)n);
  const int32_t* rq = P.rq[q];
  if (!kPersistent<KIND>) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      int rid = rq[i];
      if (!HASTY_IN_BOUNDS(rid >= 0 && rid < 2 * P.capacity, BB_QUEUE)) rid = 0;
      const SceneDev& sc = m.jobs[m.slot_meta[rid >> 1].x].sc;
      float4 o = P.ray_o[rid], d = P.ray_d[rid];
      Hit h = trace_any<KIND>(sc.nodes, sc.isect_tris, o.x, o.y, o.z, d.x, d.y, d.z);
      P.hit[rid] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
    }
    return;
  }
  const uint32_t overflows = persistent_trace<KIND>(
      n, &P.counts[kFetchCounter],
      [&](uint32_t k, typename TravOf<KIND>::T& tr, const float4*& nodes, const float4*& tris, int& rid) {
        rid = rq[k];
        if (!HASTY_IN_BOUNDS(rid >= 0 && rid < 2 * P.capacity, BB_QUEUE)) rid = 0;
        const SceneDev& sc = m.jobs[m.slot_meta[rid >> 1].x].sc;
        float4 o = P.ray_o[rid], d = P.ray_d[rid];
        tr.init(o.x, o.y, o.z, d.x, d.y, d.z);
        tr.any = sc.n_light_tris == 0 && (rid & 1);   // as k_trace
        nodes = sc.nodes;
        tris = sc.isect_tris;
        HASTY_TRAV_LIMITS(tr, sc.n_nodes, sc.n_tris);
      },
      [&](int rid, const Hit& h) { P.hit[rid] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri)); });
  add_overflows(&P.stats[ST_STACK_OVERFLOW], overflows);
}

// Resident blocks of a persistent trace kernel on the current device.
struct PersistentShape { int sms, per_sm; };
template <class K>
PersistentShape persistent_shape(K kernel) {
  int dev = 0;
  cudaGetDevice(&dev);
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0);
  return {sms < 1 ? 1 : sms, per_sm < 1 ? 1 : per_sm};
}

// Persistent grid: all resident blocks, or at most cap_per_sm per SM (to leave
// room for kernels of another stream); HASTY_TRACE_BLOCKS_PER_SM overrides
// both (tuning).
int persistent_blocks(PersistentShape s, int cap_per_sm) {
  int per = s.per_sm;
  if (cap_per_sm > 0 && cap_per_sm < per) per = cap_per_sm;
  if (const char* v = std::getenv("HASTY_TRACE_BLOCKS_PER_SM")) {
    int b = std::atoi(v);
    if (b >= 1 && b < s.per_sm) per = b;
  }
  return s.sms * per;
}

}  // namespace

// Wide BVHs of at most this many nodes are traced one ray per thread
// (simple_trace); HASTY_TRACE_SIMPLE_NODES overrides it (tuning). Cornell
// box, 36 triangles: closest hits 0.268 -> 0.235 ms per bounce launch, 664 ->
// 707 M samples/s.
constexpr int kSimpleTraceNodes = 64;
int simple_trace_nodes() {
  static const int v = [] {
    const char* e = std::getenv("HASTY_TRACE_SIMPLE_NODES");
    return e ? std::atoi(e) : kSimpleTraceNodes;
  }();
  return v;
}
bool simple_trace_bvh(const SceneDev& sc) { return sc.bvh_kind == 1 && sc.n_nodes <= simple_trace_nodes(); }

// The persistent kernels take rays through P.counts[kFetchCounter]: cleared
// on the stream before each launch of the engine's kernel, and by the kernel
// before it (ray generation, resolve) for the wavefront's. Grids: the SMs'
// resident blocks (at most blocks_per_sm per SM when given), fewer when the
// queue bound is smaller.
void launch_trace_multi(const PathsDev& p, const MultiDev& m, int bvh_kind, int max_rays, cudaStream_t st,
                        int blocks_per_sm) {
  static PersistentShape shape[2] = {{0, 0}, {0, 0}};
  int k = bvh_kind == 1 ? 1 : 0;
  if (!shape[k].sms) shape[k] = k ? persistent_shape(k_trace_multi<1>) : persistent_shape(k_trace_multi<0>);
  const int grid = persistent_blocks(shape[k], blocks_per_sm);
  // one-ray-per-thread kernels loop over the queue with a grid-sized stride
  int blocks = std::min(k ? grid : 8 * grid, std::max(1, (max_rays + 127) / 128));
  cudaMemsetAsync(&p.counts[kFetchCounter], 0, sizeof(uint32_t), st);
  if (k) k_trace_multi<1><<<blocks, 128, 0, st>>>(p, m);
  else k_trace_multi<0><<<blocks, 128, 0, st>>>(p, m);
}

void launch_trace_packed(const TraceTable& t, const PathsDev& p, int q, int max_rays, cudaStream_t st, int blocks_per_sm) {
  static PersistentShape shape[2] = {{0, 0}, {0, 0}};
  const int k = t.bvh_kind == 1 ? 1 : 0;
  if (!shape[k].sms) shape[k] = k ? persistent_shape(k_trace_packed<1>) : persistent_shape(k_trace_packed<0>);
  int max_nodes = 0;
  for (int c = 0; c < t.n; ++c) max_nodes = std::max(max_nodes, t.c[c].n_nodes);
  const int simple = k && max_nodes <= simple_trace_nodes() ? 1 : 0;
  const int grid = persistent_blocks(shape[k], blocks_per_sm);
  int blocks = k && !simple ? std::min(grid, std::max(1, (max_rays + 127) / 128))
                            : std::min(8 * grid, std::max(1, (max_rays + 127) / 128));
  if (k && simple) k_trace_packed<1, true><<<blocks, 128, 0, st>>>(t, p, q);
  else if (k) k_trace_packed<1><<<blocks, 128, 0, st>>>(t, p, q);
  else k_trace_packed<0><<<blocks, 128, 0, st>>>(t, p, q);
}

void launch_trace(const SceneDev& sc, const PathsDev& p, int q, int max_rays, cudaStream_t st, int blocks_per_sm) {
  static PersistentShape shape[2] = {{0, 0}, {0, 0}};
  int k = sc.bvh_kind == 1 ? 1 : 0;
  if (!shape[k].sms) shape[k] = k ? persistent_shape(k_trace<1>) : persistent_shape(k_trace<0>);
  const int simple = simple_trace_bvh(sc) ? 1 : 0;
  const int grid = persistent_blocks(shape[k], blocks_per_sm);
  int blocks = k && !simple ? std::min(grid, std::max(1, (max_rays + 127) / 128))
                            : std::min(8 * grid, std::max(1, (max_rays + 127) / 128));
  if (k && simple) k_trace<1, true><<<blocks, 128, 0, st>>>(sc, p, q);
  else if (k) k_trace<1><<<blocks, 128, 0, st>>>(sc, p, q);
  else k_trace<0><<<blocks, 128, 0, st>>>(sc, p, q);
}

void launch_trace_rays(const SceneDev& sc, const float* rays, int n, float4* hits, cudaStream_t st) {
  if (n <= 0) return;
  if (sc.bvh_kind == 1) k_trace_rays<1><<<(n + 127) / 128, 128, 0, st>>>(sc, rays, n, hits);
  else k_trace_rays<0><<<(n + 127) / 128, 128, 0, st>>>(sc, rays, n, hits);
}

// CPU run of the same traversal over host copies of the BVH arrays.
void host_trace_rays(int kind, const float4* nodes, const float4* tris, const float* rays, int64_t n, float4* hits) {
  for (int64_t i = 0; i < n; ++i) {
    const float* r = rays + 6 * i;
    Hit h = kind == 1 ? trace_wide(nodes, tris, r[0], r[1], r[2], r[3], r[4], r[5])
                      : trace_binary(nodes, tris, r[0], r[1], r[2], r[3], r[4], r[5]);
    int32_t id = h.tri;
    float w; std::memcpy(&w, &id, 4);
    hits[i] = make_float4(h.t, h.u, h.v, w);
  }
}

}  // namespace hasty

// Status word of this file's bounds checks (bounds-checked build).
HASTY_BOUNDS_READER(bounds_status_trace)
