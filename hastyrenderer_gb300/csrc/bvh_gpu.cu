// Binned-SAH binary BVH builder on the GPU (the role of Embree's scene build,
// core/src/Scene.cpp:122-191; split rule of the host builder in
// bvh_build.cpp: 32 centroid bins per axis, surface-area cost, a node with at
// most max_leaf triangles becomes a leaf unless a split costs less).
//
// Top-down, level by level for large nodes, then one warp per small subtree:
//  * large nodes (more than kSmall triangles): their triangle ranges are cut
//    into chunks of kChunk; per level, chunk blocks reduce centroid and box
//    bounds, bin centroids (counts + bin boxes in shared memory, merged into
//    the node's bins with one atomic per bin and value), one warp per node
//    evaluates the SAH, and chunk blocks partition the node's index range
//    stably (left block offsets from a per-node scan of chunk counts);
//  * small nodes: one warp builds the whole subtree with an explicit stack,
//    binning in shared memory and partitioning with warp ballots.
// Float min/max are reduced with integer atomics on an order-preserving
// encoding of the float bits. Node boxes are exact bounds of their
// triangles, so the layout writers' conservative quantisation holds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <climits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "bvh_build.h"

namespace hasty {
namespace {

constexpr int kBins = 32;
constexpr int kSmall = 1024;          // nodes at or below this size go to the warp builder
constexpr int kChunk = 4096;          // triangles per chunk block of a large node
constexpr int kThreads = 256;
constexpr int kWarpStack = 64;        // subtree stack entries per warp (depth bound of a small subtree)
constexpr unsigned kAll = 0xFFFFFFFFu;

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string("GPU BVH build: ") + what + ": " + cudaGetErrorString(e));
}

// order-preserving float <-> int encoding for atomicMin / atomicMax
__device__ __forceinline__ int f2o(float f) {
  int b = __float_as_int(f);
  return b >= 0 ? b : b ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float o2f(int b) { return __int_as_float(b >= 0 ? b : b ^ 0x7FFFFFFF); }

struct Task { int32_t node, first, count, depth; };
struct Chunk { int32_t task, start, len, pad; };

// Per large node: centroid bounds, box bounds, bins, split decision.
struct TaskAcc {
  int cmin[3], cmax[3];               // centroid bounds (encoded)
  int bmin[3], bmax[3];               // box bounds (encoded)
  int bin_cnt[3][kBins];
  int bin_min[3][kBins][3], bin_max[3][kBins][3];
  int axis, split_bin, by_index;      // decision (by_index: split at the middle index)
  int left;                           // left triangles
};

__device__ __forceinline__ float box_area(const float lo[3], const float hi[3]) {
  float d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
  if (d0 < 0.f) return 0.f;
  return 2.f * (d0 * d1 + d1 * d2 + d2 * d0);
}

__global__ void k_prims(const float* pos, int n, float4* tlo, float4* thi, float4* cen, int32_t* idx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* p = pos + 9 * int64_t(i);
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = fminf(fminf(p[a], p[3 + a]), p[6 + a]);
    hi[a] = fmaxf(fmaxf(p[a], p[3 + a]), p[6 + a]);
  }
  tlo[i] = make_float4(lo[0], lo[1], lo[2], 0.f);
  thi[i] = make_float4(hi[0], hi[1], hi[2], 0.f);
  cen[i] = make_float4(0.5f * (lo[0] + hi[0]), 0.5f * (lo[1] + hi[1]), 0.5f * (lo[2] + hi[2]), 0.f);
  idx[i] = i;
}

__global__ void k_acc_init(TaskAcc* acc, int n_tasks) {
  int t = blockIdx.x;
  if (t >= n_tasks) return;
  TaskAcc& a = acc[t];
  int* w = reinterpret_cast<int*>(&a);
  const int words = int(sizeof(TaskAcc) / sizeof(int));
  for (int k = threadIdx.x; k < words; k += blockDim.x) w[k] = 0;
  __syncthreads();
  if (threadIdx.x < 3) {
    a.cmin[threadIdx.x] = INT_MAX; a.cmax[threadIdx.x] = INT_MIN;
    a.bmin[threadIdx.x] = INT_MAX; a.bmax[threadIdx.x] = INT_MIN;
  }
  for (int k = threadIdx.x; k < 3 * kBins * 3; k += blockDim.x) {
    (&a.bin_min[0][0][0])[k] = INT_MAX;
    (&a.bin_max[0][0][0])[k] = INT_MIN;
  }
}

// Block reduction of 12 encoded bounds (6 min, 6 max) into the task's.
__device__ void block_bounds_merge(int v[12], int* smem, TaskAcc& a) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1)
    for (int k = 0; k < 12; ++k) {
      int u = __shfl_down_sync(kAll, v[k], o);
      v[k] = k < 6 ? min(v[k], u) : max(v[k], u);
    }
  if (lane == 0) for (int k = 0; k < 12; ++k) smem[warp * 12 + k] = v[k];
  __syncthreads();
  if (threadIdx.x < 12) {
    int k = threadIdx.x;
    int r = smem[k];
    for (int w = 1; w < nw; ++w) r = k < 6 ? min(r, smem[w * 12 + k]) : max(r, smem[w * 12 + k]);
    int* dst = k < 3 ? &a.cmin[k] : k < 6 ? &a.bmin[k - 3] : k < 9 ? &a.cmax[k - 6] : &a.bmax[k - 9];
    if (k < 6) atomicMin(dst, r); else atomicMax(dst, r);
  }
}

__global__ void __launch_bounds__(kThreads) k_chunk_bounds(const Chunk* chunks, const Task* tasks, const int32_t* idx,
                                                           const float4* tlo, const float4* thi, const float4* cen,
                                                           TaskAcc* acc) {
  __shared__ int smem[12 * (kThreads / 32)];
  const Chunk c = chunks[blockIdx.x];
  int v[12];
  for (int k = 0; k < 6; ++k) { v[k] = INT_MAX; v[6 + k] = INT_MIN; }
  for (int i = threadIdx.x; i < c.len; i += blockDim.x) {
    int t = idx[c.start + i];
    float4 ce = cen[t], lo = tlo[t], hi = thi[t];
    v[0] = min(v[0], f2o(ce.x)); v[1] = min(v[1], f2o(ce.y)); v[2] = min(v[2], f2o(ce.z));
    v[3] = min(v[3], f2o(lo.x)); v[4] = min(v[4], f2o(lo.y)); v[5] = min(v[5], f2o(lo.z));
    v[6] = max(v[6], f2o(ce.x)); v[7] = max(v[7], f2o(ce.y)); v[8] = max(v[8], f2o(ce.z));
    v[9] = max(v[9], f2o(hi.x)); v[10] = max(v[10], f2o(hi.y)); v[11] = max(v[11], f2o(hi.z));
  }
  block_bounds_merge(v, smem, acc[c.task]);
}

// The bin of centroid coordinate x on an axis with bounds [lo, lo + ext]:
// the host builder's formula, min(B - 1, int((x - lo) * (B / ext))), kept
// >= 0 for non-finite input.
__device__ __forceinline__ int bin_of(float x, float lo, float sc) { return max(0, min(kBins - 1, int((x - lo) * sc))); }

__global__ void __launch_bounds__(kThreads) k_chunk_bins(const Chunk* chunks, const int32_t* idx, const float4* tlo,
                                                         const float4* thi, const float4* cen, TaskAcc* acc) {
  __shared__ int s_cnt[3][kBins];
  __shared__ int s_min[3][kBins][3], s_max[3][kBins][3];
  const Chunk c = chunks[blockIdx.x];
  TaskAcc& a = acc[c.task];
  for (int k = threadIdx.x; k < 3 * kBins; k += blockDim.x) {
    (&s_cnt[0][0])[k] = 0;
    for (int j = 0; j < 3; ++j) { (&s_min[0][0][0])[3 * k + j] = INT_MAX; (&s_max[0][0][0])[3 * k + j] = INT_MIN; }
  }
  __syncthreads();
  float lo[3], sc[3];
  bool ok[3];
  for (int ax = 0; ax < 3; ++ax) {
    float l = o2f(a.cmin[ax]), h = o2f(a.cmax[ax]);
    float ext = h - l;
    ok[ax] = ext > 0.f;
    lo[ax] = l;
    sc[ax] = ok[ax] ? float(kBins) / ext : 0.f;
  }
  for (int i = threadIdx.x; i < c.len; i += blockDim.x) {
    int t = idx[c.start + i];
    float4 ce = cen[t], bl = tlo[t], bh = thi[t];
    float cc[3] = {ce.x, ce.y, ce.z};
    int el[3] = {f2o(bl.x), f2o(bl.y), f2o(bl.z)}, eh[3] = {f2o(bh.x), f2o(bh.y), f2o(bh.z)};
    for (int ax = 0; ax < 3; ++ax) {
      if (!ok[ax]) continue;
      int b = bin_of(cc[ax], lo[ax], sc[ax]);
      atomicAdd(&s_cnt[ax][b], 1);
      for (int j = 0; j < 3; ++j) { atomicMin(&s_min[ax][b][j], el[j]); atomicMax(&s_max[ax][b][j], eh[j]); }
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 3 * kBins; k += blockDim.x) {
    int ax = k / kBins, b = k % kBins;
    if (s_cnt[ax][b] == 0) continue;
    atomicAdd(&a.bin_cnt[ax][b], s_cnt[ax][b]);
    for (int j = 0; j < 3; ++j) { atomicMin(&a.bin_min[ax][b][j], s_min[ax][b][j]); atomicMax(&a.bin_max[ax][b][j], s_max[ax][b][j]); }
  }
}

// One thread per large task: node box and the SAH split (host builder's
// sweep: right-to-left suffix areas, then left-to-right).
__global__ void k_task_split(const Task* tasks, int n_tasks, TaskAcc* acc, TreeNode* nodes) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_tasks) return;
  const Task tk = tasks[k];
  TaskAcc& a = acc[k];
  TreeNode& nd = nodes[tk.node];
  for (int j = 0; j < 3; ++j) { nd.lo[j] = o2f(a.bmin[j]); nd.hi[j] = o2f(a.bmax[j]); }
  int axis = -1, split = -1;
  float best = FLT_MAX;
  for (int ax = 0; ax < 3; ++ax) {
    float ext = o2f(a.cmax[ax]) - o2f(a.cmin[ax]);
    if (!(ext > 0.f)) continue;
    float rarea[kBins];
    int rcnt[kBins];
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    int cnt = 0;
    for (int b = kBins - 1; b > 0; --b) {
      if (a.bin_cnt[ax][b]) for (int j = 0; j < 3; ++j) { lo[j] = fminf(lo[j], o2f(a.bin_min[ax][b][j])); hi[j] = fmaxf(hi[j], o2f(a.bin_max[ax][b][j])); }
      cnt += a.bin_cnt[ax][b];
      rarea[b] = box_area(lo, hi);
      rcnt[b] = cnt;
    }
    float llo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    int lc = 0;
    for (int b = 0; b < kBins - 1; ++b) {
      if (a.bin_cnt[ax][b]) for (int j = 0; j < 3; ++j) { llo[j] = fminf(llo[j], o2f(a.bin_min[ax][b][j])); lhi[j] = fmaxf(lhi[j], o2f(a.bin_max[ax][b][j])); }
      lc += a.bin_cnt[ax][b];
      if (lc == 0 || rcnt[b + 1] == 0) continue;
      float cost = box_area(llo, lhi) * float(lc) + rarea[b + 1] * float(rcnt[b + 1]);
      if (cost < best) { best = cost; axis = ax; split = b; }
    }
  }
  a.axis = axis;
  a.split_bin = split;
  a.by_index = axis < 0 ? 1 : 0;      // all centroids coincide: split by index
  a.left = 0;
}

__device__ __forceinline__ bool goes_left(const TaskAcc& a, const Task& tk, int pos, const float4* cen, int t) {
  if (a.by_index) return pos < tk.first + tk.count / 2;
  float l = o2f(a.cmin[a.axis]), h = o2f(a.cmax[a.axis]);
  float sc = float(kBins) / (h - l);
  float4 ce = cen[t];
  float x = a.axis == 0 ? ce.x : a.axis == 1 ? ce.y : ce.z;
  return bin_of(x, l, sc) <= a.split_bin;
}

__global__ void __launch_bounds__(kThreads) k_chunk_count(const Chunk* chunks, const Task* tasks, const int32_t* idx,
                                                          const float4* cen, const TaskAcc* acc, int* chunk_left) {
  __shared__ int s;
  const Chunk c = chunks[blockIdx.x];
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  const Task tk = tasks[c.task];
  const TaskAcc& a = acc[c.task];
  int cnt = 0;
  for (int i = threadIdx.x; i < c.len; i += blockDim.x) cnt += goes_left(a, tk, c.start + i, cen, idx[c.start + i]) ? 1 : 0;
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(kAll, cnt, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(&s, cnt);
  __syncthreads();
  if (threadIdx.x == 0) chunk_left[blockIdx.x] = s;
}

// One thread per task: exclusive scan of its chunks' left counts (its chunks
// are consecutive in the chunk list).
__global__ void k_task_scan(const int* task_chunk0, int n_tasks, int n_chunks, int* chunk_left, TaskAcc* acc) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_tasks) return;
  int c0 = task_chunk0[k], c1 = k + 1 < n_tasks ? task_chunk0[k + 1] : n_chunks;
  int run = 0;
  for (int c = c0; c < c1; ++c) { int v = chunk_left[c]; chunk_left[c] = run; run += v; }
  acc[k].left = run;
}

// Stable partition of a chunk: block-wide ordered ranks from warp ballots.
__global__ void __launch_bounds__(kThreads) k_chunk_scatter(const Chunk* chunks, const Task* tasks, const int32_t* idx,
                                                            const float4* cen, const TaskAcc* acc, const int* chunk_left,
                                                            int32_t* out) {
  __shared__ int s_w[kThreads / 32], s_in[kThreads / 32];
  __shared__ int s_run[2];
  const Chunk c = chunks[blockIdx.x];
  const Task tk = tasks[c.task];
  const TaskAcc& a = acc[c.task];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) {
    s_run[0] = tk.first + chunk_left[blockIdx.x];                                        // next left slot
    s_run[1] = tk.first + a.left + (c.start - tk.first - chunk_left[blockIdx.x]);        // next right slot
  }
  __syncthreads();
  for (int base = 0; base < c.len; base += blockDim.x) {
    int i = base + threadIdx.x;
    bool in = i < c.len;
    int t = in ? idx[c.start + i] : 0;
    bool left = in && goes_left(a, tk, c.start + i, cen, t);
    unsigned bl = __ballot_sync(kAll, left);
    unsigned bin = __ballot_sync(kAll, in);
    if (lane == 0) { s_w[warp] = __popc(bl); s_in[warp] = __popc(bin); }
    __syncthreads();
    int lbase = s_run[0], rbase = s_run[1];
    int lw = 0, rw = 0;
    for (int w = 0; w < warp; ++w) { lw += s_w[w]; rw += s_in[w] - s_w[w]; }
    unsigned below = (1u << lane) - 1u;
    if (left) out[lbase + lw + __popc(bl & below)] = t;
    else if (in) out[rbase + rw + __popc(~bl & bin & below)] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
      int lt = 0;
      for (int w = 0; w < nw; ++w) lt += s_w[w];
      int nin = min(int(blockDim.x), c.len - base);
      s_run[0] += lt;
      s_run[1] += nin - lt;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kThreads) k_chunk_copy(const Chunk* chunks, const int32_t* src, int32_t* dst) {
  const Chunk c = chunks[blockIdx.x];
  for (int i = threadIdx.x; i < c.len; i += blockDim.x) dst[c.start + i] = src[c.start + i];
}

__global__ void k_task_children(const Task* tasks, int n_tasks, const TaskAcc* acc, TreeNode* nodes, int* next_node,
                                Task* next_tasks, int* max_depth) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_tasks) return;
  const Task tk = tasks[k];
  int left = acc[k].left;
  int c0 = atomicAdd(next_node, 2);
  TreeNode& nd = nodes[tk.node];
  nd.child = c0; nd.first = 0; nd.count = 0;
  next_tasks[2 * k] = Task{c0, tk.first, left, tk.depth + 1};
  next_tasks[2 * k + 1] = Task{c0 + 1, tk.first + left, tk.count - left, tk.depth + 1};
  atomicMax(max_depth, tk.depth + 1);
}

// ---- small subtrees: one warp each -----------------------------------------
struct WarpBins {
  int cnt[3][kBins];
  int mn[3][kBins][3], mx[3][kBins][3];
};

__device__ __forceinline__ float warp_min(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kAll, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kAll, v, o));
  return v;
}

constexpr int kSmallWarps = 4;
static_assert(kBins == 32, "k_small sweeps one bin per lane");

__global__ void __launch_bounds__(32 * kSmallWarps) k_small(const Task* tasks, int n_tasks, int max_leaf, int32_t* idx,
                                                            int32_t* scratch, const float4* tlo, const float4* thi,
                                                            const float4* cen, TreeNode* nodes, int* next_node,
                                                            int* max_depth, int* overflow) {
  __shared__ WarpBins s_bins[kSmallWarps];
  __shared__ Task s_stack[kSmallWarps][kWarpStack];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int k = blockIdx.x * kSmallWarps + wid;
  if (k >= n_tasks) return;                      // whole warp
  WarpBins& bins = s_bins[wid];
  Task* stack = s_stack[wid];
  int sp = 0;
  if (lane == 0) stack[0] = tasks[k];
  sp = 1;
  __syncwarp();
  int deepest = 0;
  while (sp > 0) {
    Task tk = stack[--sp];
    __syncwarp();
    deepest = max(deepest, tk.depth);
    // node box and centroid bounds
    float bl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    float cl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, ch[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = lane; i < tk.count; i += 32) {
      int t = idx[tk.first + i];
      float4 a = tlo[t], b = thi[t], c = cen[t];
      bl[0] = fminf(bl[0], a.x); bl[1] = fminf(bl[1], a.y); bl[2] = fminf(bl[2], a.z);
      bh[0] = fmaxf(bh[0], b.x); bh[1] = fmaxf(bh[1], b.y); bh[2] = fmaxf(bh[2], b.z);
      cl[0] = fminf(cl[0], c.x); cl[1] = fminf(cl[1], c.y); cl[2] = fminf(cl[2], c.z);
      ch[0] = fmaxf(ch[0], c.x); ch[1] = fmaxf(ch[1], c.y); ch[2] = fmaxf(ch[2], c.z);
    }
    for (int j = 0; j < 3; ++j) { bl[j] = warp_min(bl[j]); bh[j] = warp_max(bh[j]); cl[j] = warp_min(cl[j]); ch[j] = warp_max(ch[j]); }
    TreeNode& nd = nodes[tk.node];
    if (lane == 0) for (int j = 0; j < 3; ++j) { nd.lo[j] = bl[j]; nd.hi[j] = bh[j]; }
    int axis = -1, split = -1;
    float best = FLT_MAX;
    if (tk.count > 1) {
      for (int q = lane; q < 3 * kBins; q += 32) {
        (&bins.cnt[0][0])[q] = 0;
        for (int j = 0; j < 3; ++j) { (&bins.mn[0][0][0])[3 * q + j] = INT_MAX; (&bins.mx[0][0][0])[3 * q + j] = INT_MIN; }
      }
      __syncwarp();
      float sc[3];
      for (int ax = 0; ax < 3; ++ax) { float ext = ch[ax] - cl[ax]; sc[ax] = ext > 0.f ? float(kBins) / ext : 0.f; }
      for (int i = lane; i < tk.count; i += 32) {
        int t = idx[tk.first + i];
        float4 a = tlo[t], b = thi[t], c = cen[t];
        float cc[3] = {c.x, c.y, c.z};
        int el[3] = {f2o(a.x), f2o(a.y), f2o(a.z)}, eh[3] = {f2o(b.x), f2o(b.y), f2o(b.z)};
        for (int ax = 0; ax < 3; ++ax) {
          if (!(ch[ax] - cl[ax] > 0.f)) continue;
          int bb = bin_of(cc[ax], cl[ax], sc[ax]);
          atomicAdd(&bins.cnt[ax][bb], 1);
          for (int j = 0; j < 3; ++j) { atomicMin(&bins.mn[ax][bb][j], el[j]); atomicMax(&bins.mx[ax][bb][j], eh[j]); }
        }
      }
      __syncwarp();
      // SAH sweep with lane b on bin b of each axis: the boxes right of and
      // left of each split come from suffix / prefix min-max over the lanes
      // (exact in any order; empty bins contribute nothing), the cost is the
      // host builder's expression, and the split kept is the first minimum
      // in (axis, bin) order, as a sequential sweep with `cost < best` keeps.
      float bestc = FLT_MAX;
      int bkey = INT_MAX;
      for (int ax = 0; ax < 3; ++ax) {
        if (!(ch[ax] - cl[ax] > 0.f)) continue;          // warp-uniform
        const int c = bins.cnt[ax][lane];
        float rlo[3], rhi[3], llo[3], lhi[3];
        for (int j = 0; j < 3; ++j) {
          rlo[j] = llo[j] = c ? o2f(bins.mn[ax][lane][j]) : FLT_MAX;
          rhi[j] = lhi[j] = c ? o2f(bins.mx[ax][lane][j]) : -FLT_MAX;
        }
        int rc = c, lc = c;
        for (int o = 1; o < 32; o <<= 1) {
          const int rco = __shfl_down_sync(kAll, rc, o), lco = __shfl_up_sync(kAll, lc, o);
          for (int j = 0; j < 3; ++j) {
            const float a0 = __shfl_down_sync(kAll, rlo[j], o), a1 = __shfl_down_sync(kAll, rhi[j], o);
            const float b0 = __shfl_up_sync(kAll, llo[j], o), b1 = __shfl_up_sync(kAll, lhi[j], o);
            if (lane + o < 32) { rlo[j] = fminf(rlo[j], a0); rhi[j] = fmaxf(rhi[j], a1); }
            if (lane >= o) { llo[j] = fminf(llo[j], b0); lhi[j] = fmaxf(lhi[j], b1); }
          }
          if (lane + o < 32) rc += rco;
          if (lane >= o) lc += lco;
        }
        const float rarea = box_area(rlo, rhi);
        const float rarea1 = __shfl_down_sync(kAll, rarea, 1);   // bins lane+1..31
        const int rc1 = __shfl_down_sync(kAll, rc, 1);
        if (lane < kBins - 1 && lc != 0 && rc1 != 0) {
          const float cost = box_area(llo, lhi) * float(lc) + rarea1 * float(rc1);
          if (cost < bestc) { bestc = cost; bkey = ax * kBins + lane; }
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const float oc = __shfl_xor_sync(kAll, bestc, o);
        const int ok = __shfl_xor_sync(kAll, bkey, o);
        if (oc < bestc || (oc == bestc && ok < bkey)) { bestc = oc; bkey = ok; }
      }
      if (bkey != INT_MAX) { axis = bkey / kBins; split = bkey % kBins; best = bestc; }
    }
    float leaf_cost = box_area(bl, bh) * float(tk.count);
    bool leaf = tk.count <= 1 || (tk.count <= max_leaf && (axis < 0 || leaf_cost <= best));
    if (!leaf && sp + 2 > kWarpStack) {           // cannot happen (smaller child first); the build then fails
      leaf = true;
      if (lane == 0) atomicAdd(overflow, 1);
    }
    if (leaf) {
      if (lane == 0) { nd.child = -1; nd.first = tk.first; nd.count = tk.count; }
      __syncwarp();
      continue;
    }
    // stable partition through the scratch range, then back
    int mid;
    {
      float sc = axis >= 0 ? float(kBins) / (ch[axis] - cl[axis]) : 0.f;
      int nl = 0;
      // count left
      for (int base = 0; base < tk.count; base += 32) {
        int i = base + lane;
        bool in = i < tk.count;
        bool left = false;
        if (in) {
          if (axis < 0) left = i < tk.count / 2;
          else {
            float4 c = cen[idx[tk.first + i]];
            float x = axis == 0 ? c.x : axis == 1 ? c.y : c.z;
            left = bin_of(x, cl[axis], sc) <= split;
          }
        }
        nl += __popc(__ballot_sync(kAll, left));
      }
      int lo_run = 0, hi_run = nl;
      for (int base = 0; base < tk.count; base += 32) {
        int i = base + lane;
        bool in = i < tk.count;
        int t = in ? idx[tk.first + i] : 0;
        bool left = false;
        if (in) {
          if (axis < 0) left = i < tk.count / 2;
          else {
            float4 c = cen[t];
            float x = axis == 0 ? c.x : axis == 1 ? c.y : c.z;
            left = bin_of(x, cl[axis], sc) <= split;
          }
        }
        unsigned bl2 = __ballot_sync(kAll, left), bi = __ballot_sync(kAll, in);
        unsigned below = (1u << lane) - 1u;
        if (left) scratch[tk.first + lo_run + __popc(bl2 & below)] = t;
        else if (in) scratch[tk.first + hi_run + __popc(~bl2 & bi & below)] = t;
        lo_run += __popc(bl2);
        hi_run += __popc(~bl2 & bi);
      }
      __syncwarp();
      for (int i = lane; i < tk.count; i += 32) idx[tk.first + i] = scratch[tk.first + i];
      __syncwarp();
      mid = nl;
    }
    int c0 = 0;
    if (lane == 0) {
      c0 = atomicAdd(next_node, 2);
      nd.child = c0; nd.first = 0; nd.count = 0;
      Task l{c0, tk.first, mid, tk.depth + 1}, r{c0 + 1, tk.first + mid, tk.count - mid, tk.depth + 1};
      // the smaller child is built next, so the stack holds at most
      // log2(kSmall) + 1 pending larger siblings
      bool left_smaller = mid <= tk.count - mid;
      stack[sp] = left_smaller ? r : l;
      stack[sp + 1] = left_smaller ? l : r;
    }
    sp += 2;
    __syncwarp();
  }
  if (lane == 0) atomicMax(max_depth, deepest);
}

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  explicit DevBuf(size_t count) : n(count) { ck(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)), "cudaMalloc"); }
  ~DevBuf() { if (p) cudaFree(p); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

// ---- compressed 8-wide layout on the device ---------------------------------
// The host writer (bvh_build.cpp, emit_wide) processes wide nodes breadth
// first: a node opens binary nodes greedily (largest surface area first) up to
// 8 children, assigns them to octant slots, quantises their boxes, and gives
// its inner children consecutive node indices and its leaves' triangles
// consecutive positions, both in slot order. Here one level of that queue is
// processed at once (one thread per wide node) and the indices come from
// exclusive scans over the level, which reproduces the host's numbering. The
// float arithmetic is the host's (this file is built without FMA
// contraction; fmaf where the host calls std::fma).

struct WideJob { int32_t bnode; uint32_t wide; int32_t depth; int32_t pad; };

__device__ __forceinline__ float area_of(const TreeNode& t) { return box_area(t.lo, t.hi); }

__device__ int grid_exponent_dev(float extent) {
  if (!(extent > 0.f)) return -100;
  int e = int(ceil(log2(double(extent) / 255.0)));
  e = max(-110, min(140, e));
  for (int g = 0; g < 300 && 255.0 * ldexp(1.0, e) < double(extent); ++g) ++e;
  for (int g = 0; g < 300 && 255.0 * ldexp(1.0, e - 1) >= double(extent); ++g) --e;
  return max(-100, min(127, e));
}

// One wide node per thread: children, slots, quantised boxes. Writes the
// node's 20 words except child base (word 4) and triangle base (word 5),
// the binary node in each slot (-1: empty) and the node's counts of inner
// children and leaf triangles.
__global__ void k_wide_collapse(const WideJob* jobs, int m, const TreeNode* tree, uint32_t* wide, int32_t* slot_kid,
                                int32_t* n_inner, int32_t* n_tris) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const WideJob jb = jobs[k];
  int kids[8];
  int nk = 0;
  const TreeNode& root = tree[jb.bnode];
  if (root.child < 0) { kids[nk++] = jb.bnode; }
  else { kids[nk++] = root.child; kids[nk++] = root.child + 1; }
  while (nk < 8) {
    int best = -1;
    float barea = -1.f;
    for (int i = 0; i < nk; ++i) {
      const TreeNode& c = tree[kids[i]];
      if (c.child >= 0 && area_of(c) > barea) { barea = area_of(c); best = i; }
    }
    if (best < 0) break;
    int c = kids[best];
    kids[best] = tree[c].child;
    kids[nk++] = tree[c].child + 1;
  }
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int i = 0; i < nk; ++i)
    for (int a = 0; a < 3; ++a) {
      // std::min / std::max order of the host's Box::grow
      float l = tree[kids[i]].lo[a], h = tree[kids[i]].hi[a];
      lo[a] = l < lo[a] ? l : lo[a];
      hi[a] = hi[a] < h ? h : hi[a];
    }
  float ctr[3] = {0.5f * (lo[0] + hi[0]), 0.5f * (lo[1] + hi[1]), 0.5f * (lo[2] + hi[2])};
  // candidates (kid, slot) with cost, generated kid-major like the host and
  // sorted stably by cost (insertion sort)
  float cost[64];
  int8_t ckid[64], cslot[64];
  int nc = 0;
  for (int i = 0; i < nk; ++i) {
    const TreeNode& cb = tree[kids[i]];
    float c[3] = {0.5f * (cb.lo[0] + cb.hi[0]) - ctr[0], 0.5f * (cb.lo[1] + cb.hi[1]) - ctr[1],
                  0.5f * (cb.lo[2] + cb.hi[2]) - ctr[2]};
    for (int sl = 0; sl < 8; ++sl) {
      float d[3] = {(sl & 4) ? 1.f : -1.f, (sl & 2) ? 1.f : -1.f, (sl & 1) ? 1.f : -1.f};
      float v = c[0] * d[0] + c[1] * d[1] + c[2] * d[2];
      int j = nc++;
      while (j > 0 && cost[j - 1] > v) { cost[j] = cost[j - 1]; ckid[j] = ckid[j - 1]; cslot[j] = cslot[j - 1]; --j; }
      cost[j] = v; ckid[j] = int8_t(i); cslot[j] = int8_t(sl);
    }
  }
  int slot_of[8], kid_in[8];
  for (int i = 0; i < 8; ++i) { slot_of[i] = -1; kid_in[i] = -1; }
  for (int q = 0; q < nc; ++q)
    if (slot_of[ckid[q]] < 0 && kid_in[cslot[q]] < 0) { slot_of[ckid[q]] = cslot[q]; kid_in[cslot[q]] = ckid[q]; }
  int ex[3];
  for (int a = 0; a < 3; ++a) ex[a] = grid_exponent_dev(hi[a] - lo[a]);
  uint8_t bytes[80];
  for (int i = 0; i < 80; ++i) bytes[i] = 0;
  for (int a = 0; a < 3; ++a) {
    uint32_t w = __float_as_uint(lo[a]);
    for (int b = 0; b < 4; ++b) bytes[4 * a + b] = uint8_t(w >> (8 * b));
  }
  bytes[12] = uint8_t(int8_t(ex[0])); bytes[13] = uint8_t(int8_t(ex[1])); bytes[14] = uint8_t(int8_t(ex[2]));
  uint8_t imask = 0;
  int inner = 0, tri_off = 0;
  int32_t* sk = slot_kid + 8 * int64_t(k);
  for (int sl = 0; sl < 8; ++sl) {
    if (kid_in[sl] < 0) {
      sk[sl] = -1;
      bytes[24 + sl] = 0;
      for (int a = 0; a < 3; ++a) { bytes[32 + 8 * a + sl] = 255; bytes[56 + 8 * a + sl] = 0; }
      continue;
    }
    const int kb = kids[kid_in[sl]];
    sk[sl] = kb;
    const TreeNode& c = tree[kb];
    for (int a = 0; a < 3; ++a) {
      float sc = ldexpf(1.0f, ex[a]);
      float l0 = lo[a];
      double ql = floor((double(c.lo[a]) - double(l0)) / double(sc));
      double qh = ceil((double(c.hi[a]) - double(l0)) / double(sc));
      int il = int(fmax(0.0, fmin(255.0, ql)));
      int ih = int(fmax(0.0, fmin(255.0, qh)));
      while (il > 0 && fmaf(float(il), sc, l0) > c.lo[a]) --il;
      while (ih < 255 && fmaf(float(ih), sc, l0) < c.hi[a]) ++ih;
      bytes[32 + 8 * a + sl] = uint8_t(il);
      bytes[56 + 8 * a + sl] = uint8_t(ih);
    }
    if (c.child >= 0) {
      imask |= uint8_t(1u << sl);
      bytes[24 + sl] = uint8_t((1u << 5) | uint32_t(24 + sl));
      ++inner;
    } else {
      int cnt = c.count;          // 0..3
      uint8_t unary = cnt == 0 ? 0 : (cnt == 1 ? 1 : (cnt == 2 ? 3 : 7));
      bytes[24 + sl] = cnt == 0 ? 0 : uint8_t((unary << 5) | uint32_t(tri_off));
      tri_off += cnt;
    }
  }
  bytes[15] = imask;
  uint32_t* out = wide + 20 * int64_t(jb.wide);
  for (int i = 0; i < 20; ++i)
    if (i != 4 && i != 5)
      out[i] = uint32_t(bytes[4 * i]) | uint32_t(bytes[4 * i + 1]) << 8 | uint32_t(bytes[4 * i + 2]) << 16 |
               uint32_t(bytes[4 * i + 3]) << 24;
  n_inner[k] = inner;
  n_tris[k] = tri_off;
}

// Exclusive scans of two arrays of m counts (one block); totals at tot[0..1].
__global__ void __launch_bounds__(1024) k_scan2(int32_t* a, int32_t* b, int m, int32_t* tot) {
  __shared__ int32_t s_w[2][32];
  __shared__ int32_t s_carry[2];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t < 2) s_carry[t] = 0;
  __syncthreads();
  for (int base = 0; base < m; base += 1024) {
    int i = base + t;
    int32_t v[2] = {i < m ? a[i] : 0, i < m ? b[i] : 0}, incl[2];
    for (int c = 0; c < 2; ++c) {
      int32_t x = v[c];
      for (int o = 1; o < 32; o <<= 1) { int32_t y = __shfl_up_sync(kAll, x, o); if (lane >= o) x += y; }
      incl[c] = x;
      if (lane == 31) s_w[c][warp] = x;
    }
    __syncthreads();
    if (warp == 0)
      for (int c = 0; c < 2; ++c) {
        int32_t x = s_w[c][lane];
        for (int o = 1; o < 32; o <<= 1) { int32_t y = __shfl_up_sync(kAll, x, o); if (lane >= o) x += y; }
        s_w[c][lane] = x;
      }
    __syncthreads();
    if (i < m) {
      a[i] = s_carry[0] + (warp ? s_w[0][warp - 1] : 0) + incl[0] - v[0];
      b[i] = s_carry[1] + (warp ? s_w[1][warp - 1] : 0) + incl[1] - v[1];
    }
    __syncthreads();
    if (t < 2) s_carry[t] += s_w[t][31];
    __syncthreads();
  }
  if (t < 2) tot[t] = s_carry[t];
}

// Child and triangle bases of each wide node; the next level's jobs; the
// triangle order of the leaves.
__global__ void k_wide_assign(const WideJob* jobs, int m, const int32_t* slot_kid, const int32_t* inner_off,
                              const int32_t* tri_off, uint32_t node_base, uint32_t tri_base, const TreeNode* tree,
                              const int32_t* idx, uint32_t* wide, int32_t* order, WideJob* next) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const WideJob jb = jobs[k];
  uint32_t cb = node_base + uint32_t(inner_off[k]);
  uint32_t tb = tri_base + uint32_t(tri_off[k]);
  uint32_t* out = wide + 20 * int64_t(jb.wide);
  out[4] = cb;
  out[5] = tb;
  int r = 0;
  uint32_t t = tb;
  for (int sl = 0; sl < 8; ++sl) {
    int kb = slot_kid[8 * int64_t(k) + sl];
    if (kb < 0) continue;
    const TreeNode& c = tree[kb];
    if (c.child >= 0) {
      next[inner_off[k] + r] = WideJob{kb, cb + uint32_t(r), jb.depth + 1, 0};
      ++r;
    } else {
      for (int q = 0; q < c.count; ++q) order[t++] = idx[c.first + q];
    }
  }
}

// Leaf-ordered triangles: v0 (w = global id), v0 - v1, v2 - v0.
__global__ void k_wide_tris(const float* pos, const int32_t* order, int n, float4* tris) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int t = order[i];
  const float* p = pos + 9 * int64_t(t);
  tris[3 * int64_t(i)] = make_float4(p[0], p[1], p[2], __int_as_float(t));
  tris[3 * int64_t(i) + 1] = make_float4(p[0] - p[3], p[1] - p[4], p[2] - p[5], 0.f);
  tris[3 * int64_t(i) + 2] = make_float4(p[6] - p[0], p[7] - p[1], p[8] - p[2], 0.f);
}

// A binary tree built on the device, kept there.
struct DeviceTree {
  cudaStream_t st = nullptr;
  std::unique_ptr<DevBuf<float>> pos;
  std::unique_ptr<DevBuf<int32_t>> idx;
  std::unique_ptr<DevBuf<TreeNode>> nodes;
  int n_nodes = 0, depth = 0;
  DeviceTree() = default;
  DeviceTree(const DeviceTree&) = delete;
  DeviceTree& operator=(const DeviceTree&) = delete;
  ~DeviceTree() { if (st) { cudaStreamSynchronize(st); cudaStreamDestroy(st); } }
};

void build_tree_device(const float* tri_pos, size_t n, int max_leaf, DeviceTree& dt) {
  if (n == 0) throw std::runtime_error("GPU BVH build: no triangles");
  if (n > size_t(INT32_MAX / 2)) throw std::runtime_error("GPU BVH build: too many triangles");
  const int ni = int(n);
  ck(cudaStreamCreateWithFlags(&dt.st, cudaStreamNonBlocking), "stream");
  cudaStream_t st = dt.st;
  dt.pos.reset(new DevBuf<float>(9 * n));
  dt.idx.reset(new DevBuf<int32_t>(n));
  dt.nodes.reset(new DevBuf<TreeNode>(2 * n + 1));
  DevBuf<float>& d_pos = *dt.pos;
  DevBuf<int32_t>& idx = *dt.idx;
  DevBuf<TreeNode>& nodes = *dt.nodes;
  DevBuf<float4> tlo(n), thi(n), cen(n);
  DevBuf<int32_t> tmp(n);
  DevBuf<int> counters(3);                       // next node, max depth, warp-stack overflow
  ck(cudaMemcpyAsync(d_pos.p, tri_pos, 9 * n * sizeof(float), cudaMemcpyHostToDevice, st), "upload triangles");
  k_prims<<<(ni + 255) / 256, 256, 0, st>>>(d_pos.p, ni, tlo.p, thi.p, cen.p, idx.p);
  int init[3] = {1, 0, 0};
  ck(cudaMemcpyAsync(counters.p, init, sizeof(init), cudaMemcpyHostToDevice, st), "counters");

  std::vector<Task> level{Task{0, 0, ni, 0}};
  std::vector<Task> small;
  // large nodes, one level per iteration
  while (!level.empty()) {
    std::vector<Task> big;
    for (const Task& t : level) (t.count > kSmall ? big : small).push_back(t);
    if (big.empty()) break;
    std::vector<Chunk> chunks;
    std::vector<int> task_chunk0;
    for (size_t k = 0; k < big.size(); ++k) {
      task_chunk0.push_back(int(chunks.size()));
      for (int s = big[k].first; s < big[k].first + big[k].count; s += kChunk)
        chunks.push_back(Chunk{int(k), s, std::min(kChunk, big[k].first + big[k].count - s), 0});
    }
    const int nt = int(big.size()), nc = int(chunks.size());
    DevBuf<Task> d_tasks(big.size()), d_next(2 * big.size());
    DevBuf<Chunk> d_chunks(chunks.size());
    DevBuf<int> d_chunk0(task_chunk0.size()), d_left(chunks.size());
    DevBuf<TaskAcc> d_acc(big.size());
    ck(cudaMemcpyAsync(d_tasks.p, big.data(), big.size() * sizeof(Task), cudaMemcpyHostToDevice, st), "tasks");
    ck(cudaMemcpyAsync(d_chunks.p, chunks.data(), chunks.size() * sizeof(Chunk), cudaMemcpyHostToDevice, st), "chunks");
    ck(cudaMemcpyAsync(d_chunk0.p, task_chunk0.data(), task_chunk0.size() * sizeof(int), cudaMemcpyHostToDevice, st), "chunk starts");
    k_acc_init<<<nt, 256, 0, st>>>(d_acc.p, nt);
    k_chunk_bounds<<<nc, kThreads, 0, st>>>(d_chunks.p, d_tasks.p, idx.p, tlo.p, thi.p, cen.p, d_acc.p);
    k_chunk_bins<<<nc, kThreads, 0, st>>>(d_chunks.p, idx.p, tlo.p, thi.p, cen.p, d_acc.p);
    k_task_split<<<(nt + 63) / 64, 64, 0, st>>>(d_tasks.p, nt, d_acc.p, nodes.p);
    k_chunk_count<<<nc, kThreads, 0, st>>>(d_chunks.p, d_tasks.p, idx.p, cen.p, d_acc.p, d_left.p);
    k_task_scan<<<(nt + 63) / 64, 64, 0, st>>>(d_chunk0.p, nt, nc, d_left.p, d_acc.p);
    k_chunk_scatter<<<nc, kThreads, 0, st>>>(d_chunks.p, d_tasks.p, idx.p, cen.p, d_acc.p, d_left.p, tmp.p);
    k_chunk_copy<<<nc, kThreads, 0, st>>>(d_chunks.p, tmp.p, idx.p);
    k_task_children<<<(nt + 63) / 64, 64, 0, st>>>(d_tasks.p, nt, d_acc.p, nodes.p, counters.p, d_next.p, counters.p + 1);
    ck(cudaGetLastError(), "large-node level");
    level.resize(2 * big.size());
    ck(cudaMemcpyAsync(level.data(), d_next.p, level.size() * sizeof(Task), cudaMemcpyDeviceToHost, st), "next level");
    ck(cudaStreamSynchronize(st), "large-node level");
  }
  if (!small.empty()) {
    DevBuf<Task> d_small(small.size());
    ck(cudaMemcpyAsync(d_small.p, small.data(), small.size() * sizeof(Task), cudaMemcpyHostToDevice, st), "small tasks");
    int ns = int(small.size());
    k_small<<<(ns + kSmallWarps - 1) / kSmallWarps, 32 * kSmallWarps, 0, st>>>(
        d_small.p, ns, max_leaf, idx.p, tmp.p, tlo.p, thi.p, cen.p, nodes.p, counters.p, counters.p + 1, counters.p + 2);
    ck(cudaGetLastError(), "small subtrees");
  }
  int cnt[3];
  ck(cudaMemcpyAsync(cnt, counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, st), "counters");
  ck(cudaStreamSynchronize(st), "build");
  if (cnt[2] != 0) throw std::runtime_error("GPU BVH build: subtree stack overflow");
  dt.n_nodes = cnt[0];
  dt.depth = cnt[1] + 1;
}

}  // namespace

void build_tree_gpu(const float* tri_pos, size_t n, int max_leaf, BinaryTree& out) {
  DeviceTree dt;
  build_tree_device(tri_pos, n, max_leaf, dt);
  out.nodes.resize(size_t(dt.n_nodes));
  out.idx.resize(n);
  ck(cudaMemcpyAsync(out.nodes.data(), dt.nodes->p, out.nodes.size() * sizeof(TreeNode), cudaMemcpyDeviceToHost, dt.st),
     "nodes");
  ck(cudaMemcpyAsync(out.idx.data(), dt.idx->p, n * sizeof(int32_t), cudaMemcpyDeviceToHost, dt.st), "order");
  ck(cudaStreamSynchronize(dt.st), "download");
  out.depth = dt.depth;
}

void build_wide_gpu(const float* tri_pos, size_t n, BvhHost& out) {
  auto t0 = std::chrono::steady_clock::now();
  DeviceTree dt;
  build_tree_device(tri_pos, n, 3, dt);
  out.tree_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  cudaStream_t st = dt.st;
  const size_t max_wide = size_t(dt.n_nodes) + 1;
  DevBuf<uint32_t> wide(20 * max_wide);
  DevBuf<int32_t> order(n);
  DevBuf<int32_t> tot(2);
  std::unique_ptr<DevBuf<WideJob>> jobs(new DevBuf<WideJob>(1));
  WideJob root{0, 0u, 1, 0};
  ck(cudaMemcpyAsync(jobs->p, &root, sizeof(root), cudaMemcpyHostToDevice, st), "root job");
  int m = 1, depth = 0;
  uint32_t node_base = 1, tri_base = 0;
  while (m > 0) {
    depth += 1;
    const size_t mm = size_t(m);
    DevBuf<int32_t> slot_kid{8 * mm}, n_inner{mm}, n_tri{mm};
    k_wide_collapse<<<(m + 127) / 128, 128, 0, st>>>(jobs->p, m, dt.nodes->p, wide.p, slot_kid.p, n_inner.p, n_tri.p);
    k_scan2<<<1, 1024, 0, st>>>(n_inner.p, n_tri.p, m, tot.p);
    int32_t t2[2];
    ck(cudaMemcpyAsync(t2, tot.p, sizeof(t2), cudaMemcpyDeviceToHost, st), "level totals");
    ck(cudaStreamSynchronize(st), "wide level");
    if (size_t(node_base) + size_t(t2[0]) > max_wide) throw std::runtime_error("GPU BVH build: wide node count out of range");
    std::unique_ptr<DevBuf<WideJob>> next(new DevBuf<WideJob>(size_t(std::max(t2[0], 1))));
    k_wide_assign<<<(m + 127) / 128, 128, 0, st>>>(jobs->p, m, slot_kid.p, n_inner.p, n_tri.p, node_base, tri_base,
                                                   dt.nodes->p, dt.idx->p, wide.p, order.p, next->p);
    ck(cudaGetLastError(), "wide level");
    node_base += uint32_t(t2[0]);
    tri_base += uint32_t(t2[1]);
    m = t2[0];
    ck(cudaStreamSynchronize(st), "wide level");
    jobs = std::move(next);
  }
  if (tri_base != uint32_t(n)) throw std::runtime_error("GPU BVH build: leaves do not hold every triangle");
  DevBuf<float4> tris(3 * n);
  k_wide_tris<<<(int(n) + 255) / 256, 256, 0, st>>>(dt.pos->p, order.p, int(n), tris.p);
  ck(cudaGetLastError(), "wide triangles");
  out.nodes.resize(20 * size_t(node_base));
  out.order.resize(n);
  out.tris.resize(12 * n);
  ck(cudaMemcpyAsync(out.nodes.data(), wide.p, out.nodes.size() * sizeof(float), cudaMemcpyDeviceToHost, st), "wide nodes");
  ck(cudaMemcpyAsync(out.order.data(), order.p, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "order");
  ck(cudaMemcpyAsync(out.tris.data(), tris.p, out.tris.size() * sizeof(float), cudaMemcpyDeviceToHost, st), "triangles");
  ck(cudaStreamSynchronize(st), "download");
  out.depth = depth;
}

}  // namespace hasty
