// Photon map built on the device (photon.h): the emission cutoff and the
// emission-order slots from the per-emission store counts (exclusive scans),
// the hash-cell coordinates, a stable LSD radix sort of the photons by cell
// and the cell table the gather searches. The order is the one the
// reference's hash cells list photons in (core/include/Hasty/HashCells.h:
// 40-104, filled in emission order by core/src/PhotonMapping.cpp:191-270):
// cells by (x, y, z), photons of a cell by emission index, then depth.
#include <cstdint>

#include "device_common.cuh"
#include "photon.h"

namespace hasty {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
// Scans and the sort work on tiles of 2048 elements: 256 threads x 8.
constexpr int kThreads = 256, kItems = 8, kTile = kThreads * kItems;

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* sh /* 8 words */) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  uint32_t s = 0;
  for (int w = 0; w < kThreads / 32; ++w) s += sh[w];
  return s;
}

// Exclusive prefix of v over the block's threads in thread order.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* sh /* 8 words */) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < warp; ++w) before += sh[w];
  return before + x - v;
}

template <class T>
__global__ void __launch_bounds__(kThreads) k_tile_sums(const T* in, uint32_t n, uint32_t* bsum) {
  __shared__ uint32_t sh[kThreads / 32];
  const uint32_t base = blockIdx.x * uint32_t(kTile);
  uint32_t s = 0;
  for (int it = 0; it < kItems; ++it) {
    const uint32_t i = base + uint32_t(it * kThreads) + threadIdx.x;
    if (i < n) s += uint32_t(in[i]);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) bsum[blockIdx.x] = s;
}

// bsum[0..nb) -> exclusive prefix sums offset by *init (0 when null);
// *total = *init + the sum (when not null; may alias init).
__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t* bsum, uint32_t nb, const uint32_t* init, uint32_t* total) {
  __shared__ uint32_t wt[32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t carry = init ? *init : 0u;
  for (uint32_t c = 0; c < nb; c += 1024u) {
    const uint32_t i = c + threadIdx.x;
    const uint32_t v = i < nb ? bsum[i] : 0u;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wt[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = wt[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, w, o);
        if (lane >= o) w += y;
      }
      wt[lane] = w;
    }
    __syncthreads();
    const uint32_t incl = x + (warp ? wt[warp - 1] : 0u);
    if (i < nb) bsum[i] = carry + incl - v;
    carry += wt[31];
    __syncthreads();
  }
  __syncthreads();                       // every thread has read *init
  if (threadIdx.x == 0 && total) *total = carry;
}

struct NoVisit {
  __device__ void operator()(uint32_t, uint32_t, uint32_t) const {}
};

// The reference emits photon after photon while fewer than `threshold` are
// stored (PhotonMapping.cpp:860-884): the cutoff is the emission whose
// stores take the running count to the threshold.
struct CutoffVisit {
  uint32_t first, threshold;
  PmStatus* st;
  __device__ void operator()(uint32_t i, uint32_t excl, uint32_t incl) const {
    if (excl < threshold && incl >= threshold) {
      st->emitted = first + i + 1u;
      st->kept = incl;
      st->done = 1u;
    }
  }
};

// out[i] = bsum[tile] + the exclusive prefix of in within the tile; thread t
// takes the tile's elements 8t..8t+7 in order.
template <class T, class Visit>
__global__ void __launch_bounds__(kThreads) k_scan_apply(const T* in, uint32_t n, const uint32_t* bsum, uint32_t* out,
                                                         Visit visit) {
  __shared__ uint32_t sh[kThreads / 32];
  const uint32_t base = blockIdx.x * uint32_t(kTile) + threadIdx.x * uint32_t(kItems);
  uint32_t v[kItems];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    const uint32_t i = base + uint32_t(k);
    v[k] = i < n ? uint32_t(in[i]) : 0u;
    s += v[k];
  }
  uint32_t excl = bsum[blockIdx.x] + block_exclusive(s, sh);
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    const uint32_t i = base + uint32_t(k);
    if (i < n) {
      if (out) out[i] = excl;
      visit(i, excl, excl + v[k]);
    }
    excl += v[k];
  }
}

template <class T, class Visit>
void scan_exclusive(const T* in, uint32_t n, uint32_t* out, uint32_t* bsum, const uint32_t* init, uint32_t* total,
                    Visit visit, cudaStream_t st) {
  const uint32_t nb = (n + uint32_t(kTile) - 1u) / uint32_t(kTile);
  if (nb == 0) return;
  k_tile_sums<T><<<nb, kThreads, 0, st>>>(in, n, bsum);
  k_scan_sums<<<1, 1024, 0, st>>>(bsum, nb, init, total);
  k_scan_apply<T, Visit><<<nb, kThreads, 0, st>>>(in, n, bsum, out, visit);
}

__global__ void k_bounds_init(PmStatus* st) {
  if (threadIdx.x < 3) {
    st->lo[threadIdx.x] = INT32_MAX;
    st->hi[threadIdx.x] = INT32_MIN;
  }
}

// Photon i of the append buffer goes to slot base[emission] + its index
// within the emission when its emission is before the cutoff; its cell
// (floor(x / cell) per axis, as HashCells::index) and the bounds of all
// cells are recorded.
__global__ void __launch_bounds__(kThreads) k_place(const PhotonRec* app, uint32_t appended, const uint32_t* base,
                                                    uint32_t emitted, PmStatus* st, float cell, uint32_t* src,
                                                    int32_t* coords, uint32_t cap) {
  __shared__ int32_t sh[6][kThreads / 32];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  int32_t c[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, d[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
  if (i < appended) {
    const PhotonRec r = app[i];
    const uint32_t e = __float_as_uint(r.wi.w), k = __float_as_uint(r.flux.w);
    if (e < emitted) {
      const uint32_t slot = base[e] + k;
      src[slot] = i;
      const float x[3] = {r.xn.x, r.xn.y, r.xn.z};
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const int32_t q = dev::floor_int32(x[a] / cell);
        coords[size_t(a) * cap + slot] = q;
        c[a] = q;
        d[a] = q;
      }
    }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int32_t mn = __reduce_min_sync(kFull, c[a]), mx = __reduce_max_sync(kFull, d[a]);
    if (lane == 0) { sh[a][warp] = mn; sh[3 + a][warp] = mx; }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int a = int(threadIdx.x);
    int32_t v = sh[a][0];
    for (int w = 1; w < kThreads / 32; ++w) v = a < 3 ? min(v, sh[a][w]) : max(v, sh[a][w]);
    if (a < 3) { if (v != INT32_MAX) atomicMin(&st->lo[a], v); }
    else if (v != INT32_MIN) atomicMax(&st->hi[a - 3], v);
  }
}

__device__ __forceinline__ uint32_t sort_digit(const int32_t* coord, int32_t lo, int shift, uint32_t p) {
  return ((uint32_t(coord[p]) - uint32_t(lo)) >> shift) & 255u;
}

// Digit histogram of each tile, digit-major: hist[d * nb + tile].
__global__ void __launch_bounds__(kThreads) k_sort_hist(const int32_t* coord, int32_t lo, int shift, uint32_t n,
                                                        const uint32_t* perm_in, uint32_t* hist, uint32_t nb) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * uint32_t(kTile);
  for (int it = 0; it < kItems; ++it) {
    const uint32_t i = base + uint32_t(it * kThreads) + threadIdx.x;
    if (i < n) atomicAdd(&h[sort_digit(coord, lo, shift, perm_in ? perm_in[i] : i)], 1u);
  }
  __syncthreads();
  hist[size_t(threadIdx.x) * nb + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: an element's position is its digit's offset for the tile
// (scanned histogram), plus the elements of that digit before it in the
// tile (earlier loop iterations, earlier warps of this iteration, earlier lanes).
__global__ void __launch_bounds__(kThreads) k_sort_scatter(const int32_t* coord, int32_t lo, int shift, uint32_t n,
                                                           const uint32_t* perm_in, uint32_t* perm_out,
                                                           const uint32_t* hist, uint32_t nb) {
  __shared__ uint32_t run[256];
  __shared__ uint32_t wcnt[kThreads / 32][256];
  const int t = int(threadIdx.x), warp = t >> 5, lane = t & 31;
  run[t] = hist[size_t(t) * nb + blockIdx.x];
  for (int w = 0; w < kThreads / 32; ++w) wcnt[w][t] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * uint32_t(kTile);
  for (int it = 0; it < kItems; ++it) {
    const uint32_t i = base + uint32_t(it * kThreads) + uint32_t(t);
    const bool valid = i < n;
    uint32_t p = 0, d = 0xFFFFFFFFu;
    if (valid) {
      p = perm_in ? perm_in[i] : i;
      d = sort_digit(coord, lo, shift, p);
    }
    const unsigned peers = __match_any_sync(kFull, d);
    const uint32_t rank = uint32_t(__popc(peers & ((1u << lane) - 1u)));
    if (valid && rank == 0) wcnt[warp][d] = uint32_t(__popc(peers));
    __syncthreads();
    if (valid) {
      uint32_t off = run[d] + rank;
      for (int w = 0; w < warp; ++w) off += wcnt[w][d];
      perm_out[off] = p;
    }
    __syncthreads();
    uint32_t add = 0;
    for (int w = 0; w < kThreads / 32; ++w) { add += wcnt[w][t]; wcnt[w][t] = 0; }
    run[t] += add;
    __syncthreads();
  }
}

// Photons in sorted order and the first photon of each cell flagged.
__global__ void __launch_bounds__(kThreads) k_sorted(const PhotonRec* app, const uint32_t* src, const int32_t* coords,
                                                     uint32_t cap, uint32_t n, const uint32_t* perm, PhotonRec* sorted,
                                                     uint32_t* flag) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const uint32_t s = perm ? perm[q] : q;
  sorted[q] = app[src[s]];
  uint32_t f = 1u;
  if (q > 0) {
    const uint32_t s0 = perm ? perm[q - 1] : q - 1;
    f = (coords[s] != coords[s0] || coords[cap + s] != coords[cap + s0] || coords[2 * cap + s] != coords[2 * cap + s0])
            ? 1u : 0u;
  }
  flag[q] = f;
}

__global__ void __launch_bounds__(kThreads) k_cells(const int32_t* coords, uint32_t cap, uint32_t n,
                                                    const uint32_t* perm, const uint32_t* flag, const uint32_t* cell_of,
                                                    int4* cells) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n || !flag[q]) return;
  const uint32_t s = perm ? perm[q] : q;
  cells[cell_of[q]] = make_int4(coords[s], coords[cap + s], coords[2 * cap + s], int(q));
}

__global__ void __launch_bounds__(kThreads) k_cell_counts(const int4* cells, const int32_t* n_cells, uint32_t n,
                                                          int32_t* counts) {
  const int c = int(blockIdx.x * blockDim.x + threadIdx.x);
  const int nc = *n_cells;
  if (c >= nc) return;
  counts[c] = (c + 1 < nc ? cells[c + 1].w : int(n)) - cells[c].w;
}

}  // namespace

void launch_pm_emit_scan(const uint8_t* stored, uint32_t n, uint32_t first, uint32_t threshold, uint32_t* base,
                         uint32_t* scratch, PmStatus* status, cudaStream_t st) {
  scan_exclusive<uint8_t>(stored, n, base + first, scratch, &status->cum, &status->cum,
                          CutoffVisit{first, threshold, status}, st);
}

void launch_pm_place(const PhotonRec* app, uint32_t appended, const uint32_t* base, uint32_t emitted,
                     PmStatus* status, float cell, uint32_t* src, int32_t* coords, uint32_t cap, cudaStream_t st) {
  k_bounds_init<<<1, 32, 0, st>>>(status);
  if (appended == 0) return;
  k_place<<<(appended + kThreads - 1) / kThreads, kThreads, 0, st>>>(app, appended, base, emitted, status, cell, src,
                                                                     coords, cap);
}

uint32_t pm_sort_tiles(uint32_t n) { return (n + uint32_t(kTile) - 1u) / uint32_t(kTile); }

void launch_pm_sort_pass(const int32_t* coord, int32_t lo, int shift, uint32_t n, const uint32_t* perm_in,
                         uint32_t* perm_out, uint32_t* hist, uint32_t* scratch, cudaStream_t st) {
  const uint32_t nb = pm_sort_tiles(n);
  if (nb == 0) return;
  k_sort_hist<<<nb, kThreads, 0, st>>>(coord, lo, shift, n, perm_in, hist, nb);
  scan_exclusive<uint32_t>(hist, 256u * nb, hist, scratch, nullptr, nullptr, NoVisit{}, st);
  k_sort_scatter<<<nb, kThreads, 0, st>>>(coord, lo, shift, n, perm_in, perm_out, hist, nb);
}

void launch_pm_cells(const PhotonRec* app, const uint32_t* src, const int32_t* coords, uint32_t cap, uint32_t n,
                     const uint32_t* perm, PhotonRec* sorted, uint32_t* flag, uint32_t* cell_of, uint32_t* scratch,
                     int4* cells, int32_t* counts, int32_t* n_cells, cudaStream_t st) {
  if (n == 0) {
    cudaMemsetAsync(n_cells, 0, sizeof(int32_t), st);
    return;
  }
  const uint32_t g = (n + kThreads - 1) / kThreads;
  k_sorted<<<g, kThreads, 0, st>>>(app, src, coords, cap, n, perm, sorted, flag);
  scan_exclusive<uint32_t>(flag, n, cell_of, scratch, nullptr, reinterpret_cast<uint32_t*>(n_cells), NoVisit{}, st);
  k_cells<<<g, kThreads, 0, st>>>(coords, cap, n, perm, flag, cell_of, cells);
  k_cell_counts<<<g, kThreads, 0, st>>>(cells, n_cells, n, counts);
}

}  // namespace hasty
