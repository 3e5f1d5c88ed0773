// Photon mapper (stochastic progressive photon mapping with a caustics map):
// device data and kernel launchers (photon.cu); the host side and the C ABI
// are in photon_map.cpp.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "hasty_types.h"

namespace hasty {

// Random-stream keys of the photon mapper: photon i of iteration t, and the
// initial radius footprint of a pixel (a pass value no render reaches).
constexpr uint64_t kPhotonKeyMix = 0x50484F544F4E5321ull;
constexpr uint32_t kFootprintPass = 0xFFFFFFFFu;
// Deepest path the gather walks (its per-depth frames live in registers /
// local memory); jobs with a larger max_depth are refused.
constexpr int kPmMaxDepth = 32;

// One stored photon: position + n_g . w_from, incoming direction (towards
// where it came from) + emission index, flux + its index among the photons
// its emission stored (in depth order).
struct PhotonRec { float4 xn, wi, flux; };

struct PmEmitOut {
  PhotonRec* photons;      // append buffer
  uint32_t* count;         // photons appended (may exceed cap: those beyond are dropped)
  uint32_t cap;
  uint8_t* stored;         // per emitted photon of the launch: photons it stored
  unsigned long long* stats;   // [0] media overflow, [1] trial cap
  uint32_t* fetch;         // emission counter of the persistent kernel (cleared per launch)
};

// Photon map of one iteration: photons sorted by (cell x, y, z, emission
// index, depth); cells sorted lexicographically with the first photon and
// the count of each.
struct PmMapDev {
  const PhotonRec* photons;
  const int4* cells;       // x, y, z, first photon
  const int32_t* cell_count;
  const int32_t* n_cells;  // in device memory (written by the map build)
  float cell;
};

// Device status of one iteration's photon map build (photon_build.cu).
struct PmStatus {
  uint32_t cum;            // photons stored by the emissions scanned so far
  uint32_t done;           // the stored count reached the threshold
  uint32_t emitted;        // emissions up to and including the cutoff (when done)
  uint32_t kept;           // photons stored by those
  uint32_t appended;       // photons in the append buffer (a copy of its counter)
  int32_t lo[3], hi[3];    // cell bounds of the kept photons
};

// Per-pixel statistics (PMRenderJobPixel) and the thread's images.
struct PmPixelsDev {
  float* radius;           // -1 until first set
  float* N;
  float* Ne;
  float4* flux;
  float4* lsum;            // xyz: sum of L, w: number of samples (int bits)
  float* radii;            // the radius image of the render thread
  float* color;            // 3 per pixel
  float* normal;
  float* albedo;
};

// Distance from the camera to the first surface with a diffuse lobe along
// each pixel centre's ray (through up to max_depth concentrated bounces), or
// -1 where the reference's footprint falls back to its default.
void launch_pm_footprint(const SceneDev& sc, uint64_t seed, float* dist, cudaStream_t st);
// Emits photons [first, first + n) of iteration `iter` and traces them;
// min_q = 1 - 0.1^(1 / max_depth), the least absorption probability per
// bounce (evaluated on the host with the reference's std::pow).
void launch_pm_emit(const SceneDev& sc, uint64_t seed, uint32_t iter, uint32_t first, uint32_t n, float min_q,
                    const PmEmitOut& out, cudaStream_t st);
// Gathers every pixel of iteration `iter` (camera offset ox, oy) and updates
// the pixel statistics; `emitted` photons were emitted this iteration.
// Photon map build on the device (photon_build.cu).
// Exclusive scan of the store counts of emissions [first, first + n) into
// base[first..] continuing status->cum; the emission that takes the count to
// `threshold` sets status->done / emitted / kept. scratch: one word per
// 2048 counts.
void launch_pm_emit_scan(const uint8_t* stored, uint32_t n, uint32_t first, uint32_t threshold, uint32_t* base,
                         uint32_t* scratch, PmStatus* status, cudaStream_t st);
// Slots of the photons of emissions [0, emitted) in emission order
// (src[slot] = append index), their hash cells (coords[axis * cap + slot])
// and the cell bounds (status->lo / hi).
void launch_pm_place(const PhotonRec* app, uint32_t appended, const uint32_t* base, uint32_t emitted,
                     PmStatus* status, float cell, uint32_t* src, int32_t* coords, uint32_t cap, cudaStream_t st);
// One stable LSD pass over n slots by the byte (coord - lo) >> shift of one
// axis (perm_in null: slots in order). hist: 256 words per 2048 slots;
// scratch as for the scan of hist.
uint32_t pm_sort_tiles(uint32_t n);
void launch_pm_sort_pass(const int32_t* coord, int32_t lo, int shift, uint32_t n, const uint32_t* perm_in,
                         uint32_t* perm_out, uint32_t* hist, uint32_t* scratch, cudaStream_t st);
// Photons in sorted order, the cell table (x, y, z, first) with counts and
// the cell count in device memory.
void launch_pm_cells(const PhotonRec* app, const uint32_t* src, const int32_t* coords, uint32_t cap, uint32_t n,
                     const uint32_t* perm, PhotonRec* sorted, uint32_t* flag, uint32_t* cell_of, uint32_t* scratch,
                     int4* cells, int32_t* counts, int32_t* n_cells, cudaStream_t st);

void launch_pm_gather(const SceneDev& sc, const PmMapDev& map, const PmPixelsDev& px, uint64_t seed, uint32_t iter,
                      float ox, float oy, int emitted, unsigned long long* stats, cudaStream_t st);

}  // namespace hasty
