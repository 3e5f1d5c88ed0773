// Wavefront path state and kernel launch interface (host + device).
//
// One path slot per camera sample of a batch: slot = k * (W*H) + pixel for
// pass pass_base + k. State lives in structure-of-arrays buffers in HBM;
// each bounce runs `trace` (closest hit of every queued ray) and `shade`
// (resolve the previous vertex's NEE and BSDF samples, shade the new vertex,
// emit its rays). Queues are compacted with warp ballots.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "hasty_types.h"

namespace hasty {

// flags word (stored as the w lane of PathsDev::rad)
enum : uint32_t {
  PF_DEPTH_MASK = 0xFFu,          // depth of the vertex the pending BRDF ray leaves from
  PF_WL_SHIFT = 8,                // wavelength + 1 (0: not chosen yet)
  PF_WL_MASK = 0x3u << 8,
  PF_PEND_B = 1u << 14,           // BSDF-sampled ray queued in ray slot 2s
  PF_PEND_L = 1u << 15,           // light-sampled ray queued in ray slot 2s+1
  PF_CAMERA = 1u << 16,           // pending ray is the camera ray
  PF_NMED_SHIFT = 17,             // media on the stack (0..kMediaMax)
  PF_NMED_MASK = 0x1Fu << 17,
  PF_CHUNK_SHIFT = 24,            // packed batches: chunk of the path's job (0 otherwise); also
  PF_CHUNK_MASK = 0xFFu << 24,    // the bits of ray_o.w of the path's rays
};
// Medium stack of a path (LightRayInfo's media, core/include/Hasty/LightRayInfo.h:51):
// the first kMaxMedia entries in the path's own slots; a path nested deeper
// takes one overflow block of kMediaBlock entries from the batch's pool
// (P.med_pool, P.counts[kMediaPoolCounter]), for kMediaMax entries in all.
// A push beyond that, or with the pool exhausted, is dropped and counted
// (ST_MEDIA_OVERFLOW).
constexpr int kMaxMedia = 4;
constexpr int kMediaBlock = 16;
constexpr int kMediaMax = kMaxMedia + kMediaBlock;
static_assert(kMediaMax < 32, "the stack depth has 5 bits in the flags");

struct PathsDev {
  uint64_t* rng;        // PCG32 state
  float4* thr;          // xyz: path throughput up to the pending BSDF sample, w: its pdf
  float4* rad;          // xyz: radiance gathered so far, w: flags
  float4* pend_b;       // xyz: BSDF-sample weight (f|cos|/pdf * RR/Beer of its vertex), w: vertex triangle;
                        // between the resolve and the sample kernel: the vertex's Beer/roulette factor
  float4* nee_c;        // xyz: throughput * f * |cos| of the light sample, w: BSDF pdf of its direction
  float4* nee_t;        // xyz: medium transmittance along the light ray, w: sampled light triangle (-1: env)
  float4* med;          // 4 per path: medium transmittance xyz, IOR
  int32_t* med_geom;    // 4 per path: OBJ shape id of the medium
  int32_t* med_block;   // per path: its overflow block in med_pool (-1: none)
  float4* med_pool;     // overflow blocks: kMediaBlock entries each (transmittance, IOR)
  int32_t* med_pool_geom;
  int32_t med_pool_blocks;
  float4* ray_o;        // 2 per path
  float4* ray_d;        // 2 per path
  float4* hit;          // 2 per path: t, u, v, triangle (-1 miss)
  int32_t* pq[2];       // path queues
  int32_t* rq[2];       // ray queues (ray ids 2s, 2s+1)
  uint32_t* counts;     // [pq0, pq1, rq0, rq1, trace fetch counter, sample-queue length, 2 spare]
  int32_t* sq;          // sample queue (paths that continue past resolve)
  float4* out_color;    // per slot: final radiance of the sample
  float4* out_normal;
  float4* out_albedo;
  unsigned long long* stats;   // see StatIndex
  int32_t capacity;
};

// ST_STACK_OVERFLOW: rays whose traversal stack was full when a subtree had
// to be pushed (the subtree is skipped; the hit may then not be the closest).
enum StatIndex { ST_RAYS = 0, ST_SHADED, ST_PATHS, ST_NAN, ST_MEDIA_OVERFLOW, ST_TRIAL_CAP, ST_STACK_OVERFLOW, ST_COUNT };
constexpr int kCountSlots = 8;
constexpr int kFetchCounter = 4;   // counts[4]: rays handed out by the persistent trace kernels
constexpr int kSampleCount = 5;    // counts[5]: length of the sample queue
constexpr int kMediaPoolCounter = 6;   // counts[6]: medium overflow blocks handed out in this batch

struct BatchDesc {
  uint64_t seed;
  uint32_t pass_base;
  int32_t n_passes;
  int32_t n_paths;      // n_passes * W * H
};

// Kernel launchers (integrator.cu / trace.cu). All launches go to `stream`.
void launch_raygen(const SceneDev& sc, const PathsDev& p, const BatchDesc& b, cudaStream_t stream);
// blocks_per_sm > 0 caps the persistent wide-BVH grid at that many resident
// blocks per SM (room for another stream's kernels); 0: all that fit.
void launch_trace(const SceneDev& sc, const PathsDev& p, int q, int max_rays, cudaStream_t stream, int blocks_per_sm = 0);
// True when sc's closest hits run one ray per thread instead of the
// persistent kernel: a wide BVH of at most simple_trace_nodes() nodes.
int simple_trace_nodes();
bool simple_trace_bvh(const SceneDev& sc);
void launch_shade(const SceneDev& sc, const PathsDev& p, const BatchDesc& b, int q, int max_paths, cudaStream_t stream);
void launch_accumulate(const SceneDev& sc, const PathsDev& p, const BatchDesc& b, double* acc_color, double* acc_normal,
                       double* acc_albedo, cudaStream_t stream);
void launch_estimate(const double* acc, int n, float den, float scale, float* out, cudaStream_t stream);

// Packed multi-job batches (batching and serving). A batch lays out chunks
// of consecutive passes of several jobs one after another in slot space:
// chunk c covers slots [first_slot, first_slot + n_passes * npix), slot
// first_slot + k * npix + px being pass pass_base + k of pixel px of its
// job. Every path carries its chunk index in its flags (PF_CHUNK_*) and its
// rays in ray_o.w, so the kernels find the job's scene, seed and accumulators
// without a per-slot table. The tables travel as kernel parameters.
constexpr int kMaxChunks = 64;
struct ChunkDev {
  SceneDev sc;
  uint64_t seed;
  int32_t first_slot;
  uint32_t pass_base;
  int32_t npix;
  int32_t n_passes;
};
struct ChunkTable {
  int32_t n;            // chunks
  int32_t n_paths;      // slots of all chunks
  ChunkDev c[kMaxChunks];
};
// The closest-hit kernel's part of a chunk.
struct TraceChunk {
  const float4* nodes;
  const float4* tris;
  int32_t nee_first_hit;   // light rays stop at their first hit (environment-only lighting)
  int32_t n_nodes, n_tris; // sizes of nodes and tris (the bounds-checked build checks them)
  int32_t pad;
};
struct TraceTable {
  int32_t n;
  int32_t bvh_kind;     // of every chunk (a context's jobs share one BVH layout)
  TraceChunk c[kMaxChunks];
};
static_assert(sizeof(ChunkTable) < 32000, "kernel parameters are limited to 32764 bytes");

void launch_raygen_packed(const ChunkTable& t, const PathsDev& p, cudaStream_t stream);
void launch_trace_packed(const TraceTable& t, const PathsDev& p, int q, int max_rays, cudaStream_t stream,
                         int blocks_per_sm = 0);
// resolve_threads 128 or 256, sample_threads 256 or 512 (block shapes; any
// other value takes 256 / 512).
void launch_shade_packed(const ChunkTable& t, const PathsDev& p, int q, int max_paths, cudaStream_t stream,
                         int resolve_threads = 256, int sample_threads = 512);
// Adds slots [first_slot, first_slot + n_passes * npix) (passes in order) into
// FP64 accumulators of npix pixels.
void launch_accumulate_range(const PathsDev& p, int first_slot, int npix, int n_passes, double* acc_color,
                             double* acc_normal, double* acc_albedo, cudaStream_t stream);

// Path kernel (scenes that stay in L1/L2): persistent threads, each carrying
// one camera sample through all its bounces in a slot of `slots` (path_slots()
// slots at least), finished samples written to `out`'s per-sample arrays
// (out_color/out_normal/out_albedo, indexed like a wavefront batch). Same
// samples as the wavefront kernels, bit for bit.
int64_t path_slots();
void launch_paths(const SceneDev& sc, const BatchDesc& b, const PathsDev& slots, const PathsDev& out, cudaStream_t stream);
void launch_paths_packed(const ChunkTable& t, int bvh_kind, const PathsDev& slots, const PathsDev& out,
                         cudaStream_t stream);

// Closest-hit queries of arbitrary rays (n x 6 floats, device memory).
void launch_trace_rays(const SceneDev& sc, const float* rays, int n, float4* hits, cudaStream_t stream);

// ---------------------------------------------------------------------------
// Multi-job engine (batching and serving). Many resident jobs share one pool
// of path slots. Work is a sequence of segments, each one pass of one job
// (W*H camera samples); camera samples are issued in global order through the
// segments into whatever slots are free, so the pool stays full until the
// last sample (path regeneration). The host appends segments between engine
// waves (serving interleaves the passes of the resident jobs this way).
// Finished samples are added to per-job int64 fixed-point accumulators
// (2^-32 units): integer addition is order-independent, so a job's image is
// bit-identical however it is mixed with other jobs.
constexpr double kFixedScale = 4294967296.0;   // 2^32

struct JobDev {
  SceneDev sc;
  unsigned long long* acc;     // [lane][9][npix] int64: colour, normal, albedo components (two's complement)
  unsigned long long* done;    // finished camera samples
  uint64_t seed;
  uint32_t npix;
  uint32_t lanes;              // a sample of pass p goes to lane p % lanes (spreads the atomics of small frames)
};

// One pass of one job: global samples [begin, begin + npix) of the job table
// entry `job`, pixel = global sample - begin.
struct SegDev {
  unsigned long long begin;
  int32_t job;
  uint32_t pass;
};

struct MultiDev {
  const JobDev* jobs;          // job table (entries are reused once a job has finished)
  const SegDev* segs;          // ring of segments, power-of-two capacity
  uint32_t seg_mask;
  const uint32_t* seg_window;  // [lo, hi): logical indices of the live segments (device-resident)
  uint4* slot_meta;            // per slot: job, pixel and pass of the path's camera sample, accumulator
                               // lane (one 16-byte load in the shading kernels)
  int32_t* free_slots;         // first slot of each free group (kGroup slots, no live path), ascending
                               // (rebuilt every iteration)
  uint8_t* flags;              // per slot: path lives on / BSDF ray queued / light ray queued
  uint32_t* block_sums;        // 3 per compaction block: counts, then exclusive offsets
  uint32_t* free_count;
  unsigned long long* next_sample;
  unsigned long long* total_samples;
  unsigned long long* regen_base;   // first global sample of the current regeneration
  uint32_t* ctl;               // kCtlWords: [0] queue parity, [1] regen count, [2] unused,
                               // [3] path-queue base, [4] ray-queue base, [5] iterations, [6] bound hit,
                               // [7] iteration at which the current wave ends, [8], [9] first and last
                               // segment (logical index) of the current regeneration
  uint32_t regen_below;        // regenerate only when fewer live paths than this
  uint32_t max_iter;           // iteration bound of one run (device-side loop guard)
};

constexpr int kCtlWords = 16;
constexpr int kGroup = 32;     // slots regenerated together (one warp); the engine's capacity is a multiple
static_assert(kGroup == 32, "a group is one warp of the compaction kernels");

enum MultiStat { MS_RAYS = ST_RAYS, MS_SHADED = ST_SHADED, MS_PATHS = ST_PATHS, MS_NAN = ST_NAN,
                 MS_MEDIA_OVERFLOW = ST_MEDIA_OVERFLOW, MS_TRIAL_CAP = ST_TRIAL_CAP, MS_SATURATED = ST_COUNT,
                 MS_COUNT };

// One engine iteration (regenerate, trace, shade, loop condition) launched
// into `stream`; `cond` is the CUDA-graph conditional handle of the enclosing
// while node (0 when launched without a graph).
void launch_multi_iteration(const PathsDev& p, const MultiDev& m, int capacity, int bvh_kind,
                            unsigned long long cond_handle, int use_cond, cudaStream_t stream, int trace_blocks_per_sm = 0);
void launch_multi_init(const PathsDev& p, const MultiDev& m, int capacity, cudaStream_t stream);
// Compaction blocks of an engine with `capacity` slots (3 block_sums entries each).
int compact_blocks(int capacity);
// Sums lanes 1.. of a job's fixed-point sums into lane 0 (integer adds:
// exact, so the result does not depend on the lane count).
void launch_fold_lanes(unsigned long long* acc, int npix, int lanes, cudaStream_t stream);
// Adds a finished job's fixed-point sums (lane 0) into FP64 accumulators (sum * 2^-32).
void launch_fixed_to_double(const unsigned long long* acc, int npix, double* c, double* n, double* a, cudaStream_t stream);
// trace.cu: closest hit of the queued rays of the multi-job engine.
void launch_trace_multi(const PathsDev& p, const MultiDev& m, int bvh_kind, int max_rays, cudaStream_t stream,
                        int blocks_per_sm = 0);

}  // namespace hasty
